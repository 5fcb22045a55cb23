"""The staggered-grid operators against the analytic 2-D SH Green's function.

Orders 6 and 8 have no counterpart in the reference (it implements 2 and 4),
so besides the Taylor conditions of their weights they are checked here
against physics: in a homogeneous medium the velocity of the reference's point
force (1e9 added to DS at the source node every step, i.e. a line force
F0 = 1e9*dx*dz switched on at t = 0, code/run_forward1_green.m:64,152-156) is

    v(r, t) = F0 / (2 pi mu) * H(t - r/c) / sqrt(t^2 - r^2/c^2),   c = sqrt(mu/rho).

Both sides are low-passed with the same Gaussian (the analytic convolution is
integrated over tau = (r/c) cosh(s), which removes the square-root
singularity).  With a time step far below the stability limit, so that the
leapfrog time error is negligible, the error must fall with the FD order.  At
the usual Courant numbers (~0.4) the second-order time error dominates and
partly cancels the spatial error of the low orders, so orders 4-8 then give
similar errors; that is a property of the scheme, not tested here.

The FP64 oracle runs the solver; the GPU forms are tied to the oracle by the
parity tests.
"""
import numpy as np
import pytest

from fd2d_noise_gb300.config import Config

N, DX, DT, T_END = 241, 1000.0, 0.02, 32.0
MU, RHO = 4.8e10, 3000.0
SIGMA = 0.4  # s, Gaussian low-pass
_trapz = getattr(np, "trapezoid", None) or np.trapz  # numpy 2 renamed it


def _lowpass(v, dt):
    k = np.arange(-int(6 * SIGMA / dt), int(6 * SIGMA / dt) + 1) * dt
    g = np.exp(-k ** 2 / (2 * SIGMA ** 2))
    return np.convolve(v, g / g.sum(), mode="same")


def _analytic(r, t):
    t0, F0 = r / np.sqrt(MU / RHO), 1e9 * DX * DX
    s = np.linspace(0.0, 12.0, 6001)
    tau = t0 * np.cosh(s)
    g = np.exp(-(t[:, None] - tau[None, :]) ** 2 / (2 * SIGMA ** 2)) / (np.sqrt(2 * np.pi) * SIGMA)
    return F0 / (2 * np.pi * MU) * _trapz(g, s, axis=1)


@pytest.fixture(scope="module")
def errors(oracle):
    L = DX * (N - 1)
    nt = int(round(T_END / DT))
    src = np.array([[L / 2, L / 2]])
    rec = np.array([[L / 2 + 30e3, L / 2], [L / 2 + 45e3, L / 2],       # along a grid axis
                    [L / 2 + 21e3, L / 2 + 21e3], [L / 2 + 32e3, L / 2 + 32e3]])  # diagonal nodes
    t = DT * np.arange(1, nt + 1)
    keep = (t > 5 * SIGMA) & (t < t[-1] - 6 * SIGMA)
    ref = [_analytic(np.hypot(*(p - src[0])), t)[keep] for p in rec]
    out = {}
    for order in (2, 4, 6, 8):
        cfg = Config(Lx=L, Lz=L, nx=N, nz=N, dt=DT, nt=nt, order=order, f_sample=np.array([0.05, 0.06]),
                     freq_samp=5, fw_nth=1, absorb_width=20 * DX)
        mu, rho = np.full((N, N), MU, order="F"), np.full((N, N), RHO, order="F")
        _, _, seis = oracle.forward1_green(cfg, mu, rho, src, rec, 0)
        out[order] = np.array([np.linalg.norm(_lowpass(seis[i], DT)[keep] - ref[i]) / np.linalg.norm(ref[i])
                               for i in range(rec.shape[0])])
    return out


def test_error_falls_with_order_along_the_axis(errors):
    e = {o: errors[o][:2] for o in errors}
    assert np.all(e[2] > 4 * e[4]) and np.all(e[4] > 2 * e[6]) and np.all(e[6] > 1.5 * e[8])
    assert np.all(e[8] < 5e-3), e[8]


def test_diagonal_propagation(errors):
    e = {o: errors[o][2:] for o in errors}
    assert np.all(e[2] > 4 * e[4]) and np.all(e[4] > 2 * e[8])
    assert np.all(e[8] < 3e-3) and np.all(e[6] < 3e-3), (e[6], e[8])
