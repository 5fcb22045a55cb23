"""Mirror equivariance of the solvers, a size-independent property.

Reflecting the medium, the noise-source distribution and every station about
the domain's centre line (x -> Lx - x, or z -> Lz - z) must reflect the Green
spectra and leave the seismograms and correlations unchanged.  The staggered
operators of code/propagation/dx_v.m and div_s.m map a field that is even
under the reflection to an odd one and back, their edge rows left at zero sit
symmetrically (rows 1 and n-1 of dx_v, rows 1, 2, n-1, n of div_s), the taper
of code/propagation/init_absbound.m is symmetric when all four sides absorb,
and the nearest-node rule maps a station on a node to the mirrored node.  A
swapped index, a staggered point off by one or a one-sided edge row breaks the
symmetry at the level of the field itself, far above rounding.

One part of the reference is not symmetric: the stress at the staggered point
between nodes i and i+1 takes mu of node i, un-averaged
(code/run_forward1_green.m:168-172, mu(1:nx-1,:)).  The relation is therefore
exact only where mu is constant along the mirrored axis; rho and the noise
distribution may vary freely.  A medium whose mu varies along that axis breaks
it, which the last test shows.

Here on the FP64 oracle at every FD order, where the relation comes out bit
for bit (a reflected difference is the negated one, and IEEE rounding commutes
with negation); the breakers change the seismograms by 3 % (mu) and 22 %
(one-sided taper).  The GPU forms are tied to the oracle by the parity tests.
"""
import numpy as np
import pytest

from tests.problems import media, noise_source, rel_l2, small_cfg

AXES = (0, 1)


def _flip(a, axis):
    return np.asfortranarray(np.flip(a, axis=axis))


def _mirror_points(cfg, pts, axis):
    out = pts.copy()
    L = cfg.Lx if axis == 0 else cfg.Lz
    out[:, axis] = L - pts[:, axis]
    return out


def _mu_constant_along(m, axis):
    """mu of the seeded medium averaged along ``axis`` (so it varies only
    along the other one); rho unchanged."""
    mu, rho = m
    return np.asfortranarray(np.broadcast_to(mu.mean(axis=axis, keepdims=True), mu.shape)), rho


def _on_nodes(cfg, idx):
    dx, dz = cfg.Lx / (cfg.nx - 1), cfg.Lz / (cfg.nz - 1)
    return np.array([[i * dx, j * dz] for i, j in idx], dtype=float)


@pytest.mark.parametrize("order", [2, 4, 6, 8])
@pytest.mark.parametrize("axis", AXES)
def test_green_and_correlation_mirror(oracle, order, axis):
    cfg = small_cfg(nx=37, nz=31, nt=70, order=order, K=12, fs=5, fw=1)
    mu, rho = _mu_constant_along(media(cfg, seed=order), axis)
    spec, sd = noise_source(cfg, seed=5)
    src = _on_nodes(cfg, [(11, 9)])
    rec = _on_nodes(cfg, [(24, 17), (8, 21), (18, 15)])
    msrc, mrec = _mirror_points(cfg, src, axis), _mirror_points(cfg, rec, axis)
    mmu, mrho, msd = _flip(mu, axis), _flip(rho, axis), _flip(sd, axis)

    G, _, seis = oracle.forward1_green(cfg, mu, rho, src, rec, 0)
    mG, _, mseis = oracle.forward1_green(cfg, mmu, mrho, msrc, mrec, 0)
    assert np.abs(G).max() > 0 and np.abs(seis).max() > 0
    assert rel_l2(mG, _flip(G, axis)) < 1e-12
    assert rel_l2(mseis, seis) < 1e-12

    c, _ = oracle.forward2_correlation(cfg, mu, rho, G, spec, sd, rec, 0)
    mc, _ = oracle.forward2_correlation(cfg, mmu, mrho, mG, spec, msd, mrec, 0)
    assert np.abs(c).max() > 0
    assert rel_l2(mc, c) < 1e-12


@pytest.mark.parametrize("what", ["one-sided taper", "mu varying along the axis"])
def test_symmetry_breakers(oracle, what):
    """The property is not vacuous: absorbing on one side only, or the
    un-averaged mu of a medium that varies along the mirrored axis, make the
    mirrored problem a different one."""
    sides = dict(absorb_left=1, absorb_right=0) if what == "one-sided taper" else {}
    cfg = small_cfg(nx=37, nz=31, nt=70, order=4, K=12, fs=5, fw=1, **sides)
    mu, rho = media(cfg, seed=4)
    if what == "one-sided taper":
        mu, rho = _mu_constant_along((mu, rho), 0)
    src, rec = _on_nodes(cfg, [(11, 9)]), _on_nodes(cfg, [(24, 17), (8, 21)])
    _, _, seis = oracle.forward1_green(cfg, mu, rho, src, rec, 0)
    _, _, mseis = oracle.forward1_green(cfg, _flip(mu, 0), _flip(rho, 0), _mirror_points(cfg, src, 0),
                                        _mirror_points(cfg, rec, 0), 0)
    assert rel_l2(mseis, seis) > 1e-4
