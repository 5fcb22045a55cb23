"""The CPU oracle against case C of the reference's own solvers
(tests/golden/make_golden_c.py): a non-square grid with absorbing layers on
the left and top only, snapshots and DFT samples every 3 steps, two point
sources in the Green run, then the correlation run and the adjoint runs of
the gradient chain.  Same bars as the other cases: <= 1e-12 relative L2,
single-precision snapshots element for element except at rounding ties."""
import os

import numpy as np
import pytest

from fd2d_noise_gb300.config import Config
from tests.golden_cases import rel

D = np.load(os.path.join(os.path.dirname(__file__), "golden", "reference_cases_c.npz"))
TOL = 1e-12


def g(k):
    return D[f"C/{k}"]


@pytest.fixture(scope="module")
def C_case():
    sides = g("cfg/sides").astype(int)
    c = Config(Lx=float(g("cfg/Lx")), Lz=float(g("cfg/Lz")), nx=int(g("cfg/nx")), nz=int(g("cfg/nz")),
               dt=float(g("cfg/dt")), nt=int(g("cfg/nt")), order=int(g("cfg/order")), n_basis_fct=int(g("cfg/nb")),
               fw_nth=int(g("cfg/fw")), f_sample=np.asarray(g("cfg/f_sample"), dtype=np.float64),
               freq_samp=int(g("cfg/fs")), absorb_width=float(g("cfg/width")), absorb_left=int(sides[0]),
               absorb_right=int(sides[1]), absorb_top=int(sides[2]), absorb_bottom=int(sides[3]))
    return c


def _snaps(a, b):
    a = np.asarray(a).reshape(b.shape)
    assert np.mean(a == b) > 0.999
    assert rel(a, b) < 1e-7


def test_case_c_chain(oracle, C_case):
    c = C_case
    i = {k: g(f"in/{k}") for k in ("mu", "rho", "src", "rec", "spec", "sd")}
    assert i["src"].shape == (2, 2) and c.nx != c.nz
    G, Gout, s = oracle.forward1_green(c, i["mu"], i["rho"], i["src"], i["rec"], 1)
    assert rel(G, g("fwd1/G")) < TOL and rel(s, g("fwd1/seis")) < TOL
    _snaps(Gout, g("fwd1/G_out"))
    cs, C = oracle.forward2_correlation(c, i["mu"], i["rho"], g("fwd1/G"), i["spec"], i["sd"], i["rec"], 1)
    assert rel(cs, g("corr/seis")) < TOL
    _snaps(C, g("corr/C_out"))
    rec = i["rec"]
    K1, sf1, _, s1 = oracle.noise_adjoint(c, i["mu"], i["rho"], g("corr/C_out"), g("in2/adstf"), rec, rec, i["spec"],
                                          None, g("fwd1/G"), 1)
    assert rel(K1, g("adj1/K")) < TOL and rel(sf1, g("adj1/stf_fft")) < TOL and rel(s1, g("adj1/seis")) < TOL
    K2, _, _, s2 = oracle.noise_adjoint(c, i["mu"], i["rho"], g("fwd1/G_out"), g("adj1/stf_fft"), rec, rec,
                                        i["spec"], i["sd"], None, 0)
    assert rel(K2, g("adj0/K")) < TOL and rel(s2, g("adj0/seis")) < TOL
