"""Pins the CPU oracle to the reference: golden vectors produced by executing
the reference's own MATLAB solvers (tests/golden/make_golden.py) must be
reproduced to round-off (<= 1e-12 relative L2); snapshot stacks, which MATLAB
stores as single, must agree element for element except at rounding ties."""
import numpy as np
import pytest

from tests.golden_cases import cfg, group, rel

TOL = 1e-12


def _snaps(a, b):
    a = np.asarray(a).reshape(b.shape)
    assert np.mean(a == b) > 0.999
    assert rel(a, b) < 1e-7


@pytest.fixture(scope="module")
def A_case(oracle):
    c = cfg("A")
    i = group("A", "in")
    return c, i, group("A", "in2")["adstf"]


def test_forward1(oracle, A_case):
    c, i, _ = A_case
    ref = group("A", "fwd1")
    G, Gout, s = oracle.forward1_green(c, i["mu"], i["rho"], i["src"], i["rec"], 1)
    assert rel(G, ref["G"]) < TOL
    assert rel(s, ref["seis"]) < TOL
    _snaps(Gout, ref["G_out"])
    ref = group("A", "fwd1_born")
    dG, dGout, ds = oracle.forward1_green(c, i["mu"], i["rho"], i["src"], i["rec"], 5, i["dmu"], Gout)
    assert rel(dG, ref["G"]) < TOL
    assert rel(ds, ref["seis"]) < TOL
    _snaps(dGout, ref["G_out"])


def test_correlation(oracle, A_case):
    c, i, _ = A_case
    G = group("A", "fwd1")["G"]
    ref = group("A", "corr")
    s, C = oracle.forward2_correlation(c, i["mu"], i["rho"], G, i["spec"], i["sd"], i["rec"], 1)
    assert rel(s, ref["seis"]) < TOL
    _snaps(C, ref["C_out"])
    ref = group("A", "corr_born")
    s, dC = oracle.forward2_correlation(c, i["mu"], i["rho"], G, i["spec"], i["sd"], i["rec"], 1, i["dmu"],
                                        group("A", "corr")["C_out"])
    assert rel(s, ref["seis"]) < TOL
    _snaps(dC, ref["C_out"])


def test_adjoint_gradient_chain(oracle, A_case):
    c, i, adstf = A_case
    G = group("A", "fwd1")["G"]
    Gout = group("A", "fwd1")["G_out"]
    C = group("A", "corr")["C_out"]
    rec = i["rec"]
    ref = group("A", "adj1")
    K, sf, _, s = oracle.noise_adjoint(c, i["mu"], i["rho"], C, adstf, rec, rec, i["spec"], None, G, 1)
    assert rel(K[:, :, 0], ref["K"][:, :, 0]) < TOL
    assert rel(K[:, :, 1], ref["K"][:, :, 1]) < TOL
    assert rel(sf, ref["stf_fft"]) < TOL
    assert rel(s, ref["seis"]) < TOL
    ref = group("A", "adj0")
    K, _, _, s = oracle.noise_adjoint(c, i["mu"], i["rho"], Gout, group("A", "adj1")["stf_fft"], rec, rec,
                                      i["spec"], i["sd"], None, 0)
    assert rel(K, ref["K"]) < TOL
    assert rel(s, ref["seis"]) < TOL


def test_adjoint_hessian_chain(oracle, A_case):
    c, i, adstf = A_case
    G = group("A", "fwd1")["G"]
    Gout = group("A", "fwd1")["G_out"]
    C = group("A", "corr")["C_out"]
    rec = i["rec"]
    r13 = group("A", "adj13")
    K, uT, ud, s = oracle.noise_adjoint(c, i["mu"], i["rho"], C, adstf, rec, rec, i["spec"], None, G, 13)
    assert rel(K, r13["K"]) < TOL and rel(uT, r13["stf_fft"]) < TOL and rel(s, r13["seis"]) < TOL
    _snaps(ud, r13["u_out"])
    r11 = group("A", "adj11")
    K, _, p, s = oracle.noise_adjoint(c, i["mu"], i["rho"], Gout, r13["stf_fft"], rec, rec, i["spec"], i["sd"],
                                      None, 11)
    assert rel(K, r11["K"]) < TOL and rel(s, r11["seis"]) < TOL
    _snaps(p, r11["u_out"])
    r12 = group("A", "adj12")
    K, kT, _, s = oracle.noise_adjoint(c, i["mu"], i["rho"], C, adstf, rec, rec, i["spec"], None, G, 12,
                                       i["dmu"], r13["u_out"])
    assert rel(K, r12["K"]) < TOL and rel(kT, r12["stf_fft"]) < TOL and rel(s, r12["seis"]) < TOL
    r10 = group("A", "adj10")
    K, _, _, s = oracle.noise_adjoint(c, i["mu"], i["rho"], Gout, r12["stf_fft"], rec, rec, i["spec"], i["sd"],
                                      None, 10, i["dmu"], r11["u_out"])
    assert rel(K, r10["K"]) < TOL and rel(s, r10["seis"]) < TOL


def test_order2_bands(oracle):
    c = cfg("B")
    i = group("B", "in")
    adstf = group("B", "in2")["adstf"]
    ref = group("B", "fwd1")
    G, Gout, s = oracle.forward1_green(c, i["mu"], i["rho"], i["src"], i["rec"], 1)
    assert rel(G, ref["G"]) < TOL and rel(s, ref["seis"]) < TOL
    _snaps(Gout, ref["G_out"])
    ref = group("B", "corr")
    s, C = oracle.forward2_correlation(c, i["mu"], i["rho"], G, i["spec"], i["sd"], i["rec"], 1)
    assert rel(s, ref["seis"]) < TOL
    _snaps(C, ref["C_out"])
    ref = group("B", "adj1")
    K, sf, _, s = oracle.noise_adjoint(c, i["mu"], i["rho"], C, adstf, i["rec"], i["rec"], i["spec"], None, G, 1)
    assert K.shape[2] == 4
    for b in range(4):
        assert rel(K[:, :, b], ref["K"][:, :, b]) < TOL, b
    assert rel(sf, ref["stf_fft"]) < TOL and rel(s, ref["seis"]) < TOL
