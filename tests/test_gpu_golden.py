"""GPU solvers against the reference's own outputs (tests/golden): the plain
FP64 form to <= 1e-10 relative L2, the FP32 form to <= 1e-4."""
import pytest

from tests.golden_cases import cfg, group, rel

pytestmark = pytest.mark.gpu
TOL = {"fp64": 1e-10, "fp32": 1e-4}


@pytest.fixture(scope="module")
def S(fd2d_lib):
    from fd2d_noise_gb300 import solvers
    return solvers


@pytest.mark.parametrize("prec", ["fp64", "fp32"])
def test_reference_chain_A(S, prec):
    c = cfg("A")
    i = group("A", "in")
    adstf = group("A", "in2")["adstf"]
    rec = i["rec"]
    ref = group("A", "fwd1")
    G, Gout, s = S.run_forward1_green(i["mu"], i["rho"], i["src"], rec, 1, cfg=c, precision=prec)
    assert rel(G, ref["G"]) < TOL[prec] and rel(s, ref["seis"]) < TOL[prec]
    assert rel(Gout, ref["G_out"]) < (1e-7 if prec == "fp64" else 1e-4)
    ref = group("A", "corr")
    cs, C = S.run_forward2_correlation(i["mu"], i["rho"], group("A", "fwd1")["G"], i["spec"], i["sd"], rec, 1,
                                       cfg=c, precision=prec)
    assert rel(cs, ref["seis"]) < TOL[prec]
    ref = group("A", "adj1")
    K, sf, _, s = S.run_noise_adjoint(i["mu"], i["rho"], group("A", "corr")["C_out"], adstf, rec, rec, i["spec"],
                                      None, group("A", "fwd1")["G"], 1, cfg=c, precision=prec)
    assert rel(K[:, :, 0], ref["K"][:, :, 0]) < TOL[prec]
    assert rel(K[:, :, 1], ref["K"][:, :, 1]) < TOL[prec]
    assert rel(sf, ref["stf_fft"]) < TOL[prec]
    ref = group("A", "adj10")
    K, _, _, s = S.run_noise_adjoint(i["mu"], i["rho"], group("A", "fwd1")["G_out"], group("A", "adj12")["stf_fft"],
                                     rec, rec, i["spec"], i["sd"], None, 10, i["dmu"], group("A", "adj11")["u_out"],
                                     cfg=c, precision=prec)
    assert rel(K, ref["K"]) < TOL[prec] and rel(s, ref["seis"]) < TOL[prec]


@pytest.mark.parametrize("prec", ["fp64", "fp32"])
def test_reference_bands_B(S, prec):
    c = cfg("B")
    i = group("B", "in")
    adstf = group("B", "in2")["adstf"]
    ref = group("B", "corr")
    cs, _ = S.run_forward2_correlation(i["mu"], i["rho"], group("B", "fwd1")["G"], i["spec"], i["sd"], i["rec"], 1,
                                       cfg=c, precision=prec)
    assert rel(cs, ref["seis"]) < TOL[prec]
    ref = group("B", "adj1")
    K, sf, _, _ = S.run_noise_adjoint(i["mu"], i["rho"], group("B", "corr")["C_out"], adstf, i["rec"], i["rec"],
                                      i["spec"], None, group("B", "fwd1")["G"], 1, cfg=c, precision=prec)
    for b in range(4):
        assert rel(K[:, :, b], ref["K"][:, :, b]) < TOL[prec], b
