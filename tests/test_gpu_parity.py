"""GPU parity of the three solvers against the FP64 CPU oracle.

Every call goes through libfd2d's C ABI (host buffers).  Bars: the plain FP64
form agrees with the oracle to <= 1e-10 relative L2 on every output; the FP32
form to <= 1e-4 on correlations, kernels and spectra (the FP32 bound) --
FP32 wavefield snapshots get 1e-4 as well.  Receiver indices and snapshot
schedules are exact: the snapshot stacks of the FP64 form equal the oracle's
single() values except for rare one-ulp rounding-boundary cases.
"""
import numpy as np
import pytest

from tests.problems import media, noise_source, rel_l2, small_cfg, stations

pytestmark = pytest.mark.gpu

TOL = {"fp64": 1e-10, "fp32": 1e-4}
PRECS = ["fp64", "fp32"]


@pytest.fixture(scope="module")
def S(fd2d_lib):
    from fd2d_noise_gb300 import solvers
    return solvers


def _snap_check(gpu, ref, prec):
    assert gpu.shape == ref.shape
    if prec == "fp64":
        # single(v) of values equal to ~1e-15: identical except at rounding ties
        same = np.mean(gpu == ref)
        assert same > 0.999, same
        assert rel_l2(gpu, ref) < 1e-7
    else:
        assert rel_l2(gpu, ref) < TOL[prec]


CFGS = {
    "o4": dict(nx=40, nz=36, nt=60, order=4, K=24, fs=5, fw=1),
    "o2": dict(nx=33, nz=41, nt=50, order=2, K=20, fs=4, fw=1),
    "o8": dict(nx=44, nz=38, nt=56, order=8, K=22, fs=5, fw=1),
}


@pytest.mark.parametrize("prec", PRECS)
@pytest.mark.parametrize("name", list(CFGS))
def test_forward1_green(S, oracle, prec, name):
    cfg = small_cfg(**CFGS[name])
    mu, rho = media(cfg)
    src = stations(cfg, 1, seed=3)
    rec = stations(cfg, 5, seed=4)
    Go, Gout_o, so = oracle.forward1_green(cfg, mu, rho, src, rec, 1)
    G, Gout, s = S.run_forward1_green(mu, rho, src, rec, 1, cfg=cfg, precision=prec)
    assert G.shape == (cfg.nx, cfg.nz, cfg.n_sample)
    assert rel_l2(G, Go) < TOL[prec]
    assert rel_l2(s, so) < TOL[prec]
    _snap_check(Gout, Gout_o, prec)
    # mode 0 returns the MATLAB scalar single(0)
    G0, Gout0, s0 = S.run_forward1_green(mu, rho, src, rec, 0, cfg=cfg, precision=prec)
    assert np.ndim(Gout0) == 0 and Gout0 == 0
    assert rel_l2(G0, Go) < TOL[prec]


@pytest.mark.parametrize("prec", PRECS)
def test_forward1_born(S, oracle, prec):
    cfg = small_cfg(**CFGS["o4"])
    mu, rho = media(cfg)
    dmu = np.asfortranarray(0.03 * mu * np.random.default_rng(7).standard_normal(mu.shape))
    src = stations(cfg, 1, seed=3)
    rec = stations(cfg, 3, seed=4)
    _, G, _ = oracle.forward1_green(cfg, mu, rho, src, rec, 1)
    dGo, dGouto, so = oracle.forward1_green(cfg, mu, rho, src, rec, 5, dmu, G)
    dG, dGout, s = S.run_forward1_green(mu, rho, src, rec, 5, dmu, G, cfg=cfg, precision=prec)
    assert rel_l2(dG, dGo) < TOL[prec]
    assert rel_l2(s, so) < TOL[prec]
    _snap_check(dGout, dGouto, prec)


@pytest.mark.parametrize("prec", PRECS)
@pytest.mark.parametrize("name,nb", [("o4", 0), ("o2", 0), ("o8", 3), ("o4", 4)])
def test_forward2_correlation(S, oracle, prec, name, nb):
    cfg = small_cfg(nb=nb, **CFGS[name])
    mu, rho = media(cfg)
    src = stations(cfg, 1, seed=3)
    rec = stations(cfg, 6, seed=5)
    G, _, _ = oracle.forward1_green(cfg, mu, rho, src, rec, 0)
    spec, sd = noise_source(cfg)
    co, Co = oracle.forward2_correlation(cfg, mu, rho, G, spec, sd, rec, 1)
    c, C = S.run_forward2_correlation(mu, rho, G, spec, sd, rec, 1, cfg=cfg, precision=prec)
    assert c.shape == (6, cfg.ntc)
    assert rel_l2(c, co) < TOL[prec]
    _snap_check(C, Co, prec)


@pytest.mark.parametrize("prec", PRECS)
def test_forward2_correlation_born(S, oracle, prec):
    cfg = small_cfg(**CFGS["o4"])
    mu, rho = media(cfg)
    dmu = np.asfortranarray(0.03 * mu * np.random.default_rng(8).standard_normal(mu.shape))
    src = stations(cfg, 1, seed=3)
    rec = stations(cfg, 4, seed=5)
    G, _, _ = oracle.forward1_green(cfg, mu, rho, src, rec, 0)
    spec, sd = noise_source(cfg)
    _, C = oracle.forward2_correlation(cfg, mu, rho, G, spec, sd, rec, 1)
    co, dCo = oracle.forward2_correlation(cfg, mu, rho, G, spec, sd, rec, 1, dmu, C)
    c, dC = S.run_forward2_correlation(mu, rho, G, spec, sd, rec, 1, dmu, C, cfg=cfg, precision=prec)
    assert rel_l2(c, co) < TOL[prec]
    _snap_check(dC, dCo, prec)


def _adjoint_inputs(cfg, oracle, fw):
    mu, rho = media(cfg)
    src = stations(cfg, 1, seed=3)
    rec = stations(cfg, 4, seed=6)
    G, Gsnap, _ = oracle.forward1_green(cfg, mu, rho, src, rec, 1)
    spec, sd = noise_source(cfg)
    _, C = oracle.forward2_correlation(cfg, mu, rho, G, spec, sd, rec, 1)
    rng = np.random.default_rng(11)
    adstf = rng.standard_normal((rec.shape[0], cfg.ntc)) * 1e-3
    return mu, rho, src, rec, G, Gsnap, spec, sd, C, adstf


@pytest.mark.parametrize("prec", PRECS)
@pytest.mark.parametrize("fw", [1, 5])
def test_adjoint_structure_kernel_chain(S, oracle, prec, fw):
    """eval_objective_and_gradient 'joint' chain: mode 1 with point stfs, then mode 0 with the field stf."""
    cfg = small_cfg(**dict(CFGS["o4"], fw=fw))
    mu, rho, src, rec, G, Gsnap, spec, sd, C, adstf = _adjoint_inputs(cfg, oracle, fw)
    Ko, sfo, _, so = oracle.noise_adjoint(cfg, mu, rho, C, adstf.astype(complex), rec, rec, spec, None, G, 1)
    K, sf, uo, s = S.run_noise_adjoint(mu, rho, C, adstf.astype(complex), rec, rec, spec, None, G, 1,
                                       cfg=cfg, precision=prec)
    assert np.ndim(uo) == 0
    assert rel_l2(K[:, :, 0], Ko[:, :, 0]) < TOL[prec]   # source kernel
    assert rel_l2(K[:, :, 1], Ko[:, :, 1]) < TOL[prec]   # mu kernel
    assert rel_l2(sf, sfo) < TOL[prec]
    assert rel_l2(s, so) < TOL[prec]
    K2o, _, _, s2o = oracle.noise_adjoint(cfg, mu, rho, Gsnap, sfo, rec, rec, spec, sd, None, 0)
    K2, _, _, s2 = S.run_noise_adjoint(mu, rho, Gsnap, sfo, rec, rec, spec, sd, None, 0, cfg=cfg, precision=prec)
    assert rel_l2(K2, K2o) < TOL[prec]
    assert rel_l2(s2, s2o) < TOL[prec]
    # truncation to nt steps (code/run_noise_adjoint.m:165-167): the tail stays zero
    assert np.all(s2[:, cfg.nt:] == 0)


@pytest.mark.parametrize("prec", PRECS)
def test_adjoint_hessian_modes(S, oracle, prec):
    """Modes 13, 11, 12 (Born), 10 (Born) in the order eval_hessian_vector_product runs them."""
    cfg = small_cfg(**CFGS["o4"])
    mu, rho, src, rec, G, Gsnap, spec, sd, C, adstf = _adjoint_inputs(cfg, oracle, 1)
    dmu = np.asfortranarray(0.02 * mu * np.random.default_rng(9).standard_normal(mu.shape))
    a = adstf.astype(complex)
    Ko, uTo, udo, so = oracle.noise_adjoint(cfg, mu, rho, C, a, rec, rec, spec, None, G, 13)
    K, uT, ud, s = S.run_noise_adjoint(mu, rho, C, a, rec, rec, spec, None, G, 13, cfg=cfg, precision=prec)
    assert rel_l2(K, Ko) < TOL[prec] and rel_l2(uT, uTo) < TOL[prec] and rel_l2(s, so) < TOL[prec]
    _snap_check(ud, udo, prec)
    # mode 11: field source from uT, snapshots of the forward field G
    Ko, _, po, so = oracle.noise_adjoint(cfg, mu, rho, Gsnap, uTo, rec, rec, spec, sd, None, 11)
    K, _, p, s = S.run_noise_adjoint(mu, rho, Gsnap, uTo, rec, rec, spec, sd, None, 11, cfg=cfg, precision=prec)
    assert rel_l2(K, Ko) < TOL[prec] and rel_l2(s, so) < TOL[prec]
    _snap_check(p, po, prec)
    # mode 12 with the Born term driven by u_dag
    Ko, kTo, _, so = oracle.noise_adjoint(cfg, mu, rho, C, a, rec, rec, spec, None, G, 12, dmu, udo)
    K, kT, _, s = S.run_noise_adjoint(mu, rho, C, a, rec, rec, spec, None, G, 12, dmu, udo, cfg=cfg, precision=prec)
    assert rel_l2(K, Ko) < TOL[prec] and rel_l2(kT, kTo) < TOL[prec] and rel_l2(s, so) < TOL[prec]
    # mode 10: field source from kT, Born term driven by p
    Ko, _, _, so = oracle.noise_adjoint(cfg, mu, rho, Gsnap, kTo, rec, rec, spec, sd, None, 10, dmu, po)
    K, _, _, s = S.run_noise_adjoint(mu, rho, Gsnap, kTo, rec, rec, spec, sd, None, 10, dmu, po, cfg=cfg, precision=prec)
    assert rel_l2(K, Ko) < TOL[prec] and rel_l2(s, so) < TOL[prec]


@pytest.mark.parametrize("prec", PRECS)
def test_adjoint_basis_functions(S, oracle, prec):
    """Source kernel with n_basis_fct = 3 bands (interpol_matrix' per pixel)."""
    cfg = small_cfg(nb=3, **CFGS["o8"])
    mu, rho, src, rec, G, Gsnap, spec, sd, C, adstf = _adjoint_inputs(cfg, oracle, 1)
    a = adstf.astype(complex)
    Ko, sfo, _, _ = oracle.noise_adjoint(cfg, mu, rho, C, a, rec, rec, spec, None, G, 1)
    K, sf, _, _ = S.run_noise_adjoint(mu, rho, C, a, rec, rec, spec, None, G, 1, cfg=cfg, precision=prec)
    assert K.shape == (cfg.nx, cfg.nz, 4)
    for b in range(4):
        assert rel_l2(K[:, :, b], Ko[:, :, b]) < TOL[prec], b
    assert rel_l2(sf, sfo) < TOL[prec]


def test_errors_match_reference_failures(S):
    from fd2d_noise_gb300 import _lib
    cfg = small_cfg(**CFGS["o4"])
    mu, rho = media(cfg)
    rec = stations(cfg, 2)
    with pytest.raises(_lib.FD2DError) as e:   # Born without enough G_in snapshots
        S.run_forward1_green(mu, rho, rec[:1], rec, 5, mu * 0.01, np.zeros((cfg.nx, cfg.nz, 3), np.float32), cfg=cfg)
    assert e.value.status == 7
    G = np.zeros((cfg.nx, cfg.nz, cfg.n_sample - 1), complex)
    spec, sd = noise_source(cfg)
    with pytest.raises(_lib.FD2DError) as e:   # fewer G planes than frequencies
        S.run_forward2_correlation(mu, rho, G, spec, sd, rec, 0, cfg=cfg)
    assert e.value.status == 7
