"""The misfit/gradient and Hessian-vector orchestration against the
reference's own inversion/optlib_callback_fct/eval_objective_and_gradient.m,
eval_hessian_vector_product.m and eval_hessian_vector_product_source.m.

tests/golden/objective_cases.npz holds what that file returns when the
MATLAB-subset interpreter runs it (tests/golden/make_golden_objective.py) with
the solvers answered by the FP64 oracle, the reference's own measurement code
(make_adjoint_sources.m), and the model map, gradient map and regularisation
as identities -- the part fd2d_noise_gb300.objective restates.  Two reference
stations, a waveform-difference source measurement and a log-amplitude-ratio
structure measurement mixed 0.7 / 0.3, for the 'source', 'structure' and
'joint' inversion types.  With the same oracle behind it, our orchestration
must call the solvers with the same arguments in the same order: misfit,
gradient and correlations agree to rounding of the measurement sums.
"""
import os

import numpy as np
import pytest

from fd2d_noise_gb300.objective import eval_objective_and_gradient
from tests.test_objective import cfg4, oracle_backend, problem

GOLDEN = np.load(os.path.join(os.path.dirname(__file__), "golden", "objective_cases.npz"))


@pytest.mark.parametrize("typ", ["source", "structure", "joint"])
def test_orchestration_matches_reference(typ):
    cfg = cfg4()
    p = problem(cfg)
    j, g, c = eval_objective_and_gradient(p["mu0"], p["rho"], p["spec"], p["sd"], GOLDEN["ref_stat"], GOLDEN["array"],
                                          GOLDEN["c_data"], GOLDEN["t"], cfg=cfg, type=typ, veldis="dis",
                                          measurement_source="waveform_difference",
                                          measurement_structure="log_amplitude_ratio",
                                          weighting=float(GOLDEN["weighting"]), backend=oracle_backend(cfg))
    jr, gr, cr = GOLDEN[f"{typ}/j"][0], GOLDEN[f"{typ}/g"], GOLDEN[f"{typ}/c_all"]
    assert abs(j - jr) <= 1e-13 * abs(jr)
    assert np.array_equal(c, cr)
    assert g.shape == gr.shape
    for q in range(g.shape[2]):
        n = np.linalg.norm(gr[:, :, q])
        if n == 0:
            assert not np.any(g[:, :, q])
        else:
            assert np.linalg.norm(g[:, :, q] - gr[:, :, q]) <= 1e-12 * n, q


@pytest.mark.parametrize("typ", ["structure", "joint"])
def test_hessian_vector_product_matches_reference(typ):
    """eval_hessian_vector_product.m (Green, Born Green, correlation, Born
    correlations, first- and second-order adjoint sources, adjoint modes 13,
    11, 12 and 10) with its regularisation term set to zero."""
    from fd2d_noise_gb300.objective import eval_hessian_vector_product
    cfg = cfg4(fw=1)
    p = problem(cfg)
    H = eval_hessian_vector_product(p["mu0"], p["rho"], p["spec"], p["sd"], GOLDEN["ref_stat"], GOLDEN["array"],
                                    GOLDEN["c_data"], GOLDEN["t"], GOLDEN["hvp/dmu"],
                                    GOLDEN["hvp/ds"] if typ == "joint" else None, cfg=cfg, type=typ, veldis="dis",
                                    measurement_source="waveform_difference",
                                    measurement_structure="log_amplitude_ratio",
                                    weighting=float(GOLDEN["weighting"]), backend=oracle_backend(cfg))
    Hr = GOLDEN[f"hvp/{typ}/H"]
    assert H.shape == Hr.shape
    for q in range(H.shape[2]):
        n = np.linalg.norm(Hr[:, :, q])
        if n == 0:
            assert not np.any(H[:, :, q])
        else:
            assert np.linalg.norm(H[:, :, q] - Hr[:, :, q]) <= 1e-12 * n, q


def _source_hvp(backend, cfg, p):
    from fd2d_noise_gb300.objective import eval_hessian_vector_product_source
    return eval_hessian_vector_product_source(p["mu0"], p["rho"], p["spec"], p["sd"], GOLDEN["ref_stat"],
                                              GOLDEN["array"], GOLDEN["c_data"], GOLDEN["t"], GOLDEN["hvp/ds"],
                                              cfg=cfg, veldis="dis", measurement_source="waveform_difference",
                                              measurement_structure="log_amplitude_ratio",
                                              weighting=float(GOLDEN["weighting"]), backend=backend)


def _close_planes(H, Hr, tol):
    assert H.shape == Hr.shape
    for q in range(H.shape[2]):
        n = np.linalg.norm(Hr[:, :, q])
        if n == 0:
            assert not np.any(H[:, :, q]), q
        else:
            assert np.linalg.norm(H[:, :, q] - Hr[:, :, q]) <= tol * n, (q, np.linalg.norm(H[:, :, q] - Hr[:, :, q]) / n)


def test_source_hessian_vector_product_matches_reference():
    """eval_hessian_vector_product_source.m (Green function, correlations of
    the reference and the perturbed distribution, second-order adjoint
    sources, adjoint mode 10) on the oracle."""
    cfg = cfg4()
    p = problem(cfg)
    _close_planes(_source_hvp(oracle_backend(cfg), cfg, p), GOLDEN["hvp/source/H"], 1e-12)


@pytest.mark.gpu
@pytest.mark.parametrize("prec,tol", [("fp64", 1e-10), ("fp32", 1e-4)])
def test_gpu_source_hessian_vector_product(fd2d_lib, prec, tol):
    from fd2d_noise_gb300.objective import gpu_backend
    cfg = cfg4()
    p = problem(cfg)
    _close_planes(_source_hvp(gpu_backend(cfg, prec), cfg, p), GOLDEN["hvp/source/H"], tol)
