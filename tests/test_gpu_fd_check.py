"""Directional derivative of the misfit at the structure-kernel workload's full
size (512x512, nt 2500, snapshots every 5 steps, 200 frequencies, 20
receivers, log-amplitude-ratio measurement) against finite differences, the
methodology of inversion/optlib/optlib_check_derivative_clean.m:17-33: the
mu kernel K of eval_objective_and_gradient predicts dJ = sum(K .* dmu), and
(J(mu + h dmu) - J(mu)) / h must approach it as h falls from 1e-2 to 1e-4.

The plain FP64 GPU form supplies the misfits and the kernel; the FP32 form's
kernel gives the same directional derivative to within 1e-4.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

HS = (1e-2, 1e-3, 1e-4)


def test_structure_gradient_against_finite_differences_at_size(fd2d_lib):
    from tests.test_gpu_fullsize import _structure_problem
    from fd2d_noise_gb300.objective import eval_objective_and_gradient, gpu_backend
    cfg, p = _structure_problem()
    nx = cfg.nx
    X, Z = np.meshgrid(np.linspace(0, cfg.Lx, nx), np.linspace(0, cfg.Lz, nx), indexing="ij")
    # a smooth perturbation across the path between the reference station and
    # the receivers east of it
    dmu = p["mu0"] * 0.05 * np.exp(-((X - 0.62e6) ** 2 + (Z - 0.52e6) ** 2) / 1.2e5 ** 2)

    def run(mu, c_data, prec, only=False):
        return eval_objective_and_gradient(mu, p["rho"], p["spec"], p["sd"], p["ref"], p["arr"], c_data, p["t"],
                                           cfg=cfg, backend=gpu_backend(cfg, prec), weighting=1.0,
                                           only_objective=only, type="structure")

    _, _, c_data = run(p["mu_true"], np.zeros((20, cfg.ntc)), "fp64", only=True)
    j0, g64, _ = run(p["mu0"], c_data, "fp64")
    _, g32, _ = run(p["mu0"], c_data, "fp32")
    pred = float(np.sum(g64[:, :, -1] * dmu))
    pred32 = float(np.sum(g32[:, :, -1] * dmu))
    assert j0 > 0 and pred != 0
    errs = []
    for h in HS:
        j1, _, _ = run(p["mu0"] + h * dmu, c_data, "fp64", only=True)
        fd = (j1 - j0) / h
        errs.append(abs(fd - pred) / abs(fd))
        print(f"h = {h:g}: finite difference {fd:.6e}, kernel {pred:.6e}, relative error {errs[-1]:.3e}")
    d32 = abs(pred32 - pred) / abs(pred)
    print(f"FP32 kernel directional derivative {pred32:.6e}: relative difference to FP64 {d32:.3e}")
    assert errs[-1] < errs[0], errs
    assert errs[-1] < 1e-2, errs
    assert d32 <= 1e-4, d32
