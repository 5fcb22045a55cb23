"""Misfit and gradient of the noise-correlation inversion (per reference station).

    [j, grad_parameters, c_all] = eval_objective_and_gradient(...)

follows inversion/optlib_callback_fct/eval_objective_and_gradient.m:24-122 for
the solver part: for every reference station the Green function and the
correlation wavefield (snapshots stored when kernels are wanted), the misfit and
adjoint sources of both measurements weighted by ``weighting`` (:76-82), and
the adjoint runs of the chosen inversion type (:88-107):

    'source'    K = run_noise_adjoint(mu, rho, [], adstf, rec, [], spectrum, [], G_fft, 0)
    'structure' [K1, S] = run_noise_adjoint(mu, rho, C, adstf, rec, [], [], [], [], 1)
                K2 = run_noise_adjoint(mu, rho, G, S, rec, [], spectrum, source_dist, [], 0)
    'joint'     as 'structure' with spectrum and G_fft in the first run (source kernel)

and ``grad_parameters = sum over stations of K1 + K2`` (:110), i.e. the source
kernel planes followed by the mu kernel.  The model map (map_m_to_parameters),
gradient smoothing and regularisation around it are not part of the path.

The solvers and the measurement run in libfd2d on the GPU (``precision``
selects the FP32 or the plain FP64 form; kernels accumulate in FP64 on the
device, and the station sum here is FP64).  ``backend`` replaces the four
calls, e.g. by the CPU oracle in tests.
"""
from __future__ import annotations

from dataclasses import dataclass
from typing import Callable, Optional

import numpy as np


@dataclass
class Backend:
    forward1: Callable
    correlation: Callable
    adjoint: Callable
    measure: Callable


def gpu_backend(cfg, precision: str = "fp32", device: int = 0) -> Backend:
    from . import measurements, solvers
    kw = dict(cfg=cfg, precision=precision, device=device)
    return Backend(
        forward1=lambda *a: solvers.run_forward1_green(*a, **kw),
        correlation=lambda *a: solvers.run_forward2_correlation(*a, **kw),
        adjoint=lambda *a: solvers.run_noise_adjoint(*a, **kw),
        measure=lambda u, u0, du, t, vd, m, order: measurements.make_adjoint_sources(
            u, u0, du, t, vd, m, None, None, order, device=device))


def receivers_of(array, src):
    """array rows that are not the source: find(~ismember(array, src, 'rows'))."""
    a = np.asarray(array, dtype=np.float64)
    keep = ~np.all(a == np.asarray(src, dtype=np.float64).reshape(1, 2), axis=1)
    return a[keep]


def eval_objective_and_gradient(mu, rho, spectrum, source_dist, ref_stat, array, c_data, t, *, cfg,
                                type="structure", veldis="dis", measurement_source="log_amplitude_ratio",
                                measurement_structure="log_amplitude_ratio", weighting=0.5,
                                only_objective=False, precision="fp32", device=0,
                                backend: Optional[Backend] = None):
    """Returns (j, grad_parameters nx-by-nz-by-planes FP64 (None when
    only_objective), c_all n_ref*n_rec-by-nt)."""
    if type not in ("source", "structure", "joint"):
        raise ValueError("type must be 'source', 'structure' or 'joint'")
    be = backend or gpu_backend(cfg, precision, device)
    ref_stat = np.asarray(ref_stat, dtype=np.float64).reshape(-1, 2)
    t = np.asarray(t, dtype=np.float64).ravel()
    nt = t.size
    n_ref = ref_stat.shape[0]
    n_rec = np.asarray(array).shape[0] - 1
    c_data = np.asarray(c_data, dtype=np.float64)
    c_all = np.zeros((n_ref * n_rec, nt))
    grad = None
    j = 0.0
    for i in range(n_ref):
        src = ref_stat[i:i + 1]
        rec = receivers_of(array, src)
        store = 0 if type == "source" else 1
        G_fft, G, _ = be.forward1(mu, rho, src, rec, store, None, None)
        c, C = be.correlation(mu, rho, G_fft, spectrum, source_dist, rec, store, None, None)
        c = np.asarray(c).reshape(n_rec, nt)
        c_all[i * n_rec:(i + 1) * n_rec] = c
        c_ref = c_data[i * n_rec:(i + 1) * n_rec]
        zero = 0.0 * c_ref
        j_s, ad_s = be.measure(c, c_ref, zero, t, veldis, measurement_source, "1st")
        j_t, ad_t = be.measure(c, c_ref, zero, t, veldis, measurement_structure, "1st")
        j_n = (1.0 - weighting) * np.asarray(j_s) + weighting * np.asarray(j_t)
        adstf = (1.0 - weighting) * np.asarray(ad_s) + weighting * np.asarray(ad_t)
        j += float(np.sum(j_n))
        if only_objective:
            continue
        if type == "source":
            K1, _, _, _ = be.adjoint(mu, rho, None, adstf.astype(np.complex128), rec, None, spectrum, None,
                                     G_fft, 0, None, None)
            K2 = 0.0 * np.asarray(K1)
        elif type == "structure":
            K1, S, _, _ = be.adjoint(mu, rho, C, adstf.astype(np.complex128), rec, None, None, None, None, 1,
                                     None, None)
            K2, _, _, _ = be.adjoint(mu, rho, G, S, rec, None, spectrum, source_dist, None, 0, None, None)
        else:
            K1, S, _, _ = be.adjoint(mu, rho, C, adstf.astype(np.complex128), rec, None, spectrum, None, G_fft,
                                     1, None, None)
            K2, _, _, _ = be.adjoint(mu, rho, G, S, rec, None, spectrum, source_dist, None, 0, None, None)
        k = np.asarray(K1, dtype=np.float64) + np.asarray(K2, dtype=np.float64)
        grad = k if grad is None else grad + k
    return j, grad, c_all
