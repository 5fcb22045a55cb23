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
        with np.errstate(invalid="ignore"):  # 0 * inf when the data are zero, as in MATLAB
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


def _nonzero(a) -> bool:
    return a is not None and bool(np.any(np.asarray(a) != 0))


def eval_hessian_vector_product(mu, rho, spectrum, source_dist, ref_stat, array, c_data, t, dmu,
                                source_dist_pert=None, *, cfg, type="structure", veldis="dis",
                                measurement_source="log_amplitude_ratio",
                                measurement_structure="log_amplitude_ratio", weighting=0.5,
                                precision="fp32", device=0, backend: Optional[Backend] = None):
    """Hessian applied to (source_dist_pert, dmu) in parameter space, summed over
    stations: inversion/optlib_callback_fct/eval_hessian_vector_product.m:45-184
    (the chain Green, Born Green, correlation, Born correlation, first- and
    second-order adjoint sources, then the YELLOW mode-13, GRAY mode-11, BLACK
    mode-12 and RED mode-10 adjoint runs).  Born runs consume stored fields every
    step, so the configuration needs fw_nth == 1.  Returns nx-by-nz-by-planes
    FP64 (source planes, then mu)."""
    if type not in ("source", "structure", "joint"):
        raise ValueError("type must be 'source', 'structure' or 'joint'")
    if cfg.fw_nth != 1:
        raise ValueError("the Hessian-vector product needs fw_nth == 1 (Born runs read every step)")
    be = backend or gpu_backend(cfg, precision, device)
    ref_stat = np.asarray(ref_stat, dtype=np.float64).reshape(-1, 2)
    t = np.asarray(t, dtype=np.float64).ravel()
    nt = t.size
    n_ref = ref_stat.shape[0]
    n_rec = np.asarray(array).shape[0] - 1
    c_data = np.asarray(c_data, dtype=np.float64)
    has_dmu = _nonzero(dmu)
    has_ds = _nonzero(source_dist_pert)
    H = None
    for i in range(n_ref):
        src = ref_stat[i:i + 1]
        rec = receivers_of(array, src)
        data = c_data[i * n_rec:(i + 1) * n_rec]
        G_fft, G, _ = be.forward1(mu, rho, src, rec, 1, None, None)
        dG_fft, dG = 0.0, None
        if has_dmu:
            dG_fft, dG, _ = be.forward1(mu, rho, src, rec, 5, dmu, G)
        c_ref, C = be.correlation(mu, rho, G_fft, spectrum, source_dist, rec, 1, None, None)
        c_ref = np.asarray(c_ref).reshape(n_rec, nt)
        c_pert = np.zeros((n_rec, nt))
        dC = None
        if has_dmu:
            c1, dC = be.correlation(mu, rho, dG_fft, spectrum, source_dist, rec, 1, dmu, C)
            c_pert = c_pert + np.asarray(c1).reshape(n_rec, nt)
        if has_ds:
            c2, dC2 = be.correlation(mu, rho, G_fft, spectrum, source_dist_pert, rec, 1, None, None)
            c_pert = c_pert + np.asarray(c2).reshape(n_rec, nt)
            dC = dC2 if dC is None else np.asarray(dC) + np.asarray(dC2)

        def adstf(order):
            _, a_s = be.measure(c_ref, data, c_pert, t, veldis, measurement_source, order)
            _, a_t = be.measure(c_ref, data, c_pert, t, veldis, measurement_structure, order)
            return ((1.0 - weighting) * np.asarray(a_s) + weighting * np.asarray(a_t)).astype(np.complex128)

        a1, a2 = adstf("1st"), adstf("2nd")
        planes = None
        K1 = K2 = K4 = 0.0
        u_dag = None
        if type != "source":
            # YELLOW: u_dagger
            dG_in = dG_fft if has_dmu else None
            K1, uT, u_dag, _ = be.adjoint(mu, rho, dC, a1, rec, None, spectrum, None, dG_in, 13, None, None)
            K1 = np.array(K1, dtype=np.float64)
            if type == "structure":
                K1[:, :, :-1] = 0.0
            p = None
            if has_dmu:  # GRAY: p (dmu dmu)
                K2, _, p, _ = be.adjoint(mu, rho, dG, uT, rec, None, spectrum, source_dist, None, 11, None, None)
                K2 = np.asarray(K2, dtype=np.float64)
            if type == "joint" and has_ds:  # GRAY: p (ds dmu)
                K2b, _, pb, _ = be.adjoint(mu, rho, G, uT, rec, None, spectrum, source_dist_pert, None, 11, None,
                                           None)
                K2 = K2 + np.asarray(K2b, dtype=np.float64)
                p = pb if p is None else np.asarray(p) + np.asarray(pb)
        # BLACK: k
        K3, kT, _, _ = be.adjoint(mu, rho, C, a2, rec, None, spectrum, None, G_fft, 12, dmu if has_dmu else None,
                                  u_dag)
        K3 = np.array(K3, dtype=np.float64)
        if type == "source":
            K3[:, :, -1] = 0.0
        elif type == "structure":
            K3[:, :, :-1] = 0.0
        if type != "source":  # RED: w and l
            K4, _, _, _ = be.adjoint(mu, rho, G, kT, rec, None, spectrum, source_dist, None, 10,
                                     dmu if has_dmu else None, p)
            K4 = np.asarray(K4, dtype=np.float64)
        h = K1 + K2 + K3 + K4
        H = h if H is None else H + h
    return H
