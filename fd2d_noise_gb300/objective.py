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
    session: object = None


def gpu_backend(cfg, precision: str = "fp32", device: int = 0) -> Backend:
    from . import measurements, solvers
    kw = dict(cfg=cfg, precision=precision, device=device)
    return Backend(
        forward1=lambda *a: solvers.run_forward1_green(*a, **kw),
        correlation=lambda *a: solvers.run_forward2_correlation(*a, **kw),
        adjoint=lambda *a: solvers.run_noise_adjoint(*a, **kw),
        measure=lambda u, u0, du, t, vd, m, order: measurements.make_adjoint_sources(
            u, u0, du, t, vd, m, None, None, order, device=device))


class DeviceSpectrum:
    """A complex nx-by-nz-by-K spectrum kept on the device as real and
    imaginary FP64 planes (flat tensors in MATLAB order)."""

    def __init__(self, re, im, planes: int):
        self.re, self.im, self.planes = re, im, planes


def device_backend(cfg, precision: str = "fp32", device: int = 0, ctx=None) -> Backend:
    """Solvers in device memspace: spectra and snapshot stacks stay on the GPU
    between the runs of a station (DeviceSpectrum and float32 tensors); models,
    positions and traces cross as numpy arrays."""
    import torch
    from . import measurements
    from .config import n_fw_corr, n_fw_green, n_kernel_planes
    from .device import DeviceSession, to_device
    sess = DeviceSession(cfg, device, precision, ctx=ctx)
    np_, K, nt, ntc = cfg.npts, cfg.n_sample, cfg.nt, cfg.ntc
    keep = {}

    def up(a):
        if a is None or isinstance(a, torch.Tensor):
            return a
        key = id(a)
        if key not in keep:
            keep[key] = (a, to_device(np.asarray(a, dtype=np.float64), np.float64, device))
        return keep[key][1]

    def pts(a):
        if a is None or np.size(a) == 0:
            return None, 0
        a = np.asarray(a, dtype=np.float64).reshape(-1, 2)
        return to_device(a, np.float64, device), a.shape[0]

    def planes(x):
        return 0 if x is None else x.numel() // np_

    def host(tns, shape):
        sess.ctx.synchronize()
        return tns.cpu().numpy().reshape(shape, order="F")

    def forward1(mu, rho, src, rec, mode, dmu, G_in):
        s, ns = pts(src)
        r, nr = pts(rec)
        G_re, G_im = sess.zeros(np_ * K, torch.float64), sess.zeros(np_ * K, torch.float64)
        G_out = sess.zeros(np_ * n_fw_green(cfg), torch.float32) if mode else None
        seis = sess.zeros(max(nr, 1) * nt, torch.float64)
        sess.forward1_green(up(mu), up(rho), s, ns, r, nr, G_re, G_im, seis, mode, G_out, up(dmu), G_in,
                            planes(G_in))
        return DeviceSpectrum(G_re, G_im, K), G_out, host(seis, (max(nr, 1), nt))

    def correlation(mu, rho, G_fft, spectrum, source_dist, rec, mode, dmu, C_in):
        r, nr = pts(rec)
        spec = np.asarray(spectrum, dtype=np.float64).reshape(K, -1, order="F")
        seis = sess.zeros(max(nr, 1) * ntc, torch.float64)
        C_out = sess.zeros(np_ * n_fw_corr(cfg), torch.float32) if mode else None
        sess.forward2_correlation(up(mu), up(rho), G_fft.re, G_fft.im, up(spec), spec.shape[1], up(source_dist),
                                  np.size(source_dist) // np_, r, nr, seis, mode, C_out, up(dmu), C_in,
                                  planes(C_in))
        return host(seis, (max(nr, 1), ntc)), C_out

    def adjoint(mu, rho, u_fwd, stf, src, rec, spectrum, source_dist, G_fft, mode, dmu, u_in):
        s, ns = pts(src)
        r, nr = pts(rec)
        if isinstance(stf, DeviceSpectrum):
            stf_re, stf_im, dims = stf.re, stf.im, (cfg.nx, cfg.nz, stf.planes)
        elif stf is None or np.size(stf) == 0:
            stf_re = stf_im = None
            dims = (0, 0, 0)
        else:
            st = np.asarray(stf)
            stf_re, stf_im = up(np.ascontiguousarray(st.real)), up(np.ascontiguousarray(st.imag))
            dims = (st.shape[0], st.shape[1], 1)
        spec = None if spectrum is None else np.asarray(spectrum, dtype=np.float64).reshape(K, -1, order="F")
        Kp = n_kernel_planes(cfg)
        Kout = sess.zeros(np_ * Kp, torch.float64)
        sf_re, sf_im = sess.zeros(np_ * K, torch.float64), sess.zeros(np_ * K, torch.float64)
        u_out = sess.zeros(np_ * n_fw_corr(cfg), torch.float32) if mode in (11, 13) else None
        seis = sess.zeros(max(nr, 1) * ntc, torch.float64)
        G_re = G_fft.re if G_fft is not None else None
        G_im = G_fft.im if G_fft is not None else None
        sess.noise_adjoint(up(mu), up(rho), u_fwd, planes(u_fwd), stf_re, stf_im, dims, s, ns, r, nr, up(spec),
                           0 if spec is None else spec.shape[1], up(source_dist),
                           0 if source_dist is None else np.size(source_dist) // np_, G_re, G_im,
                           0 if G_fft is None else G_fft.planes, mode, Kout, sf_re, sf_im, seis, u_out,
                           up(dmu), u_in, planes(u_in))
        return host(Kout, (cfg.nx, cfg.nz, Kp)), DeviceSpectrum(sf_re, sf_im, K), u_out, None

    def measure(u, u0, du, t, vd, m, order):
        return measurements.make_adjoint_sources(u, u0, du, t, vd, m, None, None, order, device=device)

    be = Backend(forward1=forward1, correlation=correlation, adjoint=adjoint, measure=measure)
    be.session = sess
    return be


def _sum(a, b):
    """a + b for device tensors or host arrays (stored fields of Born runs)."""
    return b if a is None else a + b


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
    be = backend or device_backend(cfg, precision, device)
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


def eval_hessian_vector_product_source(mu, rho, spectrum, source_dist, ref_stat, array, c_data, t,
                                       source_dist_pert, *, cfg, veldis="dis",
                                       measurement_source="log_amplitude_ratio",
                                       measurement_structure="log_amplitude_ratio", weighting=0.5,
                                       precision="fp32", device=0, backend: Optional[Backend] = None):
    """Hessian of the 'source' inversion applied to a perturbation of the noise
    distribution, summed over stations:
    inversion/optlib_callback_fct/eval_hessian_vector_product_source.m:40-100 --
    per station the Green function (no receivers), the correlations of the
    reference distribution (zero when both measurements are waveform
    differences, :60-72) and of the perturbation, the second-order adjoint
    sources of both measurements mixed by the weighting, and one adjoint run in
    mode 10 with the spectrum and the Green function (the source kernel of the
    second-order adjoint field).  Returns nx-by-nz-by-planes FP64 (source
    planes, then mu)."""
    be = backend or device_backend(cfg, precision, device)
    ref_stat = np.asarray(ref_stat, dtype=np.float64).reshape(-1, 2)
    t = np.asarray(t, dtype=np.float64).ravel()
    nt = t.size
    n_rec = np.asarray(array).shape[0] - 1
    c_data = np.asarray(c_data, dtype=np.float64)
    both_wd = measurement_source == "waveform_difference" and measurement_structure == "waveform_difference"
    H = None
    for i in range(ref_stat.shape[0]):
        src = ref_stat[i:i + 1]
        rec = receivers_of(array, src)
        data = c_data[i * n_rec:(i + 1) * n_rec]
        G_fft, _, _ = be.forward1(mu, rho, src, np.zeros((0, 2)), 0, None, None)
        if both_wd:
            c_ref = 0.0 * data
        else:
            c_ref, _ = be.correlation(mu, rho, G_fft, spectrum, source_dist, rec, 0, None, None)
            c_ref = np.asarray(c_ref).reshape(n_rec, nt)
        c_pert, _ = be.correlation(mu, rho, G_fft, spectrum, source_dist_pert, rec, 0, None, None)
        c_pert = np.asarray(c_pert).reshape(n_rec, nt)
        _, a_s = be.measure(c_ref, data, c_pert, t, veldis, measurement_source, "2nd")
        _, a_t = be.measure(c_ref, data, c_pert, t, veldis, measurement_structure, "2nd")
        a2 = ((1.0 - weighting) * np.asarray(a_s) + weighting * np.asarray(a_t)).astype(np.complex128)
        h, _, _, _ = be.adjoint(mu, rho, None, a2, rec, None, spectrum, None, G_fft, 10, None, None)
        h = np.asarray(h, dtype=np.float64)
        H = h if H is None else H + h
    return H


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
    be = backend or device_backend(cfg, precision, device)
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
            dC = _sum(dC, dC2)

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
                p = _sum(p, pb)
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
