"""The three fd2d_noise solvers with the reference's MATLAB signatures.

    [G_fft, G_out, seismograms] = run_forward1_green(mu, rho, src, rec, mode, dmu, G_in)
    [seismograms, C_out] = run_forward2_correlation(mu, rho, G_fft, spectrum,
                                                    source_dist, rec, mode, dmu, C_in)
    [K, stf_fft, u_out, seismograms] = run_noise_adjoint(mu, rho, u_fwd, stf, src, rec,
                                                         spectrum, source_dist, G_fft,
                                                         mode, dmu, u_in)

(code/run_forward1_green.m:1, code/run_forward2_correlation.m:1,
code/run_noise_adjoint.m:1).  Arguments are numpy arrays in MATLAB shape
(nx-by-nz[-by-k]); ``None`` plays the MATLAB empty array.  The configuration the
MATLAB solvers read from input_parameters()/input_interferometry()/absorb_specs()
comes from :mod:`fd2d_noise_gb300.config` (or ``cfg=``).  The ``_mex`` aliases
carry the names the reference's callers use.

Every call goes through libfd2d's C ABI with host buffers (the same entry points
a MATLAB MEX shim binds) and runs on the GPU; ``precision='fp64'`` selects the
plain FP64 form, ``'fp32'`` (default) the FP32 / split-TF32 tensor-core form.
"""
from __future__ import annotations

import contextlib
import ctypes
import threading
from typing import Optional

import numpy as np

from . import _lib
from .config import Config, get_config, n_fw_corr, n_fw_green, n_kernel_planes

_ctx_lock = threading.Lock()
_ctxs: dict = {}
_local = threading.local()


@contextlib.contextmanager
def bound_context(ctx: _lib.Context):
    """Within the block, this thread's solver calls use ``ctx`` (its own stream
    and workspace) instead of the process-wide context."""
    prev = getattr(_local, "ctx", None)
    _local.ctx = ctx
    try:
        yield ctx
    finally:
        _local.ctx = prev


def context(device: int = 0, precision: str = "fp32") -> _lib.Context:
    """The context bound to this thread, else the process-wide context of
    ``device`` (created on first use)."""
    c = getattr(_local, "ctx", None)
    if c is not None:
        c.set_memspace(_lib.MEM_HOST)
        c.set_precision(_prec(precision))
        return c
    with _ctx_lock:
        c = _ctxs.get(device)
        if c is None:
            c = _lib.Context(device, _prec(precision))
            _ctxs[device] = c
        c.set_memspace(_lib.MEM_HOST)
        c.set_precision(_prec(precision))
        return c


def _prec(p) -> int:
    if isinstance(p, int):
        return p
    p = str(p).lower()
    if p in ("fp64", "double", "float64"):
        return _lib.PREC_FP64
    if p in ("fp32", "single", "float32"):
        return _lib.PREC_FP32
    raise ValueError(f"precision must be 'fp32' or 'fp64', not {p!r}")


def _empty(x) -> bool:
    return x is None or np.size(x) == 0


def _f64(x):
    if _empty(x):
        return None
    return np.asfortranarray(np.asarray(x, dtype=np.float64))


def _f32(x):
    if _empty(x):
        return None
    return np.asfortranarray(np.asarray(x, dtype=np.float32))


def _ptr(a):
    return None if a is None else ctypes.c_void_p(a.ctypes.data)


def _planes(a) -> int:
    if a is None:
        return 0
    return 1 if a.ndim <= 2 else int(a.shape[2])


def _points(x):
    if _empty(x):
        return None, 0
    a = np.asfortranarray(np.asarray(x, dtype=np.float64).reshape(-1, 2))
    return a, a.shape[0]


def _complex_planes(x):
    if _empty(x):
        return None, None
    a = np.asarray(x)
    re = np.asfortranarray(a.real, dtype=np.float64)
    im = np.asfortranarray(a.imag, dtype=np.float64) if np.iscomplexobj(a) else np.zeros_like(re, order="F")
    return re, im


def _grid(a, cfg: Config, name: str):
    if a is not None and a.size % cfg.npts:
        raise ValueError(f"{name} has {a.size} elements, not a multiple of nx*nz = {cfg.npts}")
    if a is not None and a.ndim < 3:
        a = np.asfortranarray(a.reshape(cfg.nx, cfg.nz, -1, order="F"))
    return a


def run_forward1_green(mu, rho, src, rec, mode=0, dmu=None, G_in=None, *,
                       cfg: Optional[Config] = None, precision="fp32", device: int = 0):
    """Green function of the reference station (code/run_forward1_green.m).

    Returns ``(G_fft, G_out, seismograms)``: the conjugated on-the-fly DFT of the
    velocity (nx-by-nz-by-n_sample complex), the single-precision wavefield
    snapshots (``np.float32(0)`` when ``mode == 0``) and the receiver velocities
    (nr-by-nt).
    """
    cfg = get_config(cfg)
    ctx = context(device, precision)
    nx, nz, K = cfg.nx, cfg.nz, cfg.n_sample
    mu = _f64(mu).reshape(nx, nz, order="F")
    rho = _f64(rho).reshape(nx, nz, order="F")
    dmu = _f64(dmu)
    G_in = _grid(_f32(G_in), cfg, "G_in")
    s, ns = _points(src)
    r, nr = _points(rec)
    G_re = np.empty((nx, nz, K), order="F")
    G_im = np.empty((nx, nz, K), order="F")
    nfw = n_fw_green(cfg)
    G_out = np.empty((nx, nz, nfw), dtype=np.float32, order="F") if (mode != 0 and nfw > 0) else None
    seis = np.empty((nr, cfg.nt), order="F")
    c = cfg.to_c()
    st = ctx.L.fd2d_forward1_green(
        ctx.h, ctypes.byref(c), _ptr(mu), _ptr(rho), _ptr(s), ns, _ptr(r), nr, int(mode),
        _ptr(dmu), _ptr(G_in), _planes(G_in), _ptr(G_re), _ptr(G_im), _ptr(G_out), _ptr(seis))
    _lib.check(st, ctx.h)
    G_fft = G_re + 1j * G_im
    if G_out is None:
        G_out = np.float32(0.0) if mode == 0 else np.zeros((nx, nz, 0), dtype=np.float32)
    return G_fft, G_out, seis


def run_forward2_correlation(mu, rho, G_fft, spectrum, source_dist, rec, mode=0, dmu=None,
                             C_in=None, *, cfg: Optional[Config] = None, precision="fp32",
                             device: int = 0):
    """Correlation wavefield (code/run_forward2_correlation.m).

    Returns ``(seismograms, C_out)``: the displacement at the receivers over
    t = -(nt-1)dt..(nt-1)dt (the correlations, nr-by-(2nt-1)) and the single
    snapshots of u (``np.float32(0)`` when ``mode == 0``).
    """
    cfg = get_config(cfg)
    ctx = context(device, precision)
    nx, nz, K = cfg.nx, cfg.nz, cfg.n_sample
    mu = _f64(mu).reshape(nx, nz, order="F")
    rho = _f64(rho).reshape(nx, nz, order="F")
    dmu = _f64(dmu)
    G_re, G_im = _complex_planes(G_fft)
    G_re, G_im = _grid(G_re, cfg, "G_fft"), _grid(G_im, cfg, "G_fft")
    spec = _f64(np.asarray(spectrum, dtype=np.float64).reshape(K, -1, order="F"))
    sd = _grid(_f64(source_dist), cfg, "source_dist")
    C_in = _grid(_f32(C_in), cfg, "C_in")
    r, nr = _points(rec)
    nfw = n_fw_corr(cfg)
    seis = np.empty((nr, cfg.ntc), order="F")
    C_out = np.empty((nx, nz, nfw), dtype=np.float32, order="F") if (mode != 0 and nfw > 0) else None
    c = cfg.to_c()
    st = ctx.L.fd2d_forward2_correlation(
        ctx.h, ctypes.byref(c), _ptr(mu), _ptr(rho), _ptr(G_re), _ptr(G_im), _planes(G_re),
        _ptr(spec), spec.shape[1], _ptr(sd), _planes(sd), _ptr(r), nr, int(mode), _ptr(dmu),
        _ptr(C_in), _planes(C_in), _ptr(seis), _ptr(C_out))
    _lib.check(st, ctx.h)
    if C_out is None:
        C_out = np.float32(0.0) if mode == 0 else np.zeros((nx, nz, 0), dtype=np.float32)
    return seis, C_out


def run_noise_adjoint(mu, rho, u_fwd, stf, src, rec, spectrum, source_dist, G_fft, mode,
                      dmu=None, u_in=None, *, cfg: Optional[Config] = None, precision="fp32",
                      device: int = 0):
    """Adjoint wavefield and kernels (code/run_noise_adjoint.m).

    Returns ``(K, stf_fft, u_out, seismograms)``: the kernels (source-kernel
    planes then the mu kernel, nx-by-nz-by-(n_basis_fct+1) or -by-2), the DFT of
    the adjoint displacement (modes 1, 12, 13), the single snapshots of u (modes
    11, 13; ``np.float32(0)`` otherwise) and the receiver displacements.
    """
    cfg = get_config(cfg)
    ctx = context(device, precision)
    nx, nz, K = cfg.nx, cfg.nz, cfg.n_sample
    mu = _f64(mu).reshape(nx, nz, order="F")
    rho = _f64(rho).reshape(nx, nz, order="F")
    dmu = _f64(dmu)
    u_fwd = _grid(_f32(u_fwd), cfg, "u_fwd")
    u_in = _grid(_f32(u_in), cfg, "u_in")
    if _empty(stf):
        stf_re = stf_im = None
        dims = (ctypes.c_int64 * 3)(0, 0, 0)
    else:
        st_a = np.asarray(stf)
        shape = st_a.shape if st_a.ndim == 3 else (st_a.shape[0], st_a.shape[1] if st_a.ndim > 1 else 1, 1)
        dims = (ctypes.c_int64 * 3)(*[int(v) for v in shape])
        stf_re, stf_im = _complex_planes(st_a)
    s, ns = _points(src)
    r, nr = _points(rec)
    spec = None if _empty(spectrum) else _f64(np.asarray(spectrum, dtype=np.float64).reshape(K, -1, order="F"))
    sd = _grid(_f64(source_dist), cfg, "source_dist")
    if _empty(G_fft):
        G_re = G_im = None
    else:
        G_re, G_im = _complex_planes(G_fft)
        G_re, G_im = _grid(G_re, cfg, "G_fft"), _grid(G_im, cfg, "G_fft")
    Kout = np.empty((nx, nz, n_kernel_planes(cfg)), order="F")
    sf_re = np.empty((nx, nz, K), order="F")
    sf_im = np.empty((nx, nz, K), order="F")
    nfw = n_fw_corr(cfg)
    u_out = np.empty((nx, nz, nfw), dtype=np.float32, order="F") if (mode in (11, 13) and nfw > 0) else None
    seis = np.empty((nr, cfg.ntc), order="F")
    c = cfg.to_c()
    st = ctx.L.fd2d_noise_adjoint(
        ctx.h, ctypes.byref(c), _ptr(mu), _ptr(rho), _ptr(u_fwd), _planes(u_fwd),
        _ptr(stf_re), _ptr(stf_im), dims, _ptr(s), ns, _ptr(r), nr,
        _ptr(spec), 0 if spec is None else spec.shape[1], _ptr(sd), _planes(sd),
        _ptr(G_re), _ptr(G_im), _planes(G_re), int(mode), _ptr(dmu), _ptr(u_in), _planes(u_in),
        _ptr(Kout), _ptr(sf_re), _ptr(sf_im), _ptr(u_out), _ptr(seis))
    _lib.check(st, ctx.h)
    if u_out is None:
        u_out = np.float32(0.0) if mode not in (11, 13) else np.zeros((nx, nz, 0), dtype=np.float32)
    return Kout, sf_re + 1j * sf_im, u_out, seis


# Names under which the reference's callers reach the solvers
# (code/calculate_data.m:195,198; inversion/optlib_callback_fct/eval_*.m).
run_forward1_green_mex = run_forward1_green
run_forward2_correlation_mex = run_forward2_correlation
run_noise_adjoint_mex = run_noise_adjoint
