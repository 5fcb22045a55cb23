"""Device-resident use of the solvers (torch CUDA tensors, asynchronous calls).

A :class:`DeviceSession` owns an ``fd2d_ctx`` in device memspace bound to
torch's current CUDA stream, so solves queue on the stream torch uses and
``torch.cuda.Event`` timing sees them.  Arrays are flat tensors in MATLAB
element order (column-major, x fastest); :func:`to_device` converts numpy
arrays in MATLAB shape.  Spectra stay as separate real / imaginary FP64 planes.
"""
from __future__ import annotations

import ctypes
from typing import Optional

import numpy as np

from . import _lib
from .config import Config, n_fw_corr, n_fw_green, n_kernel_planes


def to_device(a, dtype=None, device: int = 0):
    import torch
    a = np.asarray(a)
    if dtype is not None:
        a = a.astype(dtype, copy=False)
    flat = np.ascontiguousarray(a.ravel(order="F"))
    return torch.from_numpy(flat).to(f"cuda:{device}")


def to_host(t, shape) -> np.ndarray:
    return t.detach().cpu().numpy().reshape(shape, order="F")


def _p(t) -> Optional[ctypes.c_void_p]:
    return None if t is None else ctypes.c_void_p(t.data_ptr())


class DeviceSession:
    def __init__(self, cfg: Config, device: int = 0, precision: str = "fp32", ctx: Optional[_lib.Context] = None):
        """``ctx``: an existing context to use (switched to device memspace and
        this session's stream); otherwise the session creates its own."""
        import torch
        from .solvers import _prec
        self.torch = torch
        self.cfg = cfg
        self.device = device
        self.ctx = ctx if ctx is not None else _lib.Context(device, _prec(precision))
        self.ctx.set_precision(_prec(precision))
        self.ctx.set_memspace(_lib.MEM_DEVICE)
        # time loops are captured as CUDA graphs, which the legacy default
        # stream does not allow: work on torch's current stream unless that is
        # the default one, else on a stream of our own.
        cur = torch.cuda.current_stream(device)
        self.stream = cur if cur.cuda_stream != 0 else torch.cuda.Stream(device)
        self.ctx.set_stream(self.stream.cuda_stream)
        self.c = cfg.to_c()

    def set_precision(self, precision: str):
        from .solvers import _prec
        self.ctx.set_precision(_prec(precision))

    def zeros(self, n, dtype):
        # filled on the session's stream, so the fill is ordered before the
        # library's work on the buffer
        with self.torch.cuda.stream(self.stream):
            return self.torch.zeros(int(n), dtype=dtype, device=f"cuda:{self.device}")

    def green_outputs(self, nr: int, mode: int = 0):
        t = self.torch
        cfg = self.cfg
        np_, K = cfg.npts, cfg.n_sample
        G_re = self.zeros(np_ * K, t.float64)
        G_im = self.zeros(np_ * K, t.float64)
        G_out = self.zeros(np_ * n_fw_green(cfg), t.float32) if mode else None
        seis = self.zeros(max(nr, 1) * cfg.nt, t.float64)
        return G_re, G_im, G_out, seis

    def forward1_green(self, mu, rho, src, ns, rec, nr, G_re, G_im, seis, mode=0, G_out=None,
                       dmu=None, G_in=None, n_G_in=0):
        self.ctx.set_memspace(_lib.MEM_DEVICE)  # the context may be shared with host-memspace calls
        st = self.ctx.L.fd2d_forward1_green(
            self.ctx.h, ctypes.byref(self.c), _p(mu), _p(rho), _p(src), int(ns), _p(rec), int(nr),
            int(mode), _p(dmu), _p(G_in), int(n_G_in), _p(G_re), _p(G_im), _p(G_out), _p(seis))
        _lib.check(st, self.ctx.h)

    def forward2_correlation(self, mu, rho, G_re, G_im, spectrum, n_src, source_dist, n_dist,
                             rec, nr, seis, mode=0, C_out=None, dmu=None, C_in=None, n_C_in=0):
        self.ctx.set_memspace(_lib.MEM_DEVICE)  # the context may be shared with host-memspace calls
        st = self.ctx.L.fd2d_forward2_correlation(
            self.ctx.h, ctypes.byref(self.c), _p(mu), _p(rho), _p(G_re), _p(G_im),
            int(self.cfg.n_sample), _p(spectrum), int(n_src), _p(source_dist), int(n_dist),
            _p(rec), int(nr), int(mode), _p(dmu), _p(C_in), int(n_C_in), _p(seis), _p(C_out))
        _lib.check(st, self.ctx.h)

    def noise_adjoint(self, mu, rho, u_fwd, n_u_fwd, stf_re, stf_im, stf_dims, src, ns, rec, nr,
                      spectrum, n_src, source_dist, n_dist, G_re, G_im, n_G, mode, K, sf_re, sf_im,
                      seis, u_out=None, dmu=None, u_in=None, n_u_in=0):
        self.ctx.set_memspace(_lib.MEM_DEVICE)  # the context may be shared with host-memspace calls
        dims = (ctypes.c_int64 * 3)(*[int(v) for v in stf_dims])
        st = self.ctx.L.fd2d_noise_adjoint(
            self.ctx.h, ctypes.byref(self.c), _p(mu), _p(rho), _p(u_fwd), int(n_u_fwd),
            _p(stf_re), _p(stf_im), dims, _p(src), int(ns), _p(rec), int(nr), _p(spectrum),
            int(n_src), _p(source_dist), int(n_dist), _p(G_re), _p(G_im), int(n_G), int(mode),
            _p(dmu), _p(u_in), int(n_u_in), _p(K), _p(sf_re), _p(sf_im), _p(u_out), _p(seis))
        _lib.check(st, self.ctx.h)

    def correlation_batch(self, jobs):
        """Runs fd2d_correlation_batch.  ``jobs``: list of dicts with keys cfg (Config),
        mu, rho, spectrum, n_src, source_dist, n_dist, src, rec, nr, out (tensors)."""
        self.ctx.set_memspace(_lib.MEM_DEVICE)
        arr = (_lib.FD2DJob * len(jobs))()
        keep = []
        for j, d in enumerate(jobs):
            c = d["cfg"].to_c()
            keep.append(c)
            arr[j].cfg = ctypes.pointer(c)
            arr[j].mu, arr[j].rho = d["mu"].data_ptr(), d["rho"].data_ptr()
            arr[j].spectrum, arr[j].n_noise_sources = d["spectrum"].data_ptr(), int(d.get("n_src", 1))
            arr[j].source_dist, arr[j].n_dist = d["source_dist"].data_ptr(), int(d.get("n_dist", 1))
            arr[j].src, arr[j].rec, arr[j].nr = d["src"].data_ptr(), d["rec"].data_ptr(), int(d["nr"])
            arr[j].correlations = d["out"].data_ptr()
        _lib.check(self.ctx.L.fd2d_correlation_batch(self.ctx.h, arr, len(jobs)), self.ctx.h)

    def kernel_planes(self) -> int:
        return n_kernel_planes(self.cfg)

    def corr_snapshots(self) -> int:
        return n_fw_corr(self.cfg)
