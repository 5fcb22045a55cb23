"""Misfits and adjoint source time functions (FP64, on the GPU).

    [misfit_n, adstf] = make_adjoint_sources(u, u_0, du, t, veldis, measurement,
                                             src, rec, deriv_order)

mirrors tools/measurement/make_adjoint_sources.m:31 (measurements
'log_amplitude_ratio', 'waveform_difference', 'cc_time_shift' -- first order
only, as in the reference -- and 'amplitude_difference').  u, u_0, du are
n_rec-by-nt numpy arrays; the computation runs in libfd2d
(fd2d_make_adjoint_sources).  ``src`` and ``rec`` are accepted for signature
parity; the reference only uses them in commented-out window choices.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib
from .solvers import context

KINDS = {"waveform_difference": _lib.MEAS_WAVEFORM_DIFFERENCE,
         "log_amplitude_ratio": _lib.MEAS_LOG_AMPLITUDE_RATIO,
         "cc_time_shift": _lib.MEAS_CC_TIME_SHIFT,
         "amplitude_difference": _lib.MEAS_AMPLITUDE_DIFFERENCE}


def _pd(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def make_adjoint_sources(u, u_0, du, t, veldis, measurement, src=None, rec=None, deriv_order="1st",
                         device: int = 0):
    if measurement not in KINDS:
        raise ValueError(f"unknown measurement {measurement!r}")
    if deriv_order not in ("1st", "2nd"):
        raise ValueError("deriv_order must be '1st' or '2nd'")
    u = np.asfortranarray(np.array(u, dtype=np.float64, ndmin=2))
    u_0 = np.asfortranarray(np.array(u_0, dtype=np.float64, ndmin=2))
    du = np.asfortranarray(np.array(du, dtype=np.float64, ndmin=2)) if du is not None else np.zeros_like(u)
    t = np.ascontiguousarray(np.asarray(t, dtype=np.float64).ravel())
    n_rec, nt = u.shape
    if u_0.shape != u.shape or du.shape != u.shape or t.size != nt:
        raise ValueError("u, u_0, du must be n_rec-by-nt and t must have nt samples")
    misfit = np.zeros(n_rec)
    adstf = np.zeros((n_rec, nt), order="F")
    ctx = context(device)
    ctx.set_memspace(_lib.MEM_HOST)
    st = ctx.L.fd2d_make_adjoint_sources(ctx.h, KINDS[measurement], 1 if deriv_order == "1st" else 2,
                                         1 if veldis == "vel" else 0, _pd(u), _pd(u_0), _pd(du), n_rec, nt,
                                         _pd(t), _pd(misfit), _pd(adstf))
    _lib.check(st, ctx.h)
    return misfit, adstf
