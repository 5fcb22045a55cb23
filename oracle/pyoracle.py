"""ctypes wrapper of the FP64 CPU oracle (oracle/fd2d_oracle.cpp).

TEST INFRASTRUCTURE: only tests/, ``__graft_entry__.smoke()`` and the CPU
baseline leg of ``bench.py`` use this module, and only as the checker / the CPU
baseline -- never as part of the product path.

The functions mirror the MATLAB signatures of code/run_forward1_green.m:1,
code/run_forward2_correlation.m:1 and code/run_noise_adjoint.m:1 with numpy
arrays in MATLAB (column-major, x fastest) layout.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

from fd2d_noise_gb300.config import (Config, n_fw_corr, n_fw_green, n_kernel_planes)

_HERE = os.path.dirname(os.path.abspath(__file__))
_SO = os.path.join(_HERE, "_build", "libfd2d_oracle.so")
_lib = None

P_D = ctypes.POINTER(ctypes.c_double)
P_F = ctypes.POINTER(ctypes.c_float)
P_I64 = ctypes.POINTER(ctypes.c_int64)


def build(force: bool = False) -> str:
    """Compile the oracle with its Makefile (gcc; no GPU needed)."""
    src = os.path.join(_HERE, "fd2d_oracle.cpp")
    if force or not os.path.exists(_SO) or os.path.getmtime(_SO) < os.path.getmtime(src):
        subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _SO


def lib():
    global _lib
    if _lib is None:
        build()
        _lib = ctypes.CDLL(_SO)
        _lib.oracle_last_error.restype = ctypes.c_char_p
    return _lib


def set_threads(n: int) -> None:
    lib().oracle_set_num_threads(int(n))


def num_threads() -> int:
    return int(lib().oracle_num_threads())


def _d(a):
    if a is None:
        return None
    return a.ctypes.data_as(P_D)


def _f(a):
    if a is None:
        return None
    return a.ctypes.data_as(P_F)


def _as_f64(a):
    if a is None:
        return None
    return np.asfortranarray(np.asarray(a, dtype=np.float64))


def _as_f32(a):
    if a is None:
        return None
    return np.asfortranarray(np.asarray(a, dtype=np.float32))


def _pts(a):
    a = np.zeros((0, 2)) if a is None else np.asarray(a, dtype=np.float64).reshape(-1, 2)
    return np.asfortranarray(a), a.shape[0]


def _check(rc):
    if rc != 0:
        raise RuntimeError(f"oracle error {rc}: {lib().oracle_last_error().decode()}")


def _planes(a):
    if a is None:
        return 0
    return 1 if a.ndim == 2 else a.shape[2]


def stagger_coeffs(order: int) -> np.ndarray:
    out = np.zeros(4)
    _check(lib().oracle_stagger_coeffs(int(order), _d(out)))
    return out[: order // 2].copy()


def setup_arrays(cfg: Config):
    x = np.zeros(cfg.nx)
    z = np.zeros(cfg.nz)
    ab = np.zeros((cfg.nx, cfg.nz), order="F")
    c = cfg.to_c()
    _check(lib().oracle_setup_arrays(ctypes.byref(c), _d(x), _d(z), _d(ab)))
    return x, z, ab


def nearest_indices(cfg: Config, pts):
    p, n = _pts(pts)
    ix = np.zeros(n, dtype=np.int32)
    iz = np.zeros(n, dtype=np.int32)
    c = cfg.to_c()
    _check(lib().oracle_nearest_indices(ctypes.byref(c), _d(p), ctypes.c_int(n),
                                        ix.ctypes.data_as(ctypes.POINTER(ctypes.c_int)),
                                        iz.ctypes.data_as(ctypes.POINTER(ctypes.c_int))))
    return ix, iz


def interpol_matrix(K: int, nb: int) -> np.ndarray:
    ncol = 1 if nb == 0 else nb
    out = np.zeros((K, ncol), order="F")
    _check(lib().oracle_interpol_matrix(ctypes.c_int(K), ctypes.c_int(nb), _d(out)))
    return out


def forward1_green(cfg: Config, mu, rho, src, rec, mode=0, dmu=None, G_in=None):
    """-> (G_fft complex nx-by-nz-by-K, G_out single or None, seismograms nr-by-nt)."""
    mu, rho, dmu = _as_f64(mu), _as_f64(rho), _as_f64(dmu)
    G_in = _as_f32(G_in)
    s, ns = _pts(src)
    r, nr = _pts(rec)
    nx, nz, K = cfg.nx, cfg.nz, cfg.n_sample
    G_re = np.zeros((nx, nz, K), order="F")
    G_im = np.zeros((nx, nz, K), order="F")
    nfw = n_fw_green(cfg)
    G_out = np.zeros((nx, nz, max(nfw, 1)), dtype=np.float32, order="F") if mode != 0 else None
    seis = np.zeros((nr, cfg.nt), order="F")
    c = cfg.to_c()
    rc = lib().oracle_forward1_green(
        ctypes.byref(c), _d(mu), _d(rho), _d(s), ctypes.c_int(ns), _d(r), ctypes.c_int(nr),
        ctypes.c_int(mode), _d(dmu), _f(G_in), ctypes.c_int(_planes(G_in)),
        _d(G_re), _d(G_im), _f(G_out), _d(seis))
    _check(rc)
    return G_re + 1j * G_im, G_out, seis


def forward2_correlation(cfg: Config, mu, rho, G_fft, spectrum, source_dist, rec,
                         mode=0, dmu=None, C_in=None):
    """-> (seismograms nr-by-ntc, C_out single or None)."""
    mu, rho, dmu = _as_f64(mu), _as_f64(rho), _as_f64(dmu)
    C_in = _as_f32(C_in)
    G = np.asarray(G_fft)
    G_re = _as_f64(G.real)
    G_im = _as_f64(G.imag)
    spec = _as_f64(np.asarray(spectrum, dtype=np.float64).reshape(cfg.n_sample, -1))
    sd = _as_f64(source_dist)
    r, nr = _pts(rec)
    nfw = n_fw_corr(cfg)
    seis = np.zeros((nr, cfg.ntc), order="F")
    C_out = np.zeros((cfg.nx, cfg.nz, max(nfw, 1)), dtype=np.float32, order="F") if mode != 0 else None
    c = cfg.to_c()
    rc = lib().oracle_forward2_correlation(
        ctypes.byref(c), _d(mu), _d(rho), _d(G_re), _d(G_im), ctypes.c_int(_planes(G_re)),
        _d(spec), ctypes.c_int(spec.shape[1]), _d(sd), ctypes.c_int(_planes(sd)),
        _d(r), ctypes.c_int(nr), ctypes.c_int(mode), _d(dmu), _f(C_in),
        ctypes.c_int(_planes(C_in)), _d(seis), _f(C_out))
    _check(rc)
    return seis, C_out


def noise_adjoint(cfg: Config, mu, rho, u_fwd, stf, src, rec, spectrum, source_dist, G_fft,
                  mode, dmu=None, u_in=None):
    """-> (K, stf_fft complex, u_out single or None, seismograms nr-by-ntc)."""
    mu, rho, dmu = _as_f64(mu), _as_f64(rho), _as_f64(dmu)
    u_fwd, u_in = _as_f32(u_fwd), _as_f32(u_in)
    if stf is None or np.size(stf) == 0:
        stf_re = stf_im = None
        dims = np.zeros(3, dtype=np.int64)
    else:
        st = np.asarray(stf)
        dims = np.array([st.shape[0], st.shape[1], st.shape[2] if st.ndim == 3 else 1], dtype=np.int64)
        stf_re = _as_f64(st.real)
        stf_im = _as_f64(st.imag) if np.iscomplexobj(st) else None
    s, ns = _pts(src)
    r, nr = _pts(rec)
    spec = None if spectrum is None else _as_f64(np.asarray(spectrum, dtype=np.float64).reshape(cfg.n_sample, -1))
    sd = _as_f64(source_dist)
    if G_fft is None:
        G_re = G_im = None
    else:
        G = np.asarray(G_fft)
        G_re, G_im = _as_f64(G.real), _as_f64(G.imag)
    nx, nz, K = cfg.nx, cfg.nz, cfg.n_sample
    Kout = np.zeros((nx, nz, n_kernel_planes(cfg)), order="F")
    sf_re = np.zeros((nx, nz, K), order="F")
    sf_im = np.zeros((nx, nz, K), order="F")
    nfw = n_fw_corr(cfg)
    u_out = np.zeros((nx, nz, max(nfw, 1)), dtype=np.float32, order="F") if mode in (11, 13) else None
    seis = np.zeros((nr, cfg.ntc), order="F")
    c = cfg.to_c()
    rc = lib().oracle_noise_adjoint(
        ctypes.byref(c), _d(mu), _d(rho), _f(u_fwd), ctypes.c_int(_planes(u_fwd)),
        _d(stf_re), _d(stf_im), dims.ctypes.data_as(P_I64),
        _d(s), ctypes.c_int(ns), _d(r), ctypes.c_int(nr),
        _d(spec), ctypes.c_int(0 if spec is None else spec.shape[1]),
        _d(sd), ctypes.c_int(_planes(sd)),
        _d(G_re), _d(G_im), ctypes.c_int(_planes(G_re)),
        ctypes.c_int(mode), _d(dmu), _f(u_in), ctypes.c_int(_planes(u_in)),
        _d(Kout), _d(sf_re), _d(sf_im), _f(u_out), _d(seis))
    _check(rc)
    return Kout, sf_re + 1j * sf_im, u_out, seis
