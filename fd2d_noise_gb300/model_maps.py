"""Model-space maps of the inversion with Gaussian smoothing on the GPU.

    m_parameters = map_m_to_parameters(m, ...)            map_m_to_parameters.m:15-52
    m            = map_parameters_to_m(m_parameters, ...) map_parameters_to_m.m:15-20
    grad_m       = map_gradparameters_to_gradm(g, ...)    map_gradparameters_to_gradm.m:20-57
    GY           = gaussblur2d(Y, x1, x2, sigma)          tools/addons/gaussblur2d.m:2-38

(inversion/optlib_callback_fct/).  The smoothing runs in libfd2d
(fd2d_gaussblur2d, FP64); the parameters of the reference's ``usr_par`` struct
are explicit arguments.  The smoothing acts on the interior where the taper is
1 (``find(absbound == 1, 1, 'first')``), as in the reference.  The 'ring'
parameterisation of the reference (imfilter on a ring mask) is not provided.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib
from .solvers import context


def _pd(a):
    return ctypes.c_void_p(a.ctypes.data)


def gaussblur2d(Y, x1, x2, sigma, device: int = 0) -> np.ndarray:
    Y = np.asfortranarray(np.asarray(Y, dtype=np.float64))
    x1 = np.ascontiguousarray(np.asarray(x1, dtype=np.float64).ravel())
    x2 = np.ascontiguousarray(np.asarray(x2, dtype=np.float64).ravel())
    n1, n2 = Y.shape
    if x1.size != n1 or x2.size != n2:
        raise ValueError("x1 and x2 must match the sizes of Y")
    out = np.empty((n1, n2), order="F")
    ctx = context(device)
    ctx.set_memspace(_lib.MEM_HOST)
    _lib.check(ctx.L.fd2d_gaussblur2d(ctx.h, _pd(Y), n1, n2, _pd(x1), _pd(x2), float(sigma[0]), float(sigma[1]),
                                      _pd(out)), ctx.h)
    return out


def _interior(absbound):
    k = int(np.flatnonzero(np.asarray(absbound).ravel(order="F") == 1)[0])
    nx = absbound.shape[0]
    return k % nx, k // nx


def map_m_to_parameters(m, nx, nz, absbound, x, z, sigma_source, sigma_structure, ref_source=0.0,
                        ref_structure=1.0, mu_0=4.8e10, device: int = 0) -> np.ndarray:
    p = np.array(np.reshape(m, (nx, nz, -1), order="F"), dtype=np.float64)
    ix, iz = _interior(absbound)
    sl = (slice(ix, nx - ix), slice(iz, nz - iz))
    xs, zs = np.asarray(x)[ix:nx - ix], np.asarray(z)[iz:nz - iz]
    for i in range(p.shape[2] - 1):
        p[sl + (i,)] = gaussblur2d(p[sl + (i,)], xs, zs, sigma_source, device)
    p[sl + (-1,)] = gaussblur2d(p[sl + (-1,)], xs, zs, sigma_structure, device)
    p[:, :, :-1] = ref_source + p[:, :, :-1]
    p[:, :, -1] = mu_0 * (ref_structure + p[:, :, -1])
    return p


def map_parameters_to_m(p, ref_source=0.0, ref_structure=1.0, mu_0=4.8e10) -> np.ndarray:
    p = np.array(p, dtype=np.float64)
    p[:, :, :-1] = p[:, :, :-1] - ref_source
    p[:, :, -1] = p[:, :, -1] / mu_0 - ref_structure
    return p.reshape(-1, order="F")


def map_gradparameters_to_gradm(g, absbound, x, z, sigma_source, sigma_structure, mu_0=4.8e10,
                                device: int = 0) -> np.ndarray:
    g = np.asarray(g, dtype=np.float64)
    nx, nz = g.shape[:2]
    t = np.zeros_like(g)
    ix, iz = _interior(absbound)
    sl = (slice(ix, nx - ix), slice(iz, nz - iz))
    xs, zs = np.asarray(x)[ix:nx - ix], np.asarray(z)[iz:nz - iz]
    for i in range(g.shape[2] - 1):
        t[sl + (i,)] = gaussblur2d(g[sl + (i,)], xs, zs, sigma_source, device)
    t[sl + (-1,)] = gaussblur2d(g[sl + (-1,)], xs, zs, sigma_structure, device)
    t[:, :, -1] = mu_0 * t[:, :, -1]
    return t.reshape(-1, order="F")
