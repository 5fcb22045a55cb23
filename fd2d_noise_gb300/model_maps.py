"""Model-space maps of the inversion with Gaussian smoothing on the GPU.

    m_parameters = map_m_to_parameters(m, ...)            map_m_to_parameters.m:15-52
    m            = map_parameters_to_m(m_parameters, ...) map_parameters_to_m.m:15-20
    grad_m       = map_gradparameters_to_gradm(g, ...)    map_gradparameters_to_gradm.m:20-57
    GY           = gaussblur2d(Y, x1, x2, sigma)          tools/addons/gaussblur2d.m:2-38
    B            = imfilter_circular(Y, h)                imfilter(Y, h, 'circular')

(inversion/optlib_callback_fct/).  The smoothing runs in libfd2d
(fd2d_gaussblur2d and fd2d_imfilter_circular, FP64); the parameters of the
reference's ``usr_par`` struct are explicit arguments.  The smoothing acts on
the interior where the taper is 1 (``find(absbound == 1, 1, 'first')``), as in
the reference.

With ``ring`` (usr_par.ring.switch = 'yes', map_m_to_parameters.m:22-29,
map_gradparameters_to_gradm.m:27-35) the first source plane is multiplied by a
Gaussian-tapered annulus and the structure plane is filtered with
``imfilter(., h_structure, 'circular')`` (usr_par.kernel.imfilter.structure,
e.g. ``fspecial_gaussian((40, 40), 20)``); the other source planes pass through
(model map) or are zero (gradient map), as in the reference.  The annulus comes
from ``[X, Z] = meshgrid(x, z)``, an nz-by-nx matrix multiplied element by
element into the nx-by-nz plane, so the ring needs nx == nz and element (i, j)
sees x(j), z(i); a non-square grid is rejected like the reference's
dimension mismatch.
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass
from typing import Optional

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


@dataclass
class Ring:
    """usr_par.ring of the reference (defaults: inversion/start_inversion.m:70-74)."""
    x_center_ring: float = 1.0e6
    z_center_ring: float = 1.0e6
    radius: float = 6.4e5
    thickness: float = 2.0e5
    taper_strength: float = 70e8


def fspecial_gaussian(shape=(3, 3), sigma: float = 0.5) -> np.ndarray:
    """The kernel of MATLAB's fspecial('gaussian', shape, sigma) as documented:
    exp(-(x^2 + y^2) / (2 sigma^2)) on a grid centred on the kernel, entries
    below eps times the maximum set to 0, normalised to sum 1."""
    m1, m2 = (int(shape), int(shape)) if np.isscalar(shape) else (int(shape[0]), int(shape[1]))
    y, x = np.meshgrid(np.arange(m1) - (m1 - 1) / 2, np.arange(m2) - (m2 - 1) / 2, indexing="ij")
    h = np.exp(-(x * x + y * y) / (2.0 * sigma * sigma))
    h[h < np.finfo(np.float64).eps * h.max()] = 0.0
    s = h.sum()
    return h / s if s != 0 else h


def imfilter_circular(Y, h, device: int = 0) -> np.ndarray:
    """imfilter(Y, h, 'circular'): correlation with h, output the size of Y, Y
    extended periodically, the centre of h at floor((size(h)+1)/2)."""
    Y = np.asfortranarray(np.asarray(Y, dtype=np.float64))
    h = np.asfortranarray(np.atleast_2d(np.asarray(h, dtype=np.float64)))
    if Y.ndim != 2 or h.ndim != 2:
        raise ValueError("imfilter_circular takes 2-D arrays")
    n1, n2 = Y.shape
    m1, m2 = h.shape
    out = np.empty((n1, n2), order="F")
    ctx = context(device)
    ctx.set_memspace(_lib.MEM_HOST)
    _lib.check(ctx.L.fd2d_imfilter_circular(ctx.h, _pd(Y), n1, n2, _pd(h), m1, m2, _pd(out)), ctx.h)
    return out


def _ring_factors(x, z, ring: Ring):
    """exp(-|R - radius|^2 / taper_strength) and the annulus indicator, nx-by-nz."""
    x = np.asarray(x, dtype=np.float64).ravel()
    z = np.asarray(z, dtype=np.float64).ravel()
    if x.size != z.size:
        raise ValueError("the ring parameterisation needs nx == nz (the reference multiplies an nz-by-nx "
                         "coordinate matrix into the nx-by-nz parameter plane)")
    X, Z = np.meshgrid(x, z)
    R = ((X - ring.x_center_ring) ** 2 + (Z - ring.z_center_ring) ** 2) ** 0.5
    taper = np.exp(-np.abs(R - ring.radius) ** 2 / ring.taper_strength)
    inside = ((R > ring.radius - ring.thickness / 2) & (R < ring.radius + ring.thickness / 2)).astype(np.float64)
    return taper, inside


def _ring_kernel(h_structure):
    if h_structure is None:
        raise ValueError("the ring parameterisation needs h_structure (usr_par.kernel.imfilter.structure)")
    return h_structure


def _interior(absbound):
    k = int(np.flatnonzero(np.asarray(absbound).ravel(order="F") == 1)[0])
    nx = absbound.shape[0]
    return k % nx, k // nx


def map_m_to_parameters(m, nx, nz, absbound, x, z, sigma_source, sigma_structure, ref_source=0.0,
                        ref_structure=1.0, mu_0=4.8e10, device: int = 0, ring: Optional[Ring] = None,
                        h_structure=None) -> np.ndarray:
    p = np.array(np.reshape(m, (nx, nz, -1), order="F"), dtype=np.float64)
    ix, iz = _interior(absbound)
    sl = (slice(ix, nx - ix), slice(iz, nz - iz))
    if ring is not None:
        h = _ring_kernel(h_structure)
        taper, inside = _ring_factors(x, z, ring)
        p[:, :, 0] = (p[:, :, 0] * taper) * inside
        p[sl + (-1,)] = imfilter_circular(p[sl + (-1,)], h, device)
    else:
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
                                device: int = 0, ring: Optional[Ring] = None, h_structure=None) -> np.ndarray:
    g = np.asarray(g, dtype=np.float64)
    nx, nz = g.shape[:2]
    t = 0.0 * g  # temp = 0.0 * grad_parameters (NaN and Inf carry through)
    ix, iz = _interior(absbound)
    sl = (slice(ix, nx - ix), slice(iz, nz - iz))
    if ring is not None:
        h = _ring_kernel(h_structure)
        taper, inside = _ring_factors(x, z, ring)
        t[:, :, 0] = (g[:, :, 0] * taper) * inside
        t[sl + (-1,)] = imfilter_circular(g[sl + (-1,)], h, device)
    else:
        xs, zs = np.asarray(x)[ix:nx - ix], np.asarray(z)[iz:nz - iz]
        for i in range(g.shape[2] - 1):
            t[sl + (i,)] = gaussblur2d(g[sl + (i,)], xs, zs, sigma_source, device)
        t[sl + (-1,)] = gaussblur2d(g[sl + (-1,)], xs, zs, sigma_structure, device)
    t[:, :, -1] = mu_0 * t[:, :, -1]
    return t.reshape(-1, order="F")
