"""FP64 numpy restatement of the reference's model-space maps.

TEST INFRASTRUCTURE: only tests/ use it, as the checker of fd2d_gaussblur2d and
of fd2d_noise_gb300.model_maps.

    gaussblur2d                 tools/addons/gaussblur2d.m:2-38
    map_m_to_parameters         inversion/optlib_callback_fct/map_m_to_parameters.m:15-52
    map_parameters_to_m         inversion/optlib_callback_fct/map_parameters_to_m.m:15-20
    map_gradparameters_to_gradm inversion/optlib_callback_fct/map_gradparameters_to_gradm.m:20-57
    ring branch                 map_m_to_parameters.m:22-29, map_gradparameters_to_gradm.m:27-35
    imfilter_circular           imfilter(A, h, 'circular'), MATLAB Image Processing Toolbox

Both branches of the maps ('ring' and Gaussian smoothing).  Pinned against
tests/golden/map_cases.npz: gaussblur2d and the unmodified map_*.m files run by
the MATLAB-subset interpreter.  imfilter is not part of the reference; it is
restated from its documented definition (correlation with h, output the size of
A, A extended periodically, the centre of h at floor((size(h)+1)/2)), and the
fixtures pin how the maps use it.
"""
from __future__ import annotations

import numpy as np


def gaussblur2d(Y, x1, x2, sigma):
    Y = np.asarray(Y, dtype=np.float64)
    x1 = np.asarray(x1, dtype=np.float64).ravel()
    x2 = np.asarray(x2, dtype=np.float64).ravel()
    n1, n2 = Y.shape
    Mtmp = np.zeros_like(Y)
    GY = np.zeros_like(Y)
    w1 = np.zeros(n1)
    w2 = np.zeros(n2)
    c1, c2 = np.sqrt(14.0) * sigma[0], np.sqrt(14.0) * sigma[1]
    for i in range(n1):
        for j in range(n1):
            dist = abs(x1[i] - x1[j])
            if dist < c1:
                w = np.exp(-(dist / sigma[0]) ** 2 / 2.0)
                w1[j] = w1[j] + w
                Mtmp[i, :] = Mtmp[i, :] + w * Y[j, :]
    for i in range(n2):
        for j in range(n2):
            dist = abs(x2[i] - x2[j])
            if dist < c2:
                w = np.exp(-(dist / sigma[1]) ** 2 / 2.0)
                w2[j] = w2[j] + w
                GY[:, i] = GY[:, i] + w * Mtmp[:, j]
    return GY / np.outer(w1, w2)


def _radius(x, z, ring):
    """R from [X, Z] = meshgrid(x, z): an nz-by-nx matrix that the reference
    multiplies element by element into the nx-by-nz parameter plane, so the
    ring needs nx == nz and element (i, j) sees x(j), z(i)."""
    x = np.asarray(x, dtype=np.float64).ravel()
    z = np.asarray(z, dtype=np.float64).ravel()
    if x.size != z.size:
        raise ValueError("the ring parameterisation needs nx == nz")
    X, Z = np.meshgrid(x, z)
    return ((X - ring.x_center_ring) ** 2 + (Z - ring.z_center_ring) ** 2) ** 0.5


def _annulus(x, z, ring):
    R = _radius(x, z, ring)
    return ((R > ring.radius - ring.thickness / 2) & (R < ring.radius + ring.thickness / 2)).astype(np.float64)


def interior(absbound):
    """[ix, iz] = find(absbound == 1, 1, 'first') as 0-based indices."""
    k = int(np.flatnonzero(np.asarray(absbound).ravel(order="F") == 1)[0])
    nx = absbound.shape[0]
    return k % nx, k // nx


def imfilter_circular(A, h):
    """B(i,j) = sum over (u,v) of h(u,v) A(i+u-c1, j+v-c2), indices modulo the
    size of A, c = floor((size(h)+1)/2) (1-based).  Terms are added v-major,
    u-minor, each product rounded before the addition."""
    A = np.asarray(A, dtype=np.float64)
    h = np.atleast_2d(np.asarray(h, dtype=np.float64))
    m1, m2 = h.shape
    c1, c2 = (m1 - 1) // 2, (m2 - 1) // 2
    out = np.zeros_like(A)
    for v in range(m2):
        for u in range(m1):
            out = out + h[u, v] * np.roll(A, (c1 - u, c2 - v), axis=(0, 1))
    return out


def map_m_to_parameters(m, nx, nz, absbound, x, z, sigma_source, sigma_structure, ref_source, ref_structure, mu_0,
                        ring=None, h_structure=None):
    p = np.array(np.reshape(m, (nx, nz, -1), order="F"), dtype=np.float64)
    ix, iz = interior(absbound)
    sl = (slice(ix, nx - ix), slice(iz, nz - iz))
    if ring is not None:
        p[:, :, 0] = (p[:, :, 0] * np.exp(-np.abs(_radius(x, z, ring) - ring.radius) ** 2 / ring.taper_strength)) \
            * _annulus(x, z, ring)
        p[sl + (-1,)] = imfilter_circular(p[sl + (-1,)], h_structure)
    else:
        for i in range(p.shape[2] - 1):
            p[sl + (i,)] = gaussblur2d(p[sl + (i,)], x[ix:nx - ix], z[iz:nz - iz], sigma_source)
        p[sl + (-1,)] = gaussblur2d(p[sl + (-1,)], x[ix:nx - ix], z[iz:nz - iz], sigma_structure)
    p[:, :, :-1] = ref_source + p[:, :, :-1]
    p[:, :, -1] = mu_0 * (ref_structure + p[:, :, -1])
    return p


def map_parameters_to_m(p, ref_source, ref_structure, mu_0):
    p = np.array(p, dtype=np.float64)
    p[:, :, :-1] = p[:, :, :-1] - ref_source
    p[:, :, -1] = p[:, :, -1] / mu_0 - ref_structure
    return p.reshape(-1, order="F")


def map_gradparameters_to_gradm(g, absbound, x, z, sigma_source, sigma_structure, mu_0, ring=None, h_structure=None):
    g = np.asarray(g, dtype=np.float64)
    nx, nz = g.shape[:2]
    t = 0.0 * g
    ix, iz = interior(absbound)
    sl = (slice(ix, nx - ix), slice(iz, nz - iz))
    if ring is not None:
        t[:, :, 0] = (g[:, :, 0] * np.exp(-np.abs(_radius(x, z, ring) - ring.radius) ** 2 / ring.taper_strength)) \
            * _annulus(x, z, ring)
        t[sl + (-1,)] = imfilter_circular(g[sl + (-1,)], h_structure)
    else:
        for i in range(g.shape[2] - 1):
            t[sl + (i,)] = gaussblur2d(g[sl + (i,)], x[ix:nx - ix], z[iz:nz - iz], sigma_source)
        t[sl + (-1,)] = gaussblur2d(g[sl + (-1,)], x[ix:nx - ix], z[iz:nz - iz], sigma_structure)
    t[:, :, -1] = mu_0 * t[:, :, -1]
    return t.reshape(-1, order="F")
