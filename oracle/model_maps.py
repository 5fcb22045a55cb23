"""FP64 numpy restatement of the reference's model-space maps.

TEST INFRASTRUCTURE: only tests/ use it, as the checker of fd2d_gaussblur2d and
of fd2d_noise_gb300.model_maps.

    gaussblur2d                 tools/addons/gaussblur2d.m:2-38
    map_m_to_parameters         inversion/optlib_callback_fct/map_m_to_parameters.m:15-52
    map_parameters_to_m         inversion/optlib_callback_fct/map_parameters_to_m.m:15-20
    map_gradparameters_to_gradm inversion/optlib_callback_fct/map_gradparameters_to_gradm.m:20-57
(the non-ring branch).  Pinned against tests/golden/map_cases.npz.
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


def interior(absbound):
    """[ix, iz] = find(absbound == 1, 1, 'first') as 0-based indices."""
    k = int(np.flatnonzero(np.asarray(absbound).ravel(order="F") == 1)[0])
    nx = absbound.shape[0]
    return k % nx, k // nx


def map_m_to_parameters(m, nx, nz, absbound, x, z, sigma_source, sigma_structure, ref_source, ref_structure, mu_0):
    p = np.array(np.reshape(m, (nx, nz, -1), order="F"), dtype=np.float64)
    ix, iz = interior(absbound)
    sl = (slice(ix, nx - ix), slice(iz, nz - iz))
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


def map_gradparameters_to_gradm(g, absbound, x, z, sigma_source, sigma_structure, mu_0):
    g = np.asarray(g, dtype=np.float64)
    nx, nz = g.shape[:2]
    t = np.zeros_like(g)
    ix, iz = interior(absbound)
    sl = (slice(ix, nx - ix), slice(iz, nz - iz))
    for i in range(g.shape[2] - 1):
        t[sl + (i,)] = gaussblur2d(g[sl + (i,)], x[ix:nx - ix], z[iz:nz - iz], sigma_source)
    t[sl + (-1,)] = gaussblur2d(g[sl + (-1,)], x[ix:nx - ix], z[iz:nz - iz], sigma_structure)
    t[:, :, -1] = mu_0 * t[:, :, -1]
    return t.reshape(-1, order="F")
