"""Noise-source model: spectra, spatial PSD distributions, frequency bands.

Host-side input generation with the semantics of input/make_noise_source.m,
code/propagation/integration_limits.m and code/propagation/general_source.m.
The reference hard-codes its parameters inside make_noise_source; here they are
keyword arguments whose defaults are the reference's values.
"""
from __future__ import annotations

from typing import Optional, Sequence

import numpy as np

from .config import Config, define_computational_domain, get_config


def noise_spectrum(f_sample, f_peak: Sequence[float] = (1 / 11, 1 / 7),
                   bandwidth: Sequence[float] = (0.035, 0.025),
                   strength: Sequence[float] = (0.3, 1.0), n_noise_sources: int = 1) -> np.ndarray:
    """``strength*exp(-(|f|-f_peak)^2/bandwidth^2)`` per source (make_noise_source.m:135-139).

    Note the exponent's denominator is bandwidth^2, not 2*sigma^2.
    """
    f = np.asarray(f_sample, dtype=np.float64)
    out = np.zeros((f.size, n_noise_sources))
    for ns in range(n_noise_sources):
        out[:, ns] = strength[ns] * np.exp(-(np.abs(f) - f_peak[ns]) ** 2 / bandwidth[ns] ** 2)
    return out


def integration_limits(n_sample: int, n_basis_fct: int) -> np.ndarray:
    """1-based band limits (code/propagation/integration_limits.m:4-12)."""
    step = n_sample / n_basis_fct
    lim = np.zeros((n_basis_fct, 2), dtype=np.int64)
    for i in range(1, n_basis_fct + 1):
        lim[i - 1, 0] = int(np.floor((i - 1) * step + 1))
        lim[i - 1, 1] = int(np.floor(i * step))
    return lim


def general_source(noise_spectrum_: np.ndarray, distribution: np.ndarray, n_basis_fct: int) -> np.ndarray:
    """Band-averaged source maps (code/propagation/general_source.m:13-24)."""
    K, n_src = noise_spectrum_.shape
    nx, nz = distribution.shape[:2]
    dist = distribution.reshape(nx, nz, -1, order="F")
    out = np.zeros((nx, nz, n_basis_fct), order="F")
    lim = integration_limits(K, n_basis_fct)
    for ib in range(n_basis_fct):
        idx = np.arange(lim[ib, 0], lim[ib, 1] + 1)
        ni = idx.size
        for k in idx:
            for ns in range(n_src):
                out[:, :, ib] += noise_spectrum_[k - 1, ns] * dist[:, :, ns] / ni
    return out


def gaussian_blobs(cfg: Config, x_c, z_c, width, magnitude, base: float = 1.0) -> np.ndarray:
    """``base + sum magnitude*exp(-((X-x)^2+(Z-z)^2)/width^2)'`` (make_noise_source.m:151-156)."""
    X, Z, *_ = define_computational_domain(cfg.Lx, cfg.Lz, cfg.nx, cfg.nz)
    d = np.full((cfg.nz, cfg.nx), base)
    for xs, zs, w, m in zip(np.atleast_1d(x_c), np.atleast_1d(z_c), np.atleast_1d(width), np.atleast_1d(magnitude)):
        d = d + m * np.exp(-((X - xs) ** 2 + (Z - zs) ** 2) / w ** 2)
    return np.asfortranarray(d.T)


def ring(cfg: Config, x_r=1.0e6, z_r=1.0e6, radius=6.8e5, thickness=1e5, angle_cover=60.0,
         taper_width=20.0, taper_strength=100.0, radial_scale=9e8) -> np.ndarray:
    """Ring of sources with an angular taper (make_noise_source.m:189-205).

    The reference assigns the meshgrid-shaped (nz-by-nx) result into the
    nx-by-nz plane without a transpose, so it only runs on square grids and its
    map is the transpose of the meshgrid picture; both are kept here.
    """
    if cfg.nx != cfg.nz:
        raise ValueError("the reference's ring distribution needs nx == nz")
    X, Z, *_ = define_computational_domain(cfg.Lx, cfg.Lz, cfg.nx, cfg.nz)
    R = np.sqrt((X - x_r) ** 2 + (Z - z_r) ** 2)
    with np.errstate(divide="ignore", invalid="ignore"):
        angle = np.arctan(np.abs(X - x_r) / np.abs(Z - z_r)) * 180 / np.pi
    angle[np.isnan(angle)] = 0.0
    shell = (R > (radius - thickness / 2)) & (R < (radius + thickness / 2))
    radial = np.exp(-np.abs(R - radius) ** 2 / radial_scale)
    d = radial * shell
    if angle_cover != 90:
        cov = (angle > angle_cover - taper_width) & (angle < angle_cover)
        d = d + radial * (5 * np.exp(-(angle - (angle_cover - taper_width)) ** 2 / taper_strength * cov)
                          * (shell & (angle <= angle_cover)))
    return np.asfortranarray(d)


def make_noise_source(source_type: str = "homogeneous", n_basis_fct: int = 0,
                      cfg: Optional[Config] = None, n_noise_sources: int = 1,
                      spectrum_kw: Optional[dict] = None, **dist_kw):
    """``[noise_source_distribution, noise_spectrum]`` (input/make_noise_source.m:2).

    ``source_type``: 'homogeneous', 'gaussian' (``x_c, z_c, width, magnitude``),
    'ring' (see :func:`ring`) or 'picture' (``picture=`` an nx-by-nz array in
    [0, 1], standing in for the reference's image file).  With
    ``n_basis_fct > 0`` the maps are band-averaged by :func:`general_source` and
    the spectrum becomes ones (make_noise_source.m:224-227).
    """
    cfg = get_config(cfg)
    spec = noise_spectrum(cfg.f_sample, n_noise_sources=n_noise_sources, **(spectrum_kw or {}))
    nx, nz = cfg.nx, cfg.nz
    dist = np.ones((nx, nz, n_noise_sources), order="F")
    if source_type == "gaussian":
        # the reference's two parameter sets, chosen by domain size (make_noise_source.m:13-17,47-60)
        if cfg.Lx == 2.0e6 or cfg.Lz == 2.0e6:
            kw = dict(x_c=[0.6e6, 0.5e6, 1.3e6], z_c=[0.8e6, 1.5e6, 1.6e6], width=[1.5e5, 1.5e5, 1.8e5],
                      magnitude=[6.5, 5.0, 3.0])
        else:
            kw = dict(x_c=[1.0e5], z_c=[1.6e5], width=[4e4], magnitude=[6.0])
        kw.update(dist_kw)
        for ns in range(n_noise_sources):
            dist[:, :, ns] = gaussian_blobs(cfg, kw["x_c"][ns:ns + 1], kw["z_c"][ns:ns + 1],
                                            kw["width"][ns:ns + 1], kw["magnitude"][ns:ns + 1])
    elif source_type == "ring":
        dist[:, :, 0] = ring(cfg, **dist_kw)
    elif source_type == "picture":
        dist[:, :, 0] = np.asarray(dist_kw["picture"], dtype=np.float64)
    elif source_type != "homogeneous":
        raise ValueError(f"unknown source_type {source_type!r}")
    if n_basis_fct != 0:
        dist = general_source(spec, dist, n_basis_fct)
        spec = np.ones((cfg.n_sample, 1))
    return dist, spec
