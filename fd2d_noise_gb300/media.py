"""Seeded random media and station layouts for the benchmark workloads.

The reference generates its random models with unseeded ``randn`` and a
random-phase inverse FFT (models/model_generator.m:21-50); its stream cannot be
reproduced, so workloads here use numpy's PCG64 with fixed seeds.
"""
from __future__ import annotations

import numpy as np

from .config import Config

MU0 = 4.8e10
RHO0 = 3000.0


def gaussian_random_field(cfg: Config, corr_len: float, seed: int) -> np.ndarray:
    """Zero-mean, unit-std field with Gaussian covariance of length ``corr_len`` [m]."""
    rng = np.random.default_rng(seed)
    nx, nz = cfg.nx, cfg.nz
    w = rng.standard_normal((nx, nz))
    kx = 2 * np.pi * np.fft.fftfreq(nx, d=cfg.dx)[:, None]
    kz = 2 * np.pi * np.fft.fftfreq(nz, d=cfg.dz)[None, :]
    filt = np.exp(-(kx ** 2 + kz ** 2) * corr_len ** 2 / 8.0)
    f = np.real(np.fft.ifft2(np.fft.fft2(w) * filt))
    f -= f.mean()
    f /= f.std()
    return np.asfortranarray(f)


def random_media(cfg: Config, std: float = 0.10, corr_len: float = 2.0e4, seed: int = 1):
    """mu = mu0 (1 + std * field), rho = rho0."""
    f = gaussian_random_field(cfg, corr_len, seed)
    mu = np.asfortranarray(MU0 * (1 + std * f))
    rho = np.full((cfg.nx, cfg.nz), RHO0, order="F")
    return mu, rho


def smoothed_perturbation(cfg: Config, max_abs: float = 0.05, sigma_pts: float = 8.0, seed: int = 1):
    """mu0 (1 + p), p = Gaussian-smoothed N(0,1) scaled to max |p| = max_abs."""
    f = gaussian_random_field(cfg, sigma_pts * cfg.dx, seed)
    f = f / np.abs(f).max() * max_abs
    mu = np.asfortranarray(MU0 * (1 + f))
    rho = np.full((cfg.nx, cfg.nz), RHO0, order="F")
    return mu, rho


def interior_points(cfg: Config, n: int, seed: int, margin_frac: float = 0.15) -> np.ndarray:
    """n positions uniformly at random inside the domain minus a margin (n-by-2)."""
    rng = np.random.default_rng(seed)
    lo, hi = margin_frac, 1 - margin_frac
    x = cfg.Lx * (lo + (hi - lo) * rng.random(n))
    z = cfg.Lz * (lo + (hi - lo) * rng.random(n))
    return np.stack([x, z], axis=1)
