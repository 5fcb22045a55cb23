"""Seeded small problems shared by the parity tests (MATLAB layouts)."""
from __future__ import annotations

import numpy as np

from fd2d_noise_gb300.config import Config


def small_cfg(nx=40, nz=36, nt=60, order=4, K=24, fs=5, fw=1, nb=0, width_pts=6, **kw) -> Config:
    Lx = 1.0e3 * (nx - 1) * 2.0
    Lz = 1.0e3 * (nz - 1) * 2.0
    dx = Lx / (nx - 1)
    dt = 0.45 * dx / 4200.0
    f = 0.02 + 0.0075 * np.arange(K)
    return Config(Lx=Lx, Lz=Lz, nx=nx, nz=nz, dt=dt, nt=nt, order=order, n_basis_fct=nb,
                  fw_nth=fw, f_sample=f, freq_samp=fs, absorb_width=width_pts * dx, **kw)


def media(cfg: Config, seed=0):
    rng = np.random.default_rng(seed)
    nx, nz = cfg.nx, cfg.nz
    pert = rng.standard_normal((nx, nz))
    # cheap smoothing
    for _ in range(3):
        pert = 0.25 * (np.roll(pert, 1, 0) + np.roll(pert, -1, 0) + np.roll(pert, 1, 1) + np.roll(pert, -1, 1))
    pert /= np.abs(pert).max()
    mu = np.asfortranarray(4.8e10 * (1 + 0.05 * pert))
    rho = np.asfortranarray(3000.0 * (1 + 0.02 * np.roll(pert, 3, 0)))
    return mu, rho


def stations(cfg: Config, n, seed=1):
    rng = np.random.default_rng(seed)
    lo = 0.2
    x = cfg.Lx * (lo + (1 - 2 * lo) * rng.random(n))
    z = cfg.Lz * (lo + (1 - 2 * lo) * rng.random(n))
    return np.stack([x, z], axis=1)


def noise_source(cfg: Config, seed=2):
    """Gaussian spectrum and a Gaussian-patch distribution (make_noise_source form)."""
    f = cfg.f_sample
    spec = np.exp(-(np.abs(f) - 0.08) ** 2 / 0.04 ** 2).reshape(-1, 1)
    nx, nz = cfg.nx, cfg.nz
    x = np.linspace(0, cfg.Lx, nx)[:, None]
    z = np.linspace(0, cfg.Lz, nz)[None, :]
    planes = max(cfg.n_basis_fct, 1)
    rng = np.random.default_rng(seed)
    sd = np.zeros((nx, nz, planes), order="F")
    for b in range(planes):
        cx, cz = cfg.Lx * rng.uniform(0.3, 0.7), cfg.Lz * rng.uniform(0.3, 0.7)
        sd[:, :, b] = 1 + 6.0 * np.exp(-((x - cx) ** 2 + (z - cz) ** 2) / (0.2 * cfg.Lx) ** 2)
    if cfg.n_basis_fct:
        spec = np.ones((cfg.n_sample, 1))
    return spec, sd


def rel_l2(a, b):
    a = np.asarray(a, dtype=np.complex128 if np.iscomplexobj(a) or np.iscomplexobj(b) else np.float64)
    b = np.asarray(b, dtype=a.dtype)
    den = np.linalg.norm(b.ravel())
    num = np.linalg.norm((a - b).ravel())
    if den == 0:
        return 0.0 if num == 0 else float("inf")
    return float(num / den)
