"""Named synthetic workloads (seeded) with the shapes of the benchmark configurations.

* ``plain_cpu_300``      -- 300x300, dt 0.1, nt 1200, order 4, 200 frequencies in
                            0.01-0.2 Hz, Gaussian spectrum (0.1 Hz, 0.03 Hz),
                            Gaussian-patch distribution, +-5 % smoothed mu,
                            10 receivers, one reference station, taper 20 points.
* ``single_600_o8``      -- 600x600, dt 0.05, nt 3000, order 8, 300 frequencies,
                            2 reference stations, 40 receivers, random media
                            (10 % std, 20 km correlation length), ring source.
* ``structure_512``      -- 512x512, nt 2500, snapshots every 5 steps, 200
                            frequencies, 1 reference station, 20 receivers on
                            a 450 km ring (1e6 m domain), starting and true
                            models for the misfit.
* ``large_2048_o8``      -- 2048x2048, order 8, 4 stations, 8 frequencies, nt 200:
                            fields larger than L2 (stencil HBM roofline).
* ``batch_uneven``       -- 32 reference stations on grids of 256, 384, 512 or
                            800 points square, nt 1500-4000, order 4, 4
                            frequency bands (see :func:`batch_uneven`).

The domain is 4e5 m square (the reference's "small setup") except in
``structure_512``, whose 1e6 m domain puts the arrivals inside the
measurement window.
"""
from __future__ import annotations

import dataclasses
from typing import Callable, Dict, Optional

import numpy as np

from .config import Config, matlab_colon
from .media import interior_points, random_media, smoothed_perturbation
from .noise_source import make_noise_source

L = 4.0e5


@dataclasses.dataclass
class Workload:
    name: str
    cfg: Config
    mu: np.ndarray
    rho: np.ndarray
    ref_stations: np.ndarray   # n_ref-by-2
    receivers: np.ndarray      # nr-by-2
    spectrum: np.ndarray       # K-by-n_src
    source_dist: np.ndarray    # nx-by-nz-by-n_dist
    mu_true: Optional[np.ndarray] = None  # model of the observed data (structure-kernel workload)

    def gpt_green(self) -> int:
        return self.cfg.npts * self.cfg.nt

    def gpt_correlation(self) -> int:
        return self.cfg.npts * self.cfg.ntc

    def gpt_per_station(self) -> int:
        return self.gpt_green() + self.gpt_correlation()


def _freqs(f0, f1, K):
    return matlab_colon(f0, (f1 - f0) / (K - 1), f1)[:K] if K > 1 else np.array([f0])


def plain_cpu_300(nt: int = 1200) -> Workload:
    nx = 300
    dx = L / (nx - 1)
    cfg = Config(Lx=L, Lz=L, nx=nx, nz=nx, dt=0.1, nt=nt, order=4, f_sample=_freqs(0.01, 0.2, 200),
                 freq_samp=5, fw_nth=1, absorb_width=20 * dx, source_type="gaussian")
    mu, rho = smoothed_perturbation(cfg, 0.05, seed=1)
    sd, spec = make_noise_source("gaussian", 0, cfg,
                                 spectrum_kw=dict(f_peak=[0.1], bandwidth=[0.03], strength=[1.0]),
                                 x_c=[0.3 * L], z_c=[0.6 * L], width=[0.1 * L], magnitude=[6.0])
    rec = interior_points(cfg, 10, seed=2, margin_frac=0.25)
    ref = interior_points(cfg, 1, seed=12, margin_frac=0.3)
    return Workload("plain_cpu_300", cfg, mu, rho, ref, rec, spec, sd)


def single_600_o8(nt: int = 3000, K: int = 300, n_ref: int = 2, nx: int = 600) -> Workload:
    """``nx`` (square grid) other than 600 is for profiling the step kernel
    across grid sizes; the workload is named for its grid."""
    dx = L / (nx - 1)
    cfg = Config(Lx=L, Lz=L, nx=nx, nz=nx, dt=0.05, nt=nt, order=8, f_sample=_freqs(0.01, 0.2, K),
                 freq_samp=5, fw_nth=1, absorb_width=20 * dx, source_type="ring")
    mu, rho = random_media(cfg, std=0.10, corr_len=2.0e4, seed=1)
    s = L / 2.0e6  # the reference's ring is laid out on a 2e6 m domain
    sd, spec = make_noise_source("ring", 0, cfg,
                                 spectrum_kw=dict(f_peak=[0.1], bandwidth=[0.03], strength=[1.0]),
                                 x_r=1.0e6 * s, z_r=1.0e6 * s, radius=6.8e5 * s, thickness=1e5 * s,
                                 radial_scale=9e8 * s * s)
    rec = interior_points(cfg, 40, seed=3, margin_frac=0.2)
    ref = interior_points(cfg, n_ref, seed=13, margin_frac=0.3)
    return Workload("single_600_o8" if nx == 600 else f"single_{nx}_o8", cfg, mu, rho, ref, rec, spec, sd)


def structure_512(nt: int = 2500) -> Workload:
    """Structure-kernel workload: 512x512 on a 1e6 m domain, dt 0.2 s, nt 2500,
    snapshots every 5 steps, 200 frequencies in 0.006-0.028 Hz, 4th order; one
    reference station in the centre and 20 receivers on a 450 km ring, so the
    surface waves arrive at ~110 s, inside the 100-200 s window of the
    log-amplitude-ratio measurement (tools/measurement/make_adjoint_sources.m:
    85-86).  ``mu`` is the homogeneous starting model, ``mu_true`` the model
    the observed correlations come from (a 5 % Gaussian anomaly)."""
    L2, nx = 1.0e6, 512
    dx = L2 / (nx - 1)
    cfg = Config(Lx=L2, Lz=L2, nx=nx, nz=nx, dt=0.2, nt=nt, order=4, n_basis_fct=0, fw_nth=5,
                 f_sample=np.linspace(0.006, 0.028, 200), freq_samp=5, absorb_width=20 * dx)
    X, Z = np.meshgrid(np.linspace(0, L2, nx), np.linspace(0, L2, nx), indexing="ij")
    mu = 4.8e10 * np.ones((nx, nx))
    ang = np.linspace(0, 2 * np.pi, 20, endpoint=False)
    ref = np.array([[0.5e6, 0.5e6]])
    rec = np.stack([0.5e6 + 0.45e6 * np.cos(ang), 0.5e6 + 0.45e6 * np.sin(ang)], axis=1)
    spec = np.exp(-(cfg.f_sample - 0.017) ** 2 / 0.008 ** 2).reshape(-1, 1)
    sd = np.asfortranarray((1 + 5 * np.exp(-((X - 0.3e6) ** 2 + (Z - 0.7e6) ** 2) / 1.5e5 ** 2))[:, :, None])
    w = Workload("structure_512", cfg, mu, 3000.0 * np.ones((nx, nx)), ref, rec, spec, sd)
    w.mu_true = mu * (1 + 0.05 * np.exp(-((X - 0.7e6) ** 2 + (Z - 0.55e6) ** 2) / 1.0e5 ** 2))
    return w


def large_2048_o8(nt: int = 200, K: int = 8, n_ref: int = 4) -> Workload:
    """Stencil-bandwidth case: 2048x2048, order 8, ``n_ref`` stations as lanes,
    few frequencies, so the fields (11 planes x 16.8 MB per station) exceed L2
    and the stencil streams them from HBM."""
    nx = 2048
    dx = L / (nx - 1)
    cfg = Config(Lx=L, Lz=L, nx=nx, nz=nx, dt=0.4 * dx / 4000.0, nt=nt, order=8, f_sample=_freqs(0.01, 0.2, K),
                 freq_samp=5, fw_nth=1, absorb_width=20 * dx, source_type="ring")
    mu, rho = random_media(cfg, std=0.10, corr_len=2.0e4, seed=7)
    s = L / 2.0e6
    sd, spec = make_noise_source("ring", 0, cfg,
                                 spectrum_kw=dict(f_peak=[0.1], bandwidth=[0.03], strength=[1.0]),
                                 x_r=1.0e6 * s, z_r=1.0e6 * s, radius=6.8e5 * s, thickness=1e5 * s,
                                 radial_scale=9e8 * s * s)
    rec = interior_points(cfg, 40, seed=3, margin_frac=0.2)
    ref = interior_points(cfg, n_ref, seed=17, margin_frac=0.3)
    return Workload("large_2048_o8", cfg, mu, rho, ref, rec, spec, sd)


@dataclasses.dataclass
class BatchWorkload:
    """Reference stations on grids of different sizes (one Workload per station)."""
    name: str
    stations: list

    def gpt_per_step(self) -> int:
        return sum(w.gpt_per_station() for w in self.stations)


def batch_uneven(n_stations: int = 32, n_basis: int = 4, K: int = 200, nr: int = 20, seed: int = 4,
                 nt_range=(1500, 4000), sizes=(256, 384, 512, 800)) -> BatchWorkload:
    """Reference stations on grids drawn from ``sizes`` (square), nt uniform in
    ``nt_range``, dt from CFL 0.5 at 4000 m/s, order 4, taper 30 points; one
    random medium (5 % std) per grid size; the noise source has ``n_basis``
    frequency bands (spectrum of ones, band-averaged Gaussian maps)."""
    rng = np.random.default_rng(seed)
    media, out = {}, []
    for i in range(n_stations):
        nx = int(rng.choice(sizes))
        nt = int(rng.integers(nt_range[0], nt_range[1] + 1))
        dx = L / (nx - 1)
        cfg = Config(Lx=L, Lz=L, nx=nx, nz=nx, dt=0.5 * dx / 4000.0, nt=nt, order=4, n_basis_fct=n_basis,
                     f_sample=_freqs(0.01, 0.2, K), freq_samp=5, fw_nth=1, absorb_width=30 * dx,
                     source_type="gaussian")
        if nx not in media:
            mu, rho = random_media(cfg, std=0.05, corr_len=2.0e4, seed=100 + nx)
            sd, spec = make_noise_source("gaussian", n_basis, cfg,
                                         spectrum_kw=dict(f_peak=[0.1], bandwidth=[0.03], strength=[1.0]),
                                         x_c=[0.3 * L], z_c=[0.6 * L], width=[0.1 * L], magnitude=[6.0])
            media[nx] = (mu, rho, sd, spec, interior_points(cfg, nr, seed=200 + nx, margin_frac=0.2))
        mu, rho, sd, spec, rec = media[nx]
        ref = interior_points(cfg, 1, seed=1000 + i, margin_frac=0.3)
        out.append(Workload(f"station{i}_{nx}", cfg, mu, rho, ref, rec, spec, sd))
    return BatchWorkload("batch_uneven", out)


WORKLOADS: Dict[str, Callable[..., Workload]] = {
    "plain_cpu_300": plain_cpu_300,
    "single_600_o8": single_600_o8,
    "structure_512": structure_512,
    "large_2048_o8": large_2048_o8,
    "batch_uneven": batch_uneven,
}
