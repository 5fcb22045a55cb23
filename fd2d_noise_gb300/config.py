"""Solver configuration: the hidden inputs of the fd2d_noise solvers, made explicit.

The MATLAB solvers read three parameter functions internally:

* ``input_parameters()``   -- input/input_parameters.m:2-88
* ``input_interferometry()`` -- input/input_interferometry.m:2-21
* ``absorb_specs()``       -- input/absorb_specs.m:2-15

Here they are fields of :class:`Config`.  The module keeps a *current*
configuration (the reference's defaults until :func:`set_config` is called) and
exposes getters with the reference's names and return tuples, so host code
written against the reference reads the same.  Every solver also accepts an
explicit ``cfg=``.
"""
from __future__ import annotations

import ctypes
import dataclasses
from typing import Optional

import numpy as np


def matlab_colon(a: float, d: float, b: float) -> np.ndarray:
    """MATLAB ``a:d:b``.

    Follows the published construction of MATLAB's colon operator: the number
    of intervals is rounded with a tolerance of 2*eps*max(|a|,|b|), the end
    point snaps to ``b``, and the elements are built symmetrically from both
    ends (``a + k*d`` in the first half, ``last - k*d`` in the second).
    """
    eps = np.finfo(np.float64).eps
    if d == 0 or (d > 0 and a > b) or (d < 0 and a < b):
        return np.zeros(0)
    tol = 2.0 * eps * max(abs(a), abs(b))
    sig = 1.0 if d > 0 else -1.0
    if a == np.floor(a) and d == 1:
        n = int(np.floor(b) - a)
    elif a == np.floor(a) and d == np.floor(d):
        q = np.floor(a / d)
        r = a - q * d
        n = int(np.floor((b - r) / d) - q)
    else:
        n = int(np.round((b - a) / d))
        if sig * (a + n * d - b) > tol:
            n -= 1
    if n < 0:
        return np.zeros(0)
    last = a + n * d
    if a == np.floor(a) and d == np.floor(d):
        last = float(np.floor(last))
    elif sig * (last - b) > -tol:
        last = b
    out = np.zeros(n + 1)
    k = np.arange(0, n // 2 + 1)
    out[k] = a + k * d
    out[n - k] = last - k * d
    if n % 2 == 0:
        out[n // 2] = (a + last) / 2
    return out


@dataclasses.dataclass
class Config:
    """One solver configuration (all three parameter functions)."""

    # input_parameters()
    Lx: float = 6.0e4
    Lz: float = 6.0e4
    nx: int = 50
    nz: int = 50
    dt: float = 0.09
    nt: int = 150
    order: int = 4
    model_type: int = 1
    source_type: str = "homogeneous"
    n_basis_fct: int = 0
    fw_nth: int = 1
    # input_interferometry()
    f_sample: np.ndarray = dataclasses.field(
        default_factory=lambda: matlab_colon(0.02, 0.0015, 0.2))
    freq_samp: int = 5
    # absorb_specs()
    absorb_width: float = 5000.0
    absorb_left: int = 1
    absorb_right: int = 1
    absorb_top: int = 1
    absorb_bottom: int = 1

    def __post_init__(self):
        self.f_sample = np.ascontiguousarray(np.asarray(self.f_sample, dtype=np.float64).ravel())

    # -- derived quantities --------------------------------------------------
    @property
    def n_sample(self) -> int:
        return int(self.f_sample.size)

    @property
    def w_sample(self) -> np.ndarray:
        return 2 * np.pi * self.f_sample

    @property
    def dw(self) -> float:
        w = self.w_sample
        return float(w[1] - w[0])

    @property
    def dx(self) -> float:
        return self.Lx / (self.nx - 1)

    @property
    def dz(self) -> float:
        return self.Lz / (self.nz - 1)

    @property
    def ntc(self) -> int:
        return 2 * self.nt - 1

    @property
    def npts(self) -> int:
        return self.nx * self.nz

    def replace(self, **kw) -> "Config":
        return dataclasses.replace(self, **kw)

    def to_c(self) -> "FD2DConfig":
        c = FD2DConfig()
        c.Lx, c.Lz = float(self.Lx), float(self.Lz)
        c.nx, c.nz = int(self.nx), int(self.nz)
        c.dt, c.nt = float(self.dt), int(self.nt)
        c.order = int(self.order)
        c.n_basis_fct = int(self.n_basis_fct)
        c.fw_nth = int(self.fw_nth)
        c.n_sample = self.n_sample
        c._keep = self.f_sample  # keeps the buffer alive with the struct
        c.f_sample = self.f_sample.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
        c.freq_samp = int(self.freq_samp)
        c.absorb_width = float(self.absorb_width)
        c.absorb_left, c.absorb_right = int(self.absorb_left), int(self.absorb_right)
        c.absorb_top, c.absorb_bottom = int(self.absorb_top), int(self.absorb_bottom)
        return c


class FD2DConfig(ctypes.Structure):
    """ctypes mirror of ``fd2d_config`` in include/fd2d.h."""

    _fields_ = [
        ("Lx", ctypes.c_double), ("Lz", ctypes.c_double),
        ("nx", ctypes.c_int32), ("nz", ctypes.c_int32),
        ("dt", ctypes.c_double),
        ("nt", ctypes.c_int32),
        ("order", ctypes.c_int32),
        ("n_basis_fct", ctypes.c_int32),
        ("fw_nth", ctypes.c_int32),
        ("n_sample", ctypes.c_int32),
        ("f_sample", ctypes.POINTER(ctypes.c_double)),
        ("freq_samp", ctypes.c_int32),
        ("absorb_width", ctypes.c_double),
        ("absorb_left", ctypes.c_int32), ("absorb_right", ctypes.c_int32),
        ("absorb_top", ctypes.c_int32), ("absorb_bottom", ctypes.c_int32),
    ]


class FD2DSizes(ctypes.Structure):
    """ctypes mirror of ``fd2d_sizes``."""

    _fields_ = [
        ("ntc", ctypes.c_int32), ("n_fw_green", ctypes.c_int32),
        ("n_fw_corr", ctypes.c_int32), ("n_kernel_planes", ctypes.c_int32),
        ("npts", ctypes.c_int64), ("G_fft", ctypes.c_int64), ("G_out", ctypes.c_int64),
        ("seis_green", ctypes.c_int64), ("C_out", ctypes.c_int64),
        ("seis_corr", ctypes.c_int64), ("K", ctypes.c_int64),
    ]


_current: Config = Config()


def set_config(cfg: Config) -> None:
    """Make ``cfg`` the configuration the parameter getters return."""
    global _current
    _current = cfg


def get_config(cfg: Optional[Config] = None) -> Config:
    return cfg if cfg is not None else _current


def input_parameters(cfg: Optional[Config] = None):
    """``[Lx,Lz,nx,nz,dt,nt,order,model_type,source_type,n_basis_fct,fw_nth]``
    (input/input_parameters.m:2)."""
    c = get_config(cfg)
    return (c.Lx, c.Lz, c.nx, c.nz, c.dt, c.nt, c.order, c.model_type, c.source_type,
            c.n_basis_fct, c.fw_nth)


def input_interferometry(cfg: Optional[Config] = None):
    """``[f_sample, n_sample, w_sample, dw, freq_samp]`` (input/input_interferometry.m:2)."""
    c = get_config(cfg)
    return c.f_sample, c.n_sample, c.w_sample, c.dw, c.freq_samp


def absorb_specs(cfg: Optional[Config] = None):
    """``[width, absorb_left, absorb_right, absorb_top, absorb_bottom]`` (input/absorb_specs.m:2)."""
    c = get_config(cfg)
    return c.absorb_width, c.absorb_left, c.absorb_right, c.absorb_top, c.absorb_bottom


def define_computational_domain(Lx, Lz, nx, nz):
    """``[X,Z,x,z,dx,dz]`` (code/propagation/define_computational_domain.m:18-24).

    ``X`` and ``Z`` are ``meshgrid(x, z)`` outputs (nz-by-nx, as MATLAB returns them).
    """
    dx = Lx / (nx - 1)
    dz = Lz / (nz - 1)
    x = matlab_colon(0.0, dx, Lx)
    z = matlab_colon(0.0, dz, Lz)
    X, Z = np.meshgrid(x, z)
    return X, Z, x, z, dx, dz


def n_fw_green(cfg: Config) -> int:
    """Number of G_out snapshots (code/run_forward1_green.m:98-103)."""
    n = np.arange(cfg.nt, 2 * cfg.nt)
    return int(np.count_nonzero(n % cfg.fw_nth == 0))


def n_fw_corr(cfg: Config) -> int:
    """Number of C_out / u_out snapshots: floor((2nt-1)/fw_nth)."""
    return cfg.ntc // cfg.fw_nth


def n_kernel_planes(cfg: Config) -> int:
    return 2 if cfg.n_basis_fct == 0 else cfg.n_basis_fct + 1
