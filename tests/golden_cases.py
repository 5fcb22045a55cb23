"""Access to tests/golden/reference_cases.npz (outputs of the reference's own
MATLAB solvers, executed by tests/golden/mini_matlab.py)."""
from __future__ import annotations

import os

import numpy as np

from fd2d_noise_gb300.config import Config

PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "reference_cases.npz")
_cache = None


def load():
    global _cache
    if _cache is None:
        _cache = dict(np.load(PATH))
    return _cache


def group(case: str, name: str) -> dict:
    d = load()
    pre = f"{case}/{name}/"
    return {k[len(pre):]: d[k] for k in d if k.startswith(pre)}


def cfg(case: str) -> Config:
    c = group(case, "cfg")
    return Config(Lx=float(c["Lx"]), Lz=float(c["Lz"]), nx=int(c["nx"]), nz=int(c["nz"]), dt=float(c["dt"]),
                  nt=int(c["nt"]), order=int(c["order"]), n_basis_fct=int(c["nb"]), fw_nth=int(c["fw"]),
                  f_sample=np.asarray(c["f_sample"], dtype=np.float64), freq_samp=int(c["fs"]),
                  absorb_width=float(c["width"]))


def rel(a, b) -> float:
    a = np.asarray(a)
    b = np.asarray(b)
    a = a.reshape(b.shape) if a.size == b.size else a
    num = np.linalg.norm((a.astype(np.complex128) - b.astype(np.complex128)).ravel())
    den = np.linalg.norm(b.astype(np.complex128).ravel())
    return float(num / den) if den else float(num)
