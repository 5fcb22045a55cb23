"""CPU-only checks: host-side setup, oracle helpers, library load and symbols."""
import os
import re

import numpy as np
import pytest

from fd2d_noise_gb300.config import matlab_colon, n_fw_green, n_fw_corr
from tests.problems import small_cfg

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_colon_matches_endpoints_and_length():
    x = matlab_colon(0.0, 4e5 / 299, 4e5)
    assert x.size == 300 and x[0] == 0.0 and x[-1] == 4e5
    t = matlab_colon(-119.9, 0.1, 119.9)
    assert t.size == 2399 and t[0] == -119.9 and t[-1] == 119.9
    # symmetric construction: midpoint exact
    assert t[1199] == 0.0
    f = matlab_colon(0.02, 0.0015, 0.2)
    assert f.size == 121 and abs(f[-1] - 0.2) < 1e-15


def test_stagger_coefficients_from_taylor_conditions(oracle):
    assert np.allclose(oracle.stagger_coeffs(4), [9 / 8, -1 / 24], rtol=0, atol=1e-15)
    assert np.allclose(oracle.stagger_coeffs(8), [1225 / 1024, -245 / 3072, 49 / 5120, -5 / 7168],
                       rtol=0, atol=1e-15)
    assert np.allclose(oracle.stagger_coeffs(6), [75 / 64, -25 / 384, 3 / 640], rtol=0, atol=1e-15)


def test_taper_and_grid(oracle):
    cfg = small_cfg()
    x, z, ab = oracle.setup_arrays(cfg)
    assert np.array_equal(x, matlab_colon(0.0, cfg.dx, cfg.Lx))
    w = cfg.absorb_width
    X = x[:, None] * np.ones((1, cfg.nz))
    ref = np.where(X > w, 1.0, np.exp(-(X - w) ** 2 / (2 * w) ** 2))
    ref = ref * np.where(X < cfg.Lx - w, 1.0, np.exp(-(X - (cfg.Lx - w)) ** 2 / (2 * w) ** 2))
    Z = np.ones((cfg.nx, 1)) * z[None, :]
    ref = ref * np.where(Z > w, 1.0, np.exp(-(Z - w) ** 2 / (2 * w) ** 2))
    ref = ref * np.where(Z < cfg.Lz - w, 1.0, np.exp(-(Z - (cfg.Lz - w)) ** 2 / (2 * w) ** 2))
    assert np.allclose(ab, ref, rtol=1e-14, atol=0)
    assert ab[cfg.nx // 2, cfg.nz // 2] == 1.0


def test_nearest_node_ties_go_low(oracle):
    cfg = small_cfg()
    dx = cfg.dx
    pts = np.array([[2.5 * dx, 3.5 * cfg.dz], [dx * 0.49, 0.0], [cfg.Lx + 5, cfg.Lz]])
    ix, iz = oracle.nearest_indices(cfg, pts)
    assert list(ix) == [2, 0, cfg.nx - 1]
    assert list(iz) == [3, 0, cfg.nz - 1]


def test_interpol_matrix_rows_sum_to_one_inside(oracle):
    M = oracle.interpol_matrix(24, 4)
    assert M.shape == (24, 4)
    # band b covers 6 frequencies; inside the outer half-bands the hat weights sum to 1,
    # the outermost half-bands have no neighbour to share with (code/run_forward2_correlation.m:137-160)
    assert np.allclose(M[3:21].sum(axis=1), 1.0)
    assert np.allclose(M[[0, 1, 2]].sum(axis=1), [2 / 3, 5 / 6, 1.0])
    assert np.allclose(M[[21, 22, 23]].sum(axis=1), [5 / 6, 2 / 3, 0.5])
    assert np.array_equal(oracle.interpol_matrix(10, 0), np.ones((10, 1)))


def test_snapshot_counts():
    cfg = small_cfg(nt=60, fw=5)
    assert n_fw_green(cfg) == len([n for n in range(60, 120) if n % 5 == 0])
    assert n_fw_corr(cfg) == (2 * 60 - 1) // 5


def _declared_symbols():
    hdr = open(os.path.join(ROOT, "include", "fd2d.h")).read()
    return sorted(set(re.findall(r"\b(fd2d_[a-z0-9_]+)\s*\(", hdr)))


def test_library_exports_every_declared_symbol(fd2d_lib):
    from fd2d_noise_gb300 import _lib
    syms = _declared_symbols()
    assert len(syms) >= 13
    for s in syms:
        assert hasattr(fd2d_lib, s), s
    assert set(_lib.EXPORTED) <= set(syms)
    assert fd2d_lib.fd2d_abi_version() == 1


def test_query_sizes_without_gpu(fd2d_lib):
    from fd2d_noise_gb300 import _lib
    cfg = small_cfg(nt=60, fw=5, nb=3)
    s = _lib.query_sizes(cfg, 7)
    assert s.ntc == 119 and s.n_fw_green == n_fw_green(cfg) and s.n_fw_corr == 119 // 5
    assert s.n_kernel_planes == 4 and s.G_fft == cfg.npts * cfg.n_sample
    assert s.seis_corr == 7 * 119
    with pytest.raises(_lib.FD2DError):
        _lib.query_sizes(small_cfg(order=5), 1)
    with pytest.raises(_lib.FD2DError):
        _lib.query_sizes(small_cfg(nb=1), 1)
