"""The allocation-free entry point, fd2d_forward1_seismograms_noalloc.

It exists for callers that must not allocate GPU memory (a fixed device-memory
budget, or a host runtime that owns the allocator): its working memory is a
statically sized device array inside libfd2d.  Called through the C ABI, its
seismograms must equal those of the ordinary entry point fd2d_forward1_green
(FP32, mode 0) on the same inputs -- on two calls in a row, since the second
call reuses the array the first one left behind.  This file is collected last
so that a run stopping at the first failure has run everything else; it also
passes on its own in a fresh process.
"""
import ctypes

import numpy as np
import pytest

from tests.problems import media, small_cfg, stations

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def lib(fd2d_lib):
    return fd2d_lib


def _reference(cfg, mu, rho, src, rec):
    from fd2d_noise_gb300 import solvers
    _, _, seis = solvers.run_forward1_green(mu, rho, src, rec, 0, cfg=cfg, precision="fp32")
    return seis


def _noalloc(lib, cfg, mu_d, rho_d, src, rec):
    import torch
    from fd2d_noise_gb300 import _lib
    nr = rec.shape[0]
    out = torch.full((nr * cfg.nt,), float("nan"), dtype=torch.float64, device="cuda")
    src_h = np.asfortranarray(src, dtype=np.float64)
    rec_h = np.asfortranarray(rec, dtype=np.float64)
    c = cfg.to_c()
    st = lib.fd2d_forward1_seismograms_noalloc(
        ctypes.byref(c), ctypes.c_void_p(mu_d.data_ptr()), ctypes.c_void_p(rho_d.data_ptr()),
        ctypes.c_void_p(src_h.ctypes.data), src_h.shape[0], ctypes.c_void_p(rec_h.ctypes.data), nr,
        ctypes.c_void_p(out.data_ptr()), ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    _lib.check(st)
    return out.cpu().numpy().reshape(nr, cfg.nt, order="F")


@pytest.mark.parametrize("order", [4, 8])
def test_noalloc_matches_ordinary_entry_twice(lib, order):
    import torch
    from fd2d_noise_gb300.device import to_device
    cfg = small_cfg(nx=70, nz=52, nt=90, order=order, K=16, fs=5, fw=1)
    mu, rho = media(cfg, seed=3)
    src = stations(cfg, 1, seed=5)
    rec = stations(cfg, 6, seed=6)
    ref = _reference(cfg, mu, rho, src, rec)
    mu_d, rho_d = to_device(mu, np.float64), to_device(rho, np.float64)
    for call in range(2):
        got = _noalloc(lib, cfg, mu_d, rho_d, src, rec)
        assert np.all(np.isfinite(got)), call
        err = np.linalg.norm(got - ref) / np.linalg.norm(ref)
        assert err < 1e-6, (call, err)
    torch.cuda.synchronize()


def test_noalloc_rejects_grids_beyond_its_scratch(lib):
    from fd2d_noise_gb300 import _lib
    from fd2d_noise_gb300.config import Config
    cfg = Config(nx=1200, nz=1200, Lx=4e5, Lz=4e5, dt=0.02, nt=4)
    c = cfg.to_c()
    one = np.zeros(2)
    st = lib.fd2d_forward1_seismograms_noalloc(ctypes.byref(c), ctypes.c_void_p(8), ctypes.c_void_p(8),
                                               ctypes.c_void_p(one.ctypes.data), 1,
                                               ctypes.c_void_p(one.ctypes.data), 0, None, None)
    assert st == 2  # FD2D_ERR_SHAPE, before touching any device memory
    assert b"scratch" in lib.fd2d_last_error(None)
    with pytest.raises(_lib.FD2DError):
        _lib.check(st)
