"""The allocation-free entry point, fd2d_forward1_seismograms_noalloc.

It exists for callers that must not allocate GPU memory (a fixed device-memory
budget, or a host runtime that owns the allocator): its working memory is a
statically sized device array inside libfd2d.  Called through the C ABI, its
seismograms must equal those of the ordinary entry point fd2d_forward1_green
(FP32, mode 0) on the same inputs bit for bit -- both run the same step kernel
with the same roundings -- on two calls in a row, since the second call reuses
the array the first one left behind; they also stay within the FP32 bound of
the oracle.  This file is collected last so that a run stopping at the first
failure has run everything else; it also passes on its own in a fresh process.
"""
import ctypes

import numpy as np
import pytest

from tests.problems import media, rel_l2, small_cfg, stations

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def lib(fd2d_lib):
    return fd2d_lib


def _reference(cfg, mu, rho, src, rec):
    from fd2d_noise_gb300 import solvers
    _, _, seis = solvers.run_forward1_green(mu, rho, src, rec, 0, cfg=cfg, precision="fp32")
    return seis


def _noalloc(lib, cfg, mu_d, rho_d, src, rec, stream="side"):
    """One call through the C ABI; ``stream`` "side" queues on a stream of its
    own (ordered after torch's current stream), None on the default stream."""
    import torch
    from fd2d_noise_gb300 import _lib
    nr = rec.shape[0]
    out = torch.full((max(nr, 1) * cfg.nt,), float("nan"), dtype=torch.float64, device="cuda")
    src_h = np.asfortranarray(src, dtype=np.float64)
    rec_h = np.asfortranarray(rec, dtype=np.float64).reshape(nr, 2)
    c = cfg.to_c()
    sp = None
    if stream == "side":
        side = torch.cuda.Stream()
        side.wait_stream(torch.cuda.current_stream())  # inputs and `out` are written there
        sp = ctypes.c_void_p(side.cuda_stream)
    st = lib.fd2d_forward1_seismograms_noalloc(
        ctypes.byref(c), ctypes.c_void_p(mu_d.data_ptr()), ctypes.c_void_p(rho_d.data_ptr()),
        ctypes.c_void_p(src_h.ctypes.data), src_h.shape[0], ctypes.c_void_p(rec_h.ctypes.data), nr,
        ctypes.c_void_p(out.data_ptr()) if nr else None, sp)
    _lib.check(st)
    return out[:nr * cfg.nt].cpu().numpy().reshape(nr, cfg.nt, order="F")


@pytest.mark.parametrize("stream", ["side", None], ids=["own_stream", "default_stream"])
@pytest.mark.parametrize("ns", [1, 3])
@pytest.mark.parametrize("order", [4, 8])
def test_noalloc_matches_ordinary_entry_twice(lib, oracle, order, ns, stream):
    import torch
    from fd2d_noise_gb300.device import to_device
    cfg = small_cfg(nx=70, nz=52, nt=90, order=order, K=16, fs=5, fw=1)
    mu, rho = media(cfg, seed=3)
    src = stations(cfg, ns, seed=5)
    rec = stations(cfg, 6, seed=6)
    ref = _reference(cfg, mu, rho, src, rec)
    _, _, so = oracle.forward1_green(cfg, mu, rho, src, rec, 0)
    mu_d, rho_d = to_device(mu, np.float64), to_device(rho, np.float64)
    for call in range(2):
        got = _noalloc(lib, cfg, mu_d, rho_d, src, rec, stream)
        assert np.all(np.isfinite(got)), call
        assert np.array_equal(got, ref), (call, rel_l2(got, ref))
        assert rel_l2(got, so) < 1e-4, (call, rel_l2(got, so))
    torch.cuda.synchronize()


def test_noalloc_without_receivers(lib):
    """nr = 0 (no seismograms pointer) runs and leaves the array usable: the
    next call with receivers still matches the ordinary entry point."""
    from fd2d_noise_gb300.device import to_device
    cfg = small_cfg(nx=70, nz=52, nt=60, order=4, K=16, fs=5, fw=1)
    mu, rho = media(cfg, seed=4)
    src, rec = stations(cfg, 1, seed=7), stations(cfg, 4, seed=8)
    mu_d, rho_d = to_device(mu, np.float64), to_device(rho, np.float64)
    empty = _noalloc(lib, cfg, mu_d, rho_d, src, np.zeros((0, 2)))
    assert empty.shape == (0, cfg.nt)
    got = _noalloc(lib, cfg, mu_d, rho_d, src, rec)
    assert np.array_equal(got, _reference(cfg, mu, rho, src, rec))


def test_noalloc_at_600x600(lib):
    """The documented size: a 600x600 grid at order 8 fits the scratch array
    (9 pitched FP32 planes of 608 x 600 floats); a short nt keeps it quick."""
    from fd2d_noise_gb300.device import to_device
    from fd2d_noise_gb300.workloads import single_600_o8
    w = single_600_o8(nt=120)
    cfg = w.cfg
    rec = w.receivers[:8]
    mu_d, rho_d = to_device(w.mu, np.float64), to_device(w.rho, np.float64)
    ref = _reference(cfg, w.mu, w.rho, w.ref_stations[:1], rec)
    assert np.abs(ref).max() > 0
    for call in range(2):
        got = _noalloc(lib, cfg, mu_d, rho_d, w.ref_stations[:1], rec)
        assert np.array_equal(got, ref), (call, rel_l2(got, ref))


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
