"""Device-side waits end (the library's failure detection without a GPU fault).

Every kernel that waits on an mbarrier bounds the wait by %globaltimer, flags
the context and returns when it gives up; the host reports FD2D_ERR_TIMEOUT
and the context stays usable.  fd2d_check_bounded_wait runs that path on a
barrier nothing completes (no copy, no other thread), with a short limit: the
call must come back with FD2D_ERR_TIMEOUT after about the limit, and a solve
on the same context afterwards must give the same results as on a fresh one.
"""
import time

import numpy as np
import pytest

from tests.problems import media, small_cfg, stations

pytestmark = pytest.mark.gpu

ERR_ARG, ERR_TIMEOUT = 1, 6


def _green(ctx, cfg, mu, rho, src, rec):
    from fd2d_noise_gb300 import solvers
    with solvers.bound_context(ctx):
        G, _, s = solvers.run_forward1_green(mu, rho, src, rec, 0, cfg=cfg, precision="fp32")
    return G, s


def test_a_wait_nothing_completes_gives_up_and_the_context_stays_usable(fd2d_lib):
    from fd2d_noise_gb300 import _lib
    cfg = small_cfg(nx=60, nz=50, nt=40, K=6, fs=2, order=4)
    mu, rho = media(cfg, seed=3)
    src, rec = stations(cfg, 1, seed=4), stations(cfg, 3, seed=5)
    ctx = _lib.Context(0, _lib.PREC_FP32)
    fresh = _lib.Context(0, _lib.PREC_FP32)
    try:
        for limit_us in (20000, 200000):
            t0 = time.perf_counter()
            st = ctx.L.fd2d_check_bounded_wait(ctx.h, limit_us)
            dt = time.perf_counter() - t0
            assert st == ERR_TIMEOUT, _lib.STATUS_NAMES.get(st, st)
            assert b"bounded device-side wait" in ctx.L.fd2d_last_error(ctx.h)
            assert limit_us * 1e-6 <= dt < limit_us * 1e-6 + 2.0
        assert ctx.L.fd2d_check_bounded_wait(ctx.h, 0) == ERR_ARG
        assert ctx.L.fd2d_check_bounded_wait(ctx.h, 3000000) == ERR_ARG
        # the flag was consumed: solves on the same context run and agree with a fresh context
        G1, s1 = _green(ctx, cfg, mu, rho, src, rec)
        G0, s0 = _green(fresh, cfg, mu, rho, src, rec)
        assert np.abs(s0).max() > 0
        assert np.array_equal(G1, G0) and np.array_equal(s1, s0)
    finally:
        ctx.close()
        fresh.close()
