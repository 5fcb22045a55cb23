"""Chunked contractions: with the DFT split into 32-snapshot chunks (FP64
accumulation across chunks, coefficient-image K offsets) and the injection
planes evaluated 128 events at a time (image column offsets), the FP32 solvers
give the results of the single-chunk runs and of the oracle."""
import numpy as np
import pytest

from tests.problems import media, noise_source, rel_l2, small_cfg, stations

pytestmark = pytest.mark.gpu


def _run(cfg, mu, rho, spec, sd, src, rec):
    from fd2d_noise_gb300 import solvers
    G, _, s_g = solvers.run_forward1_green(mu, rho, src, rec, 0, cfg=cfg, precision="fp32")
    c, _ = solvers.run_forward2_correlation(mu, rho, G, spec, sd, rec, 0, cfg=cfg, precision="fp32")
    # adjoint with point sources and the DFT of u (mode 1), then the field
    # source built from that spectrum (3-D stf: injection, mode 0)
    stf = np.random.default_rng(5).standard_normal((rec.shape[0], cfg.ntc)).astype(np.complex128)
    _, S, _, _ = solvers.run_noise_adjoint(mu, rho, None, stf, rec, None, None, None, None, 1, cfg=cfg,
                                           precision="fp32")
    K, _, _, _ = solvers.run_noise_adjoint(mu, rho, None, S, rec, None, spec, sd, None, 0, cfg=cfg,
                                           precision="fp32")
    return G, c, S, K


def test_small_chunks_match_single_chunk_and_oracle(fd2d_lib):
    from fd2d_noise_gb300 import _lib, solvers
    from oracle import pyoracle
    cfg = small_cfg(nx=40, nz=36, nt=200, K=12, fs=1)
    mu, rho = media(cfg, seed=3)
    spec, sd = noise_source(cfg, seed=3)
    src, rec = stations(cfg, 1, seed=30), stations(cfg, 4, seed=31)
    ref = _run(cfg, mu, rho, spec, sd, src, rec)
    ctx = solvers.context(0, "fp32")
    _lib.check(ctx.L.fd2d_ctx_set_chunks(ctx.h, 32, 128), ctx.h)
    try:
        got = _run(cfg, mu, rho, spec, sd, src, rec)
    finally:
        _lib.check(ctx.L.fd2d_ctx_set_chunks(ctx.h, 0, 0), ctx.h)
    # FP32 sums over 32-snapshot chunks, FP64 across chunks, versus one FP32
    # sum over all snapshots: the two roundings differ at the FP32 level
    for a, b in zip(got, ref):
        assert rel_l2(a, b) < 1e-5
    G, _, _ = pyoracle.forward1_green(cfg, mu, rho, src, rec, 0)
    c, _ = pyoracle.forward2_correlation(cfg, mu, rho, G, spec, sd, rec, 0)
    assert rel_l2(got[0], G) < 1e-4 and rel_l2(got[1], c) < 1e-4
