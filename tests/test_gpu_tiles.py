"""Step-kernel tile shapes: 32x16, 32x30, 32x32 and 32x40 tiles give bit-identical
results (each point's stencil arithmetic does not depend on the tiling, only
which CTA does it), and the tuner picks one of them per grid, order and lane count,
keeps it for later runs, and honours a forced shape or the size rule."""
import numpy as np
import pytest

from tests.problems import media, noise_source, small_cfg, stations

pytestmark = pytest.mark.gpu


def _run(cfg, mu, rho, spec, sd, src, rec):
    from fd2d_noise_gb300 import solvers
    G, _, s_g = solvers.run_forward1_green(mu, rho, src, rec, 0, cfg=cfg, precision="fp32")
    c, _ = solvers.run_forward2_correlation(mu, rho, G, spec, sd, rec, 0, cfg=cfg, precision="fp32")
    stf = np.random.default_rng(5).standard_normal((rec.shape[0], cfg.ntc)).astype(np.complex128)
    _, S, _, _ = solvers.run_noise_adjoint(mu, rho, None, stf, rec, None, None, None, None, 1, cfg=cfg,
                                           precision="fp32")
    K, _, _, _ = solvers.run_noise_adjoint(mu, rho, None, S, rec, None, spec, sd, None, 0, cfg=cfg,
                                           precision="fp32")
    # stored wavefields (mode 1): single(v) and single(u) before each stored step
    _, G_out, _ = solvers.run_forward1_green(mu, rho, src, rec, 1, cfg=cfg, precision="fp32")
    _, C_out = solvers.run_forward2_correlation(mu, rho, G, spec, sd, rec, 1, cfg=cfg, precision="fp32")
    return G, s_g, c, S, K, G_out, C_out


@pytest.mark.parametrize("order", [4, 8])
def test_tile_rows_give_identical_results(fd2d_lib, order):
    from fd2d_noise_gb300 import _lib, solvers
    # 150 x 141: interior tiles (no edge selects) and ragged edge tiles in both shapes
    cfg = small_cfg(nx=150, nz=141, nt=90, K=10, fs=3, fw=4, order=order)
    mu, rho = media(cfg, seed=4)
    spec, sd = noise_source(cfg, seed=4)
    src, rec = stations(cfg, 1, seed=40), stations(cfg, 6, seed=41)
    ctx = _lib.Context(0, _lib.PREC_FP32)
    out = {}
    try:
        with solvers.bound_context(ctx):
            for rows in (16, 30, 32, 40):
                ctx.set_tile_rows(rows)
                out[rows] = _run(cfg, mu, rho, spec, sd, src, rec)
                assert ctx.last_tile_rows() == rows
    finally:
        ctx.close()
    for rows in (30, 32, 40):
        for a, b in zip(out[16], out[rows]):
            assert np.array_equal(a, b)


def test_tuner_keeps_its_choice(fd2d_lib):
    from fd2d_noise_gb300 import _lib, solvers
    cfg = small_cfg(nx=96, nz=80, nt=40, K=6, fs=2, order=4)
    mu, rho = media(cfg, seed=6)
    src, rec = stations(cfg, 1, seed=60), stations(cfg, 3, seed=61)
    ctx = _lib.Context(0, _lib.PREC_FP32)
    try:
        assert ctx.last_tile_rows() == 0
        with solvers.bound_context(ctx):
            G1, _, s1 = solvers.run_forward1_green(mu, rho, src, rec, 0, cfg=cfg, precision="fp32")
            first = ctx.last_tile_rows()
            assert first in (16, 30, 32, 40)
            G2, _, s2 = solvers.run_forward1_green(mu, rho, src, rec, 0, cfg=cfg, precision="fp32")
            assert ctx.last_tile_rows() == first
        # the timed trial steps leave no trace in the results
        assert np.array_equal(G1, G2) and np.array_equal(s1, s2)
        with pytest.raises(_lib.FD2DError):
            ctx.set_tile_rows(24)
    finally:
        ctx.close()


def test_size_rule(fd2d_lib):
    from fd2d_noise_gb300 import _lib, solvers
    ctx = _lib.Context(0, _lib.PREC_FP32)
    try:
        ctx.set_tile_rows(_lib.TILE_ROWS_RULE)
        with solvers.bound_context(ctx):
            # 9 tiles of 32 rows: far fewer than four per SM, so 16 rows
            cfg = small_cfg(nx=96, nz=80, nt=20, K=4, fs=2, order=4)
            mu, rho = media(cfg, seed=7)
            solvers.run_forward1_green(mu, rho, stations(cfg, 1, seed=70), stations(cfg, 2, seed=71), 0,
                                       cfg=cfg, precision="fp32")
            assert ctx.last_tile_rows() == 16
    finally:
        ctx.close()
