"""Two time steps per launch (k32_step2, FD orders 2 and 4).

The Green-function and correlation loops may advance two steps in one launch,
recomputing the first step on a wider halo ring.  Every point is updated by
the same rounded operations, so spectra, seismograms, correlations and stored
wavefields must be bit for bit those of one step per launch -- on edge and
interior tiles, with point sources, receivers, DFT snapshots on either step of
a pair (freq_samp 1 puts them on both), injection planes, stored wavefields
(modes 1, 11: single(v) or single(u) before either step of a pair), an odd
number of steps, lanes, and every tile shape.  The time-depth tuner picks one depth per grid and keeps it;
orders 6/8 and tiles with more receivers than the kernel keeps run one step
per launch.
"""
import numpy as np
import pytest

from tests.problems import media, noise_source, small_cfg, stations

pytestmark = pytest.mark.gpu


def _green_corr(cfg, mu, rho, spec, sd, src, rec, mode=0):
    from fd2d_noise_gb300 import solvers
    G, G_out, s_g = solvers.run_forward1_green(mu, rho, src, rec, mode, cfg=cfg, precision="fp32")
    c, C_out = solvers.run_forward2_correlation(mu, rho, G, spec, sd, rec, mode, cfg=cfg, precision="fp32")
    return [G, s_g, c] + ([G_out, C_out] if mode else [])


def _with_depths(cfg, seed, depths=(1, 2), rows=None, mode=0, n_rec=6, rec=None):
    from fd2d_noise_gb300 import _lib, solvers
    mu, rho = media(cfg, seed=seed)
    spec, sd = noise_source(cfg, seed=seed)
    src = stations(cfg, 1, seed=10 + seed)
    if rec is None:
        # receivers within a few wavelengths of the source, so every trace is nonzero
        off = np.random.default_rng(20 + seed).uniform(-12, 12, (n_rec, 2)) * np.array([cfg.dx, cfg.dz])
        rec = np.clip(src + off, [2 * cfg.dx, 2 * cfg.dz], [cfg.Lx - 2 * cfg.dx, cfg.Lz - 2 * cfg.dz])
    ctx = _lib.Context(0, _lib.PREC_FP32)
    out, used = {}, {}
    try:
        with solvers.bound_context(ctx):
            if rows:
                ctx.set_tile_rows(rows)
            for d in depths:
                ctx.set_time_depth(d)
                out[d] = _green_corr(cfg, mu, rho, spec, sd, src, rec, mode)
                used[d] = ctx.last_time_depth()
    finally:
        ctx.close()
    return out, used


CASES = [
    # nx, nz, nt, fs: ragged edges everywhere; an odd nt ends on a single step
    dict(nx=70, nz=52, nt=61, fs=1),
    dict(nx=150, nz=141, nt=90, fs=3),  # interior tiles without edge selects
    dict(nx=257, nz=200, nt=50, fs=5),
    dict(nx=33, nz=17, nt=21, fs=2),  # grid smaller than one loaded box
]


@pytest.mark.parametrize("order", [2, 4])
@pytest.mark.parametrize("case", range(len(CASES)))
def test_two_steps_per_launch_are_bit_identical(fd2d_lib, order, case):
    cfg = small_cfg(K=8, order=order, **CASES[case])
    out, used = _with_depths(cfg, seed=3 + case)
    assert used == {1: 1, 2: 2}
    for a, b in zip(out[1], out[2]):
        assert np.abs(a).max() > 0
        assert np.array_equal(a, b)


@pytest.mark.parametrize("rows", [16, 30, 40])
def test_every_tile_shape(fd2d_lib, rows):
    cfg = small_cfg(nx=130, nz=97, nt=40, K=6, fs=2, order=4)
    out, used = _with_depths(cfg, seed=9, rows=rows)
    assert used[2] == 2
    for a, b in zip(out[1], out[2]):
        assert np.array_equal(a, b)


def test_stored_wavefields_inside_pairs(fd2d_lib):
    """Mode 1 stores single(v) / single(u) before every fw-th step (fw 3: on
    the first and on the second step of pairs); everything matches."""
    cfg = small_cfg(nx=96, nz=88, nt=47, K=6, fs=2, fw=3, order=4)
    out, used = _with_depths(cfg, seed=12, mode=1)
    assert used[2] == 2
    for a, b in zip(out[1], out[2]):
        assert np.array_equal(a, b)


def test_lanes_of_a_batch(fd2d_lib):
    """Reference stations of one geometry as lanes of one launch, two steps per launch."""
    import torch
    from fd2d_noise_gb300 import _lib
    from fd2d_noise_gb300.device import DeviceSession, to_device
    cfg = small_cfg(nx=120, nz=100, nt=55, K=8, fs=5, order=4)
    jobs = []
    for seed in range(3):
        mu, rho = media(cfg, seed=seed)
        spec, sd = noise_source(cfg, seed=seed)
        src = stations(cfg, 1, seed=30 + seed)
        off = np.random.default_rng(40 + seed).uniform(-10, 10, (5, 2)) * np.array([cfg.dx, cfg.dz])
        rec = np.clip(src + off, [2 * cfg.dx, 2 * cfg.dz], [cfg.Lx - 2 * cfg.dx, cfg.Lz - 2 * cfg.dz])
        jobs.append(dict(cfg=cfg, mu=to_device(mu, np.float64), rho=to_device(rho, np.float64),
                         spectrum=to_device(spec, np.float64), source_dist=to_device(sd, np.float64),
                         src=to_device(src, np.float64), rec=to_device(rec, np.float64), nr=5,
                         out=torch.zeros(5 * cfg.ntc, dtype=torch.float64, device="cuda")))
    res = {}
    for d in (1, 2):
        sess = DeviceSession(cfg, 0, "fp32")
        _lib.check(sess.ctx.L.fd2d_ctx_set_time_depth(sess.ctx.h, d), sess.ctx.h)
        for j in jobs:
            j["out"].zero_()
        sess.correlation_batch(jobs)
        sess.ctx.synchronize()
        assert sess.ctx.last_batch() == [3]
        assert sess.ctx.last_time_depth() == d
        res[d] = [j["out"].cpu().numpy().copy() for j in jobs]
        sess.ctx.close()
    for a, b in zip(res[1], res[2]):
        assert np.abs(a).max() > 0 and np.array_equal(a, b)


def test_order_8_and_crowded_tiles_run_one_step_per_launch(fd2d_lib):
    cfg8 = small_cfg(nx=90, nz=80, nt=30, K=4, fs=2, order=8)
    _, used = _with_depths(cfg8, seed=1, depths=(2,))
    assert used[2] == 1
    # 40 receivers in one 32-point-wide tile: more than the kernel keeps per tile
    cfg = small_cfg(nx=90, nz=80, nt=30, K=4, fs=2, order=4)
    x = np.linspace(20e3, 60e3, 40)
    rec = np.column_stack([x, np.full(40, 40e3)])
    out, used = _with_depths(cfg, seed=2, rec=rec)
    assert used == {1: 1, 2: 1}
    for a, b in zip(out[1], out[2]):
        assert np.array_equal(a, b)


def test_tuner_keeps_its_choice(fd2d_lib):
    """Left at 0 the depth is timed once per grid (on an idle stream) and kept;
    the timed trial steps leave no trace in the results."""
    from fd2d_noise_gb300 import _lib, solvers
    cfg = small_cfg(nx=100, nz=90, nt=40, K=6, fs=2, order=4)
    mu, rho = media(cfg, seed=7)
    spec, sd = noise_source(cfg, seed=7)
    src, rec = stations(cfg, 1, seed=70), stations(cfg, 4, seed=71)
    ctx = _lib.Context(0, _lib.PREC_FP32)
    try:
        assert ctx.last_time_depth() == 0
        with solvers.bound_context(ctx):
            a = _green_corr(cfg, mu, rho, spec, sd, src, rec)
            first = ctx.last_time_depth()
            assert first in (1, 2)
            b = _green_corr(cfg, mu, rho, spec, sd, src, rec)
            assert ctx.last_time_depth() == first
            ctx.set_time_depth(1)
            c = _green_corr(cfg, mu, rho, spec, sd, src, rec)
        for x, y, z in zip(a, b, c):
            assert np.array_equal(x, y) and np.array_equal(x, z)
        with pytest.raises(_lib.FD2DError):
            ctx.set_time_depth(3)
    finally:
        ctx.close()


@pytest.mark.parametrize("name", ["plain_cpu_300", "structure_512"])
def test_full_size_workloads_are_bit_identical(fd2d_lib, name):
    """Configuration 1 (300², nt 1200, mode 0) and the structure-kernel grid
    (512², nt 2500, Green and correlation runs in mode 1 with fw 5, whose
    stored steps split the pairs) with one and two steps per launch."""
    from fd2d_noise_gb300 import _lib, solvers
    from fd2d_noise_gb300.workloads import WORKLOADS
    w = WORKLOADS[name]()
    mode = 1 if name == "structure_512" else 0
    ctx = _lib.Context(0, _lib.PREC_FP32)
    out = {}
    try:
        with solvers.bound_context(ctx):
            for d in (1, 2):
                ctx.set_time_depth(d)
                out[d] = _green_corr(w.cfg, w.mu, w.rho, w.spectrum, w.source_dist, w.ref_stations, w.receivers,
                                     mode)
                assert ctx.last_time_depth() == d
    finally:
        ctx.close()
    for a, b in zip(out[1], out[2]):
        assert np.abs(a).max() > 0
        assert np.array_equal(a, b)


def test_adjoint_runs_are_bit_identical(fd2d_lib):
    """The structure-kernel sequence: Green and correlation runs in mode 1
    (stored wavefields), adjoint mode 1 (point adjoint sources with per-step
    amplitudes, two of them on one node, K_mu against the stored correlation
    wavefield every fw steps, the DFT of u), adjoint mode 0 (the field source
    of that spectrum, K_s and K_mu) and adjoint mode 11 (u stored every fw
    steps) -- one and two steps per launch."""
    from fd2d_noise_gb300 import _lib, solvers
    cfg = small_cfg(nx=110, nz=96, nt=57, K=8, fs=3, fw=4, order=4)
    mu, rho = media(cfg, seed=21)
    spec, sd = noise_source(cfg, seed=21)
    src = stations(cfg, 1, seed=22)
    off = np.random.default_rng(23).uniform(-10, 10, (5, 2)) * np.array([cfg.dx, cfg.dz])
    rec = np.clip(src + off, [2 * cfg.dx, 2 * cfg.dz], [cfg.Lx - 2 * cfg.dx, cfg.Lz - 2 * cfg.dz])
    rec = np.vstack([rec, rec[2:3]])  # two adjoint sources on one node
    stf = np.random.default_rng(24).standard_normal((rec.shape[0], cfg.ntc)).astype(np.complex128)
    out = {}
    for d in (1, 2):
        ctx = _lib.Context(0, _lib.PREC_FP32)
        try:
            with solvers.bound_context(ctx):
                ctx.set_time_depth(d)
                G, G_out, _ = solvers.run_forward1_green(mu, rho, src, rec, 1, cfg=cfg, precision="fp32")
                _, C_out = solvers.run_forward2_correlation(mu, rho, G, spec, sd, rec, 1, cfg=cfg, precision="fp32")
                K1, S1, _, s1 = solvers.run_noise_adjoint(mu, rho, C_out, stf, rec, rec, None, None, None, 1,
                                                          cfg=cfg, precision="fp32")
                assert ctx.last_time_depth() == d
                K0, _, _, s0 = solvers.run_noise_adjoint(mu, rho, G_out, S1, None, rec, spec, sd, G, 0, cfg=cfg,
                                                         precision="fp32")
                assert ctx.last_time_depth() == d
                # mode 11: u stored before every fw-th step
                K11, _, U11, s11 = solvers.run_noise_adjoint(mu, rho, C_out, stf, rec, rec, None, None, None, 11,
                                                             cfg=cfg, precision="fp32")
                out[d] = [K1, S1, s1, K0, s0, K11, U11, s11, G_out, C_out]
        finally:
            ctx.close()
    for a, b in zip(out[1], out[2]):
        assert np.abs(a).max() > 0
        assert np.array_equal(a, b)
