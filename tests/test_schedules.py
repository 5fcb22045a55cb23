"""Snapshot schedules and receiver indices, checked on the oracle (CPU).

The reference stores a snapshot *before* the update of step n
(code/run_forward1_green.m:133-137 when mod(n+nt-1, fw_nth) == 0;
code/run_forward2_correlation.m:182-186 when mod(n, fw_nth) == 0) and records
the receivers *after* it (run_forward1_green.m:187-189,
run_forward2_correlation.m:246-248).  So snapshot i, taken at step n, holds at
the receiver nodes exactly single(seismograms(:, n-1)) (zero for n = 1).  The
full-size GPU test (test_gpu_fullsize.py) relies on this relation to check
receiver indexing and the schedules bit-exactly at sizes the oracle cannot run
in seconds; here it is pinned on the oracle itself.
"""
import numpy as np

from tests.problems import media, noise_source, small_cfg, stations


def green_snapshot_steps(cfg):
    """1-based steps n at which run_forward1_green stores G_out."""
    return [n for n in range(1, cfg.nt + 1) if (n + cfg.nt - 1) % cfg.fw_nth == 0]


def correlation_snapshot_steps(cfg):
    """1-based steps n at which run_forward2_correlation stores C_out."""
    return [n for n in range(1, cfg.ntc + 1) if n % cfg.fw_nth == 0]


def assert_snapshots_match_traces(snaps, seis, ix, iz, steps):
    """snaps nx-by-nz-by-n float32, seis nr-by-nsteps, ix/iz 0-based nodes."""
    assert snaps.shape[2] == len(steps)
    for i, n in enumerate(steps):
        want = np.zeros(ix.size, np.float32) if n == 1 else np.asarray(seis[:, n - 2], np.float32)
        got = snaps[ix, iz, i]
        assert np.array_equal(got, want), (i, n, got, want)


def test_oracle_snapshots_hold_previous_traces(oracle):
    cfg = small_cfg(nx=44, nz=38, nt=50, order=4, K=12, fs=5, fw=3)
    mu, rho = media(cfg, 1)
    src, rec = stations(cfg, 1, 2), stations(cfg, 5, 3)
    ix, iz = oracle.nearest_indices(cfg, rec)
    G, G_out, seis = oracle.forward1_green(cfg, mu, rho, src, rec, 1)
    assert np.abs(seis).max() > 0
    assert_snapshots_match_traces(G_out, seis, ix, iz, green_snapshot_steps(cfg))
    spec, sd = noise_source(cfg)
    corr, C_out = oracle.forward2_correlation(cfg, mu, rho, G, spec, sd, rec, 1)
    assert np.abs(corr).max() > 0
    assert_snapshots_match_traces(C_out, corr, ix, iz, correlation_snapshot_steps(cfg))
