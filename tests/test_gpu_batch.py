"""Batched reference stations (fd2d_correlation_batch) against single solves.

Each job is one station of code/calculate_data.m:189-202 (Green function, then
correlation).  The batch advances jobs of one geometry together (one launch per
time step for all of them) and runs the other jobs' loops concurrently; its
correlations must equal those of the one-at-a-time entry points, for jobs of
different grid sizes and lengths, in both precisions and memory-budget
groupings.
"""
import numpy as np
import pytest

from tests.problems import media, noise_source, rel_l2, small_cfg, stations

pytestmark = pytest.mark.gpu


def _jobs():
    out = []
    # jobs 0, 2 and 3 share a geometry: one launch per step advances all three (lanes)
    for seed, kw in enumerate([dict(nx=40, nz=36, nt=60, order=4), dict(nx=52, nz=44, nt=48, order=8),
                               dict(nx=40, nz=36, nt=60, order=4), dict(nx=40, nz=36, nt=60, order=4)]):
        cfg = small_cfg(K=20, fs=5, fw=1, **kw)
        mu, rho = media(cfg, seed=seed)
        spec, sd = noise_source(cfg, seed=seed)
        src = stations(cfg, 1, seed=10 + seed)
        rec = stations(cfg, 5, seed=20 + seed)
        out.append(dict(cfg=cfg, mu=mu, rho=rho, spec=spec, sd=sd, src=src, rec=rec))
    return out


def _single(job, prec):
    from fd2d_noise_gb300 import solvers
    G, _, _ = solvers.run_forward1_green(job["mu"], job["rho"], job["src"], job["rec"], 0, cfg=job["cfg"],
                                         precision=prec)
    c, _ = solvers.run_forward2_correlation(job["mu"], job["rho"], G, job["spec"], job["sd"], job["rec"], 0,
                                            cfg=job["cfg"], precision=prec)
    return c


@pytest.mark.parametrize("prec", ["fp32", "fp64"])
@pytest.mark.parametrize("budget", [0, 1])
def test_batch_matches_single_solves(fd2d_lib, prec, budget):
    import torch
    from fd2d_noise_gb300 import _lib
    from fd2d_noise_gb300.device import DeviceSession, to_device
    jobs = _jobs()
    sess = DeviceSession(jobs[0]["cfg"], 0, prec)
    if budget:
        _lib.check(sess.ctx.L.fd2d_ctx_set_memory_budget(sess.ctx.h, 1), sess.ctx.h)  # one job per group
    dj = []
    for j in jobs:
        c = j["cfg"]
        dj.append(dict(cfg=c, mu=to_device(j["mu"], np.float64), rho=to_device(j["rho"], np.float64),
                       spectrum=to_device(j["spec"], np.float64), source_dist=to_device(j["sd"], np.float64),
                       src=to_device(j["src"], np.float64), rec=to_device(j["rec"], np.float64),
                       nr=j["rec"].shape[0],
                       out=torch.zeros(j["rec"].shape[0] * c.ntc, dtype=torch.float64, device="cuda")))
    for rep in range(3):  # launched eagerly, then captured, then replayed
        sess.correlation_batch(dj)
        sess.ctx.synchronize()
        groups = sess.ctx.last_batch()
        if prec == "fp32" and not budget:
            assert sorted(groups) == [1, 3], groups  # jobs 0, 2, 3 are lanes of one launch
        else:
            assert sum(groups) == len(jobs) and max(groups) == 1, groups
        for j, d in zip(jobs, dj):
            got = d["out"].cpu().numpy().reshape(j["rec"].shape[0], j["cfg"].ntc, order="F")
            ref = _single(j, prec)
            assert rel_l2(got, ref) < (1e-12 if prec == "fp64" else 1e-6), rep


def _uneven_jobs(sizes=(256, 384, 512, 800), nts=(150, 220, 180, 120, 260)):
    """Stations on the grid sizes of the uneven-batch configuration (order 4,
    four frequency bands, dt from CFL 0.5 at 4000 m/s, taper 30 points), each
    with its own nt, short enough for a test."""
    from fd2d_noise_gb300.workloads import batch_uneven
    b = batch_uneven(n_stations=16, K=24, nr=6, sizes=sizes, nt_range=(100, 300))
    picked = [next(w for w in b.stations if w.cfg.nx == nx) for nx in sizes]
    picked.append(next(w for w in b.stations if w.cfg.nx == sizes[-1] and w is not picked[-1]))
    out = []
    for i, w in enumerate(picked):
        cfg = w.cfg.replace(nt=nts[i])
        out.append(dict(cfg=cfg, mu=w.mu, rho=w.rho, spec=w.spectrum, sd=w.source_dist, src=w.ref_stations,
                        rec=w.receivers))
    return out


def test_uneven_grids_advance_in_one_launch_per_step(fd2d_lib):
    """Stations on 256^2 to 800^2 grids with different nt: one multi-geometry
    launch per time step (one launch group of every job), correlations bit for
    bit those of the single solves, on the eager run, the captured run and a
    replay."""
    import torch
    from fd2d_noise_gb300.device import DeviceSession, to_device
    jobs = _uneven_jobs()
    assert len({j["cfg"].nx for j in jobs}) >= 3 and len({j["cfg"].nt for j in jobs}) == len(jobs)
    sess = DeviceSession(jobs[0]["cfg"], 0, "fp32")
    dj = []
    for j in jobs:
        c = j["cfg"]
        n_dist = j["sd"].shape[2] if j["sd"].ndim == 3 else 1
        dj.append(dict(cfg=c, mu=to_device(j["mu"], np.float64), rho=to_device(j["rho"], np.float64),
                       spectrum=to_device(j["spec"], np.float64), source_dist=to_device(j["sd"], np.float64),
                       n_dist=n_dist, src=to_device(j["src"], np.float64), rec=to_device(j["rec"], np.float64),
                       nr=j["rec"].shape[0],
                       out=torch.zeros(j["rec"].shape[0] * c.ntc, dtype=torch.float64, device="cuda")))
    refs = [_single(j, "fp32") for j in jobs]
    for rep in range(3):
        for d in dj:
            d["out"].zero_()
        sess.correlation_batch(dj)
        sess.ctx.synchronize()
        assert sess.ctx.last_batch() == [len(jobs)], sess.ctx.last_batch()
        for i, (j, d, ref) in enumerate(zip(jobs, dj, refs)):
            got = d["out"].cpu().numpy().reshape(j["rec"].shape[0], j["cfg"].ntc, order="F")
            assert np.abs(ref).max() > 0
            assert np.array_equal(got, ref), (rep, i, rel_l2(got, ref))
    sess.ctx.close()
