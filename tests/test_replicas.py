"""Replicas over ranks (gloo, world size 2, CPU): station sharding, gathering of
per-station correlations and the FP64 kernel sum of
inversion/optlib_callback_fct/eval_objective_and_gradient.m:110.

The per-station solves here are the FP64 oracle on a tiny grid; what is tested
is the host logic around them: every station computed exactly once, results
identical to a one-process run, and the reduced kernel equal to the sum of the
per-station arrays.
"""
import os
import socket

import numpy as np
import pytest

from fd2d_noise_gb300.replicas import station_shard, sum_kernels


def test_shard_covers_every_station_once_and_balances():
    costs = [5.0, 1.0, 3.0, 3.0, 2.0, 8.0, 1.0]
    for world in (1, 2, 3, 4):
        parts = [station_shard(costs, world, r) for r in range(world)]
        flat = sorted(i for p in parts for i in p)
        assert flat == list(range(len(costs)))
        loads = [sum(costs[i] for i in p) for p in parts]
        assert max(loads) - min(loads) <= max(costs)
    with pytest.raises(ValueError):
        station_shard(costs, 2, 2)


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _stations():
    from tests.problems import media, noise_source, small_cfg, stations
    cfg = small_cfg(nx=24, nz=20, nt=30, K=8, fs=5, fw=1)
    mu, rho = media(cfg, seed=1)
    spec, sd = noise_source(cfg, seed=1)
    refs = stations(cfg, 3, seed=5)
    rec = stations(cfg, 4, seed=6)
    return cfg, mu, rho, spec, sd, refs, rec


def _solve(i):
    from oracle import pyoracle
    cfg, mu, rho, spec, sd, refs, rec = _stations()
    G, _, _ = pyoracle.forward1_green(cfg, mu, rho, refs[i:i + 1], rec, 0)
    c, _ = pyoracle.forward2_correlation(cfg, mu, rho, G, spec, sd, rec, 0)
    # a kernel-shaped FP64 array per station (nx*nz planes) for the reduction
    return c, np.real(G[:, :, :2]).copy()


def _rank(rank, world, port, out_dir):
    import torch.distributed as dist
    from fd2d_noise_gb300.replicas import gather_rows
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        n = 3
        cfg = _stations()[0]
        mine = station_shard([cfg.npts * (cfg.nt + cfg.ntc)] * n, world, rank)
        corr, ksum = {}, None
        for i in mine:
            c, k = _solve(i)
            corr[i] = c
            ksum = k if ksum is None else ksum + k
        if ksum is None:
            ksum = np.zeros((cfg.nx, cfg.nz, 2))
        total = sum_kernels(ksum)
        rows = gather_rows(corr, n)
        np.save(os.path.join(out_dir, f"k{rank}.npy"), total)
        if rank == 0:
            np.save(os.path.join(out_dir, "corr.npy"), np.stack(rows))
    finally:
        dist.destroy_process_group()


def test_two_ranks_match_one_process(tmp_path):
    import torch.multiprocessing as mp
    from oracle import pyoracle
    pyoracle.build()
    port = _free_port()
    mp.start_processes(_rank, args=(2, port, str(tmp_path)), nprocs=2, join=True, start_method="spawn")
    ref = [_solve(i) for i in range(3)]
    corr = np.load(tmp_path / "corr.npy")
    for i in range(3):
        np.testing.assert_array_equal(corr[i], ref[i][0])
    want = ref[0][1] + ref[1][1] + ref[2][1]
    for r in range(2):
        got = np.load(tmp_path / f"k{r}.npy")
        np.testing.assert_allclose(got, want, rtol=1e-14, atol=0)
