"""Serving loop: admission by device-memory footprint, continuous batching, and
results identical alone and in the mix.

The host tests drive the scheduler with fake runners (no GPU); the GPU test
submits a mix of correlation, kernel and Hessian requests concurrently and
compares every result with the same request run alone."""
import threading
import time

import numpy as np
import pytest

from fd2d_noise_gb300.serving import AdmissionError, Request, Server


def _req(kind="correlation", tag=0):
    from tests.problems import small_cfg
    cfg = small_cfg(nx=24, nz=20, nt=20, K=6)
    z = np.zeros((cfg.nx, cfg.nz))
    r = Request(kind, cfg, z, z, np.ones((6, 1)), z, np.zeros((1, 2)), np.zeros((2, 2)))
    r.tag = tag
    return r


def test_oversize_request_is_refused():
    with Server(budget_bytes=10, slots=2, contexts=False, runner=lambda r: 1,
                footprint_fn=lambda r: 11) as s:
        f = s.submit(_req())
        with pytest.raises(AdmissionError):
            f.result(timeout=5)


def test_admission_respects_budget_and_slots():
    sizes = {0: 6, 1: 6, 2: 3, 3: 4, 4: 1}
    lock = threading.Lock()
    live = {"bytes": 0, "n": 0, "max_bytes": 0, "max_n": 0}

    def runner(r):
        with lock:
            live["bytes"] += sizes[r.tag]
            live["n"] += 1
            live["max_bytes"] = max(live["max_bytes"], live["bytes"])
            live["max_n"] = max(live["max_n"], live["n"])
        time.sleep(0.05)
        with lock:
            live["bytes"] -= sizes[r.tag]
            live["n"] -= 1
        return r.tag * 10

    with Server(budget_bytes=10, slots=3, contexts=False, runner=runner,
                footprint_fn=lambda r: sizes[r.tag]) as s:
        futs = [s.submit(_req(tag=k)) for k in range(5)]
        assert [f.result(timeout=10) for f in futs] == [0, 10, 20, 30, 40]
    assert live["max_bytes"] <= 10 and live["max_n"] <= 3
    assert live["max_n"] >= 2  # requests that fit ran together


def test_bypass_is_bounded():
    """A large head request waits for memory while small ones pass it, but only
    max_bypass times; then it runs."""
    order = []

    def runner(r):
        order.append(r.tag)
        time.sleep(0.02)
        return r.tag

    sizes = lambda r: 8 if r.tag == 100 else 4  # noqa: E731
    with Server(budget_bytes=10, slots=2, contexts=False, runner=runner, footprint_fn=sizes, max_bypass=2) as s:
        first = s.submit(_req(tag=1))  # occupies 4 of 10
        time.sleep(0.005)
        big = s.submit(_req(tag=100))  # needs 8: waits
        small = [s.submit(_req(tag=k)) for k in range(2, 8)]
        big.result(timeout=10)
        for f in small + [first]:
            f.result(timeout=10)
    i = order.index(100)
    assert sum(1 for t in order[:i] if t >= 2) <= 2, order


def test_runner_errors_reach_the_caller():
    def runner(r):
        raise ValueError("boom")

    with Server(budget_bytes=10, slots=1, contexts=False, runner=runner, footprint_fn=lambda r: 1) as s:
        with pytest.raises(ValueError):
            s.submit(_req()).result(timeout=5)
        assert s.free == 10


@pytest.mark.gpu
def test_results_alone_equal_results_in_the_mix(fd2d_lib):
    from fd2d_noise_gb300 import _lib, solvers
    from fd2d_noise_gb300.serving import run_request
    from tests.test_objective import cfg4, problem, oracle_backend, run

    reqs = []
    for fw, kind in ((5, "correlation"), (5, "kernel"), (1, "hvp"), (5, "correlation"), (5, "kernel")):
        cfg = cfg4(fw=fw)
        p = problem(cfg)
        _, _, c_data = run(cfg, p, p["mu_true"], np.zeros((3, cfg.ntc)), oracle_backend(cfg), only=True)
        recv = p["arr"] if kind != "correlation" else p["arr"][1:]
        reqs.append(Request(kind, cfg, p["mu0"], p["rho"], p["spec"], p["sd"], p["ref"], recv, c_data=c_data,
                            dmu=p["dmu"]))
    alone = []
    ctx = _lib.Context(0, _lib.PREC_FP32)
    with solvers.bound_context(ctx):
        for r in reqs:
            alone.append(run_request(r))
            ctx.release()
    ctx.close()
    with Server(budget_bytes=8 << 30, slots=3) as s:
        futs = [s.submit(r) for r in reqs]
        mixed = [f.result(timeout=300) for f in futs]
        stats = s.latency_stats()
    assert stats["requests"] == len(reqs) and stats["peak_concurrent"] >= 2
    for a, m in zip(alone, mixed):
        assert a.keys() == m.keys()
        for k in a:
            x, y = np.asarray(a[k], dtype=np.float64), np.asarray(m[k], dtype=np.float64)
            np.testing.assert_allclose(y, x, rtol=1e-12, atol=0)
