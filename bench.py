#!/usr/bin/env python
"""Benchmark of the fd2d_noise wave-propagation hot path on GB300.

Metric: grid-point updates per second (one (ix,iz) node advanced one time step
of one solve; a reference station costs nx*nz*(nt + 2nt-1) updates: its Green
run plus its correlation run) of the FP32 form, beside the plain FP64 GPU form
and the CPU restatement of the reference (the oracle).

One step = every reference station of the workload: run_forward1_green (mode 0)
followed by run_forward2_correlation (mode 0), i.e. code/calculate_data.m:189-202.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Under torchrun every rank runs the full workload on its own GPU (independent
replicas, weak scaling); the timed region is bracketed by a barrier and a
device synchronisation and the max over ranks is reported.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

B_STEP_V = 36   # algorithmic bytes per update, Green step: read v,sxy,szy,dt/rho,taper,dt*mu; write v,sxy,szy
B_STEP_VU = 44  # correlation step: + read/write u
METRIC = "Gpt-updates/s batched FP32 vs plain FP64 GPU at <=1e-4 rel L2; p50/p99 latency"


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d.get("hbm_gbs", 6800.0)), "measured"
    return 6800.0, "fallback"


def profiled_traffic(kernel: str, workload: str):
    """DRAM bytes per launch from the committed ncu summary, or None."""
    p = os.path.join(ROOT, "profiles", "traffic.txt")
    if not os.path.exists(p):
        return None
    with open(p) as f:
        for line in f:
            parts = line.split()
            if len(parts) >= 3 and parts[0] == kernel and parts[1] == workload:
                try:
                    return float(parts[2])
                except ValueError:
                    return None
    return None


class Clocks:
    """Samples SM clocks and throttle reasons with nvidia-smi during the timed region."""

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.path = None

    def start(self):
        fd, self.path = tempfile.mkstemp(prefix="clk", suffix=".csv")
        os.close(fd)
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={q}", "--format=csv,noheader,nounits", "-lms", "200",
                 "-i", str(self.device)], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        rows = []
        with open(self.path) as f:
            for line in f:
                c = [x.strip() for x in line.split(",")]
                if len(c) >= 9:
                    rows.append(c)
        os.unlink(self.path)
        if not rows:
            return None
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = max(float(r[2]) for r in rows if r[2].replace(".", "").isdigit())
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            for n, v in zip(names, r[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(rows)}


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def cpu_sample(w, nt_cpu: int, threads: int):
    """Times the FP64 CPU oracle on a truncated-nt sample of the same workload."""
    from oracle import pyoracle
    pyoracle.build()
    pyoracle.set_threads(threads)
    cfg = w.cfg.replace(nt=nt_cpu)
    t0 = time.perf_counter()
    G, _, _ = pyoracle.forward1_green(cfg, w.mu, w.rho, w.ref_stations[:1], w.receivers, 0)
    pyoracle.forward2_correlation(cfg, w.mu, w.rho, G, w.spectrum, w.source_dist, w.receivers, 0)
    dt = time.perf_counter() - t0
    gpt = cfg.npts * (cfg.nt + cfg.ntc)
    return gpt / dt / 1e9, dt, gpt, cfg


def one_thread_sample(w, nt_cpu: int) -> dict:
    """The CPU oracle on one thread, on an eighth of the all-core sample's
    steps (at least 4): the single-core figure beside the all-core one."""
    nt1 = max(4, nt_cpu // 8)
    v, dt, gpt, cfg = cpu_sample(w, nt1, 1)
    return {"value_1thread": v,
            "sample_1thread": f"one station, nt truncated to {cfg.nt} ({gpt:.3g} updates, {dt:.1f} s), 1 thread"}


def workload_config(w, world):
    """The ``config`` object of both arms' lines for a single-grid workload."""
    cfg = w.cfg
    np_, K = cfg.npts, cfg.n_sample
    return {"workload": w.name, "nx": cfg.nx, "nz": cfg.nz, "nt": cfg.nt, "ntc": cfg.ntc,
            "order": cfg.order, "n_sample": K, "freq_samp": cfg.freq_samp,
            "reference_stations": int(w.ref_stations.shape[0]), "receivers": int(w.receivers.shape[0]),
            "gpt_per_step": int(w.ref_stations.shape[0] * w.gpt_per_station()),
            "parallelism": f"replicas x{world}",
            "l2": "inputs > L2 per step (FP64 Green spectra %.2f GB, injection planes %.2f GB)"
                  % (2 * np_ * K * 8 / 1e9, (cfg.ntc // cfg.freq_samp) * np_ * 4 / 1e9)}


def run_reference(args, w, world, rank):
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    vals = []
    dts = []
    for _ in range(args.warmup):
        cpu_sample(w, args.cpu_nt, threads)
    for _ in range(args.steps):
        v, dt, gpt, cfg = cpu_sample(w, args.cpu_nt, threads)
        vals.append(v)
        dts.append(dt)
    value = statistics.median(vals)
    sample = (f"one reference station of {w.name} with nt truncated to {args.cpu_nt}: "
              f"Green {cfg.nt} + correlation {cfg.ntc} steps on {cfg.nx}x{cfg.nz}, K={cfg.n_sample}")
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "Gpt-updates/s",
        "n_gpus": world, "gpus_used": 0, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * statistics.median(dts), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        # the workload is the GPU arm's; each step times a bounded sample of it
        # (cpu_baseline.sample) and reports the same per-update rate
        "config": workload_config(w, world),
        "cpu_baseline": {"value": value, "unit": "Gpt-updates/s", "cores": threads, "kind": "port",
                         "sample": sample, **one_thread_sample(w, args.cpu_nt)},
        "e2e": {"value": value, "unit": "Gpt-updates/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": "CPU restatement of the reference's MATLAB solvers (MATLAB unavailable), OpenMP over grid points",
    }
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="single_600_o8")
    ap.add_argument("--cpu-nt", type=int, default=400,
                    help="nt of the CPU oracle sample (one station; about 10 s on 16 cores)")
    ap.add_argument("--nt", type=int, default=0, help="override the workload's nt (profiling runs)")
    ap.add_argument("--stations", type=int, default=0, help="override the number of reference stations")
    ap.add_argument("--grid", type=int, default=0, help="square grid size of single_600_o8 (profiling runs)")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-fp64", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--serve-requests", type=int, default=24,
                    help="requests of the serving measurement (0: skip it)")
    ap.add_argument("--serve-fp64-s", type=float, default=90.0,
                    help="the plain FP64 form serves the leading requests of the same stream whose "
                         "estimated FP64 time (at 1.1 Gpt/s) adds up to this (at least one; 0: skip it)")
    ap.add_argument("--no-configs", action="store_true",
                    help="skip the configuration-1, -3 and -4 measurements")
    ap.add_argument("--serve-rate", type=float, default=50.0, help="mean Poisson arrival rate [1/s]")
    ap.add_argument("--serve-slots", type=int, default=8, help="concurrent solves of the serving loop")
    ap.add_argument("--no-hbm-probe", action="store_true",
                    help="skip the stencil roofline on a grid whose fields exceed L2")
    ap.add_argument("--probe-nt", type=int, default=200, help="nt of the large-grid stencil probe")
    ap.add_argument("--no-timing", action="store_true",
                    help="do not bracket kernels with CUDA events (no roofline)")
    args = ap.parse_args()
    world, rank, local = dist_setup()

    from fd2d_noise_gb300.workloads import WORKLOADS
    if args.workload == "batch_uneven":
        # a smaller batch of the same kind for profiling: --stations stations,
        # nt in [--nt, 1.5 --nt]
        kw = {"n_stations": args.stations} if args.stations else {}
        if args.nt:
            kw["nt_range"] = (args.nt, args.nt + args.nt // 2)
    else:
        kw = {"nt": args.nt} if args.nt else {}
        if args.stations:
            kw["n_ref"] = args.stations
        if args.grid:
            kw["nx"] = args.grid
    w = WORKLOADS[args.workload](**kw)
    if args.impl == "reference":
        run_reference(args, w, world, rank)
        return

    import numpy as np
    import torch
    from fd2d_noise_gb300 import _lib
    from fd2d_noise_gb300.build import build
    from fd2d_noise_gb300.device import DeviceSession, to_device

    build()
    torch.cuda.set_device(local)
    if hasattr(w, "stations"):
        run_batch_workload(args, w, local, world, rank)
        return
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    dev = local
    cfg = w.cfg
    np_, K, nr = cfg.npts, cfg.n_sample, w.receivers.shape[0]
    n_ref = w.ref_stations.shape[0]

    sess = DeviceSession(cfg, dev, "fp32")
    mu = to_device(w.mu, np.float64, dev)
    rho = to_device(w.rho, np.float64, dev)
    spec = to_device(w.spectrum, np.float64, dev)
    sd = to_device(w.source_dist, np.float64, dev)
    rec = to_device(w.receivers, np.float64, dev)
    refs = [to_device(w.ref_stations[i:i + 1], np.float64, dev) for i in range(n_ref)]
    G_re, G_im, _, seis_g = sess.green_outputs(nr)
    seis_c = [sess.zeros(nr * cfg.ntc, torch.float64) for _ in range(n_ref)]
    batch = [dict(cfg=cfg, mu=mu, rho=rho, spectrum=spec, source_dist=sd, src=refs[i], rec=rec, nr=nr,
                  out=seis_c[i]) for i in range(n_ref)]

    def step(s: DeviceSession, outs):
        # one call = the station loop of code/calculate_data.m:189-202
        s.correlation_batch(batch)

    gpt_step = n_ref * w.gpt_per_station()
    torch.cuda.synchronize()
    stream = sess.stream
    for _ in range(max(args.warmup, 0)):
        step(sess, seis_c)
    torch.cuda.synchronize()

    def barrier():
        if world > 1:
            import torch.distributed as dist
            dist.barrier()

    clocks = Clocks(dev)
    launches0 = sess.ctx.kernel_launches
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    barrier()
    torch.cuda.synchronize()
    clocks.start()
    ev0.record(stream)
    for _ in range(args.steps):
        step(sess, seis_c)
    ev1.record(stream)
    torch.cuda.synchronize()
    barrier()
    clk = clocks.stop()
    launches = sess.ctx.kernel_launches - launches0
    ms = ev0.elapsed_time(ev1)
    # one more step, instrumented: CUDA events around every time loop and every
    # contraction on the library's stream (the instrumentation waits for the
    # stream after each graph, so it is kept out of the timed steps above)
    tim = [(0.0, 0, 0)] * 3
    if not args.no_timing:
        sess.ctx.timing()  # reset
        sess.ctx.set_timing(True)
        step(sess, seis_c)
        sess.ctx.set_timing(False)
        tim = sess.ctx.timing()
    if world > 1:
        import torch.distributed as dist
        t = torch.tensor([ms], device=f"cuda:{dev}")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    value = world * gpt_step * args.steps / (ms / 1e3) / 1e9

    # roofline of the dominant kernel (the fused stencil step), live CUDA-event durations
    # The library brackets each time loop (its step launches) with one event
    # pair and each contraction inside it with another: stencil time is the
    # loop time minus the contractions it contains.
    (msV, nV, uV), (msVU, nVU, uVU), (msC, nC, uC) = tim
    peak, peak_kind = measured_peaks()
    st_ms = msV + msVU - msC
    achieved = (B_STEP_V * uV + B_STEP_VU * uVU) / (st_ms / 1e3) / 1e9 if st_ms > 0 else None
    traffic = profiled_traffic("k32_step", w.name)
    roof = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
            "frac": (achieved / peak) if achieved else None, "traffic": traffic,
            "kernel": "k32_step<R> (fused velocity/stress stencil)",
            "peak_source": f"{peak_kind} hbm_gbs (burst)",
            "stencil_ms_per_launch": st_ms / max(nV + nVU, 1),
            "stencil_share_of_step": st_ms / (ms / args.steps) if ms else None,
            "contract_ms": msC, "contract_tflops": (2 * uC / (msC / 1e3) / 1e12) if msC else None}

    result = {
        "metric": METRIC, "value": value, "unit": "Gpt-updates/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic",
        "config": workload_config(w, world),
        "roofline": roof, "gpu_launches": launches, "clocks": clk,
    }
    result["config"]["launch_groups"] = sess.ctx.last_batch()  # lanes per launch group

    if rank == 0 and not args.no_fp64:
        # plain FP64 GPU form, one station, and the FP32 error against it
        s64 = DeviceSession(cfg, dev, "fp64")
        out64 = [sess.zeros(nr * cfg.ntc, torch.float64)]
        s64.forward1_green(mu, rho, refs[0], 1, rec, nr, G_re, G_im, seis_g)
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(s64.stream)
        s64.forward1_green(mu, rho, refs[0], 1, rec, nr, G_re, G_im, seis_g)
        s64.forward2_correlation(mu, rho, G_re, G_im, spec, 1, sd, 1, rec, nr, out64[0])
        e1.record(s64.stream)
        torch.cuda.synchronize()
        ms64 = e0.elapsed_time(e1)
        v64 = w.gpt_per_station() / (ms64 / 1e3) / 1e9
        c32 = seis_c[0].double()
        c64 = out64[0]
        rel = float(torch.linalg.norm(c32 - c64) / torch.linalg.norm(c64))
        result["fp64_plain"] = {"value": v64, "unit": "Gpt-updates/s", "ms_per_station": ms64,
                                "speedup_fp32_over_fp64": value / world / v64,
                                "rel_l2_correlations_fp32_vs_fp64": rel,
                                "roofline": fp64_roofline(cfg, ms64, w.spectrum.shape[1])}
        s64.ctx.close()

    if rank == 0 and not args.no_e2e:
        result["e2e"] = e2e(args, w, dev)

    if rank == 0 and args.serve_requests > 0:
        result["serving"] = serving_run(args, dev, "fp32", args.serve_requests)
        if args.serve_fp64_s > 0:
            result["serving_fp64"] = serving_run(args, dev, "fp64", fp64_prefix(args))
            result["serving_fp64"]["fp32_gpt_per_s_over_fp64"] = (
                result["serving"]["gpt_per_s"] / result["serving_fp64"]["gpt_per_s"])

    if rank == 0 and not args.no_configs:
        result["plain_cpu_300"] = config1_run(dev)
        result["batch_uneven"] = batch_run(dev)
        result["structure_512"] = structure_run(dev)

    if rank == 0 and not args.no_hbm_probe:
        result["roofline_large_grid"] = hbm_probe(args, dev)

    if rank == 0 and not args.no_cpu:
        threads = os.cpu_count() or 1
        v, dt, gpt, ccfg = cpu_sample(w, args.cpu_nt, threads)
        result["cpu_baseline"] = {
            "value": v, "unit": "Gpt-updates/s", "cores": threads, "kind": "port",
            "sample": f"one station, nt truncated to {ccfg.nt} ({gpt:.3g} updates, {dt:.1f} s): "
                      "FP64 C++ restatement of the reference solvers, MATLAB unavailable",
            **one_thread_sample(w, args.cpu_nt)}
    if rank == 0:
        print(json.dumps(result), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


def hbm_probe(args, dev):
    """Stencil roofline where HBM is the bound: large_2048_o8 (4 stations as
    lanes of 2048x2048, fields 4 x 11 x 16.8 MB > L2), one instrumented batch
    call after one warm-up call; the library's CUDA events bracket each time
    loop and each contraction, so stencil time = loop time - contractions."""
    import numpy as np
    import torch
    from fd2d_noise_gb300.device import DeviceSession, to_device
    from fd2d_noise_gb300.workloads import large_2048_o8

    w = large_2048_o8(nt=args.probe_nt)
    cfg = w.cfg
    nr = w.receivers.shape[0]
    sess = DeviceSession(cfg, dev, "fp32")
    mu, rho = to_device(w.mu, np.float64, dev), to_device(w.rho, np.float64, dev)
    spec, sd = to_device(w.spectrum, np.float64, dev), to_device(w.source_dist, np.float64, dev)
    rec = to_device(w.receivers, np.float64, dev)
    n_ref = w.ref_stations.shape[0]
    batch = [dict(cfg=cfg, mu=mu, rho=rho, spectrum=spec, source_dist=sd,
                  src=to_device(w.ref_stations[i:i + 1], np.float64, dev), rec=rec, nr=nr,
                  out=sess.zeros(nr * cfg.ntc, torch.float64)) for i in range(n_ref)]
    sess.correlation_batch(batch)
    torch.cuda.synchronize()
    sess.ctx.timing()
    sess.ctx.set_timing(True)
    sess.correlation_batch(batch)
    sess.ctx.set_timing(False)
    (msV, nV, uV), (msVU, nVU, uVU), (msC, nC, uC) = sess.ctx.timing()
    lanes = sess.ctx.last_batch()
    sess.ctx.close()
    del batch, mu, rho, spec, sd, rec
    torch.cuda.empty_cache()
    st_ms = msV + msVU - msC
    peak, peak_kind = measured_peaks()
    achieved = (B_STEP_V * uV + B_STEP_VU * uVU) / (st_ms / 1e3) / 1e9 if st_ms > 0 else None
    return {"workload": w.name, "nx": cfg.nx, "nz": cfg.nz, "nt": cfg.nt, "ntc": cfg.ntc, "order": cfg.order,
            "lanes": lanes, "bound": "hbm", "unit": "GB/s", "achieved": achieved, "peak": peak,
            "frac": (achieved / peak) if achieved else None, "peak_source": f"{peak_kind} hbm_gbs (burst)",
            "stencil_us_per_launch": 1e3 * st_ms / max(nV + nVU, 1), "launches": nV + nVU,
            "gpt_per_s": (uV + uVU) / (st_ms / 1e3) / 1e9 if st_ms > 0 else None,
            "traffic": profiled_traffic("k32_step", w.name),
            "bytes_per_update": "36 (Green step) / 44 (correlation step), algorithmic"}


def run_batch_workload(args, w, dev, world, rank):
    """Reference stations on uneven grids in one fd2d_correlation_batch call per
    step (device buffers): every station advances in one multi-geometry launch
    per time step."""
    import torch
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
        dist.barrier()
    clocks = Clocks(dev)
    clocks.start()
    ms, launches, groups, sess, _, roof = batch_measure(w, dev, args.steps, args.warmup)
    clk = clocks.stop()
    sess.ctx.close()
    if world > 1:
        t = torch.tensor([ms], device=f"cuda:{dev}")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    gpt = w.gpt_per_step()
    value = world * gpt / (ms / 1e3) / 1e9
    sizes = {}
    for s in w.stations:
        sizes[s.cfg.nx] = sizes.get(s.cfg.nx, 0) + 1
    line = {"metric": METRIC, "value": value, "unit": "Gpt-updates/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": w.name, "stations": len(w.stations), "grids": sizes,
                       "gpt_per_step": gpt, "launch_groups": groups,
                       "l2": "inputs > L2 per step (FP64 Green spectra of every station)"},
            "gpu_launches": int(launches * args.steps), "clocks": clk, "roofline": roof}
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()


def fp64_prefix(args) -> int:
    """Leading requests of the serving stream whose FP64 time, estimated at
    1.1 Gpt/s, adds up to --serve-fp64-s (at least one)."""
    from fd2d_noise_gb300.serving import make_request_cfg, serving_mix
    n, acc = 0, 0.0
    for (_, kind, nx, nt, n_ref, _sd) in serving_mix(args.serve_requests, args.serve_rate):
        acc += gpt_of_request(kind, make_request_cfg(kind, nx, nt), n_ref) / 1.1e9
        if n and acc > args.serve_fp64_s:
            break
        n += 1
    return n


def gpt_of_request(kind, cfg, n_ref) -> int:
    runs = {"correlation": cfg.nt + cfg.ntc, "kernel": cfg.nt + cfg.ntc + cfg.ntc + cfg.nt,
            "hvp": 2 * cfg.nt + 2 * cfg.ntc + 4 * cfg.ntc}[kind]
    return cfg.npts * runs * n_ref


def serving_run(args, dev, precision, n_requests):
    """Continuous-batching serving loop at the serving configuration's sizes: a
    seeded Poisson stream (mean --serve-rate req/s) of correlation (60 %),
    kernel (30 %) and Hessian-vector (10 %) requests on grids 256^2-1024^2
    (Hessian requests up to 512^2), nt 1000-5000, 1-8 reference stations each,
    served by ``slots`` concurrent solves with admission by device-memory
    footprint; p50/p99 of arrival-to-result latency, requests/s and grid-point
    updates/s.  ``capacity_req_s`` is what the GPU can serve of this mix: the
    requests over the sum of their run times alone (the first run of each kind,
    untimed, warms the tables and graphs)."""
    import torch
    from fd2d_noise_gb300.serving import Server, make_request, serving_mix
    mix = serving_mix(n_requests, args.serve_rate)
    reqs = [make_request(kind, nx, nt, n_ref=n_ref, seed=sd) for (_, kind, nx, nt, n_ref, sd) in mix]
    from fd2d_noise_gb300 import _lib
    torch.cuda.empty_cache()
    # free device memory, counting released workspace still held by the pool
    budget = int(_lib.device_free_bytes(dev) * 0.6)
    with Server(budget_bytes=budget, slots=args.serve_slots, device=dev, precision=precision) as srv:
        if precision == "fp32":
            # warm-up: one request of each kind alone (graph capture, tables)
            seen = set()
            for r in reqs:
                if r.kind not in seen:
                    seen.add(r.kind)
                    srv.submit(r).result()
        srv.log.clear()
        srv.peak_running = srv.peak_bytes = 0
        t0 = time.perf_counter()
        futs = []
        for (off, *_), r in zip(mix, reqs):
            now = time.perf_counter() - t0
            if off > now:
                time.sleep(off - now)
            r.arrival = time.perf_counter()
            futs.append(srv.submit(r))
        for f in futs:
            f.result()
        st = srv.latency_stats()
    kinds = {}
    for (kind, *_rest) in srv.log:
        kinds[kind] = kinds.get(kind, 0) + 1
    grids = sorted({r.cfg.nx for r in reqs})
    st.update({"precision": precision, "offered_rate_req_s": args.serve_rate, "slots": args.serve_slots,
               "budget_bytes": budget, "mix": kinds,
               "workload": (f"synthetic Poisson stream: {len(reqs)} requests, grids {grids[0]}-{grids[-1]} "
                            f"square, nt {min(r.cfg.nt for r in reqs)}-{max(r.cfg.nt for r in reqs)}, "
                            f"{min(len(r.ref_stat) for r in reqs)}-{max(len(r.ref_stat) for r in reqs)} "
                            f"reference stations, {precision} form")})
    return st


def fp64_roofline(cfg, ms, n_src=1):
    """HBM roofline of the plain FP64 form for one station (Green run and
    correlation run): per update 72 B (Green step) / 88 B (correlation step)
    of fields and coefficients, plus the reference's per-step K-term sums --
    a read-modify-write of the FP64 complex spectra (32 B per point and
    frequency) at every DFT step, and reads of distribution, Re G and Im G
    (24 B per point, frequency and noise source) at every injection step."""
    peak, kind = measured_peaks()
    np_, K, fs = cfg.npts, cfg.n_sample, cfg.freq_samp
    n_dft = sum(1 for n in range(1, cfg.nt + 1) if (n + cfg.nt - 1) % fs == 0)
    n_inj = cfg.ntc // fs
    b = (72 * np_ * cfg.nt + 88 * np_ * cfg.ntc + 32 * np_ * K * n_dft + 24 * np_ * K * n_src * n_inj)
    achieved = b / (ms / 1e3) / 1e9
    return {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
            "bytes_per_station": b, "peak_source": f"{kind} hbm_gbs (burst)"}


def _time_gpu(fn, stream):
    """CUDA-event milliseconds of fn() on ``stream`` (after a synchronisation)."""
    import torch
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    fn()
    e1.record(stream)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1)


def config1_run(dev):
    """Configuration 1 at its full size (300x300, nt 1200, order 4, K 200, one
    station, 10 receivers): the Green run and the correlation run in the plain
    FP64 form and the FP32 form on the GPU, the CPU oracle on all host cores,
    and each GPU form's error against the oracle."""
    import numpy as np
    import torch
    from oracle import pyoracle
    from fd2d_noise_gb300.device import DeviceSession, to_device
    from fd2d_noise_gb300.workloads import plain_cpu_300
    w = plain_cpu_300()
    cfg, nr = w.cfg, w.receivers.shape[0]
    gpt = w.gpt_per_station()
    out = {"workload": w.name, "nx": cfg.nx, "nz": cfg.nz, "nt": cfg.nt, "order": cfg.order,
           "n_sample": cfg.n_sample, "receivers": nr, "gpt": gpt}
    pyoracle.build()
    threads = os.cpu_count() or 1
    pyoracle.set_threads(threads)
    t0 = time.perf_counter()
    Go, _, _ = pyoracle.forward1_green(cfg, w.mu, w.rho, w.ref_stations, w.receivers, 0)
    co, _ = pyoracle.forward2_correlation(cfg, w.mu, w.rho, Go, w.spectrum, w.source_dist, w.receivers, 0)
    dt = time.perf_counter() - t0
    del Go
    out["cpu_oracle"] = {"value": gpt / dt / 1e9, "unit": "Gpt-updates/s", "seconds": dt, "cores": threads,
                         "kind": "port"}
    d = {k: to_device(getattr(w, k), np.float64, dev) for k in ("mu", "rho", "spectrum", "source_dist", "receivers")}
    src = to_device(w.ref_stations, np.float64, dev)
    for prec in ("fp64", "fp32"):
        sess = DeviceSession(cfg, dev, prec)
        G_re, G_im, _, seis = sess.green_outputs(nr)
        corr = sess.zeros(nr * cfg.ntc, torch.float64)

        def run():
            sess.forward1_green(d["mu"], d["rho"], src, 1, d["receivers"], nr, G_re, G_im, seis)
            sess.forward2_correlation(d["mu"], d["rho"], G_re, G_im, d["spectrum"], 1, d["source_dist"], 1,
                                      d["receivers"], nr, corr)
        run()  # warm-up: tables, tile shape, time depth (eager run)
        run()  # the second run of a time loop captures its CUDA graph
        ms = float(np.median([_time_gpu(run, sess.stream) for _ in range(3)]))  # replays
        c = corr.cpu().numpy().reshape(nr, cfg.ntc, order="F")
        out[prec] = {"value": gpt / (ms / 1e3) / 1e9, "unit": "Gpt-updates/s", "ms": ms,
                     "rel_l2_correlations_vs_oracle": float(np.linalg.norm(c - co) / np.linalg.norm(co))}
        if prec == "fp32":
            out[prec]["steps_per_launch"] = sess.ctx.last_time_depth()
            out[prec]["tile_rows"] = sess.ctx.last_tile_rows()
        if prec == "fp64":
            out[prec]["roofline"] = fp64_roofline(cfg, ms, w.spectrum.shape[1])
        sess.ctx.close()
        del G_re, G_im, seis, corr
    out["speedup_fp32_over_fp64"] = out["fp32"]["value"] / out["fp64"]["value"]
    out["speedup_fp32_over_cpu"] = out["fp32"]["value"] / out["cpu_oracle"]["value"]
    torch.cuda.empty_cache()
    return out


def batch_measure(w, dev, steps, warmup):
    """fd2d_correlation_batch over every station of a BatchWorkload (device
    buffers, one call per step); returns (ms per step, launches per step,
    launch groups, the session, the jobs)."""
    import numpy as np
    import torch
    from fd2d_noise_gb300.device import DeviceSession, to_device
    sess = DeviceSession(w.stations[0].cfg, dev, "fp32")
    cache, batch = {}, []
    for s in w.stations:
        key = id(s.mu)
        if key not in cache:
            cache[key] = dict(mu=to_device(s.mu, np.float64, dev), rho=to_device(s.rho, np.float64, dev),
                              spectrum=to_device(s.spectrum, np.float64, dev),
                              source_dist=to_device(s.source_dist, np.float64, dev),
                              rec=to_device(s.receivers, np.float64, dev))
        c = cache[key]
        n_dist = s.source_dist.shape[2] if s.source_dist.ndim == 3 else 1
        batch.append(dict(cfg=s.cfg, mu=c["mu"], rho=c["rho"], spectrum=c["spectrum"], source_dist=c["source_dist"],
                          n_dist=n_dist, src=to_device(s.ref_stations, np.float64, dev), rec=c["rec"],
                          nr=s.receivers.shape[0],
                          out=sess.zeros(s.receivers.shape[0] * s.cfg.ntc, torch.float64)))
    for _ in range(max(warmup, 0)):
        sess.correlation_batch(batch)
    torch.cuda.synchronize()
    l0 = sess.ctx.kernel_launches

    def run():
        for _ in range(steps):
            sess.correlation_batch(batch)
    ms = _time_gpu(run, sess.stream) / max(steps, 1)
    launches = (sess.ctx.kernel_launches - l0) / max(steps, 1)
    # one more call, instrumented: stencil time = time loops minus the
    # contractions (and their operand images) inside them
    sess.ctx.timing()
    sess.ctx.set_timing(True)
    sess.correlation_batch(batch)
    sess.ctx.set_timing(False)
    (msV, nV, uV), (msVU, nVU, uVU), (msC, nC, uC) = sess.ctx.timing()
    st_ms = msV + msVU - msC
    peak, kind = measured_peaks()
    ach = (B_STEP_V * uV + B_STEP_VU * uVU) / (st_ms / 1e3) / 1e9 if st_ms > 0 else None
    roof = {"bound": "hbm", "achieved": ach, "peak": peak, "unit": "GB/s", "frac": ach / peak if ach else None,
            "peak_source": f"{kind} hbm_gbs (burst)", "kernel": "k32_step_multi (all solves, one launch per step)",
            "stencil_ms_per_step": st_ms, "stencil_launches": nV + nVU, "contract_ms_per_step": msC,
            "bytes_per_update": "36 (Green step) / 44 (correlation step), algorithmic"}
    return ms, launches, sess.ctx.last_batch(), sess, batch, roof


def batch_run(dev, steps=2, warmup=2):
    """Configuration 3: 32 reference stations on grids of 256-800 points
    square, nt 1500-4000, order 4, four frequency bands, in one
    fd2d_correlation_batch call per step; the FP32 correlations of the
    smallest- and the largest-grid station against the plain FP64 form."""
    import numpy as np
    import torch
    from fd2d_noise_gb300.device import DeviceSession
    from fd2d_noise_gb300.workloads import batch_uneven
    w = batch_uneven()
    ms, launches, groups, sess, batch, roof = batch_measure(w, dev, steps, warmup)
    gpt = w.gpt_per_step()
    sizes = {}
    for s in w.stations:
        sizes[s.cfg.nx] = sizes.get(s.cfg.nx, 0) + 1
    errs = {}
    picks = [min(range(len(w.stations)), key=lambda i: w.stations[i].cfg.npts),
             max(range(len(w.stations)), key=lambda i: w.stations[i].cfg.npts)]
    for i in picks:
        s, j = w.stations[i], batch[i]
        cfg, nr = s.cfg, s.receivers.shape[0]
        s64 = DeviceSession(cfg, dev, "fp64")
        G_re, G_im, _, seis = s64.green_outputs(nr)
        out = s64.zeros(nr * cfg.ntc, torch.float64)
        s64.forward1_green(j["mu"], j["rho"], j["src"], 1, j["rec"], nr, G_re, G_im, seis)
        s64.forward2_correlation(j["mu"], j["rho"], G_re, G_im, j["spectrum"], 1, j["source_dist"], j["n_dist"],
                                 j["rec"], nr, out)
        torch.cuda.synchronize()
        c64, c32 = out.cpu().numpy(), j["out"].cpu().numpy()
        errs[f"station{i}_{cfg.nx}"] = float(np.linalg.norm(c32 - c64) / np.linalg.norm(c64))
        s64.ctx.close()
        del G_re, G_im, seis, out
    sess.ctx.close()
    del batch
    torch.cuda.empty_cache()
    return {"workload": w.name, "value": gpt / (ms / 1e3) / 1e9, "unit": "Gpt-updates/s", "ms_per_step": ms,
            "steps": steps, "warmup": warmup, "stations": len(w.stations), "grids": sizes, "gpt_per_step": gpt,
            "launch_groups": groups, "gpu_launches_per_step": launches, "roofline": roof,
            "rel_l2_correlations_fp32_vs_fp64": errs}


def structure_run(dev):
    """Configuration 4: the structure-kernel path on 512x512, nt 2500 --
    Green (mode 1) + correlation (mode 1), log-amplitude-ratio adjoint
    sources of 20 receivers around one reference station, adjoint mode 1 and
    adjoint mode 0 (eval_objective_and_gradient, inversion type 'structure',
    spectra and snapshot stacks kept on the device) in the FP32 form and the
    plain FP64 form: seconds, updates/s, and the FP32 misfit and mu kernel
    against FP64."""
    import numpy as np
    import torch
    from fd2d_noise_gb300.objective import device_backend, eval_objective_and_gradient
    from fd2d_noise_gb300.workloads import structure_512
    w = structure_512()
    cfg = w.cfg
    arr = np.concatenate([w.ref_stations, w.receivers])
    t = (-(cfg.nt - 1) + np.arange(cfg.ntc)) * cfg.dt
    # Green (nt) + correlation (ntc) + adjoint mode 1 (ntc) + adjoint mode 0 (nt: 3-D source)
    gpt = cfg.npts * (cfg.nt + cfg.ntc + cfg.ntc + cfg.nt)

    def run(mu, c_data, be, only=False):
        return eval_objective_and_gradient(mu, w.rho, w.spectrum, w.source_dist, w.ref_stations, arr, c_data, t,
                                           cfg=cfg, type="structure", weighting=1.0, only_objective=only,
                                           backend=be)
    be32 = device_backend(cfg, "fp32", dev)
    _, _, c_data = run(w.mu_true, np.zeros((w.receivers.shape[0], cfg.ntc)), be32, only=True)
    out = {"workload": w.name, "nx": cfg.nx, "nt": cfg.nt, "fw_nth": cfg.fw_nth, "n_sample": cfg.n_sample,
           "receivers": int(w.receivers.shape[0]), "gpt": gpt,
           "runs": "Green mode 1 + correlation mode 1 + adjoint mode 1 + adjoint mode 0"}
    res = {}
    for prec, be in (("fp32", be32), ("fp64", device_backend(cfg, "fp64", dev))):
        if prec == "fp32":
            run(w.mu, c_data, be)  # warm-up
        secs = []
        for _ in range(3 if prec == "fp32" else 1):  # FP32: median of three runs (~0.1 s each)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            res[prec] = run(w.mu, c_data, be)
            torch.cuda.synchronize()
            secs.append(time.perf_counter() - t0)
        sec = float(np.median(secs))
        out[prec] = {"seconds": sec, "value": gpt / sec / 1e9, "unit": "Gpt-updates/s", "misfit": res[prec][0]}
        if be.session is not None:
            be.session.ctx.close()
    (j32, g32, _), (j64, g64, _) = res["fp32"], res["fp64"]
    out["rel_misfit_fp32_vs_fp64"] = abs(j32 - j64) / abs(j64)
    out["rel_l2_mu_kernel_fp32_vs_fp64"] = float(np.linalg.norm(g32[:, :, -1] - g64[:, :, -1]) /
                                                np.linalg.norm(g64[:, :, -1]))
    out["speedup_fp32_over_fp64"] = out["fp64"]["seconds"] / out["fp32"]["seconds"]
    torch.cuda.empty_cache()
    return out


def e2e(args, w, dev):
    """Same metric through the C ABI with host buffers (pinned), copies inside the timed region."""
    import ctypes
    import numpy as np
    import torch
    from fd2d_noise_gb300 import _lib

    cfg = w.cfg
    np_, K, nr = cfg.npts, cfg.n_sample, w.receivers.shape[0]
    n_ref = w.ref_stations.shape[0]

    def pinned(a, dtype):
        a = np.asarray(a, dtype=dtype).ravel(order="F")
        t = torch.empty(a.size, dtype=torch.from_numpy(a[:1].copy()).dtype, pin_memory=True)
        t.numpy()[:] = a
        return t

    def p(t):
        return ctypes.c_void_p(t.data_ptr())

    ctx = _lib.Context(dev, _lib.PREC_FP32)
    mu, rho = pinned(w.mu, np.float64), pinned(w.rho, np.float64)
    spec, sd = pinned(w.spectrum, np.float64), pinned(w.source_dist, np.float64)
    rec = pinned(w.receivers, np.float64)
    refs = [pinned(w.ref_stations[i:i + 1], np.float64) for i in range(n_ref)]
    c = cfg.to_c()
    L = ctx.L
    outs = [torch.empty(nr * cfg.ntc, dtype=torch.float64, pin_memory=True) for _ in range(n_ref)]
    jobs = (_lib.FD2DJob * n_ref)()
    for i in range(n_ref):
        jobs[i].cfg = ctypes.pointer(c)
        jobs[i].mu, jobs[i].rho = mu.data_ptr(), rho.data_ptr()
        jobs[i].spectrum, jobs[i].n_noise_sources = spec.data_ptr(), 1
        jobs[i].source_dist, jobs[i].n_dist = sd.data_ptr(), 1
        jobs[i].src, jobs[i].rec, jobs[i].nr = refs[i].data_ptr(), rec.data_ptr(), nr
        jobs[i].correlations = outs[i].data_ptr()

    def step():
        # host buffers in, correlations back to the host: code/calculate_data.m:189-202
        _lib.check(L.fd2d_correlation_batch(ctx.h, jobs, n_ref), ctx.h)

    for _ in range(max(1, min(args.warmup, 2))):
        step()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        step()
    dt = time.perf_counter() - t0
    gpt = n_ref * w.gpt_per_station() * args.steps
    # per station: mu, rho, spectrum, source distribution and positions in; correlations out
    h2d = n_ref * (2 * np_ * 8 + K * 8 + np_ * 8 + 16 + nr * 16)
    d2h = n_ref * (nr * cfg.ntc * 8)
    ctx.close()
    return {"value": gpt / dt / 1e9, "unit": "Gpt-updates/s", "h2d_bytes_per_step": h2d,
            "d2h_bytes_per_step": d2h, "ms_per_step": 1e3 * dt / args.steps,
            "path": "fd2d_correlation_batch (Green + correlation per station), host (pinned) buffers"}


if __name__ == "__main__":
    main()
