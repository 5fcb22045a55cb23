"""Continuous-batching request loop on one GPU.

Requests of three kinds arrive at any time:

  'correlation'  the Green function and correlation wavefield of each of its
                 reference stations (code/calculate_data.m:189-202) -- one
                 fd2d_correlation_batch call, stations of one grid as lanes;
  'kernel'       misfit and structure kernel summed over its stations
                 (inversion/optlib_callback_fct/eval_objective_and_gradient.m);
  'hvp'          Hessian-vector product along dmu
                 (inversion/optlib_callback_fct/eval_hessian_vector_product.m).

The server owns ``slots`` worker threads, each with its own libfd2d context
(own CUDA stream, workspace and cached graphs).  A queued request is admitted
when a slot is idle and its device-memory footprint fits in what the admitted
requests leave of the budget; it then runs on its slot's stream while the
other slots' requests keep running, so their kernels overlap on the GPU.  The
queue is served in arrival order, except that a request that fits may pass a
head request that does not, at most ``max_bypass`` times per head request (no
starvation).  A request larger than the whole budget fails at submission.
After each request the slot releases its workspace back to the device pool.

Results are the same as those of the request run alone: every request runs on
its own stream with its own buffers, and the kernels are deterministic.
"""
from __future__ import annotations

import threading
import time
from collections import deque
from concurrent.futures import Future
from dataclasses import dataclass, field
from typing import Callable, Optional

import numpy as np

from .config import Config, n_fw_corr, n_fw_green


class AdmissionError(RuntimeError):
    pass


@dataclass
class Request:
    kind: str                       # 'correlation' | 'kernel' | 'hvp'
    cfg: Config
    mu: np.ndarray
    rho: np.ndarray
    spectrum: np.ndarray
    source_dist: np.ndarray
    ref_stat: np.ndarray            # n_ref-by-2
    receivers: np.ndarray           # correlation: nr-by-2; kernel / hvp: the station array
    c_data: Optional[np.ndarray] = None
    dmu: Optional[np.ndarray] = None
    measurement: str = "log_amplitude_ratio"
    weighting: float = 1.0
    arrival: float = field(default_factory=time.perf_counter)

    def gpt(self) -> int:
        """Grid-point updates of the request (Green + correlation + adjoint runs)."""
        c = self.cfg
        n_ref = np.asarray(self.ref_stat).reshape(-1, 2).shape[0]
        runs = {"correlation": c.nt + c.ntc, "kernel": c.nt + c.ntc + c.ntc + c.nt,
                "hvp": 2 * c.nt + 2 * c.ntc + 4 * c.ntc}[self.kind]
        return c.npts * runs * n_ref


def footprint(req: Request, precision: str = "fp32") -> int:
    """Upper bound of the device bytes a request holds while it runs.  FP32
    form: per-lane fields and coefficient planes, the DFT snapshot chunk, FP64
    spectra, injection planes; plain FP64 form (one station at a time): FP64
    fields and coefficients, spectra and per-frequency distributions of every
    station of the call.  Kernel / Hessian requests add the staged snapshot
    stacks of the Green and correlation runs."""
    if precision == "fp64":
        return footprint_fp64(req)
    c = req.cfg
    P = (c.nx + 31) // 32 * 32
    plane = ((P * c.nz + 127) // 128 * 128) * 4
    np_, K = c.npts, c.n_sample
    n_ref = np.asarray(req.ref_stat).reshape(-1, 2).shape[0]
    nr = max(np.asarray(req.receivers).reshape(-1, 2).shape[0], 1)
    n_dft = min(c.nt // max(c.freq_samp, 1) + 1, 640, (2 << 30) // plane)  # the library's DFT chunk
    n_inj = min(c.ntc // max(c.freq_samp, 1), (4 << 30) // plane)
    per = (11 * plane + 3 * n_dft * plane + 16 * np_ * K + 3 * 2 * K * plane + n_inj * plane
           + 8 * nr * (c.nt + c.ntc) + 8 * np_ * (3 + np.asarray(req.source_dist).size // max(np_, 1)))
    if req.kind == "correlation":
        return int(n_ref * per + (1 << 20))
    snaps = (n_fw_green(c) + n_fw_corr(c)) * np_ * 4
    extra = 2 * snaps + 3 * 16 * np_ * K  # staged inputs and outputs of the adjoint runs
    if req.kind == "hvp":
        extra = 3 * extra
    return int(per + extra + (1 << 20))


def footprint_fp64(req: Request) -> int:
    c = req.cfg
    np_, K = c.npts, c.n_sample
    n_ref = np.asarray(req.ref_stat).reshape(-1, 2).shape[0]
    nr = max(np.asarray(req.receivers).reshape(-1, 2).shape[0], 1)
    n_dist = max(np.asarray(req.source_dist).size // max(np_, 1), 1)
    # fields, coefficients, staged model and source maps (FP64), Green spectra
    # (16 B per point and frequency) and per-frequency distribution (8 B)
    per = 8 * np_ * (12 + n_dist) + 24 * np_ * K + 8 * nr * (c.nt + c.ntc)
    if req.kind == "correlation":
        return int(n_ref * per + (1 << 20))
    snaps = (n_fw_green(c) + n_fw_corr(c)) * np_ * 4
    extra = 2 * snaps + 3 * 16 * np_ * K
    if req.kind == "hvp":
        extra = 3 * extra
    return int(per + extra + (1 << 20))


def run_request(req: Request, precision: str = "fp32", device: int = 0):
    """Runs one request on the calling thread's bound context (see
    solvers.bound_context) and returns its result dict."""
    from . import objective
    from .solvers import context
    t = (-(req.cfg.nt - 1) + np.arange(req.cfg.ntc)) * req.cfg.dt
    if req.kind == "correlation":
        return {"correlations": _correlations(req, precision, device)}
    # kernel and Hessian requests keep spectra and snapshot stacks on the device
    be = objective.device_backend(req.cfg, precision, device, ctx=context(device, precision))
    if req.kind == "kernel":
        j, g, c = objective.eval_objective_and_gradient(
            req.mu, req.rho, req.spectrum, req.source_dist, req.ref_stat, req.receivers, req.c_data, t,
            cfg=req.cfg, type="structure", measurement_source=req.measurement,
            measurement_structure=req.measurement, weighting=req.weighting, backend=be)
        return {"misfit": j, "gradient": g, "correlations": c}
    if req.kind == "hvp":
        H = objective.eval_hessian_vector_product(
            req.mu, req.rho, req.spectrum, req.source_dist, req.ref_stat, req.receivers, req.c_data, t, req.dmu,
            cfg=req.cfg, type="structure", measurement_source=req.measurement,
            measurement_structure=req.measurement, weighting=req.weighting, backend=be)
        return {"hvp": H}
    raise ValueError(f"unknown request kind {req.kind!r}")


def _correlations(req: Request, precision: str, device: int) -> np.ndarray:
    import ctypes
    from . import _lib
    from .solvers import context
    ctx = context(device, precision)
    c = req.cfg
    cc = c.to_c()
    ref = np.asarray(req.ref_stat, dtype=np.float64).reshape(-1, 2)
    rec = np.asfortranarray(np.asarray(req.receivers, dtype=np.float64).reshape(-1, 2))
    mu = np.asfortranarray(req.mu, dtype=np.float64)
    rho = np.asfortranarray(req.rho, dtype=np.float64)
    spec = np.asfortranarray(np.asarray(req.spectrum, dtype=np.float64).reshape(c.n_sample, -1))
    sd = np.asfortranarray(req.source_dist, dtype=np.float64)
    n_dist = 1 if sd.ndim == 2 else sd.shape[2]
    nr = rec.shape[0]
    out = np.zeros((ref.shape[0], nr, c.ntc))
    srcs = [np.asfortranarray(ref[i:i + 1]) for i in range(ref.shape[0])]
    outs = [np.zeros((nr, c.ntc), order="F") for _ in srcs]
    jobs = (_lib.FD2DJob * len(srcs))()
    for i, s in enumerate(srcs):
        jobs[i].cfg = ctypes.pointer(cc)
        jobs[i].mu, jobs[i].rho = mu.ctypes.data, rho.ctypes.data
        jobs[i].spectrum, jobs[i].n_noise_sources = spec.ctypes.data, spec.shape[1]
        jobs[i].source_dist, jobs[i].n_dist = sd.ctypes.data, n_dist
        jobs[i].src, jobs[i].rec, jobs[i].nr = s.ctypes.data, rec.ctypes.data, nr
        jobs[i].correlations = outs[i].ctypes.data
    _lib.check(ctx.L.fd2d_correlation_batch(ctx.h, jobs, len(srcs)), ctx.h)
    for i, o in enumerate(outs):
        out[i] = o
    return out


@dataclass
class _Entry:
    req: Request
    fut: Future
    bytes: int
    bypassed: int = 0


class Server:
    def __init__(self, budget_bytes: int, slots: int = 4, device: int = 0, precision: str = "fp32",
                 max_bypass: int = 4, runner: Optional[Callable] = None, footprint_fn: Optional[Callable] = None,
                 contexts: bool = True):
        """``runner(req)`` replaces run_request and ``contexts=False`` skips the
        per-slot libfd2d contexts (host-only tests of the admission logic);
        ``footprint_fn(req)`` defaults to the footprint of ``precision``."""
        if slots < 1 or budget_bytes <= 0:
            raise ValueError("need at least one slot and a positive budget")
        self.budget = int(budget_bytes)
        self.free = int(budget_bytes)
        self.max_bypass = max_bypass
        self.device, self.precision = device, precision
        self.runner = runner or (lambda r: run_request(r, precision, device))
        self.footprint = footprint_fn or (lambda r: footprint(r, precision))
        self.queue: deque = deque()
        self.cv = threading.Condition()
        self.stop = False
        self.running = 0
        self.peak_bytes = 0
        self.peak_running = 0
        self.log = []  # (kind, arrival, start, finish, bytes, gpt)
        self.threads = [threading.Thread(target=self._worker, args=(i, contexts), daemon=True)
                        for i in range(slots)]
        for t in self.threads:
            t.start()

    # -- client side --------------------------------------------------------------
    def submit(self, req: Request) -> Future:
        fut: Future = Future()
        b = int(self.footprint(req))
        if b > self.budget:
            fut.set_exception(AdmissionError(f"request needs {b} B of device memory; the budget is {self.budget} B"))
            return fut
        with self.cv:
            if self.stop:
                raise RuntimeError("server closed")
            self.queue.append(_Entry(req, fut, b))
            self.cv.notify_all()
        return fut

    def close(self):
        with self.cv:
            self.stop = True
            self.cv.notify_all()
        for t in self.threads:
            t.join()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # -- admission ----------------------------------------------------------------
    def _pick(self) -> Optional[_Entry]:
        """First queued entry that fits (called with the lock held)."""
        if not self.queue:
            return None
        head = self.queue[0]
        if head.bytes <= self.free:
            return self.queue.popleft()
        if head.bypassed >= self.max_bypass:
            return None  # the head waits for memory; nobody passes it any more
        for k in range(1, len(self.queue)):
            e = self.queue[k]
            if e.bytes <= self.free:
                head.bypassed += 1
                del self.queue[k]
                return e
        return None

    def _worker(self, slot: int, contexts: bool):
        ctx = None
        bind = None
        if contexts:
            from . import _lib, solvers
            from .solvers import _prec
            ctx = _lib.Context(self.device, _prec(self.precision))
            # slots share the GPU: steps without programmatic early launch and
            # tile shapes by the size rule (no timed trials on a busy queue)
            ctx.set_shared_gpu(True)
            bind = solvers.bound_context(ctx)
            bind.__enter__()
        try:
            while True:
                with self.cv:
                    e = None
                    while not self.stop:
                        e = self._pick()
                        if e is not None:
                            break
                        self.cv.wait()
                    if e is None:
                        return
                    self.free -= e.bytes
                    self.running += 1
                    self.peak_bytes = max(self.peak_bytes, self.budget - self.free)
                    self.peak_running = max(self.peak_running, self.running)
                start = time.perf_counter()
                try:
                    res = self.runner(e.req)
                    err = None
                except BaseException as x:  # reported through the future
                    res, err = None, x
                finally:
                    if ctx is not None:
                        try:
                            ctx.release()
                        except Exception:
                            pass
                finish = time.perf_counter()
                with self.cv:
                    self.free += e.bytes
                    self.running -= 1
                    self.log.append((e.req.kind, e.req.arrival, start, finish, e.bytes, e.req.gpt()))
                    self.cv.notify_all()
                if err is not None:
                    e.fut.set_exception(err)
                else:
                    e.fut.set_result(res)
        finally:
            if bind is not None:
                bind.__exit__(None, None, None)
            if ctx is not None:
                ctx.close()

    # -- statistics ---------------------------------------------------------------
    def latency_stats(self):
        lat = np.array([f - a for (_, a, _, f, _, _) in self.log])
        if lat.size == 0:
            return {}
        t0 = min(a for (_, a, _, _, _, _) in self.log)
        t1 = max(f for (_, _, _, f, _, _) in self.log)
        gpt = sum(g for (*_, g) in self.log)
        return {"requests": int(lat.size), "p50_s": float(np.percentile(lat, 50)),
                "p99_s": float(np.percentile(lat, 99)), "mean_s": float(lat.mean()),
                "throughput_req_s": lat.size / (t1 - t0), "gpt_per_s": gpt / (t1 - t0),
                "peak_concurrent": self.peak_running, "peak_bytes": self.peak_bytes}


def make_request_cfg(kind: str, nx: int, nt: int, K: int = 64) -> Config:
    """Configuration of a synthetic request on an nx-by-nx grid of 4e5 m: dt at
    Courant number 0.45 for 4000 m/s, nt stretched to cover the 100-200 s
    measurement window, 4th order, K frequencies in 0.01-0.2 Hz, snapshots
    every step (Hessian requests) or every 5 steps."""
    from .config import matlab_colon
    L = 4.0e5
    dx = L / (nx - 1)
    dt = 0.45 * dx / 4000.0
    nt = max(int(nt), int(np.ceil(130.0 / dt)) + 1)
    f = matlab_colon(0.01, (0.2 - 0.01) / (K - 1), 0.2)[:K]
    return Config(Lx=L, Lz=L, nx=nx, nz=nx, dt=dt, nt=nt, order=4, f_sample=f, freq_samp=5,
                  fw_nth=1 if kind == "hvp" else 5, absorb_width=20 * dx, source_type="gaussian")


def make_request(kind: str, nx: int, nt: int, n_ref: int = 1, K: int = 64, nr: int = 8, seed: int = 0,
                 arrival: Optional[float] = None) -> Request:
    """A seeded synthetic request on an nx-by-nx grid of 4e5 m: random medium
    (5 % std), Gaussian noise source, ``n_ref`` reference stations and ``nr``
    receivers; kernel and Hessian requests get synthetic data traces.  The
    time axis is stretched so that it covers the 100-200 s measurement window
    (tools/measurement/make_adjoint_sources.m:87-88)."""
    from .media import interior_points, random_media
    from .noise_source import make_noise_source
    cfg = make_request_cfg(kind, nx, nt, K)
    L = cfg.Lx
    mu, rho = random_media(cfg, std=0.05, corr_len=2.0e4, seed=seed)
    sd, spec = make_noise_source("gaussian", 0, cfg,
                                 spectrum_kw=dict(f_peak=[0.1], bandwidth=[0.03], strength=[1.0]),
                                 x_c=[0.3 * L], z_c=[0.6 * L], width=[0.1 * L], magnitude=[6.0])
    pts = interior_points(cfg, n_ref + nr, seed=seed + 1, margin_frac=0.2)
    ref = pts[:n_ref]
    recv = pts[n_ref:] if kind == "correlation" else pts
    c_data = dmu = None
    if kind != "correlation":
        rng = np.random.default_rng(seed + 2)
        n_rec = pts.shape[0] - 1
        tt = (-(cfg.nt - 1) + np.arange(cfg.ntc)) * cfg.dt
        c_data = np.zeros((n_ref * n_rec, cfg.ntc))
        for r in range(c_data.shape[0]):
            for sgn in (1.0, -1.0):
                t0 = sgn * rng.uniform(110.0, 190.0)
                c_data[r] += rng.uniform(0.5, 2.0) * np.exp(-((tt - t0) / 12.0) ** 2)
        if kind == "hvp":
            dmu = 0.01 * mu * rng.standard_normal(mu.shape)
    r = Request(kind, cfg, mu, rho, spec, sd, ref, recv, c_data=c_data, dmu=dmu)
    if arrival is not None:
        r.arrival = arrival
    return r


def poisson_mix(n_requests: int, rate: float, seed: int = 6, sizes=(256, 320, 384), nt_range=(800, 1600),
                mix=(0.6, 0.3, 0.1), max_ref: int = 4, max_ref_kernel: int = 1, hvp_sizes=None):
    """[(arrival offset s, kind, nx, nt, n_ref, seed)] for a seeded Poisson stream
    of correlation / kernel / Hessian requests in the proportions ``mix``.
    Correlation requests have 1..max_ref reference stations, kernel and Hessian
    requests 1..max_ref_kernel.  Hessian requests store the wavefields of every
    step (their Born runs read G_in(:,:,i) at each step,
    code/run_forward1_green.m:140-144), so their grids are drawn from
    ``hvp_sizes`` (default: the smallest size)."""
    rng = np.random.default_rng(seed)
    t = 0.0
    out = []
    kinds = ("correlation", "kernel", "hvp")
    hvp_sizes = tuple(hvp_sizes) if hvp_sizes else (min(sizes),)
    for i in range(n_requests):
        t += rng.exponential(1.0 / rate)
        kind = kinds[int(rng.choice(3, p=np.asarray(mix) / np.sum(mix)))]
        nx = int(rng.choice(sizes))
        nt = int(rng.integers(nt_range[0], nt_range[1] + 1))
        top = max_ref if kind == "correlation" else max_ref_kernel
        n_ref = int(rng.integers(1, top + 1)) if top > 1 else 1
        if kind == "hvp" and nx not in hvp_sizes:
            nx = hvp_sizes[0] if len(hvp_sizes) == 1 else int(hvp_sizes[int(rng.integers(len(hvp_sizes)))])
        out.append((t, kind, nx, nt, n_ref, seed * 1000 + i))
    return out


# Request stream of the serving measurement at the sizes of the serving
# configuration: grids 256^2-1024^2, nt 1000-5000, 1-8 reference stations per
# request; Hessian-vector requests on grids up to 512^2 (at 1024^2 and nt 5000
# their every-step wavefield stores alone would need ~380 GB).
SERVE_SIZES = (256, 384, 512, 640, 768, 896, 1024)
SERVE_NT = (1000, 5000)
SERVE_HVP_SIZES = (256, 384, 512)


def serving_mix(n_requests: int, rate: float = 50.0, seed: int = 6):
    return poisson_mix(n_requests, rate, seed=seed, sizes=SERVE_SIZES, nt_range=SERVE_NT, max_ref=8,
                       max_ref_kernel=8, hvp_sizes=SERVE_HVP_SIZES)
