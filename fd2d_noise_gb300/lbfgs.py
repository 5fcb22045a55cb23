"""L-BFGS with the Powell-Wolfe step-size rule, FP64 vectors on the device.

    optlib_lbfgs   inversion/optlib/optlib_lbfgs.m:1-210
    optlib_wolfe   inversion/optlib/optlib_wolfe.m:1-159
    defaults       inversion/optlib/optlib_init_default_parameters_lbfgs.m

Vectors are torch FP64 tensors on the device of ``m0`` (CUDA or CPU); the
callbacks receive and return tensors of that device: ``fun(m) -> (j, g)``
(eval_objective_and_gradient), ``fun_j(m) -> j`` (eval_objective) and
``fun_g(m) -> g`` (eval_grad_objective).  The iteration log, the stopping rules
(relative gradient norm, iteration cap, stagnation over
``successive_iterations``) and the curvature / descent-angle safeguards are
the reference's; file output and the restore of earlier iterations are not.
"""
from __future__ import annotations

from dataclasses import dataclass, field
from typing import Callable, Optional

import numpy as np


def _div(a, b) -> float:
    """IEEE division as in MATLAB (x/0 = +-Inf, 0/0 = NaN), no exception."""
    with np.errstate(divide="ignore", invalid="ignore"):
        return float(np.float64(a) / np.float64(b))


@dataclass
class Options:
    init_step_length: float = 1.0
    wolfe_delta: float = 0.001
    wolfe_theta: float = 0.6
    wolfe_try_to_increase_step_length: bool = True
    sufficient_decrease_angle: float = 0.1
    max_memory: int = 5
    max_iterations: int = 100
    tolerance: float = 1e-3
    successive_change: float = 1e0
    successive_iterations: int = 5
    bisection_max: int = 5


@dataclass
class Result:
    flag: int                 # 0 gradient tolerance, 1 iteration cap, 2 stagnation
    m: object
    objective: float
    gradient: object
    history: list = field(default_factory=list)  # (it, objective, ||g||, sigma, step)


def wolfe(xj, s, stg, f, delta, theta, sig0, try_larger, fun, fun_j, fun_g, bisection_max=5):
    """Step sig with xn = xj - sig*s satisfying Armijo f - fn >= delta*sig*stg
    and Wolfe gn's <= theta*stg (optlib_wolfe.m:19-159).  Returns
    (sig, xn, fn, gn, evaluations)."""
    import torch
    evals = 0
    sig = sig0
    xn = xj - sig * s
    fn, gn = fun(xn)
    evals += 1
    while f - fn < delta * sig * stg:  # halve until Armijo holds
        sig = 0.5 * sig
        xn = xj - sig * s
        fn = fun_j(xn)
        evals += 1
    if sig != sig0:
        gn = fun_g(xn)
        evals += 1
    wolfe_ok = float(torch.dot(gn, s)) <= theta * stg
    armijo = (sig, xn, fn, gn)
    if not wolfe_ok or try_larger:
        if sig == sig0:
            xnn = xj - 2 * sig * s
            fnn, gnn = fun(xnn)
            evals += 1
            while float(torch.dot(gn, s)) > theta * stg and f - fnn >= 2 * delta * sig * stg:
                sig = 2 * sig
                xn, fn, gn = xnn, fnn, gnn
                xnn = xj - 2 * sig * s
                fnn, gnn = fun(xnn)
                evals += 1
        sigp = 2 * sig
        it_bisec = 1
        while float(torch.dot(gn, s)) > theta * stg:
            if it_bisec > bisection_max:
                sig, xn, fn, gn = armijo  # keep the Armijo step
                break
            sigb = 0.5 * (sig + sigp)
            xb = xj - sigb * s
            fnn, gnn = fun(xb)
            evals += 1
            if f - fnn >= delta * sigb * stg:
                sig, xn, fn, gn = sigb, xb, fnn, gnn
            else:
                sigp = sigb
            it_bisec += 1
    return sig, xn, fn, gn, evals


def lbfgs(m0, fun: Callable, fun_j: Optional[Callable] = None, fun_g: Optional[Callable] = None,
          options: Optional[Options] = None) -> Result:
    import torch
    o = options or Options()
    fun_j = fun_j or (lambda x: fun(x)[0])
    fun_g = fun_g or (lambda x: fun(x)[1])
    m = m0.to(torch.float64).clone()
    j, g = fun(m)
    normg0 = float(torch.linalg.norm(g))
    normg = normg0
    hist = [(0, float(j), normg, None, None)]
    n, lmax = m.numel(), o.max_memory
    P = torch.zeros((lmax, n), dtype=torch.float64, device=m.device)
    D = torch.zeros_like(P)
    rho = [0.0] * lmax
    ga = [0.0] * lmax
    l, ln, gak = 0, 1, 1.0  # ln is the reference's 1-based ring position
    it = 0
    flag = None
    while normg > o.tolerance * normg0 and it < o.max_iterations:
        if it >= o.successive_iterations and abs(hist[it][1] - hist[it - o.successive_iterations][1]) < \
                o.successive_change:
            flag = 2
            break
        it += 1
        # two-loop recursion: s = B g
        q = g.clone()
        for jj in range(1, l + 1):
            i = (ln - jj - 1) % lmax
            ga[i] = rho[i] * float(torch.dot(P[i], q))
            q = q - ga[i] * D[i]
        r = gak * q
        for jj in range(l, 0, -1):
            i = (ln - jj - 1) % lmax
            be = rho[i] * float(torch.dot(D[i], r))
            r = r + (ga[i] - be) * P[i]
        s = r
        step = "LBFGS"
        stg = float(torch.dot(s, g))
        if _div(stg, normg * float(torch.linalg.norm(s))) < o.sufficient_decrease_angle:
            s = g.clone()  # bad angle: steepest descent
            stg = float(torch.dot(s, g))
            step = "Grad"
        sigma0 = o.init_step_length if it == 1 else 1.0
        sigma, mn, jn, gn, _ = wolfe(m, s, stg, float(j), o.wolfe_delta, o.wolfe_theta, sigma0,
                                     o.wolfe_try_to_increase_step_length, fun, fun_j, fun_g, o.bisection_max)
        d = g - gn
        p = m - mn
        dtp = float(torch.dot(d, p))
        if dtp >= 1e-8 * float(torch.linalg.norm(d)) * float(torch.linalg.norm(p)):
            rho[ln - 1] = _div(1.0, dtp)
            D[ln - 1] = d
            P[ln - 1] = p
            l = min(l + 1, lmax)
            ln = ln % lmax + 1
            gak = _div(dtp, float(torch.dot(d, d)))
        m, j, g = mn, jn, gn
        normg = float(torch.linalg.norm(g))
        hist.append((it, float(j), normg, sigma, step))
    if flag is None:
        flag = 0 if normg <= o.tolerance * normg0 else 1
    return Result(flag, m, float(j), g, hist)
