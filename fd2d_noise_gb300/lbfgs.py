"""L-BFGS with the Powell-Wolfe step-size rule, FP64 vectors on the device.

    optlib_lbfgs   inversion/optlib/optlib_lbfgs.m:1-210
    optlib_wolfe   inversion/optlib/optlib_wolfe.m:1-159
    defaults       inversion/optlib/optlib_init_default_parameters_lbfgs.m
    restore        inversion/optlib_callback_fct/optlib_restore_lbfgs_information.m:20-54
    model history  inversion/optlib_callback_fct/new_iteration.m:31 (usr_par.model(it+1) = model)

Vectors are torch FP64 tensors on the device of ``m0`` (CUDA or CPU); the
callbacks receive and return tensors of that device: ``fun(m) -> (j, g)``
(eval_objective_and_gradient), ``fun_j(m) -> j`` (eval_objective) and
``fun_g(m) -> g`` (eval_grad_objective).  The iteration log, the stopping rules
(relative gradient norm, iteration cap, stagnation over
``successive_iterations``) and the curvature / descent-angle safeguards are
the reference's.

``Result.models`` is the reference's ``usr_par.model``: one entry per iteration
(``m``, ``objective``, ``gradient``, ``normg``), entry ``it`` written when
iteration ``it`` ends.  Passing it back as ``stored`` warm-starts a new run as
optlib_restore_lbfgs_information.m does: entry 0 becomes the new start, and up
to five of the remaining most recent entries (all but the last) seed the
curvature pairs, ``rho`` and the initial scaling.  The restored ring pointer is
the reference's (``l = ln = l_history``): the first new pair overwrites the
newest restored one, and the recursion visits the restored pairs in the
reference's order.

``Options.output_file`` appends the reference's iteration table
(iterations_lbfgs.tab: one line per iteration, the descent-angle and curvature
warnings and the termination line) in its format; None writes no file.
"""
from __future__ import annotations

from dataclasses import dataclass, field
from typing import Callable, List, Optional

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
    output_file: Optional[str] = None  # the reference writes 'iterations_lbfgs.tab'


NUM_MOD_GRAD_STORED = 5  # optlib_restore_lbfgs_information.m:21


@dataclass
class Result:
    flag: int                 # 0 gradient tolerance, 1 iteration cap, 2 stagnation
    m: object
    objective: float
    gradient: object
    history: list = field(default_factory=list)  # (it, objective, ||g||, sigma, step)
    models: list = field(default_factory=list)   # usr_par.model: dicts m, objective, gradient, normg


def _num(fmt: str, v: float) -> str:
    """One number as MATLAB's fprintf writes it (NaN and Inf spelt its way)."""
    v = float(v)
    if v != v:
        return "NaN"
    if v in (float("inf"), float("-inf")):
        return "Inf" if v > 0 else "-Inf"
    return fmt % v


class _Table:
    """The iteration table of optlib_lbfgs.m:11,25,112,169,188,198-204."""

    def __init__(self, path: Optional[str]):
        self.f = open(path, "a+") if path else None

    def write(self, text: str):
        if self.f:
            self.f.write(text)

    def close(self):
        if self.f:
            self.f.close()


def restore_lbfgs_information(models: List[dict]):
    """(previous_models, previous_gradients) as lists, oldest first, the
    newest last: entries end-1-maxprev .. end-2 of ``models`` (all but the
    last, at most NUM_MOD_GRAD_STORED)."""
    nprev = len(models) - 1
    if nprev <= 0:
        return [], []
    maxprev = min(nprev, NUM_MOD_GRAD_STORED)
    picked = [models[len(models) - 1 - iprev] for iprev in range(maxprev, 0, -1)]
    return [e["m"] for e in picked], [e["gradient"] for e in picked]


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
          options: Optional[Options] = None, stored: Optional[List[dict]] = None) -> Result:
    import torch
    o = options or Options()
    fun_j = fun_j or (lambda x: fun(x)[0])
    fun_g = fun_g or (lambda x: fun(x)[1])
    table = _Table(o.output_file)
    try:
        return _lbfgs(m0, fun, fun_j, fun_g, o, list(stored or []), table, torch)
    finally:
        table.close()


def _new_iteration(models: list, it: int, m, j: float, g, normg: float):
    entry = dict(m=m, objective=float(j), gradient=g, normg=normg)
    if it < len(models):
        models[it] = entry
    else:
        models.append(entry)


def _lbfgs(m0, fun, fun_j, fun_g, o: Options, models: list, table: _Table, torch) -> Result:
    m = m0.to(torch.float64).clone()
    j, g = fun(m)
    normg0 = float(torch.linalg.norm(g))
    normg = normg0
    _new_iteration(models, 0, m, j, g, normg)
    table.write("it=%d   j=%s   ||g||=%s  \n" % (0, _num("%e", j), _num("%e", normg)))
    hist = [(0, float(j), normg, None, None)]
    n = m.numel()
    prev_m, prev_g = restore_lbfgs_information(models)
    l_history = len(prev_m)
    if l_history > 0:
        lmax = max(o.max_memory, l_history)
        P = torch.zeros((lmax, n), dtype=torch.float64, device=m.device)
        D = torch.zeros_like(P)
        rho = [0.0] * lmax
        ga = [0.0] * lmax
        for i in range(1, l_history):
            P[i - 1] = prev_m[i - 1].to(m) - prev_m[i].to(m)
            D[i - 1] = prev_g[i - 1].to(m) - prev_g[i].to(m)
        P[l_history - 1] = prev_m[l_history - 1].to(m) - m
        D[l_history - 1] = prev_g[l_history - 1].to(m) - g
        for i in range(l_history):
            rho[i] = _div(1.0, float(torch.dot(D[i], P[i])))
        dl = D[l_history - 1]
        gak = _div(float(torch.dot(dl, P[l_history - 1])), float(torch.linalg.norm(dl)) ** 2)
        l = ln = min(lmax, l_history)
    else:
        lmax = o.max_memory
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
            table.write("\tWarning: Bad angle of search direction. Use steepest descent instead.\n")
            s = g.clone()  # bad angle: steepest descent
            stg = float(torch.dot(s, g))
            step = "Grad"
        sigma0 = o.init_step_length if it == 1 else 1.0
        sigma, mn, jn, gn, _ = wolfe(m, s, stg, float(j), o.wolfe_delta, o.wolfe_theta, sigma0,
                                     o.wolfe_try_to_increase_step_length, fun, fun_j, fun_g, o.bisection_max)
        normgn = float(torch.linalg.norm(gn))
        table.write("it=%d   j=%s   ||g||=%s   sigma=%s ||s||=%s  step=%s\n"
                    % (it, _num("%e", jn), _num("%e", normgn), _num("%6.5f", sigma),
                       _num("%e", float(torch.linalg.norm(s))), step))
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
        else:
            table.write("\tWarning: Bad angle of search direction. Update of BFGS curvature information "
                        "skipped.\n")
        m, j, g = mn, jn, gn
        normg = normgn
        _new_iteration(models, it, m, j, g, normg)
        hist.append((it, float(j), normg, sigma, step))
    if flag is None:  # optlib_lbfgs.m:197-206 (a NaN gradient norm ends the loop with flag 2)
        flag = 0 if normg <= o.tolerance * normg0 else (1 if it >= o.max_iterations else 2)
    if flag == 0:
        table.write("Successful termination with ||g||<%s*min(1,||g0||):\n" % _num("%e", o.tolerance))
    elif flag == 1:
        table.write("Maximum number of iterations reached.\n")
    else:
        table.write("Improvement of misfit over %d iterations smaller than %s.\n"
                    % (o.successive_iterations, _num("%f", o.successive_change)))
    return Result(flag, m, float(j), g, hist, models)
