"""The Powell-Wolfe line search against the reference's optlib_wolfe.m.

tests/golden/wolfe_cases.npz holds what inversion/optlib/optlib_wolfe.m, run by
the MATLAB-subset interpreter (tests/golden/make_golden_wolfe.py), returns on
the problems of tests/golden/wolfe_problems.py, and every point it evaluated
with which callback (0: objective and gradient, 1: objective, 2: gradient).
The cases take the Armijo halving, expansion, bisection and
immediate-acceptance paths; fd2d_noise_gb300.lbfgs.wolfe must take the same
steps to the last bit.
"""
import os
import sys

import numpy as np
import pytest

sys.path.insert(0, os.path.join(os.path.dirname(__file__), "golden"))
import wolfe_problems as wp  # noqa: E402

_WOLFE = np.load(os.path.join(os.path.dirname(__file__), "golden", "wolfe_cases.npz"))


@pytest.mark.parametrize("case", wp.CASES, ids=[c[0] for c in wp.CASES])
def test_wolfe_matches_reference(case):
    import torch
    from fd2d_noise_gb300.lbfgs import wolfe
    name, fun, x0, rule, sig0, larger = case
    calls = []

    def fg(x):
        calls.append((0, x.numpy().copy()))
        f, g = fun(x.numpy())
        return f, torch.from_numpy(g)

    def f_only(x):
        calls.append((1, x.numpy().copy()))
        return fun(x.numpy())[0]

    def g_only(x):
        calls.append((2, x.numpy().copy()))
        return torch.from_numpy(fun(x.numpy())[1])

    x = np.asarray(x0, dtype=np.float64)
    f, g, s = wp.direction(fun, x, rule)
    stg = float(s @ g)
    sig, xn, fn, gn, _ = wolfe(torch.from_numpy(x), torch.from_numpy(s), stg, f, wp.DELTA, wp.THETA, sig0,
                               bool(larger), fg, f_only, g_only)
    ref = lambda k: _WOLFE[f"{name}/{k}"]  # noqa: E731
    assert sig == ref("sig")[0]
    assert np.array_equal(xn.numpy(), ref("m")) and fn == ref("objective")[0]
    assert np.array_equal(gn.numpy(), ref("gradient"))
    assert [k for k, _ in calls] == list(ref("call_kinds"))
    assert np.array_equal(np.array([p for _, p in calls]), ref("call_points"))
