"""Generate golden vectors of the reference's Powell-Wolfe line search.

TEST INFRASTRUCTURE.  The unmodified inversion/optlib/optlib_wolfe.m is run by
the MATLAB-subset interpreter in mini_matlab.py on the problems of
wolfe_problems.py; the objective callbacks it calls by name
(eval_objective_and_gradient, eval_objective, eval_grad_objective) and
optlib_generate_random_string are supplied as builtins that record every
point the line search evaluates.  Outputs go to tests/golden/wolfe_cases.npz.

    python tests/golden/make_golden_wolfe.py <path-to-reference-checkout> (or FD2D_REFERENCE set)
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
from mini_matlab import A, Interpreter, reference_checkout  # noqa: E402
from wolfe_problems import CASES, DELTA, THETA, direction  # noqa: E402

OUT = os.path.join(HERE, "wolfe_cases.npz")


def main():
    ref = reference_checkout(sys.argv)
    paths = [os.path.join(ref, "inversion", "optlib")]
    out = {}
    for name, fun, x0, rule, sig0, larger in CASES:
        calls = []  # (kind, point): 0 = objective and gradient, 1 = objective, 2 = gradient

        def fg(x, *_):
            calls.append((0, np.asarray(x, dtype=np.float64).ravel().copy()))
            f, g = fun(x)
            return [A(f), np.asfortranarray(g.reshape(-1, 1)), A(0.0)]

        def f_only(x, *_):
            calls.append((1, np.asarray(x, dtype=np.float64).ravel().copy()))
            return [A(fun(x)[0])]

        def g_only(x, *_):
            calls.append((2, np.asarray(x, dtype=np.float64).ravel().copy()))
            return [np.asfortranarray(fun(x)[1].reshape(-1, 1)), A(0.0)]

        ov = {"eval_objective_and_gradient": fg, "eval_objective": f_only, "eval_grad_objective": g_only,
              "optlib_generate_random_string": lambda *_: "abcdefgh"}
        I = Interpreter(paths, ov)
        x = np.asarray(x0, dtype=np.float64)
        f, g, s = direction(fun, x, rule)
        stg = float(s @ g)
        col = lambda v: np.asfortranarray(np.asarray(v, dtype=np.float64).reshape(-1, 1))  # noqa: E731
        sig, model = I.call("optlib_wolfe", [col(x), col(s), A(stg), A(f), A(DELTA), A(THETA), A(sig0),
                                             A(float(larger)), A(0.0), A(0.0)], nargout=2)
        out[f"{name}/sig"] = np.asarray(sig, dtype=np.float64).ravel()
        out[f"{name}/m"] = np.asarray(model["m"], dtype=np.float64).ravel()
        out[f"{name}/objective"] = np.asarray(model["objective"], dtype=np.float64).ravel()
        out[f"{name}/gradient"] = np.asarray(model["gradient"], dtype=np.float64).ravel()
        out[f"{name}/call_kinds"] = np.array([k for k, _ in calls], dtype=np.int64)
        out[f"{name}/call_points"] = np.array([p for _, p in calls])
        print(f"  {name}: sig {float(np.ravel(sig)[0]):.6g}, {len(calls)} evaluations "
              f"{[k for k, _ in calls]}", flush=True)
    np.savez_compressed(OUT, **out)
    print(f"wrote {OUT} ({os.path.getsize(OUT) / 1e3:.1f} kB, {len(out)} arrays)")


if __name__ == "__main__":
    main()
