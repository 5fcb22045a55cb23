"""Generate golden vectors of the reference's L-BFGS driver.

TEST INFRASTRUCTURE.  The unmodified inversion/optlib/optlib_lbfgs.m (with
optlib_wolfe.m and optlib_init_default_parameters_lbfgs.m) is run by the
MATLAB-subset interpreter in mini_matlab.py on the problems of
wolfe_problems.py.  The callbacks it calls by name are builtins: the
objective (eval_objective_and_gradient, eval_objective, eval_grad_objective),
new_iteration (keeps each iteration's model in usr_par.model, as the
reference's inversion callback does), optlib_restore_lbfgs_information (no
stored iterations) and optlib_generate_random_string.  Outputs go to
tests/golden/lbfgs_cases.npz.

    python tests/golden/make_golden_lbfgs.py <path-to-reference-checkout> (or FD2D_REFERENCE set)
"""
from __future__ import annotations

import copy
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
from mini_matlab import A, Interpreter, reference_checkout  # noqa: E402
from wolfe_problems import LBFGS_CASES  # noqa: E402

OUT = os.path.join(HERE, "lbfgs_cases.npz")


def main():
    ref = reference_checkout(sys.argv)
    paths = [os.path.join(ref, "inversion", "optlib")]
    out = {}
    for name, fun, m0, opts in LBFGS_CASES:
        n = len(m0)
        col = lambda v: np.asfortranarray(np.asarray(v, dtype=np.float64).reshape(-1, 1))  # noqa: E731

        def fg(x, *_):
            f, g = fun(x)
            return [A(f), col(g), A(0.0)]

        def new_iteration(it, model, usr_par):
            usr_par.setdefault("model", []).append(copy.deepcopy(model))
            return [usr_par]

        ov = {"eval_objective_and_gradient": fg,
              "eval_objective": lambda x, *_: [A(fun(x)[0])],
              "eval_grad_objective": lambda x, *_: [col(fun(x)[1]), A(0.0)],
              "new_iteration": new_iteration,
              "optlib_restore_lbfgs_information": lambda *_: [np.zeros((n, 0)), np.zeros((n, 0))],
              "optlib_generate_random_string": lambda *_: "abcdefgh"}
        I = Interpreter(paths, ov)
        options = {k: (A(float(v)) if not isinstance(v, str) else v) for k, v in opts.items()}
        flag, mfinal, usr_par = I.call("optlib_lbfgs", [col(m0), options, {}], nargout=3)
        hist = np.array([float(np.ravel(m["objective"])[0]) for m in usr_par["model"]])
        out[f"{name}/flag"] = np.asarray(flag, dtype=np.float64).ravel()
        out[f"{name}/m"] = np.asarray(mfinal, dtype=np.float64).ravel()
        out[f"{name}/objectives"] = hist
        print(f"  {name}: flag {int(np.ravel(flag)[0])}, {hist.size - 1} iterations, j = {hist[-1]:.6g}", flush=True)
    np.savez_compressed(OUT, **out)
    print(f"wrote {OUT} ({os.path.getsize(OUT) / 1e3:.1f} kB, {len(out)} arrays)")


if __name__ == "__main__":
    main()
