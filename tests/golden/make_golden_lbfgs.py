"""Generate golden vectors of the reference's L-BFGS driver.

TEST INFRASTRUCTURE.  The unmodified inversion/optlib/optlib_lbfgs.m (with
optlib_wolfe.m and optlib_init_default_parameters_lbfgs.m) is run by the
MATLAB-subset interpreter in mini_matlab.py on the problems of
wolfe_problems.py.  The callbacks it calls by name are builtins: the
objective (eval_objective_and_gradient, eval_objective, eval_grad_objective),
new_iteration (usr_par.model(it+1) = model, as the reference's inversion
callback does) and optlib_generate_random_string; fopen/fprintf/fclose keep
the iteration table (options.output_file) as text.  The unmodified
inversion/optlib_callback_fct/optlib_restore_lbfgs_information.m runs too:
every case starts without stored iterations, and the restart cases then run
optlib_lbfgs.m again from the final model with the first run's usr_par.model.
Outputs go to tests/golden/lbfgs_cases.npz.

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
from wolfe_problems import LBFGS_CASES, RESTART_CASES  # noqa: E402

OUT = os.path.join(HERE, "lbfgs_cases.npz")


def _fprintf_text(fmt, args):
    """MATLAB's fprintf formatting for the specifiers optlib_lbfgs.m uses."""
    fmt = str(fmt).replace("\\n", "\n").replace("\\t", "\t")
    vals = []
    for a in args:
        if isinstance(a, str):
            vals.append(a)
        else:
            vals.extend(float(v) for v in np.asarray(a, dtype=np.float64).ravel(order="F"))
    out, k, i = [], 0, 0
    while i < len(fmt):
        c = fmt[i]
        if c != "%":
            out.append(c)
            i += 1
            continue
        jdx = i + 1
        while fmt[jdx] not in "dieEfgs":
            jdx += 1
        spec, conv = fmt[i:jdx + 1], fmt[jdx]
        v = vals[k]
        k += 1
        if conv == "s":
            out.append(spec % v)
        elif isinstance(v, float) and (v != v or abs(v) == float("inf")):
            out.append("NaN" if v != v else ("Inf" if v > 0 else "-Inf"))
        elif conv in "di":
            out.append(spec % int(v))
        else:
            out.append(spec % v)
        i = jdx + 1
    return "".join(out)


def run_lbfgs(paths, fun, m0, opts, usr_par):
    n = len(m0)
    col = lambda v: np.asfortranarray(np.asarray(v, dtype=np.float64).reshape(-1, 1))  # noqa: E731
    table = []

    def fg(x, *_):
        f, g = fun(x)
        return [A(f), col(g), A(0.0)]

    def new_iteration(it, model, usr):
        lst = usr.setdefault("model", [])
        k = int(np.ravel(it)[0])
        if k < len(lst):
            lst[k] = copy.deepcopy(model)
        else:
            lst.append(copy.deepcopy(model))
        return [usr]

    def fprintf(*a):
        if a and not isinstance(a[0], str) and float(np.ravel(a[0])[0]) == 3.0:
            table.append(_fprintf_text(a[1], a[2:]))
        return []

    ov = {"eval_objective_and_gradient": fg,
          "eval_objective": lambda x, *_: [A(fun(x)[0])],
          "eval_grad_objective": lambda x, *_: [col(fun(x)[1]), A(0.0)],
          "new_iteration": new_iteration,
          "optlib_generate_random_string": lambda *_: "abcdefgh",
          "fopen": lambda *a: A(3.0), "fclose": lambda *a: A(0.0), "fprintf": fprintf}
    I = Interpreter(paths, ov)
    options = {k: (A(float(v)) if not isinstance(v, str) else v) for k, v in opts.items()}
    flag, mfinal, usr_par = I.call("optlib_lbfgs", [col(m0), options, usr_par], nargout=3)
    hist = np.array([float(np.ravel(m["objective"])[0]) for m in usr_par["model"]])
    assert n == np.asarray(mfinal).size
    return flag, mfinal, usr_par, hist, "".join(table)


def main():
    ref = reference_checkout(sys.argv)
    paths = [os.path.join(ref, "inversion", "optlib"), os.path.join(ref, "inversion", "optlib_callback_fct")]
    out = {}
    for name, fun, m0, opts in LBFGS_CASES:
        flag, mfinal, _, hist, table = run_lbfgs(paths, fun, m0, opts, {})
        out[f"{name}/flag"] = np.asarray(flag, dtype=np.float64).ravel()
        out[f"{name}/m"] = np.asarray(mfinal, dtype=np.float64).ravel()
        out[f"{name}/objectives"] = hist
        out[f"{name}/table"] = np.array(table)
        print(f"  {name}: flag {int(np.ravel(flag)[0])}, {hist.size - 1} iterations, j = {hist[-1]:.6g}", flush=True)
    for name, fun, m0, opts1, opts2 in RESTART_CASES:
        _, m1, usr, hist1, _ = run_lbfgs(paths, fun, m0, opts1, {})
        stored = {"model": copy.deepcopy(usr["model"])}
        flag, mfinal, usr2, hist, table = run_lbfgs(paths, fun, np.asarray(m1).ravel(), opts2, stored)
        out[f"{name}/first_m"] = np.asarray(m1, dtype=np.float64).ravel()
        out[f"{name}/first_models_m"] = np.array([np.asarray(e["m"], dtype=np.float64).ravel() for e in usr["model"]])
        out[f"{name}/first_models_g"] = np.array([np.asarray(e["gradient"], dtype=np.float64).ravel()
                                                 for e in usr["model"]])
        out[f"{name}/first_objectives"] = hist1
        out[f"{name}/flag"] = np.asarray(flag, dtype=np.float64).ravel()
        out[f"{name}/m"] = np.asarray(mfinal, dtype=np.float64).ravel()
        out[f"{name}/objectives"] = hist
        out[f"{name}/table"] = np.array(table)
        print(f"  {name}: first run {hist1.size - 1} iterations, restart flag {int(np.ravel(flag)[0])}, "
              f"{len(usr2['model'])} stored entries, j = {hist[-1]:.6g}", flush=True)
    np.savez_compressed(OUT, **out)
    print(f"wrote {OUT} ({os.path.getsize(OUT) / 1e3:.1f} kB, {len(out)} arrays)")


if __name__ == "__main__":
    main()
