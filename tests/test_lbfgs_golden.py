"""The L-BFGS driver against the reference's optlib_lbfgs.m.

tests/golden/lbfgs_cases.npz holds what inversion/optlib/optlib_lbfgs.m (with
optlib_wolfe.m and optlib_init_default_parameters_lbfgs.m), run by the
MATLAB-subset interpreter (tests/golden/make_golden_lbfgs.py), returns on the
problems of tests/golden/wolfe_problems.py: the exit flag (0 gradient
tolerance, 1 iteration cap, 2 stagnation), the final model and the objective
of every iteration.  fd2d_noise_gb300.lbfgs.lbfgs must stop the same way after
the same number of iterations; values agree to rounding (vector products are
summed in a different order), relative to the starting objective.  The
iteration table (iterations_lbfgs.tab) must read the same, line by line, with
its numbers equal to the printed digits; the restart cases warm-start from the
first run's stored iterations through the unmodified
optlib_restore_lbfgs_information.m.
"""
import os
import re
import sys

import numpy as np
import pytest

sys.path.insert(0, os.path.join(os.path.dirname(__file__), "golden"))
import wolfe_problems as wp  # noqa: E402

_LBFGS = np.load(os.path.join(os.path.dirname(__file__), "golden", "lbfgs_cases.npz"))


NUM = re.compile(r"-?(?:NaN|Inf|\d+\.\d+e[+-]\d+|\d+\.\d+|\d+)")


def _run(fun, m0, opts, tmp_path, stored=None):
    import torch
    from fd2d_noise_gb300.lbfgs import Options, lbfgs
    table = tmp_path / "iterations_lbfgs.tab"
    o = Options(**{k: v for k, v in opts.items() if k != "verbose"}, output_file=str(table))
    fg = lambda x: (lambda r: (r[0], torch.from_numpy(r[1])))(fun(x.numpy()))  # noqa: E731
    r = lbfgs(torch.tensor(m0, dtype=torch.float64), fg, lambda x: fun(x.numpy())[0],
              lambda x: torch.from_numpy(fun(x.numpy())[1]), options=o, stored=stored)
    return r, table.read_text()


def _same_table(got, want, scale):
    """Same lines and words; numbers equal to the printed digits (7 significant)
    or within the rounding of the run, relative to ``scale``."""
    g, w = got.splitlines(), want.splitlines()
    assert len(g) == len(w), (len(g), len(w))
    for a, b in zip(g, w):
        assert NUM.sub("#", a) == NUM.sub("#", b), (a, b)
        for x, y in zip(NUM.findall(a), NUM.findall(b)):
            fx, fy = float(x.replace("Inf", "inf")), float(y.replace("Inf", "inf"))
            if fx != fx or fy != fy:
                assert fx != fx and fy != fy, (a, b)
            else:
                assert abs(fx - fy) <= max(1e-6 * abs(fy), 1e-9 * scale), (a, b)


def _check(r, name):
    ref_j = _LBFGS[f"{name}/objectives"]
    j = np.array([h[1] for h in r.history])
    assert r.flag == int(_LBFGS[f"{name}/flag"][0])
    assert j.size == ref_j.size  # same number of iterations
    np.testing.assert_allclose(j, ref_j, rtol=0, atol=1e-10 * abs(ref_j[0]))
    np.testing.assert_allclose(r.m.numpy(), _LBFGS[f"{name}/m"], rtol=0, atol=1e-10)


@pytest.mark.parametrize("case", wp.LBFGS_CASES, ids=[c[0] for c in wp.LBFGS_CASES])
def test_lbfgs_matches_reference(case, tmp_path):
    name, fun, m0, opts = case
    r, table = _run(fun, m0, opts, tmp_path)
    _check(r, name)
    _same_table(table, str(_LBFGS[f"{name}/table"]), abs(r.history[0][1]))
    assert len(r.models) == len(r.history)  # usr_par.model: one entry per iteration


@pytest.mark.parametrize("case", wp.RESTART_CASES, ids=[c[0] for c in wp.RESTART_CASES])
def test_lbfgs_restart_matches_reference(case, tmp_path):
    """Warm start from the stored iterations of a first run
    (optlib_restore_lbfgs_information.m): the restored curvature pairs, rho,
    scaling and ring pointer steer the second run exactly as in the reference,
    down to the NaN run that follows a restore whose only pair is the current
    model itself."""
    import torch
    name, fun, m0, opts1, opts2 = case
    (tmp_path / "a").mkdir()
    r1, _ = _run(fun, m0, opts1, tmp_path / "a")
    np.testing.assert_allclose(np.array([h[1] for h in r1.history]), _LBFGS[f"{name}/first_objectives"], rtol=0,
                               atol=1e-12 * abs(r1.history[0][1]))
    # restart from the reference's own stored iterations (so that only the
    # second run's rounding enters)
    stored = [dict(m=torch.from_numpy(m), gradient=torch.from_numpy(g)) for m, g in
              zip(_LBFGS[f"{name}/first_models_m"], _LBFGS[f"{name}/first_models_g"])]
    r2, table = _run(fun, _LBFGS[f"{name}/first_m"], opts2, tmp_path, stored=stored)
    _check(r2, name)
    _same_table(table, str(_LBFGS[f"{name}/table"]), abs(r2.history[0][1]))


def test_restore_picks_the_reference_columns():
    from fd2d_noise_gb300.lbfgs import restore_lbfgs_information
    models = [dict(m=k, gradient=-k) for k in range(9)]
    pm, pg = restore_lbfgs_information(models)
    assert pm == [3, 4, 5, 6, 7] and pg == [-3, -4, -5, -6, -7]  # entries end-5 .. end-1, oldest first
    assert restore_lbfgs_information(models[:1]) == ([], [])
    assert restore_lbfgs_information(models[:3])[0] == [0, 1]


def test_restart_changes_the_path(tmp_path):
    """The restored pairs matter: a restart from the first run's final model
    without its history takes a different path."""
    name, fun, m0, opts1, opts2 = wp.RESTART_CASES[0]
    cold, _ = _run(fun, _LBFGS[f"{name}/first_m"], opts2, tmp_path)
    ref_j = _LBFGS[f"{name}/objectives"]
    j = np.array([h[1] for h in cold.history])
    n = min(j.size, ref_j.size)
    assert j.size != ref_j.size or np.abs(j[:n] - ref_j[:n]).max() > 1e-6 * abs(ref_j[0])
