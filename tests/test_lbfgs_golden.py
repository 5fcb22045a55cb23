"""The L-BFGS driver against the reference's optlib_lbfgs.m.

tests/golden/lbfgs_cases.npz holds what inversion/optlib/optlib_lbfgs.m (with
optlib_wolfe.m and optlib_init_default_parameters_lbfgs.m), run by the
MATLAB-subset interpreter (tests/golden/make_golden_lbfgs.py), returns on the
problems of tests/golden/wolfe_problems.py: the exit flag (0 gradient
tolerance, 1 iteration cap, 2 stagnation), the final model and the objective
of every iteration.  fd2d_noise_gb300.lbfgs.lbfgs must stop the same way after
the same number of iterations; values agree to rounding (vector products are
summed in a different order), relative to the starting objective.
"""
import os
import sys

import numpy as np
import pytest

sys.path.insert(0, os.path.join(os.path.dirname(__file__), "golden"))
import wolfe_problems as wp  # noqa: E402

_LBFGS = np.load(os.path.join(os.path.dirname(__file__), "golden", "lbfgs_cases.npz"))


@pytest.mark.parametrize("case", wp.LBFGS_CASES, ids=[c[0] for c in wp.LBFGS_CASES])
def test_lbfgs_matches_reference(case):
    import torch
    from fd2d_noise_gb300.lbfgs import Options, lbfgs
    name, fun, m0, opts = case
    o = Options(**{k: v for k, v in opts.items() if k != "verbose"})
    fg = lambda x: (lambda r: (r[0], torch.from_numpy(r[1])))(fun(x.numpy()))  # noqa: E731
    r = lbfgs(torch.tensor(m0, dtype=torch.float64), fg, lambda x: fun(x.numpy())[0],
              lambda x: torch.from_numpy(fun(x.numpy())[1]), options=o)
    ref_j = _LBFGS[f"{name}/objectives"]
    j = np.array([h[1] for h in r.history])
    assert r.flag == int(_LBFGS[f"{name}/flag"][0])
    assert j.size == ref_j.size  # same number of iterations
    np.testing.assert_allclose(j, ref_j, rtol=0, atol=1e-10 * ref_j[0])
    np.testing.assert_allclose(r.m.numpy(), _LBFGS[f"{name}/m"], rtol=0, atol=1e-10)
