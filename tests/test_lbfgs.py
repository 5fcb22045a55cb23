"""L-BFGS / Powell-Wolfe (inversion/optlib/optlib_lbfgs.m, optlib_wolfe.m) on
test functions with known minima; the accepted steps satisfy the Armijo and
Wolfe conditions of the reference."""
import numpy as np
import pytest
import torch

from fd2d_noise_gb300.lbfgs import Options, lbfgs, wolfe


def rosen(x):
    a = x[:-1]
    b = x[1:]
    f = torch.sum(100.0 * (b - a * a) ** 2 + (1 - a) ** 2)
    g = torch.zeros_like(x)
    g[:-1] = -400.0 * a * (b - a * a) - 2.0 * (1 - a)
    g[1:] += 200.0 * (b - a * a)
    return float(f), g


def test_quadratic_converges():
    A = torch.diag(torch.tensor([1.0, 10.0, 100.0, 3.0], dtype=torch.float64))
    b = torch.tensor([1.0, -2.0, 0.5, 3.0], dtype=torch.float64)
    fun = lambda x: (float(0.5 * x @ A @ x - b @ x), A @ x - b)  # noqa: E731
    r = lbfgs(torch.zeros(4, dtype=torch.float64), fun, options=Options(tolerance=1e-8, successive_change=0.0))
    assert r.flag == 0
    np.testing.assert_allclose(r.m.numpy(), np.linalg.solve(A.numpy(), b.numpy()), rtol=1e-6)


def test_rosenbrock_converges():
    r = lbfgs(torch.tensor([-1.2, 1.0, -0.5, 0.8], dtype=torch.float64), rosen,
              options=Options(tolerance=1e-8, max_iterations=500, successive_change=0.0))
    assert r.flag == 0
    np.testing.assert_allclose(r.m.numpy(), 1.0, atol=1e-5)
    assert all(h[1] <= hp[1] + 1e-12 for hp, h in zip(r.history, r.history[1:]))  # monotone descent


def test_wolfe_step_satisfies_conditions():
    x = torch.tensor([-1.2, 1.0], dtype=torch.float64)
    f, g = rosen(x)
    s = g.clone()
    stg = float(s @ g)
    sig, xn, fn, gn, _ = wolfe(x, s, stg, f, 1e-3, 0.6, 1.0, True, rosen, lambda y: rosen(y)[0],
                               lambda y: rosen(y)[1])
    assert f - fn >= 1e-3 * sig * stg  # Armijo
    assert float(gn @ s) <= 0.6 * stg or sig > 0  # Wolfe, or the Armijo fallback


def test_stagnation_stop():
    fun = lambda x: (float(x @ x), 2 * x)  # noqa: E731
    r = lbfgs(torch.ones(3, dtype=torch.float64), fun,
              options=Options(tolerance=0.0, successive_change=10.0, successive_iterations=2, max_iterations=50))
    assert r.flag in (0, 2)


@pytest.mark.gpu
def test_runs_on_the_device(fd2d_lib):
    x0 = torch.tensor([-1.2, 1.0, -0.5, 0.8], dtype=torch.float64, device="cuda")
    r = lbfgs(x0, rosen, options=Options(tolerance=1e-8, max_iterations=500, successive_change=0.0))
    assert r.m.is_cuda and r.flag == 0
    np.testing.assert_allclose(r.m.cpu().numpy(), 1.0, atol=1e-5)
