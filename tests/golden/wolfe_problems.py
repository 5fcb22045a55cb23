"""Line-search test problems shared by make_golden_wolfe.py and the tests.

TEST INFRASTRUCTURE.  Each case: objective and gradient (numpy, FP64), start
point, search direction rule and the optlib_wolfe arguments.
"""
import numpy as np


def rosenbrock(x):
    x = np.asarray(x, dtype=np.float64).ravel()
    f = 100.0 * (x[1] - x[0] ** 2) ** 2 + (1.0 - x[0]) ** 2
    g = np.array([-400.0 * x[0] * (x[1] - x[0] ** 2) - 2.0 * (1.0 - x[0]), 200.0 * (x[1] - x[0] ** 2)])
    return f, g


DIAG = np.array([1.0, 3.0, 10.0, 30.0, 100.0])


def quadratic(x):
    x = np.asarray(x, dtype=np.float64).ravel()
    return 0.5 * float(np.sum(DIAG * x * x)), DIAG * x


# name, function, start, direction ('gradient' or 'newton'), sig0, try_larger_steps
CASES = [
    ("rosen_far", rosenbrock, [-1.2, 1.0], "gradient", 1.0, 1),
    ("rosen_small_step", rosenbrock, [0.5, 0.2], "gradient", 1e-3, 1),
    ("rosen_no_expand", rosenbrock, [0.5, 0.2], "gradient", 1e-3, 0),
    ("quad_gradient", quadratic, [1.0, -1.0, 1.0, -1.0, 1.0], "gradient", 0.05, 0),
    ("quad_gradient_long", quadratic, [1.0, 1.0, 1.0, 1.0, 1.0], "gradient", 0.002, 1),
    ("quad_newton", quadratic, [1.0, 2.0, 3.0, 4.0, 5.0], "newton", 1.0, 1),
    ("rosen_bisect", rosenbrock, [-0.2125, -0.4], "gradient", 0.0557, 1),
    ("rosen_halve_bisect", rosenbrock, [-1.4323, 1.317], "gradient", 0.0125, 1),
]
DELTA, THETA = 0.001, 0.6  # optlib_init_default_parameters_lbfgs defaults (wolfe_delta, wolfe_theta)


def direction(fun, x, rule):
    f, g = fun(x)
    s = g.copy() if rule == "gradient" else g / DIAG
    return f, g, s

# L-BFGS driver cases: name, function, start, options given to optlib_lbfgs
# (the rest take the defaults of optlib_init_default_parameters_lbfgs)
LBFGS_CASES = [
    ("rosen_converge", rosenbrock, [-1.2, 1.0],
     dict(verbose=0, tolerance=1e-8, max_iterations=200, successive_change=0.0)),
    ("rosen_stagnation", rosenbrock, [-1.2, 1.0], dict(verbose=0)),
    ("rosen_capped", rosenbrock, [-1.2, 1.0], dict(verbose=0, max_iterations=7, successive_change=0.0)),
    ("quad_defaults", quadratic, [1.0, 1.0, 1.0, 1.0, 1.0], dict(verbose=0)),
    ("quad_tight", quadratic, [1.0, -2.0, 3.0, -4.0, 5.0],
     dict(verbose=0, tolerance=1e-10, successive_change=0.0, init_step_length=0.01)),
]

# Warm restarts (optlib_restore_lbfgs_information.m): name, function, start,
# options of the first run, options of the run restarted from its final model
# with its stored iterations.  Histories of 7 (five pairs restored), 2 (one
# pair) and 7 entries with max_memory 3 (lmax = max(3, 5) = 5).
RESTART_CASES = [
    ("restart_rosen", rosenbrock, [-1.2, 1.0],
     dict(verbose=0, max_iterations=6, successive_change=0.0),
     dict(verbose=0, tolerance=1e-8, max_iterations=60, successive_change=0.0)),
    ("restart_rosen_short", rosenbrock, [0.5, 0.2],
     dict(verbose=0, max_iterations=1, successive_change=0.0),
     dict(verbose=0, max_iterations=12, successive_change=0.0)),
    ("restart_quad_mem3", quadratic, [1.0, -2.0, 3.0, -4.0, 5.0],
     dict(verbose=0, max_iterations=6, successive_change=0.0, max_memory=3),
     dict(verbose=0, tolerance=1e-9, max_iterations=40, successive_change=0.0, max_memory=3)),
]
