"""Grid and absorbing taper against the reference's own code.

tests/golden/setup_cases.npz holds what the unmodified
code/propagation/define_computational_domain.m and init_absbound.m return when
run by the MATLAB-subset interpreter (tests/golden/make_golden_setup.py):
non-square grids, narrow and half-domain layers, all four sides or some.  The
grid coordinates (MATLAB's colon operator) must match exactly; the taper to a
few units in the last place, the difference between two libm exp
implementations (the interpreter uses numpy's, the oracle the C library's;
MATLAB's is a third).
"""
import os

import numpy as np
import pytest

from fd2d_noise_gb300.config import Config, define_computational_domain

GOLDEN = np.load(os.path.join(os.path.dirname(__file__), "golden", "setup_cases.npz"))
CASES = sorted({k.split("/")[0] for k in GOLDEN.files})


def _cfg(name):
    g = lambda k: np.asarray(GOLDEN[f"{name}/{k}"]).ravel()  # noqa: E731
    fl = g("flags").astype(int)
    return Config(Lx=float(g("Lx")[0]), Lz=float(g("Lz")[0]), nx=int(g("nx")[0]), nz=int(g("nz")[0]),
                  absorb_width=float(g("width")[0]), absorb_left=int(fl[0]), absorb_right=int(fl[1]),
                  absorb_top=int(fl[2]), absorb_bottom=int(fl[3]))


@pytest.mark.parametrize("name", CASES)
def test_oracle_grid_and_taper_match_reference(oracle, name):
    cfg = _cfg(name)
    x, z, ab = oracle.setup_arrays(cfg)
    assert np.array_equal(x, GOLDEN[f"{name}/x"].ravel())
    assert np.array_equal(z, GOLDEN[f"{name}/z"].ravel())
    ref = GOLDEN[f"{name}/absbound"]
    assert ab.shape == ref.shape
    np.testing.assert_allclose(ab, ref, rtol=1e-15, atol=0)


@pytest.mark.parametrize("name", CASES)
def test_host_grid_matches_reference(name):
    cfg = _cfg(name)
    X, Z, x, z, dx, dz = define_computational_domain(cfg.Lx, cfg.Lz, cfg.nx, cfg.nz)
    assert np.array_equal(x, GOLDEN[f"{name}/x"].ravel()) and np.array_equal(z, GOLDEN[f"{name}/z"].ravel())
    assert dx == GOLDEN[f"{name}/dx"].ravel()[0] and dz == GOLDEN[f"{name}/dz"].ravel()[0]
    assert X.shape == (cfg.nz, cfg.nx)
