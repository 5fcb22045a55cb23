"""Gaussian smoothing of model and gradient maps (tools/addons/gaussblur2d.m,
inversion/optlib_callback_fct/map_*.m) against the reference's own gaussblur2d
run by the MATLAB-subset interpreter (tests/golden/map_cases.npz)."""
import os

import numpy as np
import pytest

from oracle import model_maps as om

GOLD = np.load(os.path.join(os.path.dirname(__file__), "golden", "map_cases.npz"))
CASES = sorted({k.split("/")[0] for k in GOLD.files})


def _case(c):
    return GOLD[c + "/Y"], GOLD[c + "/x1"].ravel(), GOLD[c + "/x2"].ravel(), GOLD[c + "/sigma"].ravel(), GOLD[c + "/GY"]


@pytest.mark.parametrize("c", CASES)
def test_oracle_matches_reference(c):
    Y, x1, x2, s, GY = _case(c)
    # rounding differs only in elements close to zero (interpreter vs numpy)
    np.testing.assert_allclose(om.gaussblur2d(Y, x1, x2, s), GY, rtol=1e-13, atol=1e-15)


def test_smoothing_keeps_constants_and_is_local():
    # normalised weights: a constant map stays constant; the weights vanish
    # beyond sqrt(14) sigma
    x1, x2 = np.arange(20) * 1e3, np.arange(15) * 1e3
    s = (2e3, 3e3)
    np.testing.assert_allclose(om.gaussblur2d(np.full((20, 15), 2.5), x1, x2, s), 2.5, rtol=1e-13)
    d = np.zeros((20, 15))
    d[10, 7] = 1.0
    g = om.gaussblur2d(d, x1, x2, s)
    assert g[10, 7] > 0 and g[17, 7] > 0 and g[18, 7] == 0.0


def test_map_round_trip():
    nx, nz = 24, 20
    ab = np.zeros((nx, nz))
    ab[3:nx - 3, 3:nz - 3] = 1.0
    p = np.random.default_rng(1).standard_normal((nx, nz, 2)) * 0.01
    p[:, :, -1] = 4.8e10 * (1.0 + p[:, :, -1])
    m = om.map_parameters_to_m(p, 0.0, 1.0, 4.8e10)
    np.testing.assert_allclose(m.reshape(nx, nz, 2, order="F")[:, :, -1], p[:, :, -1] / 4.8e10 - 1.0)


@pytest.mark.gpu
@pytest.mark.parametrize("c", CASES)
def test_gpu_matches_reference(fd2d_lib, c):
    from fd2d_noise_gb300.model_maps import gaussblur2d
    Y, x1, x2, s, GY = _case(c)
    # CUDA's exp differs from the host's by an ulp at most
    np.testing.assert_allclose(gaussblur2d(Y, x1, x2, s), GY, rtol=1e-13, atol=1e-15)


@pytest.mark.gpu
def test_gpu_gradient_map_matches_oracle(fd2d_lib):
    from fd2d_noise_gb300 import model_maps as mm
    nx, nz = 40, 36
    x, z = np.arange(nx) * 2e3, np.arange(nz) * 2e3
    ab = np.zeros((nx, nz))
    ab[5:nx - 5, 4:nz - 4] = 1.0
    g = np.random.default_rng(7).standard_normal((nx, nz, 3))
    got = mm.map_gradparameters_to_gradm(g, ab, x, z, (4e3, 4e3), (6e3, 5e3), 4.8e10)
    want = om.map_gradparameters_to_gradm(g, ab, x, z, (4e3, 4e3), (6e3, 5e3), 4.8e10)
    np.testing.assert_allclose(got, want, rtol=1e-12, atol=1e-25)
    m = mm.map_parameters_to_m(om.map_m_to_parameters(g.ravel(order="F"), nx, nz, ab, x, z, (4e3, 4e3),
                                                      (6e3, 5e3), 0.0, 1.0, 4.8e10), 0.0, 1.0, 4.8e10)
    p = mm.map_m_to_parameters(m, nx, nz, ab, x, z, (4e3, 4e3), (6e3, 5e3), 0.0, 1.0, 4.8e10)
    q = om.map_m_to_parameters(m, nx, nz, ab, x, z, (4e3, 4e3), (6e3, 5e3), 0.0, 1.0, 4.8e10)
    np.testing.assert_allclose(p, q, rtol=1e-12)
