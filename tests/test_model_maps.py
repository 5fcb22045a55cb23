"""Model and gradient maps (tools/addons/gaussblur2d.m,
inversion/optlib_callback_fct/map_*.m) against the reference's own gaussblur2d
and map_*.m files run by the MATLAB-subset interpreter
(tests/golden/map_cases.npz), in the Gaussian-smoothing branch and the 'ring'
branch (annulus taper on the first source plane, imfilter 'circular' on the
structure plane)."""
import os
import types

import numpy as np
import pytest

from oracle import model_maps as om

GOLD = np.load(os.path.join(os.path.dirname(__file__), "golden", "map_cases.npz"))
CASES = sorted({k.split("/")[0] for k in GOLD.files if not k.startswith("map_")})
MAP_CASES = sorted({k.split("/")[0] for k in GOLD.files if k.startswith("map_")})


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


def _map_case(c):
    """Inputs of one map_m_to_parameters / map_gradparameters_to_gradm case:
    the domain of define_computational_domain.m (x = 0:dx:Lx, z = 0:dz:Lz)."""
    from fd2d_noise_gb300.config import matlab_colon
    g = lambda k: GOLD[f"{c}/{k}"]  # noqa: E731
    nx, nz, Lx, Lz = g("shape")
    nx, nz = int(nx), int(nz)
    x, z = matlab_colon(0.0, Lx / (nx - 1), Lx), matlab_colon(0.0, Lz / (nz - 1), Lz)
    ring = h = None
    if f"{c}/ring" in GOLD.files:
        r = g("ring")
        ring = types.SimpleNamespace(x_center_ring=r[0], z_center_ring=r[1], radius=r[2], thickness=r[3],
                                     taper_strength=r[4])
        h = g("h")
    p = g("p").reshape(nx, nz, -1, order="F")
    args = dict(m=g("m"), nx=nx, nz=nz, absbound=g("absbound"), x=x, z=z, sigma=g("sigma"), ring=ring, h=h,
                g=g("g").reshape(nx, nz, -1, order="F"))
    return args, p, g("gm")


def _oracle_maps(a, om_=om):
    p = om_.map_m_to_parameters(a["m"], a["nx"], a["nz"], a["absbound"], a["x"], a["z"], a["sigma"][0],
                                a["sigma"][1], 0.25, 1.0, 4.8e10, ring=a["ring"], h_structure=a["h"])
    gm = om_.map_gradparameters_to_gradm(a["g"], a["absbound"], a["x"], a["z"], a["sigma"][0], a["sigma"][1],
                                         4.8e10, ring=a["ring"], h_structure=a["h"])
    return p, gm


def _close(got, want):
    # exp, pow and the filter sums round differently in numpy and the
    # interpreter's numpy calls (different summation order)
    np.testing.assert_allclose(got, want, rtol=0, atol=1e-13 * np.abs(want).max())


@pytest.mark.parametrize("c", MAP_CASES)
def test_oracle_maps_match_reference(c):
    a, p, gm = _map_case(c)
    got_p, got_gm = _oracle_maps(a)
    _close(got_p, p)
    _close(got_gm, gm)


def test_ring_fixtures_pin_the_orientation_and_the_masked_plane():
    """The off-centre ring case rejects a transposed annulus (X from z, Z from
    x) and a mask applied to every source plane."""
    a, p, _ = _map_case("map_ring_offcentre")
    assert a["ring"].x_center_ring != a["ring"].z_center_ring and a["x"][-1] != a["z"][-1]
    swapped = dict(a, x=a["z"], z=a["x"],
                   ring=types.SimpleNamespace(**dict(vars(a["ring"]), x_center_ring=a["ring"].z_center_ring,
                                                     z_center_ring=a["ring"].x_center_ring)))
    sw_p, _ = _oracle_maps(swapped)
    assert np.abs(sw_p[:, :, 0] - p[:, :, 0]).max() > 1e-3
    b, p3, _ = _map_case("map_ring3")
    assert p3.shape[2] == 3
    # the second source plane passes through untouched: only plane 1 is masked
    m = b["m"].reshape(b["nx"], b["nz"], 3, order="F")
    np.testing.assert_array_equal(p3[:, :, 1], 0.25 + m[:, :, 1])
    assert (p3[:, :, 0] == 0.25).mean() > 0.5  # most of plane 1 lies outside the annulus


def test_imfilter_restatement():
    """Against window sums over a periodically padded copy, odd and even
    kernels, a kernel wider than the image."""
    rng = np.random.default_rng(3)
    for (n1, n2), (m1, m2) in [((20, 17), (5, 5)), ((12, 9), (4, 6)), ((6, 7), (9, 3)), ((8, 8), (1, 1))]:
        Y, h = rng.standard_normal((n1, n2)), rng.standard_normal((m1, m2))
        c1, c2 = (m1 + 1) // 2 - 1, (m2 + 1) // 2 - 1
        want = np.zeros((n1, n2))
        for i in range(n1):
            for j in range(n2):
                for u in range(m1):
                    for v in range(m2):
                        want[i, j] += h[u, v] * Y[(i + u - c1) % n1, (j + v - c2) % n2]
        np.testing.assert_allclose(om.imfilter_circular(Y, h), want, rtol=0, atol=1e-13)


def test_fspecial_gaussian_is_the_fixture_kernel():
    from fd2d_noise_gb300.model_maps import fspecial_gaussian
    for c, shape, s in [("map_ring3", (5, 5), 1.5), ("map_ring_offcentre", (4, 6), 2.0), ("map_ring_single", (3, 3), 1.0)]:
        h = fspecial_gaussian(shape, s)
        np.testing.assert_array_equal(h, GOLD[f"{c}/h"])
        assert abs(h.sum() - 1.0) < 1e-15 and np.array_equal(h, h[::-1, ::-1])


def test_ring_arguments_are_checked():
    from fd2d_noise_gb300 import model_maps as mm
    a, _, _ = _map_case("map_ring3")
    with pytest.raises(ValueError, match="h_structure"):
        mm.map_m_to_parameters(a["m"], a["nx"], a["nz"], a["absbound"], a["x"], a["z"], a["sigma"][0],
                               a["sigma"][1], ring=mm.Ring())
    with pytest.raises(ValueError, match="nx == nz"):
        mm.map_gradparameters_to_gradm(np.zeros((10, 12, 2)), np.pad(np.ones((4, 6)), 3), np.arange(10.0),
                                       np.arange(12.0), (1, 1), (1, 1), ring=mm.Ring(), h_structure=np.ones((1, 1)))


@pytest.mark.gpu
@pytest.mark.parametrize("c", MAP_CASES)
def test_gpu_maps_match_reference(fd2d_lib, c):
    from fd2d_noise_gb300 import model_maps as mm
    a, p, gm = _map_case(c)
    ring = None if a["ring"] is None else mm.Ring(**vars(a["ring"]))
    got_p = mm.map_m_to_parameters(a["m"], a["nx"], a["nz"], a["absbound"], a["x"], a["z"], a["sigma"][0],
                                   a["sigma"][1], 0.25, 1.0, 4.8e10, ring=ring, h_structure=a["h"])
    got_gm = mm.map_gradparameters_to_gradm(a["g"], a["absbound"], a["x"], a["z"], a["sigma"][0], a["sigma"][1],
                                            4.8e10, ring=ring, h_structure=a["h"])
    _close(got_p, p)
    _close(got_gm, gm)
    # bit for bit the oracle: same products, same summation order
    want_p, want_gm = _oracle_maps(a)
    if ring is not None:
        np.testing.assert_array_equal(got_p, want_p)
        np.testing.assert_array_equal(got_gm, want_gm)


@pytest.mark.gpu
def test_gpu_imfilter_matches_oracle(fd2d_lib):
    from fd2d_noise_gb300.model_maps import imfilter_circular
    rng = np.random.default_rng(5)
    for (n1, n2), (m1, m2) in [((300, 260), (40, 40)), ((31, 17), (4, 6)), ((5, 6), (9, 11)), ((64, 64), (1, 1))]:
        Y, h = rng.standard_normal((n1, n2)), rng.standard_normal((m1, m2))
        np.testing.assert_array_equal(imfilter_circular(Y, h), om.imfilter_circular(Y, h))
