"""On-disk formats of code/calculate_data.m:206-223 (array / data MAT files,
Green-spectrum files) and the station loop that fills them."""
import numpy as np
import pytest

from fd2d_noise_gb300 import matio


def test_formats_round_trip(tmp_path):
    array = np.array([[1.0e5, 2.0e5], [1.5e5, 2.5e5], [3.0e5, 1.0e5]])
    ref = array[:2]
    p = matio.save_array(str(tmp_path), array, ref)
    assert p.endswith("array_2_ref.mat")
    a, r = matio.load_array(p)
    np.testing.assert_array_equal(a, array)
    np.testing.assert_array_equal(r, ref)
    c = np.random.default_rng(0).standard_normal((4, 9))
    t = np.linspace(-4, 4, 9)
    p = matio.save_data(str(tmp_path), c, t, 2, 0)
    assert p.endswith("data_2_ref_0.mat")
    c2, t2 = matio.load_data(p)
    np.testing.assert_array_equal(c2, c)
    assert t2.shape == (1, 9)
    G = np.random.default_rng(1).standard_normal((5, 4, 3)) + 1j * np.random.default_rng(2).standard_normal((5, 4, 3))
    for name in ("G_2", "G_fft"):
        p = matio.save_green(str(tmp_path), 2, G, name=name)
        np.testing.assert_array_equal(matio.load_green(p), G)


def test_receivers_exclude_the_source():
    array = np.array([[1.0, 2.0], [3.0, 4.0], [5.0, 6.0]])
    np.testing.assert_array_equal(matio.receivers_of(array, [3.0, 4.0]), array[[0, 2]])


@pytest.mark.gpu
@pytest.mark.parametrize("green_files", [False, True])
def test_calculate_data_stacks_stations(fd2d_lib, tmp_path, green_files):
    from oracle import pyoracle
    from tests.problems import media, noise_source, rel_l2, small_cfg, stations
    cfg = small_cfg(nx=36, nz=30, nt=40, K=10)
    mu, rho = media(cfg, seed=2)
    spec, sd = noise_source(cfg, seed=2)
    array = stations(cfg, 5, seed=4)
    ref = array[:2]
    c_data, t = matio.calculate_data(mu, rho, spec, sd, array, ref, cfg=cfg, out_dir=str(tmp_path),
                                     save_green_spectra=green_files, precision="fp64")
    assert c_data.shape == (2 * 4, cfg.ntc)
    for i in range(2):
        rec = matio.receivers_of(array, ref[i])
        G, _, _ = pyoracle.forward1_green(cfg, mu, rho, ref[i:i + 1], rec, 0)
        c, _ = pyoracle.forward2_correlation(cfg, mu, rho, G, spec, sd, rec, 0)
        assert rel_l2(c_data[i * 4:(i + 1) * 4], c) < 1e-10
    c2, t2 = matio.load_data(str(tmp_path / "data_2_ref_0.mat"))
    np.testing.assert_array_equal(c2, c_data)
    if green_files:
        G2 = matio.load_green(str(tmp_path / "G_2_1.mat"))
        assert G2.shape == (cfg.nx, cfg.nz, cfg.n_sample)
