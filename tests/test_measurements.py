"""Misfits and adjoint sources (tools/measurement/make_adjoint_sources.m:31-175,
log_amp_ratio.m:23-93, waveform_difference.m:23-48, cc_time_shift.m:21-61,
amp_diff.m:22-66) against the golden vectors
of the reference's own .m files (tests/golden/measurement_cases.npz): the
numpy oracle on CPU, the library kernel on the GPU."""
import os

import numpy as np
import pytest

from oracle import measurements as om

GOLD = np.load(os.path.join(os.path.dirname(__file__), "golden", "measurement_cases.npz"))
CASES = sorted({k.rsplit("/", 1)[0] for k in GOLD.files if not k.startswith("in/")})


def _inputs(key):
    meas, veldis, order, obs = key.split("/")
    # the time-shift and amplitude measurements use synthetics "us" and
    # shifted, scaled observations "u0s"
    shifted = meas in ("cc_time_shift", "amplitude_difference")
    u = GOLD["in/us"] if shifted else GOLD["in/u"]
    u0 = GOLD["in/u0s"] if shifted else GOLD["in/u0"]
    if obs == "zero":
        u0 = np.zeros_like(u0)
    return u, u0, GOLD["in/du"], GOLD["in/t"].ravel(), veldis, meas, order


def _close(got, want, tol):
    want = np.asarray(want, dtype=np.float64)
    got = np.asarray(got, dtype=np.float64).reshape(want.shape)
    fin = np.isfinite(want)
    assert np.array_equal(fin, np.isfinite(got))
    assert np.array_equal(want[~fin], got[~fin])
    d = np.linalg.norm(got[fin] - want[fin])
    n = np.linalg.norm(want[fin])
    assert d <= tol * max(n, 1e-300), (d, n)


@pytest.mark.parametrize("key", CASES)
def test_oracle_matches_reference(key):
    u, u0, du, t, veldis, meas, order = _inputs(key)
    m, ad = om.make_adjoint_sources(u, u0, du, t, veldis, meas, order)
    _close(ad, GOLD[key + "/adstf"], 1e-13)
    if order == "1st":
        _close(m, GOLD[key + "/misfit"].ravel(), 1e-13)


def test_windows_follow_get_window():
    t = GOLD["in/t"].ravel()
    w = om.get_window(t, 100.0, 200.0, "hann")
    span = np.nonzero((t > 100.0) & (t < 200.0))[0]
    assert np.all(w[: span[0]] == 0) and np.all(w[span[-1] + 1:] == 0)
    np.testing.assert_array_equal(w[span], om.hann(span.size))  # zero at both ends, symmetric
    assert w[span[0]] == 0.0 and w.max() <= 1.0


@pytest.mark.gpu
@pytest.mark.parametrize("key", CASES)
def test_gpu_matches_reference(fd2d_lib, key):
    from fd2d_noise_gb300.measurements import make_adjoint_sources
    u, u0, du, t, veldis, meas, order = _inputs(key)
    m, ad = make_adjoint_sources(u, u0, du, t, veldis, meas, None, None, order)
    # FP64 block reductions sum in another order than MATLAB's sequential sums
    _close(ad, GOLD[key + "/adstf"], 1e-11)
    if order == "1st":
        _close(m, GOLD[key + "/misfit"].ravel(), 1e-11)
