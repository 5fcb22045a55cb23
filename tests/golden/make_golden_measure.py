"""Golden vectors of the reference's measurement code (adjoint sources).

TEST INFRASTRUCTURE.  Runs the unmodified reference sources
tools/measurement/make_adjoint_sources.m, log_amp_ratio.m,
waveform_difference.m, cc_time_shift.m, amp_diff.m, addons/get_window.m,
addons/cross_correlation_td.m and tools/addons/swap.m through the MATLAB-subset
interpreter (mini_matlab.py) on seeded synthetic correlations and writes inputs
and outputs to tests/golden/measurement_cases.npz.  MATLAB's closed built-ins
used there (hann, trapz, xcorr) are restated in mini_matlab.py from their
documented definitions.

    python tests/golden/make_golden_measure.py <path-to-reference-checkout> (or FD2D_REFERENCE set)
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
from mini_matlab import A, Interpreter, reference_checkout  # noqa: E402

OUT = os.path.join(HERE, "measurement_cases.npz")


def traces(rng, n_rec, t):
    """Correlation-like traces: a causal and an acausal wave packet per receiver."""
    u = np.zeros((n_rec, t.size))
    for r in range(n_rec):
        for sgn in (1.0, -1.0):
            t0 = sgn * rng.uniform(120.0, 180.0)
            amp = rng.uniform(0.5, 2.0)
            u[r] += amp * np.exp(-((t - t0) / 12.0) ** 2) * np.cos(2 * np.pi * 0.05 * (t - t0))
        u[r] += 0.01 * rng.standard_normal(t.size)
    return np.asfortranarray(u)


def run_cases(ref_root):
    paths = [os.path.join(ref_root, "tools", "measurement"),
             os.path.join(ref_root, "tools", "measurement", "addons"),
             os.path.join(ref_root, "tools", "addons")]
    I = Interpreter(paths)
    rng = np.random.default_rng(11)
    out = {}
    dt = 0.5
    nt = 801
    t = (-(nt - 1) // 2 + np.arange(nt)) * dt  # -200 .. 200 s, symmetric
    t = t.reshape(1, -1)
    n_rec = 3
    u = traces(rng, n_rec, t[0])
    u0 = traces(rng, n_rec, t[0])
    du = np.asfortranarray(0.1 * traces(rng, n_rec, t[0]))
    out["in/t"], out["in/u"], out["in/u0"], out["in/du"] = t, u, u0, du
    src = np.array([[1.0e5, 1.0e5]])
    rec = np.array([[2.0e5, 1.0e5], [1.0e5, 2.0e5], [2.0e5, 2.0e5]])
    for meas in ("log_amplitude_ratio", "waveform_difference"):
        for veldis in ("dis", "vel"):
            for order in ("1st", "2nd"):
                for zero_obs in (False, True):
                    if zero_obs and (order == "2nd" or meas == "waveform_difference"):
                        continue
                    obs = np.zeros_like(u0) if zero_obs else u0
                    m, ad = I.call("make_adjoint_sources",
                                   [A(u), A(obs), A(du), A(t), veldis, meas, A(src), A(rec), order], nargout=2)
                    key = f"{meas}/{veldis}/{order}/{'zero' if zero_obs else 'obs'}"
                    out[key + "/misfit"] = np.asarray(m)
                    out[key + "/adstf"] = np.asarray(ad)
                    print("  ", key, flush=True)
    # cc_time_shift and amplitude_difference: observations that are the
    # synthetics shifted by 0.8-2.5 s (inside the 3.5 s the time-shift
    # measurement accepts) and scaled, plus noise
    rng2 = np.random.default_rng(12)
    us = np.zeros((n_rec, nt))
    u0s = np.zeros((n_rec, nt))
    for r in range(n_rec):
        for sgn in (1.0, -1.0):
            t0 = sgn * rng2.uniform(120.0, 180.0)
            amp = rng2.uniform(0.5, 2.0)
            shift, scale = rng2.uniform(0.8, 2.5), rng2.uniform(0.8, 1.25)
            us[r] += amp * np.exp(-((t[0] - t0) / 12.0) ** 2) * np.cos(2 * np.pi * 0.05 * (t[0] - t0))
            t1 = t0 + sgn * shift
            u0s[r] += scale * amp * np.exp(-((t[0] - t1) / 12.0) ** 2) * np.cos(2 * np.pi * 0.05 * (t[0] - t1))
        u0s[r] += 0.01 * rng2.standard_normal(nt)
    us, u0s = np.asfortranarray(us), np.asfortranarray(u0s)
    out["in/us"], out["in/u0s"] = us, u0s
    for meas in ("cc_time_shift", "amplitude_difference"):
        for veldis in ("dis", "vel"):
            for order in ("1st", "2nd"):
                for zero_obs in (False, True):
                    if order == "2nd" and (zero_obs or meas == "cc_time_shift"):
                        continue
                    obs = np.zeros_like(u0s) if zero_obs else u0s
                    m, ad = I.call("make_adjoint_sources",
                                   [A(us), A(obs), A(du), A(t), veldis, meas, A(src), A(rec), order], nargout=2)
                    key = f"{meas}/{veldis}/{order}/{'zero' if zero_obs else 'shift'}"
                    out[key + "/misfit"] = np.asarray(m)
                    out[key + "/adstf"] = np.asarray(ad)
                    print("  ", key, flush=True)
    np.savez_compressed(OUT, **out)
    print("wrote", OUT, len(out), "arrays")


if __name__ == "__main__":
    run_cases(reference_checkout(sys.argv))
