"""Golden vectors of the reference's measurement code (adjoint sources).

TEST INFRASTRUCTURE.  Runs the unmodified reference sources
tools/measurement/make_adjoint_sources.m, log_amp_ratio.m,
waveform_difference.m and addons/get_window.m through the MATLAB-subset
interpreter (mini_matlab.py) on seeded synthetic correlations and writes inputs
and outputs to tests/golden/measurement_cases.npz.  MATLAB's closed built-ins
used there (hann, trapz) are restated in mini_matlab.py from their documented
definitions.

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
    np.savez_compressed(OUT, **out)
    print("wrote", OUT, len(out), "arrays")


if __name__ == "__main__":
    run_cases(reference_checkout(sys.argv))
