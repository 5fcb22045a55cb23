"""Generate golden vectors of the reference's noise-source model.

TEST INFRASTRUCTURE.  The unmodified reference sources input/make_noise_source.m,
code/propagation/general_source.m, integration_limits.m and
define_computational_domain.m are executed by the MATLAB-subset interpreter in
mini_matlab.py; the configuration getters input_parameters and
input_interferometry, which the reference hard-codes, are supplied as builtins
returning the cases below.  The 'small' (4e5 m) and 'big' (2e6 m) domains take
the two parameter sets the reference selects by domain size; 'point' indexes
past its one-source arrays and 'picture' reads an image file, so neither runs.
Outputs go to tests/golden/noise_source_cases.npz.

    python tests/golden/make_golden_noise.py <path-to-reference-checkout> (or FD2D_REFERENCE set)
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
from mini_matlab import A, Interpreter, reference_checkout  # noqa: E402

OUT = os.path.join(HERE, "noise_source_cases.npz")

# (name, source type, n_basis_fct, L [m], nx = nz, number of frequencies)
CASES = [
    ("homogeneous", "homogeneous", 0, 4.0e5, 30, 25),
    ("gaussian_small", "gaussian", 0, 4.0e5, 41, 25),
    ("gaussian_big", "gaussian", 0, 2.0e6, 48, 31),
    ("ring_big", "ring", 0, 2.0e6, 64, 31),
    ("gaussian_small_bands", "gaussian", 3, 4.0e5, 41, 25),
    ("ring_big_bands", "ring", 4, 2.0e6, 64, 31),
]


def overrides(L, n, f):
    def input_parameters(*_):
        return [A(L), A(L), A(float(n)), A(float(n)), A(0.1), A(100.0), A(4.0), A(1.0), "homogeneous", A(0.0),
                A(1.0)]

    def input_interferometry(*_):
        ff = f.reshape(1, -1)
        w = 2 * np.pi * ff
        return [ff, A(float(ff.size)), w, A(w[0, 1] - w[0, 0]), A(5.0)]

    return {"input_parameters": input_parameters, "input_interferometry": input_interferometry}


def main():
    ref = reference_checkout(sys.argv)
    paths = [os.path.join(ref, "input"), os.path.join(ref, "code", "propagation"), os.path.join(ref, "code")]
    out = {}
    for name, kind, nb, L, n, K in CASES:
        f = np.linspace(0.01, 0.2, K)
        I = Interpreter(paths, overrides(L, n, f))
        dist, spec = I.call("make_noise_source", [kind, A(float(nb)), "no"], nargout=2)
        out[f"{name}/L"] = np.asarray(L)
        out[f"{name}/n"] = np.asarray(n)
        out[f"{name}/nb"] = np.asarray(nb)
        out[f"{name}/type"] = np.asarray(kind)
        out[f"{name}/f_sample"] = f
        out[f"{name}/dist"] = np.asarray(dist, dtype=np.float64)
        out[f"{name}/spectrum"] = np.asarray(spec, dtype=np.float64)
        print(f"  {name}: dist {np.asarray(dist).shape}, spectrum {np.asarray(spec).shape}", flush=True)
    np.savez_compressed(OUT, **out)
    print(f"wrote {OUT} ({os.path.getsize(OUT) / 1e6:.2f} MB, {len(out)} arrays)")


if __name__ == "__main__":
    main()
