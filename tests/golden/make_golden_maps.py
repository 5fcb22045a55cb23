"""Golden vectors of the reference's gaussblur2d (model and gradient smoothing).

TEST INFRASTRUCTURE.  Runs the unmodified tools/addons/gaussblur2d.m through
the MATLAB-subset interpreter (mini_matlab.py) on seeded maps and writes inputs
and outputs to tests/golden/map_cases.npz.

    python tests/golden/make_golden_maps.py <path-to-reference-checkout> (or FD2D_REFERENCE set)
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
from mini_matlab import A, Interpreter, reference_checkout  # noqa: E402

OUT = os.path.join(HERE, "map_cases.npz")


def run_cases(ref_root):
    I = Interpreter([os.path.join(ref_root, "tools", "addons")])
    rng = np.random.default_rng(21)
    out = {}
    for name, (n1, n2, s1, s2) in {"a": (30, 24, 2.5e3, 4.0e3), "b": (17, 40, 6.0e3, 1.5e3)}.items():
        x1 = np.linspace(0.0, 1.0e3 * (n1 - 1), n1).reshape(1, -1)
        x2 = np.linspace(0.0, 1.2e3 * (n2 - 1), n2).reshape(1, -1)
        Y = np.asfortranarray(rng.standard_normal((n1, n2)))
        sigma = np.array([[s1, s2]])
        (GY,) = I.call("gaussblur2d", [A(Y), A(x1), A(x2), A(sigma)], nargout=1)
        out.update({f"{name}/Y": Y, f"{name}/x1": x1, f"{name}/x2": x2, f"{name}/sigma": sigma,
                    f"{name}/GY": np.asarray(GY)})
        print(" ", name, np.asarray(GY).shape, flush=True)
    np.savez_compressed(OUT, **out)
    print("wrote", OUT, len(out), "arrays")


if __name__ == "__main__":
    run_cases(reference_checkout(sys.argv))
