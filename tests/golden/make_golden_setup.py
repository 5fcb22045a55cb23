"""Generate golden vectors of the reference's grid and absorbing taper.

TEST INFRASTRUCTURE.  The unmodified reference sources
code/propagation/init_absbound.m and define_computational_domain.m are run by
the MATLAB-subset interpreter in mini_matlab.py, with input_parameters and
absorb_specs supplied as builtins returning the cases below (non-square grids,
narrow and wide layers, all four sides or only some).  Outputs go to
tests/golden/setup_cases.npz.

    python tests/golden/make_golden_setup.py <path-to-reference-checkout> (or FD2D_REFERENCE set)
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
from mini_matlab import A, Interpreter, reference_checkout  # noqa: E402

OUT = os.path.join(HERE, "setup_cases.npz")

# (name, Lx, Lz, nx, nz, width [m], left, right, top, bottom)
CASES = [
    ("all_sides", 58.0e3, 42.0e3, 30, 22, 6.0e3, 1, 1, 1, 1),
    ("square_left_bottom", 4.0e5, 4.0e5, 41, 41, 2.0e5, 1, 0, 0, 1),
    ("tall_right_top", 3.0e5, 5.0e5, 25, 37, 5.0e4, 0, 1, 1, 0),
    ("none", 1.0e5, 1.0e5, 12, 15, 1.0e4, 0, 0, 0, 0),
]


def main():
    ref = reference_checkout(sys.argv)
    paths = [os.path.join(ref, "code", "propagation")]
    out = {}
    for name, Lx, Lz, nx, nz, w, l, r, t, b in CASES:
        ov = {
            "input_parameters": lambda *_, Lx=Lx, Lz=Lz, nx=nx, nz=nz: [A(Lx), A(Lz), A(float(nx)), A(float(nz))],
            "absorb_specs": lambda *_, w=w, l=l, r=r, t=t, b=b: [A(w), A(float(l)), A(float(r)), A(float(t)),
                                                                  A(float(b))],
        }
        I = Interpreter(paths, ov)
        ab = I.call("init_absbound", [], nargout=1)[0]
        X, Z, x, z, dx, dz = I.call("define_computational_domain", [A(Lx), A(Lz), A(float(nx)), A(float(nz))],
                                    nargout=6)
        for k, v in dict(Lx=Lx, Lz=Lz, nx=nx, nz=nz, width=w, flags=np.array([l, r, t, b], dtype=np.float64),
                         absbound=ab, x=x, z=z, dx=dx, dz=dz).items():
            out[f"{name}/{k}"] = np.asarray(v, dtype=np.float64)
        print(f"  {name}: absbound {np.asarray(ab).shape}, min {np.asarray(ab).min():.3g}", flush=True)
    np.savez_compressed(OUT, **out)
    print(f"wrote {OUT} ({os.path.getsize(OUT) / 1e6:.3f} MB, {len(out)} arrays)")


if __name__ == "__main__":
    main()
