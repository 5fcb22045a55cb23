"""Golden vectors of the reference's model-space maps.

TEST INFRASTRUCTURE.  Runs the unmodified tools/addons/gaussblur2d.m and
inversion/optlib_callback_fct/map_m_to_parameters.m and
map_gradparameters_to_gradm.m (with code/propagation/
define_computational_domain.m) through the MATLAB-subset interpreter
(mini_matlab.py) on seeded maps, in the Gaussian-smoothing branch and the
'ring' branch, and writes inputs and outputs to tests/golden/map_cases.npz.
The reference reads the domain (input_parameters) and the taper
(init_absbound) from its input files; here they are given by the case.
imfilter (MATLAB Image Processing Toolbox, not part of the reference) is
supplied from its documented definition: correlation, output the size of the
input, periodic extension, the kernel's centre at floor((size(h)+1)/2).

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
    out.update(run_map_cases(ref_root, rng))
    np.savez_compressed(OUT, **out)
    print("wrote", OUT, len(out), "arrays")


def imfilter_circular(Y, h):
    """Window sums over a periodically padded copy of Y."""
    Y, h = np.asarray(Y, dtype=np.float64), np.asarray(h, dtype=np.float64)
    m1, m2 = h.shape
    c1, c2 = (m1 + 1) // 2 - 1, (m2 + 1) // 2 - 1
    P = np.pad(Y, ((c1, m1 - 1 - c1), (c2, m2 - 1 - c2)), mode="wrap")
    win = np.lib.stride_tricks.sliding_window_view(P, (m1, m2))
    return np.asfortranarray(np.einsum("ijuv,uv->ij", win, h))


def gaussian_kernel(m1, m2, s):
    """fspecial('gaussian', [m1 m2], s): documented construction."""
    y, x = np.meshgrid(np.arange(m1) - (m1 - 1) / 2, np.arange(m2) - (m2 - 1) / 2, indexing="ij")
    h = np.exp(-(x * x + y * y) / (2 * s * s))
    h[h < np.finfo(float).eps * h.max()] = 0
    return h / h.sum()


MAP_CASES = {
    # name: nx, nz, Lx, Lz, taper width, planes, ring (x_c, z_c, radius, thickness, taper_strength) or None, h
    "smooth3": (36, 30, 6.0e4, 5.0e4, 4, 3, None, None),
    "ring3": (40, 40, 2.0e6, 2.0e6, 5, 3, (1.0e6, 1.0e6, 6.4e5, 2.0e5, 70e8), (5, 5, 1.5)),
    "ring_offcentre": (38, 38, 2.0e6, 1.6e6, 4, 2, (0.9e6, 0.7e6, 5.0e5, 3.0e5, 30e8), (4, 6, 2.0)),
    "ring_single": (30, 30, 1.0e6, 1.0e6, 3, 1, (0.5e6, 0.45e6, 3.0e5, 2.0e5, 20e8), (3, 3, 1.0)),
}


def run_map_cases(ref_root, rng):
    out = {}
    paths = [os.path.join(ref_root, "inversion", "optlib_callback_fct"), os.path.join(ref_root, "code", "propagation"),
             os.path.join(ref_root, "tools", "addons")]
    for name, (nx, nz, Lx, Lz, w, planes, ring, hk) in MAP_CASES.items():
        ab = np.zeros((nx, nz))
        ab[w:nx - w, w:nz - w] = 1.0
        ab[w - 1, w - 1:nz - w + 1] = 0.5  # a partial taper row before the interior
        h = gaussian_kernel(*hk) if hk else None
        ov = {"init_absbound": lambda: [np.asfortranarray(ab)],
              "input_parameters": lambda: [A(Lx), A(Lz), A(float(nx)), A(float(nz))],
              "imfilter": lambda Y, hh, mode: [imfilter_circular(Y, hh)]}
        I = Interpreter(paths, ov)
        usr = {"config": {"nx": A(float(nx)), "nz": A(float(nz))},
               "kernel": {"sigma": {"source": np.array([[3.0e3, 2.0e3]]) * Lx / 6.0e4,
                                    "structure": np.array([[2.0e3, 4.0e3]]) * Lx / 6.0e4}},
               "initial": {"ref_source": A(0.25), "ref_structure": A(1.0), "mu_0": A(4.8e10)},
               "ring": {"switch": "no"}}
        if ring:
            usr["ring"] = {"switch": "yes", "x_center_ring": A(ring[0]), "z_center_ring": A(ring[1]),
                           "radius": A(ring[2]), "thickness": A(ring[3]), "taper_strength": A(ring[4])}
            usr["kernel"]["imfilter"] = {"structure": np.asfortranarray(h)}
        m = np.asfortranarray(rng.standard_normal((nx * nz * planes, 1)) * 0.05)
        g = np.asfortranarray(rng.standard_normal((nx, nz, planes)))
        (p,) = I.call("map_m_to_parameters", [m, usr], nargout=1)
        (gm,) = I.call("map_gradparameters_to_gradm", [m, g, usr], nargout=1)
        out.update({f"map_{name}/m": m.ravel(), f"map_{name}/g": g, f"map_{name}/absbound": ab,
                    f"map_{name}/shape": np.array([nx, nz, Lx, Lz]),
                    f"map_{name}/sigma": np.vstack([usr["kernel"]["sigma"]["source"],
                                                   usr["kernel"]["sigma"]["structure"]]),
                    f"map_{name}/p": np.asarray(p).reshape(nx, nz, planes, order="F"),
                    f"map_{name}/gm": np.asarray(gm).ravel()})
        if ring:
            out[f"map_{name}/ring"] = np.array(ring)
            out[f"map_{name}/h"] = h
        print(" ", name, np.asarray(p).shape, flush=True)
    return out


if __name__ == "__main__":
    run_cases(reference_checkout(sys.argv))
