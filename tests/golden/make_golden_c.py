"""Generate golden vectors of a third solver case (C).

TEST INFRASTRUCTURE, as make_golden.py: the unmodified reference solvers run
by the MATLAB-subset interpreter, with the configuration getters supplied as
builtins.  Case C exercises what cases A and B do not: a non-square grid with
absorbing layers on two sides only (left and top), snapshots and DFT samples
every 3 steps, and two point sources in the Green run; then the correlation
run and the adjoint runs of the gradient chain.  (Several noise sources are
not a case: with n_basis_fct == 0 the reference forms the per-frequency
distribution as ones(n_sample,1) times the source maps, which only conforms
for one source.)  Outputs go to tests/golden/reference_cases_c.npz.

    python tests/golden/make_golden_c.py <path-to-reference-checkout> (or FD2D_REFERENCE set)
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
from make_golden import E, S, config, inputs, overrides  # noqa: E402
from mini_matlab import A, Interpreter, reference_checkout  # noqa: E402

OUT = os.path.join(HERE, "reference_cases_c.npz")
SIDES = (1.0, 0.0, 1.0, 0.0)  # absorb_left, absorb_right, absorb_top, absorb_bottom


def main():
    ref = reference_checkout(sys.argv)
    paths = [os.path.join(ref, "code"), os.path.join(ref, "code", "propagation")]
    c = config(nx=21, nz=15, nt=36, order=4, K=9, fs=3, fw=3, nb=0, width_pts=3)
    ov = overrides(c)
    ov["absorb_specs"] = lambda *_: [A(c["width"]), *[A(v) for v in SIDES]]
    I = Interpreter(paths, ov)
    inp = inputs(c, 3)
    rng = np.random.default_rng(9)
    Lx, Lz = c["Lx"], c["Lz"]
    inp["src"] = np.array([[0.4 * Lx, 0.5 * Lz], [0.62 * Lx, 0.41 * Lz]])
    out = {f"C/cfg/{k}": np.asarray(v) for k, v in c.items()}
    out["C/cfg/sides"] = np.asarray(SIDES)
    out.update({f"C/in/{k}": np.asarray(v) for k, v in inp.items()})
    G, Gout, s = I.call("run_forward1_green", [A(inp["mu"]), A(inp["rho"]), A(inp["src"]), A(inp["rec"]), A(1.0),
                                               E(), S()], nargout=3)
    out.update({"C/fwd1/G": G, "C/fwd1/G_out": Gout, "C/fwd1/seis": s})
    cs, C = I.call("run_forward2_correlation", [A(inp["mu"]), A(inp["rho"]), G, A(inp["spec"]), A(inp["sd"]),
                                                A(inp["rec"]), A(1.0), E(), S()], nargout=2)
    out.update({"C/corr/seis": cs, "C/corr/C_out": C})
    ntc = 2 * c["nt"] - 1
    adstf = (rng.standard_normal((inp["rec"].shape[0], ntc)) * 1e-3).astype(complex)
    out["C/in2/adstf"] = adstf
    rec = A(inp["rec"])
    K1, sf1, _, s1 = I.call("run_noise_adjoint", [A(inp["mu"]), A(inp["rho"]), C, A(adstf), rec, rec,
                                                  A(inp["spec"]), E(), G, A(1.0), E(), S()], nargout=4)
    out.update({"C/adj1/K": K1, "C/adj1/stf_fft": sf1, "C/adj1/seis": s1})
    K2, _, _, s2 = I.call("run_noise_adjoint", [A(inp["mu"]), A(inp["rho"]), Gout, sf1, rec, rec,
                                                A(inp["spec"]), A(inp["sd"]), E(), A(0.0), E(), S()], nargout=4)
    out.update({"C/adj0/K": K2, "C/adj0/seis": s2})
    np.savez_compressed(OUT, **{k: np.asarray(v) for k, v in out.items()})
    print(f"wrote {OUT} ({os.path.getsize(OUT) / 1e3:.1f} kB, {len(out)} arrays)")


if __name__ == "__main__":
    main()
