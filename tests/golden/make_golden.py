"""Generate golden vectors by running the reference's own MATLAB solvers.

TEST INFRASTRUCTURE.  MATLAB is not available, so the unmodified reference
sources code/run_forward1_green.m, code/run_forward2_correlation.m,
code/run_noise_adjoint.m and code/propagation/*.m are executed by the
MATLAB-subset interpreter in mini_matlab.py.  The three configuration getters
(input_parameters, input_interferometry, absorb_specs), which the reference
hard-codes, are supplied as builtins returning the small test configurations
below.  Inputs are seeded; inputs and outputs are written to
tests/golden/reference_cases.npz, which the oracle and GPU tests compare
against.

    python tests/golden/make_golden.py <path-to-reference-checkout> (or FD2D_REFERENCE set)
"""
from __future__ import annotations

import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
from mini_matlab import A, Interpreter, reference_checkout  # noqa: E402

OUT = os.path.join(HERE, "reference_cases.npz")


def config(nx=18, nz=16, nt=40, order=4, K=10, fs=5, fw=1, nb=0, width_pts=3):
    Lx = 1.0e3 * (nx - 1) * 2.0
    Lz = 1.0e3 * (nz - 1) * 2.0
    dx = Lx / (nx - 1)
    dt = 0.45 * dx / 4200.0
    f = 0.02 + 0.0075 * np.arange(K)
    return dict(Lx=Lx, Lz=Lz, nx=nx, nz=nz, dt=dt, nt=nt, order=order, K=K, fs=fs, fw=fw, nb=nb,
                f_sample=f, width=width_pts * dx)


def overrides(c):
    def input_parameters(*_):
        return [A(c["Lx"]), A(c["Lz"]), A(float(c["nx"])), A(float(c["nz"])), A(c["dt"]),
                A(float(c["nt"])), A(float(c["order"])), A(1.0), "homogeneous", A(float(c["nb"])),
                A(float(c["fw"]))]

    def input_interferometry(*_):
        f = c["f_sample"].reshape(1, -1)
        w = 2 * np.pi * f
        return [f, A(float(f.size)), w, A(w[0, 1] - w[0, 0]), A(float(c["fs"]))]

    def absorb_specs(*_):
        return [A(c["width"]), A(1.0), A(1.0), A(1.0), A(1.0)]

    return {"input_parameters": input_parameters, "input_interferometry": input_interferometry,
            "absorb_specs": absorb_specs}


def inputs(c, seed):
    rng = np.random.default_rng(seed)
    nx, nz = c["nx"], c["nz"]
    p = rng.standard_normal((nx, nz))
    for _ in range(2):
        p = 0.25 * (np.roll(p, 1, 0) + np.roll(p, -1, 0) + np.roll(p, 1, 1) + np.roll(p, -1, 1))
    p /= np.abs(p).max()
    mu = np.asfortranarray(4.8e10 * (1 + 0.05 * p))
    rho = np.asfortranarray(3000.0 * (1 + 0.02 * np.roll(p, 3, 0)))
    Lx, Lz = c["Lx"], c["Lz"]
    src = np.array([[0.45 * Lx + 0.1 * Lx * rng.random(), 0.5 * Lz + 0.05 * Lz * rng.random()]])
    rec = np.stack([Lx * (0.25 + 0.5 * rng.random(3)), Lz * (0.25 + 0.5 * rng.random(3))], axis=1)
    f = c["f_sample"]
    planes = max(c["nb"], 1)
    x = np.linspace(0, Lx, nx)[:, None]
    z = np.linspace(0, Lz, nz)[None, :]
    sd = np.zeros((nx, nz, planes), order="F")
    for b in range(planes):
        cx, cz = Lx * rng.uniform(0.3, 0.7), Lz * rng.uniform(0.3, 0.7)
        sd[:, :, b] = 1 + 6.0 * np.exp(-((x - cx) ** 2 + (z - cz) ** 2) / (0.3 * Lx) ** 2)
    spec = np.exp(-(np.abs(f) - 0.05) ** 2 / 0.04 ** 2).reshape(-1, 1) if c["nb"] == 0 else np.ones((f.size, 1))
    dmu = np.asfortranarray(0.02 * mu * rng.standard_normal((nx, nz)))
    return dict(mu=mu, rho=rho, src=src, rec=rec, sd=np.asfortranarray(sd), spec=spec, dmu=dmu)


def E():
    return np.zeros((0, 0))


def S():
    return np.zeros((0, 0), dtype=np.float32)


def run_cases(ref_root):
    paths = [os.path.join(ref_root, "code"), os.path.join(ref_root, "code", "propagation")]
    out = {}

    def save(prefix, d):
        for k, v in d.items():
            out[f"{prefix}/{k}"] = np.asarray(v)

    def solver(c):
        return Interpreter(paths, overrides(c))

    # ---- case A: order 4, fw 1, the Green/correlation/adjoint chains --------------
    c = config()
    inp = inputs(c, 1)
    I = solver(c)
    save("A/cfg", {k: (np.asarray(v) if not isinstance(v, (int, float)) else np.asarray(v)) for k, v in c.items()})
    save("A/in", inp)
    t0 = time.time()
    G, Gout, s = I.call("run_forward1_green", [A(inp["mu"]), A(inp["rho"]), A(inp["src"]), A(inp["rec"]), A(1.0),
                                               E(), S()], nargout=3)
    save("A/fwd1", dict(G=G, G_out=Gout, seis=s))
    dG, dGout, ds = I.call("run_forward1_green", [A(inp["mu"]), A(inp["rho"]), A(inp["src"]), A(inp["rec"]),
                                                  A(5.0), A(inp["dmu"]), Gout], nargout=3)
    save("A/fwd1_born", dict(G=dG, G_out=dGout, seis=ds))
    print(f"  forward1 done ({time.time() - t0:.1f} s)", flush=True)
    cs, C = I.call("run_forward2_correlation", [A(inp["mu"]), A(inp["rho"]), G, A(inp["spec"]), A(inp["sd"]),
                                                A(inp["rec"]), A(1.0), E(), S()], nargout=2)
    save("A/corr", dict(seis=cs, C_out=C))
    cb, dC = I.call("run_forward2_correlation", [A(inp["mu"]), A(inp["rho"]), G, A(inp["spec"]), A(inp["sd"]),
                                                 A(inp["rec"]), A(1.0), A(inp["dmu"]), C], nargout=2)
    save("A/corr_born", dict(seis=cb, C_out=dC))
    print(f"  correlation done ({time.time() - t0:.1f} s)", flush=True)
    rng = np.random.default_rng(7)
    ntc = 2 * c["nt"] - 1
    adstf = (rng.standard_normal((inp["rec"].shape[0], ntc)) * 1e-3).astype(complex)
    save("A/in2", dict(adstf=adstf))
    rec = A(inp["rec"])
    # eval_objective_and_gradient 'joint' chain
    K1, sf1, _, s1 = I.call("run_noise_adjoint", [A(inp["mu"]), A(inp["rho"]), C, A(adstf), rec, rec,
                                                  A(inp["spec"]), E(), G, A(1.0), E(), S()], nargout=4)
    save("A/adj1", dict(K=K1, stf_fft=sf1, seis=s1))
    K2, _, _, s2 = I.call("run_noise_adjoint", [A(inp["mu"]), A(inp["rho"]), Gout, sf1, rec, rec,
                                                A(inp["spec"]), A(inp["sd"]), E(), A(0.0), E(), S()], nargout=4)
    save("A/adj0", dict(K=K2, seis=s2))
    print(f"  adjoint (gradient) done ({time.time() - t0:.1f} s)", flush=True)
    # eval_hessian_vector_product chain: modes 13, 11, 12 (Born), 10 (Born)
    K13, uT, udag, s13 = I.call("run_noise_adjoint", [A(inp["mu"]), A(inp["rho"]), C, A(adstf), rec, rec,
                                                      A(inp["spec"]), E(), G, A(13.0), E(), S()], nargout=4)
    save("A/adj13", dict(K=K13, stf_fft=uT, u_out=udag, seis=s13))
    K11, _, p, s11 = I.call("run_noise_adjoint", [A(inp["mu"]), A(inp["rho"]), Gout, uT, rec, rec,
                                                  A(inp["spec"]), A(inp["sd"]), E(), A(11.0), E(), S()], nargout=4)
    save("A/adj11", dict(K=K11, u_out=p, seis=s11))
    K12, kT, _, s12 = I.call("run_noise_adjoint", [A(inp["mu"]), A(inp["rho"]), C, A(adstf), rec, rec,
                                                   A(inp["spec"]), E(), G, A(12.0), A(inp["dmu"]), udag], nargout=4)
    save("A/adj12", dict(K=K12, stf_fft=kT, seis=s12))
    K10, _, _, s10 = I.call("run_noise_adjoint", [A(inp["mu"]), A(inp["rho"]), Gout, kT, rec, rec,
                                                  A(inp["spec"]), A(inp["sd"]), E(), A(10.0), A(inp["dmu"]), p],
                            nargout=4)
    save("A/adj10", dict(K=K10, seis=s10))
    print(f"  adjoint (Hessian) done ({time.time() - t0:.1f} s)", flush=True)

    # ---- case B: order 2, fw 2, three frequency bands -----------------------------------
    c = config(nx=15, nz=17, nt=30, order=2, K=12, fs=4, fw=2, nb=3)
    inp = inputs(c, 2)
    I = solver(c)
    save("B/cfg", {k: np.asarray(v) for k, v in c.items()})
    save("B/in", inp)
    G, Gout, s = I.call("run_forward1_green", [A(inp["mu"]), A(inp["rho"]), A(inp["src"]), A(inp["rec"]), A(1.0),
                                               E(), S()], nargout=3)
    save("B/fwd1", dict(G=G, G_out=Gout, seis=s))
    cs, C = I.call("run_forward2_correlation", [A(inp["mu"]), A(inp["rho"]), G, A(inp["spec"]), A(inp["sd"]),
                                                A(inp["rec"]), A(1.0), E(), S()], nargout=2)
    save("B/corr", dict(seis=cs, C_out=C))
    ntc = 2 * c["nt"] - 1
    adstf = (np.random.default_rng(8).standard_normal((inp["rec"].shape[0], ntc)) * 1e-3).astype(complex)
    save("B/in2", dict(adstf=adstf))
    rec = A(inp["rec"])
    K1, sf1, _, s1 = I.call("run_noise_adjoint", [A(inp["mu"]), A(inp["rho"]), C, A(adstf), rec, rec,
                                                  A(inp["spec"]), E(), G, A(1.0), E(), S()], nargout=4)
    save("B/adj1", dict(K=K1, stf_fft=sf1, seis=s1))
    print(f"  case B done ({time.time() - t0:.1f} s)", flush=True)
    return out


def main():
    ref = reference_checkout(sys.argv)
    out = run_cases(ref)
    np.savez_compressed(OUT, **out)
    print(f"wrote {OUT} ({os.path.getsize(OUT) / 1e6:.2f} MB, {len(out)} arrays)")


if __name__ == "__main__":
    main()
