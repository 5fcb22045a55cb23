"""Generate golden vectors of the reference's misfit/gradient orchestration.

TEST INFRASTRUCTURE.  The unmodified
inversion/optlib_callback_fct/eval_objective_and_gradient.m and the
measurement code it calls (tools/measurement/make_adjoint_sources.m and its
helpers) are run by the MATLAB-subset interpreter in mini_matlab.py.  Only
the solver part is kept, as fd2d_noise_gb300.objective restates it: the three
solvers it calls (run_*_mex) are answered by the FP64 oracle (itself pinned
to the reference solvers by make_golden.py); the model map, the gradient map
and the regularisation are identities; the configuration getters, the noise
spectrum and the density return the test problem; G_fft files are never
found, so every station computes its Green function.  Cases: the 'source',
'structure' and 'joint' inversion types with two reference stations, a
waveform-difference source measurement and a log-amplitude-ratio structure
measurement mixed by the weighting; and eval_hessian_vector_product.m for the
'structure' and 'joint' types (its model-space regularisation term set to
zero, its Hessian map an identity) and eval_hessian_vector_product_source.m
for the 'source' type.  Outputs go to
tests/golden/objective_cases.npz.

    python tests/golden/make_golden_objective.py <path-to-reference-checkout> (or FD2D_REFERENCE set)
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, HERE)
sys.path.insert(0, ROOT)
from mini_matlab import A, Interpreter, reference_checkout  # noqa: E402

OUT = os.path.join(HERE, "objective_cases.npz")
TYPES = ("source", "structure", "joint")
WEIGHTING = 0.3


def problem():
    """The structure-kernel test problem of tests/test_objective.py with two reference stations."""
    from tests.test_objective import cfg4, problem as p4
    cfg = cfg4()
    p = p4(cfg)
    p["ref"] = p["arr"][:2].copy()
    return cfg, p


def main():
    from oracle import pyoracle
    pyoracle.build()
    ref = reference_checkout(sys.argv)
    cfg, p = problem()
    paths = [os.path.join(ref, "inversion", "optlib_callback_fct"), os.path.join(ref, "tools", "measurement"),
             os.path.join(ref, "tools", "measurement", "addons"), os.path.join(ref, "tools", "addons")]

    def arr(x):
        return None if (x is None or isinstance(x, str) or np.asarray(x).size == 0) else np.asarray(x)

    def pts(x):
        return np.zeros((0, 2)) if arr(x) is None else np.asarray(x, dtype=np.float64).reshape(-1, 2)

    def empty_single():
        return np.zeros((0, 0), dtype=np.float32)

    def fwd1(mu, rho, src, rec, mode, dmu, G_in):
        G, Gout, seis = pyoracle.forward1_green(cfg, arr(mu), arr(rho), pts(src), pts(rec), int(np.ravel(mode)[0]),
                                                arr(dmu), arr(G_in))
        return [np.asfortranarray(G), Gout if Gout is not None else empty_single(), np.asfortranarray(seis)]

    def corr(mu, rho, G, spec, sd, rec, mode, dmu, C_in):
        seis, C = pyoracle.forward2_correlation(cfg, arr(mu), arr(rho), arr(G), arr(spec), arr(sd), pts(rec),
                                                int(np.ravel(mode)[0]), arr(dmu), arr(C_in))
        return [np.asfortranarray(seis), C if C is not None else empty_single()]

    def adj(mu, rho, u_fwd, stf, src, rec, spec, sd, G, mode, dmu, u_in):
        K, sf, u_out, seis = pyoracle.noise_adjoint(cfg, arr(mu), arr(rho), arr(u_fwd), arr(stf), pts(src), pts(rec),
                                                    arr(spec), arr(sd), arr(G), int(np.ravel(mode)[0]), arr(dmu),
                                                    arr(u_in))
        return [np.asfortranarray(K), np.asfortranarray(sf), u_out if u_out is not None else empty_single(),
                np.asfortranarray(seis)]

    def input_parameters(*_):
        return [A(cfg.Lx), A(cfg.Lz), A(float(cfg.nx)), A(float(cfg.nz)), A(cfg.dt), A(float(cfg.nt)),
                A(float(cfg.order)), A(1.0), "homogeneous", A(float(cfg.n_basis_fct)), A(float(cfg.fw_nth))]

    ov = {"run_forward1_green_mex": fwd1, "run_forward2_correlation_mex": corr, "run_noise_adjoint_mex": adj,
          "input_parameters": input_parameters,
          "map_m_to_parameters": lambda m, *_: [m],
          "map_gradparameters_to_gradm": lambda m, g, *_: [g],
          "regularization": lambda j, g, *_: [j, g],
          "make_noise_source": lambda *_: [A(0.0), np.asfortranarray(p["spec"])],
          "define_material_parameters": lambda *_: [np.asfortranarray(p["mu0"]), np.asfortranarray(p["rho"])],
          "exist": lambda *_: A(0.0), "parsave": lambda *_: [], "parload": lambda *_: [A(0.0)]}
    # synthetic data: the correlations of the true model, station after station
    c_data = []
    for i in range(p["ref"].shape[0]):
        src = p["ref"][i:i + 1]
        rec = p["arr"][~np.all(p["arr"] == src, axis=1)]
        G, _, _ = pyoracle.forward1_green(cfg, p["mu_true"], p["rho"], src, rec, 0)
        c, _ = pyoracle.forward2_correlation(cfg, p["mu_true"], p["rho"], G, p["spec"], p["sd"], rec, 0)
        c_data.append(c)
    c_data = np.asfortranarray(np.concatenate(c_data, axis=0))
    m = np.asfortranarray(np.concatenate([p["sd"], p["mu0"][:, :, None]], axis=2))
    out = {"c_data": c_data, "ref_stat": p["ref"], "array": p["arr"], "t": p["t"], "weighting": np.asarray(WEIGHTING)}
    for typ in TYPES:
        usr_par = {"config": {"nx": A(float(cfg.nx)), "nz": A(float(cfg.nz))},
                   "data": {"t": np.asfortranarray(p["t"].reshape(1, -1)), "c_data": c_data},
                   "network": {"ref_stat": np.asfortranarray(p["ref"]), "array": np.asfortranarray(p["arr"])},
                   "type": typ, "filter": {"apply_filter": "no"}, "veldis": "dis",
                   "measurement": {"source": "waveform_difference", "structure": "log_amplitude_ratio"},
                   "kernel": {"weighting": A(WEIGHTING)}}
        I = Interpreter(paths, ov)
        j, g, c_all = I.call("eval_objective_and_gradient", [m, "abcdefgh", usr_par], nargout=3)
        out[f"{typ}/j"] = np.asarray(j, dtype=np.float64).ravel()
        out[f"{typ}/g"] = np.asarray(g, dtype=np.float64)
        out[f"{typ}/c_all"] = np.asarray(c_all, dtype=np.float64)
        print(f"  {typ}: j = {float(np.ravel(j)[0]):.10g}, |g| = {np.linalg.norm(g):.4g}", flush=True)
    # Hessian-vector products (stored fields every step: fw_nth = 1), regularisation weights zero
    from tests.test_objective import cfg4
    cfg = cfg4(fw=1)
    hpaths = paths + [os.path.join(ref, "code", "propagation")]
    ds = np.asfortranarray(0.1 * p["sd"])
    out["hvp/ds"] = ds
    out["hvp/dmu"] = np.asfortranarray(p["dmu"])
    for typ in ("structure", "joint"):
        dm = np.asfortranarray(np.concatenate([ds if typ == "joint" else 0 * ds, p["dmu"][:, :, None]], axis=2))
        usr_par = {"config": {"nx": A(float(cfg.nx)), "nz": A(float(cfg.nz))},
                   "data": {"t": np.asfortranarray(p["t"].reshape(1, -1)), "c_data": c_data},
                   "network": {"ref_stat": np.asfortranarray(p["ref"]), "array": np.asfortranarray(p["arr"])},
                   "type": typ, "veldis": "dis", "verbose": "no",
                   "measurement": {"source": "waveform_difference", "structure": "log_amplitude_ratio"},
                   "kernel": {"weighting": A(WEIGHTING)},
                   "regularization": {"alpha": A(0.0), "beta": A(0.0), "weighting": A(1.0)}}
        hov = dict(ov)
        hov["map_Hparameters_to_Hm"] = lambda H, *_: [np.asfortranarray(np.asarray(H).reshape(-1, 1, order="F"))]
        hov["absorb_specs"] = lambda *_: [A(cfg.absorb_width), A(1.0), A(1.0), A(1.0), A(1.0)]
        I = Interpreter(hpaths, hov)
        Hm = I.call("eval_hessian_vector_product", [m, dm, "abcdefgh", usr_par], nargout=1)[0]
        out[f"hvp/{typ}/H"] = np.asarray(Hm, dtype=np.float64).reshape(m.shape, order="F")
        print(f"  hvp {typ}: |H| = {np.linalg.norm(Hm):.4g}", flush=True)
    # eval_hessian_vector_product_source.m: a perturbation of the noise
    # distribution (the mu plane of dm zero), the same measurement mix
    cfg = cfg4()
    dm = np.asfortranarray(np.concatenate([ds, 0 * p["dmu"][:, :, None]], axis=2))
    usr_par = {"config": {"nx": A(float(cfg.nx)), "nz": A(float(cfg.nz))},
               "data": {"t": np.asfortranarray(p["t"].reshape(1, -1)), "c_data": c_data},
               "network": {"ref_stat": np.asfortranarray(p["ref"]), "array": np.asfortranarray(p["arr"])},
               "type": "source", "veldis": "dis", "verbose": "no",
               "measurement": {"source": "waveform_difference", "structure": "log_amplitude_ratio"},
               "kernel": {"weighting": A(WEIGHTING)}}
    sov = dict(ov)
    sov["map_Hparameters_to_Hm"] = lambda H, *_: [np.asfortranarray(np.asarray(H).reshape(-1, 1, order="F"))]
    I = Interpreter(paths, sov)
    Hm = I.call("eval_hessian_vector_product_source", [m, dm, "abcdefgh", usr_par], nargout=1)[0]
    out["hvp/source/H"] = np.asarray(Hm, dtype=np.float64).reshape(m.shape, order="F")
    print(f"  hvp source: |H| = {np.linalg.norm(Hm):.4g}", flush=True)
    np.savez_compressed(OUT, **out)
    print(f"wrote {OUT} ({os.path.getsize(OUT) / 1e3:.1f} kB, {len(out)} arrays)")


if __name__ == "__main__":
    main()
