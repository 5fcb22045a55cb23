"""The MATLAB MEX gateways (fd2d_noise_gb300/mex/fd2d_mex.cpp) on the CPU.

MATLAB is not installed, so each gateway is compiled with g++ against a test
double of the MEX API (tests/mex_stub/mex.h, mex_runtime.cpp) and a recording
fake of the libfd2d entry points it calls (tests/mex_stub/fake_fd2d.cpp).  The
tests check what a MATLAB caller of run_*_mex relies on: the argument order of
the reference's signatures (code/run_forward1_green.m:1,
code/run_forward2_correlation.m:1, code/run_noise_adjoint.m:1), the hidden
configuration read from input_parameters / input_interferometry /
absorb_specs at every call, empties passed as NULL, complex arrays split into
planes and merged back, output shapes, and "fd2d:*" error identifiers.  The
library itself is tested through its C ABI elsewhere.
"""
import ctypes
import os
import shutil
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
STUB = os.path.join(ROOT, "tests", "mex_stub")
DOUBLE, SINGLE = 6, 7
FP32, FP64 = 1, 0  # FD2D_PREC_* of include/fd2d.h

pytestmark = pytest.mark.skipif(shutil.which("g++") is None, reason="needs g++")


class MexError(Exception):
    def __init__(self, ident, msg):
        super().__init__(f"{ident}: {msg}")
        self.ident, self.msg = ident, msg


class Gateway:
    """One compiled gateway with the MEX runtime double and the fake library."""

    def __init__(self, path):
        L = self.L = ctypes.CDLL(path)
        vp, sz = ctypes.c_void_p, ctypes.POINTER(ctypes.c_size_t)
        L.stub_array.restype = vp
        L.stub_array.argtypes = [ctypes.c_int, sz, ctypes.c_int, ctypes.c_int]
        L.stub_data.restype = vp
        L.stub_data.argtypes = [vp]
        L.stub_ndims.argtypes = [vp, sz]
        L.stub_class.argtypes = [vp]
        L.stub_is_complex.argtypes = [vp]
        L.stub_free.argtypes = [vp]
        L.stub_call.argtypes = [ctypes.c_int, ctypes.POINTER(vp), ctypes.c_int, ctypes.POINTER(vp), ctypes.c_char_p,
                                ctypes.c_int]
        L.stub_set_config.argtypes = [ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double), ctypes.c_int,
                                      ctypes.c_double, ctypes.POINTER(ctypes.c_double)]
        L.fake_last_call.argtypes = [ctypes.c_char_p, ctypes.c_int]
        L.fake_set_status.argtypes = [ctypes.c_int, ctypes.c_char_p]

    def set_config(self, Lx=4e4, Lz=3e4, nx=5, nz=4, dt=0.1, nt=6, order=4, nb=0, fw=2, f=(0.02, 0.03, 0.04),
                   fs=2, width=5e3, sides=(1, 1, 0, 1)):
        dbl = lambda v: (ctypes.c_double * len(v))(*v)  # noqa: E731
        self.cfg = dict(Lx=Lx, Lz=Lz, nx=nx, nz=nz, dt=dt, nt=nt, order=order, nb=nb, fw=fw, K=len(f), f=f, fs=fs,
                        width=width, sides=sides)
        self.L.stub_set_config(dbl([Lx, Lz, nx, nz, dt, nt, order, 1, 0, nb, fw]), dbl(list(f)), len(f), fs,
                               dbl([width, *sides]))

    def array(self, a=None, single=False, complex_=False, shape=None):
        a = np.zeros(shape if shape is not None else (0, 0)) if a is None else np.asarray(a)
        if a.ndim < 2:
            a = a.reshape(1, -1) if a.ndim == 1 else a.reshape(1, 1)
        cx = complex_ or np.iscomplexobj(a)
        dims = (ctypes.c_size_t * a.ndim)(*a.shape)
        h = self.L.stub_array(a.ndim, dims, SINGLE if single else DOUBLE, 1 if cx else 0)
        if a.size:
            flat = np.asfortranarray(a.astype(np.complex128 if cx else (np.float32 if single else np.float64)))
            buf = flat.ravel(order="F").tobytes()
            ctypes.memmove(self.L.stub_data(h), buf, len(buf))
        return h

    def numpy(self, h):
        dims = (ctypes.c_size_t * 8)()
        nd = self.L.stub_ndims(h, dims)
        shape = tuple(int(dims[i]) for i in range(nd))
        cx, cls = self.L.stub_is_complex(h), self.L.stub_class(h)
        dt = np.complex128 if cx else (np.float32 if cls == SINGLE else np.float64)
        n = int(np.prod(shape))
        raw = ctypes.string_at(self.L.stub_data(h), n * np.dtype(dt).itemsize) if n else b""
        return np.frombuffer(raw, dtype=dt).reshape(shape, order="F")

    def call(self, nlhs, args):
        prhs = (ctypes.c_void_p * len(args))(*args)
        plhs = (ctypes.c_void_p * max(nlhs, 1))()
        err = ctypes.create_string_buffer(2048)
        if self.L.stub_call(nlhs, plhs, len(args), prhs, err, len(err)):
            ident, _, msg = err.value.decode().partition("|")
            raise MexError(ident, msg)
        out = [self.numpy(plhs[i]) for i in range(nlhs)]
        for i in range(nlhs):
            self.L.stub_free(plhs[i])
        return out

    def last_call(self):
        buf = ctypes.create_string_buffer(8192)
        self.L.fake_last_call(buf, len(buf))
        kind, *rest = buf.value.decode().split()
        return kind, {k: float(v) for k, v in (x.split("=") for x in rest)}


def _build(tmp, variant, name):
    out = os.path.join(tmp, name)
    cmd = ["g++", "-std=c++17", "-O1", "-shared", "-fPIC", f"-DFD2D_MEX_{variant}", "-I", STUB, "-I",
           os.path.join(ROOT, "include"), os.path.join(ROOT, "fd2d_noise_gb300", "mex", "fd2d_mex.cpp"),
           os.path.join(STUB, "mex_runtime.cpp"), os.path.join(STUB, "fake_fd2d.cpp"), "-o", out]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return out


@pytest.fixture(scope="module")
def built(tmp_path_factory):
    tmp = str(tmp_path_factory.mktemp("mex"))
    return {v: _build(tmp, v, f"{v.lower()}.so") for v in ("FORWARD1", "CORRELATION", "ADJOINT")} | {"tmp": tmp}


def _ramp(shape, scale=1.0):
    return scale * (1.0 + np.arange(int(np.prod(shape)), dtype=np.float64)).reshape(shape, order="F")


def _check_cfg(rec, g):
    c = g.cfg
    for k in ("Lx", "Lz", "nx", "nz", "dt", "nt", "order", "nb", "fw", "K", "fs", "width"):
        assert rec[k] == pytest.approx(c[k], rel=0, abs=0), k
    assert rec["f0"] == c["f"][0] and rec["fK"] == c["f"][-1]
    assert [rec["left"], rec["right"], rec["top"], rec["bottom"]] == list(c["sides"])


def test_forward1_arguments_and_outputs(built):
    g = Gateway(built["FORWARD1"])
    g.set_config()
    nx, nz, nt, K = 5, 4, 6, 3
    mu, rho = _ramp((nx, nz), 4.8e10), _ramp((nx, nz), 3e3)
    src, rec = np.array([[1e4, 2e4]]), np.array([[1e3, 2e3], [3e3, 4e3], [5e3, 6e3]])
    G, G_out, seis = g.call(3, [g.array(mu), g.array(rho), g.array(src), g.array(rec), g.array(1.0), g.array(),
                                 g.array(single=True)])
    kind, r = g.last_call()
    assert kind == "forward1"
    _check_cfg(r, g)
    assert r["precision"] == FP64  # the reference's precision unless FP32 is asked for
    assert r["mu"] == mu.sum() and r["rho"] == rho.sum() and r["src"] == src.sum() and r["rec"] == rec.sum()
    assert (r["ns"], r["nr"], r["mode"]) == (1, 3, 1)
    assert (r["dmu_set"], r["G_in_set"], r["n_G_in"], r["G_out_set"]) == (0, 0, 0, 1)
    # conjugated spectrum handed back as one complex array, planes merged element by element
    i = np.arange(nx * nz * K, dtype=np.float64).reshape((nx, nz, K), order="F")
    assert G.shape == (nx, nz, K) and np.iscomplexobj(G)
    assert np.array_equal(G.real, i) and np.array_equal(G.imag, -0.5 * i)
    n_fw = len([n for n in range(nt, 2 * nt) if n % 2 == 0])
    assert G_out.dtype == np.float32 and G_out.shape == (nx, nz, n_fw)
    assert np.array_equal(G_out, np.arange(nx * nz * n_fw, dtype=np.float32).reshape(G_out.shape, order="F"))
    assert seis.shape == (3, nt) and np.array_equal(seis, 0.25 * np.arange(3 * nt).reshape((3, nt), order="F"))
    # one output requested: no wavefield buffer handed to the library when mode is 0
    (G1,) = g.call(1, [g.array(mu), g.array(rho), g.array(src), g.array(rec), g.array(0.0), g.array(),
                       g.array(single=True)])
    assert G1.shape == (nx, nz, K) and g.last_call()[1]["G_out_set"] == 0


def test_forward1_born_run_passes_dmu_and_stored_field(built):
    g = Gateway(built["FORWARD1"])
    g.set_config()
    nx, nz, nt = 5, 4, 6
    dmu, G_in = _ramp((nx, nz)), _ramp((nx, nz, nt)).astype(np.float32)
    g.call(3, [g.array(_ramp((nx, nz))), g.array(_ramp((nx, nz))), g.array(np.array([[1e4, 2e4]])),
               g.array(np.array([[1e3, 2e3]])), g.array(5.0), g.array(dmu), g.array(G_in, single=True)])
    r = g.last_call()[1]
    assert (r["dmu_set"], r["G_in_set"], r["n_G_in"], r["mode"]) == (1, 1, nt, 5)


def test_correlation_arguments_and_outputs(built):
    g = Gateway(built["CORRELATION"])
    g.set_config(nb=2)
    nx, nz, nt, K = 5, 4, 6, 3
    ntc = 2 * nt - 1
    G = _ramp((nx, nz, K)) - 1j * _ramp((nx, nz, K), 0.5)
    spec, sd = _ramp((K, 1)), _ramp((nx, nz, 2))
    rec = np.array([[1e3, 2e3], [3e3, 4e3]])
    C_in = _ramp((nx, nz, ntc)).astype(np.float32)
    seis, C_out = g.call(2, [g.array(_ramp((nx, nz))), g.array(_ramp((nx, nz))), g.array(G), g.array(spec),
                              g.array(sd), g.array(rec), g.array(1.0), g.array(_ramp((nx, nz))),
                              g.array(C_in, single=True)])
    kind, r = g.last_call()
    assert kind == "correlation"
    _check_cfg(r, g)
    assert r["G_re"] == G.real.sum() and r["G_im"] == G.imag.sum() and r["n_G"] == K
    assert (r["spectrum"], r["n_src"]) == (spec.sum(), 1)
    assert (r["sd"], r["n_dist"], r["nr"], r["mode"]) == (sd.sum(), 2, 2, 1)
    assert (r["dmu_set"], r["C_in_set"], r["n_C_in"], r["C_out_set"]) == (1, 1, ntc, 1)
    assert r["C_in"] == pytest.approx(float(C_in.astype(np.float64).sum()), rel=1e-12)
    assert seis.shape == (2, ntc) and np.array_equal(seis, 2.0 * np.arange(2 * ntc).reshape((2, ntc), order="F"))
    assert C_out.dtype == np.float32 and C_out.shape == (nx, nz, ntc // 2)
    # a 2-D source distribution is one plane; a real G_fft gets zero imaginary planes
    g.call(1, [g.array(_ramp((nx, nz))), g.array(_ramp((nx, nz))), g.array(G.real), g.array(spec),
               g.array(_ramp((nx, nz))), g.array(rec), g.array(0.0), g.array(), g.array(single=True)])
    r = g.last_call()[1]
    assert (r["n_dist"], r["G_im"], r["C_out_set"], r["dmu_set"], r["C_in_set"]) == (1, 0, 0, 0, 0)


@pytest.mark.parametrize("mode", [1, 11, 13])
def test_adjoint_point_sources(built, mode):
    g = Gateway(built["ADJOINT"])
    g.set_config()
    nx, nz, nt, K = 5, 4, 6, 3
    ntc = 2 * nt - 1
    stf = _ramp((2, ntc)) + 1j * _ramp((2, ntc), 0.1)
    u_fwd = _ramp((nx, nz, 5)).astype(np.float32)
    rec = np.array([[1e3, 2e3], [3e3, 4e3]])
    Kk, sf, u_out, seis = g.call(4, [g.array(_ramp((nx, nz))), g.array(_ramp((nx, nz))),
                                     g.array(u_fwd, single=True), g.array(stf), g.array(rec), g.array(rec),
                                     g.array(_ramp((K, 1))), g.array(), g.array(), g.array(float(mode)), g.array(),
                                     g.array(single=True)])
    kind, r = g.last_call()
    assert kind == "adjoint"
    _check_cfg(r, g)
    assert (r["d0"], r["d1"], r["d2"]) == (2, ntc, 1)
    assert r["stf_re"] == stf.real.sum() and r["stf_im"] == pytest.approx(stf.imag.sum(), rel=1e-15)
    assert (r["n_u_fwd"], r["ns"], r["nr"], r["spectrum_set"], r["sd_set"], r["G_set"]) == (5, 2, 2, 1, 0, 0)
    assert (r["mode"], r["dmu_set"], r["u_in_set"]) == (mode, 0, 0)
    assert r["u_out_set"] == (1 if mode in (11, 13) else 0)
    assert Kk.shape == (nx, nz, 2) and np.array_equal(Kk, 3.0 * np.arange(nx * nz * 2).reshape(Kk.shape, order="F"))
    i = np.arange(nx * nz * K, dtype=np.float64).reshape((nx, nz, K), order="F")
    assert sf.shape == (nx, nz, K) and np.array_equal(sf.real, i) and np.array_equal(sf.imag, 1.0 + i)
    assert u_out.dtype == np.float32 and u_out.shape[:2] == (nx, nz)
    assert seis.shape == (2, ntc)


def test_adjoint_field_source_and_born_term(built):
    g = Gateway(built["ADJOINT"])
    g.set_config(nb=3)
    nx, nz, nt, K = 5, 4, 6, 3
    ntc = 2 * nt - 1
    S = _ramp((nx, nz, K)) + 2j * _ramp((nx, nz, K))
    G = _ramp((nx, nz, K), 0.5) - 1j * _ramp((nx, nz, K))
    u_in = _ramp((nx, nz, ntc)).astype(np.float32)
    (Kk,) = g.call(1, [g.array(_ramp((nx, nz))), g.array(_ramp((nx, nz))), g.array(single=True), g.array(S),
                       g.array(), g.array(np.array([[1e3, 2e3]])), g.array(_ramp((K, 1))),
                       g.array(_ramp((nx, nz, 3))), g.array(G), g.array(10.0), g.array(_ramp((nx, nz))),
                       g.array(u_in, single=True)])
    r = g.last_call()[1]
    assert (r["d0"], r["d1"], r["d2"]) == (nx, nz, K)
    assert (r["ns"], r["n_u_fwd"], r["n_dist"], r["G_set"], r["n_G"]) == (0, 0, 3, 1, K)
    assert r["G_re"] == G.real.sum()
    assert (r["dmu_set"], r["u_in_set"], r["n_u_in"], r["u_out_set"]) == (1, 1, ntc, 0)
    assert Kk.shape == (nx, nz, 4)  # n_basis_fct source planes + K_mu


def test_errors_carry_fd2d_identifiers(built):
    g = Gateway(built["FORWARD1"])
    g.set_config()
    mu = _ramp((5, 4))
    good = lambda: [g.array(mu), g.array(mu), g.array(np.array([[1e4, 2e4]])),  # noqa: E731
                    g.array(np.array([[1e3, 2e3]])), g.array(0.0), g.array(), g.array(single=True)]
    with pytest.raises(MexError) as e:
        g.call(1, good()[:6])
    assert e.value.ident == "fd2d:nargin"
    args = good()
    args[3] = g.array(np.ones((2, 3)))
    with pytest.raises(MexError) as e:
        g.call(1, args)
    assert e.value.ident == "fd2d:shape" and "rec" in e.value.msg
    args = good()
    args[6] = g.array(np.ones((5, 4, 2)))  # G_in must be single
    with pytest.raises(MexError) as e:
        g.call(1, args)
    assert e.value.ident == "fd2d:type" and "G_in" in e.value.msg
    g.L.fake_set_status(7, b"device gave up")
    with pytest.raises(MexError) as e:
        g.call(1, good())
    assert e.value.ident == "fd2d:7" and "run_forward1_green: device gave up" in e.value.msg
    g.set_config(nx=1)
    with pytest.raises(MexError) as e:
        g.call(1, good())
    assert e.value.ident.startswith("fd2d:") and "configuration" in e.value.msg


def test_fp32_form_selected_by_environment(built, monkeypatch):
    # a fresh copy of the gateway: the context is created at its first call
    path = _build(built["tmp"], "FORWARD1", "forward1_fp32.so")
    g = Gateway(path)
    g.set_config()
    monkeypatch.setenv("FD2D_PRECISION", "fp32")
    mu = _ramp((5, 4))
    g.call(1, [g.array(mu), g.array(mu), g.array(np.array([[1e4, 2e4]])), g.array(np.array([[1e3, 2e3]])),
               g.array(0.0), g.array(), g.array(single=True)])
    assert g.last_call()[1]["precision"] == FP32
