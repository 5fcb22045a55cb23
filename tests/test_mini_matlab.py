"""Semantics of the MATLAB-subset interpreter that produces the golden vectors."""
import os
import sys

import numpy as np

sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden"))
from mini_matlab import A, Interpreter, Parser, tokenize  # noqa: E402


def run(src, fn, *args, nargout=1):
    funcs = Parser(tokenize(src)).parse_file()
    I = Interpreter([])
    for f in funcs:
        I.cache[f[1]] = f
    return I.call(fn, [A(a) if not isinstance(a, (str, dict, np.ndarray)) else a for a in args], nargout=nargout)


def test_single_arithmetic_stays_single():
    src = "function out = f(v, dx)\nout = zeros(3,1);\nout(2,:) = 9*(v(3,:)-v(2,:))/(8*dx);\n"
    v = np.array([[1.0], [2.5], [7.25]], dtype=np.float32)
    (out,) = run(src, "f", v, 0.3)
    expect = np.float32(9.0) * (np.float32(7.25) - np.float32(2.5)) / np.float32(8 * 0.3)
    assert out.dtype == np.float64 and out[1, 0] == np.float64(expect)


def test_colon_end_and_linear_indexing():
    src = ("function [a, b, c] = f(x)\na = x(end-1, :);\nb = x(5);\nt = 0:0.1:0.3;\nc = t(end);\n")
    x = np.asfortranarray(np.arange(12.0).reshape(3, 4, order="F"))
    a, b, c = run(src, "f", x, nargout=3)
    assert np.array_equal(a, x[1:2, :]) and b[0, 0] == 4.0 and c[0, 0] == 0.3


def test_precedence_and_min_find():
    src = ("function [r, k] = f(x, p)\nr = -2^2 + 3*2 - 1;\n"
           "k = min( find( min(abs(x-p)) == abs(x-p) ) );\n")
    r, k = run(src, "f", np.array([[0.0, 1.0, 2.0, 3.0]]), 1.5, nargout=2)
    assert r[0, 0] == 1.0 and k[0, 0] == 2.0  # tie at 1 and 2 goes to the lower index


def test_slice_assignment_and_complex():
    src = ("function G = f(v, c)\nG = zeros(2,2,3) + 1i*zeros(2,2,3);\n"
           "for k = 1:3\n  G(:,:,k) = G(:,:,k) + v * c(k);\nend\nG(:,:,2) = conj(G(:,:,2));\n")
    v = np.asfortranarray(np.array([[1.0, 2.0], [3.0, 4.0]]))
    c = np.array([[1 + 1j, 2 - 1j, 0.5j]])
    (G,) = run(src, "f", v, c)
    assert G.shape == (2, 2, 3)
    assert np.allclose(G[:, :, 0], v * (1 + 1j)) and np.allclose(G[:, :, 1], np.conj(v * (2 - 1j)))


def test_while_break_and_nargin():
    src = ("function [n, k] = f(a, b)\nif nargin < 2\n  b = 10;\nend\nn = 0; k = 1;\n"
           "while k < b\n  k = 2*k;\n  n = n + 1;\n  if n >= a\n    break\n  end\nend\n")
    n, k = run(src, "f", 100.0, nargout=2)
    assert n[0, 0] == 4.0 and k[0, 0] == 16.0  # nargin == 1: b = 10
    n, k = run(src, "f", 2.0, 1000.0, nargout=2)
    assert n[0, 0] == 2.0 and k[0, 0] == 4.0


def test_structs_and_struct_arrays():
    src = ("function [s, v] = f(p)\ns.a = 1;\ns.b.c = [1 2 3];\ns.b.c(2) = 7;\n"
           "if isfield(s, 'a') && ~isfield(s, 'z')\n  s.a = s.a + p.model(2).objective;\nend\nv = s.b.c;\n")
    p = {"model": [{"objective": A(5.0)}, {"objective": A(11.0)}]}
    s, v = run(src, "f", p, nargout=2)
    assert s["a"][0, 0] == 12.0 and np.array_equal(v, np.array([[1.0, 7.0, 3.0]]))


def test_rows_find_reshape_and_strings():
    src = ("function [rec, r, c, x, name] = f(a, src)\n"
           "rec = a( find(~ismember(a, src, 'rows')), :);\n"
           "[r, c] = find([0 1; 1 0; 0 1]);\n"
           "t = reshape(1:24, 2, 3, 4);\nx = reshape(t(2,:,:), [], 4);\n"
           "name = ['G_fft_' num2str(3) '.mat'];\n"
           "total = 0;\nparfor i = 1:3\n  total = total + i;\nend\n")
    a = np.array([[1.0, 2.0], [3.0, 4.0], [5.0, 6.0]])
    rec, r, c, x, name = run(src, "f", a, np.array([[3.0, 4.0]]), nargout=5)
    assert np.array_equal(rec, a[[0, 2]])
    assert r.ravel().tolist() == [2.0, 1.0, 3.0] and c.ravel().tolist() == [1.0, 2.0, 2.0]
    assert x.shape == (3, 4) and x[0, 0] == 2.0 and x[2, 3] == 24.0
    assert name == "G_fft_3.mat"
