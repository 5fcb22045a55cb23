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
    return I.call(fn, [A(a) if not isinstance(a, (str, np.ndarray)) else a for a in args], nargout=nargout)


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
