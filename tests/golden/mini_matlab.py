"""A small MATLAB-subset interpreter (test infrastructure).

It executes the reference's own sources as written -- the solvers
(code/run_*.m, code/propagation/*.m), the noise-source model, the
measurements, the model maps, the optimiser (inversion/optlib) and the
misfit / gradient / Hessian orchestration -- so that golden vectors can be
produced here without MATLAB.  It implements the subset those files use:
function files with multiple outputs and ``nargin``, for / parfor / while /
if-elseif-else, indexed reads and writes with ``:`` and ``end``, column-major
linear indexing, implicit expansion, complex values, ``single`` arithmetic (an
operation with a single operand is carried out in single precision, as MATLAB
does), scalar structs (Python dicts) and struct arrays (lists of dicts),
string concatenation, and the builtins listed in ``BUILTINS``.  Functions
outside the reference checkout (solver MEX calls in the orchestration cases,
user callbacks of the optimiser, configuration getters) are supplied by the
caller as overrides.

Values are numpy arrays with at least two dimensions in Fortran order; strings
are Python ``str``.  Anything outside the subset raises ``MatlabError``.
"""
from __future__ import annotations

import os
import re
from typing import Any, Callable, Dict, List, Optional

import numpy as np


class MatlabError(RuntimeError):
    pass


def reference_checkout(argv: List[str]) -> str:
    """The reference checkout a fixture generator reads: its first command-line
    argument, else the FD2D_REFERENCE environment variable (no default)."""
    if len(argv) > 1:
        return argv[1]
    path = os.environ.get("FD2D_REFERENCE")
    if not path:
        raise SystemExit(f"usage: python {os.path.basename(argv[0])} <reference checkout> "
                         "(or set FD2D_REFERENCE)")
    return path


# ---------------------------------------------------------------------------
# tokenizer
# ---------------------------------------------------------------------------
TOKEN_RE = re.compile(r"""
    (?P<num>(?:\d+\.\d*|\.\d+|\d+)(?:[eE][+-]?\d+)?[ij]?)
  | (?P<id>[A-Za-z_][A-Za-z0-9_]*)
  | (?P<op>\.\*|\./|\.\^|\.'|==|~=|<=|>=|&&|\|\||[-+*/^\\<>&|~=(),;:\[\]'{}.@])
  | (?P<nl>\n)
  | (?P<ws>[ \t\r]+)
""", re.VERBOSE)

KEYWORDS = {"function", "for", "parfor", "end", "if", "elseif", "else", "while", "return", "break"}


class Tok:
    __slots__ = ("kind", "val", "line")

    def __init__(self, kind, val, line):
        self.kind, self.val, self.line = kind, val, line

    def __repr__(self):
        return f"Tok({self.kind},{self.val!r},{self.line})"


def tokenize(src: str) -> List[Tok]:
    out: List[Tok] = []
    line = 1
    i = 0
    n = len(src)
    bracket = 0
    while i < n:
        c = src[i]
        if c == "%":
            while i < n and src[i] != "\n":
                i += 1
            continue
        if src.startswith("...", i):
            while i < n and src[i] != "\n":
                i += 1
            i += 1
            line += 1
            continue
        if c == "'":
            prev = out[-1] if out else None
            transpose = prev is not None and (
                prev.kind in ("id", "num") or (prev.kind == "op" and prev.val in (")", "]", "'", ".'", "}")))
            # inside [] a space before ' starts a string
            if transpose and not (bracket and i > 0 and src[i - 1] in " \t"):
                out.append(Tok("op", "'", line))
                i += 1
                continue
            j = i + 1
            s = []
            while True:
                if j >= n:
                    raise MatlabError("unterminated string")
                if src[j] == "'":
                    if j + 1 < n and src[j + 1] == "'":
                        s.append("'")
                        j += 2
                        continue
                    break
                s.append(src[j])
                j += 1
            out.append(Tok("str", "".join(s), line))
            i = j + 1
            continue
        if c == '"':  # double-quoted string literal ("" escapes a quote)
            j = i + 1
            s = []
            while True:
                if j >= n:
                    raise MatlabError("unterminated string")
                if src[j] == '"':
                    if j + 1 < n and src[j + 1] == '"':
                        s.append('"')
                        j += 2
                        continue
                    break
                s.append(src[j])
                j += 1
            out.append(Tok("str", "".join(s), line))
            i = j + 1
            continue
        m = TOKEN_RE.match(src, i)
        if not m:
            raise MatlabError(f"line {line}: cannot tokenize {src[i:i+20]!r}")
        kind = m.lastgroup
        val = m.group(kind)
        i = m.end()
        if kind == "ws":
            continue
        if kind == "nl":
            out.append(Tok("nl", "\n", line))
            line += 1
            continue
        if kind == "id" and val in KEYWORDS:
            kind = "kw"
        if kind == "op" and val in ("[", "{"):
            bracket += 1
        if kind == "op" and val in ("]", "}"):
            bracket -= 1
        out.append(Tok(kind, val, line))
    out.append(Tok("eof", None, line))
    return out


# ---------------------------------------------------------------------------
# parser (AST as tuples)
# ---------------------------------------------------------------------------
class Parser:
    def __init__(self, toks: List[Tok]):
        self.t = toks
        self.i = 0
        self.in_index = 0

    def peek(self, k=0) -> Tok:
        return self.t[self.i + k]

    def next(self) -> Tok:
        tok = self.t[self.i]
        self.i += 1
        return tok

    def accept(self, kind, val=None) -> Optional[Tok]:
        tok = self.peek()
        if tok.kind == kind and (val is None or tok.val == val):
            self.i += 1
            return tok
        return None

    def expect(self, kind, val=None) -> Tok:
        tok = self.accept(kind, val)
        if tok is None:
            p = self.peek()
            raise MatlabError(f"line {p.line}: expected {val or kind}, got {p.val!r}")
        return tok

    def skip_sep(self):
        while self.peek().kind == "nl" or (self.peek().kind == "op" and self.peek().val in (";", ",")):
            self.i += 1

    # -- program ---------------------------------------------------------------
    def parse_file(self):
        funcs = []
        self.skip_sep()
        while self.peek().kind != "eof":
            if self.peek().kind == "kw" and self.peek().val == "function":
                funcs.append(self.parse_function())
            else:
                raise MatlabError(f"line {self.peek().line}: only function files are supported")
            self.skip_sep()
        return funcs

    def parse_function(self):
        self.expect("kw", "function")
        outs: List[str] = []
        # [a, b] = name(...)  |  a = name(...)  |  name(...)
        save = self.i
        if self.accept("op", "["):
            while not self.accept("op", "]"):
                tok = self.next()
                if tok.kind == "id":
                    outs.append(tok.val)
            self.expect("op", "=")
        else:
            if self.peek().kind == "id" and self.peek(1).kind == "op" and self.peek(1).val == "=":
                outs.append(self.next().val)
                self.next()
            else:
                self.i = save
        name = self.expect("id").val
        params: List[str] = []
        if self.accept("op", "("):
            while not self.accept("op", ")"):
                tok = self.next()
                if tok.kind == "id":
                    params.append(tok.val)
                elif tok.kind == "op" and tok.val == "~":
                    params.append("~")
        body = self.parse_block(("function", "eof"), allow_end=True)
        return ("function", name, params, outs, body)

    def parse_block(self, stops, allow_end=False):
        stmts = []
        while True:
            self.skip_sep()
            tok = self.peek()
            if tok.kind == "eof":
                return stmts
            if tok.kind == "kw" and tok.val in stops:
                return stmts
            if tok.kind == "kw" and tok.val == "end":
                if allow_end:
                    self.next()
                    return stmts
                return stmts
            if tok.kind == "kw" and tok.val in ("elseif", "else"):
                return stmts
            stmts.append(self.parse_statement())

    def parse_statement(self):
        tok = self.peek()
        if tok.kind == "kw":
            if tok.val in ("for", "parfor"):
                self.next()
                paren = self.accept("op", "(")
                var = self.expect("id").val
                self.expect("op", "=")
                rng = self.parse_expr()
                if paren:
                    self.expect("op", ")")
                body = self.parse_block(())
                self.expect("kw", "end")
                return ("for", var, rng, body)
            if tok.val == "while":
                self.next()
                cond = self.parse_expr()
                body = self.parse_block(())
                self.expect("kw", "end")
                return ("while", cond, body)
            if tok.val == "if":
                self.next()
                clauses = []
                cond = self.parse_expr()
                body = self.parse_block(())
                clauses.append((cond, body))
                els = None
                while True:
                    if self.accept("kw", "elseif"):
                        c = self.parse_expr()
                        b = self.parse_block(())
                        clauses.append((c, b))
                        continue
                    if self.accept("kw", "else"):
                        els = self.parse_block(())
                    self.expect("kw", "end")
                    break
                return ("if", clauses, els)
            if tok.val == "return":
                self.next()
                return ("return",)
            if tok.val == "break":
                self.next()
                return ("break",)
            raise MatlabError(f"line {tok.line}: unsupported keyword {tok.val}")
        # multi-assignment [a, ~, b] = f(...)
        if tok.kind == "op" and tok.val == "[":
            save = self.i
            try:
                self.next()
                targets = []
                while True:
                    if self.accept("op", "~"):
                        targets.append(None)
                    else:
                        targets.append(self.parse_postfix())
                    if self.accept("op", "]"):
                        break
                    self.accept("op", ",")
                if self.accept("op", "="):
                    rhs = self.parse_expr()
                    return ("massign", targets, rhs)
            except MatlabError:
                pass
            self.i = save
        expr = self.parse_expr()
        if self.accept("op", "="):
            rhs = self.parse_expr()
            return ("assign", expr, rhs)
        return ("expr", expr)

    # -- expressions ------------------------------------------------------------
    def parse_expr(self):
        return self.parse_oror()

    def parse_oror(self):
        e = self.parse_andand()
        while self.accept("op", "||"):
            e = ("||", e, self.parse_andand())
        return e

    def parse_andand(self):
        e = self.parse_or()
        while self.accept("op", "&&"):
            e = ("&&", e, self.parse_or())
        return e

    def parse_or(self):
        e = self.parse_and()
        while self.accept("op", "|"):
            e = ("bin", "|", e, self.parse_and())
        return e

    def parse_and(self):
        e = self.parse_cmp()
        while self.accept("op", "&"):
            e = ("bin", "&", e, self.parse_cmp())
        return e

    def parse_cmp(self):
        e = self.parse_range()
        while True:
            tok = self.peek()
            if tok.kind == "op" and tok.val in ("==", "~=", "<", "<=", ">", ">="):
                self.next()
                e = ("bin", tok.val, e, self.parse_range())
            else:
                return e

    def parse_range(self):
        if self.in_index and self.peek().kind == "op" and self.peek().val == ":":
            nxt = self.peek(1)
            if nxt.kind == "op" and nxt.val in (",", ")"):
                self.next()
                return ("colon_all",)
        e = self.parse_add()
        if self.peek().kind == "op" and self.peek().val == ":":
            self.next()
            e2 = self.parse_add()
            if self.peek().kind == "op" and self.peek().val == ":":
                self.next()
                e3 = self.parse_add()
                return ("range", e, e2, e3)
            return ("range", e, None, e2)
        return e

    def parse_add(self):
        e = self.parse_mul()
        while True:
            tok = self.peek()
            if tok.kind == "op" and tok.val in ("+", "-"):
                self.next()
                e = ("bin", tok.val, e, self.parse_mul())
            else:
                return e

    def parse_mul(self):
        e = self.parse_unary()
        while True:
            tok = self.peek()
            if tok.kind == "op" and tok.val in ("*", "/", ".*", "./", "\\"):
                self.next()
                e = ("bin", tok.val, e, self.parse_unary())
            else:
                return e

    def parse_unary(self):
        tok = self.peek()
        if tok.kind == "op" and tok.val in ("-", "+", "~"):
            self.next()
            return ("un", tok.val, self.parse_unary())
        return self.parse_power()

    def parse_power(self):
        e = self.parse_postfix()
        while True:
            tok = self.peek()
            if tok.kind == "op" and tok.val in ("^", ".^"):
                self.next()
                # the exponent may carry a unary sign: 2^-1
                if self.peek().kind == "op" and self.peek().val in ("-", "+"):
                    sgn = self.next().val
                    rhs = ("un", sgn, self.parse_postfix())
                else:
                    rhs = self.parse_postfix()
                e = ("bin", tok.val, e, rhs)
            else:
                return e

    def parse_postfix(self):
        e = self.parse_primary()
        while True:
            tok = self.peek()
            if tok.kind == "op" and tok.val == "(":
                self.next()
                args = []
                self.in_index += 1
                if not self.accept("op", ")"):
                    while True:
                        args.append(self.parse_expr())
                        if self.accept("op", ")"):
                            break
                        self.expect("op", ",")
                self.in_index -= 1
                e = ("call", e, args)
            elif tok.kind == "op" and tok.val in ("'", ".'"):
                self.next()
                e = ("transpose", tok.val, e)
            elif tok.kind == "op" and tok.val == "." and self.peek(1).kind == "id":
                # struct field (scalar structs are dicts)
                self.next()
                e = ("field", e, self.next().val)
            else:
                return e

    def parse_primary(self):
        tok = self.next()
        if tok.kind == "num":
            v = tok.val
            if v[-1] in "ij":
                return ("num", complex(0, float(v[:-1])))
            return ("num", float(v))
        if tok.kind == "str":
            return ("str", tok.val)
        if tok.kind == "id":
            return ("id", tok.val)
        if tok.kind == "kw" and tok.val == "end" and self.in_index:
            return ("end",)
        if tok.kind == "op" and tok.val == "(":
            saved = self.in_index
            self.in_index = 0
            e = self.parse_expr()
            self.in_index = saved
            self.expect("op", ")")
            return ("paren", e)
        if tok.kind == "op" and tok.val == "[":
            rows = [[]]
            saved = self.in_index
            self.in_index = 0
            while True:
                if self.accept("op", "]"):
                    break
                if self.accept("op", ";") or self.accept("nl"):
                    rows.append([])
                    continue
                if self.accept("op", ","):
                    continue
                rows[-1].append(self.parse_expr())
            self.in_index = saved
            return ("matrix", [r for r in rows if r])
        raise MatlabError(f"line {tok.line}: unexpected token {tok.val!r}")


# ---------------------------------------------------------------------------
# values
# ---------------------------------------------------------------------------
def A(x) -> np.ndarray:
    """Any scalar/array -> ndarray with ndim >= 2 (MATLAB shape)."""
    if isinstance(x, np.ndarray):
        if x.ndim >= 2:
            return x
        if x.ndim == 0:
            return x.reshape(1, 1)
        return x.reshape(1, -1)
    if isinstance(x, (bool, np.bool_)):
        return np.array([[bool(x)]])
    if isinstance(x, (int, float, np.integer, np.floating)):
        return np.array([[float(x)]])
    if isinstance(x, (complex, np.complexfloating)):
        return np.array([[complex(x)]])
    raise MatlabError(f"not an array: {type(x)}")


def is_single(a: np.ndarray) -> bool:
    return a.dtype in (np.float32, np.complex64)


def scalar(a) -> Any:
    a = A(a)
    if a.size != 1:
        raise MatlabError(f"expected a scalar, got shape {a.shape}")
    v = a.reshape(-1)[0]
    if np.iscomplexobj(a):
        return complex(v)
    if a.dtype == np.bool_:
        return bool(v)
    return float(v)


def trim(a: np.ndarray) -> np.ndarray:
    """Drop trailing singleton dimensions beyond the second."""
    while a.ndim > 2 and a.shape[-1] == 1:
        a = a.reshape(a.shape[:-1], order="F")
    return a


def to_float(a: np.ndarray) -> np.ndarray:
    if a.dtype == np.bool_:
        return a.astype(np.float64)
    return a


def promote(x: np.ndarray, y: np.ndarray):
    """MATLAB: an operation with a single operand is computed in single."""
    x, y = to_float(x), to_float(y)
    if is_single(x) or is_single(y):
        cx = np.complex64 if np.iscomplexobj(x) else np.float32
        cy = np.complex64 if np.iscomplexobj(y) else np.float32
        x, y = x.astype(cx), y.astype(cy)
    return x, y


def expand(x: np.ndarray, y: np.ndarray):
    nd = max(x.ndim, y.ndim)
    if x.ndim < nd:
        x = x.reshape(x.shape + (1,) * (nd - x.ndim), order="F")
    if y.ndim < nd:
        y = y.reshape(y.shape + (1,) * (nd - y.ndim), order="F")
    return x, y


def simplify_complex(a: np.ndarray) -> np.ndarray:
    return a


def elementwise(op, x, y):
    x, y = promote(A(x), A(y))
    x, y = expand(x, y)
    with np.errstate(divide="ignore", invalid="ignore", over="ignore"):
        r = op(x, y)
    return np.asfortranarray(trim(A(r)))


def binop(op: str, x, y):
    x, y = A(x), A(y)
    if op == "+":
        return elementwise(np.add, x, y)
    if op == "-":
        return elementwise(np.subtract, x, y)
    if op == ".*":
        return elementwise(np.multiply, x, y)
    if op == "./":
        return elementwise(np.divide, x, y)
    if op == ".^":
        return elementwise(lambda a, b: np.power(a, b), x, y)
    if op == "*":
        if x.size == 1 or y.size == 1:
            return elementwise(np.multiply, x, y)
        if x.ndim != 2 or y.ndim != 2:
            raise MatlabError("matrix product of N-D arrays")
        if x.shape[1] != y.shape[0]:
            raise MatlabError(f"inner dimensions must agree: {x.shape} * {y.shape}")
        x, y = promote(x, y)
        return np.asfortranarray(x @ y)
    if op == "/":
        if y.size == 1:
            return elementwise(np.divide, x, y)
        raise MatlabError("matrix right division is not supported")
    if op == "^":
        if x.size == 1 and y.size == 1:
            return elementwise(np.power, x, y)
        raise MatlabError("matrix power is not supported")
    if op in ("==", "~=", "<", "<=", ">", ">="):
        f = {"==": np.equal, "~=": np.not_equal, "<": np.less, "<=": np.less_equal,
             ">": np.greater, ">=": np.greater_equal}[op]
        if op in ("<", "<=", ">", ">="):
            x, y = np.real(x), np.real(y)
        return elementwise(f, x, y)
    if op == "&":
        return elementwise(np.logical_and, x != 0, y != 0)
    if op == "|":
        return elementwise(np.logical_or, x != 0, y != 0)
    raise MatlabError(f"operator {op}")


def truth(v) -> bool:
    a = A(v)
    if a.size == 0:
        return False
    return bool(np.all(a != 0))


def colon(a: float, d: float, b: float) -> np.ndarray:
    """a:d:b (published construction of MATLAB's colon operator)."""
    eps = np.finfo(np.float64).eps
    if d == 0 or (d > 0 and a > b) or (d < 0 and a < b):
        return np.zeros((1, 0))
    tol = 2.0 * eps * max(abs(a), abs(b))
    sig = 1.0 if d > 0 else -1.0
    if a == np.floor(a) and d == 1:
        n = int(np.floor(b) - a)
    elif a == np.floor(a) and d == np.floor(d):
        q = np.floor(a / d)
        r = a - q * d
        n = int(np.floor((b - r) / d) - q)
    else:
        n = int(np.round((b - a) / d))
        if sig * (a + n * d - b) > tol:
            n -= 1
    if n < 0:
        return np.zeros((1, 0))
    last = a + n * d
    if a == np.floor(a) and d == np.floor(d):
        last = float(np.floor(last))
    elif sig * (last - b) > -tol:
        last = b
    out = np.zeros(n + 1)
    k = np.arange(0, n // 2 + 1)
    out[k] = a + k * d
    out[n - k] = last - k * d
    if n % 2 == 0:
        out[n // 2] = (a + last) / 2
    return out.reshape(1, -1)


# ---------------------------------------------------------------------------
# indexing
# ---------------------------------------------------------------------------
class ColonAll:
    pass


COLON_ALL = ColonAll()


def index_list(sub, dim_size):
    """1-based MATLAB subscript -> 0-based integer array."""
    if isinstance(sub, ColonAll):
        return np.arange(dim_size)
    s = A(sub)
    if s.dtype == np.bool_:
        return np.nonzero(s.reshape(-1, order="F"))[0]
    v = np.real(s).reshape(-1, order="F")
    iv = v.astype(np.int64)
    if np.any(iv != v) or np.any(iv < 1):
        raise MatlabError("subscript indices must be positive integers")
    return iv - 1


def effective_shape(a: np.ndarray, k: int):
    """Shape seen by k subscripts (the last one spans the remaining dims)."""
    sh = list(a.shape)
    if k >= len(sh):
        return sh + [1] * (k - len(sh))
    return sh[:k - 1] + [int(np.prod(sh[k - 1:]))]


def mread(a, subs):
    a = A(a)
    if len(subs) == 1:
        flat = a.reshape(-1, order="F")
        if isinstance(subs[0], ColonAll):
            return np.asfortranarray(flat.reshape(-1, 1))
        idx = index_list(subs[0], flat.size)
        if idx.size and idx.max() >= flat.size:
            raise MatlabError("index exceeds the number of array elements")
        s = A(subs[0])
        res = flat[idx]
        if a.shape[0] == 1 and a.ndim == 2 and (s.shape[0] == 1 or s.size == 1):
            return res.reshape(1, -1)
        if a.ndim == 2 and a.shape[1] == 1:
            return res.reshape(-1, 1)
        return np.asfortranarray(res.reshape(s.shape, order="F") if s.size == res.size else res.reshape(1, -1))
    shape = effective_shape(a, len(subs))
    v = a.reshape(shape, order="F")
    idx = [index_list(s, shape[d]) for d, s in enumerate(subs)]
    for d, ix in enumerate(idx):
        if ix.size and ix.max() >= shape[d]:
            raise MatlabError(f"index exceeds array bounds (dim {d + 1})")
    res = v[np.ix_(*idx)]
    return np.asfortranarray(trim(A(res)))


def massign_into(a: Optional[np.ndarray], subs, rhs) -> np.ndarray:
    rhs = A(rhs)
    if a is None:
        a = np.zeros((0, 0))
    a = A(a)
    if len(subs) == 1:
        flat = a.reshape(-1, order="F").copy()
        idx = index_list(subs[0], flat.size) if not isinstance(subs[0], ColonAll) else np.arange(flat.size)
        if idx.size and idx.max() >= flat.size:
            raise MatlabError("linear-index growth is not supported")
        vals = rhs.reshape(-1, order="F")
        if vals.size == 1:
            vals = np.repeat(vals, idx.size)
        if vals.size != idx.size:
            raise MatlabError("number of elements must match")
        flat = flat.astype(np.result_type(flat, vals)) if np.iscomplexobj(vals) and not np.iscomplexobj(flat) else flat
        flat[idx] = vals
        return np.asfortranarray(flat.reshape(a.shape, order="F"))
    k = len(subs)
    shape = effective_shape(a, k)
    idx = [index_list(s, shape[d]) for d, s in enumerate(subs)]
    # A(1,:) = v into an empty (or new) A: the ':' dimension takes its length
    # from v, as in MATLAB
    empty_colon = [d for d, sb in enumerate(subs) if isinstance(sb, ColonAll) and shape[d] == 0]
    if len(empty_colon) == 1 and rhs.size > 1:
        rest = int(np.prod([ix.size for d, ix in enumerate(idx) if d != empty_colon[0]]))
        if rest and rhs.size % rest == 0:
            idx[empty_colon[0]] = np.arange(rhs.size // rest)
    need = [max(shape[d], (ix.max() + 1) if ix.size else 0) for d, ix in enumerate(idx)]
    if need != shape:
        if k < a.ndim and any(n != s for n, s in zip(need[:-1], shape[:-1])):
            raise MatlabError("growth of a collapsed array is not supported")
        grown = np.zeros(need + list(a.shape[k:]) if k > a.ndim else need, dtype=a.dtype, order="F")
        grown[tuple(slice(0, s) for s in shape)] = a.reshape(shape, order="F")
        a = grown
        shape = need
    v = a.reshape(shape, order="F").copy(order="F")
    if np.iscomplexobj(rhs) and not np.iscomplexobj(v):
        v = v.astype(np.complex64 if v.dtype == np.float32 else np.complex128)
    target_shape = tuple(ix.size for ix in idx)
    vals = rhs
    if vals.size == 1:
        vals = np.full(target_shape, vals.reshape(-1)[0])
    elif vals.size == int(np.prod(target_shape)):
        vals = vals.reshape(target_shape, order="F")
    else:
        raise MatlabError(f"assignment dimension mismatch {rhs.shape} -> {target_shape}")
    v[np.ix_(*idx)] = vals
    out_shape = list(a.shape) if k <= a.ndim else shape
    return np.asfortranarray(trim(v.reshape(out_shape, order="F")))


# ---------------------------------------------------------------------------
# builtins
# ---------------------------------------------------------------------------
def _dims(args):
    cls = "double"
    nums = []
    for x in args:
        if isinstance(x, str):
            cls = x
        else:
            nums.extend(int(v) for v in A(x).reshape(-1))
    if len(nums) == 0:
        nums = [1, 1]
    if len(nums) == 1:
        nums = [nums[0], nums[0]]
    dtype = np.float32 if cls == "single" else np.float64
    return nums, dtype


def b_zeros(*args):
    d, t = _dims(args)
    return np.asfortranarray(trim(np.zeros(d, dtype=t, order="F")))


def b_ones(*args):
    d, t = _dims(args)
    return np.asfortranarray(trim(np.ones(d, dtype=t, order="F")))


def b_size(x, dim=None):
    a = A(x)
    if dim is None:
        return np.array([list(a.shape)], dtype=np.float64)
    d = int(scalar(dim))
    return A(float(a.shape[d - 1]) if d <= a.ndim else 1.0)


def b_reshape(x, *dims):
    a = A(x)
    if len(dims) > 1:
        # one dimension may be [] (computed from the others)
        d = [None if A(v).size == 0 else int(scalar(v)) for v in dims]
        if None in d:
            known = int(np.prod([v for v in d if v is not None]))
            d[d.index(None)] = a.size // known if known else 0
    else:
        d = [int(v) for v in A(dims[0]).reshape(-1)]
    if int(np.prod(d)) != a.size:
        raise MatlabError("reshape: number of elements must not change")
    return np.asfortranarray(trim(a.reshape(d, order="F")))


def b_find(x, k=None):
    a = A(x)
    idx = np.nonzero(a.reshape(-1, order="F") != 0)[0] + 1.0
    if k is not None:
        idx = idx[: int(scalar(k))]
    if a.shape[0] == 1 and a.ndim == 2:
        return idx.reshape(1, -1)
    return idx.reshape(-1, 1)


def b_find_n(x, k=None, direction=None):
    if direction is None or str(direction) == "first":
        return b_find(x, k)
    a = A(x)
    idx = np.nonzero(a.reshape(-1, order="F") != 0)[0] + 1.0
    idx = idx[-int(scalar(k)):] if k is not None else idx
    if a.shape[0] == 1 and a.ndim == 2:
        return idx.reshape(1, -1)
    return idx.reshape(-1, 1)


def b_max(x, *rest):
    """max of a vector: [value, first index of the maximum]; max(a, b) elementwise."""
    if len(rest) == 1:
        return elementwise(np.fmax, A(x), A(rest[0]))
    if rest:
        raise MatlabError("max with more than two arguments")
    v = A(x).reshape(-1, order="F")
    i = int(np.argmax(v))
    return [A(v[i]), A(float(i + 1))]


def b_sum(x):
    a = A(x)
    if a.ndim == 2 and (a.shape[0] == 1 or a.shape[1] == 1):
        acc = a.dtype.type(0) if a.dtype != bool else 0.0
        for v in a.reshape(-1, order="F"):
            acc = acc + v
        return A(acc)
    return np.asfortranarray(A(np.sum(a, axis=0, keepdims=True)))


def b_diff(x):
    a = A(x)
    if a.ndim == 2 and a.shape[0] == 1:
        return np.asfortranarray(a[:, 1:] - a[:, :-1])
    return np.asfortranarray(a[1:] - a[:-1])


def b_trapz(y):
    """trapz(Y) of a vector: trapezoidal rule with unit spacing."""
    v = A(y).reshape(-1, order="F")
    acc = 0.0
    for i in range(v.size - 1):
        acc = acc + (v[i] + v[i + 1]) / 2.0
    return A(acc)


def b_xcorr(x, y):
    """xcorr(x, y) of two real vectors of length N: R(m) = sum_n x(n+m) y(n)
    for lags m = -(N-1) .. N-1 (a row for row inputs), a direct sum in
    ascending n."""
    xv = A(x).reshape(-1, order="F")
    yv = A(y).reshape(-1, order="F")
    n = xv.size
    if yv.size != n:
        raise MatlabError("xcorr of vectors of different lengths")
    out = np.zeros(2 * n - 1)
    for m in range(-(n - 1), n):
        acc = 0.0
        for j in range(max(0, -m), min(n, n - m)):
            acc = acc + xv[j + m] * yv[j]
        out[m + n - 1] = acc
    row = A(x).shape[0] == 1
    return np.asfortranarray(out.reshape(1, -1) if row else out.reshape(-1, 1))


def b_hann(n):
    """Symmetric Hann window (column): 0.5*(1 - cos(2*pi*k/(N-1))), k = 0..N-1."""
    N = int(scalar(n))
    if N == 1:
        return A(1.0)
    k = np.arange(N, dtype=np.float64)
    return np.asfortranarray((0.5 * (1.0 - np.cos(2.0 * np.pi * k / (N - 1)))).reshape(-1, 1))


def b_min(x, *rest):
    if len(rest) == 1:  # min(a, b): elementwise, NaN ignored as in MATLAB
        return elementwise(np.fmin, A(x), A(rest[0]))
    if rest:
        raise MatlabError("min with more than two arguments")
    a = A(x)
    v = a.reshape(-1, order="F")
    if a.ndim == 2 and (a.shape[0] == 1 or a.shape[1] == 1):
        return A(np.min(v)) if v.size else np.zeros((0, 0))
    return np.asfortranarray(A(np.min(a, axis=0)))


def b_mod(x, y):
    return elementwise(lambda a, b: a - np.floor(a / b) * b, A(x), A(y))


def b_squeeze(x):
    a = A(x)
    if a.ndim <= 2:
        return a
    sh = [s for s in a.shape if s != 1]
    while len(sh) < 2:
        sh.append(1)
    if len(sh) == 2 and (a.shape[0] == 1 and a.shape[1] == 1):
        sh = [sh[0], sh[1]] if sh[0] != 1 else [sh[1], sh[0]]
    return np.asfortranarray(a.reshape(sh, order="F"))


def b_meshgrid(x, y):
    xv = A(x).reshape(-1, order="F")
    yv = A(y).reshape(-1, order="F")
    X, Y = np.meshgrid(xv, yv)
    return [np.asfortranarray(X), np.asfortranarray(Y)]


def b_length(x):
    a = A(x)
    return A(float(max(a.shape)) if a.size else 0.0)


def b_ismember(a, b, mode=None):
    """ismember(A, B, 'rows'): which rows of A occur among the rows of B."""
    if mode is None or str(mode) != "rows":
        raise MatlabError("ismember: only the 'rows' form is supported")
    a2, b2 = A(a), A(b)
    a2 = a2.reshape(a2.shape[0], -1, order="F")
    b2 = b2.reshape(b2.shape[0], -1, order="F")
    hit = np.array([[float(any(np.array_equal(r, q) for q in b2))] for r in a2])
    return np.asfortranarray(hit.reshape(-1, 1))


BUILTINS: Dict[str, Callable] = {
    "zeros": b_zeros, "ones": b_ones, "size": b_size, "length": lambda x: b_length(x),
    "reshape": b_reshape, "min": b_min, "mod": b_mod, "squeeze": b_squeeze,
    "meshgrid": b_meshgrid,
    "abs": lambda x: np.asfortranarray(np.abs(A(x))),
    "exp": lambda x: np.asfortranarray(np.exp(to_float(A(x)))),
    "sqrt": lambda x: np.asfortranarray(np.sqrt(to_float(A(x)))),
    "floor": lambda x: np.asfortranarray(np.floor(A(x))),
    "conj": lambda x: np.asfortranarray(np.conj(A(x))),
    "real": lambda x: np.asfortranarray(np.real(A(x)).copy()),
    "single": lambda x: np.asfortranarray(A(x).astype(np.complex64 if np.iscomplexobj(A(x)) else np.float32)),
    "double": lambda x: np.asfortranarray(A(x).astype(np.complex128 if np.iscomplexobj(A(x)) else np.float64)),
    "isempty": lambda x: A(A(x).size == 0),
    "isscalar": lambda x: A(A(x).size == 1),
    "all": lambda x: A(bool(np.all(A(x) != 0))),
    "numel": lambda x: A(float(len(x) if isinstance(x, list) else 1 if isinstance(x, dict) else A(x).size)),
    "pi": lambda: A(np.pi),
    "complex": lambda x, y=None: np.asfortranarray(A(x).astype(np.complex128) + (0 if y is None else 1j * A(y))),
    "num2str": lambda x: str(int(scalar(x))) if float(scalar(x)).is_integer() else repr(float(scalar(x))),
    "ismember": b_ismember,
    "repmat": lambda x, m, n=None: np.asfortranarray(np.tile(A(x), (int(scalar(m)), int(scalar(m if n is None else n))))),
    "true": lambda: A(1.0),
    "false": lambda: A(0.0),
    "isfield": lambda st, name: A(isinstance(st, dict) and str(name) in st),
    "norm": lambda x: A(float(np.linalg.norm(A(x).ravel()))),
    "fopen": lambda *a: A(1.0),
    "fclose": lambda *a: A(0.0),
    "disp": lambda *a: [],
    "eps": lambda: A(np.finfo(np.float64).eps),
    "log": lambda x: np.asfortranarray(np.log(to_float(A(x)))),
    "cos": lambda x: np.asfortranarray(np.cos(to_float(A(x)))),
    "atan": lambda x: np.asfortranarray(np.arctan(to_float(A(x)))),
    "isnan": lambda x: np.asfortranarray(np.isnan(A(x))),
    "fliplr": lambda x: np.asfortranarray(A(x)[:, ::-1]),
    "strcmp": lambda a, b: A(isinstance(a, str) and isinstance(b, str) and a == b),
    "fprintf": lambda *a: [],
    "error": lambda *a: (_ for _ in ()).throw(MatlabError(str(a[0]) if a else "error")),
    "find": b_find_n, "max": b_max, "xcorr": b_xcorr, "sum": b_sum, "diff": b_diff, "trapz": b_trapz, "hann": b_hann,
    "floor_": None,
}
del BUILTINS["floor_"]


# ---------------------------------------------------------------------------
# interpreter
# ---------------------------------------------------------------------------
class _Return(Exception):
    pass


class _Break(Exception):
    pass


class Interpreter:
    def __init__(self, search_paths: List[str], overrides: Optional[Dict[str, Callable]] = None):
        self.paths = search_paths
        self.overrides = dict(overrides or {})
        self.cache: Dict[str, tuple] = {}

    def find_function(self, name):
        if name in self.cache:
            return self.cache[name]
        for p in self.paths:
            f = os.path.join(p, name + ".m")
            if os.path.exists(f):
                funcs = Parser(tokenize(open(f).read())).parse_file()
                for fn in funcs:
                    self.cache.setdefault(fn[1], fn)
                if name in self.cache:
                    return self.cache[name]
        return None

    def call(self, name, args, nargout=1):
        if name in self.overrides:
            r = self.overrides[name](*args)
            return r if isinstance(r, list) else [r]
        fn = self.find_function(name)
        if fn is not None:
            return self.run_function(fn, args, nargout)
        if name == "size" and nargout > 1 and len(args) == 1:
            # [n1, n2, ...] = size(A): one output per dimension, the last one
            # the product of the remaining dimensions
            sh = list(A(args[0]).shape)
            while len(sh) < nargout:
                sh.append(1)
            out = sh[:nargout - 1] + [int(np.prod(sh[nargout - 1:]))]
            return [A(float(d)) for d in out]
        if name == "find" and nargout == 2 and len(args) in (1, 2, 3):
            # [row, col] = find(A[, k[, 'first'|'last']]): 1-based subscripts of
            # the nonzeros, column-major order, the first (or last) k of them
            a = A(args[0])
            a = a.reshape(a.shape[0], -1, order="F")
            lin = np.nonzero(a.reshape(-1, order="F") != 0)[0]
            if len(args) > 1:
                k = int(scalar(args[1]))
                lin = lin[-k:] if len(args) > 2 and str(args[2]) == "last" else lin[:k]
            r, c = lin % a.shape[0] + 1.0, lin // a.shape[0] + 1.0
            return [r.reshape(-1, 1), c.reshape(-1, 1)]
        if name in BUILTINS:
            r = BUILTINS[name](*args)
            return r if isinstance(r, list) else [r]
        raise MatlabError(f"undefined function {name}")

    def run_function(self, fn, args, nargout):
        _, name, params, outs, body = fn
        env: Dict[str, Any] = {"nargin": A(float(len(args)))}
        for p, a in zip(params, args):
            if p != "~":
                env[p] = a
        try:
            self.exec_block(body, env)
        except _Return:
            pass
        res = []
        for o in outs[: max(nargout, 1)]:
            if o not in env:
                if len(res) < nargout:
                    raise MatlabError(f"{name}: output {o} not assigned")
                break
            res.append(env[o])
        return res

    # -- statements ---------------------------------------------------------------
    def exec_block(self, stmts, env):
        for s in stmts:
            self.exec_stmt(s, env)

    def exec_stmt(self, s, env):
        kind = s[0]
        if kind == "assign":
            self.assign(s[1], self.eval(s[2], env), env)
        elif kind == "massign":
            targets, rhs = s[1], s[2]
            if len(targets) == 1 and (rhs[0] != "call" or rhs[1][0] != "id" or rhs[1][1] in env):
                # [a] = expression
                if targets[0] is not None:
                    self.assign(targets[0], self.eval(rhs, env), env)
                return
            if rhs[0] != "call" or rhs[1][0] != "id":
                raise MatlabError(f"multiple assignment needs a function call: {rhs!r:.200}")
            args = [self.eval_arg(a, env) for a in rhs[2]]
            vals = self.call(rhs[1][1], args, nargout=len(targets))
            for t, v in zip(targets, vals):
                if t is not None:
                    self.assign(t, v, env)
        elif kind == "expr":
            self.eval(s[1], env, nargout=0)
        elif kind == "for":
            rng = A(self.eval(s[2], env))
            cols = rng.reshape(rng.shape[0], -1, order="F")
            for j in range(cols.shape[1]):
                env[s[1]] = np.asfortranarray(cols[:, j:j + 1])
                try:
                    self.exec_block(s[3], env)
                except _Break:
                    break
        elif kind == "while":
            while truth(self.eval(s[1], env)):
                try:
                    self.exec_block(s[2], env)
                except _Break:
                    break
        elif kind == "if":
            for cond, body in s[1]:
                if truth(self.eval(cond, env)):
                    self.exec_block(body, env)
                    return
            if s[2] is not None:
                self.exec_block(s[2], env)
        elif kind == "return":
            raise _Return()
        elif kind == "break":
            raise _Break()
        else:
            raise MatlabError(f"statement {kind}")

    def assign(self, target, value, env):
        if target[0] == "id":
            env[target[1]] = value
            return
        if target[0] == "call" and target[1][0] == "id":
            name = target[1][1]
            base = env.get(name)
            subs = [self.eval_sub(a, env, base, d, len(target[2])) for d, a in enumerate(target[2])]
            env[name] = massign_into(base, subs, value)
            return
        if target[0] == "call" and target[1][0] == "field":
            # s.a(i) = v: assign into the field's value, then store it back
            base = self.eval(target[1], env)
            subs = [self.eval_sub(a, env, base, d, len(target[2])) for d, a in enumerate(target[2])]
            self.assign(target[1], massign_into(base, subs, value), env)
            return
        if target[0] == "field":
            # s.a.b = v on scalar structs (dicts), created as needed
            path, t = [], target
            while t[0] == "field":
                path.append(t[2])
                t = t[1]
            if t[0] != "id":
                raise MatlabError("unsupported struct assignment target")
            node = env.get(t[1])
            if not isinstance(node, dict):
                node = env[t[1]] = {}
            for name in reversed(path[1:]):
                if not isinstance(node.get(name), dict):
                    node[name] = {}
                node = node[name]
            node[path[0]] = value
            return
        raise MatlabError("unsupported assignment target")

    # -- expressions --------------------------------------------------------------
    def eval_arg(self, e, env):
        return self.eval(e, env)

    def eval_sub(self, e, env, base, d, k):
        if e[0] == "colon_all":
            return COLON_ALL
        self._end_stack.append((base, d, k))
        try:
            return self.eval(e, env)
        finally:
            self._end_stack.pop()

    _end_stack: List = []  # (base, dim, n_subscripts) of the subscripts being evaluated

    def eval(self, e, env, nargout=1):
        kind = e[0]
        if kind == "num":
            return A(e[1])
        if kind == "str":
            return e[1]
        if kind == "paren":
            return self.eval(e[1], env)
        if kind == "id":
            name = e[1]
            if name in env:
                return env[name]
            r = self.call(name, [], nargout=max(nargout, 1))
            return r[0] if r else None
        if kind == "field":
            v = self.eval(e[1], env)
            if not isinstance(v, dict) or e[2] not in v:
                raise MatlabError(f"reference to non-existent field {e[2]}")
            return v[e[2]]
        if kind == "end":
            base, d, k = self._end_stack[-1]
            if isinstance(base, list):  # struct array
                return A(float(len(base)))
            a = A(base)
            if k == 1:
                return A(float(a.size))
            sh = effective_shape(a, k)
            return A(float(sh[d]))
        if kind == "un":
            v = A(self.eval(e[2], env))
            if e[1] == "-":
                return np.asfortranarray(-to_float(v))
            if e[1] == "+":
                return v
            return np.asfortranarray(A(v == 0))
        if kind == "bin":
            return binop(e[1], self.eval(e[2], env), self.eval(e[3], env))
        if kind == "&&":
            return A(truth(self.eval(e[1], env)) and truth(self.eval(e[2], env)))
        if kind == "||":
            return A(truth(self.eval(e[1], env)) or truth(self.eval(e[2], env)))
        if kind == "transpose":
            v = A(self.eval(e[2], env))
            if v.ndim != 2:
                raise MatlabError("transpose of N-D array")
            r = v.T if e[1] == ".'" else np.conj(v.T)
            return np.asfortranarray(r)
        if kind == "range":
            a = scalar(self.eval(e[1], env))
            d = 1.0 if e[2] is None else scalar(self.eval(e[2], env))
            b = scalar(self.eval(e[3], env))
            return colon(float(np.real(a)), float(np.real(d)), float(np.real(b)))
        if kind == "colon_all":
            return COLON_ALL
        if kind == "matrix":
            if len(e[1]) == 1:
                parts = [self.eval(x, env) for x in e[1][0]]
                if parts and all(isinstance(p, str) for p in parts):
                    return "".join(parts)  # ['abc' num2str(i) '.mat']
            rows = []
            for r in e[1]:
                vals = [A(self.eval(x, env)) for x in r]
                vals = [v for v in vals if v.size]
                rows.append(np.concatenate(vals, axis=1) if vals else np.zeros((0, 0)))
            rows = [r for r in rows if r.size]
            if not rows:
                return np.zeros((0, 0))
            return np.asfortranarray(np.concatenate(rows, axis=0))
        if kind == "call":
            f = e[1]
            if f[0] == "id" and f[1] in env:
                base = env[f[1]]
                subs = [self.eval_sub(a, env, base, d, len(e[2])) for d, a in enumerate(e[2])]
                return mread(base, subs)
            if f[0] == "field":
                base = self.eval(f, env)
                if isinstance(base, list):  # struct array (list of dicts), one 1-based index
                    self._end_stack.append((base, 0, 1))
                    try:
                        k = int(scalar(self.eval(e[2][0], env)))
                    finally:
                        self._end_stack.pop()
                    return base[k - 1]
            if f[0] == "id":
                args = [self.eval(a, env) for a in e[2]]
                r = self.call(f[1], args, nargout=max(nargout, 1))
                return r[0] if r else None
            base = self.eval(f, env)
            subs = [self.eval_sub(a, env, base, d, len(e[2])) for d, a in enumerate(e[2])]
            return mread(base, subs)
        raise MatlabError(f"expression {kind}")
