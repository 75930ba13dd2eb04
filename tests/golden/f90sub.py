"""Runs a subset of Fortran 90 by translating it to Python: enough of the
language for the hot-path files of SuLi-IC (module globals, subroutines with
explicit-shape and assumed-shape array arguments, DO / DO WHILE / IF blocks,
array sections and whole-array assignments, the numeric intrinsics), so that
the reference's own routines can be executed in this container, which has no
Fortran compiler, to produce golden vectors for the oracle.

Semantics follow gfortran with the reference's flags (-fdefault-real-8
-fdefault-double-8, no fast-math): every REAL is IEEE binary64, expressions
evaluate left to right with Fortran precedence, integer division truncates
toward zero, x**2 is x*x (GCC folds pow(x, 2.0) that way), other powers and
the transcendental functions call the C library through Python's math
module (glibc, as gfortran does).  Arguments pass by reference: arrays as
views of the caller's storage (explicit-shape dummies by sequence
association), sections and expressions through temporaries, scalars by
copy-in/copy-out.  OpenMP directives are comments (the serial semantics).
Unformatted WRITEs are kept in memory as gfortran's records (FILES);
formatted I/O and character data are dropped.  Every subscript is checked
against its declared bounds (FBounds): an access outside them touches
memory the Fortran does not define, so no result may rest on it.  Routines
outside the subset become call-time errors.

This is test infrastructure: it reads the reference's sources where they
lie and is never part of the product.
"""
from __future__ import annotations

import keyword
import math
import re

import numpy as np

np.seterr(all="ignore")


# ---------------------------------------------------------------------------
# runtime
class FStop(Exception):
    pass


class FArr:
    """A Fortran array: F-ordered numpy storage and per-dimension lower bounds."""
    __slots__ = ("d", "l")

    def __init__(self, d, lbounds):
        self.d = d
        self.l = tuple(int(x) for x in lbounds)

    @staticmethod
    def alloc(bounds, kind):
        lb = [b[0] for b in bounds]
        ext = [max(0, int(b[1]) - int(b[0]) + 1) for b in bounds]
        dt = {"i": np.int64, "l": np.bool_}.get(kind, np.float64)
        return FArr(np.zeros(ext, dtype=dt, order="F"), lb)


def _as_view(actual, bounds, offset=0):
    """An explicit-shape dummy over the caller's storage (sequence
    association): `bounds` = [(lb, ub), ...], starting `offset` elements into
    the actual's column-major storage."""
    ext = [max(0, int(ub) - int(lb) + 1) for lb, ub in bounds]
    n = int(np.prod(ext)) if ext else 1
    if not actual.d.flags.f_contiguous:
        raise RuntimeError("non-contiguous actual argument for an explicit-shape dummy")
    flat = actual.d.reshape(-1, order="F")
    if offset + n > flat.size:
        # a dummy declared longer than its actual (the Fortran reads past
        # it only if the routine indexes there): a copy padded with NaN, so
        # such a read shows in the results; meant for intent(in) dummies
        pad = np.full(offset + n, np.nan if flat.dtype.kind == "f" else 0, dtype=flat.dtype)
        pad[:flat.size] = flat
        flat = pad
    return FArr(flat[offset:offset + n].reshape(ext, order="F"), [b[0] for b in bounds])


class FBounds(IndexError):
    pass


# Reads outside an array that a caller chooses to resolve: array name ->
# function(index tuple) -> in-bounds index tuple.  Empty by default; a
# golden case that sets one says which undefined read it replaces and by
# what (the oracle's documented choice).
OOB_READS = {}


def _ix(arr, name, idx):
    out = []
    for q, i in enumerate(idx):
        z = int(i) - arr.l[q]
        if (z < 0 or z >= arr.d.shape[q]) and name in OOB_READS:
            return _ix(arr, name + " (resolved)", OOB_READS[name](tuple(int(x) for x in idx)))
        if z < 0 or z >= arr.d.shape[q]:
            raise FBounds("%s%r outside its bounds (lower %r, extents %r)" % (name, tuple(int(x) for x in idx),
                                                                             arr.l, arr.d.shape))
        out.append(z)
    return tuple(out)


def _ix1(arr, name, q, i):
    z = int(i) - arr.l[q]
    if z < 0 or z >= arr.d.shape[q]:
        raise FBounds("%s: subscript %d = %d outside %d..%d" % (name, q + 1, int(i), arr.l[q],
                                                                arr.l[q] + arr.d.shape[q] - 1))
    return z


def _sl(arr, name, q, lo, hi, st):
    a = arr.l[q] if lo is None else int(lo)
    b = arr.l[q] + arr.d.shape[q] - 1 if hi is None else int(hi)
    step = 1 if st is None else int(st)
    if (b - a) * step >= 0:             # a non-empty section: both ends inside
        for v in (a, b):
            if v < arr.l[q] or v > arr.l[q] + arr.d.shape[q] - 1:
                raise FBounds("%s: section %d:%d of dimension %d outside %d..%d" % (
                    name, a, b, q + 1, arr.l[q], arr.l[q] + arr.d.shape[q] - 1))
    stop = b - arr.l[q] + (1 if step > 0 else -1)
    return slice(a - arr.l[q], stop if stop >= 0 else None, step)


def _elem_offset(arr, idx):
    off, mul = 0, 1
    for q, i in enumerate(idx):
        off += (int(i) - arr.l[q]) * mul
        mul *= arr.d.shape[q]
    return off


def _idiv(a, b):
    q = abs(a) // abs(b)
    return q if (a >= 0) == (b >= 0) else -q


def _ipow(x, n):
    if n < 0:
        return 1.0 / _ipow(x, -n)
    if n == 0:
        return type(x)(1)
    r = None
    base = x
    while n:
        if n & 1:
            r = base if r is None else r * base
        n >>= 1
        if n:
            base = base * base
    return r


def _libm(fn, npfn):
    """A C-library function on a scalar (glibc through Python's math module,
    as gfortran calls it), NumPy's value where math raises (NaN, inf); on an
    array element by element the same way (NumPy's own vectorised versions
    may differ from glibc in the last place)."""
    def one(*xs):
        try:
            return np.float64(fn(*[float(x) for x in xs]))
        except (ValueError, OverflowError, ZeroDivisionError):
            return np.float64(npfn(*[np.float64(x) for x in xs]))

    def f(*xs):
        if any(isinstance(x, np.ndarray) for x in xs):
            return np.vectorize(one, otypes=[np.float64])(*xs)
        return one(*xs)
    return f


_pow = _libm(math.pow, np.power)


def _rpow(x, y):
    if not isinstance(y, np.ndarray) and float(y) == 2.0:
        return x * x
    return _pow(x, y)


def _m1(fn, npfn):
    return _libm(fn, npfn)


def _sign(a, b):
    if isinstance(a, (int, np.integer)) and isinstance(b, (int, np.integer)):
        return abs(a) if b >= 0 else -abs(a)
    return np.float64(math.copysign(abs(float(a)), float(b)))


def _mod(a, b):
    if isinstance(a, (int, np.integer)) and isinstance(b, (int, np.integer)):
        return int(a) - _idiv(int(a), int(b)) * int(b)
    return np.float64(math.fmod(float(a), float(b)))


def _nint(x):
    x = float(x)
    return int(math.floor(abs(x) + 0.5)) * (1 if x >= 0 else -1)


def _fsum(x):
    """SUM in array-element order, one addition after another."""
    a = np.asarray(x)
    s = np.float64(0.0) if a.dtype.kind == "f" else 0
    for v in a.ravel(order="F"):
        s = s + v
    return s


def _max(*a):
    if any(isinstance(x, np.ndarray) for x in a):
        r = a[0]
        for x in a[1:]:
            r = np.maximum(r, x)
        return r
    r = a[0]
    for x in a[1:]:
        if x > r:
            r = x
    return r


def _min(*a):
    if any(isinstance(x, np.ndarray) for x in a):
        r = a[0]
        for x in a[1:]:
            r = np.minimum(r, x)
        return r
    r = a[0]
    for x in a[1:]:
        if x < r:
            r = x
    return r


def _real(x):
    if isinstance(x, np.ndarray):
        return x.astype(np.float64)
    return np.float64(x)


def _int(x):
    if isinstance(x, np.ndarray):
        return np.trunc(x).astype(np.int64)
    return int(x)


def _abs(x):
    return np.abs(x) if isinstance(x, np.ndarray) else abs(x)


def _sqrt(x):
    return np.sqrt(x) if isinstance(x, np.ndarray) else np.sqrt(np.float64(x))


def _real4(x):
    if isinstance(x, np.ndarray):
        return x.astype(np.float32)
    return np.float32(x)


# unformatted sequential files, kept in memory: unit -> list of records
FILES = {}


def _fopen(unit):
    FILES[int(unit)] = []


def _fclose(unit):
    pass


def _fwrite(unit, items):
    data = b""
    for x in items:
        a = np.asarray(x)
        if a.dtype.kind == "i":
            a = a.astype(np.int32)     # default INTEGER is 4 bytes
        data += a.ravel(order="F").tobytes()
    n = len(data).to_bytes(4, "little", signed=True)
    FILES.setdefault(int(unit), []).append(n + data + n)


def _random_number(*_a):
    raise RuntimeError("random_number is outside the subset (no reference RNG stream to match)")


RUNTIME = {
    "np": np, "math": math, "FArr": FArr, "FStop": FStop, "_as_view": _as_view, "_elem_offset": _elem_offset,
    "_idiv": _idiv, "_ipow": _ipow, "_rpow": _rpow, "_sign": _sign, "_mod": _mod, "_nint": _nint,
    "_fsum": _fsum, "_max": _max, "_min": _min, "_real": _real, "_int": _int, "_abs": _abs, "_sqrt": _sqrt,
    "_exp": _m1(math.exp, np.exp), "_log": _m1(math.log, np.log), "_log10": _m1(math.log10, np.log10),
    "_sin": _m1(math.sin, np.sin), "_cos": _m1(math.cos, np.cos), "_tan": _m1(math.tan, np.tan),
    "_asin": _m1(math.asin, np.arcsin), "_acos": _m1(math.acos, np.arccos), "_atan": _m1(math.atan, np.arctan),
    "_sinh": _m1(math.sinh, np.sinh), "_cosh": _m1(math.cosh, np.cosh), "_tanh": _m1(math.tanh, np.tanh),
    "_atan2": lambda a, b: np.float64(math.atan2(float(a), float(b))),
    "_floor": lambda x: int(math.floor(float(x))), "_ceiling": lambda x: int(math.ceil(float(x))),
    "_random_number": _random_number, "_ix": _ix, "_ix1": _ix1, "_sl": _sl, "FBounds": FBounds, "_real4": _real4, "_fopen": _fopen, "_fclose": _fclose, "_fwrite": _fwrite,
    "FILES": FILES,
}

PYRESERVED = {"np", "math", "M", "FArr", "FStop", "print", "exec", "eval", "range", "int", "float", "abs", "max", "min", "len", "type", "object", "sum"}

INTRINSIC = {
    "abs": ("_abs", None), "dabs": ("_abs", None), "sqrt": ("_sqrt", "r"), "dsqrt": ("_sqrt", "r"),
    "exp": ("_exp", "r"), "log": ("_log", "r"), "log10": ("_log10", "r"), "sin": ("_sin", "r"),
    "cos": ("_cos", "r"), "tan": ("_tan", "r"), "asin": ("_asin", "r"), "acos": ("_acos", "r"),
    "atan": ("_atan", "r"), "sinh": ("_sinh", "r"), "cosh": ("_cosh", "r"), "tanh": ("_tanh", "r"),
    "atan2": ("_atan2", "r"), "datan": ("_atan", "r"), "dexp": ("_exp", "r"), "dlog": ("_log", "r"),
    "sign": ("_sign", None), "mod": ("_mod", None), "nint": ("_nint", "i"), "int": ("_int", "i"),
    "floor": ("_floor", "i"), "ceiling": ("_ceiling", "i"), "real": ("_real", "r"), "dble": ("_real", "r"),
    "float": ("_real", "r"), "max": ("_max", None), "min": ("_min", None), "amax1": ("_max", "r"),
    "amin1": ("_min", "r"), "dmax1": ("_max", "r"), "dmin1": ("_min", "r"),
    "sum": ("_fsum", None), "maxval": ("np.max", None), "minval": ("np.min", None),
}


# ---------------------------------------------------------------------------
# source handling
def _strip_comment(line):
    out, q = [], None
    for ch in line:
        if q:
            out.append(ch)
            if ch == q:
                q = None
        elif ch in "'\"":
            q = ch
            out.append(ch)
        elif ch == "!":
            break
        else:
            out.append(ch)
    return "".join(out)


def _lower_code(s):
    out, q = [], None
    for ch in s:
        if q:
            out.append(ch)
            if ch == q:
                q = None
        elif ch in "'\"":
            q = ch
            out.append(ch)
        else:
            out.append(ch.lower())
    return "".join(out)


def _split_semicolons(s):
    out, cur, q = [], [], None
    for ch in s:
        if q:
            cur.append(ch)
            if ch == q:
                q = None
        elif ch in "'\"":
            q = ch
            cur.append(ch)
        elif ch == ";":
            out.append("".join(cur))
            cur = []
        else:
            cur.append(ch)
    out.append("".join(cur))
    return [x for x in out if x.strip()]


def statements(text):
    """Logical statements (comments stripped, continuations joined, lowercase)
    with the source line number of their first line."""
    lines = text.splitlines()
    out = []
    buf, start = "", 0
    for no, raw in enumerate(lines, 1):
        s = _strip_comment(raw.replace("\t", " ")).rstrip()
        if not s.strip():
            continue
        st = s.strip()
        if buf:
            if st.startswith("&"):
                st = st[1:]
            buf += " " + st
        else:
            buf, start = st, no
        if buf.endswith("&"):
            buf = buf[:-1]
            continue
        for part in _split_semicolons(_lower_code(buf)):
            out.append((start, part.strip()))
        buf = ""
    return out


# ---------------------------------------------------------------------------
# expressions
_TOK = re.compile(r"""
    (?P<num>(\d+\.\d*|\.\d+|\d+)([ed][+-]?\d+)?(_\d+)?)
  | (?P<dop>\.(eq|ne|lt|le|gt|ge|and|or|not|eqv|neqv|true|false)\.)
  | (?P<str>'[^']*'|"[^"]*")
  | (?P<id>[a-z_][a-z0-9_]*)
  | (?P<op>\*\*|==|/=|<=|>=|//|[-+*/(),:<>=%])
  | (?P<ws>\s+)
""", re.X)


def tokenize(s):
    pos, out = 0, []
    while pos < len(s):
        m = _TOK.match(s, pos)
        if not m:
            raise SyntaxError("cannot tokenize %r at %d" % (s, pos))
        pos = m.end()
        k = m.lastgroup
        if k == "ws":
            continue
        v = m.group(k)
        if k == "num":
            # a number glued to a dotted operator: "1.eq.x" -> "1" ".eq."
            mm = re.match(r"(\d+)\.(eq|ne|lt|le|gt|ge|and|or)\.", s[m.start():])
            if mm:
                out.append(("num", mm.group(1)))
                pos = m.start() + len(mm.group(1))
                continue
        out.append((k, v))
    return out


_BIN = {
    ".eqv.": 1, ".neqv.": 1, ".or.": 2, ".and.": 3,
    "==": 5, "/=": 5, "<": 5, "<=": 5, ">": 5, ">=": 5,
    ".eq.": 5, ".ne.": 5, ".lt.": 5, ".le.": 5, ".gt.": 5, ".ge.": 5,
    "+": 6, "-": 6, "*": 7, "/": 7, "**": 9,
}
_PYCMP = {".eq.": "==", ".ne.": "!=", ".lt.": "<", ".le.": "<=", ".gt.": ">", ".ge.": ">=", "==": "==",
          "/=": "!=", "<": "<", "<=": "<=", ">": ">", ">=": ">="}


class Node:
    __slots__ = ("code", "t", "arr", "lit")

    def __init__(self, code, t, arr=False, lit=None):
        self.code, self.t, self.arr, self.lit = code, t, arr, lit


class ExprParser:
    def __init__(self, scope, toks):
        self.s = scope
        self.toks = toks
        self.i = 0

    def peek(self, k=0):
        j = self.i + k
        return self.toks[j] if j < len(self.toks) else (None, None)

    def take(self, v=None):
        t = self.toks[self.i]
        if v is not None and t[1] != v:
            raise SyntaxError("expected %r, got %r" % (v, t))
        self.i += 1
        return t

    def parse(self, minp=0):
        k, v = self.peek()
        if v == ".not.":
            self.take()
            a = self.parse(4)
            left = Node("(not %s)" % a.code, "l")
        elif v in ("-", "+"):
            self.take()
            a = self.parse(8)       # unary minus binds below ** and above * /
            left = Node("(-%s)" % a.code if v == "-" else a.code, a.t, a.arr,
                        (-a.lit if (v == "-" and a.lit is not None) else a.lit))
        else:
            left = self.primary()
        while True:
            k, v = self.peek()
            if v not in _BIN:
                break
            p = _BIN[v]
            if p < minp:
                break
            self.take()
            right = self.parse(p if v == "**" else p + 1)
            left = self.binop(v, left, right)
        return left

    def binop(self, op, a, b):
        arr = a.arr or b.arr
        if op in (".and.", ".or."):
            return Node("(%s %s %s)" % (a.code, op.strip("."), b.code), "l", arr)
        if op in (".eqv.", ".neqv."):
            return Node("(%s %s %s)" % (a.code, "==" if op == ".eqv." else "!=", b.code), "l", arr)
        if op in _PYCMP:
            return Node("(%s %s %s)" % (a.code, _PYCMP[op], b.code), "l", arr)
        t = "i" if (a.t == "i" and b.t == "i") else "r"
        if op == "**":
            if b.t == "i":
                if b.lit is not None and b.lit == 2:
                    return Node("(%s*%s)" % (a.code, a.code), a.t, arr)
                return Node("_ipow(%s, %s)" % (a.code, b.code), a.t, arr)
            return Node("_rpow(%s, %s)" % (a.code, b.code), "r", arr)
        if op == "/" and t == "i":
            return Node("_idiv(%s, %s)" % (a.code, b.code), "i", arr)
        return Node("(%s %s %s)" % (a.code, op, b.code), t, arr)

    def primary(self):
        k, v = self.take()
        if k == "num":
            m = re.match(r"(\d+\.\d*|\.\d+|\d+)([ed]([+-]?\d+))?(_\d+)?$", v)
            mant, exp = m.group(1), m.group(3)
            if "." in mant or m.group(2):
                val = float(mant + ("e" + exp if exp else ""))
                return Node("np.float64(%r)" % val, "r", lit=val)
            return Node(str(int(mant)), "i", lit=int(mant))
        if k == "dop":
            if v == ".true.":
                return Node("True", "l")
            if v == ".false.":
                return Node("False", "l")
            raise SyntaxError(v)
        if k == "str":
            return Node(repr(v[1:-1]), "s")
        if v == "(":
            e = self.parse()
            self.take(")")
            return Node("(%s)" % e.code, e.t, e.arr, e.lit)
        if k == "id":
            if self.peek()[1] == "(":
                return self.call_or_ref(v)
            return self.s.name_ref(v)
        raise SyntaxError("unexpected %r" % v)

    def args(self):
        """Argument / subscript list after '(' (consumed here): entries are
        ('expr', Node) or ('slice', lo, hi, step) or ('kw', name, Node)."""
        self.take("(")
        out = []
        if self.peek()[1] == ")":
            self.take()
            return out
        while True:
            if self.peek()[0] == "id" and self.peek(1)[1] == "=" :
                name = self.take()[1]
                self.take("=")
                out.append(("kw", name, self.parse()))
            else:
                lo = hi = st = None
                if self.peek()[1] != ":":
                    lo = self.parse()
                if self.peek()[1] == ":":
                    self.take()
                    if self.peek()[1] not in (",", ")", ":"):
                        hi = self.parse()
                    if self.peek()[1] == ":":
                        self.take()
                        st = self.parse()
                    out.append(("slice", lo, hi, st))
                else:
                    out.append(("expr", lo))
            if self.peek()[1] == ",":
                self.take()
                continue
            self.take(")")
            return out

    def call_or_ref(self, name):
        var = self.s.lookup(name)
        if var is not None and var.dims is not None:
            subs = self.args()
            return self.s.array_ref(name, var, subs)
        if name in INTRINSIC:
            fn, rt = INTRINSIC[name]
            a = self.args()
            nodes = [x[1] if x[0] == "expr" else x[2] for x in a]
            arr = any(n.arr for n in nodes)
            if name == "real" and len(nodes) == 2:
                if nodes[1].lit != 4:
                    raise SyntaxError("real(x, kind) with kind %r" % nodes[1].lit)
                return Node("_real4(%s)" % nodes[0].code, "r", arr)
            if name in ("sum", "maxval", "minval"):
                t = nodes[0].t
                return Node("%s(%s)" % (fn, nodes[0].code), t, False)
            if rt is None:
                if name in ("abs", "dabs", "sign", "mod"):
                    t = nodes[0].t
                else:   # max, min
                    t = "i" if all(n.t == "i" for n in nodes) else "r"
            else:
                t = rt
            return Node("%s(%s)" % (fn, ", ".join(n.code for n in nodes)), t, arr)
        fn = self.s.unit.prog.functions.get(name)
        if fn is not None:
            a = self.args()
            return Node("F_%s(%s)" % (name, ", ".join(x[1].code for x in a)), fn.rtype, False)
        raise NameError("unknown function or array %r in %s" % (name, self.s.unit.name))


# ---------------------------------------------------------------------------
# declarations and scopes
class Var:
    __slots__ = ("name", "t", "dims", "alloc", "param", "save", "init", "module", "dummy")

    def __init__(self, name, t):
        self.name, self.t = name, t
        self.dims = None        # list of (lo_expr, hi_expr) strings, or ':' entries
        self.alloc = False
        self.param = False
        self.save = False
        self.init = None
        self.module = None
        self.dummy = False


_TYPE_RE = re.compile(r"^(real\s*(\(\s*(kind\s*=\s*)?\d+\s*\))?|double\s+precision|integer\s*(\(\s*\d+\s*\))?|"
                      r"logical|character\s*(\*\s*\d+|\(\s*[^)]*\))?)\s*(,|::|\s)", re.I)


def _split_top(s, sep=","):
    out, depth, cur, q = [], 0, [], None
    for ch in s:
        if q:
            cur.append(ch)
            if ch == q:
                q = None
            continue
        if ch in "'\"":
            q = ch
        elif ch == "(":
            depth += 1
        elif ch == ")":
            depth -= 1
        if ch == sep and depth == 0:
            out.append("".join(cur))
            cur = []
        else:
            cur.append(ch)
    out.append("".join(cur))
    return [x.strip() for x in out]


def parse_decl(stmt):
    """A type declaration -> (type letter, attrs, entities) or None."""
    m = _TYPE_RE.match(stmt + " ")
    if not m:
        return None
    tword = m.group(1).lower()
    t = "r" if (tword.startswith("real") or tword.startswith("double")) else \
        "i" if tword.startswith("integer") else "l" if tword.startswith("logical") else "c"
    rest = stmt[len(m.group(1)):].strip()
    if "::" in rest:
        attrs_s, ents_s = rest.split("::", 1)
        attrs = [a.strip() for a in _split_top(attrs_s.strip().lstrip(","))] if attrs_s.strip() else []
    else:
        attrs, ents_s = [], rest
    attrs = [a for a in attrs if a]
    ents = []
    for e in _split_top(ents_s):
        if not e:
            continue
        init = None
        if "=" in e and not e.startswith("="):
            # name[(dims)] = init  (not '==')
            depth, cut = 0, -1
            for q, ch in enumerate(e):
                if ch == "(":
                    depth += 1
                elif ch == ")":
                    depth -= 1
                elif ch == "=" and depth == 0:
                    cut = q
                    break
            if cut >= 0:
                e, init = e[:cut].strip(), e[cut + 1:].strip()
        mm = re.match(r"([a-z_][a-z0-9_]*)\s*(\*\s*\d+)?\s*(\((.*)\))?$", e)
        if not mm:
            raise SyntaxError("declaration entity %r" % e)
        ents.append((mm.group(1), mm.group(4), init))
    return t, attrs, ents


def parse_dims(s):
    out = []
    for d in _split_top(s):
        if d == ":":
            out.append(":")
        elif ":" in d:
            lo, hi = _split_top(d, ":")
            out.append((lo, hi))
        else:
            out.append(("1", d))
    return out


class Unit:
    """A subroutine (or the module-variable table)."""

    def __init__(self, prog, name, args, kind="subroutine"):
        self.prog = prog
        self.name = name
        self.args = args
        self.kind = kind
        self.vars = {}
        self.body = []          # (line, stmt)
        self.rtype = "r"


class Scope:
    def __init__(self, unit):
        self.unit = unit

    def lookup(self, name):
        v = self.unit.vars.get(name)
        if v is not None:
            return v
        return self.unit.prog.modvars.get(name)

    def pyname(self, name):
        if keyword.iskeyword(name) or name in PYRESERVED:
            raise NameError("Fortran name %r clashes with a Python name" % name)
        v = self.lookup(name)
        if v is None:
            raise NameError("undeclared %r in %s" % (name, self.unit.name))
        if v.module:
            return "M." + name
        if v.save and not v.dummy:
            return "S_%s[%r]" % (self.unit.name, name)
        return name

    def name_ref(self, name):
        v = self.lookup(name)
        if v is None:
            if name in INTRINSIC:
                raise SyntaxError("intrinsic %r without arguments" % name)
            raise NameError("undeclared %r in %s" % (name, self.unit.name))
        py = self.pyname(name)
        if v.dims is not None:
            return Node(py + ".d", v.t, True)
        return Node(py, v.t)

    def array_ref(self, name, var, subs):
        """An element or section reference, bounds-checked: a subscript
        outside the declared bounds reads or writes memory the Fortran does
        not define, which no golden vector may depend on (FBounds)."""
        py = self.pyname(name)
        if all(s[0] == "expr" for s in subs):
            return Node("%s.d[_ix(%s, %r, (%s,))]" % (py, py, name, ", ".join(s[1].code for s in subs)), var.t)
        idx = []
        for q, s in enumerate(subs):
            if s[0] == "expr":
                idx.append("_ix1(%s, %r, %d, %s)" % (py, name, q, s[1].code))
            elif s[0] == "slice":
                _, lo, hi, st = s
                idx.append("_sl(%s, %r, %d, %s, %s, %s)" % (py, name, q, lo.code if lo is not None else "None",
                                                            hi.code if hi is not None else "None",
                                                            st.code if st is not None else "None"))
            else:
                raise SyntaxError("keyword subscript")
        return Node("%s.d[%s]" % (py, ", ".join(idx)), var.t, True)


# ---------------------------------------------------------------------------
# program: parse every file, generate Python
class Program:
    def __init__(self):
        self.modvars = {}
        self.mod_order = []     # (module name, [Var]) in source order
        self.units = {}
        self.functions = {}
        self.ns = None

    # ---- parsing
    def add_source(self, text, fname="?"):
        st = statements(text)
        i = 0
        while i < len(st):
            no, s = st[i]
            m = re.match(r"^module\s+([a-z_][a-z0-9_]*)$", s)
            if m and not s.startswith("module procedure"):
                i = self._module(st, i + 1, m.group(1))
                continue
            m = re.match(r"^(recursive\s+)?subroutine\s+([a-z_][a-z0-9_]*)\s*(\((.*)\))?$", s)
            if m:
                i = self._unit(st, i + 1, m.group(2), m.group(4), "subroutine")
                continue
            m = re.match(r"^((real|integer|logical)[^ ]*\s+)?function\s+([a-z_][a-z0-9_]*)\s*\((.*)\)$", s)
            if m:
                i = self._unit(st, i + 1, m.group(3), m.group(4), "function",
                               rtype=("i" if (m.group(2) or "") == "integer" else "r"))
                continue
            if re.match(r"^program\s+", s):
                # the main program is not run: skip to its end
                while i < len(st) and not re.match(r"^end(\s*program.*)?$", st[i][1]):
                    i += 1
                i += 1
                continue
            i += 1

    def _module(self, st, i, name):
        vars_ = []
        while i < len(st):
            no, s = st[i]
            if re.match(r"^end(\s*module.*)?$", s):
                break
            d = parse_decl(s)
            if d:
                for v in self._vars_from_decl(d):
                    v.module = name
                    self.modvars[v.name] = v
                    vars_.append(v)
            i += 1
        self.mod_order.append((name, vars_))
        return i + 1

    def _vars_from_decl(self, d):
        t, attrs, ents = d
        dims_attr = None
        flags = set()
        for a in attrs:
            m = re.match(r"dimension\s*\((.*)\)$", a)
            if m:
                dims_attr = m.group(1)
            else:
                flags.add(re.sub(r"\s*\(.*\)$", "", a))
        out = []
        for name, dims, init in ents:
            v = Var(name, t)
            ds = dims if dims is not None else dims_attr
            if ds is not None:
                v.dims = parse_dims(ds)
            v.alloc = "allocatable" in flags
            v.param = "parameter" in flags
            v.save = "save" in flags
            v.init = init
            out.append(v)
        return out

    def _unit(self, st, i, name, args, kind, rtype="r"):
        args = [a.strip() for a in (args or "").split(",") if a.strip()]
        u = Unit(self, name, args, kind)
        u.rtype = rtype
        depth = 0
        while i < len(st):
            no, s = st[i]
            if re.match(r"^end\s*(subroutine|function)\b.*$", s) or (s == "end" and depth == 0):
                break
            if s.startswith("use ") or s.startswith("implicit") or s.startswith("interface") or \
                    re.match(r"^\d+\s+format", s) or s.startswith("format"):
                i += 1
                continue
            d = parse_decl(s)
            if d:
                for v in self._vars_from_decl(d):
                    if v.name in u.args:
                        v.dummy = True
                    u.vars[v.name] = v
                i += 1
                continue
            u.body.append((no, s))
            i += 1
        for a in u.args:
            if a not in u.vars:
                u.vars[a] = Var(a, "i" if a[0] in "ijklmn" else "r")
                u.vars[a].dummy = True
        if kind == "function" and name not in u.vars:
            u.vars[name] = Var(name, rtype)
        (self.functions if kind == "function" else self.units)[name] = u
        return i + 1

    # ---- code generation
    def build(self):
        src = ["# generated from Fortran sources", "class _M: pass", "M = _M()"]
        self.untranslated = {}
        for name, u in list(self.units.items()) + list(self.functions.items()):
            try:
                src.append(self._gen_unit(u))
            except (SyntaxError, NameError) as e:
                # outside the subset (character handling, formats, ...): an
                # error if the routine is ever called
                self.untranslated[name] = str(e)
                pre = "F_" if u.kind == "function" else "S_"
                src.append("def %s%s(*_a):\n    raise RuntimeError(%r)" % (pre, name, "%s: %s" % (name, e)))
        code = "\n".join(src)
        ns = dict(RUNTIME)
        exec(compile(code, "<f90sub>", "exec"), ns)
        self.ns = ns
        self.M = ns["M"]
        self._init_modules()
        return self

    def _init_modules(self):
        M = self.M
        mscope = Scope(Unit(self, "<modules>", []))
        for name, vars_ in self.mod_order:
            for v in vars_:
                if v.dims is not None and not v.alloc and all(d != ":" for d in v.dims):
                    bounds = [(self.eval_expr(mscope, lo), self.eval_expr(mscope, hi)) for lo, hi in v.dims]
                    setattr(M, v.name, FArr.alloc(bounds, v.t))
                elif v.dims is not None:
                    setattr(M, v.name, None)
                elif v.init is not None:
                    setattr(M, v.name, self._coerce(v.t, self.eval_expr(mscope, v.init)))
                else:
                    setattr(M, v.name, self._coerce(v.t, 0))

    @staticmethod
    def _coerce(t, x):
        if t == "r":
            return np.float64(x)
        if t == "i":
            return int(x)
        if t == "l":
            return bool(x)
        return x

    def eval_expr(self, scope, s):
        n = ExprParser(scope, tokenize(s)).parse()
        return eval(n.code, self.ns)

    def expr(self, scope, s):
        p = ExprParser(scope, tokenize(s))
        n = p.parse()
        if p.i != len(p.toks):
            raise SyntaxError("trailing tokens in %r" % s)
        return n

    def _conv(self, t, n):
        if t == "r" and n.t != "r":
            return "_real(%s)" % n.code
        if t == "i" and n.t == "r":
            return "_int(%s)" % n.code
        return n.code

    def _gen_unit(self, u):
        sc = Scope(u)
        L = []
        fname = ("F_" if u.kind == "function" else "S_") + u.name
        L.append("%s_saved = {}" % ("S_" + u.name))
        L.append("def %s(%s):" % (fname, ", ".join(u.args)))
        body = []
        # local arrays (automatic or fixed) and scalars
        for v in u.vars.values():
            if v.dummy:
                if v.dims is not None and all(d != ":" for d in v.dims):
                    b = ", ".join("(%s, %s)" % (self.expr(sc, lo).code, self.expr(sc, hi).code) for lo, hi in v.dims)
                    body.append("if isinstance(%s, tuple): %s = _as_view(%s[0], [%s], %s[1])" %
                                (v.name, v.name, v.name, b, v.name))
                    body.append("else: %s = _as_view(%s, [%s])" % (v.name, v.name, b))
                elif v.dims is not None:
                    body.append("if isinstance(%s, tuple): raise RuntimeError('element actual for an assumed-shape dummy')"
                                % v.name)
                    body.append("%s = FArr(%s.d, [1]*%s.d.ndim)" % (v.name, v.name, v.name))
                continue
            if v.save or v.param:
                key = "S_%s[%r]" % (u.name, v.name)
                init = None
                if v.dims is not None and not v.alloc:
                    b = ", ".join("(%s, %s)" % (self.expr(sc, lo).code, self.expr(sc, hi).code) for lo, hi in v.dims)
                    init = "FArr.alloc([%s], %r)" % (b, v.t)
                elif v.dims is None:
                    init = repr(self._coerce(v.t, 0)) if v.init is None else self._conv(v.t, self.expr(sc, v.init))
                    if v.t == "r" and v.init is None:
                        init = "np.float64(0.0)"
                if init is not None:
                    body.append("if %r not in S_%s_saved: S_%s_saved[%r] = %s" % (v.name, u.name, u.name, v.name, init))
                continue
            if v.dims is not None and not v.alloc:
                b = ", ".join("(%s, %s)" % (self.expr(sc, lo).code, self.expr(sc, hi).code) for lo, hi in v.dims)
                body.append("%s = FArr.alloc([%s], %r)" % (v.name, b, v.t))
            elif v.dims is not None:
                body.append("%s = None" % v.name)
            elif v.init is not None:
                body.append("%s = %s" % (v.name, self._conv(v.t, self.expr(sc, v.init))))
            else:
                body.append("%s = %s" % (v.name, "np.float64(0.0)" if v.t == "r" else
                                         ("False" if v.t == "l" else "0")))
        # saved variables are addressed as S_<unit>[name]
        body = [b.replace("S_%s[" % u.name, "S_%s_saved[" % u.name) for b in body]
        scal = [a for a in u.args if u.vars[a].dims is None]
        ret = "return (%s)" % "".join("%s, " % a for a in scal) if u.kind == "subroutine" else "return %s" % u.name
        self._ret = ret
        stmts = self._gen_block(sc, u.body)
        stmts = [x.replace("S_%s[" % u.name, "S_%s_saved[" % u.name) for x in stmts]
        for b in body + stmts:
            L.append("    " + b)
        L.append("    " + ret)
        return "\n".join(_fix_dedents(L))

    # statements -> python lines (with relative indentation)
    def _gen_block(self, sc, body):
        out = []
        ind = 0
        for no, s in body:
            try:
                lines, dind = self._gen_stmt(sc, s)
            except Exception as e:
                raise SyntaxError("%s:%d: %r: %s" % (sc.unit.name, no, s, e)) from e
            for ln in lines:
                out.append("    " * ind + ln)
            ind += dind
            if ind < 0:
                raise SyntaxError("%s:%d: unbalanced block end" % (sc.unit.name, no))
        if ind != 0:
            raise SyntaxError("%s: %d blocks left open" % (sc.unit.name, ind))
        return out

    def _gen_stmt(self, sc, s):
        s = re.sub(r"^\d+\s+", "", s)           # statement label
        # block structure
        m = re.match(r"^(\w+\s*:\s*)?do\s+while\s*\((.*)\)$", s)
        if m:
            c = self.expr(sc, m.group(2))
            return ["while %s:" % c.code], 1
        m = re.match(r"^(\w+\s*:\s*)?do\s+([a-z_][a-z0-9_]*)\s*=\s*(.*)$", s)
        if m:
            var = m.group(2)
            parts = _split_top(m.group(3))
            a, b = self.expr(sc, parts[0]), self.expr(sc, parts[1])
            st = self.expr(sc, parts[2]) if len(parts) > 2 else None
            py = sc.pyname(var)
            if st is None:
                rng = "range(%s, (%s) + 1)" % (a.code, b.code)
            else:
                rng = "range(%s, (%s) + (1 if (%s) > 0 else -1), %s)" % (a.code, b.code, st.code, st.code)
            if "." in py or "[" in py:
                return ["for _lv in %s:" % rng, "    %s = _lv" % py], 1
            return ["for %s in %s:" % (py, rng)], 1
        if re.match(r"^end\s*do$", s):
            return ["pass"], -1
        m = re.match(r"^if\s*\((.*)\)\s*then$", s)
        if m and self._balanced_if(s):
            c = self.expr(sc, m.group(1))
            return ["if %s:" % c.code], 1
        m = re.match(r"^else\s*if\s*\((.*)\)\s*then$", s)
        if m:
            c = self.expr(sc, m.group(1))
            return ["pass", "__DEDENT__elif %s:" % c.code], 0
        if s == "else":
            return ["pass", "__DEDENT__else:"], 0
        if re.match(r"^end\s*if$", s):
            return ["pass"], -1
        if s.startswith("if"):
            cond, rest = self._split_logical_if(s)
            if cond is not None:
                c = self.expr(sc, cond)
                lines, d = self._gen_stmt(sc, rest)
                if d != 0:
                    raise SyntaxError("block statement in a logical IF")
                return ["if %s:" % c.code] + ["    " + x for x in lines], 0
        if s in ("return",):
            return [self._ret], 0
        if s == "exit":
            return ["break"], 0
        if s == "cycle":
            return ["continue"], 0
        if s == "stop" or s.startswith("stop ") or s.startswith("stop'") or s.startswith("stop\""):
            return ["raise FStop(%r)" % s], 0
        if s == "continue":
            return ["pass"], 0
        m = re.match(r"^write\s*\(\s*([a-z_][a-z0-9_]*|\d+)\s*\)\s*(.*)$", s)
        if m:
            # an unformatted record: the items' bytes, gfortran's 4-byte
            # length markers around them (formatted writes are dropped below)
            unit = self.expr(sc, m.group(1)).code
            items = [self.expr(sc, x).code for x in _split_top(m.group(2))] if m.group(2).strip() else []
            return ["_fwrite(%s, [%s])" % (unit, ", ".join(items))], 0
        m = re.match(r"^(open|close)\s*\((.*)\)$", s)
        if m:
            spec = _split_top(m.group(2))
            unit = None
            for x in spec:
                if x.startswith("unit"):
                    unit = x.split("=", 1)[1].strip()
            if unit is None and spec and "=" not in spec[0]:
                unit = spec[0]
            if unit is None:
                return ["pass"], 0
            return ["_f%s(%s)" % (m.group(1), self.expr(sc, unit).code)], 0
        if re.match(r"^(write|print|read|flush|format|rewind|backspace)\b", s):
            return ["pass"], 0
        if s.startswith("call "):
            return self._gen_call(sc, s[5:].strip()), 0
        if s.startswith("allocate"):
            return self._gen_alloc(sc, s), 0
        if s.startswith("deallocate"):
            inner = s[s.index("(") + 1:s.rindex(")")]
            return ["%s = None" % sc.pyname(x.strip()) for x in _split_top(inner) if "=" not in x], 0
        # assignment
        lhs, rhs = self._split_assign(s)
        if lhs is None:
            raise SyntaxError("unsupported statement")
        return [self._gen_assign(sc, lhs, rhs)], 0

    @staticmethod
    def _balanced_if(s):
        # 'if (...) then' where the parenthesis after 'if' closes right before 'then'
        depth = 0
        start = s.index("(")
        for q in range(start, len(s)):
            if s[q] == "(":
                depth += 1
            elif s[q] == ")":
                depth -= 1
                if depth == 0:
                    return s[q + 1:].strip() == "then"
        return False

    @staticmethod
    def _split_logical_if(s):
        m = re.match(r"^if\s*\(", s)
        if not m:
            return None, None
        depth = 0
        for q in range(m.end() - 1, len(s)):
            if s[q] == "(":
                depth += 1
            elif s[q] == ")":
                depth -= 1
                if depth == 0:
                    return s[m.end():q], s[q + 1:].strip()
        return None, None

    @staticmethod
    def _split_assign(s):
        depth, q = 0, None
        for i, ch in enumerate(s):
            if q:
                if ch == q:
                    q = None
                continue
            if ch in "'\"":
                q = ch
            elif ch == "(":
                depth += 1
            elif ch == ")":
                depth -= 1
            elif ch == "=" and depth == 0:
                nxt = s[i + 1:i + 2]
                prv = s[i - 1:i]
                if nxt != "=" and prv not in "<>=/":
                    return s[:i].strip(), s[i + 1:].strip()
        return None, None

    def _gen_assign(self, sc, lhs, rhs):
        mt = re.match(r"^([a-z_][a-z0-9_]*)", lhs)
        vt = sc.lookup(mt.group(1)) if mt else None
        if vt is not None and vt.t == "c":
            return "pass"           # character data (file names): not needed
        r = self.expr(sc, rhs)
        m = re.match(r"^([a-z_][a-z0-9_]*)\s*(\((.*)\))?$", lhs)
        if not m:
            raise SyntaxError("assignment target %r" % lhs)
        name = m.group(1)
        v = sc.lookup(name)
        if v is None:
            raise NameError("undeclared %r" % name)
        py = sc.pyname(name)
        val = self._conv(v.t, r)
        if v.dims is None:
            return "%s = %s" % (py, val)
        if m.group(2) is None:
            return "%s.d[...] = %s" % (py, val)
        p = ExprParser(sc, tokenize(lhs))
        p.take()
        subs = p.args()
        ref = sc.array_ref(name, v, subs)
        return "%s = %s" % (ref.code, val)

    def _gen_alloc(self, sc, s):
        inner = s[s.index("(") + 1:s.rindex(")")]
        out = []
        for item in _split_top(inner):
            if "=" in item.split("(")[0]:
                continue            # stat=
            m = re.match(r"([a-z_][a-z0-9_]*)\s*\((.*)\)$", item)
            name, dims = m.group(1), parse_dims(m.group(2))
            v = sc.lookup(name)
            b = ", ".join("(%s, %s)" % (self.expr(sc, lo).code, self.expr(sc, hi).code) for lo, hi in dims)
            out.append("%s = FArr.alloc([%s], %r)" % (sc.pyname(name), b, v.t))
        return out

    def _gen_call(self, sc, s):
        m = re.match(r"^([a-z_][a-z0-9_]*)\s*(\((.*)\))?$", s)
        name = m.group(1)
        if name.startswith("omp_") or name in ("date_and_time", "cpu_time", "system_clock", "flush"):
            return ["pass"]
        if name == "random_number":
            # a fixed 0.5: the golden cases run random_number only where the
            # amplitude it scales is zero (iturb = 0), so no stream is matched
            a = m.group(3).strip()
            av = sc.lookup(a)
            if av is None:
                raise SyntaxError("random_number(%r)" % a)
            py = sc.pyname(a)
            return ["%s.d[...] = 0.5" % py] if av.dims is not None else ["%s = np.float64(0.5)" % py]
        u = self.units.get(name)
        if u is None:
            return ["raise RuntimeError('call of %s, outside the translated sources')" % name]
        acts = _split_top(m.group(3)) if m.group(3) else []
        if len(acts) != len(u.args):
            # legal Fortran for an external procedure but undefined when run:
            # an error if the call is ever reached
            return ["raise RuntimeError('call of %s with %d arguments for %d dummies')" % (name, len(acts), len(u.args))]
        pre, argcodes, back, post = [], [], [], []
        scal_pos = [q for q, a in enumerate(u.args) if u.vars[a].dims is None]
        for q, a in enumerate(acts):
            dv = u.vars[u.args[q]]
            mm = re.match(r"^([a-z_][a-z0-9_]*)\s*(\((.*)\))?$", a)
            av = sc.lookup(mm.group(1)) if mm else None
            if dv.dims is not None:
                # array dummy: the caller's array, or (element actual) the
                # storage from that element on
                if av is None or av.dims is None:
                    # an array expression: a temporary (copy-in only)
                    n = self.expr(sc, a)
                    if not n.arr:
                        raise SyntaxError("array dummy %s of %s gets %r" % (dv.name, name, a))
                    tmp = "_t%d" % q
                    pre.append("%s_v = %s" % (tmp, n.code))
                    pre.append("%s = FArr(np.array(%s_v, order='F'), [1] * np.ndim(%s_v))" % (tmp, tmp, tmp))
                    argcodes.append(tmp)
                    continue
                if mm.group(2) is None:
                    argcodes.append(sc.pyname(mm.group(1)))
                else:
                    p = ExprParser(sc, tokenize(a))
                    p.take()
                    subs = p.args()
                    if any(x[0] != "expr" for x in subs):
                        # a section: copy-in / copy-out through a temporary
                        ref = sc.array_ref(mm.group(1), av, subs)
                        tmp = "_t%d" % q
                        pre.append("%s = FArr(np.array(%s, order='F'), [1] * np.ndim(%s))" % (tmp, ref.code, ref.code))
                        argcodes.append(tmp)
                        post.append("%s = %s.d" % (ref.code, tmp))
                        continue
                    idx = ", ".join(x[1].code for x in subs)
                    argcodes.append("(%s, _elem_offset(%s, (%s,)))" % (sc.pyname(mm.group(1)), sc.pyname(mm.group(1)), idx))
            else:
                n = self.expr(sc, a)
                argcodes.append(self._conv(dv.t, n))
                if mm and av is not None and not av.param:
                    if mm.group(2) is None and av.dims is None:
                        back.append((scal_pos.index(q), sc.pyname(mm.group(1)), av.t))
                    elif mm.group(2) is not None and av.dims is not None:
                        back.append((scal_pos.index(q), self.expr(sc, a).code, av.t))
        out = pre + ["_r = S_%s(%s)" % (name, ", ".join(argcodes))] + post
        for k, tgt, t in back:
            out.append("%s = %s" % (tgt, "np.float64(_r[%d])" % k if t == "r" else "_r[%d]" % k))
        return out


def _fix_dedents(code_lines):
    """'__DEDENT__' marks an elif/else that closes the block above."""
    out = []
    for ln in code_lines:
        if "__DEDENT__" in ln:
            pre, rest = ln.split("__DEDENT__", 1)
            out.append(pre[:-4] + rest if pre.endswith("    ") else pre + rest)
        else:
            out.append(ln)
    return out



def load(paths):
    """Translate the given Fortran files; returns the Program (its module
    globals in .M, subroutines as .call(name, *args))."""
    p = Program()
    for path in paths:
        with open(path, encoding="utf-8", errors="replace") as f:
            p.add_source(f.read(), path)
    return p.build()


def call(prog, name, *args):
    return prog.ns["S_" + name](*args)
