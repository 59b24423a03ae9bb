"""Executes the reference's own Fortran source by mechanical translation.

TEST INFRASTRUCTURE ONLY.  The reference (peter-reinholdt/fmm) is Fortran and
neither machine of this project has a Fortran compiler, so this module turns
the reference's source files into Python source, statement by statement, and
runs that.  It is used by ``make_ref_golden.py`` (in this directory) to write
golden fixtures; nothing in the product, the GPU tests or the benchmark
imports it, and it only runs where the reference's source is present.

What is translated, and how:
* the free-form subset the reference uses: modules with module variables,
  derived types with default initialisation, pointer and allocatable
  components, subroutines and functions (``result``), recursion,
  ``do``/``do while``/``do concurrent``, ``if``/``select case``,
  ``cycle``/``exit``, ``allocate``/``deallocate``/``nullify``/``move_alloc``,
  pointer assignment, array sections and vector subscripts, array
  constructors, and the intrinsics the source calls;
* integers follow the kinds of the default build (``ip`` = int32): every
  store into an integer variable or array wraps to two's-complement 32 bits,
  so an overflowing expression gives what the reference's gfortran build
  gives in practice (signed overflow is undefined in Fortran; the wrap is the
  hardware's behaviour without optimisations that exploit it);
* ``real(rp)`` is IEEE binary64 (Python floats and numpy float64 arrays);
  literals without a kind are default REAL and are rounded to binary32 first;
  ``SUM`` accumulates in element order; ``NORM2`` uses the scaled sum of
  squares (scale, ssq) that gfortran expands it to; ``MATMUL`` sums over the
  inner index in order;
* preprocessor branches are taken as in the reference's default CMake build
  (``__GNUC__`` defined, no ``VAR_MPI``);
* arrays are column-major numpy arrays with Fortran lower bounds
  (``FA``); sections are numpy views, so a section passed to a dummy argument
  is written through; scalars and allocatable dummies that a procedure may
  change are handed back to the caller and stored into the actual argument
  (copy-in/copy-out, equivalent to reference passing for the reference's
  argument patterns, which never alias two actual arguments);
* intrinsic assignment of a derived-type variable binds the same object
  (the reference only reads the copies it makes, e.g. ``node =
  tree%node_list(i)%node``).
A statement outside this subset raises ``NotImplementedError`` rather than
being guessed at.

Numeric back ends: ``set_mode("float")`` evaluates in binary64 (what the
reference computes, up to the last-bit differences of libm and of
operation order); ``set_mode("mp")`` evaluates the same statements with
mpmath numbers at 50 digits (the exact value of the reference's formulas for
the given binary64 inputs and constants).
"""
import math
import re

import numpy as np

try:
    import mpmath
except ImportError:  # pragma: no cover
    mpmath = None

# ---------------------------------------------------------------------------
# runtime


class FortranStop(RuntimeError):
    pass


_MODE = {"mp": False}


def set_mode(mode):
    if mode not in ("float", "mp"):
        raise ValueError(mode)
    if mode == "mp" and mpmath is None:
        raise RuntimeError("mpmath is not available")
    _MODE["mp"] = mode == "mp"
    if mode == "mp":
        mpmath.mp.dps = 50


_IBITS = {"off": 0x80000000, "mask": 0xFFFFFFFF}


def set_int_bits(bits):
    """Width of integer(ip): 32 (the default build) or 64 (a -DINT64 build)."""
    if bits not in (32, 64):
        raise ValueError(bits)
    _IBITS["off"] = 1 << (bits - 1)
    _IBITS["mask"] = (1 << bits) - 1


def _w32(v):
    v = int(v)
    off = _IBITS["off"]
    return ((v + off) & _IBITS["mask"]) - off


def _w32a(a):
    a = np.asarray(a)
    if a.dtype == object or _IBITS["off"] != 0x80000000:
        return np.array([_w32(t) for t in a.flat], dtype=np.int64).reshape(a.shape)
    a = a.astype(np.int64)
    return ((a + 0x80000000) & 0xFFFFFFFF) - 0x80000000


class _Sl:
    __slots__ = ("lo", "hi", "st")

    def __init__(self, lo, hi, st):
        self.lo, self.hi, self.st = lo, hi, st


def _S(lo=None, hi=None, st=None):
    return _Sl(lo, hi, st)


_ALL = _Sl(None, None, None)


def _item(v):
    if isinstance(v, np.ndarray):
        if v.ndim == 0:
            return v.item() if v.dtype != object else v[()]
        return v
    if isinstance(v, np.generic):
        return v.item()
    return v


class FA:
    """A Fortran array: column-major numpy storage plus lower bounds."""
    __slots__ = ("a", "lb", "i32")

    def __init__(self, a, lb=None, i32=False):
        self.a = a
        self.lb = tuple(lb) if lb is not None else (1,) * a.ndim
        self.i32 = i32
        if len(self.lb) != a.ndim:
            raise ValueError("rank mismatch")

    def _conv(self, idx):
        if type(idx) is not tuple:
            idx = (idx,)
        a, lbs = self.a, self.lb
        if len(idx) != a.ndim:
            raise IndexError("rank %d array indexed with %d subscripts" % (a.ndim, len(idx)))
        out = []
        nvec = 0
        for k, s in enumerate(idx):
            lb = lbs[k]
            t = type(s)
            if t is int:
                i = s - lb
                if i < 0 or i >= a.shape[k]:
                    raise IndexError("subscript %d out of bounds (lb %d, extent %d)" % (s, lb, a.shape[k]))
                out.append(i)
            elif t is _Sl:
                if s.st is not None and s.st < 0:
                    lo = None if s.lo is None else s.lo - lb
                    hi = None if s.hi is None else s.hi - lb - 1
                    if hi is not None and hi < 0:
                        hi = None
                    out.append(slice(lo, hi, s.st))
                else:
                    lo = None if s.lo is None else s.lo - lb
                    hi = None if s.hi is None else s.hi - lb + 1
                    if lo is not None and lo < 0:
                        raise IndexError("section below lower bound")
                    if hi is not None and hi > a.shape[k]:
                        raise IndexError("section above upper bound")
                    if lo is not None and hi is not None and hi < lo:
                        hi = lo
                    out.append(slice(lo, hi, s.st))
            elif t is np.ndarray or t is FA:
                v = s.a if t is FA else s
                v = np.asarray(v, dtype=np.int64) - lb
                if v.size and (v.min() < 0 or v.max() >= a.shape[k]):
                    raise IndexError("vector subscript out of bounds")
                out.append(v)
                nvec += 1
            else:
                i = int(s) - lb
                if i < 0 or i >= a.shape[k]:
                    raise IndexError("subscript %d out of bounds (lb %d, extent %d)" % (int(s), lb, a.shape[k]))
                out.append(i)
        if nvec > 1:
            raise NotImplementedError("more than one vector subscript")
        return tuple(out)

    def __getitem__(self, idx):
        v = self.a[self._conv(idx)]
        if isinstance(v, np.generic):
            return v.item()
        if isinstance(v, np.ndarray) and v.ndim == 0:
            return v.item() if v.dtype != object else v[()]
        return v

    def __setitem__(self, idx, v):
        if isinstance(v, FA):
            v = v.a
        if self.i32:
            v = _w32a(v) if isinstance(v, np.ndarray) else _w32(v)
        self.a[self._conv(idx)] = v


def _val(v):
    """Value of an array operand in an expression."""
    return v.a if isinstance(v, FA) else v


def _dummy(actual, lbs, shape=None):
    """Binds an actual array argument to an array dummy with lower bounds lbs."""
    if actual is None:
        return None
    a = actual.a if isinstance(actual, FA) else actual
    i32 = actual.i32 if isinstance(actual, FA) else False
    if not isinstance(a, np.ndarray):
        a = np.asarray(a)
    if shape is not None:
        shape = tuple(int(s) for s in shape)
        if a.ndim != len(shape):
            if a.size >= int(np.prod(shape)) and a.flags.f_contiguous:
                a = a.reshape(-1, order="F")[: int(np.prod(shape))].reshape(shape, order="F")
            else:
                raise NotImplementedError("sequence association with a non-contiguous actual")
    return FA(a, lbs if len(lbs) == a.ndim else (1,) * a.ndim, i32)


def _asgn(fa, v, kind, lb_default=None):
    """Whole-array assignment (with Fortran 2003 reallocation of allocatables)."""
    if isinstance(v, FA):
        v = v.a
    if fa is not None and (np.ndim(v) == 0 or np.shape(v) == fa.a.shape):
        if fa.i32:
            v = _w32a(v) if isinstance(v, np.ndarray) else _w32(v)
        fa.a[...] = v
        return fa
    arr = np.array(v, order="F", copy=True)
    if arr.ndim == 0:
        raise NotImplementedError("scalar assigned to an unallocated array")
    if kind == "int":
        return FA(_w32a(arr), None, True)
    if kind == "real":
        return FA(np.asfortranarray(arr.astype(np.float64) if arr.dtype != object else arr), None)
    return FA(np.asfortranarray(arr), None)


def _alloc(kind, dims, factory=None, source=None):
    """ALLOCATE of an array: dims is a list of (lb, ub)."""
    shape = tuple(max(0, int(ub) - int(lb) + 1) for lb, ub in dims)
    lbs = tuple(int(lb) for lb, _ in dims)
    if kind == "int":
        a = np.zeros(shape, dtype=np.int64, order="F")
    elif kind == "real":
        a = np.zeros(shape, dtype=object if _MODE["mp"] else np.float64, order="F")
        if _MODE["mp"]:
            a[...] = mpmath.mpf(0)
    elif kind == "log":
        a = np.zeros(shape, dtype=bool, order="F")
    elif kind == "type":
        a = np.empty(shape, dtype=object, order="F")
        for ix in np.ndindex(*shape):
            a[ix] = factory()
    else:
        raise NotImplementedError(kind)
    fa = FA(a, lbs, kind == "int")
    if source is not None:
        fa.a[...] = _w32(source) if kind == "int" else source
    return fa


def _idiv(a, b):
    if isinstance(a, np.ndarray) or isinstance(b, np.ndarray):
        return np.trunc(np.asarray(a) / np.asarray(b)).astype(np.int64)
    a, b = int(a), int(b)
    q = abs(a) // abs(b)
    return q if (a >= 0) == (b >= 0) else -q


def _ipow(a, b):
    a, b = int(a), int(b)
    if b >= 0:
        return a ** b
    if a == 1:
        return 1
    if a == -1:
        return 1 if b % 2 == 0 else -1
    return 0


def _f32(x):
    return float(np.float32(x))


def _streq(a, b):
    return a.rstrip(" ") == b.rstrip(" ")


def _fn_real(x, kind=None):
    if isinstance(x, np.ndarray):
        return x.astype(np.float64) if kind is not None else x.astype(np.float32).astype(np.float64)
    if _MODE["mp"] and mpmath is not None and isinstance(x, mpmath.mpf):
        return x
    return float(x) if kind is not None else _f32(x)


def _elem(fn_float, fn_np, fn_mp):
    def f(x):
        if isinstance(x, FA):
            x = x.a
        if isinstance(x, np.ndarray):
            if x.dtype == object:
                out = np.empty(x.shape, dtype=object)
                for ix in np.ndindex(*x.shape):
                    out[ix] = f(x[ix])
                return out
            return fn_np(x)
        if mpmath is not None and isinstance(x, mpmath.mpf):
            return fn_mp(x)
        if _MODE["mp"]:
            return fn_mp(mpmath.mpf(x))
        return fn_float(x)
    return f


def _np_erf(x):
    from scipy.special import erf
    return erf(x)


_fn_sqrt = _elem(math.sqrt, np.sqrt, lambda v: mpmath.sqrt(v))
_fn_exp = _elem(math.exp, np.exp, lambda v: mpmath.exp(v))
_fn_erf = _elem(math.erf, _np_erf, lambda v: mpmath.erf(v))


def _fn_abs(x):
    if isinstance(x, FA):
        x = x.a
    return np.abs(x) if isinstance(x, np.ndarray) else abs(x)


def _fn_size(x, dim=None):
    a = x.a if isinstance(x, FA) else np.asarray(x)
    return int(a.size) if dim is None else int(a.shape[int(dim) - 1])


def _seqsum(v):
    if v.dtype.kind in "iub":
        return int(v.sum())
    if v.size == 0:
        return 0.0
    if v.dtype != object:
        return float(np.cumsum(v.reshape(-1, order="F"))[-1])  # cumsum adds in element order
    s = mpmath.mpf(0)
    for t in v.flat:
        s = s + t
    return s


def _cut(v, shape):
    """Operand of an array assignment, indexed over the assignment's extent.

    gfortran's scalarizer runs an array assignment over the extent of the
    section being assigned and indexes every operand by the same loop index,
    so a longer whole-array operand contributes its leading elements (the
    reference relies on this: local_to_particle adds dx**k over the whole
    ncrit-long dx to a section of nleaf elements, src/fmm.F90:1117-1118)."""
    if isinstance(v, np.ndarray) and v.ndim == len(shape) and any(a > b for a, b in zip(v.shape, shape)):
        return v[tuple(slice(0, b) for b in shape)]
    return v


def _ptr(v):
    """Target of an array pointer or allocatable dummy: sections get lower bound 1."""
    if v is None or isinstance(v, FA):
        return v
    return FA(np.asarray(v), None, np.asarray(v).dtype.kind == "i")


_LENIENT = {"dealloc": False}


def set_lenient_dealloc(on):
    """With on, DEALLOCATE of an unallocated array is skipped instead of
    stopping the program (to read out what a routine computed before such a
    DEALLOCATE, e.g. the reference's QM/MM helpers, whose `finalize` frees
    interaction lists they never built)."""
    _LENIENT["dealloc"] = bool(on)


def _dealloc(v, what):
    if v is None and not _LENIENT["dealloc"]:
        raise FortranStop("Attempt to DEALLOCATE unallocated '%s'" % what)
    return None


def _fn_sum(x, dim=None):
    a = x.a if isinstance(x, FA) else np.asarray(x)
    if dim is None:
        return _item(_seqsum(np.asarray(a).reshape(-1, order="F")))
    d = int(dim) - 1
    moved = np.moveaxis(a, d, 0)
    out = np.zeros(moved.shape[1:], dtype=a.dtype if a.dtype.kind != "b" else np.int64)
    for ix in np.ndindex(*moved.shape[1:]):
        out[ix] = _seqsum(moved[(slice(None),) + ix])
    return out


def _fn_maxval(x):
    a = x.a if isinstance(x, FA) else x
    return _item(np.max(a))


def _fn_max(*xs):
    return max(xs)


def _fn_norm2(x):
    a = x.a if isinstance(x, FA) else np.asarray(x)
    scale, ssq = 0.0, 1.0
    for v in a.reshape(-1, order="F"):
        v = float(v)
        if v != 0.0:
            ax = abs(v)
            if scale < ax:
                t = scale / ax
                ssq = 1.0 + (ssq * t) * t
                scale = ax
            else:
                t = ax / scale
                ssq = ssq + t * t
    return scale * math.sqrt(ssq)


def _fn_matmul(A, v):
    A = A.a if isinstance(A, FA) else np.asarray(A)
    v = v.a if isinstance(v, FA) else np.asarray(v)
    if A.ndim != 2 or v.ndim != 1:
        raise NotImplementedError("matmul of these ranks")
    out = np.zeros(A.shape[0])
    for i in range(A.shape[0]):
        s = 0.0
        for k in range(A.shape[1]):
            s = s + float(A[i, k]) * float(v[k])
        out[i] = s
    return out


def _fn_nint(x):
    x = float(x)
    return int(math.floor(abs(x) + 0.5)) * (1 if x >= 0 else -1)


def _fn_mod(a, b):
    if isinstance(a, float) or isinstance(b, float):
        return math.fmod(a, b)
    a, b = int(a), int(b)
    return a - _idiv(a, b) * b


def _fn_all(x):
    return bool(np.all(_val(x)))


def _fn_any(x):
    return bool(np.any(_val(x)))


def _fn_trim(s):
    return s.rstrip(" ")


def _fn_iand(a, b):
    return int(a) & int(b)


def _fn_pow(a, b):
    """Real base to any power (elementwise for arrays)."""
    if isinstance(a, np.ndarray) and a.dtype == object:
        out = np.empty(a.shape, dtype=object)
        for ix in np.ndindex(*a.shape):
            out[ix] = a[ix] ** b
        return out
    return a ** b


# kind parameters of the reference's default build (src/precision.F90)
KINDS = {"rp": 8, "ip": 4, "lp": 4}

INTRINSICS = {
    "real": ("_fn_real", "real"), "sqrt": ("_fn_sqrt", "same"), "exp": ("_fn_exp", "same"),
    "erf": ("_fn_erf", "same"), "abs": ("_fn_abs", "same"), "size": ("_fn_size", "int0"),
    "sum": ("_fn_sum", "sum"), "maxval": ("_fn_maxval", "same0"), "max": ("_fn_max", "same"),
    "norm2": ("_fn_norm2", "real0"), "matmul": ("_fn_matmul", "real1"), "nint": ("_fn_nint", "int0"),
    "mod": ("_fn_mod", "same"), "all": ("_fn_all", "log0"), "any": ("_fn_any", "log0"),
    "trim": ("_fn_trim", "char0"), "iand": ("_fn_iand", "int0"),
    "allocated": (None, "log0"), "associated": (None, "log0"),
}

# ---------------------------------------------------------------------------
# source handling


def preprocess(text, defines):
    out = []
    stack = []  # (active, taken)
    active = True
    for line in text.splitlines():
        s = line.strip()
        if s.startswith("#"):
            d = s[1:].strip()
            word = d.split()[0] if d else ""
            if word in ("ifdef", "ifndef", "if"):
                if word == "ifdef":
                    cond = d.split()[1] in defines
                elif word == "ifndef":
                    cond = d.split()[1] not in defines
                else:
                    cond = _pp_cond(d[2:].strip(), defines)
                stack.append((active, cond))
                active = active and cond
            elif word == "elif":
                parent, taken = stack[-1]
                cond = (not taken) and _pp_cond(d[4:].strip(), defines)
                stack[-1] = (parent, taken or cond)
                active = parent and cond
            elif word == "else":
                parent, taken = stack[-1]
                stack[-1] = (parent, True)
                active = parent and not taken
            elif word == "endif":
                parent, _ = stack.pop()
                active = parent
            else:
                raise NotImplementedError("preprocessor directive " + s)
            out.append("")
            continue
        out.append(line if active else "")
    if stack:
        raise ValueError("unbalanced preprocessor conditionals")
    return out


def _pp_cond(expr, defines):
    m = re.fullmatch(r"defined\s*\(\s*(\w+)\s*\)", expr)
    if m:
        return m.group(1) in defines
    if re.fullmatch(r"\w+", expr):
        return expr in defines and defines[expr] not in ("0", "")
    raise NotImplementedError("#if " + expr)


def _strip_comment(line):
    q = None
    for i, ch in enumerate(line):
        if q:
            if ch == q:
                q = None
        elif ch in "'\"":
            q = ch
        elif ch == "!":
            return line[:i]
    return line


def _lower_code(s):
    out, q = [], None
    for ch in s:
        if q:
            out.append(ch)
            if ch == q:
                q = None
        else:
            if ch in "'\"":
                q = ch
            out.append(ch.lower())
    return "".join(out)


def logical_lines(lines):
    """Comments removed, continuations joined, code lower-cased; (lineno, text)."""
    out = []
    buf, start = None, 0
    for no, raw in enumerate(lines, 1):
        s = _strip_comment(raw).rstrip()
        if buf is not None:
            t = s.lstrip()
            if t.startswith("&"):
                t = t[1:]
            else:
                t = " " + t
            s = buf + t
        else:
            start = no
            s = s.strip()
        if s.endswith("&"):
            buf = s[:-1]
            continue
        buf = None
        if s.strip():
            out.append((start, _lower_code(s.strip())))
    return out


# ---------------------------------------------------------------------------
# expressions

_TOK = re.compile(r"""
    (?P<ws>\s+)
  | (?P<str>'[^']*'|"[^"]*")
  | (?P<real>(?:\d+\.\d*|\.\d+)(?:[ed][+-]?\d+)?(?:_\w+)?|\d+[ed][+-]?\d+(?:_\w+)?)
  | (?P<int>\d+(?:_\w+)?)
  | (?P<dot>\.(?:and|or|not|true|false|eq|ne|lt|le|gt|ge|eqv|neqv)\.)
  | (?P<op>\*\*|//|==|/=|<=|>=|=>|[-+*/<>=(),:%\[\]])
  | (?P<name>[a-z_][a-z0-9_]*)
""", re.X)


def tokenize(s):
    toks, i = [], 0
    while i < len(s):
        # a number directly followed by a dot-operator: '1.and.' is not a real
        m = _TOK.match(s, i)
        if not m:
            raise SyntaxError("cannot tokenize: " + s[i:])
        kind = m.lastgroup
        text = m.group(kind)
        if kind == "real" and re.match(r"\d+\.(and|or|not|eq|ne|lt|le|gt|ge|eqv|neqv)\.", s[i:]):
            m2 = re.match(r"\d+", s[i:])
            kind, text = "int", m2.group(0)
        i += len(text)
        if kind != "ws":
            toks.append((kind, text))
    return toks


class Parser:
    def __init__(self, toks):
        self.t = toks
        self.i = 0

    def peek(self, k=0):
        j = self.i + k
        return self.t[j] if j < len(self.t) else (None, None)

    def take(self, text=None):
        tok = self.peek()
        if text is not None and tok[1] != text:
            raise SyntaxError("expected %r, got %r" % (text, tok[1]))
        self.i += 1
        return tok

    def at(self, text):
        return self.peek()[1] == text

    def done(self):
        return self.i >= len(self.t)

    # precedence climbing
    def expr(self):
        return self.p_eqv()

    def p_eqv(self):
        a = self.p_or()
        while self.peek()[1] in (".eqv.", ".neqv."):
            op = self.take()[1]
            a = ("bin", op, a, self.p_or())
        return a

    def p_or(self):
        a = self.p_and()
        while self.at(".or."):
            self.take()
            a = ("bin", ".or.", a, self.p_and())
        return a

    def p_and(self):
        a = self.p_not()
        while self.at(".and."):
            self.take()
            a = ("bin", ".and.", a, self.p_not())
        return a

    def p_not(self):
        if self.at(".not."):
            self.take()
            return ("un", ".not.", self.p_not())
        return self.p_rel()

    _REL = {"==": "==", "/=": "/=", "<": "<", "<=": "<=", ">": ">", ">=": ">=", ".eq.": "==", ".ne.": "/=",
            ".lt.": "<", ".le.": "<=", ".gt.": ">", ".ge.": ">="}

    def p_rel(self):
        a = self.p_concat()
        if self.peek()[1] in self._REL:
            op = self._REL[self.take()[1]]
            a = ("bin", op, a, self.p_concat())
        return a

    def p_concat(self):
        a = self.p_add()
        while self.at("//"):
            self.take()
            a = ("bin", "//", a, self.p_add())
        return a

    def p_add(self):
        if self.peek()[1] in ("+", "-"):
            op = self.take()[1]
            a = ("un", op, self.p_mul())
        else:
            a = self.p_mul()
        while self.peek()[1] in ("+", "-"):
            op = self.take()[1]
            a = ("bin", op, a, self.p_mul())
        return a

    def p_mul(self):
        a = self.p_pow()
        while self.peek()[1] in ("*", "/"):
            op = self.take()[1]
            a = ("bin", op, a, self.p_pow())
        return a

    def p_pow(self):
        a = self.p_primary()
        if self.at("**"):
            self.take()
            if self.peek()[1] in ("+", "-"):  # x**-1 extension
                op = self.take()[1]
                return ("bin", "**", a, ("un", op, self.p_pow()))
            return ("bin", "**", a, self.p_pow())
        return a

    def p_primary(self):
        kind, text = self.peek()
        if kind == "real":
            self.take()
            return ("num", "real", text)
        if kind == "int":
            self.take()
            return ("num", "int", text)
        if kind == "str":
            self.take()
            return ("str", text[1:-1])
        if kind == "dot" and text in (".true.", ".false."):
            self.take()
            return ("log", text == ".true.")
        if text == "(":
            self.take()
            e = self.expr()
            self.take(")")
            return ("paren", e)
        if text == "[":
            self.take()
            items = []
            if not self.at("]"):
                items.append(self.expr())
                while self.at(","):
                    self.take()
                    items.append(self.expr())
            self.take("]")
            return ("arr", items)
        if kind == "name":
            self.take()
            node = ("name", text)
            while True:
                if self.at("("):
                    self.take()
                    node = ("call", node, self.arglist(")"))
                elif self.at("%"):
                    self.take()
                    node = ("comp", node, self.take()[1])
                else:
                    break
            return node
        raise SyntaxError("unexpected token %r" % (text,))

    def arglist(self, close):
        args = []
        if self.at(close):
            self.take()
            return args
        while True:
            args.append(self.arg())
            if self.at(","):
                self.take()
                continue
            self.take(close)
            return args

    def arg(self):
        # keyword argument
        if self.peek()[0] == "name" and self.peek(1)[1] == "=":
            name = self.take()[1]
            self.take("=")
            return ("kw", name, self.expr())
        # section triplet
        lo = hi = st = None
        if not self.at(":"):
            lo = self.expr()
            if not self.at(":"):
                return lo
        self.take(":")
        if self.peek()[1] not in (",", ")", ":"):
            hi = self.expr()
        if self.at(":"):
            self.take()
            st = self.expr()
        return ("range", lo, hi, st)


def parse_expr(s):
    p = Parser(tokenize(s))
    e = p.expr()
    if not p.done():
        raise SyntaxError("trailing tokens in %r" % s)
    return e


def split_top(s, sep=","):
    """Split s at top-level occurrences of sep (outside brackets and strings)."""
    parts, depth, q, cur = [], 0, None, []
    i = 0
    while i < len(s):
        ch = s[i]
        if q:
            cur.append(ch)
            if ch == q:
                q = None
        elif ch in "'\"":
            q = ch
            cur.append(ch)
        elif ch in "([":
            depth += 1
            cur.append(ch)
        elif ch in ")]":
            depth -= 1
            cur.append(ch)
        elif depth == 0 and s.startswith(sep, i):
            parts.append("".join(cur))
            cur = []
            i += len(sep)
            continue
        else:
            cur.append(ch)
        i += 1
    parts.append("".join(cur))
    return [p.strip() for p in parts]


def find_top(s, pat):
    """Index of the first top-level regex match of pat in s, or -1."""
    depth, q = 0, None
    for i, ch in enumerate(s):
        if q:
            if ch == q:
                q = None
            continue
        if ch in "'\"":
            q = ch
        elif ch in "([":
            depth += 1
        elif ch in ")]":
            depth -= 1
        elif depth == 0 and re.match(pat, s[i:]):
            return i
    return -1


def match_paren(s, i):
    """Index just after the parenthesis group that opens at s[i]."""
    depth, q = 0, None
    for j in range(i, len(s)):
        ch = s[j]
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
            if depth == 0:
                return j + 1
    raise SyntaxError("unbalanced parentheses: " + s)


# ---------------------------------------------------------------------------
# declarations

class Var:
    def __init__(self, name, kind, tname=None, dims=None, attrs=(), init=None):
        self.name = name
        self.kind = kind          # int, real, log, char, type
        self.tname = tname        # derived type name
        self.dims = dims          # None for scalars, else list of (lo_ast|None, hi_ast|None|':')
        self.attrs = set(attrs)
        self.init = init

    @property
    def rank(self):
        return 0 if self.dims is None else len(self.dims)

    @property
    def is_array(self):
        return self.dims is not None

    @property
    def alloc(self):
        return "allocatable" in self.attrs or "pointer" in self.attrs

    @property
    def intent(self):
        for a in self.attrs:
            if a.startswith("intent"):
                return a[7:-1].replace(" ", "")
        return None


_DECL = re.compile(r"^(integer|real|logical|character|type\s*\()")


def parse_typespec(ts):
    ts = ts.strip()
    if ts.startswith("integer"):
        return "int", None
    if ts.startswith("real"):
        return "real", None
    if ts.startswith("logical"):
        return "log", None
    if ts.startswith("character"):
        return "char", None
    m = re.fullmatch(r"type\s*\(\s*(\w+)\s*\)", ts)
    if m:
        return "type", m.group(1)
    raise NotImplementedError("type spec " + ts)


def parse_dims(s):
    dims = []
    for d in split_top(s):
        if d == ":":
            dims.append((None, None))
        elif d == "*":
            dims.append((None, "*"))
        else:
            parts = split_top(d, ":")
            if len(parts) == 1:
                dims.append((None, parse_expr(parts[0])))
            else:
                lo = parse_expr(parts[0]) if parts[0] else None
                hi = parse_expr(parts[1]) if parts[1] else None
                dims.append((lo, hi))
    return dims


def parse_decl(text):
    k = find_top(text, r"::")
    if k >= 0:
        head, ents = text[:k], text[k + 2:]
    else:
        m = re.match(r"^(integer|real|logical|character)(\s*\([^)]*\))?\s+", text) or \
            re.match(r"^type\s*\(\s*\w+\s*\)\s+", text)
        if not m:
            raise NotImplementedError("declaration " + text)
        head, ents = text[:m.end()], text[m.end():]
    hp = split_top(head.strip())
    kind, tname = parse_typespec(hp[0])
    attrs, adims = [], None
    for a in hp[1:]:
        a = a.replace(" ", "")
        if a.startswith("dimension("):
            adims = parse_dims(a[len("dimension("):-1])
        else:
            attrs.append(a)
    out = []
    for e in split_top(ents):
        init = None
        j = find_top(e, r"=(?!=)")
        if j >= 0:
            init = parse_expr(e[j + 1:].lstrip(">").strip())
            e = e[:j].strip()
        m = re.match(r"^(\w+)\s*(\(.*\))?$", e)
        if not m:
            raise NotImplementedError("entity " + e)
        dims = parse_dims(m.group(2)[1:-1]) if m.group(2) else adims
        out.append(Var(m.group(1), kind, tname, dims, attrs, init))
    return out


class Proc:
    def __init__(self, kind, name, args, result, module):
        self.kind = kind
        self.name = name
        self.args = args
        self.result = result
        self.module = module
        self.decls = {}
        self.body = []

    def wb(self):
        """Dummies whose final value is handed back to the caller."""
        out = []
        for i, a in enumerate(self.args):
            v = self.decls.get(a)
            if v is None:
                raise NotImplementedError("undeclared dummy %s of %s" % (a, self.name))
            if v.intent == "in":
                continue
            if v.kind == "type" and not v.is_array and not v.alloc:
                continue
            if v.is_array and not v.alloc:
                continue
            out.append(i)
        return out


class TypeDef:
    def __init__(self, name):
        self.name = name
        self.comps = {}


# ---------------------------------------------------------------------------
# program model


class Program:
    def __init__(self):
        self.types = {}
        self.procs = {}
        self.modvars = {}
        self.comp = {}  # component name -> Var (names are unique across the reference's types)

    def load(self, text, defines):
        lines = logical_lines(preprocess(text, defines))
        i = 0
        module = None
        cur_type = None
        stack = []
        while i < len(lines):
            no, s = lines[i]
            i += 1
            if cur_type is not None:
                if re.match(r"^end\s*type", s):
                    self.types[cur_type.name] = cur_type
                    cur_type = None
                    continue
                for v in parse_decl(s):
                    if v.name in self.comp and self.comp[v.name].kind != v.kind:
                        raise NotImplementedError("component name reused with another type: " + v.name)
                    cur_type.comps[v.name] = v
                    self.comp[v.name] = v
                continue
            m = re.match(r"^module\s+(\w+)$", s)
            if m:
                module = m.group(1)
                continue
            if re.match(r"^end\s*module", s):
                module = None
                continue
            if s in ("contains", "implicit none", "private") or s.startswith("use ") or s.startswith("use,") \
                    or s.startswith("public") or s.startswith("private"):
                continue
            m = re.match(r"^type\s*(?:::)?\s*(\w+)$", s)
            if m and not stack:
                cur_type = TypeDef(m.group(1))
                continue
            m = re.match(r"^((?:pure|recursive|elemental|\s)*)(subroutine|function)\s+(\w+)\s*(?:\(([^)]*)\))?"
                         r"\s*(?:result\s*\(\s*(\w+)\s*\))?$", s)
            if m:
                args = [a.strip() for a in (m.group(4) or "").split(",") if a.strip()]
                kind = "sub" if m.group(2) == "subroutine" else "func"
                res = m.group(5) or (m.group(3) if kind == "func" else None)
                p = Proc(kind, m.group(3), args, res, module)
                stack.append(p)
                continue
            if re.match(r"^end\s*(subroutine|function)\b", s):
                p = stack.pop()
                if stack:
                    raise NotImplementedError("internal procedures")
                self.procs[p.name] = p
                continue
            if stack:
                p = stack[-1]
                if _is_decl(s):
                    for v in parse_decl(s):
                        p.decls[v.name] = v
                    continue
                if s == "implicit none" or s.startswith("use "):
                    continue
                p.body.append((no, s))
                continue
            if _is_decl(s):
                for v in parse_decl(s):
                    self.modvars[v.name] = v
                continue
            raise NotImplementedError("module-level statement: " + s)


def _is_decl(s):
    if not _DECL.match(s):
        return False
    if "::" in s:
        return True
    return bool(re.match(r"^(integer|real|logical|character)(\s*\([^)]*\))?\s+\w+", s)
                or re.match(r"^type\s*\(\s*\w+\s*\)\s+\w+", s))


# ---------------------------------------------------------------------------
# code generation

_PY_OPS = {"+": "+", "-": "-", "*": "*", "/": "/", "==": "==", "/=": "!=", "<": "<", "<=": "<=", ">": ">",
           ">=": ">="}


class Gen:
    def __init__(self, prog):
        self.prog = prog
        self.out = []
        self.cut = None  # name of the extent variable while emitting an array assignment's right side

    # --- lookups
    def var(self, name, proc):
        if proc is not None and name in proc.decls:
            return proc.decls[name]
        if name in self.prog.modvars:
            return self.prog.modvars[name]
        return None

    def pyname(self, name, proc):
        if proc is not None and name in proc.decls:
            return "f_" + name
        if name in self.prog.modvars:
            return "f_" + name
        raise NameError("unknown name %s in %s" % (name, proc.name if proc else "<module>"))

    # --- expression typing: returns (kind, rank)
    def typeof(self, e, proc):
        t = e[0]
        if t == "num":
            return ("int" if e[1] == "int" else "real"), 0
        if t == "str":
            return "char", 0
        if t == "log":
            return "log", 0
        if t == "paren":
            return self.typeof(e[1], proc)
        if t == "arr":
            ks = [self.typeof(x, proc)[0] for x in e[1]]
            return ("real" if "real" in ks else ks[0] if ks else "int"), 1
        if t == "name":
            v = self.var(e[1], proc)
            if v is None:
                if e[1] in KINDS:
                    return "int", 0
                raise NameError("unknown name " + e[1])
            return v.kind, v.rank
        if t == "comp":
            v = self.prog.comp[e[2]]
            return v.kind, v.rank
        if t == "call":
            base = e[1]
            v = self.decl_of(base, proc)
            if v is not None and v.is_array:
                nr = sum(1 for a in e[2] if a[0] == "range" or self.typeof(a, proc)[1] > 0)
                return v.kind, nr
            if base[0] == "name":
                n = base[1]
                if n in self.prog.procs:
                    p = self.prog.procs[n]
                    rv = p.decls[p.result]
                    return rv.kind, rv.rank
                if n in INTRINSICS:
                    how = INTRINSICS[n][1]
                    args = [a for a in e[2] if a[0] != "kw"]
                    k0, r0 = self.typeof(args[0], proc) if args else ("int", 0)
                    if how == "same":
                        ks = [self.typeof(a, proc) for a in args]
                        kind = "real" if any(k == "real" for k, _ in ks) else k0
                        return kind, max(r for _, r in ks)
                    if how == "same0":
                        return k0, 0
                    if how == "real":
                        return "real", r0
                    if how == "sum":
                        return k0, (r0 - 1 if len(e[2]) > 1 else 0)
                    return {"int0": ("int", 0), "real0": ("real", 0), "real1": ("real", 1),
                            "log0": ("log", 0), "char0": ("char", 0)}[how]
            raise NameError("cannot type call of %r" % (base,))
        if t == "un":
            k, r = self.typeof(e[2], proc)
            return ("log" if e[1] == ".not." else k), r
        if t == "bin":
            ka, ra = self.typeof(e[2], proc)
            kb, rb = self.typeof(e[3], proc)
            r = max(ra, rb)
            if e[1] in ("==", "/=", "<", "<=", ">", ">=", ".and.", ".or.", ".eqv.", ".neqv."):
                return "log", r
            if e[1] == "//":
                return "char", 0
            if ka == "real" or kb == "real":
                return "real", r
            return ka, r
        raise NotImplementedError(t)

    def decl_of(self, d, proc):
        """Declaration of the entity a designator names (without subscripts)."""
        if d[0] == "name":
            return self.var(d[1], proc)
        if d[0] == "comp":
            return self.prog.comp.get(d[2])
        if d[0] == "call":
            return None
        return None

    # --- expressions
    def ex(self, e, proc, as_arg=False):
        t = e[0]
        if t == "num":
            txt = e[2]
            if e[1] == "int":
                return str(int(txt.split("_")[0]))
            body, _, kind = txt.partition("_")
            body = body.replace("d", "e")
            if kind or "d" in e[2]:
                return repr(float(body))
            return repr(_f32(float(body)))
        if t == "str":
            return repr(e[1])
        if t == "log":
            return "True" if e[1] else "False"
        if t == "paren":
            return "(" + self.ex(e[1], proc) + ")"
        if t == "arr":
            return "np.array([%s])" % ", ".join(self.ex(x, proc) for x in e[1])
        if t == "name":
            v = self.var(e[1], proc)
            if v is None:
                if e[1] in KINDS:
                    return str(KINDS[e[1]])
                raise NameError("unknown name %s in %s" % (e[1], proc.name if proc else ""))
            pn = self.pyname(e[1], proc)
            if v.is_array and not as_arg:
                return self.cutwrap("_val(%s)" % pn)
            return pn
        if t == "comp":
            v = self.prog.comp[e[2]]
            s = "%s.f_%s" % (self.ex(e[1], proc, as_arg=True), e[2])
            if v.is_array and not as_arg:
                return self.cutwrap("_val(%s)" % s)
            return s
        if t == "call":
            return self.ex_call(e, proc, as_arg)
        if t == "un":
            if e[1] == ".not.":
                _, r = self.typeof(e[2], proc)
                return ("(~%s)" if r else "(not %s)") % self.ex(e[2], proc)
            return "(%s%s)" % (e[1], self.ex(e[2], proc))
        if t == "bin":
            op = e[1]
            a, b = self.ex(e[2], proc), self.ex(e[3], proc)
            ka, ra = self.typeof(e[2], proc)
            kb, rb = self.typeof(e[3], proc)
            if op in (".and.", ".or."):
                if ra or rb:
                    return "(%s %s %s)" % (a, "&" if op == ".and." else "|", b)
                return "(%s %s %s)" % (a, "and" if op == ".and." else "or", b)
            if op == "//":
                return "(%s + %s)" % (a, b)
            if ka == "char" and kb == "char" and op in ("==", "/="):
                return "(%s_streq(%s, %s))" % ("" if op == "==" else "not ", a, b)
            if op == "/" and ka == "int" and kb == "int":
                return "_idiv(%s, %s)" % (a, b)
            if op == "**":
                if ka == "int" and kb == "int":
                    return "_ipow(%s, %s)" % (a, b)
                return "_fn_pow(%s, %s)" % (a, b)
            return "(%s %s %s)" % (a, _PY_OPS[op], b)
        raise NotImplementedError(t)

    def cutwrap(self, code):
        return "_cut(%s, %s)" % (code, self.cut) if self.cut else code

    def nocut(self, fn, *a, **k):
        saved, self.cut = self.cut, None
        try:
            return fn(*a, **k)
        finally:
            self.cut = saved

    def subs(self, args, proc):
        return self.nocut(self._subs, args, proc)

    def _subs(self, args, proc):
        out = []
        for a in args:
            if a[0] == "range":
                if a[1] is None and a[2] is None and a[3] is None:
                    out.append("_ALL")
                else:
                    out.append("_S(%s, %s, %s)" % tuple("None" if x is None else self.ex(x, proc) for x in a[1:]))
            else:
                out.append(self.ex(a, proc))
        return "(" + ", ".join(out) + ("," if len(out) == 1 else "") + ")"

    def ex_call(self, e, proc, as_arg=False):
        base, args = e[1], e[2]
        v = self.decl_of(base, proc)
        if v is not None and v.is_array:
            code = "%s[%s]" % (self.nocut(self.ex, base, proc, as_arg=True), self.subs(args, proc)[1:-1] or "()")
            if not as_arg and self.typeof(e, proc)[1] > 0:
                return self.cutwrap(code)
            return code
        if base[0] != "name":
            raise NotImplementedError("call through component %r" % (base,))
        n = base[1]
        if n in self.prog.procs:
            p = self.prog.procs[n]
            if p.kind != "func":
                raise NotImplementedError("subroutine %s used as a function" % n)
            return "f_%s(%s)" % (n, self.nocut(self.actuals, p, args, proc))
        if n in INTRINSICS:
            if n in ("sum", "maxval", "size", "norm2", "matmul", "all", "any", "trim"):
                return self.nocut(self._intrinsic, n, args, proc)
            return self._intrinsic(n, args, proc)
        raise NameError("unknown procedure or array %s in %s" % (n, proc.name if proc else ""))

    def _intrinsic(self, n, args, proc):
        if True:
            if n == "allocated":
                return "(%s is not None)" % self.ex(args[0], proc, as_arg=True)
            if n == "associated":
                return "(%s is not None)" % self.ex(args[0], proc, as_arg=True)
            fn = INTRINSICS[n][0]
            parts = []
            for a in args:
                if a[0] == "kw":
                    if n in ("real",) and a[1] == "kind":
                        parts.append("1")
                    else:
                        parts.append("%s=%s" % (a[1], self.ex(a[2], proc)))
                else:
                    parts.append(self.ex(a, proc))
            if n == "real" and len(args) == 2 and args[1][0] != "kw":
                parts[1] = "1"
            return "%s(%s)" % (fn, ", ".join(parts))

    def actuals(self, p, args, proc):
        out = []
        for k, a in enumerate(args):
            if a[0] == "kw":
                raise NotImplementedError("keyword actual arguments")
            dn = p.args[k]
            dv = p.decls[dn]
            if dv.is_array or dv.kind == "type":
                out.append(self.ex(a, proc, as_arg=True))
            else:
                out.append(self.ex(a, proc))
        if len(args) != len(p.args):
            raise NotImplementedError("optional arguments (%s)" % p.name)
        return ", ".join(out)

    # --- statements
    def emit(self, ind, line):
        self.out.append("    " * ind + line)

    def lhs_store(self, d, value, proc, ind):
        """Emits the store of python expression `value` into designator d."""
        t = d[0]
        if t == "name":
            v = self.var(d[1], proc)
            pn = self.pyname(d[1], proc)
            if v.is_array:
                self.emit(ind, "%s = _asgn(%s, %s, %r)" % (pn, pn, value, v.kind))
            else:
                self.emit(ind, "%s = %s" % (pn, self.conv(v.kind, value)))
            return
        if t == "comp":
            v = self.prog.comp[d[2]]
            obj = self.ex(d[1], proc, as_arg=True)
            if v.is_array:
                self.emit(ind, "%s.f_%s = _asgn(%s.f_%s, %s, %r)" % (obj, d[2], obj, d[2], value, v.kind))
            else:
                self.emit(ind, "%s.f_%s = %s" % (obj, d[2], self.conv(v.kind, value)))
            return
        if t == "call":
            v = self.decl_of(d[1], proc)
            if v is None or not v.is_array:
                raise NotImplementedError("store into %r" % (d,))
            self.emit(ind, "%s[%s] = %s" % (self.ex(d[1], proc, as_arg=True), self.subs(d[2], proc)[1:-1],
                                             value if v.kind != "real" else value))
            return
        raise NotImplementedError("store into %r" % (d,))

    @staticmethod
    def conv(kind, value):
        if kind == "int":
            return "_w32(%s)" % value
        if kind == "log":
            return "bool(%s)" % value
        return value

    def gen_proc(self, p):
        modnames = set(self.prog.modvars) - set(p.decls)
        used = set(re.findall(r"[a-z_][a-z0-9_]*", " ".join(s for _, s in p.body)))
        for v in p.decls.values():
            if v.dims:
                for lo, hi in v.dims:
                    for x in (lo, hi):
                        if x is not None and x != "*":
                            used |= set(re.findall(r"[a-z_][a-z0-9_]*", repr(x)))
        glob = sorted(n for n in modnames if n in used)
        self.emit(0, "def f_%s(%s):" % (p.name, ", ".join("f_" + a for a in p.args)))
        if glob:
            self.emit(1, "global " + ", ".join("f_" + g for g in glob))
        # dummies
        for a in p.args:
            v = p.decls[a]
            if v.is_array and v.alloc:
                self.emit(1, "f_%s = _ptr(f_%s)" % (a, a))
            if v.is_array and not v.alloc:
                lbs = [0 if False else 1 for _ in v.dims]
                lbs = []
                shape = []
                explicit = True
                for lo, hi in v.dims:
                    lbs.append(self.ex(lo, p) if lo is not None else "1")
                    if hi is None or hi == "*":
                        explicit = False
                    else:
                        shape.append(self.ex(hi, p) if lo is None else "(%s) - (%s) + 1" % (self.ex(hi, p), self.ex(lo, p)))
                self.emit(1, "f_%s = _dummy(f_%s, (%s,), %s)" % (a, a, ", ".join(lbs),
                                                                  "(%s,)" % ", ".join(shape) if explicit else "None"))
        # locals
        for n, v in p.decls.items():
            if n in p.args:
                continue
            if v.init is not None:
                if "parameter" in v.attrs:
                    self.emit(1, "f_%s = %s" % (n, self.conv(v.kind, self.ex(v.init, p))))
                    continue
                raise NotImplementedError("initialised local (implies SAVE): %s in %s" % (n, p.name))
            if v.is_array:
                if v.alloc:
                    self.emit(1, "f_%s = None" % n)
                else:
                    dims = []
                    for lo, hi in v.dims:
                        dims.append("(%s, %s)" % (self.ex(lo, p) if lo is not None else "1", self.ex(hi, p)))
                    self.emit(1, "f_%s = _alloc(%r, [%s]%s)" % (
                        n, v.kind, ", ".join(dims), ", T_%s" % v.tname if v.kind == "type" else ""))
            elif v.kind == "type":
                self.emit(1, "f_%s = %s" % (n, "None" if "pointer" in v.attrs else "T_%s()" % v.tname))
            else:
                self.emit(1, "f_%s = %s" % (n, {"int": "0", "real": "0.0", "log": "False", "char": "''"}[v.kind]))
        self.ret = self.ret_expr(p)
        self.block(p.body, 0, len(p.body), p, 1)
        self.emit(1, "return " + self.ret)
        self.emit(0, "")

    def ret_expr(self, p):
        if p.kind == "func":
            v = p.decls[p.result]
            return "_val(f_%s)" % p.result if v.is_array else "f_%s" % p.result
        wb = p.wb()
        return "(" + "".join("f_%s, " % p.args[i] for i in wb) + ")"

    def block(self, body, i, end, p, ind):
        """Emits statements body[i:end]; returns nothing."""
        start_len = len(self.out)
        while i < end:
            no, s = body[i]
            i = self.stmt(body, i, end, p, ind)
        if len(self.out) == start_len:
            self.emit(ind, "pass")

    def find_end(self, body, i, end, opener, closer, mids=()):
        """Index of the matching closer of the construct opened at body[i]; and mid-split indices."""
        depth = 0
        marks = []
        for j in range(i, end):
            s = body[j][1]
            if opener(s):
                depth += 1
            elif closer(s):
                depth -= 1
                if depth == 0:
                    return j, marks
            elif depth == 1 and any(m(s) for m in mids):
                marks.append(j)
        raise SyntaxError("unterminated construct at line %d" % body[i][0])

    def stmt(self, body, i, end, p, ind):
        no, s = body[i]
        is_do = lambda x: bool(re.match(r"^do\b", x)) and not re.match(r"^do\s*=", x)
        end_do = lambda x: bool(re.match(r"^end\s*do\b", x))
        if is_do(s):
            j, _ = self.find_end(body, i, end, is_do, end_do)
            m = re.match(r"^do\s+(\w+)\s*=\s*(.*)$", s)
            if m:
                parts = split_top(m.group(2))
                lo, hi = self.ex(parse_expr(parts[0]), p), self.ex(parse_expr(parts[1]), p)
                st = self.ex(parse_expr(parts[2]), p) if len(parts) > 2 else "1"
                var = self.pyname(m.group(1), p)
                if len(parts) > 2:
                    self.emit(ind, "for %s in _drange(%s, %s, %s):" % (var, lo, hi, st))
                else:
                    self.emit(ind, "for %s in range(%s, (%s) + 1):" % (var, lo, hi))
            elif re.match(r"^do\s+while\b", s):
                k = s.index("(")
                cond = s[k:match_paren(s, k)]
                self.emit(ind, "while %s:" % self.ex(parse_expr(cond), p))
            elif re.match(r"^do\s+concurrent\b", s):
                k = s.index("(")
                inner = s[k + 1:match_paren(s, k) - 1]
                mm = re.match(r"^(\w+)\s*=\s*(.*)$", inner)
                parts = split_top(mm.group(2), ":")
                self.emit(ind, "for %s in range(%s, (%s) + 1):" % (
                    self.pyname(mm.group(1), p), self.ex(parse_expr(parts[0]), p), self.ex(parse_expr(parts[1]), p)))
            else:
                raise NotImplementedError("do form: " + s)
            self.block(body, i + 1, j, p, ind + 1)
            return j + 1
        if re.match(r"^if\s*\(", s):
            k = s.index("(")
            kend = match_paren(s, k)
            cond = self.ex(parse_expr(s[k:kend]), p)
            rest = s[kend:].strip()
            if rest == "then":
                is_if = lambda x: bool(re.match(r"^if\s*\(", x)) and x.rstrip().endswith("then")
                end_if = lambda x: bool(re.match(r"^end\s*if\b", x))
                mid = lambda x: bool(re.match(r"^else\b", x))
                j, marks = self.find_end(body, i, end, is_if, end_if, (mid,))
                bounds = [i] + marks + [j]
                for q in range(len(bounds) - 1):
                    hs = body[bounds[q]][1]
                    if q == 0:
                        self.emit(ind, "if %s:" % cond)
                    else:
                        mm = re.match(r"^else\s*if\s*(\(.*\))\s*then$", hs)
                        if mm:
                            self.emit(ind, "elif %s:" % self.ex(parse_expr(mm.group(1)), p))
                        elif hs == "else":
                            self.emit(ind, "else:")
                        else:
                            raise NotImplementedError(hs)
                    self.block(body, bounds[q] + 1, bounds[q + 1], p, ind + 1)
                return j + 1
            self.emit(ind, "if %s:" % cond)
            self.simple(rest, p, ind + 1, no)
            return i + 1
        if re.match(r"^select\s+case\b", s):
            k = s.index("(")
            sel = self.ex(parse_expr(s[k:match_paren(s, k)]), p)
            is_sel = lambda x: bool(re.match(r"^select\s+case\b", x))
            end_sel = lambda x: bool(re.match(r"^end\s*select\b", x))
            mid = lambda x: bool(re.match(r"^case\b", x))
            j, marks = self.find_end(body, i, end, is_sel, end_sel, (mid,))
            self.emit(ind, "_sel = %s" % sel)
            first = True
            for q, mk in enumerate(marks):
                hs = body[mk][1]
                stop = marks[q + 1] if q + 1 < len(marks) else j
                if re.match(r"^case\s+default$", hs):
                    self.emit(ind, "else:" if not first else "if True:")
                else:
                    kk = hs.index("(")
                    conds = []
                    for item in split_top(hs[kk + 1:match_paren(hs, kk) - 1]):
                        rr = split_top(item, ":")
                        if len(rr) == 1:
                            conds.append("_sel == %s" % self.ex(parse_expr(rr[0]), p))
                        else:
                            c = []
                            if rr[0]:
                                c.append("_sel >= %s" % self.ex(parse_expr(rr[0]), p))
                            if rr[1]:
                                c.append("_sel <= %s" % self.ex(parse_expr(rr[1]), p))
                            conds.append("(" + " and ".join(c) + ")")
                    self.emit(ind, "%s %s:" % ("if" if first else "elif", " or ".join(conds)))
                first = False
                self.block(body, mk + 1, stop, p, ind + 1)
            return j + 1
        self.simple(s, p, ind, no)
        return i + 1

    def simple(self, s, p, ind, no):
        if s == "cycle":
            self.emit(ind, "continue")
            return
        if s == "exit":
            self.emit(ind, "break")
            return
        if s == "continue":
            self.emit(ind, "pass")
            return
        if s == "return":
            self.emit(ind, "return " + self.ret)
            return
        m = re.match(r"^error\s+stop\b(.*)$", s)
        if m:
            msg = m.group(1).strip()
            self.emit(ind, "raise FortranStop(%s)" % (self.ex(parse_expr(msg), p) if msg else "''"))
            return
        m = re.match(r"^call\s+(\w+)\s*(\(.*\))?$", s)
        if m:
            self.call_stmt(m.group(1), m.group(2), p, ind)
            return
        m = re.match(r"^(allocate|deallocate|nullify)\s*(\(.*\))$", s)
        if m:
            getattr(self, "st_" + m.group(1))(m.group(2)[1:-1], p, ind)
            return
        k = find_top(s, r"=>")
        if k >= 0:
            lhs = parse_expr(s[:k])
            rhs = parse_expr(s[k + 2:])
            self.lhs_bind(lhs, self.ex(rhs, p, as_arg=True), p, ind)
            return
        k = find_top(s, r"=(?![=>])")
        if k >= 0 and (k == 0 or s[k - 1] not in "<>/="):
            lhs = parse_expr(s[:k])
            rhs = parse_expr(s[k + 1:])
            kind, rank = self.typeof(rhs, p)
            dv = self.decl_of(lhs, p) if lhs[0] != "call" else None
            if dv is not None and dv.kind == "type" and not dv.is_array:
                self.lhs_bind(lhs, self.ex(rhs, p, as_arg=True), p, ind)
                return
            if lhs[0] == "call" and self.typeof(lhs, p)[1] > 0 and rank > 0:
                self.emit(ind, "_ext = np.shape(%s)" % self.ex(lhs, p))
                self.cut = "_ext"
                try:
                    value = self.ex(rhs, p)
                finally:
                    self.cut = None
                self.lhs_store(lhs, value, p, ind)
                return
            self.lhs_store(lhs, self.ex(rhs, p), p, ind)
            return
        raise NotImplementedError("statement at line %d: %s" % (no, s))

    def lhs_bind(self, d, value, p, ind):
        v = self.decl_of(d, p)
        if v is not None and v.is_array and value != "None":
            value = "_ptr(%s)" % value
        if d[0] == "name":
            self.emit(ind, "%s = %s" % (self.pyname(d[1], p), value))
        elif d[0] == "comp":
            self.emit(ind, "%s.f_%s = %s" % (self.ex(d[1], p, as_arg=True), d[2], value))
        else:
            raise NotImplementedError("pointer assignment to %r" % (d,))

    def call_stmt(self, name, argtext, p, ind):
        args = Parser(tokenize(argtext)).arglist(")") if False else []
        if argtext:
            pr = Parser(tokenize(argtext[1:]))
            args = pr.arglist(")")
        if name == "move_alloc":
            a, b = args
            self.lhs_bind(b, self.ex(a, p, as_arg=True), p, ind)
            self.lhs_bind(a, "None", p, ind)
            return
        if name.startswith("mpi_"):
            raise NotImplementedError("MPI call outside the serial build")
        if name not in self.prog.procs:
            raise NameError("unknown subroutine " + name)
        q = self.prog.procs[name]
        call = "f_%s(%s)" % (name, self.actuals(q, args, p))
        wb = q.wb()
        if not wb:
            self.emit(ind, call)
            return
        self.emit(ind, "_r = " + call)
        for j, k in enumerate(wb):
            a = args[k]
            if a[0] in ("name", "comp") or (a[0] == "call" and self.decl_of(a[1], p) is not None):
                dv = q.decls[q.args[k]]
                if dv.is_array or dv.kind == "type":
                    self.lhs_bind(a, "_r[%d]" % j, p, ind)
                else:
                    self.lhs_store(a, "_r[%d]" % j, p, ind)

    def st_allocate(self, text, p, ind):
        items = split_top(text)
        source = None
        objs = []
        for it in items:
            m = re.match(r"^source\s*=\s*(.*)$", it)
            if m:
                source = self.ex(parse_expr(m.group(1)), p)
            else:
                objs.append(parse_expr(it))
        for o in objs:
            if o[0] == "call":
                d, dims = o[1], o[2]
                v = self.decl_of(d, p)
                if v is None:
                    raise NameError("allocate of unknown %r" % (d,))
                ds = []
                for a in dims:
                    if a[0] == "range":
                        ds.append("(%s, %s)" % (self.ex(a[1], p), self.ex(a[2], p)))
                    else:
                        ds.append("(1, _w32(%s))" % self.ex(a, p))
                val = "_alloc(%r, [%s]%s%s)" % (v.kind, ", ".join(ds),
                                                ", T_%s" % v.tname if v.kind == "type" else ", None",
                                                ", source=%s" % source if source else "")
                self.lhs_bind(d, val, p, ind)
            else:
                v = self.decl_of(o, p)
                if v is None or v.kind != "type" or v.is_array:
                    raise NotImplementedError("allocate of %r" % (o,))
                self.lhs_bind(o, "T_%s()" % v.tname, p, ind)

    def st_deallocate(self, text, p, ind):
        for it in split_top(text):
            d = parse_expr(it)
            self.emit(ind, "_dealloc(%s, %r)" % (self.ex(d, p, as_arg=True), it))
            self.lhs_bind(d, "None", p, ind)

    def st_nullify(self, text, p, ind):
        for it in split_top(text):
            self.lhs_bind(parse_expr(it), "None", p, ind)

    def gen_type(self, t):
        self.emit(0, "class T_%s:" % t.name)
        self.emit(1, "def __init__(self):")
        for n, v in t.comps.items():
            if v.alloc:
                self.emit(2, "self.f_%s = None" % n)
            elif v.is_array:
                dims = ", ".join("(%s, %s)" % (self.ex(lo, None) if lo is not None else "1", self.ex(hi, None))
                                 for lo, hi in v.dims)
                val = "_alloc(%r, [%s]%s)" % (v.kind, dims, ", T_%s" % v.tname if v.kind == "type" else "")
                self.emit(2, "self.f_%s = %s" % (n, val))
                if v.init is not None:
                    self.emit(2, "self.f_%s.a[...] = %s" % (n, self.ex(v.init, None)))
            elif v.kind == "type":
                self.emit(2, "self.f_%s = T_%s()" % (n, v.tname))
            else:
                init = self.ex(v.init, None) if v.init is not None else \
                    {"int": "0", "real": "0.0", "log": "False", "char": "''"}[v.kind]
                self.emit(2, "self.f_%s = %s" % (n, self.conv(v.kind, init)))
        self.emit(0, "")

    def generate(self):
        self.emit(0, "# generated from the reference's Fortran source; do not edit")
        for t in self.prog.types.values():
            self.gen_type(t)
        for n, v in self.prog.modvars.items():
            if v.kind == "type" and not v.is_array:
                self.emit(0, "f_%s = %s" % (n, "None" if "pointer" in v.attrs else "T_%s()" % v.tname))
            elif v.is_array:
                self.emit(0, "f_%s = None" % n)
            else:
                init = self.ex(v.init, None) if v.init is not None else {"int": "0", "real": "0.0", "log": "False",
                                                                          "char": "''"}[v.kind]
                self.emit(0, "f_%s = %s" % (n, self.conv(v.kind, init)))
        for p in self.prog.procs.values():
            self.gen_proc(p)
        return "\n".join(self.out)


def _drange(lo, hi, st):
    lo, hi, st = int(lo), int(hi), int(st)
    return range(lo, hi + 1, st) if st > 0 else range(lo, hi - 1, st)


class Translated:
    """The translated program; ``new()`` gives a fresh instance (module
    variables in their initial state, as in a new process), whose procedures
    are ``ns['f_<name>']`` (lower-case Fortran names)."""

    def __init__(self, paths, defines=None):
        defines = {"__GNUC__": "1"} if defines is None else defines
        prog = Program()
        for path in paths:
            with open(path) as f:
                prog.load(f.read(), defines)
        self.program = prog
        self.source = Gen(prog).generate()
        self.code = compile(self.source, "<fortran:%s>" % ",".join(p.split("/")[-1] for p in paths), "exec")

    def new(self):
        ns = {k: v for k, v in globals().items()
              if k.startswith("_") or k in ("np", "math", "FA", "FortranStop")}
        exec(self.code, ns)
        return ns
