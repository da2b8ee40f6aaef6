"""Executor for the Fortran 90 subset of the reference's hot-path routines.

TEST INFRASTRUCTURE ONLY: it runs the reference's own source files to make
the golden vectors under tests/golden/ (make_golden.py); nothing in the
library, the bench or the GPU tests uses it.

No Fortran compiler exists in the build image or on the GPU machine, so the
reference (gfortran -O2, x86-64: SSE2 arithmetic, no fused multiply-add, no
reassociation -- Makefile:6-10) cannot be built.  This module translates
each subroutine of a reference source file into a Python function and runs
it, with the arithmetic of that build:

  * real(prec)/real(dp) values are numpy float64 scalars and arrays;
    default-real values and literals (`1.`, `0.0`, `1.e20`, `small = 1e-30`)
    are numpy float32, rounded from the decimal literal exactly, so mixed
    expressions promote as Fortran's do (float32 op float64 -> float64,
    float32 op float32 -> float32);
  * every binary operation is emitted fully parenthesised in source order
    (Fortran's left-to-right association, parentheses respected);
  * integer division truncates towards zero; x**n with an integer literal
    n is the multiplication chain gfortran expands it into;
  * intrinsics map to correctly rounded IEEE operations (sqrt) or to the
    C library calls gfortran makes (exp, log, pow);
  * arrays are stored with one unused leading element per dimension, so a
    Fortran subscript indexes the numpy array directly;
  * a DO variable after a loop that ran to completion holds last + step,
    as the solver report lines read it;
  * scalar dummy arguments are passed by reference (the callee returns
    their final values and the caller stores them back);
  * WRITE statements are formatted (the A, I, X, E/ES with 1P, F edit
    descriptors and literal strings) and appended to `ns.units[unit]`.

Supported statements: declarations, USE, IMPLICIT, PARAMETER entities, DO
(with step), DO WHILE, IF blocks and one-line IF, EXIT, CYCLE, RETURN,
CALL, assignment (scalar, element, whole array), WRITE.  Anything else
raises, so a routine outside the subset cannot run silently wrong.
"""
from fractions import Fraction
import math
import pathlib
import re

import numpy as np

# ------------------------------------------------------------------ source


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


def _lower_outside_strings(s):
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


def statements(text):
    """Free-form source -> list of statements (comments dropped,
    continuations joined, lower case outside strings)."""
    out, cur = [], None
    for raw in text.splitlines():
        line = _strip_comment(raw).rstrip()
        if not line.strip():
            continue
        s = line.strip()
        if cur is not None:
            if s.startswith("&"):
                s = s[1:]
            cur += s
        else:
            cur = s
        if cur.endswith("&"):
            cur = cur[:-1]
            continue
        cur = _lower_outside_strings(cur).strip()
        for part in _split_semicolons(cur):
            if part:
                out.append(part)
        cur = None
    return out


def _split_semicolons(s):
    parts, q, start = [], None, 0
    for i, ch in enumerate(s):
        if q:
            if ch == q:
                q = None
        elif ch in "'\"":
            q = ch
        elif ch == ";":
            parts.append(s[start:i].strip())
            start = i + 1
    parts.append(s[start:].strip())
    return parts


# ------------------------------------------------------------------ literals


def exact_f32(text):
    """Decimal literal -> the nearest float32 (ties to even), rounded once
    from the exact decimal value as the compiler does."""
    v = Fraction(text)
    f = np.float32(float(v))
    best = None
    with np.errstate(over="ignore"):
        cands = (np.nextafter(f, np.float32(-np.inf)), f, np.nextafter(f, np.float32(np.inf)))
    for c in cands:
        if not np.isfinite(c):
            continue
        d = abs(Fraction(float(c)) - v)
        key = (d, int(np.array(c).view(np.uint32)) & 1)
        if best is None or key < best[0]:
            best = (key, c)
    return np.float32(best[1])


# ------------------------------------------------------------------ lexer

_DOTOPS = ("eqv", "neqv", "and", "or", "not", "eq", "ne", "lt", "le", "gt", "ge")
_TOKEN = re.compile(r"""
   (?P<ws>\s+)
 | (?P<int_before_dot>\d+(?=\.(?:eq|ne|lt|le|gt|ge|and|or|not|eqv|neqv|true|false)\.))
 | (?P<real>(?:\d+\.\d*|\.\d+)(?:[ed][+-]?\d+)?(?:_\w+)?|\d+[ed][+-]?\d+(?:_\w+)?)
 | (?P<int>\d+(?:_\w+)?)
 | (?P<logical>\.(?:true|false)\.(?:_\w+)?)
 | (?P<dotop>\.(?:eqv|neqv|and|or|not|eq|ne|lt|le|gt|ge)\.)
 | (?P<str>'(?:[^']|'')*'|"(?:[^"]|"")*")
 | (?P<name>[a-z_][a-z0-9_]*)
 | (?P<op>\*\*|//|==|/=|<=|>=|<|>|\+|-|\*|/|\(|\)|,|:|%|=)
""", re.X)


def tokens(s):
    pos, out = 0, []
    while pos < len(s):
        m = _TOKEN.match(s, pos)
        if not m:
            raise SyntaxError(f"cannot read {s[pos:]!r} in {s!r}")
        pos = m.end()
        kind = m.lastgroup
        if kind == "ws":
            continue
        val = m.group(kind)
        if kind == "int_before_dot":
            kind = "int"
        out.append((kind, val))
    return out


# ------------------------------------------------------------------ parser
# nodes: ("int", v) ("real", text, kind) ("log", b) ("str", s) ("name", n)
#        ("ref", n, [args]) ("bin", op, a, b) ("un", op, a) ("slice", lo, hi)

_BINARY = {".eqv.": 10, ".neqv.": 10, ".or.": 20, ".and.": 30,
           ".eq.": 50, ".ne.": 50, ".lt.": 50, ".le.": 50, ".gt.": 50, ".ge.": 50,
           "==": 50, "/=": 50, "<": 50, "<=": 50, ">": 50, ">=": 50,
           "//": 60, "+": 70, "-": 70, "*": 80, "/": 80, "**": 90}
_REL = {".eq.": "==", ".ne.": "!=", ".lt.": "<", ".le.": "<=", ".gt.": ">", ".ge.": ">=",
        "==": "==", "/=": "!=", "<": "<", "<=": "<=", ">": ">", ">=": ">="}


class Parser:
    def __init__(self, text):
        self.t = tokens(text)
        self.i = 0

    def peek(self):
        return self.t[self.i] if self.i < len(self.t) else (None, None)

    def take(self, val=None):
        tok = self.peek()
        if val is not None and tok[1] != val:
            raise SyntaxError(f"expected {val!r}, got {tok!r}")
        self.i += 1
        return tok

    def done(self):
        return self.i >= len(self.t)

    def expr(self, rbp=0):
        left = self.nud()
        while True:
            kind, val = self.peek()
            op = val if kind in ("op", "dotop") else None
            if op not in _BINARY or _BINARY[op] <= rbp:
                break
            self.take()
            bp = _BINARY[op]
            right = self.expr(bp - 1 if op == "**" else bp)
            left = ("bin", op, left, right)
        return left

    def nud(self):
        kind, val = self.take()
        if kind == "int":
            return ("int", int(val.split("_")[0]))
        if kind == "real":
            return ("real",) + _real_literal(val)
        if kind == "logical":
            return ("log", val.startswith(".true."))
        if kind == "str":
            q = val[0]
            return ("str", val[1:-1].replace(q + q, q))
        if kind == "dotop" and val == ".not.":
            return ("un", ".not.", self.expr(40))
        if kind == "op" and val in ("+", "-"):
            return ("un", val, self.expr(75))
        if kind == "op" and val == "(":
            e = self.expr()
            self.take(")")
            return e
        if kind == "name":
            if self.peek()[1] == "(":
                self.take("(")
                args = []
                if self.peek()[1] != ")":
                    while True:
                        args.append(self.subscript())
                        if self.peek()[1] == ",":
                            self.take(",")
                            continue
                        break
                self.take(")")
                return ("ref", val, args)
            return ("name", val)
        raise SyntaxError(f"unexpected {val!r}")

    def subscript(self):
        if self.peek()[1] == ":":
            self.take(":")
            hi = None if self.peek()[1] in (",", ")") else self.expr()
            return ("slice", None, hi)
        e = self.expr()
        if self.peek()[1] == ":":
            self.take(":")
            hi = None if self.peek()[1] in (",", ")") else self.expr()
            return ("slice", e, hi)
        if self.peek()[1] == "=":          # keyword argument (kind=...)
            self.take("=")
            return ("kw", e, self.expr())
        return e


def _real_literal(text):
    kind = None
    if "_" in text:
        text, kind = text.split("_", 1)
    double = "d" in text
    mant = text.replace("d", "e")
    if kind in ("dp", "prec") or double:
        return (mant, "r8")
    if kind is not None:
        raise NotImplementedError(f"real kind {kind}")
    return (mant, "r4")


def parse_expr(text):
    p = Parser(text)
    e = p.expr()
    if not p.done():
        raise SyntaxError(f"trailing tokens in {text!r}: {p.t[p.i:]}")
    return e


# ------------------------------------------------------------------ symbols


class Sym:
    """A variable: type 'i', 'r4', 'r8', 'l' or 's'; rank; where it lives."""

    def __init__(self, name, typ, dims, scope, param=None, intent=None):
        self.name, self.typ, self.dims, self.scope = name, typ, dims, scope
        self.param, self.intent = param, intent

    @property
    def rank(self):
        return len(self.dims)


_TYPESPEC = re.compile(r"^(integer|real|logical|character|double precision)\s*(\([^)]*\)|\*\d+)?")


def _base_type(spec, kind):
    if spec == "integer":
        return "i"
    if spec == "logical":
        return "l"
    if spec == "character":
        return "s"
    if spec == "double precision":
        return "r8"
    k = (kind or "").strip("()").replace("kind=", "").strip()
    if k in ("", "4"):
        return "r4"
    if k in ("dp", "prec", "8"):
        return "r8"
    raise NotImplementedError(f"real kind {k!r}")


def split_top(s, sep=","):
    """Split on sep outside parentheses and strings."""
    parts, depth, q, start = [], 0, None, 0
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
        elif ch == sep and depth == 0:
            parts.append(s[start:i].strip())
            start = i + 1
    parts.append(s[start:].strip())
    return [p for p in parts if p]


def parse_declaration(stmt):
    """A type declaration -> list of (name, typ, dims, init_text, attrs)
    or None when stmt is not one."""
    m = _TYPESPEC.match(stmt)
    if not m:
        return None
    rest = stmt[m.end():]
    if rest.lstrip().startswith("function"):
        raise NotImplementedError("function definitions")
    typ = _base_type(m.group(1), m.group(2))
    if "::" in rest:
        attr_text, ent_text = rest.split("::", 1)
    else:
        attr_text, ent_text = "", rest
    attrs = split_top(attr_text.lstrip(","))
    common_dims = None
    for a in attrs:
        if a.startswith("dimension"):
            common_dims = split_top(a[a.index("(") + 1:a.rindex(")")])
    out = []
    for ent in split_top(ent_text):
        init = None
        if "=" in ent and not ent.startswith("("):
            name_part, init = ent.split("=", 1)
            if init.startswith(">"):
                raise NotImplementedError("pointer initialisation")
        else:
            name_part = ent
        name_part = name_part.strip()
        dims = common_dims
        mm = re.match(r"(\w+)\s*(\((.*)\))?\s*(\*\s*\d+)?$", name_part)
        if not mm:
            raise SyntaxError(f"declaration entity {ent!r}")
        if mm.group(2):
            dims = split_top(mm.group(3))
        out.append((mm.group(1), typ, dims or [], init.strip() if init else None, attrs))
    return out


# ------------------------------------------------------------------ runtime helpers

F4, F8 = np.float32, np.float64


def _idiv(a, b):
    q = abs(a) // abs(b)
    return q if (a >= 0) == (b >= 0) else -q


def _powi(x, n):
    """x**n for an integer constant n as gfortran -O2 expands it
    (__builtin_powi: square-and-multiply on the exponent's bits)."""
    if n < 0:
        return type(x)(1) / _powi(x, -n)
    if n == 0:
        return type(x)(1) if not isinstance(x, int) else 1
    if n == 1:
        return x
    if n == 2:
        return x * x
    if n == 3:
        return x * x * x
    half = _powi(x, n // 2)
    sq = half * half
    return sq * x if n % 2 else sq


def _rpow(x, y):
    if isinstance(x, int) and isinstance(y, int):
        return x ** y
    t = F8 if (type(x) is F8 or type(y) is F8) else F4
    return t(math.pow(float(x), float(y)))


def _libm(fn):
    def f(x):
        t = F8 if type(x) is F8 or isinstance(x, float) else F4
        return t(fn(float(x)))
    return f


def _sqrt(x):
    return np.sqrt(x) if not isinstance(x, int) else np.sqrt(F4(x))


def _abs(x):
    return abs(x)


def _max(*a):
    r = a[0]
    for v in a[1:]:
        if v > r:
            r = v
    return _promote(r, a)


def _min(*a):
    r = a[0]
    for v in a[1:]:
        if v < r:
            r = v
    return _promote(r, a)


def _promote(r, args):
    if any(type(v) is F8 for v in args):
        return F8(r)
    if any(type(v) is F4 for v in args):
        return F4(r)
    return r


def _sign(a, b):
    r = abs(a)
    return r if b >= 0 else -r


def _mod(a, b):
    if isinstance(a, int) and isinstance(b, int):
        return a - _idiv(a, b) * b
    return type(a)(math.fmod(float(a), float(b)))


def _int(x):
    return int(x)    # truncation towards zero


def _nint(x):
    return int(math.floor(float(x) + 0.5)) if x >= 0 else -int(math.floor(-float(x) + 0.5))


INTRINSICS = {
    "abs": ("_abs", None), "dabs": ("_abs", None), "iabs": ("_abs", None),
    "sqrt": ("_sqrt", None), "dsqrt": ("_sqrt", None),
    "max": ("_max", None), "min": ("_min", None), "dmax1": ("_max", None), "dmin1": ("_min", None),
    "amax1": ("_max", None), "amin1": ("_min", None), "max0": ("_max", None), "min0": ("_min", None),
    "sign": ("_sign", None), "dsign": ("_sign", None), "mod": ("_mod", None),
    "exp": ("_exp", None), "dexp": ("_exp", None), "log": ("_log", None), "dlog": ("_log", None),
    "log10": ("_log10", None), "sin": ("_sin", None), "cos": ("_cos", None), "tan": ("_tan", None),
    "atan": ("_atan", None), "tanh": ("_tanh", None), "sinh": ("_sinh", None), "cosh": ("_cosh", None),
    "asin": ("_asin", None), "acos": ("_acos", None), "atan2": ("_atan2", None),
    "dble": ("F8", "r8"), "dfloat": ("F8", "r8"), "float": ("F4", "r4"), "sngl": ("F4", "r4"),
    "int": ("_int", "i"), "nint": ("_nint", "i"), "idint": ("_int", "i"),
    "trim": ("_trim", "s"), "adjustl": ("_adjustl", "s"),
}

_RUNTIME = dict(F4=F4, F8=F8, np=np, _idiv=_idiv, _powi=_powi, _rpow=_rpow, _sqrt=_sqrt, _abs=_abs,
                _max=_max, _min=_min, _sign=_sign, _mod=_mod, _int=_int, _nint=_nint,
                _exp=_libm(math.exp), _log=_libm(math.log), _log10=_libm(math.log10),
                _sin=_libm(math.sin), _cos=_libm(math.cos), _tan=_libm(math.tan), _atan=_libm(math.atan),
                _tanh=_libm(math.tanh), _sinh=_libm(math.sinh), _cosh=_libm(math.cosh),
                _asin=_libm(math.asin), _acos=_libm(math.acos),
                _atan2=lambda y, x: F8(math.atan2(float(y), float(x))),
                _trim=lambda s: s.rstrip(), _adjustl=lambda s: s.lstrip() + " " * (len(s) - len(s.lstrip())))


# ------------------------------------------------------------------ formatted output


def _format_items(fmt):
    """'(3a,1pe10.3,"x",i0)' -> list of edit descriptors, repeats expanded."""
    body = fmt.strip()
    if body.startswith("(") and body.endswith(")"):
        body = body[1:-1]
    items = []
    for it in split_top(body):
        if it[0] in "'\"":
            items.append(("lit", it[1:-1].replace(it[0] * 2, it[0])))
            continue
        g = re.match(r"(\d*)\((.*)\)$", it)
        if g:                                   # group repeat n(...)
            items.extend(_format_items("(" + g.group(2) + ")") * int(g.group(1) or 1))
            continue
        it = it.lower()
        m = re.match(r"(\d*)(x)$", it)
        if m:
            items.append(("lit", " " * int(m.group(1) or 1)))
            continue
        m = re.match(r"(?:(\d+)p)?(\d*)(a|i|es|e|f|g|l)(\d*)(?:\.(\d+))?(?:e(\d+))?$", it)
        if not m:
            raise NotImplementedError(f"edit descriptor {it!r}")
        scale, rep, code, w, d = m.group(1), m.group(2), m.group(3), m.group(4), m.group(5)
        for _ in range(int(rep or 1)):
            items.append((code, int(w) if w else None, int(d) if d else None, int(scale) if scale else 0))
    return items


def _fmt_e(v, w, d, scale):
    v = float(v)
    if scale != 1:
        raise NotImplementedError("E editing without 1P")
    if v == 0.0:
        mant, exp = "0." + "0" * d, 0
        s = f"{mant}E+00"
    else:
        s = f"{abs(v):.{d}e}"          # one digit before the point = 1P scaling
        mant, e = s.split("e")
        exp = int(e)
        s = mant + (f"E{exp:+03d}" if abs(exp) <= 99 else f"{exp:+04d}")
    if v < 0:
        s = "-" + s
    return s.rjust(w) if len(s) <= w else "*" * w


def fortran_format(fmt, values):
    items = _format_items(fmt)
    out, vi = [], 0
    for it in items:
        if it[0] == "lit":
            out.append(it[1])
            continue
        if vi >= len(values):
            break
        code, w, d, scale = it
        v = values[vi]
        vi += 1
        if code == "a":
            s = str(v)
            out.append(s if w is None else s[:w].rjust(w))
        elif code == "i":
            s = str(int(v))
            out.append(s if not w else (s.rjust(w) if len(s) <= w else "*" * w))
        elif code in ("e", "es"):
            out.append(_fmt_e(v, w, d, scale if code == "e" else 1))
        elif code == "f":
            out.append(f"{float(v):{w}.{d}f}")
        elif code == "l":
            out.append(("T" if v else "F").rjust(w or 1))
        else:
            raise NotImplementedError(code)
    return "".join(out)


# ------------------------------------------------------------------ translator


class Translator:
    """One subroutine -> Python source of a function f(M, *args)."""

    def __init__(self, mod_syms, routines, stub_functions=(), functions=None):
        self.mod = mod_syms          # name -> Sym (scope 'mod')
        self.routines = routines     # name -> (dummies) of routines that can be called
        self.stub_functions = set(stub_functions)
        self.functions = dict(functions or {})   # translated functions -> result type
        self.consts = {}

    # -- names
    def sym(self, n):
        if n in self.loc:
            return self.loc[n]
        if n in self.mod:
            return self.mod[n]
        return None

    def var(self, n):
        s = self.sym(n)
        if s is None:
            raise NameError(f"{n} is not declared (routine {self.rname})")
        if s.param is not None:
            return self.const_name(n, s)
        if s.scope == "mod":
            return f"A_{n}" if s.rank else f"M.m_{n}"
        return f"L_{n}"

    def const_name(self, n, s):
        return f"P_{n}"

    def lit_r(self, text, kind):
        key = (text, kind)
        if key not in self.consts:
            self.consts[key] = f"K{len(self.consts)}"
        return self.consts[key]

    # -- types
    def ty(self, e):
        k = e[0]
        if k == "int":
            return "i"
        if k == "real":
            return e[2]
        if k == "log":
            return "l"
        if k == "str":
            return "s"
        if k == "name":
            s = self.sym(e[1])
            if s is None:
                raise NameError(e[1])
            return s.typ
        if k == "ref":
            s = self.sym(e[1])
            if s is not None and (s.rank or s.typ == "s"):
                return s.typ
            if e[1] in self.stub_functions:
                return "r8"
            if e[1] in self.functions:
                return self.functions[e[1]]
            if e[1] == "real":
                kw = [a for a in e[2] if a[0] == "kw"]
                pos = [a for a in e[2] if a[0] != "kw"]
                return self.kind_of(kw[0][2] if kw else (pos[1] if len(pos) > 1 else None))
            name, rt = INTRINSICS.get(e[1], (None, None))
            if name is None:
                raise NameError(f"unknown function or array {e[1]}")
            if rt:
                return rt
            args = [a for a in e[2] if a[0] != "kw"]
            tys = [self.ty(a) for a in args]
            return "r8" if "r8" in tys else ("r4" if "r4" in tys else "i")
        if k == "bin":
            op = e[1]
            if op in _REL or op in (".and.", ".or.", ".eqv.", ".neqv."):
                return "l"
            if op == "//":
                return "s"
            a, b = self.ty(e[2]), self.ty(e[3])
            if a == "i" and b == "i":
                return "i"
            return "r8" if "r8" in (a, b) else "r4"
        if k == "un":
            return "l" if e[1] == ".not." else self.ty(e[2])
        raise TypeError(e)

    # -- expressions
    def ex(self, e):
        k = e[0]
        if k == "int":
            return str(e[1])
        if k == "real":
            return self.lit_r(e[1], e[2])
        if k == "log":
            return "True" if e[1] else "False"
        if k == "str":
            return repr(e[1])
        if k == "name":
            return self.var(e[1])
        if k == "ref":
            return self.ref(e)
        if k == "un":
            if e[1] == ".not.":
                return f"(not {self.ex(e[2])})"
            return f"({e[1]}{self.ex(e[2])})"
        if k == "bin":
            op, a, b = e[1], e[2], e[3]
            if op in _REL:
                return f"({self.ex(a)} {_REL[op]} {self.ex(b)})"
            if op in (".and.", ".or."):
                return f"({self.ex(a)} {op.strip('.')} {self.ex(b)})"
            if op == ".eqv.":
                return f"({self.ex(a)} == {self.ex(b)})"
            if op == ".neqv.":
                return f"({self.ex(a)} != {self.ex(b)})"
            if op == "//":
                return f"({self.ex(a)} + {self.ex(b)})"
            if op == "/" and self.ty(a) == "i" and self.ty(b) == "i":
                return f"_idiv({self.ex(a)}, {self.ex(b)})"
            if op == "**":
                if b[0] == "int":
                    return f"_powi({self.ex(a)}, {b[1]})"
                if b[0] == "un" and b[1] == "-" and b[2][0] == "int":
                    return f"_powi({self.ex(a)}, {-b[2][1]})"
                return f"_rpow({self.ex(a)}, {self.ex(b)})"
            return f"({self.ex(a)} {op} {self.ex(b)})"
        raise TypeError(e)

    def ref(self, e):
        n, args = e[1], e[2]
        s = self.sym(n)
        if s is not None and s.rank:
            return f"{self.var(n)}[{', '.join(self.sub(a) for a in args)}]"
        if s is not None and s.typ == "s":
            raise NotImplementedError("substrings")
        if n in self.stub_functions:
            return f"_fstub({n!r})"
        if n in self.functions:
            codes = []
            for a in args:
                s2 = self.sym(a[1]) if a[0] == "name" else None
                codes.append(self.var(a[1]) if s2 is not None and s2.rank else self.ex(a))
            return f"M.call({n!r}{''.join(', ' + c for c in codes)})"
        if n == "real":
            kw = [a for a in args if a[0] == "kw"]
            pos = [a for a in args if a[0] != "kw"]
            kind = self.kind_of(kw[0][2] if kw else (pos[1] if len(pos) > 1 else None))
            return f"{'F8' if kind == 'r8' else 'F4'}({self.ex(pos[0])})"
        if n not in INTRINSICS:
            raise NameError(f"unknown function or array {n} (routine {self.rname})")
        fn = INTRINSICS[n][0]
        return f"{fn}({', '.join(self.ex(a) for a in args if a[0] != 'kw')})"

    def kind_of(self, e):
        if e is None:
            return "r4"
        if e[0] == "name" and e[1] in ("dp", "prec"):
            return "r8"
        if e[0] == "int" and e[1] == 8:
            return "r8"
        if e[0] == "int" and e[1] == 4:
            return "r4"
        raise NotImplementedError(f"kind {e}")

    def sub(self, a):
        if a[0] == "slice":
            lo = "" if a[1] is None else self.ex(a[1])
            hi = "" if a[2] is None else f"({self.ex(a[2])}) + 1"
            return f"{lo}:{hi}"
        return self.ex(a)

    # -- statements
    def translate(self, name, dummies, body, result=None):
        self.rname = name
        self.result = result
        self.loc = {}
        self.dummies = dummies
        self.lines = []
        self.ind = 1
        self.nloop = 0
        decls, exec_start = [], 0
        for i, st in enumerate(body):
            if st.startswith("use ") or st == "use" or st.startswith("implicit"):
                continue
            d = parse_declaration(st)
            if d is None:
                exec_start = i
                break
            decls.extend(d)
        else:
            exec_start = len(body)
        for n, typ, dims, init, attrs in decls:
            intent = next((a for a in attrs if a.startswith("intent")), None)
            param = init if "parameter" in attrs else None
            self.loc[n] = Sym(n, typ, dims, "arg" if n in dummies else "loc", param, intent)
        for d in dummies:
            if d not in self.loc:
                raise NameError(f"dummy {d} of {name} has no declaration")
        # prologue: parameters, local arrays, module arrays
        pro = []
        for n, s in self.loc.items():
            if s.param is not None:
                pro.append(f"P_{n} = {self.cast(s.typ, self.ex(parse_expr(s.param)))}")
        for n, s in self.loc.items():
            if s.scope == "loc" and s.param is None:
                if s.rank:
                    shape = ", ".join(f"({self.ex(parse_expr(d))}) + 1" for d in s.dims)
                    dt = {"i": "np.int64", "r4": "np.float32", "r8": "np.float64", "l": "bool"}[s.typ]
                    # local work arrays start at zero (their contents are undefined in Fortran)
                    pro.append(f"L_{n} = np.zeros(({shape},), dtype={dt})")
                else:
                    pro.append(f"L_{n} = {self.zero(s.typ)}")
        body_exec = body[exec_start:]
        used = set(re.findall(r"[a-z_][a-z0-9_]*", " ".join(body_exec)))
        for n in sorted(used):
            s = self.mod.get(n)
            if s is not None and n not in self.loc and s.rank and s.param is None:
                pro.append(f"A_{n} = M.m_{n}")
        for p in pro:
            self.emit(p)
        self.block(body_exec)
        self.emit("return " + self.ret_tuple())
        head = f"def R_{name}(M, {', '.join('L_' + d for d in dummies)}):"
        return "\n".join([head] + self.lines)

    def ret_tuple(self):
        if self.result is not None:          # a function returns its result variable
            return f"L_{self.result}"
        return "(" + "".join(f"L_{d}, " for d in self.dummies) + ")"

    def zero(self, typ):
        return {"i": "0", "r4": "F4(0)", "r8": "F8(0)", "l": "False", "s": "''"}[typ]

    def cast(self, typ, code):
        return {"i": f"_int({code})", "r4": f"F4({code})", "r8": f"F8({code})",
                "l": f"bool({code})", "s": code}[typ]

    def emit(self, line):
        self.lines.append("    " * self.ind + line)

    def block(self, stmts):
        i = 0
        while i < len(stmts):
            i = self.stmt(stmts, i)

    def stmt(self, stmts, i):
        st = stmts[i]
        st = re.sub(r"^\d+\s+", "", st)     # statement labels
        m = re.match(r"do\s+(\w+)\s*=\s*(.*)$", st)
        if m and not st.startswith("do while"):
            var, rng = m.group(1), split_top(m.group(2))
            end = self.find_end(stmts, i, "do")
            lo, hi = self.ex(parse_expr(rng[0])), self.ex(parse_expr(rng[1]))
            step = self.ex(parse_expr(rng[2])) if len(rng) > 2 else "1"
            v = self.var(var)
            self.nloop += 1
            t = f"_d{self.nloop}"
            self.emit(f"{t}lo, {t}hi, {t}st = {lo}, {hi}, {step}")
            self.emit(f"for {v} in range({t}lo, {t}hi + (1 if {t}st > 0 else -1), {t}st):")
            self.ind += 1
            n0 = len(self.lines)
            self.block(stmts[i + 1:end])
            if len(self.lines) == n0:
                self.emit("pass")
            self.ind -= 1
            self.emit("else:")
            self.ind += 1
            self.emit(f"{v} = {t}lo + max(0, ({t}hi - {t}lo + {t}st) // {t}st) * {t}st")
            self.ind -= 1
            return end + 1
        m = re.match(r"do\s+while\s*\((.*)\)$", st)
        if m:
            end = self.find_end(stmts, i, "do")
            self.emit(f"while {self.ex(parse_expr(m.group(1)))}:")
            self.ind += 1
            self.block(stmts[i + 1:end])
            self.emit("pass")
            self.ind -= 1
            return end + 1
        if re.match(r"if\s*\(", st):
            cond, rest = self.paren(st[2:].lstrip())
            if rest.strip() == "then":
                return self.if_block(stmts, i, cond)
            self.emit(f"if {self.ex(parse_expr(cond))}:")
            self.ind += 1
            self.simple(rest.strip())
            self.ind -= 1
            return i + 1
        self.simple(st)
        return i + 1

    def paren(self, s):
        assert s.startswith("(")
        depth, q = 0, None
        for j, ch in enumerate(s):
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
                    return s[1:j], s[j + 1:]
        raise SyntaxError(s)

    @staticmethod
    def is_end(st, kind):
        st = re.sub(r"^\d+\s+", "", st)
        return bool(re.match(r"end\s*%s\b" % kind, st))

    @staticmethod
    def opens(st, kind):
        st = re.sub(r"^\d+\s+", "", st)
        if kind == "do":
            return bool(re.match(r"do\b(?!\s*\d)", st))
        if kind == "if":
            if not re.match(r"(else\s*)?if\s*\(", st) or st.startswith("else"):
                return False
            return st.rstrip().endswith("then")
        return False

    def find_end(self, stmts, i, kind):
        depth = 0
        for j in range(i, len(stmts)):
            if self.opens(stmts[j], kind):
                depth += 1
            elif self.is_end(stmts[j], kind):
                depth -= 1
                if depth == 0:
                    return j
        raise SyntaxError(f"no end {kind} for {stmts[i]!r}")

    def if_block(self, stmts, i, cond):
        end = self.find_end(stmts, i, "if")
        # split at else if / else of depth 1
        branches, start, depth, cur_cond = [], i + 1, 0, cond
        for j in range(i + 1, end):
            st = stmts[j]
            if self.opens(st, "if"):
                depth += 1
            elif self.is_end(st, "if"):
                depth -= 1
            elif depth == 0 and re.match(r"else\s*if\s*\(", st):
                branches.append((cur_cond, stmts[start:j]))
                c, rest = self.paren(re.sub(r"^else\s*if\s*", "", st))
                assert rest.strip() == "then", st
                cur_cond, start = c, j + 1
            elif depth == 0 and st == "else":
                branches.append((cur_cond, stmts[start:j]))
                cur_cond, start = None, j + 1
        branches.append((cur_cond, stmts[start:end]))
        for bi, (c, body) in enumerate(branches):
            if c is None:
                self.emit("else:")
            else:
                self.emit(f"{'if' if bi == 0 else 'elif'} {self.ex(parse_expr(c))}:")
            self.ind += 1
            n0 = len(self.lines)
            self.block(body)
            if len(self.lines) == n0:
                self.emit("pass")
            self.ind -= 1
        return end + 1

    def simple(self, st):
        st = re.sub(r"^\d+\s+", "", st)
        if st == "exit":
            return self.emit("break")
        if st == "cycle":
            return self.emit("continue")
        if st == "return":
            return self.emit("return " + self.ret_tuple())
        if st == "continue":
            return self.emit("pass")
        if st.startswith("call "):
            return self.call(st[5:].strip())
        if st.startswith("write") and st[5:].lstrip().startswith("("):
            return self.write(st)
        if st.startswith(("print ", "print*")):
            return self.emit("pass")
        m = re.match(r"([a-z_]\w*)\s*(\(.*?\))?\s*=(?!=)(.*)$", st)
        if m:
            return self.assign(st)
        raise NotImplementedError(f"statement {st!r} in {self.rname}")

    def assign(self, st):
        lhs_text, rhs_text = self.split_assign(st)
        lhs = parse_expr(lhs_text)
        rhs = parse_expr(rhs_text)
        code = self.ex(rhs)
        if lhs[0] == "name":
            s = self.sym(lhs[1])
            if s is None:
                raise NameError(f"{lhs[1]} is not declared (routine {self.rname})")
            if s.rank:
                return self.emit(f"{self.var(lhs[1])}[...] = {code}")
            return self.emit(f"{self.var(lhs[1])} = {self.cast(s.typ, code)}")
        if lhs[0] == "ref":
            s = self.sym(lhs[1])
            if s is None or not s.rank:
                raise NameError(f"assignment to {lhs[1]}")
            return self.emit(f"{self.ref(lhs)} = {code}")
        raise SyntaxError(st)

    @staticmethod
    def split_assign(st):
        depth, q = 0, None
        for j, ch in enumerate(st):
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
            elif ch == "=" and depth == 0 and st[j + 1:j + 2] != "=" and st[j - 1] not in "<>/=":
                return st[:j].strip(), st[j + 1:].strip()
        raise SyntaxError(st)

    def call(self, text):
        m = re.match(r"(\w+)\s*(\((.*)\))?\s*$", text)
        name = m.group(1)
        args = split_top(m.group(3)) if m.group(3) else []
        if name in NOOP_CALLS:
            return self.emit("pass")
        if name not in self.routines:
            raise NameError(f"call of {name} from {self.rname}: not in the executed set")
        exprs = [parse_expr(a) for a in args]
        codes = []
        for e in exprs:
            if e[0] == "name" and self.sym(e[1]) is not None and self.sym(e[1]).rank:
                codes.append(self.var(e[1]))
            elif e[0] == "ref" and any(a[0] == "slice" for a in e[2]):
                codes.append(self.ref(e))
            else:
                codes.append(self.ex(e))
        res = f"_r = M.call({name!r}, {', '.join(codes)}{',' if len(codes) == 1 else ''})"
        self.emit(res)
        for k, e in enumerate(exprs):           # scalar actuals by reference
            if e[0] == "name" and self.sym(e[1]) is not None and not self.sym(e[1]).rank \
                    and self.sym(e[1]).param is None:
                self.emit(f"{self.var(e[1])} = _r[{k}]")
            elif e[0] == "ref" and self.sym(e[1]) is not None and self.sym(e[1]).rank \
                    and not any(a[0] == "slice" for a in e[2]):
                self.emit(f"{self.ref(e)} = _r[{k}]")

    def write(self, st):
        ctl, rest = self.paren(st[5:].lstrip())
        parts = split_top(ctl)
        unit = self.ex(parse_expr(parts[0])) if parts[0] != "*" else "6"
        fmt = parts[1] if len(parts) > 1 else "*"
        if fmt.startswith("fmt="):
            fmt = fmt[4:]
        items = split_top(rest.strip())
        vals = ", ".join(self.ex(parse_expr(x)) for x in items)
        if fmt == "*":
            self.emit(f"M.write({unit}, None, [{vals}])")
        else:
            f = parse_expr(fmt)
            if f[0] != "str":
                raise NotImplementedError(f"format {fmt}")
            self.emit(f"M.write({unit}, {f[1]!r}, [{vals}])")


# kind parameters of module types (modules_allocatable.f90:1-13): double precision
KIND_PARAMS = {"dp": 8, "prec": 8}

# first extents of the module's rank-2 and rank-3 allocatables (allocate.f90)
FIRST_EXTENTS = {"gradu": (3,), "gradv": (3,), "gradw": (3,), "gradte": (3,), "graded": (3,), "gradp": (3,),
                 "gradt": (3,), "gradvart": (3,), "gradcon": (3,), "d": (6,), "bij": (5,), "dqr": (3, 6)}

# single-rank MPI routines: no neighbours, sums and maxima over one rank
NOOP_CALLS = {"global_sum", "global_max", "global_isum", "exchange", "exchange_mpi"}


# ------------------------------------------------------------------ program


class Namespace:
    """Module variables of one run; arrays are numpy with a leading pad."""

    def __init__(self, program):
        self._prog = program
        self.units = {}

    def get(self, name):
        return getattr(self, "m_" + name)

    def set(self, name, value):
        setattr(self, "m_" + name, value)

    def write(self, unit, fmt, vals):
        text = fortran_format(fmt, vals) if fmt else " ".join(str(v) for v in vals)
        self.units.setdefault(int(unit), []).append(text)

    def call(self, name, *args):
        return self._prog.funcs[name](self, *args)


_FUNCTION = re.compile(r"(?:(?:pure|elemental|recursive)\s+)*(?:(?:real|integer|logical)(?:\([^)]*\))?\s+)?"
                       r"function\s+(\w+)\s*\(([^)]*)\)\s*(?:result\s*\(\s*(\w+)\s*\))?\s*$")


def _stub(name):
    def f(*_):
        raise RuntimeError(f"{name} was called: it is outside the executed set")
    return f


class Program:
    """Module declarations plus translated subroutines of reference files."""

    def __init__(self, module_text):
        self.mod = {}
        self.mod_params = {}
        self.funcs = {}
        self.sources = {}
        self.subs = {}
        self.fsubs = {}      # functions: name -> (dummies, body, result variable)
        for st in statements(module_text):
            if st.startswith(("module", "end module", "use ", "implicit", "end")):
                continue
            d = parse_declaration(st)
            if d is None:
                continue
            for n, typ, dims, init, attrs in d:
                param = init if "parameter" in attrs else None
                if n in self.mod:
                    raise NameError(f"module variable {n} declared twice")
                self.mod[n] = Sym(n, typ, dims, "mod", param)
                if init is not None and param is None:
                    self.mod_params[n] = init      # initialised module variable (chvar, ...)

    def add_snippet(self, name, text, include_dir=None):
        """Statements cut from a larger routine (e.g. the constant
        assignments of init.f90), run as a subroutine without arguments
        that uses every module."""
        self.add_source(f"subroutine {name}\n{text}\nend subroutine\n", include_dir=include_dir)

    def add_source(self, text, only=None, include_dir=None):
        """Add the subroutines of one source file; INCLUDE lines are
        replaced by the statements of the named file in include_dir."""
        st = []
        for s in statements(text):
            m = re.match(r"include\s+['\"]([^'\"]+)['\"]$", s)
            if m:
                if include_dir is None:
                    raise NotImplementedError(f"include {m.group(1)} without an include directory")
                st.extend(statements((pathlib.Path(include_dir) / m.group(1)).read_text()))
            else:
                st.append(s)
        i = 0
        while i < len(st):
            m = re.match(r"subroutine\s+(\w+)\s*(\((.*)\))?\s*$", st[i])
            fm = _FUNCTION.match(st[i])
            if not m and not fm:
                i += 1
                continue
            kind = "subroutine" if m else "function"
            name = (m or fm).group(1)
            arglist = m.group(3) if m else fm.group(2)
            dummies = split_top(arglist) if arglist else []
            j = i + 1
            while not re.match(r"end(\s*%s\b.*)?$" % kind, st[j]):
                if st[j].startswith(("contains", "subroutine ")) or _FUNCTION.match(st[j]):
                    raise NotImplementedError(f"internal procedures in {name}")
                j += 1
            if only is None or name in only:
                if m:
                    self.subs[name] = (dummies, st[i + 1:j])
                else:
                    self.fsubs[name] = (dummies, st[i + 1:j], fm.group(3) or name)
            i = j + 1

    def compile(self, stubs=()):
        """Translate every added subroutine.  stubs: routines that the
        translated code calls on branches these runs do not take; calling
        one raises."""
        routines = {n: d for n, (d, _) in self.subs.items()}
        for n in stubs:
            routines.setdefault(n, None)
        ftypes = {}
        for n, (dummies, body, res) in self.fsubs.items():
            for st in body:
                d = parse_declaration(st)
                for ent in d or []:
                    if ent[0] == res:
                        ftypes[n] = ent[1]
            if n not in ftypes:
                raise NameError(f"function {n}: no declaration of its result {res}")
        tr = Translator(self.mod, routines, stub_functions=stubs, functions=ftypes)
        mod_consts = []
        for n, s in self.mod.items():
            if s.param is not None:
                tr.loc = {}
                tr.rname = "module"
                if n in KIND_PARAMS:
                    mod_consts.append(f"P_{n} = {KIND_PARAMS[n]}")
                    continue
                mod_consts.append(f"P_{n} = {tr.cast(s.typ, tr.ex(parse_expr(s.param)))}")
        srcs = []
        for n, (dummies, body) in self.subs.items():
            srcs.append(tr.translate(n, dummies, body))
        for n, (dummies, body, res) in self.fsubs.items():
            srcs.append(tr.translate(n, dummies, body, result=res))
        konst = [f"{v} = {'exact_f32' if k[1] == 'r4' else 'F8'}({k[0]!r})" for k, v in tr.consts.items()]
        code = "\n".join(konst + mod_consts + srcs)
        g = dict(_RUNTIME)
        g["exact_f32"] = exact_f32
        g["_fstub"] = lambda name: _stub(name)()
        exec(compile(code, "<reference>", "exec"), g)
        self.code = code
        for n in list(self.subs) + list(self.fsubs):
            self.funcs[n] = g["R_" + n]
        for n in stubs:
            if n not in self.subs:
                self.funcs[n] = _stub(n)
        self.mod_const_values = {n: g["P_" + n] for n, s in self.mod.items() if s.param is not None}
        return self

    def namespace(self, dims):
        """Module arrays allocated as allocate.f90 would for an ni x nj x nk
        grid (1-D fields of length nxyza = ni*nj*nk, (3,nxyza) gradients)."""
        ns = Namespace(self)
        ni, nj, nk = dims
        nijk = ni * nj * nk
        env = {"nxyza": nijk, "nxyz": nijk, "nphi": 10, "ni": ni, "nj": nj, "nk": nk, "nx": ni, "ny": nj, "nz": nk}
        for n, s in self.mod.items():
            if s.param is not None:
                ns.set(n, self.mod_const_values[n])
                continue
            dt = {"i": np.int64, "r4": np.float32, "r8": np.float64, "l": bool, "s": object}[s.typ]
            if s.rank == 0:
                ns.set(n, {"i": 0, "r4": F4(0), "r8": F8(0), "l": False, "s": ""}[s.typ])
                continue
            if s.dims[0] == ":":
                lead = FIRST_EXTENTS.get(n, (1,) * (s.rank - 1))
                shape = tuple(e + 1 for e in lead) + (nijk + 1,)
            else:
                shape = tuple(int(eval(d, {}, env)) + 1 for d in s.dims)
            if s.typ == "s":
                arr = np.full(shape, "", dtype=object)
                init = self.mod_params.get(n)
                if init:
                    body = init.strip()[2:-2]
                    for k, item in enumerate(split_top(body)):
                        arr[k + 1] = item[1:-1]
                ns.set(n, arr)
                continue
            ns.set(n, np.zeros(shape, dtype=dt))
        # extents of set_parameters.f90:34-41 (nx = nicv+2 ... = ni, nj, nk of
        # the storage) and the work-array length nxyza (= nxyz, set once)
        ext = dict(nx=ni, ny=nj, nz=nk, nxy=ni * nj, nxz=ni * nk, nyz=nj * nk, nxyz=nijk, nxyza=nijk,
                   ni=ni, nj=nj, nk=nk)
        for n, v in ext.items():
            ns.set(n, v)
        return ns
