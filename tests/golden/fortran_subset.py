"""Run the reference's own Fortran 90 source, on one rank, on the CPU.

The reference (Fortran 90 + MPI + 2DECOMP&FFT + FFTW + HDF5 + LAPACK) cannot
be compiled in this image: there is no Fortran compiler, MPI, FFTW or LAPACK
library.  This module translates the subset of Fortran 90 that the time-step
routines of the reference use into Python, statement by statement, and
supplies a one-rank runtime for what those routines call outside the
reference tree:

* LAPACK ``?gttrf``/``?gttrs``: the real LAPACK routines, through SciPy;
* FFTW guru plans: recorded when planned, executed with ``numpy.fft``
  (pocketfft) over the same lengths, strides and batch dimensions;
* 2DECOMP&FFT on one rank: ``decomp_2d_init`` and the pencil descriptors,
  the transposes as element copies (what ``mem_split``/``mem_merge`` do with
  a single block), ``update_halo`` as the one-rank branch of
  ``halo_common.f90`` (the in-memory copies of its periodic planes);
* MPI on one rank: broadcasts and reductions are identities;
* HDF5: the continua fields that ``ReadFlowField`` reads come from arrays the
  caller supplies; the ``HdfRoutines.F90`` writers (``HdfCreateBlankFile``,
  the serial scalar, 1-D and 2-D writers, ``HdfWriteReal2D``,
  ``HdfWriteRealHalo3D``) record the datasets they leave in each file, with
  the files' create-or-open semantics, and the readers of scalars and 2-D
  arrays read those files back (statistics read at a restart);
* ``QuitRoutine`` on a normal exit runs the reference's ``WriteStats`` and
  ``WriteFlowField`` before the stop;
* list-directed ``read`` from texts the caller supplies (``bou.in``,
  ``rcuts.in``; a single implied-DO list is expanded), internal ``write``
  with I edit descriptors (the time tags of the dump file names); records
  written to chosen units (97: ``CalcTorque``, 92: ``CalcDissipation``, 98:
  the velocity rms of ``CalcVelocityStats``) are kept.

Arithmetic follows gfortran's x86-64 code for ``-O3 -fdefault-real-8``
(no FMA contraction on that target): every real is a binary64, expressions
evaluate in their parse order with parentheses honoured, ``x**2`` and ``x**3``
are the products ``x*x`` and ``(x*x)*x`` (gfortran's expansion of integer
powers), a complex divided by a real divides both parts by it, ``mod`` of
reals is ``fmod``.  OpenMP directives are comments, i.e. the serial
semantics (the reference's OpenMP clauses are racy).  Automatic and locally
allocated real arrays start as NaN, so a read of an undefined value shows up
in the results instead of passing silently.

This is test infrastructure: tests/golden/make_reference_runs.py uses it to
write the golden fixtures under tests/golden/.  Nothing in the library, the
benchmark or the GPU tests imports it.
"""
from __future__ import annotations

import keyword
import math
import os
import re
import sys
import types

import numpy as np

np.seterr(all="ignore")

# --------------------------------------------------------------------------
# Source text: preprocessing, comments, continuation lines
# --------------------------------------------------------------------------


def preprocess(path, defines, _depth=0):
    """Lines of `path` after the cpp directives the reference uses
    (#ifdef/#ifndef/#else/#endif/#include); dropped lines become blank so
    that line numbers stay those of the file."""
    with open(path) as f:
        text = f.read()
    out, stack = [], []
    for line in text.split("\n"):
        s = line.strip()
        if s.startswith("#"):
            parts = s[1:].split()
            d = parts[0] if parts else ""
            if d == "ifdef":
                stack.append(parts[1] in defines)
            elif d == "ifndef":
                stack.append(parts[1] not in defines)
            elif d == "else":
                stack[-1] = not stack[-1]
            elif d == "endif":
                stack.pop()
            elif d == "include" and all(stack):
                inc = os.path.join(os.path.dirname(path), parts[1].strip('"<>'))
                out.extend(preprocess(inc, defines, _depth + 1))
                continue
            out.append("")
            continue
        out.append(line if all(stack) else "")
    return out


def _strip_comment(line):
    res, q = [], None
    for ch in line:
        if q:
            res.append(ch)
            if ch == q:
                q = None
        elif ch in "\"'":
            q = ch
            res.append(ch)
        elif ch == "!":
            break
        else:
            res.append(ch)
    return "".join(res)


def _lower_code(s):
    res, q = [], None
    for ch in s:
        if q:
            res.append(ch)
            if ch == q:
                q = None
        elif ch in "\"'":
            q = ch
            res.append(ch)
        else:
            res.append(ch.lower())
    return "".join(res)


def statements(lines):
    """(line number, label, statement text) of each free-form statement:
    comments removed, continuation lines joined, code lowercased."""
    buf, start = None, 0
    for no, raw in enumerate(lines, 1):
        st = _strip_comment(raw).strip()
        if not st:
            continue
        if buf is not None and st.startswith("&"):
            st = st[1:]
            joiner = ""
        else:
            joiner = " "
        cont = st.endswith("&")
        if cont:
            st = st[:-1].rstrip()
        if buf is None:
            buf, start = st, no
        else:
            buf = buf + joiner + st
        if not cont:
            text = _lower_code(buf).strip()
            buf = None
            label = None
            m = re.match(r"^(\d+)\s+(.*)$", text)
            if m:
                label, text = int(m.group(1)), m.group(2)
            for part in _split_top(text, ";"):
                if part.strip():
                    yield start, label, part.strip()


def _split_top(s, sep=","):
    """Split at `sep` outside parentheses and strings."""
    out, depth, q, cur = [], 0, None, []
    for ch in s:
        if q:
            cur.append(ch)
            if ch == q:
                q = None
            continue
        if ch in "\"'":
            q = ch
        elif ch == "(":
            depth += 1
        elif ch == ")":
            depth -= 1
        elif ch == sep and depth == 0:
            out.append("".join(cur))
            cur = []
            continue
        cur.append(ch)
    out.append("".join(cur))
    return out


def _match_paren(s, i):
    """Index of the parenthesis closing the one at s[i]."""
    depth, q = 0, None
    for j in range(i, len(s)):
        ch = s[j]
        if q:
            if ch == q:
                q = None
            continue
        if ch in "\"'":
            q = ch
        elif ch == "(":
            depth += 1
        elif ch == ")":
            depth -= 1
            if depth == 0:
                return j
    raise SyntaxError("unbalanced parentheses: " + s)


def _top_assign(s):
    """Index of a top-level '=' that makes `s` an assignment, or -1."""
    depth, q = 0, None
    for j, ch in enumerate(s):
        if q:
            if ch == q:
                q = None
            continue
        if ch in "\"'":
            q = ch
        elif ch == "(":
            depth += 1
        elif ch == ")":
            depth -= 1
        elif ch == "=" and depth == 0:
            prev = s[j - 1] if j else ""
            nxt = s[j + 1] if j + 1 < len(s) else ""
            if nxt == "=" or prev in "=/<>":
                continue
            return j
    return -1


# --------------------------------------------------------------------------
# Expressions
# --------------------------------------------------------------------------

_DOTOPS = "eq|ne|lt|le|gt|ge|and|or|not|eqv|neqv|true|false"
_TOKEN = re.compile(
    r"(?P<ws>\s+)"
    r"|(?P<str>'(?:[^']|'')*'|\"(?:[^\"]|\"\")*\")"
    r"|(?P<real>(?:\d+\.\d*(?!(?:" + _DOTOPS + r")\.)|\.\d+)(?:[ed][+-]?\d+)?(?:_\w+)?|\d+[ed][+-]?\d+(?:_\w+)?)"
    r"|(?P<int>\d+(?:_\w+)?)"
    r"|(?P<dotop>\.(?:" + _DOTOPS + r")\.)"
    r"|(?P<name>[a-z_]\w*)"
    r"|(?P<op>\*\*|//|==|/=|<=|>=|\(/|/\)|[-+*/<>=(),:%])")


def tokenize(s):
    toks, pos = [], 0
    while pos < len(s):
        m = _TOKEN.match(s, pos)
        if not m:
            raise SyntaxError(f"cannot tokenize {s[pos:]!r} in {s!r}")
        pos = m.end()
        kind = m.lastgroup
        if kind == "ws":
            continue
        toks.append((kind, m.group(kind)))
    toks.append(("end", None))
    return toks


class Parser:
    """Recursive descent over Fortran's operator precedence.  Nodes are
    tuples: ('num', value, type), ('str', s), ('log', bool), ('name', n),
    ('ref', base, args) for name(args) (array element, section or call),
    ('comp', base, field), ('bin', op, a, b), ('un', op, a),
    ('slice', lo, hi, step), ('kw', name, expr), ('cplx', re, im),
    ('arr', items)."""

    _REL = {"==": "==", "/=": "!=", "<": "<", "<=": "<=", ">": ">", ">=": ">=", ".eq.": "==", ".ne.": "!=",
            ".lt.": "<", ".le.": "<=", ".gt.": ">", ".ge.": ">="}

    def __init__(self, text):
        self.t = tokenize(text)
        self.i = 0
        self.text = text

    def peek(self, k=0):
        return self.t[self.i + k]

    def take(self, val=None):
        tok = self.t[self.i]
        if val is not None and tok[1] != val:
            raise SyntaxError(f"expected {val!r}, got {tok[1]!r} in {self.text!r}")
        self.i += 1
        return tok

    def at(self, val):
        return self.t[self.i][1] == val

    def parse_all(self):
        e = self.expr()
        if self.peek()[0] != "end":
            raise SyntaxError(f"trailing text in {self.text!r}")
        return e

    def expr(self):
        a = self.or_()
        while self.at(".eqv.") or self.at(".neqv."):
            op = "==" if self.take()[1] == ".eqv." else "!="
            a = ("bin", op, a, self.or_())
        return a

    def or_(self):
        a = self.and_()
        while self.at(".or."):
            self.take()
            a = ("bin", "or", a, self.and_())
        return a

    def and_(self):
        a = self.not_()
        while self.at(".and."):
            self.take()
            a = ("bin", "and", a, self.not_())
        return a

    def not_(self):
        if self.at(".not."):
            self.take()
            return ("un", "not", self.not_())
        return self.rel()

    def rel(self):
        a = self.concat()
        tok = self.peek()[1]
        if tok in self._REL:
            self.take()
            a = ("bin", self._REL[tok], a, self.concat())
        return a

    def concat(self):
        a = self.add()
        while self.at("//"):
            self.take()
            a = ("bin", "//", a, self.add())
        return a

    def add(self):
        if self.at("-") or self.at("+"):
            op = self.take()[1]
            a = self.mul()
            if op == "-":
                a = ("un", "-", a)
        else:
            a = self.mul()
        while self.at("+") or self.at("-"):
            op = self.take()[1]
            a = ("bin", op, a, self.mul())
        return a

    def mul(self):
        a = self.power()
        while self.at("*") or self.at("/"):
            op = self.take()[1]
            a = ("bin", op, a, self.power())
        return a

    def power(self):
        a = self.primary()
        if self.at("**"):
            self.take()
            if self.at("-") or self.at("+"):
                op = self.take()[1]
                b = self.power()
                b = ("un", "-", b) if op == "-" else b
            else:
                b = self.power()
            return ("bin", "**", a, b)
        return a

    def primary(self):
        kind, val = self.peek()
        if kind == "real":
            self.take()
            v = re.sub(r"_\w+$", "", val).replace("d", "e")
            return ("num", float(v), "r")
        if kind == "int":
            self.take()
            return ("num", int(re.sub(r"_\w+$", "", val)), "i")
        if kind == "str":
            self.take()
            q = val[0]
            return ("str", val[1:-1].replace(q + q, q))
        if val in (".true.", ".false."):
            self.take()
            return ("log", val == ".true.")
        if val == "(/":
            self.take()
            items = [self.expr()]
            while self.at(","):
                self.take()
                items.append(self.expr())
            self.take("/)")
            return ("arr", items)
        if val == "(":
            self.take()
            a = self.expr()
            if self.at(","):
                self.take()
                b = self.expr()
                self.take(")")
                return ("cplx", a, b)
            self.take(")")
            return ("paren", a)
        if kind == "name":
            self.take()
            node = ("name", val)
            while True:
                if self.at("("):
                    self.take()
                    args = self.args()
                    self.take(")")
                    node = ("ref", node, args)
                elif self.at("%"):
                    self.take()
                    node = ("comp", node, self.take()[1])
                else:
                    break
            return node
        raise SyntaxError(f"unexpected {val!r} in {self.text!r}")

    def args(self):
        out = []
        if self.at(")"):
            return out
        while True:
            out.append(self.arg())
            if self.at(","):
                self.take()
                continue
            return out

    def arg(self):
        if self.peek()[0] == "name" and self.peek(1)[1] == "=":
            name = self.take()[1]
            self.take("=")
            return ("kw", name, self.expr())
        lo = hi = st = None
        if not self.at(":"):
            lo = self.expr()
            if not self.at(":"):
                return lo
        self.take(":")
        if not (self.at(",") or self.at(")") or self.at(":")):
            hi = self.expr()
        if self.at(":"):
            self.take()
            st = self.expr()
        return ("slice", lo, hi, st)


def parse_expr(text):
    return Parser(text).parse_all()


# --------------------------------------------------------------------------
# Runtime values
# --------------------------------------------------------------------------


class FArray:
    """A Fortran array: numpy data in Fortran order and the lower bound of
    each dimension.  Allocation fills the object in place, so a dummy
    argument bound to it sees an ALLOCATE made by the callee."""
    __slots__ = ("d", "o", "t")

    def __init__(self, t, d=None, o=()):
        self.t, self.d, self.o = t, d, tuple(o)

    def allocate(self, bounds, fill=None):
        shape = [hi - lo + 1 for lo, hi in bounds]
        dt = {"r": np.float64, "i": np.int64, "c": np.complex128, "l": np.bool_}.get(self.t, object)
        if dt is object:
            d = np.empty(shape, dtype=object, order="F")
            for idx in np.ndindex(*shape):
                d[idx] = new_derived(self.t[2:])
        else:
            d = np.zeros(shape, dtype=dt, order="F")
            if fill is not None:
                d[...] = fill
        self.d = d
        self.o = tuple(lo for lo, _ in bounds)
        return self

    def rebased(self, lows):
        return FArray(self.t, self.d, lows)

    @staticmethod
    def view(t, d):
        return FArray(t, d, (1,) * d.ndim)


_DERIVED = {}


def _pyname(field):
    """A component name as a Python attribute (fftw_iodim has one named 'is')."""
    return field + "_" if keyword.iskeyword(field) else field


def new_derived(t):
    """A fresh value of derived type `t` (None for an opaque library type
    such as C_PTR)."""
    fields = _DERIVED.get(t)
    if fields is None:
        return None
    obj = types.SimpleNamespace()
    for name, (ft, rank) in fields.items():
        setattr(obj, _pyname(name), 0 if ft == "i" else 0.0 if ft == "r" else None)
    return obj


class FortranStop(Exception):
    pass


class Quit(Exception):
    """QuitRoutine of the reference: the run ends with `errorcode`."""

    def __init__(self, errorcode, normalexit):
        super().__init__(f"QuitRoutine({errorcode})")
        self.errorcode, self.normalexit = errorcode, normalexit


def _idiv(a, b):
    q = abs(a) // abs(b)
    return q if (a >= 0) == (b >= 0) else -q


def _imod(a, b):
    return a - b * _idiv(a, b)


def _nint(x):
    f = math.floor(x)
    r = x - f
    if r > 0.5 or (r == 0.5):
        return int(f) + 1 if x >= 0 or r > 0.5 else int(f)
    return int(f)


def _cdiv_real(c, r):
    """complex / real as gfortran lowers it: both parts divided by r."""
    if isinstance(c, np.ndarray):
        out = np.empty_like(c)
        out.real = c.real / r
        out.imag = c.imag / r
        return out
    return complex(c.real / r, c.imag / r)


def _to_int(x):
    return int(x)


# --------------------------------------------------------------------------
# Program units
# --------------------------------------------------------------------------


class Var:
    __slots__ = ("name", "t", "dims", "alloc", "param", "init", "intent", "save", "is_dummy", "charlen")

    def __init__(self, name, t):
        self.name, self.t = name, t
        self.dims = None          # None: scalar; list of (lo, hi) nodes, ':' or '*'
        self.alloc = False
        self.param = False
        self.init = None
        self.intent = None
        self.save = False
        self.is_dummy = False
        self.charlen = None

    @property
    def rank(self):
        return 0 if self.dims is None else len(self.dims)


class Unit:
    def __init__(self, kind, name, args, file, line):
        self.kind, self.name, self.args = kind, name, args
        self.file, self.line = file, line
        self.vars = {}
        self.body = []            # (line, label, text)
        self.result = None        # function result variable


_TYPES = {"real": "r", "integer": "i", "logical": "l", "complex": "c", "character": "s",
          "doubleprecision": "r", "doublecomplex": "c"}


def _parse_decl(text):
    """Type declaration statement -> (type, attrs, entities) or None."""
    m = re.match(r"^(double\s*precision|double\s*complex|real|integer|logical|complex|character|type\s*\(\s*(\w+)\s*\))",
                 text)
    if not m:
        return None
    rest = text[m.end():]
    if m.group(2):
        t = "t:" + m.group(2)
    else:
        t = _TYPES[re.sub(r"\s+", "", m.group(1))]
    rest = rest.lstrip()
    charlen = None
    if rest.startswith("("):
        j = _match_paren(rest, 0)
        sel = rest[1:j]
        if t == "s":
            charlen = sel
        rest = rest[j + 1:].lstrip()
    elif rest.startswith("*"):
        m2 = re.match(r"^\*\s*(\d+|\(\*\))", rest)
        charlen = m2.group(1)
        rest = rest[m2.end():].lstrip()
    # 'function' after a type: a typed function statement, not a declaration
    if re.match(r"^function\b", rest):
        return None
    attrs = []
    if rest.startswith(","):
        k = rest.find("::")
        if k < 0:
            raise SyntaxError("attributes without '::': " + text)
        attrs = [a.strip() for a in _split_top(rest[1:k]) if a.strip()]
        rest = rest[k + 2:]
    elif rest.startswith("::"):
        rest = rest[2:]
    elif rest and not re.match(r"^[a-z_]", rest):
        return None
    ents = [e.strip() for e in _split_top(rest) if e.strip()]
    return t, attrs, ents, charlen


def _parse_dims(spec):
    dims = []
    for d in _split_top(spec):
        d = d.strip()
        if d == ":":
            dims.append(":")
        elif d == "*":
            dims.append("*")
        else:
            parts = _split_top(d, ":")
            if len(parts) == 1:
                dims.append((("num", 1, "i"), parse_expr(parts[0])))
            else:
                lo = parse_expr(parts[0]) if parts[0].strip() else ("num", 1, "i")
                hi = parts[1].strip()
                dims.append((lo, parse_expr(hi) if hi and hi != "*" else (":" if not hi else "*")))
    return dims


def declare(unit, decl):
    t, attrs, ents, charlen = decl
    dims_attr = None
    flags = set()
    intent = None
    for a in attrs:
        if a.startswith("dimension"):
            dims_attr = _parse_dims(a[a.index("(") + 1:a.rindex(")")])
        elif a.startswith("intent"):
            intent = a[a.index("(") + 1:a.rindex(")")].strip()
        else:
            flags.add(a.split("(")[0].strip())
    for e in ents:
        init = None
        k = _top_assign(e)
        if k >= 0:
            init = parse_expr(e[k + 1:].replace(">", "", 1) if e[k + 1:].startswith(">") else e[k + 1:])
            e = e[:k].strip()
        m = re.match(r"^(\w+)\s*(\((.*)\))?\s*(\*\s*\d+)?$", e)
        if not m:
            raise SyntaxError("declaration entity: " + e)
        name = m.group(1)
        v = unit.vars.get(name) or Var(name, t)
        v.t = t
        if m.group(3) is not None:
            v.dims = _parse_dims(m.group(3))
        elif dims_attr is not None:
            v.dims = list(dims_attr)
        v.alloc = v.alloc or "allocatable" in flags or "pointer" in flags
        v.param = v.param or "parameter" in flags
        v.save = v.save or "save" in flags
        v.intent = intent or v.intent
        v.charlen = charlen
        if init is not None:
            v.init = init
        unit.vars[name] = v


def parse_file(path, defines, units, modules, types_):
    """Parse the program units of one file into `units` (subroutines,
    functions, programs) and `modules`."""
    lines = preprocess(path, defines)
    stack = []
    skip = 0                    # depth inside INTERFACE blocks
    in_type = None
    fname = os.path.basename(path)
    for line, label, text in statements(lines):
        if skip:
            if re.match(r"^end\s*interface\b", text):
                skip -= 1
            elif re.match(r"^(abstract\s+)?interface\b", text):
                skip += 1
            continue
        if in_type is not None:
            if re.match(r"^end\s*type\b", text):
                in_type = None
                continue
            d = _parse_decl(text)
            if d:
                t, attrs, ents, _ = d
                for e in ents:
                    nm = re.match(r"^(\w+)", e).group(1)
                    types_[in_type][nm] = (t, 0)
            continue
        if re.match(r"^(abstract\s+)?interface\b", text):
            skip = 1
            continue
        m = re.match(r"^type\s*(,\s*[\w()\s,]+)?\s*(::)?\s*(\w+)$", text)
        if m and not text.startswith("type("):
            in_type = m.group(3)
            types_[in_type] = {}
            continue
        m = re.match(r"^module\s+(\w+)$", text)
        if m and not stack:
            u = Unit("module", m.group(1), [], fname, line)
            modules[u.name] = u
            stack.append(u)
            continue
        m = re.match(r"^program\s+(\w+)$", text)
        if m:
            u = Unit("program", m.group(1), [], fname, line)
            units[u.name] = u
            stack.append(u)
            continue
        m = re.match(r"^((recursive|pure|elemental)\s+)*(subroutine)\s+(\w+)\s*(\((.*)\))?\s*$", text)
        m2 = re.match(r"^((?:(?:double\s+precision|real|integer|logical|complex)(?:\s*\(\s*\w+\s*\))?)\s+)?function\s+(\w+)\s*\((.*)\)\s*(result\s*\((\w+)\))?$", text)
        if m or m2:
            if m:
                u = Unit("subroutine", m.group(4), [a.strip() for a in (m.group(6) or "").split(",") if a.strip()],
                         fname, line)
            else:
                u = Unit("function", m2.group(2), [a.strip() for a in m2.group(3).split(",") if a.strip()],
                         fname, line)
                u.result = m2.group(5) or u.name
                if m2.group(1):
                    tn = re.sub(r"\(.*\)", "", m2.group(1)).strip()
                    u.vars[u.result] = Var(u.result, _TYPES[re.sub(r"\s+", "", tn)])
            for a in u.args:
                v = u.vars.get(a) or Var(a, None)
                v.is_dummy = True
                u.vars[a] = v
            units[u.name] = u
            stack.append(u)
            continue
        if re.match(r"^end(\s*(subroutine|function|program|module)(\s+\w+)?)?$", text):
            if not stack:
                raise SyntaxError(f"{fname}:{line}: unmatched end")
            # a plain 'end' may close a subroutine; 'end do'/'end if' do not match here
            stack.pop()
            continue
        if not stack:
            continue
        cur = stack[-1]
        if text == "contains":
            continue
        if re.match(r"^(use|implicit|include|private|public|external|intrinsic|save|sequence)\b", text):
            continue
        m = re.match(r"^parameter\s*\((.*)\)$", text)
        if m:
            for item in _split_top(m.group(1)):
                nm, val = item.split("=", 1)
                v = cur.vars.get(nm.strip()) or Var(nm.strip(), "i")
                v.param = True
                v.init = parse_expr(val)
                cur.vars[v.name] = v
            continue
        d = _parse_decl(text) if _top_assign(text) < 0 or "::" in text else None
        if d:
            declare(cur, d)
            continue
        if cur.kind == "module":
            raise SyntaxError(f"{fname}:{line}: executable statement in a module: {text}")
        cur.body.append((line, label, text))
    if stack:
        raise SyntaxError(f"{fname}: unterminated {stack[-1].kind} {stack[-1].name}")


# --------------------------------------------------------------------------
# Code generation
# --------------------------------------------------------------------------

_INTRINSIC_TYPES = {
    "float": "r", "dble": "r", "real": "r", "sngl": "r", "dfloat": "r", "sqrt": "r", "dsqrt": "r", "sin": "r",
    "cos": "r", "tan": "r", "tanh": "r", "sinh": "r", "cosh": "r", "exp": "r", "log": "r", "dlog": "r",
    "log10": "r", "asin": "r", "dasin": "r", "acos": "r", "dacos": "r", "atan": "r", "datan": "r",
    "atan2": "r", "dexp": "r", "dcos": "r", "dsin": "r", "huge": None, "tiny": None, "epsilon": None,
    "int": "i", "nint": "i", "floor": "i", "ceiling": "i", "size": "i", "len": "i", "lbound": "i",
    "ubound": "i", "mod": None, "abs": None, "dabs": "r", "max": None, "min": None, "dmax1": "r",
    "dmin1": "r", "sign": None, "allocated": "l", "present": "l", "trim": "s", "adjustl": "s",
    "cmplx": "c", "dcmplx": "c", "aimag": "r", "dimag": "r", "conjg": "c", "sum": None, "maxval": None,
    "minval": None, "mpi_wtime": "r",
}


class Gen:
    """Python source for one program unit."""

    def __init__(self, unit, world):
        self.u = unit
        self.w = world
        self.lines = []
        self.ind = 1
        self.tmp = 0
        self.arrays = set()       # arrays (local or module) referenced: bound as d_/o_ locals
        self.loops = []

    # ---- symbols
    def var(self, name):
        v = self.u.vars.get(name)
        if v is not None:
            return v, ("module" if self.u.kind == "module" else "local")
        v = self.w.module_vars.get(name)
        if v is not None:
            return v, "module"
        return None, None

    def vtype(self, name):
        v, _ = self.var(name)
        if v is None:
            return None
        t = v.t
        if t is None and v.is_dummy:
            t = "r" if name[0] not in "ijklmn" else "i"
            v.t = t
        return t

    def emit(self, s):
        self.lines.append("    " * self.ind + s)

    def newtmp(self):
        self.tmp += 1
        return f"_t{self.tmp}"

    # ---- expressions: (code, type, rank)
    def ex(self, n):
        k = n[0]
        if k == "num":
            return (repr(n[1]), n[2], 0)
        if k == "str":
            return (repr(n[1]), "s", 0)
        if k == "log":
            return (repr(n[1]), "l", 0)
        if k == "paren":
            c, t, r = self.ex(n[1])
            return ("(" + c + ")", t, r)
        if k == "cplx":
            a, b = self.ex(n[1]), self.ex(n[2])
            return (f"complex({a[0]}, {b[0]})", "c", 0)
        if k == "arr":
            items = [self.ex(x) for x in n[1]]
            t = items[0][1]
            dt = {"r": "np.float64", "i": "np.int64", "l": "np.bool_", "c": "np.complex128"}[t]
            return (f"np.array([{', '.join(c for c, _, _ in items)}], dtype={dt})", t, 1)
        if k == "name":
            return self.name_value(n[1])
        if k == "comp":
            base = self.ex(n[1])[0]
            return (f"{base}.{_pyname(n[2])}", self.comp_type(n), 0)
        if k == "ref":
            return self.ref_value(n)
        if k == "un":
            a = self.ex(n[2])
            if n[1] == "not":
                return (f"(not {a[0]})" if a[2] == 0 else f"np.logical_not({a[0]})", "l", a[2])
            return (f"(-{a[0]})", a[1], a[2])
        if k == "bin":
            return self.binop(n)
        raise SyntaxError(f"expression node {k}")

    def comp_type(self, n):
        # the type of a derived-type component: look it up through the base
        base = n[1]
        bt = None
        if base[0] == "name":
            bt = self.vtype(base[1])
        elif base[0] == "ref" and base[1][0] == "name":
            bt = self.vtype(base[1][1])
        if bt and bt.startswith("t:"):
            f = _DERIVED.get(bt[2:], {}).get(n[2])
            if f:
                return f[0]
        return "i"

    def binop(self, n):
        op, a, b = n[1], self.ex(n[2]), self.ex(n[3])
        rank = max(a[2], b[2])
        if op in ("and", "or"):
            if rank:
                fn = "np.logical_and" if op == "and" else "np.logical_or"
                return (f"{fn}({a[0]}, {b[0]})", "l", rank)
            return (f"({a[0]} {op} {b[0]})", "l", 0)
        if op in ("==", "!=", "<", "<=", ">", ">="):
            return (f"({a[0]} {op} {b[0]})", "l", rank)
        if op == "//":
            return (f"({a[0]} + {b[0]})", "s", 0)
        t = self.promote(a[1], b[1])
        if op == "**":
            if b[1] == "i" and n[3][0] == "num" and n[3][1] in (2, 3, 4):
                x = a[0]
                if rank == 0 and not re.match(r"^[\w.\[\], ()+\-*/]*$", x):
                    pass
                e = n[3][1]
                if e == 2:
                    return (f"({x} * {x})", a[1], rank)
                if e == 3:
                    return (f"(({x} * {x}) * {x})", a[1], rank)
                return (f"(({x} * {x}) * ({x} * {x}))", a[1], rank)
            if a[1] == "i" and b[1] == "i":
                return (f"({a[0]} ** {b[0]})", "i", rank)
            return (f"math.pow({a[0]}, {b[0]})" if rank == 0 else f"np.power({a[0]}, {b[0]})", t, rank)
        if op == "/":
            if a[1] == "i" and b[1] == "i":
                if rank:
                    raise NotImplementedError("integer array division")
                return (f"_idiv({a[0]}, {b[0]})", "i", 0)
            if a[1] == "c" and b[1] in ("r", "i"):
                return (f"_cdiv_real({a[0]}, {b[0]})", "c", rank)
            return (f"({a[0]} / {b[0]})", t, rank)
        return (f"({a[0]} {op} {b[0]})", t, rank)

    @staticmethod
    def promote(a, b):
        order = {"i": 0, "r": 1, "c": 2}
        if a in order and b in order:
            return a if order[a] >= order[b] else b
        return a or b

    def name_value(self, name):
        v, where = self.var(name)
        if v is None:
            if name in _INTRINSIC_TYPES:
                return (self.intrinsic(name, []), _INTRINSIC_TYPES[name] or "r", 0)
            if name in self.w.functions:
                return (f"F.{name}()", "r", 0)
            # a name only the runtime defines (an MPI or library constant)
            return (f"G.{name}", self.w.runtime_types.get(name, "i"), 0)
        t = self.vtype(name)
        if v.param:
            return (f"G.{name}" if where == "module" else f"v_{name}", t, 0)
        if v.rank:
            self.arrays.add(name)
            return (f"d_{name}", t, v.rank)
        if where == "module":
            return (f"G.{name}", t, 0)
        return (f"v_{name}", t, 0)

    def array_obj(self, name):
        v, where = self.var(name)
        return f"a_{name}"

    def index(self, name, args):
        """numpy index expression for name(args) and the result rank."""
        self.arrays.add(name)
        parts, rank = [], 0
        for i, a in enumerate(args):
            o = f"o_{name}[{i}]"
            if a[0] == "slice":
                lo = self.ex(a[1])[0] + f" - {o}" if a[1] is not None else ""
                hi = "(" + self.ex(a[2])[0] + f") - {o} + 1" if a[2] is not None else ""
                st = ":" + self.ex(a[3])[0] if a[3] is not None else ""
                parts.append(f"{lo}:{hi}{st}")
                rank += 1
            else:
                c, t, r = self.ex(a)
                if r:
                    raise NotImplementedError("vector subscripts")
                parts.append(f"{c} - {o}")
        return ", ".join(parts), rank

    def ref_value(self, n):
        base, args = n[1], n[2]
        if base[0] == "comp":
            # component array of a derived-type value: x%arr(i)
            b = self.ex(base)[0]
            idx = []
            for a in args:
                if a[0] == "slice":
                    raise NotImplementedError("section of a component")
                idx.append(f"{self.ex(a)[0]} - {b}.o[{len(idx)}]")
            return (f"{b}.d[{', '.join(idx)}]", self.comp_array_type(base), 0)
        if base[0] != "name":
            raise NotImplementedError("reference to an expression")
        name = base[1]
        v, where = self.var(name)
        if v is not None and v.rank:
            idx, rank = self.index(name, args)
            return (f"d_{name}[{idx}]", self.vtype(name), rank)
        if v is not None and v.t == "s" and args and args[0][0] == "slice":
            raise NotImplementedError("substring")
        if name in self.w.functions and name not in self.w.units_sub:
            cargs = [self.actual(a) for a in args]
            rt = self.w.function_types.get(name, "r")
            return (f"F.{name}({', '.join(cargs)})", rt, 0)
        if name in _INTRINSIC_TYPES:
            return self.intrinsic_call(name, args)
        raise NameError(f"{self.u.file}: '{name}' is neither an array, an intrinsic nor a function")

    def actual(self, node):
        """An actual argument of a function reference: arrays and sections
        are passed as arrays, everything else by value."""
        if node[0] == "name":
            v, _ = self.var(node[1])
            if v is not None and v.rank:
                self.arrays.add(node[1])
                return f"a_{node[1]}"
        if node[0] == "ref" and node[1][0] == "name":
            v, _ = self.var(node[1][1])
            if v is not None and v.rank:
                code, t, rank = self.ex(node)
                if rank:
                    return f"FArray.view({t!r}, {code})"
        return self.ex(node)[0]

    def comp_array_type(self, base):
        return "i"

    def intrinsic(self, name, args):
        if name == "mpi_wtime":
            return "0.0"
        raise NotImplementedError(name)

    def intrinsic_call(self, name, args):
        ea = [self.ex(a) if a[0] != "kw" else self.ex(a[2]) for a in args]
        c = [x[0] for x in ea]
        t0 = ea[0][1] if ea else None
        rank = max([x[2] for x in ea] or [0])
        if name in ("float", "dble", "real", "dfloat", "sngl"):
            if t0 == "c":
                return (f"({c[0]}).real", "r", rank)
            return ((f"float({c[0]})" if rank == 0 else f"np.asarray({c[0]}, dtype=np.float64)"), "r", rank)
        if name == "int":
            return ((f"int({c[0]})" if rank == 0 else f"np.trunc({c[0]}).astype(np.int64)"), "i", rank)
        if name == "nint":
            return (f"_nint({c[0]})", "i", 0)
        if name == "floor":
            return (f"math.floor({c[0]})", "i", 0)
        if name == "ceiling":
            return (f"math.ceil({c[0]})", "i", 0)
        if name in ("sqrt", "dsqrt", "sin", "cos", "tan", "tanh", "sinh", "cosh", "exp", "log", "log10",
                    "asin", "acos", "atan", "dasin", "dacos", "datan", "dexp", "dcos", "dsin", "dlog"):
            fn = {"dsqrt": "sqrt", "dasin": "asin", "dacos": "acos", "datan": "atan", "dexp": "exp",
                  "dcos": "cos", "dsin": "sin", "dlog": "log"}.get(name, name)
            if rank:
                return (f"np.vectorize(math.{fn}, otypes=[np.float64])({c[0]})", "r", rank)
            return (f"math.{fn}({c[0]})", "r", 0)
        if name == "atan2":
            return (f"math.atan2({c[0]}, {c[1]})", "r", 0)
        if name == "mod":
            if t0 == "i" and ea[1][1] == "i":
                return (f"_imod({c[0]}, {c[1]})", "i", 0)
            return (f"math.fmod({c[0]}, {c[1]})", "r", 0)
        if name in ("abs", "dabs"):
            return ((f"abs({c[0]})" if rank == 0 else f"np.abs({c[0]})"), "r" if t0 == "c" else t0, rank)
        if name in ("max", "min", "dmax1", "dmin1"):
            fn = "max" if name in ("max", "dmax1") else "min"
            t = t0
            for x in ea[1:]:
                t = self.promote(t, x[1])
            return (f"_f{fn}({', '.join(c)})", t, 0)
        if name == "sign":
            if t0 == "i":
                return (f"(abs({c[0]}) if {c[1]} >= 0 else -abs({c[0]}))", "i", 0)
            return (f"math.copysign(abs({c[0]}), {c[1]})", "r", 0)
        if name == "huge":
            return ("sys.float_info.max" if t0 == "r" else "(2**31 - 1)", t0, 0)
        if name == "tiny":
            return ("sys.float_info.min", "r", 0)
        if name == "epsilon":
            return ("sys.float_info.epsilon", "r", 0)
        if name == "size":
            arr = args[0]
            obj = self.ex(arr)[0]
            if len(args) > 1:
                return (f"np.shape({obj})[{c[1]} - 1]", "i", 0)
            return (f"np.size({obj})", "i", 0)
        if name in ("lbound", "ubound"):
            nm = args[0][1]
            self.arrays.add(nm)
            if name == "lbound":
                return (f"o_{nm}[{c[1]} - 1]", "i", 0)
            return (f"(o_{nm}[{c[1]} - 1] + d_{nm}.shape[{c[1]} - 1] - 1)", "i", 0)
        if name == "allocated":
            nm = args[0][1]
            return (f"(a_{nm}.d is not None)", "l", 0)
        if name == "present":
            return (f"({c[0]} is not None)", "l", 0)
        if name in ("trim", "adjustl"):
            return (f"str({c[0]}).strip()", "s", 0)
        if name == "len":
            return (f"len({c[0]})", "i", 0)
        if name in ("cmplx", "dcmplx"):
            im = c[1] if len(c) > 1 else "0.0"
            return (f"complex({c[0]}, {im})", "c", 0)
        if name in ("aimag", "dimag"):
            return (f"({c[0]}).imag", "r", rank)
        if name == "conjg":
            return (f"({c[0]}).conjugate()", "c", rank)
        if name == "sum":
            return (f"_fsum({c[0]})", t0, 0)
        if name in ("maxval", "minval"):
            return (f"np.{name[:3]}({c[0]})", t0, 0)
        if name == "mpi_wtime":
            return ("0.0", "r", 0)
        raise NotImplementedError(name)

    # ---- statements
    def rebind(self, names=None):
        for nm in sorted(names if names is not None else self.arrays):
            self.emit(f"d_{nm} = a_{nm}.d; o_{nm} = a_{nm}.o")

    def assign_target(self, lhs_node, rhs):
        """Python statement assigning code `rhs` (type, rank) to the Fortran
        designator lhs_node."""
        code, rt, rr = rhs
        if lhs_node[0] == "name":
            name = lhs_node[1]
            v, where = self.var(name)
            if v is None:
                self.emit(f"G.{name} = {code}")
                return
            t = self.vtype(name)
            if v.rank:
                self.arrays.add(name)
                self.emit(f"d_{name}[...] = {code}")
                return
            code = self.convert(code, rt, t)
            self.emit(f"{'G.' if where == 'module' else 'v_'}{name} = {code}")
            return
        if lhs_node[0] == "ref" and lhs_node[1][0] == "name":
            name = lhs_node[1][1]
            v, where = self.var(name)
            if v is None or not v.rank:
                raise SyntaxError(f"{self.u.name}: assignment to '{name}(...)' which is not an array")
            idx, rank = self.index(name, lhs_node[2])
            t = self.vtype(name)
            if rank == 0:
                code = self.convert(code, rt, t)
            self.emit(f"d_{name}[{idx}] = {code}")
            return
        if lhs_node[0] == "comp":
            base = self.ex(lhs_node[1])[0]
            self.emit(f"{base}.{_pyname(lhs_node[2])} = {code}")
            return
        if lhs_node[0] == "ref" and lhs_node[1][0] == "comp":
            b = self.ex(lhs_node[1])[0]
            idx = [f"{self.ex(a)[0]} - {b}.o[{i}]" for i, a in enumerate(lhs_node[2])]
            self.emit(f"{b}.d[{', '.join(idx)}] = {code}")
            return
        raise SyntaxError(f"assignment target {lhs_node}")

    @staticmethod
    def convert(code, from_t, to_t):
        if to_t == from_t or to_t is None or from_t is None:
            return code
        if to_t == "i" and from_t == "r":
            return f"int({code})"
        if to_t == "r" and from_t == "i":
            return f"float({code})"
        if to_t == "c" and from_t in ("r", "i"):
            return f"complex({code}, 0.0)"
        if to_t == "r" and from_t == "c":
            return f"({code}).real"
        return code

    def gen_call(self, name, args):
        callee = self.w.units.get(name)
        parts = []
        backs = []
        for i, a in enumerate(args):
            if a[0] == "kw":
                c = self.ex(a[2])
                parts.append(f"{a[1]}={c[0]}")
                continue
            node = a
            dummy = None
            if callee is not None and i < len(callee.args):
                dummy = callee.vars.get(callee.args[i])
            if node[0] == "name":
                v, where = self.var(node[1])
                if v is not None and v.rank:
                    self.arrays.add(node[1])
                    parts.append(f"a_{node[1]}")
                    continue
                c = self.ex(node)
                parts.append(c[0])
                if v is not None and not v.param:
                    backs.append((i, node))
                elif v is None:
                    backs.append((i, node))
                continue
            if node[0] == "ref" and node[1][0] == "name":
                v, where = self.var(node[1][1])
                if v is not None and v.rank:
                    code, t, rank = self.ex(node)
                    if rank:
                        parts.append(f"FArray.view({t!r}, {code})")
                        continue
                    if dummy is not None and dummy.rank:
                        raise NotImplementedError(f"array element passed to the array dummy of {name}")
                    parts.append(code)
                    backs.append((i, node))
                    continue
            parts.append(self.ex(node)[0])
        r = self.newtmp()
        self.emit(f"{r} = F.{name}({', '.join(parts)})")
        if backs:
            self.emit(f"if {r} is not None:")
            self.ind += 1
            for i, node in backs:
                self.assign_target(node, (f"{r}[{i}]", None, 0))
            self.ind -= 1

    def gen_io(self, kind, text):
        m = re.match(r"^(write|read|print)\s*(\(.*?\))?\s*(.*)$", text)
        ctl = ""
        if text.startswith(("write", "read")):
            j = text.index("(")
            k = _match_paren(text, j)
            ctl, items = text[j + 1:k], text[k + 1:].strip()
        else:
            items = re.sub(r"^print\s*[^,]*,?", "", text)
        cparts = _split_top(ctl) if ctl else ["6"]
        unit = cparts[0].strip()
        fmt = cparts[1].strip() if len(cparts) > 1 else "*"
        its = [x.strip() for x in _split_top(items) if x.strip()] if items else []
        if kind == "write":
            if re.fullmatch(r"[a-z_]\w*", unit) and self.vtype(unit) == "s":
                # internal WRITE into a character variable
                vals = [self.ex(parse_expr(x))[0] for x in its]
                tmp = self.newtmp()
                self.emit(f"{tmp} = R.internal_write({self.format_text(fmt)!r}, [{', '.join(vals)}])")
                self.assign_target(parse_expr(unit), (tmp, "s", 0))
                return
            if unit.isdigit() and int(unit) in self.w.capture_units:
                vals = []
                for x in its:
                    if x.startswith("(") and _top_assign(x[1:-1]) >= 0:
                        continue
                    vals.append(self.ex(parse_expr(x))[0])
                self.emit(f"R.write({unit}, [{', '.join(vals)}])")
            else:
                self.emit("pass")
            return
        if kind == "read":
            if len(its) == 1 and its[0].startswith("(") and _top_assign(its[0][1:-1]) >= 0:
                # one implied-DO list: (target, var = lo, hi)
                parts = [x.strip() for x in _split_top(its[0][1:-1])]
                if len(parts) != 3:
                    raise SyntaxError(f"{self.u.name}: implied-DO list {its[0]}")
                tnode = parse_expr(parts[0])
                var, lo = [x.strip() for x in parts[1].split("=", 1)]
                hi = self.ex(parse_expr(parts[2]))[0]
                lo = self.ex(parse_expr(lo))[0]
                nm = tnode[1] if tnode[0] == "name" else tnode[1][1]
                rng, vals, k = self.newtmp(), self.newtmp(), self.newtmp()
                _, where = self.var(var)
                loopv = f"G.{var}" if where == "module" else f"v_{var}"
                self.emit(f"{rng} = _frange({lo}, {hi}, 1)")
                self.emit(f"{vals} = R.read({unit}, {fmt!r}, [{self.vtype(nm)!r}] * len({rng}))")
                self.emit(f"for {k}, {loopv} in enumerate({rng}):")
                self.ind += 1
                self.assign_target(tnode, (f"{vals}[{k}]", None, 0))
                self.ind -= 1
                return
            targets = [parse_expr(x) for x in its]
            tmp = self.newtmp()
            types_ = []
            for tnode in targets:
                nm = tnode[1] if tnode[0] == "name" else tnode[1][1]
                types_.append(self.vtype(nm))
            self.emit(f"{tmp} = R.read({unit}, {fmt!r}, {types_!r})")
            for i, tnode in enumerate(targets):
                self.assign_target(tnode, (f"{tmp}[{i}]", None, 0))
            return
        self.emit("pass")

    def format_text(self, fmt):
        """The edit descriptors of a WRITE: a FORMAT statement of this unit
        by its label, or a character constant."""
        if fmt.isdigit():
            for _, label, text in self.u.body:
                if label == int(fmt) and re.match(r"^format\s*\(", text):
                    return text[text.index("("):].strip()
            raise SyntaxError(f"{self.u.name}: no FORMAT labelled {fmt}")
        if fmt[:1] in "'\"" and fmt[-1:] == fmt[:1]:
            return fmt[1:-1]
        raise SyntaxError(f"{self.u.name}: format {fmt}")

    def gen_allocate(self, text, dealloc=False):
        inner = text[text.index("(") + 1:text.rindex(")")]
        for item in _split_top(inner):
            item = item.strip()
            if item.startswith(("stat", "errmsg", "source")):
                continue
            if dealloc:
                nm = re.match(r"^(\w+)", item).group(1)
                self.emit(f"a_{nm}.d = None")
                continue
            m = re.match(r"^(\w+)\s*\((.*)\)$", item)
            nm = m.group(1)
            bounds = []
            for d in _split_top(m.group(2)):
                p = _split_top(d, ":")
                if len(p) == 1:
                    bounds.append(f"(1, {self.ex(parse_expr(p[0]))[0]})")
                else:
                    bounds.append(f"({self.ex(parse_expr(p[0]))[0]}, {self.ex(parse_expr(p[1]))[0]})")
            v, _ = self.var(nm)
            fill = "np.nan" if (v.t in ("r", "c") and self.w.nan_fill) else "None"
            self.emit(f"a_{nm}.allocate([{', '.join(bounds)}], fill={fill})")
            self.arrays.add(nm)
        self.rebind()

    def block(self, stmts, i, stop):
        """Generate statements from index i until one matching `stop`
        (a regex) at this nesting level; returns (index of the stopper, its
        text)."""
        n = len(stmts)
        while i < n:
            line, label, text = stmts[i]
            if stop and re.match(stop, text):
                return i, text
            i = self.stmt(stmts, i)
        if stop:
            raise SyntaxError(f"{self.u.file}: block not closed ({stop}) in {self.u.name}")
        return i, None

    def body_or_pass(self, start_len):
        if len(self.lines) == start_len:
            self.emit("pass")

    def stmt(self, stmts, i):
        line, label, text = stmts[i]
        self.emit(f"# {self.u.file}:{line}")
        # block IF
        m = re.match(r"^if\s*\(", text)
        if m:
            j = _match_paren(text, text.index("("))
            cond = self.ex(parse_expr(text[text.index("(") + 1:j]))[0]
            rest = text[j + 1:].strip()
            if rest == "then":
                self.emit(f"if {cond}:")
                self.ind += 1
                n0 = len(self.lines)
                k, stop = self.block(stmts, i + 1, r"^(else\b|elseif\b|end\s*if$|endif$)")
                self.body_or_pass(n0)
                self.ind -= 1
                while True:
                    if re.match(r"^(end\s*if|endif)$", stop):
                        return k + 1
                    mm = re.match(r"^else\s*if\s*\(", stop)
                    if mm:
                        jj = _match_paren(stop, stop.index("("))
                        c2 = self.ex(parse_expr(stop[stop.index("(") + 1:jj]))[0]
                        self.emit(f"elif {c2}:")
                    else:
                        self.emit("else:")
                    self.ind += 1
                    n0 = len(self.lines)
                    k, stop = self.block(stmts, k + 1, r"^(else\b|elseif\b|end\s*if$|endif$)")
                    self.body_or_pass(n0)
                    self.ind -= 1
            self.emit(f"if {cond}:")
            self.ind += 1
            self.stmt([(line, None, rest)], 0)
            self.ind -= 1
            return i + 1
        m = re.match(r"^do\s+while\s*\((.*)\)$", text)
        if m:
            self.emit(f"while {self.ex(parse_expr(m.group(1)))[0]}:")
            self.ind += 1
            n0 = len(self.lines)
            k, _ = self.block(stmts, i + 1, r"^(end\s*do|enddo)$")
            self.body_or_pass(n0)
            self.ind -= 1
            return k + 1
        m = re.match(r"^do\s+(\w+)\s*=\s*(.*)$", text)
        if m:
            # a GOTO inside the loop to the CONTINUE labelled right after its
            # END DO leaves the loop (an EXIT): remember that label
            depth, e = 0, i + 1
            while e < len(stmts):
                t_e = stmts[e][2]
                if re.match(r"^do\b", t_e):
                    depth += 1
                elif re.match(r"^(end\s*do|enddo)$", t_e):
                    if depth == 0:
                        break
                    depth -= 1
                e += 1
            after = stmts[e + 1] if e + 1 < len(stmts) else None
            self.loops.append(after[1] if after is not None and after[2] == "continue" else None)
            var = m.group(1)
            b = [self.ex(parse_expr(x))[0] for x in _split_top(m.group(2))]
            step = b[2] if len(b) > 2 else "1"
            v, where = self.var(var)
            target = f"G.{var}" if where == "module" else f"v_{var}"
            rng = self.newtmp()
            self.emit(f"{rng} = _frange({b[0]}, {b[1]}, {step})")
            self.emit(f"for {target} in {rng}:")
            self.ind += 1
            n0 = len(self.lines)
            k, _ = self.block(stmts, i + 1, r"^(end\s*do|enddo)$")
            self.body_or_pass(n0)
            self.ind -= 1
            self.emit("else:")
            self.emit(f"    {target} = {rng}.start + len({rng}) * {rng}.step")
            self.loops.pop()
            return k + 1
        m = re.match(r"^select\s+case\s*\((.*)\)$", text)
        if m:
            sel = self.ex(parse_expr(m.group(1)))[0]
            k = i + 1
            first = True
            _, _, t2 = stmts[k]
            while True:
                _, _, t2 = stmts[k]
                if re.match(r"^end\s*select$", t2):
                    return k + 1
                mm = re.match(r"^case\s*\((.*)\)$", t2)
                if mm:
                    vals = [self.ex(parse_expr(x))[0] for x in _split_top(mm.group(1))]
                    self.emit(f"{'if' if first else 'elif'} {sel} in ({', '.join(vals)},):")
                elif re.match(r"^case\s+default$", t2):
                    self.emit("else:" if not first else "if True:")
                else:
                    raise SyntaxError("select case: " + t2)
                first = False
                self.ind += 1
                n0 = len(self.lines)
                k, _ = self.block(stmts, k + 1, r"^(case\b|end\s*select$)")
                self.body_or_pass(n0)
                self.ind -= 1
        if text in ("exit",):
            self.emit("break")
            return i + 1
        m = re.match(r"^go\s*to\s+(\d+)$", text)
        if m:
            if not self.loops or self.loops[-1] != int(m.group(1)):
                raise SyntaxError(f"{self.u.file}:{line}: only a GOTO to the CONTINUE after the enclosing loop is "
                                  f"supported: {text}")
            self.emit("break")
            return i + 1
        if text == "cycle":
            self.emit("continue")
            return i + 1
        if text == "return":
            self.emit(f"return {self.ret_tuple()}")
            return i + 1
        if text == "continue":
            self.emit("pass")
            return i + 1
        if re.match(r"^stop\b", text):
            self.emit("raise FortranStop()")
            return i + 1
        m = re.match(r"^call\s+(\w+)\s*(\((.*)\))?$", text)
        if m:
            args = Parser("(" + (m.group(3) or "") + ")")
            args.take("(")
            al = args.args()
            self.gen_call(m.group(1), al)
            self.rebind()
            return i + 1
        if re.match(r"^(write|print)\b", text):
            self.gen_io("write", text)
            return i + 1
        if re.match(r"^read\s*\(", text):
            self.gen_io("read", text)
            return i + 1
        if re.match(r"^format\s*\(", text):
            self.emit("pass")
            return i + 1
        m = re.match(r"^open\s*\((.*)\)$", text)
        if m:
            kw = {}
            for p in _split_top(m.group(1)):
                if "=" in p:
                    a, b = p.split("=", 1)
                    kw[a.strip()] = self.ex(parse_expr(b))[0]
            self.emit(f"R.open({kw.get('unit', '0')}, {kw.get('file', repr(''))})")
            return i + 1
        if re.match(r"^(close|rewind)\s*\(", text):
            self.emit("pass")
            return i + 1
        m = re.match(r"^inquire\s*\((.*)\)$", text)
        if m:
            kw = {}
            for p in _split_top(m.group(1)):
                a, b = p.split("=", 1)
                kw[a.strip()] = b.strip()
            self.assign_target(parse_expr(kw["exist"]), (f"R.exists({self.ex(parse_expr(kw['file']))[0]})", "l", 0))
            return i + 1
        if re.match(r"^allocate\s*\(", text):
            self.gen_allocate(text)
            return i + 1
        if re.match(r"^deallocate\s*\(", text):
            self.gen_allocate(text, dealloc=True)
            return i + 1
        k = _top_assign(text)
        if k >= 0:
            lhs = parse_expr(text[:k])
            rhs = self.ex(parse_expr(text[k + 1:]))
            self.assign_target(lhs, rhs)
            return i + 1
        raise SyntaxError(f"{self.u.file}:{line}: unsupported statement: {text}")

    def ret_tuple(self):
        if self.u.kind == "function":
            return f"v_{self.u.result}"
        items = []
        for a in self.u.args:
            v = self.u.vars[a]
            items.append(f"a_{a}" if v.rank else f"v_{a}")
        return "(" + "".join(x + ", " for x in items) + ")"

    def generate(self):
        u = self.u
        params = ", ".join(("a_" if (u.vars[a].rank) else "v_") + a + "=None" for a in u.args)
        head = f"def {u.name}({params}):"
        # dummy arrays: rebase to their declared lower bounds
        pre = []
        for a in u.args:
            v = u.vars[a]
            if v.rank and not v.alloc:
                lows = []
                ok = True
                for d in v.dims:
                    if d in (":", "*"):
                        lows.append("1")
                    else:
                        lows.append(self.ex(d[0])[0])
                pre.append(f"a_{a} = a_{a}.rebased(({', '.join(lows)},))")
                if any(isinstance(d, tuple) for d in v.dims):
                    shape = []
                    for d in v.dims:
                        if isinstance(d, tuple) and d[1] not in (":", "*"):
                            shape.append(f"({self.ex(d[1])[0]}) - ({self.ex(d[0])[0]}) + 1")
                        else:
                            shape = None
                            break
                    if shape:
                        pre.append(f"a_{a} = _explicit(a_{a}, ({', '.join(shape)},))")
        # locals
        for name, v in u.vars.items():
            if v.is_dummy or name == "":
                continue
            if v.rank:
                self.arrays.add(name)
                if v.alloc or any(d in (":", "*") for d in v.dims):
                    pre.append(f"a_{name} = FArray({v.t!r})")
                else:
                    bounds = ", ".join(f"({self.ex(lo)[0]}, {self.ex(hi)[0]})" for lo, hi in v.dims)
                    fill = "np.nan" if v.t in ("r", "c") and self.w.nan_fill else "None"
                    if v.init is not None:
                        pre.append(f"a_{name} = FArray({v.t!r}).allocate([{bounds}], fill={self.ex(v.init)[0]})")
                    else:
                        pre.append(f"a_{name} = FArray({v.t!r}).allocate([{bounds}], fill={fill})")
            else:
                if v.param or v.init is not None:
                    pre.append(f"v_{name} = {self.convert(self.ex(v.init)[0], self.ex(v.init)[1], v.t)}")
                else:
                    zero = {"r": "0.0", "i": "0", "l": "False", "c": "0j", "s": "''"}.get(v.t, "None")
                    if v.t and v.t.startswith("t:"):
                        zero = f"new_derived({v.t[2:]!r})"
                    pre.append(f"v_{name} = {zero}")
        self.lines = []
        self.ind = 1
        stmts = u.body
        self.block(stmts, 0, None)
        body = self.lines
        self.lines = []
        self.ind = 1
        # module arrays first: the bounds of dummy and local arrays may use them
        mod_arrays = [nm for nm in sorted(self.arrays) if self.var(nm)[1] == "module"]
        for nm in mod_arrays:
            self.emit(f"a_{nm} = G.{nm}")
        self.rebind(mod_arrays)
        for p in pre:
            self.emit(p)
        self.rebind()
        out = [head] + self.lines + body
        out.append("    return " + self.ret_tuple())
        return "\n".join(out)


def _frange(a, b, s):
    return range(a, b + 1, s) if s > 0 else range(a, b - 1, s)


def _fmax(*xs):
    m = xs[0]
    for x in xs[1:]:
        if x > m:
            m = x
    return m


def _fmin(*xs):
    m = xs[0]
    for x in xs[1:]:
        if x < m:
            m = x
    return m


def _fsum(a):
    s = 0.0
    for x in np.asarray(a).reshape(-1, order="F"):
        s = s + x
    return s


def _explicit(a, shape):
    """Explicit-shape dummy bound to actual `a`: the same elements in array
    element order, viewed with the dummy's shape (sequence association)."""
    if tuple(a.d.shape) == tuple(shape):
        return a
    flat = a.d.reshape(-1, order="F")
    if not np.shares_memory(flat, a.d):
        raise NotImplementedError("sequence association with a non-contiguous actual")
    n = int(np.prod(shape))
    return FArray(a.t, flat[:n].reshape(shape, order="F"), a.o)


# --------------------------------------------------------------------------
# The world: modules, units, runtime
# --------------------------------------------------------------------------


class World:
    def __init__(self, ref_dir, files, module_files, runtime, defines=("DOUBLE_PREC",), capture_units=(97,),
                 nan_fill=True):
        self.units, self.modules = {}, {}
        self.capture_units = set(capture_units)
        self.nan_fill = nan_fill
        for f in list(module_files) + list(files):
            parse_file(os.path.join(ref_dir, f), set(defines), self.units, self.modules, _DERIVED)
        self.module_vars = {}
        for m in self.modules.values():
            for name, v in m.vars.items():
                self.module_vars[name] = v
        for name, (t, rank) in runtime.module_vars().items():
            if name not in self.module_vars:
                v = Var(name, t)
                if rank:
                    v.dims = [":"] * rank
                    v.alloc = True
                self.module_vars[name] = v
        self.runtime_types = {}
        self.functions = {n for n, u in self.units.items() if u.kind == "function"} | set(runtime.functions())
        self.function_types = dict(runtime.function_types())
        self.units_sub = {n for n, u in self.units.items() if u.kind in ("subroutine", "program")}
        self.G = types.SimpleNamespace()
        self.F = types.SimpleNamespace()
        self.R = runtime
        runtime.world = self
        self.sources = {}
        runtime.preinstall(self.G)
        ns = dict(G=self.G, F=self.F, R=runtime, np=np, math=math, sys=sys, FArray=FArray, FortranStop=FortranStop,
                  new_derived=new_derived, _idiv=_idiv, _imod=_imod, _nint=_nint, _cdiv_real=_cdiv_real,
                  _frange=_frange, _fmax=_fmax, _fmin=_fmin, _fsum=_fsum, _explicit=_explicit)
        self.ns = ns
        # module variables
        for m in self.modules.values():
            g = Gen(m, self)
            for name, v in m.vars.items():
                if v.rank:
                    a = FArray(v.t)
                    if not v.alloc and all(isinstance(d, tuple) for d in v.dims):
                        bounds = [(eval(g.ex(lo)[0], ns), eval(g.ex(hi)[0], ns)) for lo, hi in v.dims]
                        a.allocate(bounds, fill=(eval(g.ex(v.init)[0], ns) if v.init is not None else None))
                    setattr(self.G, name, a)
                else:
                    if v.init is not None:
                        val = eval(Gen.convert(g.ex(v.init)[0], g.ex(v.init)[1], v.t), ns)
                    else:
                        val = {"r": 0.0, "i": 0, "l": False, "c": 0j, "s": ""}.get(v.t)
                        if v.t and v.t.startswith("t:"):
                            val = new_derived(v.t[2:])
                    setattr(self.G, name, val)
        runtime.install(self.G, self.F)
        for name, u in self.units.items():
            if u.kind == "module":
                continue
            src = Gen(u, self).generate()
            self.sources[name] = src
            code = compile(src, f"<fortran:{u.file}:{name}>", "exec")
            exec(code, ns)
            setattr(self.F, name, ns[name])


# --------------------------------------------------------------------------
# One-rank runtime of the libraries the reference calls
# --------------------------------------------------------------------------


class DecompInfo(types.SimpleNamespace):
    pass


def _decomp_info(nx, ny, nz):
    d = DecompInfo()
    for p in ("x", "y", "z"):
        setattr(d, p + "st", FArray("i", np.array([1, 1, 1], dtype=np.int64), (1,)))
        setattr(d, p + "en", FArray("i", np.array([nx, ny, nz], dtype=np.int64), (1,)))
        setattr(d, p + "sz", FArray("i", np.array([nx, ny, nz], dtype=np.int64), (1,)))
    return d


class Plan:
    def __init__(self, kind, n, is_, os_, howmany, sign):
        self.kind, self.n, self.is_, self.os_, self.howmany, self.sign = kind, n, is_, os_, howmany, sign


class OneRank:
    """MPI, 2DECOMP&FFT, FFTW, HDF5 and LAPACK as seen by one rank."""

    def __init__(self, files, continua):
        self.files = files              # name -> text, for OPEN/READ and INQUIRE
        self.continua = continua        # 'qt'/'qr'/'qz' -> (nr, nzm, nthm) arrays; 'time' etc.
        self.units = {}
        self.written = {}
        self.h5 = {}                    # file name -> {dataset: C-order array}, what the run wrote
        self.world = None

    # ---- declarations the translated code sees as module variables
    def module_vars(self):
        return {"xstart": ("i", 1), "xend": ("i", 1), "ystart": ("i", 1), "yend": ("i", 1), "zstart": ("i", 1),
                "zend": ("i", 1), "nrank": ("i", 0), "nproc": ("i", 0), "ph": ("t:decomp_info", 0),
                "sp": ("t:decomp_info", 0), "decomp_2d_comm_cart_x": ("i", 0), "mpi_comm_world": ("i", 0),
                "mpi_double_precision": ("i", 0), "mpi_integer": ("i", 0), "mpi_max": ("i", 0),
                "mpi_sum": ("i", 0), "mpi_min": ("i", 0), "mpi_in_place": ("i", 0)}

    def functions(self):
        return ["fftw_plan_guru_dft", "fftw_plan_guru_dft_r2c", "fftw_plan_guru_dft_c2r", "mpi_wtime"]

    def function_types(self):
        return {"fftw_plan_guru_dft": "t:plan", "fftw_plan_guru_dft_r2c": "t:plan",
                "fftw_plan_guru_dft_c2r": "t:plan", "mpi_wtime": "r"}

    def preinstall(self, G):
        """Module variables and constants of the libraries, before the
        reference's own modules take their initial values."""
        for name, (t, rank) in self.module_vars().items():
            if rank:
                setattr(G, name, FArray(t))
            elif t.startswith("t:"):
                setattr(G, name, None)
            else:
                setattr(G, name, 0)
        G.nrank, G.nproc = 0, 1
        self.G = G

    def install(self, G, F):
        stubs = dict(
            decomp_2d_init=self.decomp_2d_init, decomp_2d_fft_init=self.decomp_2d_fft_init,
            update_halo=self.update_halo, transpose_x_to_y=self.transpose, transpose_y_to_z=self.transpose,
            transpose_z_to_y=self.transpose, transpose_y_to_x=self.transpose,
            fftw_plan_guru_dft=self.plan_dft, fftw_plan_guru_dft_r2c=self.plan_r2c,
            fftw_plan_guru_dft_c2r=self.plan_c2r, dfftw_execute_dft=self.execute,
            dfftw_execute_dft_r2c=self.execute, dfftw_execute_dft_c2r=self.execute,
            zgttrf=self.gttrf, dgttrf=self.gttrf, zgttrs=self.gttrs, dgttrs=self.gttrs,
            mpibarrier=self.none, mpibcastint=self.ident, mpibcastreal=self.ident, mpisumrealscalar=self.ident,
            mpimaxrealscalar=self.ident, mpiallmaxrealscalar=self.ident, mpiminrealscalar=self.ident,
            mpisumreal1d=self.ident, mpiallsumreal1d=self.ident, mpiabort=self.abort,
            hdfstart=self.none, hdfclose=self.none, openlogs=self.none, writegridinfo=self.none,
            initdumprcuts=self.none, hdfserialreadintscalar=self.read_scalar,
            hdfserialreadrealscalar=self.read_scalar, hdfreadcontinua=self.read_continua,
            hdfcreateblankfile=self.h5_blank, hdfserialwriterealscalar=self.h5_scalar,
            hdfserialwriteintscalar=self.h5_int_scalar, hdfserialwritereal1d=self.h5_1d,
            hdfwritereal2d=self.h5_2d_slab, hdfwriteserialreal2d=self.h5_2d, hdfwriterealhalo3d=self.h5_halo_3d,
            hdfreadserialreal2d=self.h5_read_2d,
            quitroutine=self.quit, mpi_wtime=lambda: 0.0)
        self.F = F
        for name, fn in stubs.items():
            if not hasattr(F, name):
                setattr(F, name, fn)

    @staticmethod
    def none(*a, **k):
        return None

    @staticmethod
    def ident(*a, **k):
        return a

    def abort(self, *a):
        raise FortranStop("MpiAbort")

    def quit(self, tin, normalexit, errorcode):
        """QuitRoutine.F90:10-43: a normal exit writes the statistics and the
        continuation files (WriteStats, WriteFlowField) before the stop."""
        if int(errorcode) != 100 and normalexit:
            for name in ("writestats", "writeflowfield"):
                if hasattr(self.F, name):
                    getattr(self.F, name)()
        raise Quit(errorcode, normalexit)

    # ---- 2DECOMP&FFT
    def decomp_2d_init(self, nx, ny, nz, p_row, p_col, periodic=None):
        G = self.G
        for nm, vals in (("xstart", (1, 1, 1)), ("xend", (nx, ny, nz)), ("ystart", (1, 1, 1)),
                         ("yend", (nx, ny, nz)), ("zstart", (1, 1, 1)), ("zend", (nx, ny, nz))):
            a = getattr(G, nm)
            a.d = np.array(vals, dtype=np.int64)
            a.o = (1,)
        return None

    def decomp_2d_fft_init(self, *a):
        G = self.G
        G.ph = _decomp_info(G.nrm, G.nzm, G.nthm)
        G.sp = _decomp_info(G.nrm, G.nzm // 2 + 1, G.nthm)
        return None

    def update_halo(self, arr, level, opt_global=None, opt_decomp=None):
        """halo_common.f90, the in-memory branch taken when a pencil is its
        own neighbour (one rank, periodic in y and z): first the y planes
        over the whole array, then the z planes including the new y halos."""
        d = arr.d
        s2, s3 = d.shape[1], d.shape[2]
        ys, ye = 1 + level, s2 - level
        zs, ze = 1 + level, s3 - level
        for ilvl in range(1, level + 1):
            d[:, ye + ilvl - 1, :] = d[:, ys + (ilvl - 1) - 1, :]
            d[:, ys - ilvl - 1, :] = d[:, ye - (ilvl - 1) - 1, :]
        for ilvl in range(1, level + 1):
            d[:, :, ze + ilvl - 1] = d[:, :, zs + (ilvl - 1) - 1]
            d[:, :, zs - ilvl - 1] = d[:, :, ze - (ilvl - 1) - 1]
        return None

    def transpose(self, src, dst, decomp=None):
        """A transpose between pencils on one rank: mem_split packs the
        source in array element order, the all-to-all moves it to itself,
        mem_merge unpacks it in the destination's element order; for the
        common index ranges the destination element (i, j, k) receives the
        source element (i, j, k)."""
        n = [min(a, b) for a, b in zip(src.d.shape, dst.d.shape)]
        dst.d[:n[0], :n[1], :n[2]] = src.d[:n[0], :n[1], :n[2]]
        return None

    # ---- FFTW (guru interface), executed with numpy.fft
    @staticmethod
    def _dims(arr, count):
        out = []
        for i in range(count):
            o = arr.d[i]
            out.append((int(o.n), int(o.is_), int(o.os)))
        return out

    def plan_dft(self, rank, dims, howmany_rank, howmany_dims, a_in, a_out, sign, flags):
        (n, is_, os_), = self._dims(dims, rank)
        return Plan("c2c", n, is_, os_, self._dims(howmany_dims, howmany_rank), sign)

    def plan_r2c(self, rank, dims, howmany_rank, howmany_dims, a_in, a_out, flags):
        (n, is_, os_), = self._dims(dims, rank)
        return Plan("r2c", n, is_, os_, self._dims(howmany_dims, howmany_rank), -1)

    def plan_c2r(self, rank, dims, howmany_rank, howmany_dims, a_in, a_out, flags):
        (n, is_, os_), = self._dims(dims, rank)
        return Plan("c2r", n, is_, os_, self._dims(howmany_dims, howmany_rank), 1)

    def execute(self, plan, a_in, a_out):
        """The transform of every batch element: element t of a transform
        sits at base + t*stride of the flat (array element order) data."""
        src = a_in.d.reshape(-1, order="F")
        dst = a_out.d.reshape(-1, order="F")
        if not (np.shares_memory(src, a_in.d) and np.shares_memory(dst, a_out.d)):
            raise RuntimeError("FFTW execute on a non-contiguous array")
        ib = np.zeros(1, dtype=np.int64)
        ob = np.zeros(1, dtype=np.int64)
        for n_h, is_h, os_h in plan.howmany:
            ib = (ib[:, None] + np.arange(n_h) * is_h).reshape(-1)
            ob = (ob[:, None] + np.arange(n_h) * os_h).reshape(-1)
        n = plan.n
        if plan.kind == "c2c":
            x = src[ib[:, None] + np.arange(n) * plan.is_]
            y = np.fft.fft(x, axis=1) if plan.sign < 0 else np.fft.ifft(x, axis=1) * n
            dst[ob[:, None] + np.arange(n) * plan.os_] = y
        elif plan.kind == "r2c":
            x = src[ib[:, None] + np.arange(n) * plan.is_]
            y = np.fft.rfft(x, axis=1)
            dst[ob[:, None] + np.arange(n // 2 + 1) * plan.os_] = y
        else:
            x = src[ib[:, None] + np.arange(n // 2 + 1) * plan.is_]
            y = np.fft.irfft(x, n=n, axis=1) * n
            dst[ob[:, None] + np.arange(n) * plan.os_] = y
        return None

    # ---- LAPACK, through SciPy
    def gttrf(self, n, dl, d, du, du2, ipiv, info):
        from scipy.linalg import lapack
        fn = lapack.zgttrf if d.t == "c" else lapack.dgttrf
        n = int(n)
        r = fn(dl.d[:n - 1].copy(), d.d[:n].copy(), du.d[:n - 1].copy())
        dl2, d2, du2n, du2x, ipv, inf = r
        dl.d[:n - 1] = dl2
        d.d[:n] = d2
        du.d[:n - 1] = du2n
        du2.d[:max(n - 2, 0)] = du2x[:max(n - 2, 0)]
        ipiv.d[:n] = ipv
        return (n, dl, d, du, du2, ipiv, int(inf))

    def gttrs(self, trans, n, nrhs, dl, d, du, du2, ipiv, b, ldb, info):
        from scipy.linalg import lapack
        fn = lapack.zgttrs if d.t == "c" else lapack.dgttrs
        n = int(n)
        x, inf = fn(dl.d[:n - 1], d.d[:n], du.d[:n - 1], du2.d[:max(n - 2, 0)], ipiv.d[:n], b.d[:n].copy(),
                    trans=trans.upper())
        b.d[:n] = x
        return (trans, n, nrhs, dl, d, du, du2, ipiv, b, ldb, int(inf))

    # ---- HDF5 continua files
    def read_scalar(self, dsetname, filnam, var):
        """HdfSerialReadIntScalar / HdfSerialReadRealScalar
        (HdfRoutines.F90:217-269): from a file the run holds (written by it
        or given before it), else from the continua master scalars."""
        name = self._h5_name(filnam)
        if name in self.h5:
            v = self.h5[name][str(dsetname).strip()][0]
            return (dsetname, filnam, int(v) if np.asarray(v).dtype.kind == "i" else float(v))
        return (dsetname, filnam, self.continua[dsetname.strip()])

    def h5_read_2d(self, filename, dsetname, ndx, ndy, var):
        """HdfReadSerialReal2D (HdfRoutines.F90:501-529): var(ndx, ndy) from
        a file the run holds."""
        a = self.h5[self._h5_name(filename)][str(dsetname).strip()]
        var.d[:int(ndx), :int(ndy)] = a.T

    def read_continua(self, n1o, n2o, n3o, xs2, xe2, xs3, xe3, intvar, qua):
        """HdfReadContinua: the file's (nr, nz-1, nth-1) values into
        qua(1:n3o, xs2:xe2, xs3:xe3), the dummy being declared
        qua(1:n3o, xs2-lvlhalo:xe2+lvlhalo, xs3-lvlhalo:xe3+lvlhalo)
        (HdfReadContinua.F90:32-33) whatever the bounds of the actual."""
        name = {1: "qt", 2: "qr", 3: "qz"}[int(intvar)]
        src = self.continua[name]
        d = qua.d
        o = (1, xs2 - 1, xs3 - 1)
        d[1 - o[0]:n3o + 1 - o[0], xs2 - o[1]:xe2 + 1 - o[1], xs3 - o[2]:xe3 + 1 - o[2]] = src
        return None

    # ---- HDF5 output files: the datasets each write leaves in its file
    # (HdfRoutines.F90), C order (the reverse of the Fortran dims), copied
    # (the written arrays are often locals that the next call reuses)
    @staticmethod
    def _h5_name(filename):
        return os.path.normpath(str(filename).strip())

    def _h5_open(self, filename):
        """h5fopen_f(H5F_ACC_RDWR_F): the file must exist."""
        name = self._h5_name(filename)
        if name not in self.h5:
            raise RuntimeError(f"HDF5 file {name} opened for writing before it was created")
        return self.h5[name]

    def _h5_create(self, filename):
        """h5fcreate_f(H5F_ACC_TRUNC_F): a new, empty file."""
        self.h5[self._h5_name(filename)] = {}
        return self.h5[self._h5_name(filename)]

    def h5_blank(self, filename):
        """HdfCreateBlankFile (HdfRoutines.F90:11-22)."""
        self._h5_create(filename)

    def h5_scalar(self, dsetname, filename, n):
        """HdfSerialWriteRealScalar (HdfRoutines.F90:25-59): dims (1)."""
        self._h5_open(filename)[str(dsetname).strip()] = np.array([float(n)])

    def h5_int_scalar(self, dsetname, filename, n):
        """HdfSerialWriteIntScalar (HdfRoutines.F90:62-96): dims (1), integer."""
        self._h5_open(filename)[str(dsetname).strip()] = np.array([int(n)], dtype=np.int32)

    def h5_1d(self, dsetname, filename, var, sz):
        """HdfSerialWriteReal1D (HdfRoutines.F90:99-137): var(1:sz)."""
        self._h5_open(filename)[str(dsetname).strip()] = np.array(var.d.reshape(-1, order="F")[:int(sz)], copy=True)

    def h5_2d_slab(self, dsetname, filename, var):
        """HdfWriteReal2D (HdfRoutines.F90:139-214): a new file holding
        var(xstart(2):xend(2), xstart(3):xend(3)), dims (nzm, nthm)."""
        self._h5_create(filename)[str(dsetname).strip()] = np.array(var.d.T, order="C", copy=True)

    def h5_2d(self, filename, dsetname, ndx, ndy, var):
        """HdfWriteSerialReal2D (HdfRoutines.F90:533-566): a new file
        holding var(ndx, ndy)."""
        a = var.d.reshape(-1, order="F")[:int(ndx) * int(ndy)].reshape((int(ndx), int(ndy)), order="F")
        self._h5_create(filename)[str(dsetname).strip()] = np.array(a.T, order="C", copy=True)

    def h5_halo_3d(self, filnam1, qua):
        """HdfWriteRealHalo3D (HdfRoutines.F90:388-477): a new file holding
        dataset 'var' = qua(1:nr, xstart(2):xend(2), xstart(3):xend(3)) of
        the haloed array (1:nr, 0:nzm+1, 0:nthm+1)."""
        self._h5_create(filnam1)["var"] = np.array(qua.d[:, 1:-1, 1:-1].transpose(2, 1, 0), order="C", copy=True)

    # ---- formatted I/O
    @staticmethod
    def internal_write(fmt, values):
        """WRITE into a character variable with I edit descriptors only
        (Iw, Iw.m: right-justified in w columns, at least m digits)."""
        descs = [d.strip() for d in fmt.strip()[1:-1].split(",")]
        if len(descs) != len(values):
            raise RuntimeError(f"internal WRITE {fmt} of {len(values)} values")
        out = []
        for d, v in zip(descs, values):
            m = re.fullmatch(r"i(\d+)(?:\.(\d+))?", d)
            if not m:
                raise RuntimeError(f"internal WRITE: edit descriptor {d}")
            w, mn = int(m.group(1)), int(m.group(2) or 1)
            digits = str(abs(int(v))).rjust(mn, "0")
            txt = ("-" if int(v) < 0 else "") + digits
            out.append("*" * w if len(txt) > w else txt.rjust(w))
        return "".join(out)

    def open(self, unit, name):
        """OPEN: a file the caller supplied is read; any other name opens
        an output unit (what is written to it is dropped unless its unit
        number is captured)."""
        text = self.files.get(str(name).strip(), "")
        self.units[int(unit)] = [ln for ln in text.split("\n")]

    def exists(self, name):
        """INQUIRE(EXIST=): a file the caller supplied, or an HDF5 file the
        run holds."""
        return (str(name).strip().lstrip("./") in {k.lstrip("./") for k in self.files}
                or self._h5_name(name) in self.h5)

    def read(self, unit, fmt, types_):
        """One READ statement: list-directed (fmt '*') takes values from as
        many records as it needs and drops the rest of the last one; a
        character format takes the next record."""
        lines = self.units[int(unit)]
        if fmt != "*":
            lines.pop(0)
            return [""] * len(types_)
        vals = []
        while len(vals) < len(types_):
            rec = lines.pop(0)
            vals.extend(t for t in re.split(r"[,\s]+", rec.strip()) if t)
        out = []
        for v, t in zip(vals, types_):
            if t == "i":
                out.append(int(v))
            elif t == "r":
                out.append(float(v.lower().replace("d", "e")))
            elif t == "l":
                out.append(v.strip(".").lower().startswith("t"))
            else:
                out.append(v)
        return out

    def write(self, unit, values):
        self.written.setdefault(int(unit), []).append(list(values))
