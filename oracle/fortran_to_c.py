"""Build recipe for oracle/_ref: the reference's own Fortran routines, compiled.

TEST INFRASTRUCTURE ONLY.  Neither the library nor bench.py's timed GPU path
uses anything this script makes.

There is no Fortran compiler in this image, so the reference's hot-path
routines (code/sub_*.f90, code/cft_*.f90 of itsmoosh/g3m3) cannot be built
by its makefile.  This script is a translator for the small Fortran 90
subset those files use: it reads them where they lie, writes one C file
(oracle/_ref/g3m3_ref.c, never committed) with one function per subroutine,
``ref_<name>(...)``, every argument by reference as in Fortran, and compiles
it with gcc into oracle/_ref/libg3m3_ref.so.  A JSON file beside it lists
every routine's dummy arguments (name, type, rank) and every common block's
layout, which the tests use to call the routines through ctypes.

Semantics, chosen to match how the reference's makefile builds it
(``ifort -zero -save``):
- default REAL is float, REAL(dp)/DOUBLE PRECISION is double, INTEGER and
  LOGICAL are 32-bit; implicit typing i-n integer, a-h/o-z real;
- every local scalar and fixed-size local array is static and starts at
  zero (-save -zero); automatic arrays (bounds from dummies), which the
  reference's build keeps on the stack, get a buffer per call site and
  recursion depth that is reused, not zeroed, from call to call, except
  divB_correct's, which start at zero (its solver's first iterate);
- expressions are evaluated in the declared precision in source order, one
  rounding per operation (compiled with -ffp-contract=off, no fast-math);
  integer powers are multiplications (x**2 = x*x);
- MAX(a,b) is ``a > b ? a : b`` and MIN(a,b) is ``a < b ? a : b``, folded
  left over more arguments; SIGN(a,b) is |a| for b >= 0, so b = -0.0 gives
  +|a| (ifort's default, no -assume minus0);
- arrays are column-major with the declared lower bounds, array-element
  actual arguments pass the element's address (sequence association);
- OpenMP directives are comments; WRITE statements are dropped.

Usage: python oracle/fortran_to_c.py [reference_code_dir]
(default $G3M3_REFERENCE/code; with neither, only sources translated
earlier are compiled).  Exits 0 without output when that directory is
absent.
"""
from __future__ import annotations

import json
import os
import re
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")

# Routines whose automatic arrays start at zero on every call (see unit()).
ZERO_AUTOMATIC = {"divb_correct"}

# The hot-path routines, one file each (code/<file>.f90).
FILES = [
    "sub_push_ion", "sub_push_elec", "sub_push_bfld", "sub_BandE",
    "sub_fnd_evel", "sub_fnd_vtot", "sub_fnd_pres", "sub_calcur",
    "sub_lap_plasma", "sub_lap_elec", "sub_lap_bfld", "sub_flux_correct",
    "sub_fcsmooth", "sub_set_rho", "sub_set_speed_agrd", "sub_store_array",
    "sub_bndry_outer", "sub_bndry_inner", "sub_bndry_flanks", "sub_flanks",
    "sub_bndry_corer", "sub_corer", "sub_flanks_synced", "sub_divB_correct",
    "sub_sparse_solver", "sub_banded_tpose", "cft_trilin_interp",
    "cft_findgrid", "sub_flux_counter", "sub_dipole", "sub_set_resist",
]


class TranslateError(Exception):
    pass


# --------------------------------------------------------------------------
# Source form: comments, continuation lines, case
# --------------------------------------------------------------------------

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
        else:
            if ch in "'\"":
                q = ch
            out.append(ch.lower())
    return "".join(out)


def _split_semicolons(s):
    parts, q, cur = [], None, []
    for ch in s:
        if q:
            cur.append(ch)
            if ch == q:
                q = None
        elif ch in "'\"":
            q = ch
            cur.append(ch)
        elif ch == ";":
            parts.append("".join(cur))
            cur = []
        else:
            cur.append(ch)
    parts.append("".join(cur))
    return [p.strip() for p in parts if p.strip()]


def statements(text):
    """Yield (line_number, statement) with comments removed and free-form
    continuation lines joined (blank and comment lines inside a continued
    statement are skipped, as the standard allows)."""
    buf, start = "", None
    for n, raw in enumerate(text.splitlines(), 1):
        d = raw.strip().lower()
        if d.startswith("!$omp") and not buf:
            yield n, "!$omp " + " ".join(d[5:].split())   # an OpenMP directive
            continue
        s = _strip_comment(raw.replace("\t", " ")).strip()
        if not s:
            continue
        if buf:
            if s.startswith("&"):
                buf += s[1:]
            else:
                buf += " " + s
        else:
            buf, start = s, n
        if buf.endswith("&"):
            buf = buf[:-1].rstrip()
            continue
        for part in _split_semicolons(_lower_outside_strings(buf)):
            yield start, part
        buf = ""
    if buf:
        raise TranslateError(f"line {start}: file ends inside a continued statement")


# --------------------------------------------------------------------------
# Expressions
# --------------------------------------------------------------------------

_TOKEN = re.compile(r"""
    (?P<ws>\s+)
  | (?P<str>'(?:[^']|'')*'|"(?:[^"]|"")*")
  | (?P<real>(?:\d+\.(?!(?:eq|ne|lt|le|gt|ge|and|or|not|eqv|neqv)\.)\d*|\.\d+)(?:[ed][+-]?\d+)?(?:_\w+)?
            |\d+[ed][+-]?\d+(?:_\w+)?)
  | (?P<int>\d+(?:_\w+)?)
  | (?P<dotop>\.(?:eq|ne|lt|le|gt|ge|and|or|not|eqv|neqv|true|false)\.)
  | (?P<op>\*\*|==|/=|<=|>=|::|=>|[-+*/()<>=,:%])
  | (?P<name>[a-z_][a-z0-9_]*)
""", re.X)


def tokenize(s):
    pos, out = 0, []
    while pos < len(s):
        m = _TOKEN.match(s, pos)
        if not m:
            raise TranslateError(f"cannot tokenize {s[pos:pos + 20]!r} in {s!r}")
        pos = m.end()
        kind = m.lastgroup
        if kind == "ws":
            continue
        out.append((kind, m.group()))
    return out


_DOT = {".eq.": "==", ".ne.": "/=", ".lt.": "<", ".le.": "<=", ".gt.": ">",
        ".ge.": ">="}


class Parser:
    """Recursive descent over Fortran expression precedence:
    .or. < .and. < .not. < relational < +,- (binary and unary) < *,/ < **."""

    def __init__(self, toks):
        self.t = toks
        self.i = 0

    def peek(self, k=0):
        j = self.i + k
        return self.t[j] if j < len(self.t) else (None, None)

    def take(self, val=None):
        tok = self.peek()
        if val is not None and tok[1] != val:
            raise TranslateError(f"expected {val!r}, got {tok[1]!r}")
        self.i += 1
        return tok

    def at(self, *vals):
        return self.peek()[1] in vals

    def done(self):
        return self.i >= len(self.t)

    def expr(self):
        e = self.and_()
        while self.at(".or."):
            self.take()
            e = ("bin", "||", e, self.and_())
        return e

    def and_(self):
        e = self.not_()
        while self.at(".and."):
            self.take()
            e = ("bin", "&&", e, self.not_())
        return e

    def not_(self):
        if self.at(".not."):
            self.take()
            return ("not", self.not_())
        return self.rel()

    def rel(self):
        e = self.add()
        tok = self.peek()[1]
        tok = _DOT.get(tok, tok)
        if tok in ("==", "/=", "<", "<=", ">", ">="):
            self.take()
            e = ("rel", tok, e, self.add())
        return e

    def add(self):
        if self.at("+", "-"):
            op = self.take()[1]
            e = self.mul()
            if op == "-":
                e = ("neg", e)
        else:
            e = self.mul()
        while self.at("+", "-"):
            op = self.take()[1]
            e = ("bin", op, e, self.mul())
        return e

    def mul(self):
        e = self.pow_()
        while self.at("*", "/"):
            op = self.take()[1]
            e = ("bin", op, e, self.pow_())
        return e

    def pow_(self):
        base = self.unary_operand()
        if self.at("**"):
            self.take()
            return ("pow", base, self.pow_operand())
        return base

    def pow_operand(self):
        # the exponent of ** may itself carry a sign and is right-associative
        if self.at("-", "+"):
            op = self.take()[1]
            e = self.pow_()
            return ("neg", e) if op == "-" else e
        return self.pow_()

    def unary_operand(self):
        # extension accepted by every compiler: a * -b
        if self.at("-", "+"):
            op = self.take()[1]
            e = self.pow_()
            return ("neg", e) if op == "-" else e
        return self.primary()

    def primary(self):
        kind, val = self.take()
        if kind == "real":
            return ("real", val)
        if kind == "int":
            return ("int", val)
        if kind == "str":
            return ("str", val)
        if kind == "dotop" and val in (".true.", ".false."):
            return ("logic", val == ".true.")
        if val == "(":
            e = self.expr()
            self.take(")")
            return ("paren", e)
        if kind == "name":
            if self.at("("):
                self.take("(")
                args = []
                if not self.at(")"):
                    while True:
                        args.append(self.subscript())
                        if self.at(","):
                            self.take()
                            continue
                        break
                self.take(")")
                return ("ref", val, args)
            return ("name", val)
        raise TranslateError(f"unexpected token {val!r}")

    def subscript(self):
        if self.at(":"):
            self.take()
            hi = None if self.at(",", ")") else self.expr()
            return ("slice", None, hi)
        e = self.expr()
        if self.at(":"):
            self.take()
            hi = None if self.at(",", ")") else self.expr()
            return ("slice", e, hi)
        return e


def parse_expr(s):
    p = Parser(tokenize(s))
    e = p.expr()
    if not p.done():
        raise TranslateError(f"trailing tokens in expression {s!r}: {p.t[p.i:]}")
    return e


def split_top(s, sep=","):
    """Split at top-level separators (outside parentheses and strings)."""
    parts, depth, q, cur = [], 0, None, []
    for ch in s:
        if q:
            cur.append(ch)
            if ch == q:
                q = None
            continue
        if ch in "'\"":
            q = ch
        elif ch in "([":
            depth += 1
        elif ch in ")]":
            depth -= 1
        if ch == sep and depth == 0:
            parts.append("".join(cur).strip())
            cur = []
        else:
            cur.append(ch)
    if "".join(cur).strip():
        parts.append("".join(cur).strip())
    return parts


def matching_paren(s, i):
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
                return j
    raise TranslateError(f"unbalanced parentheses in {s!r}")


# --------------------------------------------------------------------------
# Symbols
# --------------------------------------------------------------------------

# the C type of default REAL: float, or double for the reference's FP64 build
# (what -fdefault-real-8 gives: default REAL variables and literals in
# double precision; REAL(dp) stays double)
REAL = {"t": "float"}

CTYPE = {"int": "int", "float": "float", "double": "double", "logical": "int",
         "char": "char"}
RANK = {"logical": 0, "int": 1, "float": 2, "double": 3}
SIZE = {"int": 4, "float": 4, "double": 8, "logical": 4, "char": 1}


DEFERRED = ("deferred", None)     # a ':' bound of an allocatable array


def pexpr(e):
    """The AST of a parameter or initialiser, parsing lazy ones on use."""
    if e is not None and e[0] == "lazy":
        return parse_expr(e[1])
    return e


class Sym:
    def __init__(self, name):
        self.name = name
        self.type = None          # int, float, double, logical, char
        self.dims = None          # list of (lo_ast, hi_ast or None for '*')
        self.param = None         # AST of a PARAMETER value
        self.init = None          # AST of an initialiser (implies SAVE)
        self.common = None        # (block, byte offset)
        self.is_dummy = False
        self.charlen = 1


class Unit:
    def __init__(self, name, args, src):
        self.name = name
        self.args = args
        self.src = src
        self.syms = {}
        self.implicit_none = False
        self.body = []            # (lineno, stmt) after the declarations
        self.commons = {}         # block -> [names in order]
        self.uses = []            # modules named in USE statements
        self.kind = "subroutine"  # or "program", "module"

    def sym(self, name):
        if name not in self.syms:
            self.syms[name] = Sym(name)
        return self.syms[name]

    def type_of(self, name):
        s = self.syms.get(name)
        if s is not None and s.type is not None:
            return s.type
        if self.implicit_none:
            raise TranslateError(f"{self.name}: {name} has no type under implicit none")
        return "int" if name[0] in "ijklmn" else REAL["t"]


_DECL = re.compile(r"^(integer|real|double\s*precision|logical|character)\b(.*)$")


def parse_units(path):
    text = open(path, encoding="latin-1").read()
    units, cur, in_decl = [], None, False
    for ln, st in statements(text):
        m = re.match(r"^(?:recursive\s+)?subroutine\s+(\w+)\s*(?:\((.*)\))?\s*$", st)
        if m:
            args = [a.strip() for a in (m.group(2) or "").split(",") if a.strip()]
            cur = Unit(m.group(1), args, os.path.basename(path))
            for a in args:
                cur.sym(a).is_dummy = True
            in_decl = True
            units.append(cur)
            continue
        if re.match(r"^end(\s*subroutine\b.*)?$", st):
            cur = None
            continue
        if cur is None:
            raise TranslateError(f"{path}:{ln}: statement outside a subroutine: {st!r}")
        if in_decl and declaration(cur, st, ln):
            continue
        in_decl = False
        cur.body.append((ln, st))
    return units


def _kind_type(base, spec):
    base = re.sub(r"\s+", " ", base)
    if base == "double precision":
        return "double"
    if base == "integer":
        return "int"
    if base == "logical":
        return "logical"
    if base == "character":
        return "char"
    # real, real(dp), real(kind=dp), real*8
    spec = spec.replace(" ", "")
    if spec in ("(dp)", "(kind=dp)", "*8", "(8)", "(kind=8)"):
        return "double"
    if spec in ("", "*4", "(4)", "(kind=4)"):
        return REAL["t"]
    raise TranslateError(f"unsupported real kind {spec!r}")


def _entity_dims(u, s):
    """'a(1:n, m)' -> ('a', [(lo, hi)...]); 'a' -> ('a', None)."""
    m = re.match(r"^(\w+)\s*(\(.*\))?\s*(\*\s*\d+)?\s*(=.*)?$", s)
    if not m:
        raise TranslateError(f"{u.name}: cannot read declaration entity {s!r}")
    name, dims, init = m.group(1), m.group(2), m.group(4)
    dl = None
    if dims:
        dl = []
        for d in split_top(dims[1:-1]):
            if d == "*":
                dl.append((("int", "1"), None))
            elif d.strip() == ":":
                dl.append(DEFERRED)
            elif ":" in d and not d.startswith("("):
                lo, hi = d.split(":", 1)
                dl.append((parse_expr(lo), None if hi.strip() == "*" else parse_expr(hi)))
            else:
                dl.append((("int", "1"), parse_expr(d)))
    # initialisers are parsed when used: some (array constructors, strings)
    # are never needed
    return name, dl, (("lazy", init[1:].strip()) if init else None)


def declaration(u, st, ln):
    if st == "implicit none":
        u.implicit_none = True
        return True
    if st.startswith("implicit "):
        raise TranslateError(f"{u.name}: IMPLICIT other than none is not supported")
    if st.startswith("!$omp"):
        return False           # a directive starts the executable part
    if st.startswith("!$") or st in ("save",):
        return True
    m = re.match(r"^dimension\s+(.*)$", st)
    if m and "::" not in st:
        for ent in split_top(m.group(1)):
            name, dl, _ = _entity_dims(u, ent)
            u.sym(name).dims = dl
        return True
    m = re.match(r"^common\s*/\s*(\w+)\s*/\s*(.*)$", st)
    if m:
        blk = m.group(1)
        names = []
        for ent in split_top(m.group(2)):
            name, dl, _ = _entity_dims(u, ent)
            if dl is not None:
                u.sym(name).dims = dl
            names.append(name)
        u.commons.setdefault(blk, []).extend(names)
        return True
    m = re.match(r"^parameter\s*\((.*)\)$", st)
    if m:
        for ent in split_top(m.group(1)):
            name, val = ent.split("=", 1)
            u.sym(name.strip()).param = ("lazy", val.strip())
        return True
    m = re.match(r"^use\s+(\w+)", st)
    if m:
        u.uses.append(m.group(1))
        return True
    if st.startswith("namelist"):
        return True
    m = _DECL.match(st)
    if not m:
        return False
    base, rest = m.group(1), m.group(2)
    # kind / length selector
    spec = ""
    km = re.match(r"^\s*(\((?:[^()]|\([^()]*\))*\)|\*\s*\d+)", rest)
    if km and not rest.lstrip().startswith("::"):
        spec = km.group(1)
        rest = rest[km.end():]
    typ = _kind_type(base, spec)
    attrs, ents = [], rest
    if "::" in rest:
        head, ents = rest.split("::", 1)
        attrs = [a.strip() for a in split_top(head) if a.strip()]
    else:
        ents = rest.strip()
        if ents.startswith(","):
            raise TranslateError(f"{u.name}: attributes need '::' in {st!r}")
    is_param, adims = False, None
    for a in attrs:
        if a == "parameter":
            is_param = True
        elif a.startswith("dimension"):
            _, adims, _ = _entity_dims(u, "x" + a[len("dimension"):])
        elif a.startswith("intent") or a in ("save", "target", "optional", "allocatable"):
            pass
        else:
            raise TranslateError(f"{u.name}: unsupported attribute {a!r}")
    for ent in split_top(ents):
        name, dl, init = _entity_dims(u, ent)
        s = u.sym(name)
        s.type = typ
        if dl is not None:
            s.dims = dl
        elif adims is not None:
            s.dims = adims
        if is_param:
            s.param = init
        elif init is not None:
            s.init = init
    return True


# --------------------------------------------------------------------------
# Code generation
# --------------------------------------------------------------------------

INTRINSIC_REAL = {"sqrt": "sqrt", "exp": "exp", "log": "log", "alog": "log",
                  "sin": "sin", "cos": "cos", "tan": "tan", "atan": "atan",
                  "asin": "asin", "acos": "acos", "sinh": "sinh",
                  "cosh": "cosh", "tanh": "tanh", "log10": "log10",
                  "alog10": "log10"}


class Gen:
    def __init__(self, units):
        self.units = {u.name: u for u in units}
        self.commons = {}     # block -> (size, [(name, type, offset, count)])
        self.u = None
        self.tmp = 0
        self.loop = 0
        self.retyped = {}     # unit -> {dummy: type its callee reads it as}
        self.main = False     # translating the main program's loop
        self.omp = False      # OpenMP directives become parallel loops
        for u in units:
            self.layout_commons(u)

    # ---- common blocks: byte layout from each unit's own declaration ----
    def layout_commons(self, u):
        for blk, names in u.commons.items():
            off, members = 0, []
            for n in names:
                s = u.sym(n)
                t = u.type_of(n)
                cnt = 1
                if s.dims:
                    for lo, hi in s.dims:
                        cnt *= self.const_int(u, hi) - self.const_int(u, lo) + 1
                align = SIZE[t]
                if off % align:
                    raise TranslateError(f"common /{blk}/ member {n} misaligned")
                s.common = (blk, off)
                members.append((n, t, off, cnt))
                off += SIZE[t] * cnt
            prev = self.commons.get(blk)
            if prev is None or prev[0] < off:
                self.commons[blk] = (off, members)

    def const_int(self, u, e):
        v = self.eval_const(u, e)
        if not isinstance(v, int):
            raise TranslateError(f"{u.name}: {e} is not an integer constant")
        return v

    def eval_const(self, u, e):
        k = e[0]
        if k == "int":
            return int(e[1].split("_")[0])
        if k == "real":
            return float(e[1].split("_")[0].replace("d", "e"))
        if k == "name":
            s = u.syms.get(e[1])
            if s is not None and s.param is not None:
                v = self.eval_const(u, pexpr(s.param))
                return int(v) if u.type_of(e[1]) == "int" else v
            raise TranslateError(f"{u.name}: {e[1]} is not a constant")
        if k == "ref" and e[1] == "kind":
            a = e[2][0]
            return 8 if (a[0] == "real" and "d" in a[1]) else 4
        if k == "neg":
            return -self.eval_const(u, e[1])
        if k == "paren":
            return self.eval_const(u, e[1])
        if k == "bin":
            a, b = self.eval_const(u, e[2]), self.eval_const(u, e[3])
            return {"+": a + b, "-": a - b, "*": a * b,
                    "/": (int(a / b) if isinstance(a, int) and isinstance(b, int) else a / b)}[e[1]]
        raise TranslateError(f"{u.name}: not a constant expression: {e}")

    def is_array(self, name):
        s = self.u.syms.get(name)
        return s is not None and s.dims is not None

    def new_tmp(self):
        self.tmp += 1
        return f"t_{self.tmp}"

    # ---- expressions: return (C code, type) ----
    def ex(self, e):
        k = e[0]
        if k == "int":
            return e[1].split("_")[0], "int"
        if k == "real":
            txt = e[1]
            kind = ""
            if "_" in txt:
                txt, kind = txt.split("_", 1)
            dbl = "d" in txt or kind in ("dp", "8")
            txt = txt.replace("d", "e")
            if txt.startswith("."):
                txt = "0" + txt
            txt = re.sub(r"\.(e|$)", r".0\1", txt)
            if REAL["t"] == "double":
                return f"{txt}", "double"
            return (f"{txt}", "double") if dbl else (f"{txt}f", "float")
        if k == "logic":
            return ("1" if e[1] else "0"), "logical"
        if k == "str":
            return '"' + e[1][1:-1].replace('"', '\\"') + '"', "char"
        if k == "paren":
            c, t = self.ex(e[1])
            return f"({c})", t
        if k == "neg":
            c, t = self.ex(e[1])
            return f"(-{c})", t
        if k == "not":
            c, _ = self.ex(e[1])
            return f"(!{c})", "logical"
        if k == "bin":
            op = e[1]
            a, ta = self.ex(e[2])
            b, tb = self.ex(e[3])
            if op in ("&&", "||"):
                return f"({a} {op} {b})", "logical"
            t = ta if RANK[ta] >= RANK[tb] else tb
            return f"({a} {op} {b})", t
        if k == "rel":
            op = {"/=": "!="}.get(e[1], e[1])
            a, _ = self.ex(e[2])
            b, _ = self.ex(e[3])
            return f"({a} {op} {b})", "logical"
        if k == "pow":
            return self.power(e[1], e[2])
        if k == "name":
            return self.name_ref(e[1])
        if k == "ref":
            return self.ref(e[1], e[2])
        raise TranslateError(f"unsupported expression {e}")

    def power(self, base, expo):
        b, tb = self.ex(base)
        if expo[0] == "int":
            n = int(expo[1])
            if 1 <= n <= 4:
                t = self.new_tmp()
                # gcc's powi expansion: x*x, (x*x)*x, (x*x)*(x*x)
                chain = {1: f"{t}", 2: f"{t}*{t}", 3: f"({t}*{t})*{t}",
                         4: f"({t}*{t})*({t}*{t})"}[n]
                return f"({{ {CTYPE[tb]} {t} = {b}; {chain}; }})", tb
        e, te = self.ex(expo)
        if te == "int":
            fn = {"float": "ref_powif", "double": "ref_powid", "int": "ref_powii"}[tb]
            return f"{fn}({b}, {e})", tb
        t = tb if RANK[tb] >= RANK[te] else te
        if t == "int":
            t = REAL["t"]
        fn = "powf" if t == "float" else "pow"
        return f"{fn}({b}, {e})", t

    def name_ref(self, n):
        u = self.u
        s = u.syms.get(n)
        if s is not None and s.param is not None and s.dims is None:
            t = u.type_of(n)
            if t == "int":
                return str(int(self.eval_const(u, pexpr(s.param)))), "int"
            # a REAL parameter is its defining expression, converted once
            c, _ = self.ex(pexpr(s.param))
            return f"(({CTYPE[t]})({c}))", t
        t = u.type_of(n)
        if s is not None and s.dims is not None:
            return self.cn(n), t + "[]"
        if s is not None and s.common is not None:
            blk, off = s.common
            return f"(*({CTYPE[t]}*)(ref_common_{blk} + {off}))", t
        if s is not None and s.is_dummy:
            return f"(*{n})", t
        if not n.startswith("s_"):
            self.locals_used.add(n)
        return self.cn(n), t

    def cn(self, n):
        """C name of a variable: the main program's variables are globals."""
        if self.main and not n.startswith("s_"):
            s = self.u.syms.get(n)
            if s is None or (s.common is None and not s.is_dummy):
                return "ref_main_" + n
        return n

    def index(self, n, args):
        s = self.u.syms[n]
        if len(args) != len(s.dims):
            raise TranslateError(f"{self.u.name}: {n} has rank {len(s.dims)}, indexed with {len(args)}")
        terms = []
        for d in range(len(args) - 1, -1, -1):
            c, t = self.ex(args[d])
            if t != "int":
                raise TranslateError(f"{self.u.name}: non-integer subscript of {n}")
            lo = f"{self.cn(n)}_lo{d}"
            term = f"((long)({c}) - {lo})"
            if terms:
                terms = [f"({term} + {self.cn(n)}_ex{d} * {terms[0]})"]
            else:
                terms = [term]
        return terms[0]

    def ref(self, n, args):
        u = self.u
        if self.is_array(n):
            if any(a[0] == "slice" for a in args):
                raise TranslateError(f"{u.name}: array section {n} outside an assignment")
            t = u.type_of(n)
            return f"{self.cn(n)}[{self.index(n, args)}]", t
        return self.intrinsic(n, args)

    def intrinsic(self, n, args):
        cs = [self.ex(a) for a in args]
        codes = [c for c, _ in cs]
        types = [t for _, t in cs]
        if n in ("max", "min", "amax1", "amin1", "max0", "min0", "dmax1", "dmin1"):
            t = max(types, key=lambda x: RANK[x])
            if n in ("amax1", "amin1"):
                t = REAL["t"]
            fn = f"ref_{'max' if 'max' in n else 'min'}_{CTYPE[t]}"
            acc = f"(({CTYPE[t]}){codes[0]})"
            for c in codes[1:]:
                acc = f"{fn}({acc}, ({CTYPE[t]})({c}))"
            return acc, t
        if n in ("abs", "iabs", "dabs"):
            t = types[0]
            fn = {"int": "abs", "float": "fabsf", "double": "fabs"}[t]
            return f"{fn}({codes[0]})", t
        if n == "sign":
            t = types[0]
            fn = {"int": "ref_sign_int", "float": "ref_sign_float", "double": "ref_sign_double"}[t]
            return f"{fn}({codes[0]}, {codes[1]})", t
        if n in INTRINSIC_REAL:
            t = types[0]
            if t == "int":
                raise TranslateError(f"{self.u.name}: {n} of an integer")
            fn = INTRINSIC_REAL[n] + ("f" if t == "float" else "")
            return f"{fn}({codes[0]})", t
        if n == "atan2":
            t = types[0]
            return f"{'atan2f' if t == 'float' else 'atan2'}({codes[0]}, {codes[1]})", t
        if n in ("float", "real", "sngl"):
            if len(args) == 2 or REAL["t"] == "double":
                return f"((double)({codes[0]}))", "double"
            return f"((float)({codes[0]}))", "float"
        if n == "dble":
            return f"((double)({codes[0]}))", "double"
        if n in ("int", "ifix", "idint"):
            return f"((int)({codes[0]}))", "int"
        if n == "nint":
            fn = "lroundf" if types[0] == "float" else "lround"
            return f"((int){fn}({codes[0]}))", "int"
        if n == "mod":
            t = types[0]
            if t == "int":
                return f"(({codes[0]}) % ({codes[1]}))", "int"
            return f"{'fmodf' if t == 'float' else 'fmod'}({codes[0]}, {codes[1]})", t
        raise TranslateError(f"{self.u.name}: unknown function or undeclared array {n!r}")

    # ---- statements ----
    def lhs(self, s):
        """Return (target-code, type) for an assignment target."""
        e = parse_expr(s)
        if e[0] == "name":
            c, t = self.name_ref(e[1])
            if t.endswith("[]"):
                return ("whole", e[1]), t[:-2]
            return c, t
        if e[0] == "ref" and self.is_array(e[1]):
            if any(a[0] == "slice" for a in e[2]):
                return ("section", e), self.u.type_of(e[1])
            return self.ref(e[1], e[2])
        raise TranslateError(f"{self.u.name}: cannot assign to {s!r}")

    def section_assign(self, target, rhs_s, out, ind):
        """a(:,:,:) = expr over full-extent sections (elementwise)."""
        if target[0] == "whole":
            name = target[1]
            s = self.u.syms[name]
            targ = ("ref", name, [("slice", None, None)] * len(s.dims))
        else:
            targ = target[1]
        rhs = parse_expr(rhs_s)
        name, subs = targ[1], targ[2]
        loopvars, k = [], 0
        for d, sub in enumerate(subs):
            if sub[0] == "slice":
                if sub[1] is not None or sub[2] is not None:
                    raise TranslateError(f"{self.u.name}: partial section of {name}")
                loopvars.append((d, f"s_{k}"))
                k += 1
        rank = len(loopvars)

        def subst(e):
            # replace every full section's ':' by the loop variables in order
            if e[0] == "name" and self.is_array(e[1]):
                ds = self.u.syms[e[1]].dims
                if len(ds) != rank:
                    raise TranslateError(f"{self.u.name}: shape mismatch in section assignment")
                return ("ref", e[1], [("name", f"s_{i}") for i in range(rank)])
            if e[0] == "ref" and self.is_array(e[1]):
                kk, na = 0, []
                for a in e[2]:
                    if a[0] == "slice":
                        na.append(("name", f"s_{kk}"))
                        kk += 1
                    else:
                        na.append(a)
                if kk not in (0, rank):
                    raise TranslateError(f"{self.u.name}: shape mismatch in section assignment")
                return ("ref", e[1], na)
            if e[0] == "ref":          # elemental intrinsic
                return ("ref", e[1], [subst(a) for a in e[2]])
            if e[0] in ("bin", "rel"):
                return (e[0], e[1], subst(e[2]), subst(e[3]))
            if e[0] in ("neg", "not", "paren"):
                return (e[0], subst(e[1]))
            if e[0] == "pow":
                return ("pow", subst(e[1]), subst(e[2]))
            return e

        # number the slice loop variables in order of the slices
        kk, na = 0, []
        for sub in subs:
            if sub[0] == "slice":
                na.append(("name", f"s_{kk}"))
                kk += 1
            else:
                na.append(sub)
        lhs = ("ref", name, na)
        # loop bounds from the target's declared bounds; the s_* are ints
        for i in range(rank):
            self.u.sym(f"s_{i}").type = "int"
        # outermost loop over the last sliced dimension (column-major order)
        body_ind = ind
        opened = 0
        for i in range(rank - 1, -1, -1):
            d = loopvars[i][0]
            cb = self.cn(name)
            out.append(f"{'  ' * body_ind}for (int s_{i} = (int){cb}_lo{d}; s_{i} < (int)({cb}_lo{d} + {cb}_ex{d}); s_{i}++) {{")
            body_ind += 1
            opened += 1
        lc, lt = self.ex(lhs)
        rc, _ = self.ex(subst(rhs))
        out.append(f"{'  ' * body_ind}{lc} = ({CTYPE[lt]})({rc});")
        for i in range(opened):
            body_ind -= 1
            out.append(f"{'  ' * body_ind}}}")

    def section_temp(self, e, ct, pre, post):
        """An array section as an actual argument: a contiguous copy made
        before the call and copied back after it (what a compiler does for a
        non-contiguous section such as grid_minvals(1,:))."""
        name, subs = e[1], e[2]
        tmp = self.new_tmp()
        cb = self.cn(name)
        vars_, na = [], []
        for d, sub in enumerate(subs):
            if sub[0] == "slice":
                if sub[1] is not None or sub[2] is not None:
                    raise TranslateError(f"{self.u.name}: partial section of {name} as an argument")
                v = f"s_{tmp}_{d}"
                self.u.sym(v).type = "int"
                vars_.append((d, v))
                na.append(("name", v))
            else:
                na.append(sub)
        elem, _ = self.ref(name, na)
        size = " * ".join(f"{cb}_ex{d}" for d, _ in vars_)
        pre.append(f"{ct}* {tmp} = ({ct}*)malloc(sizeof({ct}) * (size_t)({size})); long n_{tmp} = 0;")
        loops_open = ""
        for d, v in reversed(vars_):
            loops_open += f"for (int {v} = (int){cb}_lo{d}; {v} < (int)({cb}_lo{d} + {cb}_ex{d}); {v}++) "
        pre.append(loops_open + f"{tmp}[n_{tmp}++] = {elem};")
        post.append(f"n_{tmp} = 0; " + loops_open + f"{elem} = {tmp}[n_{tmp}++];")
        post.append(f"free({tmp});")
        return tmp

    def call(self, name, argstr, out, ind):
        pad = "  " * ind
        if name not in self.units:
            if not self.main:
                raise TranslateError(f"{self.u.name}: call to {name}, which is not translated")
            # the main loop's calls outside the hot path are recorded, not run
            out.append(f'{pad}ref_untranslated("{name}");')
            return
        callee = self.units[name]
        actuals = split_top(argstr) if argstr.strip() else []
        if len(actuals) != len(callee.args):
            raise TranslateError(f"{self.u.name}: call {name} with {len(actuals)} of {len(callee.args)} arguments")
        pre, cargs, post = [], [], []
        for a_s, dummy in zip(actuals, callee.args):
            # a dummy the callee only hands on is read as its callee's type
            dt = self.retyped.get(name, {}).get(dummy, callee.type_of(dummy))
            e = parse_expr(a_s)
            if e[0] == "ref" and self.is_array(e[1]) and any(a[0] == "slice" for a in e[2]):
                cargs.append(self.section_temp(e, CTYPE[self.u.type_of(e[1])], pre, post))
                continue
            sym = self.u.syms.get(e[1]) if e[0] == "name" else None
            if e[0] == "name" and not (sym is not None and sym.param is not None and sym.dims is None):
                c, t = self.name_ref(e[1])
                if t.endswith("[]"):
                    cargs.append(c)
                    continue
                s = self.u.syms.get(e[1])
                if CTYPE[t] != CTYPE[dt]:
                    # Without interfaces the compiler passes the address and
                    # the callee reads it as its own type.  A dummy handed on
                    # unread keeps the caller's bits (bndry_flanks declares
                    # its t implicitly REAL but only passes it to flanks,
                    # which reads REAL(dp)); anything else is an error.
                    if not (s is not None and s.is_dummy):
                        raise TranslateError(f"{self.u.name}: call {name}: {e[1]} is {t}, dummy {dummy} is {dt}")
                    cargs.append(f"({CTYPE[dt]}*){e[1]}")
                    self.retyped.setdefault(self.u.name, {})[e[1]] = dt
                    continue
                if s is not None and s.is_dummy and s.common is None:
                    arg = e[1]
                else:
                    arg = f"&{c}" if not c.startswith("(*") else c[2:-1]
                declared = CTYPE[callee.type_of(dummy)]
                if declared != CTYPE[dt]:      # the callee only hands it on
                    arg = f"({declared}*){arg}"
                cargs.append(arg)
                continue
            if e[0] == "ref" and self.is_array(e[1]):
                c, t = self.ref(e[1], e[2])
                cargs.append(f"&{c}")
                continue
            c, t = self.ex(e)
            tmp = self.new_tmp()
            pre.append(f"{CTYPE[dt]} {tmp} = ({CTYPE[dt]})({c});")
            cargs.append(f"&{tmp}")
        out.append(pad + "{ " + " ".join(pre) + f" ref_{name}(" + ", ".join(cargs) + "); "
                   + " ".join(post) + " }")

    def omp_private(self, u, start):
        """Scalars a parallel loop assigns (its temporaries and inner loop
        indices): private to each thread, which is what the loop's
        iterations being independent requires.  The reference's directives
        name no clauses, so its own OpenMP build shares them and races."""
        depth, names = 0, []
        for _, st in u.body[start:]:
            if _DO_START.match(st):
                depth += 1
                m = re.match(r"^do\s+(\w+)\s*=", st)
                if m and m.group(1) not in names:
                    names.append(m.group(1))
            elif _DO_END.match(st):
                depth -= 1
                if depth == 0:
                    break
            else:
                tail = st
                m = re.match(r"^if\s*\(", st)
                if m:
                    j = matching_paren(st, m.end() - 1)
                    tail = st[j + 1:].strip()
                m = re.match(r"^(\w+)\s*=(?!=)", tail)
                if m and m.group(1) not in names:
                    names.append(m.group(1))
        out = []
        for n in names[1:] if names else []:
            sym = u.syms.get(n)
            if sym is not None and sym.dims is not None:
                continue
            if sym is not None and (sym.is_dummy or sym.common is not None):
                raise TranslateError(f"{u.name}: parallel loop assigns the shared scalar {n}")
            self.locals_used.add(n)
            out.append(self.cn(n))
        return out

    def body(self, u):
        out = []
        ind = 1
        stack = []
        pending_omp = False
        for idx, (ln, st) in enumerate(u.body):
            self.where = (u.src, ln, st)
            pad = "  " * ind
            out.append(f"{pad}/* {u.src}:{ln} */")
            if st.startswith("!$"):
                pending_omp = st.startswith("!$omp parallel do")
                continue
            omp_here, pending_omp = pending_omp, False
            m = re.match(r"^(\d+)\s+(.*)$", st)
            if m:
                raise TranslateError(f"{u.src}:{ln}: labels are not supported")
            if re.match(r"^do\s+while\s*\(", st):
                cond = st[st.index("("):]
                j = matching_paren(cond, 0)
                c, _ = self.ex(parse_expr(cond[1:j]))
                out.append(f"{pad}while ({c}) {{")
                stack.append("do")
                ind += 1
                continue
            m = re.match(r"^do\s+(\w+)\s*=\s*(.*)$", st)
            if m:
                var = m.group(1)
                parts = split_top(m.group(2))
                lo, _ = self.ex(parse_expr(parts[0]))
                hi, _ = self.ex(parse_expr(parts[1]))
                step = self.ex(parse_expr(parts[2]))[0] if len(parts) > 2 else "1"
                vc, _ = self.name_ref(var)
                self.loop += 1
                L = self.loop
                if omp_here and self.omp and len(parts) > 2:
                    try:
                        self.eval_const(u, parse_expr(parts[2]))
                    except TranslateError:
                        omp_here = False      # a step known only at run time: kept serial
                if omp_here and self.omp:
                    priv = self.omp_private(u, idx)
                    clause = f" private({', '.join(priv)})" if priv else ""
                    out.append(f"{pad}{{ const int lo_{L} = {lo}, hi_{L} = {hi};")
                    sv = int(self.eval_const(u, parse_expr(parts[2]))) if len(parts) > 2 else 1
                    cmp = "<=" if sv > 0 else ">="
                    out.append(f"{pad}  _Pragma(\"omp parallel for schedule(static){clause}\")")
                    out.append(f"{pad}  for ({vc} = lo_{L}; {vc} {cmp} hi_{L}; {vc} += {sv}) {{")
                    stack.append("dofor")
                    ind += 1
                    continue
                # trip count fixed at entry, as Fortran defines it
                out.append(f"{pad}{{ const int lo_{L} = {lo}, hi_{L} = {hi}, st_{L} = {step};")
                out.append(f"{pad}  long tc_{L} = ((long)hi_{L} - lo_{L} + st_{L}) / st_{L};")
                out.append(f"{pad}  {vc} = lo_{L};")
                out.append(f"{pad}  for (; tc_{L} > 0; tc_{L}--, {vc} += st_{L}) {{")
                stack.append("dofor")
                ind += 1
                continue
            if st in ("enddo", "end do"):
                k = stack.pop()
                ind -= 1
                pad = "  " * ind
                if k == "dofor":
                    out.append(f"{pad}  }} }}")
                elif k == "do":
                    out.append(f"{pad}}}")
                else:
                    raise TranslateError(f"{u.src}:{ln}: ENDDO closes {k}")
                continue
            m = re.match(r"^(else\s*if)\s*\(", st)
            if m:
                rest = st[m.end() - 1:]
                j = matching_paren(rest, 0)
                c, _ = self.ex(parse_expr(rest[1:j]))
                if stack[-1] != "if":
                    raise TranslateError(f"{u.src}:{ln}: ELSE IF outside IF")
                out.append(f"{'  ' * (ind - 1)}}} else if ({c}) {{")
                continue
            if st == "else":
                out.append(f"{'  ' * (ind - 1)}}} else {{")
                continue
            if st in ("endif", "end if"):
                if stack.pop() != "if":
                    raise TranslateError(f"{u.src}:{ln}: ENDIF mismatch")
                ind -= 1
                out.append(f"{'  ' * ind}}}")
                continue
            m = re.match(r"^if\s*\(", st)
            if m:
                rest = st[m.end() - 1:]
                j = matching_paren(rest, 0)
                c, _ = self.ex(parse_expr(rest[1:j]))
                tail = rest[j + 1:].strip()
                if tail == "then":
                    out.append(f"{pad}if ({c}) {{")
                    stack.append("if")
                    ind += 1
                else:
                    out.append(f"{pad}if ({c}) {{")
                    self.simple(tail, out, ind + 1, u, ln)
                    out.append(f"{pad}}}")
                continue
            self.simple(st, out, ind, u, ln)
        if stack:
            raise TranslateError(f"{u.name}: unclosed blocks {stack}")
        return out

    def unformatted_io(self, st, out, pad):
        """OPEN(unit, ..., form='unformatted'), CLOSE(unit) and the
        unformatted sequential WRITE(unit) item, ... of the fluid (restart)
        files: unit u goes to <ref_unit_dir>/fort.<u>, each WRITE one record
        between 4-byte length markers, items in order, whole arrays in
        storage order.  Formatted output is dropped by the caller."""
        m = re.match(r"^(open|close|write)\s*\(", st)
        if not m:
            return False
        j = matching_paren(st, m.end() - 1)
        ctl = split_top(st[m.end():j])
        if m.group(1) == "open":
            if not any(re.match(r"^form\s*=\s*'unformatted'$", c) for c in ctl):
                return False
            unit = next(c for c in ctl if "=" not in c or c.startswith("unit"))
            unit = unit.split("=", 1)[1] if unit.startswith("unit") else unit
            out.append(f"{pad}ref_open_unit((int)({self.ex(parse_expr(unit))[0]}));")
            return True
        if m.group(1) == "close":
            out.append(f"{pad}ref_close_unit((int)({self.ex(parse_expr(ctl[0]))[0]}));")
            return True
        if len(ctl) != 1 or ctl[0] == "*" or ctl[0].startswith("'") or "=" in ctl[0]:
            return False                  # list-directed or formatted
        unit_c = self.ex(parse_expr(ctl[0]))[0]
        if ctl[0] in self.u.syms and self.u.type_of(ctl[0]) == "char":
            return False                  # an internal write
        ptrs, sizes = [], []
        for item in split_top(st[j + 1:].strip()):
            e = parse_expr(item)
            if e[0] != "name":
                raise TranslateError(f"{self.u.name}: unformatted item {item!r}")
            c, t = self.name_ref(e[1])
            sym = self.u.syms.get(e[1])
            ct = CTYPE[t[:-2]] if t.endswith("[]") else CTYPE[t]
            if t.endswith("[]"):
                cb = self.cn(e[1])
                ext = " * ".join(f"{cb}_ex{d}" for d in range(len(sym.dims)))
                ptrs.append(f"(const void*){c}")
                sizes.append(f"(size_t)({ext}) * sizeof({ct})")
            else:
                ptrs.append(f"(const void*)&{c}" if not c.startswith("(*") else f"(const void*){c[2:-1]}")
                sizes.append(f"sizeof({ct})")
        out.append(f"{pad}{{ const void* p_[] = {{{', '.join(ptrs)}}}; const size_t n_[] = {{{', '.join(sizes)}}}; "
                   f"ref_write_record((int)({unit_c}), {len(ptrs)}, p_, n_); }}")
        return True

    def simple(self, st, out, ind, u, ln):
        pad = "  " * ind
        if st == "return":
            out.append(f"{pad}goto L_return;")
            return
        if st == "exit":
            out.append(f"{pad}break;")
            return
        if st == "cycle":
            out.append(f"{pad}continue;")
            return
        if st == "continue":
            out.append(f"{pad};")
            return
        if st.startswith("stop") or st.startswith("call exit"):
            out.append(f'{pad}ref_stop("{u.name}");')
            return
        if self.unformatted_io(st, out, pad):
            return
        if re.match(r"^(write|print|open|close|read|inquire|rewind|backspace|flush)\b", st):
            out.append(f"{pad}/* formatted or inquiry statement dropped */")
            return
        m = re.match(r"^call\s+(\w+)\s*(\((.*)\))?\s*$", st)
        if m:
            self.call(m.group(1), m.group(3) or "", out, ind)
            return
        # assignment: the first top-level '=' that is not part of an operator
        depth, q, eq = 0, None, -1
        for i, ch in enumerate(st):
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
                prev = st[i - 1] if i else ""
                nxt = st[i + 1] if i + 1 < len(st) else ""
                if prev in "<>/=" or nxt in "=>":
                    continue
                eq = i
                break
        if eq < 0:
            raise TranslateError(f"{u.src}:{ln}: unsupported statement {st!r}")
        lhs_s, rhs_s = st[:eq].strip(), st[eq + 1:].strip()
        tc, tt = self.lhs(lhs_s)
        if isinstance(tc, tuple):
            self.section_assign(tc, rhs_s, out, ind)
            return
        rc, _ = self.ex(parse_expr(rhs_s))
        out.append(f"{pad}{tc} = ({CTYPE[tt]})({rc});")

    # ---- one subroutine ----
    def unit(self, u):
        self.u = u
        params = []
        for a in u.args:
            t = u.type_of(a)
            params.append(f"{CTYPE[t]}* {a}")
        head = f"void ref_{u.name}({', '.join(params) if params else 'void'})"
        decl, setup, free = [], [], []
        self.locals_used = set()
        body = self.body(u)
        for n in self.locals_used:
            u.sym(n)
        # locals: every symbol that is not a dummy, parameter or common member
        for name, s in sorted(u.syms.items()):
            if s.is_dummy or s.param is not None or s.common is not None:
                continue
            if name.startswith("s_"):
                continue
            t = u.type_of(name)
            ct = CTYPE[t]
            if s.dims is None:
                init = self.ex(pexpr(s.init))[0] if s.init is not None else "0"
                decl.append(f"  static {ct} {name} = {init};")
                continue
            try:
                n = 1
                for lo, hi in s.dims:
                    n *= self.const_int(u, hi) - self.const_int(u, lo) + 1
                decl.append(f"  static {ct} {name}[{n}];")
            except TranslateError:
                setup.append(("auto", name, ct))
        # every array: lower bounds and extents
        lines = []
        for name, s in sorted(u.syms.items()):
            if s.dims is None or s.param is not None:
                continue
            if s.common is not None:
                blk, off = s.common
                lines.append(f"  {CTYPE[u.type_of(name)]}* {name} = ({CTYPE[u.type_of(name)]}*)(ref_common_{blk} + {off});")
            for d, (lo, hi) in enumerate(s.dims):
                lc = self.ex(lo)[0]
                lines.append(f"  const long {name}_lo{d} = {lc};")
                if hi is None:
                    lines.append(f"  const long {name}_ex{d} = 1L << 40;")
                else:
                    hc = self.ex(hi)[0]
                    lines.append(f"  const long {name}_ex{d} = (long)({hc}) - {name}_lo{d} + 1;")
        # Automatic arrays (bounds from dummies) live on the stack in the
        # reference's build: no allocation and no zeroing per call.  Here each
        # gets a buffer per call site and recursion depth, kept between calls
        # (sparse_solver calls itself, and the caller's arrays must survive).
        # Only divB_correct's are zeroed on every call: its soln_vec is the
        # solver's starting iterate, uninitialised in the reference and zero
        # here, as everywhere in this build.
        if setup:
            lines.append(f"  static int ref_depth_{u.name} = 0;")
            lines.append(f"  const int d_ = ref_depth_{u.name}++;")
            lines.append(f"  if (d_ >= 16) ref_stop(\"{u.name}: recursion deeper than 16\");")
            free.append(f"  ref_depth_{u.name}--;")
        for _, name, ct in setup:
            s = u.syms[name]
            ext = " * ".join(f"{name}_ex{d}" for d in range(len(s.dims)))
            zero = 1 if u.name in ZERO_AUTOMATIC else 0
            lines.append(f"  static void* {name}_buf[16]; static size_t {name}_cap[16];")
            lines.append(f"  {ct}* {name} = ({ct}*)ref_auto(&{name}_buf[d_], &{name}_cap[d_], "
                         f"(size_t)({ext}) * sizeof({ct}), {zero});")
        # section-assignment loop counters are declared in their loops
        out = [f"/* ---- {u.src}: subroutine {u.name} ---- */", head + " {"]
        out += decl + lines + body
        out.append("  goto L_return;")
        out.append("L_return:;")
        out += free
        out.append("}")
        return out

    def module(self, order):
        out = [
            "/* Generated from the reference's Fortran sources by oracle/fortran_to_c.py.",
            "   Not part of the repository: it is rebuilt wherever the sources exist. */",
            "#include <math.h>",
            "#include <stdio.h>",
            "#include <stdlib.h>",
            "#include <string.h>",
            "static inline int ref_max_int(int a, int b) { return a > b ? a : b; }",
            "static inline int ref_min_int(int a, int b) { return a < b ? a : b; }",
            "static inline float ref_max_float(float a, float b) { return a > b ? a : b; }",
            "static inline float ref_min_float(float a, float b) { return a < b ? a : b; }",
            "static inline double ref_max_double(double a, double b) { return a > b ? a : b; }",
            "static inline double ref_min_double(double a, double b) { return a < b ? a : b; }",
            "static inline int ref_sign_int(int a, int b) { int m = abs(a); return b >= 0 ? m : -m; }",
            "static inline float ref_sign_float(float a, float b) { float m = fabsf(a); return b >= 0.0f ? m : -m; }",
            "static inline double ref_sign_double(double a, double b) { double m = fabs(a); return b >= 0.0 ? m : -m; }",
            "static inline float ref_powif(float x, int n) { float r = 1.0f; int k = n < 0 ? -n : n;"
            " for (int i = 0; i < k; i++) r = r * x; return n < 0 ? 1.0f / r : r; }",
            "static inline double ref_powid(double x, int n) { double r = 1.0; int k = n < 0 ? -n : n;"
            " for (int i = 0; i < k; i++) r = r * x; return n < 0 ? 1.0 / r : r; }",
            "static inline int ref_powii(int x, int n) { int r = 1; for (int i = 0; i < n; i++) r *= x; return r; }",
            "#include <setjmp.h>",
            "int ref_main_stopped = 0;",
            "int ref_untranslated_calls = 0;",
            "char ref_untranslated_last[64];",
            "static jmp_buf ref_jmp;",
            "static int ref_jmp_armed = 0;",
            "static void ref_stop(const char* who) {",
            "  fprintf(stderr, \"STOP in %s\\n\", who);",
            "  ref_main_stopped = 1;",
            "  if (ref_jmp_armed) longjmp(ref_jmp, 1);",
            "  exit(3);",
            "}",
            "char ref_unit_dir[512] = \".\";",
            "static FILE* ref_units[100];",
            "static void ref_open_unit(int u) {",
            "  if (u < 0 || u >= 100) return;",
            "  if (ref_units[u]) fclose(ref_units[u]);",
            "  char path[640];",
            "  snprintf(path, sizeof path, \"%s/fort.%d\", ref_unit_dir, u);",
            "  ref_units[u] = fopen(path, \"wb\");",
            "}",
            "static void ref_close_unit(int u) {",
            "  if (u >= 0 && u < 100 && ref_units[u]) { fclose(ref_units[u]); ref_units[u] = 0; }",
            "}",
            "static void ref_write_record(int u, int k, const void** p, const size_t* n) {",
            "  if (u < 0 || u >= 100 || !ref_units[u]) return;",
            "  size_t len = 0;",
            "  for (int i = 0; i < k; i++) len += n[i];",
            "  const int marker = (int)len;   /* 4-byte record length before and after */",
            "  fwrite(&marker, 4, 1, ref_units[u]);",
            "  for (int i = 0; i < k; i++) fwrite(p[i], 1, n[i], ref_units[u]);",
            "  fwrite(&marker, 4, 1, ref_units[u]);",
            "}",
            "static void* ref_auto(void** buf, size_t* cap, size_t bytes, int zero) {",
            "  if (bytes == 0) bytes = 1;",
            "  if (*cap < bytes) { free(*buf); *buf = malloc(bytes); *cap = bytes; if (!*buf) ref_stop(\"out of memory\"); }",
            "  if (zero) memset(*buf, 0, bytes);",
            "  return *buf;",
            "}",
            "static void ref_untranslated(const char* who) {",
            "  ref_untranslated_calls++;",
            "  strncpy(ref_untranslated_last, who, sizeof ref_untranslated_last - 1);",
            "}",
        ]
        for blk, (size, _) in sorted(self.commons.items()):
            out.append(f"unsigned char ref_common_{blk}[{max(size, 8)}] __attribute__((aligned(16)));")
        # prototypes (calls may go forwards)
        for name in order:
            u = self.units[name]
            params = [f"{CTYPE[u.type_of(a)]}* {a}" for a in u.args]
            out.append(f"void ref_{name}({', '.join(params) if params else 'void'});")
        for name in order:
            out += self.unit(self.units[name])
        return out

    def main_unit(self, u):
        """One C function running the time loop's body *nsteps times, the
        main program's variables as exported globals ref_main_<name>."""
        self.u = u
        self.main = True
        self.locals_used = set()
        body = self.body(u)
        loop_body = u.body
        u.body = u.init_body
        init_body = self.body(u)
        u.body = u.fresh_body
        fresh_body = self.body(u)
        u.body = loop_body
        for n in self.locals_used:
            u.sym(n)
        glob, prolog, meta, allocs = [], [], {}, []
        for name, sym in sorted(u.syms.items()):
            if (sym.param is not None and sym.dims is None) or name.startswith("s_"):
                continue
            self.where = (u.src, "declaration of", name)
            t = u.type_of(name)
            ct = CTYPE[t]
            if t == "char":        # names and formats of files: not on the path
                continue
            if sym.param is not None:
                # a PARAMETER array from an array constructor [a, b, ...]
                src = sym.param[1].strip()
                if src.startswith("(/"):
                    src = "[" + src[2:-2] + "]"
                if not (src.startswith("[") and src.endswith("]")):
                    raise TranslateError(f"parameter array {name}: {src!r}")
                vals = [self.ex(parse_expr(v))[0] for v in split_top(src[1:-1])]
                g = "ref_main_" + name
                glob.append(f"{ct} {g}[{len(vals)}] = {{{', '.join(vals)}}};")
                glob.append(f"const long {g}_lo0 = 1;")
                glob.append(f"const long {g}_ex0 = {len(vals)};")
                continue
            if sym.common is not None:
                if sym.dims is not None:
                    blk, off = sym.common
                    prolog.append(f"  {ct}* {name} = ({ct}*)(ref_common_{blk} + {off});")
                    for d, (lo, hi) in enumerate(sym.dims):
                        prolog.append(f"  const long {name}_lo{d} = {self.ex(lo)[0]};")
                        prolog.append(f"  const long {name}_ex{d} = (long)({self.ex(hi)[0]}) - {name}_lo{d} + 1;")
                continue
            g = "ref_main_" + name
            if sym.dims is None:
                init = self.ex(pexpr(sym.init))[0] if sym.init is not None else "0"
                glob.append(f"{ct} {g} = {init};")
                meta[name] = {"type": t, "dims": None}
            elif any(d is DEFERRED or d == DEFERRED for d in sym.dims):
                glob.append(f"{ct}* {g} = 0;")
                for d in range(len(sym.dims)):
                    glob.append(f"long {g}_lo{d} = 1;")
                    glob.append(f"long {g}_ex{d} = 0;")
                meta[name] = {"type": t, "dims": "allocatable", "rank": len(sym.dims)}
            else:
                ext = []
                for d, (lo, hi) in enumerate(sym.dims):
                    l0 = self.const_int(u, lo)
                    e = self.const_int(u, hi) - l0 + 1
                    ext.append(e)
                    glob.append(f"const long {g}_lo{d} = {l0};")
                    glob.append(f"const long {g}_ex{d} = {e};")
                n = 1
                for e in ext:
                    n *= e
                # on the heap (the production grid's arrays exceed what a
                # shared library's static data may hold), with a guard of
                # zeros on both sides: the loop reads t_old(0) and t_new(0)
                # (box - 1 with box = 1)
                glob.append(f"{ct}* {g} = 0;")
                allocs.append(f"  {g} = ({ct}*)calloc({n + 16}, sizeof({ct})) + 8;")
                meta[name] = {"type": t, "dims": ext}
        out = [f"/* ---- {u.src}: the body of the time loop, lines {u.loop_lines[0]}-{u.loop_lines[1]} ---- */"]
        out += glob
        out.append("__attribute__((constructor)) static void ref_main_alloc(void) {")
        out += allocs
        out.append("}")
        out.append(f"/* the time-step set-up before the loop, lines {u.init_lines[0]}-{u.init_lines[1]} */")
        out.append("void ref_main_init_steps(void) {")
        out += prolog
        out.append("  if (setjmp(ref_jmp)) { ref_jmp_armed = 0; return; }")
        out.append("  ref_jmp_armed = 1;")
        out += init_body
        out.append("  goto L_return;")
        out.append("L_return:;")
        out.append("  ref_jmp_armed = 0;")
        out.append("}")
        out.append(f"/* the fresh start (initial state), lines {u.fresh_lines[0]}-{u.fresh_lines[1]} */")
        out.append("void ref_main_fresh_start(void) {")
        out += prolog
        out.append("  if (setjmp(ref_jmp)) { ref_jmp_armed = 0; return; }")
        out.append("  ref_jmp_armed = 1;")
        out += fresh_body
        out.append("  goto L_return;")
        out.append("L_return:;")
        out.append("  ref_jmp_armed = 0;")
        out.append("}")
        out.append("void ref_main_steps(int* nsteps) {")
        out += prolog
        out.append("  if (setjmp(ref_jmp)) { ref_jmp_armed = 0; return; }")
        out.append("  ref_jmp_armed = 1;")
        out.append("  for (int it_ = 0; it_ < *nsteps; it_++) {")
        out += body
        out.append("  }")
        out.append("  goto L_return;")
        out.append("L_return:;")
        out.append("  ref_jmp_armed = 0;")
        out.append("}")
        self.main = False
        return out, meta

    def meta(self, order):
        subs = {}
        for name in order:
            u = self.units[name]
            args = []
            for a in u.args:
                s = u.syms[a]
                t = self.retyped.get(name, {}).get(a, u.type_of(a))
                args.append({"name": a, "type": t,
                             "rank": len(s.dims) if s.dims else 0})
            subs[name] = {"file": u.src, "args": args}
        commons = {blk: {"size": size, "members": [
            {"name": n, "type": t, "offset": off, "count": c} for n, t, off, c in mem]}
            for blk, (size, mem) in self.commons.items()}
        return {"subroutines": subs, "commons": commons}


_DO_START = re.compile(r"^do(\s+while\b|\s+\w+\s*=)")
_DO_END = re.compile(r"^end\s*do$")


def parse_module_params(path, into):
    """The declarations of a module up to CONTAINS, merged into unit `into`
    where it declares nothing of the same name (USE association)."""
    text = open(path, encoding="latin-1").read()
    m = Unit("module", [], os.path.basename(path))
    for ln, st in statements(text):
        if st.startswith("module ") or st == "implicit none":
            continue
        if st == "contains" or st.startswith("end module"):
            break
        if not declaration(m, st, ln):
            raise TranslateError(f"{path}:{ln}: unexpected statement in module: {st!r}")
    for n, sym in m.syms.items():
        if n not in into.syms or into.syms[n].type is None:
            into.syms[n] = sym


def parse_main_loop(path, module_dir, overrides):
    """The main program's declarations and the body of its time loop
    ``do while(t.lt.tmax)`` (code/3d_main.f90), as a unit whose variables
    become C globals.  `overrides` replaces PARAMETER values (grid size)."""
    text = open(path, encoding="latin-1").read()
    sts = list(statements(text))
    st0 = sts[0][1]
    m = re.match(r"^program\s+(\w+)$", st0)
    if not m:
        raise TranslateError(f"{path}: does not start with PROGRAM")
    u = Unit("main_steps", [], os.path.basename(path))
    u.kind = "program"
    i = 1
    while i < len(sts) and declaration(u, sts[i][1], sts[i][0]):
        i += 1
    body = sts[i:]
    start = next(j for j, (_, st) in enumerate(body)
                 if re.match(r"^do\s+while\s*\(\s*t\s*\.lt\.\s*tmax\s*\)$", st))
    depth = 0
    for k in range(start, len(body)):
        st = body[k][1]
        if _DO_START.match(st):
            depth += 1
        elif _DO_END.match(st):
            depth -= 1
            if depth == 0:
                break
    else:
        raise TranslateError("the time loop has no ENDDO")
    u.body = body[start + 1:k]
    u.loop_lines = (body[start][0], body[k][0])
    # the time-step set-up just before the loop: the last top-level
    # "do box=n_grids,1,-1" that checks densities and speeds of every box
    depth, init = 0, None
    for j in range(start):
        st = body[j][1]
        if depth == 0 and re.match(r"^do\s+box\s*=\s*n_grids\s*,\s*1\s*,\s*-1$", st):
            d2 = 0
            for e in range(j, start):
                if _DO_START.match(body[e][1]):
                    d2 += 1
                elif _DO_END.match(body[e][1]):
                    d2 -= 1
                    if d2 == 0:
                        break
            if any(x[1].startswith("call set_speed_agrd") for x in body[j:e]):
                init = (j, e)
        if _DO_START.match(st):
            depth += 1
        elif _DO_END.match(st):
            depth -= 1
    if init is None:
        raise TranslateError("no time-step set-up loop before the time loop")
    u.init_body = body[init[0]:init[1] + 1]
    u.init_lines = (body[init[0]][0], body[init[1]][0])
    # the fresh start: the ELSE branch of the top-level "if(.not.start)"
    # before the loop (the initial state, dipole, inner-boundary lists,
    # resistivity)
    u.fresh_body, u.fresh_lines = [], (0, 0)
    for j in range(start):
        if re.match(r"^if\s*\(\s*\.not\.\s*start\s*\)\s*then$", body[j][1]):
            d, e_else = 0, None
            for e in range(j, start):
                st = body[e][1]
                if re.match(r"^if\s*\(.*\)\s*then$", st):
                    d += 1
                elif re.match(r"^end\s*if$", st):
                    d -= 1
                    if d == 0:
                        break
                elif d == 1 and st == "else":
                    e_else = e
            if e_else is not None:
                u.fresh_body = body[e_else + 1:e]
                u.fresh_lines = (body[e_else + 1][0], body[e - 1][0])
            break
    for mod in u.uses:
        parse_module_params(os.path.join(module_dir, f"mod_{mod}.f90"), u)
    for n, v in overrides.items():
        u.sym(n).param = ("lazy", str(v))
    return u


def translate(code_dir, out_dir=OUT):
    units = []
    for f in FILES:
        path = os.path.join(code_dir, f + ".f90")
        units += parse_units(path)
    g = Gen(units)
    order = [u.name for u in units]
    g.where = None
    try:
        src = g.module(order)
    except (TranslateError, KeyError, ValueError, IndexError) as e:
        raise TranslateError(f"at {g.where}: {type(e).__name__}: {e}") from e
    os.makedirs(out_dir, exist_ok=True)
    cpath = os.path.join(out_dir, "g3m3_ref.c")
    with open(cpath, "w") as fh:
        fh.write("\n".join(src) + "\n")
    with open(os.path.join(out_dir, "g3m3_ref.json"), "w") as fh:
        json.dump(g.meta(order), fh, indent=1)
    return cpath


# Grid sizes of the main-loop builds: the main program's PARAMETERs
# limit (nx = ny = 2*limit+1, nz = limit+1), n_grids and mbndry.
MAIN_CONFIGS = {
    "tiny": {"limit": "8.", "n_grids": "1", "mbndry": "1"},
    "tiny3": {"limit": "8.", "n_grids": "3", "mbndry": "1"},
    "small": {"limit": "30.", "n_grids": "1", "mbndry": "1"},   # one box 61x61x31
    "nested": {},            # the reference's own: limit 60 (121x121x61), 5 boxes
}
# (grid, OpenMP): the serial builds are the parity reference; the OpenMP
# builds time the reference on all host cores and make the production-size
# digests (tiny3 is checked against its serial build bit for bit)
MAIN_BUILDS = [("tiny", False), ("tiny3", False), ("small", False), ("tiny3", True), ("nested", True)]
# the reference in FP64 (default REAL as double), to state the FP32 error:
# (grid, OpenMP)
R8_BUILDS = [("tiny3", False), ("small", False), ("nested", True)]


def main_stem(tag, omp, real8=False):
    return f"g3m3_ref_main_{tag}" + ("_r8" if real8 else "") + ("_omp" if omp else "")


def translate_main(code_dir, tag, overrides, out_dir=OUT, omp=False, real8=False):
    """All routines plus the main program's time loop for one grid size:
    <stem>.c and its variable list <stem>.json (stem from main_stem)."""
    REAL["t"] = "double" if real8 else "float"
    try:
        return _translate_main(code_dir, tag, overrides, out_dir, omp, real8)
    finally:
        REAL["t"] = "float"


def _translate_main(code_dir, tag, overrides, out_dir, omp, real8):
    units = []
    for f in FILES:
        units += parse_units(os.path.join(code_dir, f + ".f90"))
    prog = parse_main_loop(os.path.join(code_dir, "3d_main.f90"), code_dir, overrides)
    g = Gen(units)
    g.omp = omp
    g.layout_commons(prog)
    order = [u.name for u in units]
    g.where = None
    try:
        src = g.module(order)
        main_src, main_meta = g.main_unit(prog)
    except (TranslateError, KeyError, ValueError, IndexError, StopIteration) as e:
        raise TranslateError(f"at {g.where}: {type(e).__name__}: {e}") from e
    os.makedirs(out_dir, exist_ok=True)
    stem = main_stem(tag, omp, real8)
    cpath = os.path.join(out_dir, stem + ".c")
    with open(cpath, "w") as fh:
        fh.write("\n".join(src + main_src) + "\n")
    meta = g.meta(order)
    meta["main"] = {"variables": main_meta, "overrides": overrides, "openmp": omp,
                    "loop_lines": list(prog.loop_lines), "init_lines": list(prog.init_lines),
                    "fresh_lines": list(prog.fresh_lines)}
    with open(os.path.join(out_dir, stem + ".json"), "w") as fh:
        json.dump(meta, fh, indent=1)
    return cpath


def compile_ref(out_dir=OUT, cc="gcc", stem="g3m3_ref"):
    cpath = os.path.join(out_dir, stem + ".c")
    so = os.path.join(out_dir, "lib" + stem + ".so")
    omp = ["-fopenmp"] if stem.endswith("_omp") else []
    # the OpenMP builds time the reference's CPU path: -O3 (vectorised loops;
    # the same bits, contraction and fast-math staying off)
    opt = "-O3" if omp else "-O2"
    # warnings are not shown, but the ones that reveal a mistranslated
    # argument (a pointer where a value belongs, or the reverse) are errors
    r = subprocess.run([cc] + omp + [opt, "-fPIC", "-shared", "-std=gnu11", "-ffp-contract=off",
                        "-fno-fast-math", "-fwrapv", "-Werror=int-conversion",
                        "-Werror=incompatible-pointer-types", "-Werror=implicit-function-declaration",
                        "-Werror=pointer-to-int-cast", "-Werror=int-to-pointer-cast",
                        "-Wl,-Bsymbolic", "-o", so, cpath, "-lm"], capture_output=True, text=True)
    if r.returncode:
        errs = [ln for ln in r.stderr.splitlines() if "error" in ln]
        raise TranslateError(f"{cpath} does not compile:\n" + "\n".join(errs[:20]))
    return so


def reference_code_dir():
    ref = os.environ.get("G3M3_REFERENCE")
    return os.path.join(ref, "code") if ref else None


def main(argv):
    code_dir = argv[1] if len(argv) > 1 else reference_code_dir()
    stems = (["g3m3_ref"] + [main_stem(t, o) for t, o in MAIN_BUILDS]
             + [main_stem(t, o, True) for t, o in R8_BUILDS])
    if code_dir and os.path.isdir(code_dir):
        translate(code_dir)
        for tag, omp in MAIN_BUILDS:
            translate_main(code_dir, tag, MAIN_CONFIGS[tag], omp=omp)
        for tag, omp in R8_BUILDS:
            translate_main(code_dir, tag, MAIN_CONFIGS[tag], omp=omp, real8=True)
    from concurrent.futures import ThreadPoolExecutor
    todo = [st for st in stems if os.path.exists(os.path.join(OUT, st + ".c"))]
    # sources translated elsewhere may have travelled here without the reference
    with ThreadPoolExecutor(len(todo) or 1) as ex:
        list(ex.map(lambda st: compile_ref(stem=st), todo))
    return 0


if __name__ == "__main__":
    sys.exit(main(sys.argv))
