"""Reverse-mode source transformation for the per-cell arithmetic of the
step's kernels (build-time tool; writes csrc/adj_cells.cuh).

Each cell function in ``adcells.py`` states, in a small Python subset, the
arithmetic one thread does for one cell: named scalar inputs (the stencil
values it loads), non-differentiated parameters, straight-line assignments
and a tuple of outputs.  This module turns each into a C++ struct with

* ``fwd(in_, par_, out_)``: the same arithmetic (used by the tests to check the
  statement against the library's forward kernels and the oracle), and
* ``adj(in_, par_, out_b_, acc_)``: the forward sweep again (primal values),
  then the reverse sweep, which calls ``acc_(slot, value)`` once for every
  contribution ``value`` to the adjoint of input ``slot``.  The kernel that
  calls it decides where a contribution goes (a register, a shared-memory
  adjoint tile, a global adjoint array).

The subset: ``x = expr`` with + - * /, unary -, numeric literals, the
functions sqrt, fabs, amax1, amin1 (the forward kernels' ``a > b ? a : b``
and ``a < b ? a : b``), and conditional expressions ``a if cond else b``
with one comparison as cond.  Names are single assignment.  Derivatives
follow the forward semantics: amax1 passes the adjoint to the operand it
returned, fabs multiplies by the sign (0 at 0), sqrt by 1/(2 sqrt) (0 at
0), a conditional to the branch it took.

    python -m g3m3_gb300.adgen          # regenerate csrc/adj_cells.cuh
"""
from __future__ import annotations

import ast
import inspect
import os
import textwrap

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "csrc", "adj_cells.cuh")

_CMP = {ast.Gt: ">", ast.Lt: "<", ast.GtE: ">=", ast.LtE: "<=", ast.Eq: "==", ast.NotEq: "!="}
_BIN = {ast.Add: "+", ast.Sub: "-", ast.Mult: "*", ast.Div: "/"}


class Cell:
    """Declared signature of a cell function."""

    def __init__(self, fn, inputs, params, outputs):
        self.fn = fn
        self.name = fn.__name__
        self.inputs = list(inputs)
        self.params = list(params)
        self.outputs = list(outputs)


def cell(inputs, params, outputs):
    def deco(fn):
        fn.__cell__ = Cell(fn, inputs, params, outputs)
        return fn
    return deco


def _lit(v):
    s = repr(float(v))
    if "e" not in s and "." not in s:
        s += ".0"
    return f"T({s})"


class _Flatten:
    """Three-address form: [(target, op, args)] with op one of
    'copy', '+', '-', '*', '/', 'neg', 'sqrt', 'fabs', 'amax1', 'amin1',
    'select' (args: cmp, l, r, a, b)."""

    def __init__(self, inputs, params):
        self.code = []
        self.n = 0
        self.known = set(inputs) | set(params)
        self.params = set(params)

    def tmp(self):
        self.n += 1
        return f"_t{self.n}"

    def atom(self, node):
        if isinstance(node, ast.Name):
            if node.id not in self.known:
                raise NameError(f"{node.id} used before assignment")
            return node.id
        if isinstance(node, ast.Constant):
            return _lit(node.value)
        if isinstance(node, ast.UnaryOp) and isinstance(node.op, ast.USub) and isinstance(node.operand, ast.Constant):
            return _lit(-node.operand.value)
        return self.expr(node)

    def expr(self, node, target=None):
        t = target or self.tmp()
        if isinstance(node, (ast.Name, ast.Constant)):
            self.code.append((t, "copy", [self.atom(node)]))
        elif isinstance(node, ast.BinOp):
            a, b = self.atom(node.left), self.atom(node.right)
            self.code.append((t, _BIN[type(node.op)], [a, b]))
        elif isinstance(node, ast.UnaryOp) and isinstance(node.op, ast.USub):
            self.code.append((t, "neg", [self.atom(node.operand)]))
        elif isinstance(node, ast.Call):
            fn = node.func.id
            args = [self.atom(x) for x in node.args]
            if fn not in ("sqrt", "fabs", "amax1", "amin1"):
                raise ValueError(f"unsupported call {fn}")
            self.code.append((t, fn, args))
        elif isinstance(node, ast.IfExp):
            c = node.test
            if not (isinstance(c, ast.Compare) and len(c.ops) == 1):
                raise ValueError("condition must be one comparison")
            l, r = self.atom(c.left), self.atom(c.comparators[0])
            a, b = self.atom(node.body), self.atom(node.orelse)
            self.code.append((t, "select", [_CMP[type(c.ops[0])], l, r, a, b]))
        else:
            raise ValueError(f"unsupported expression {ast.dump(node)}")
        self.known.add(t)
        return t

    def stmt(self, node):
        if not (isinstance(node, ast.Assign) and len(node.targets) == 1 and isinstance(node.targets[0], ast.Name)):
            raise ValueError(f"unsupported statement {ast.dump(node)}")
        name = node.targets[0].id
        if name in self.known:
            raise ValueError(f"{name} assigned twice")
        self.expr(node.value, target=name)


def flatten(c: Cell):
    src = textwrap.dedent(inspect.getsource(c.fn))
    fdef = ast.parse(src).body[0]
    fl = _Flatten(c.inputs, c.params)
    ret = None
    for node in fdef.body:
        if isinstance(node, ast.Expr) and isinstance(node.value, ast.Constant):
            continue   # docstring
        if isinstance(node, ast.Return):
            ret = node.value
            break
        fl.stmt(node)
    names = [e.id for e in (ret.elts if isinstance(ret, ast.Tuple) else [ret])]
    if names != c.outputs:
        raise ValueError(f"{c.name}: returns {names}, declared {c.outputs}")
    return fl.code


def _rhs(op, a):
    if op == "copy":
        return a[0]
    if op in ("+", "-", "*", "/"):
        return f"{a[0]} {op} {a[1]}"
    if op == "neg":
        return f"-{a[0]}"
    if op == "sqrt":
        return f"sqrt({a[0]})"
    if op == "fabs":
        return f"fabs({a[0]})"
    if op == "amax1":
        return f"({a[0]} > {a[1]} ? {a[0]} : {a[1]})"
    if op == "amin1":
        return f"({a[0]} < {a[1]} ? {a[0]} : {a[1]})"
    if op == "select":
        return f"({a[1]} {a[0]} {a[2]} ? {a[3]} : {a[4]})"
    raise ValueError(op)


def emit(c: Cell):
    code = flatten(c)
    inp = {n: i for i, n in enumerate(c.inputs)}
    par = {n: i for i, n in enumerate(c.params)}
    L = []
    w = L.append
    doc = (c.fn.__doc__ or "").strip().splitlines()
    w(f"// {c.name}: " + (doc[0] if doc else ""))
    for d in doc[1:]:
        w("//   " + d.strip() if d.strip() else "//")
    w(f"template <class T>")
    w(f"struct {c.name} {{")
    w(f"  static constexpr int NIN = {len(c.inputs)}, NPAR = {len(c.params)}, NOUT = {len(c.outputs)};")
    for n, i in inp.items():
        w(f"  static constexpr int I_{n} = {i};")
    for n, i in par.items():
        w(f"  static constexpr int P_{n} = {i};")
    for i, n in enumerate(c.outputs):
        w(f"  static constexpr int O_{n} = {i};")

    def prologue():
        for n, i in inp.items():
            w(f"    const T {n} = in_[{i}];")
        for n, i in par.items():
            w(f"    const T {n} = par_[{i}];")
        for t, op, a in code:
            w(f"    const T {t} = {_rhs(op, a)};")

    w("  __host__ __device__ __forceinline__ static void fwd(const T* in_, const T* par_, T* out_) {")
    w("    using std::sqrt; using std::fabs;")
    prologue()
    for i, n in enumerate(c.outputs):
        w(f"    out_[{i}] = {n};")
    w("  }")

    # reverse sweep
    w("  template <class Acc>")
    w("  __host__ __device__ __forceinline__ static void adj(const T* in_, const T* par_, const T* out_b_, Acc&& acc_) {")
    w("    using std::sqrt; using std::fabs;")
    prologue()
    assigned = {t for t, _, _ in code}
    bar = {}

    def b(name):   # adjoint variable of a temp/output
        if name not in bar:
            bar[name] = f"{name}_b"
            w(f"    T {name}_b = T(0);")
        return bar[name]

    for i, n in enumerate(c.outputs):
        w(f"    T {n}_b = out_b_[{i}];")
        bar[n] = f"{n}_b"

    # An input's contributions are summed in a local and handed to acc_ once,
    # right after the last of them: one accumulation (an atomic, in the
    # scattering kernels) per input instead of one per use.
    body_start = len(L)

    def add(name, expr):
        if name.startswith("T(") or name in par:
            return
        if name in inp:
            L.append(("IN", name, expr))
        elif name in assigned:
            w(f"    {b(name)} += {expr};")
        else:
            raise NameError(name)

    for t, op, a in reversed(code):
        if t not in bar:
            continue   # never used towards an output
        tb = bar[t]
        if op == "copy":
            add(a[0], tb)
        elif op == "+":
            add(a[0], tb)
            add(a[1], tb)
        elif op == "-":
            add(a[0], tb)
            add(a[1], f"-{tb}")
        elif op == "*":
            add(a[0], f"{tb} * {a[1]}")
            add(a[1], f"{tb} * {a[0]}")
        elif op == "/":
            add(a[0], f"{tb} / {a[1]}")
            add(a[1], f"-{tb} * {t} / {a[1]}")
        elif op == "neg":
            add(a[0], f"-{tb}")
        elif op == "sqrt":
            add(a[0], f"({t} > T(0) ? {tb} / (T(2) * {t}) : T(0))")
        elif op == "fabs":
            add(a[0], f"({a[0]} > T(0) ? {tb} : ({a[0]} < T(0) ? -{tb} : T(0)))")
        elif op == "amax1":
            add(a[0], f"({a[0]} > {a[1]} ? {tb} : T(0))")
            add(a[1], f"({a[0]} > {a[1]} ? T(0) : {tb})")
        elif op == "amin1":
            add(a[0], f"({a[0]} < {a[1]} ? {tb} : T(0))")
            add(a[1], f"({a[0]} < {a[1]} ? T(0) : {tb})")
        elif op == "select":
            cond = f"{a[1]} {a[0]} {a[2]}"
            add(a[3], f"({cond} ? {tb} : T(0))")
            add(a[4], f"({cond} ? T(0) : {tb})")
        else:
            raise ValueError(op)
    body = L[body_start:]
    del L[body_start:]
    last, count = {}, {}
    for k, item in enumerate(body):
        if isinstance(item, tuple):
            last[item[1]] = k
            count[item[1]] = count.get(item[1], 0) + 1
    seen = set()
    for k, item in enumerate(body):
        if not isinstance(item, tuple):
            w(item)
            continue
        _, name, expr = item
        if count[name] == 1:
            w(f"    acc_({inp[name]}, {expr});")
            continue
        if name in seen:
            w(f"    {name}_ib += {expr};")
        else:
            seen.add(name)
            w(f"    T {name}_ib = {expr};")
        if last[name] == k:
            w(f"    acc_({inp[name]}, {name}_ib);")
    w("  }")
    w("};")
    return "\n".join(L)


def generate(path=OUT):
    from . import adcells
    cells = [v.__cell__ for v in vars(adcells).values() if hasattr(v, "__cell__")]
    cells.sort(key=lambda c: c.fn.__code__.co_firstlineno)
    head = [
        "// adj_cells.cuh -- GENERATED by g3m3_gb300/adgen.py from g3m3_gb300/adcells.py; do not edit.",
        "//",
        "// Per-cell forward arithmetic and its reverse sweep for the adjoint",
        "// kernels (k_adj_*.cu).  T is float on the GPU and double in the tests.",
        "#pragma once",
        "",
        "#include <cmath>",
        "",
        "namespace g3m3 {",
        "namespace adj {",
        "",
    ]
    body = [emit(c) + "\n" for c in cells]
    text = "\n".join(head + body + ["}  // namespace adj", "}  // namespace g3m3", ""])
    old = open(path).read() if os.path.exists(path) else None
    if text != old:
        with open(path, "w") as fh:
            fh.write(text)
    return path


if __name__ == "__main__":
    print(generate())
