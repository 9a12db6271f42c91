"""Loader for libg3m3_gpu.so with ctypes signatures read from include/g3m3.h.

The product path has no CPU fallback: if the library is missing or cannot be
loaded this module raises.  Argument types are derived from the public
header, so the binding and the C ABI cannot drift apart.
"""
from __future__ import annotations

import ctypes
import os
import re

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
HEADER = os.path.join(ROOT, "include", "g3m3.h")
LIB_PATH = os.path.join(HERE, "lib", "libg3m3_gpu.so")

_C2CT = {
    "int": ctypes.c_int,
    "float": ctypes.c_float,
    "double": ctypes.c_double,
    "void": None,
    "size_t": ctypes.c_size_t,
}


def header_functions(path: str = HEADER, prefix: str = "g3m3_"):
    """[(name, restype_str, [param type strings])] for every prefix* prototype."""
    text = open(path).read()
    text = re.sub(r"/\*.*?\*/", " ", text, flags=re.S)
    out = []
    for m in re.finditer(r"\b(int|size_t|void\s*\*|const\s+char\s*\*|void)\s+(" + prefix + r"\w+)\s*\(([^;{]*?)\)\s*;", text, re.S):
        ret, name, params = m.group(1), m.group(2), m.group(3)
        plist = [] if params.strip() in ("", "void") else [p.strip() for p in params.split(",")]
        out.append((name, " ".join(ret.split()), plist))
    return out


def ctype_of(param: str):
    p = " ".join(param.replace("const", " ").split())
    if "*" in p or "[" in p:
        return ctypes.c_void_p
    if p.startswith("unsigned long long"):
        return ctypes.c_ulonglong
    base = p.split()[0]
    if base in ("int32_t",):
        return ctypes.c_int32
    return _C2CT[base]


def restype_of(ret: str):
    if ret == "int":
        return ctypes.c_int
    if ret == "size_t":
        return ctypes.c_size_t
    if ret == "void":
        return None
    if "char" in ret:
        return ctypes.c_char_p
    return ctypes.c_void_p


_LIB = None


def load(build_if_missing: bool = False):
    global _LIB
    if _LIB is not None:
        return _LIB
    if not os.path.exists(LIB_PATH):
        if build_if_missing:
            from . import build
            build.build()
        else:
            raise RuntimeError(f"{LIB_PATH} is missing: run g3m3_gb300.build.build() (nvcc, sm_103a)")
    lib = ctypes.CDLL(LIB_PATH)
    for name, ret, params in header_functions():
        fn = getattr(lib, name)   # AttributeError: header declares a symbol the library lacks
        fn.restype = restype_of(ret)
        fn.argtypes = [ctype_of(p) for p in params]
    _LIB = lib
    return lib
