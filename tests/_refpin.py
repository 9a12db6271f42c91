"""ctypes access to oracle/_ref/libg3m3_ref.so: the reference's own Fortran
routines, translated to C and compiled by oracle/fortran_to_c.py.

TEST INFRASTRUCTURE ONLY.  The library is built where the reference's
sources exist (``__graft_entry__.build()`` or the first use here); where they
do not, the tests that need it skip.  Every routine takes its Fortran dummy
arguments in order, each by reference: numpy arrays pass their data pointer,
ctypes objects their address, and Python numbers are converted to the
dummy's declared type (INTEGER/LOGICAL int32, REAL float32, REAL(dp)
float64).
"""
from __future__ import annotations

import ctypes
import json
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF = os.path.join(ROOT, "oracle", "_ref")
_CT = {"int": ctypes.c_int32, "logical": ctypes.c_int32, "float": ctypes.c_float,
       "double": ctypes.c_double}
_NP = {"int": np.int32, "logical": np.int32, "float": np.float32, "double": np.float64}

_LIB = None


def load():
    """(CDLL, metadata) or None when neither the library nor the sources exist."""
    global _LIB
    if _LIB is not None:
        return _LIB
    so = os.path.join(REF, "libg3m3_ref.so")
    if not os.path.exists(so):
        if ROOT not in sys.path:
            sys.path.insert(0, ROOT)
        from oracle import fortran_to_c
        import __graft_entry__
        try:
            fortran_to_c.main(["fortran_to_c", os.path.join(__graft_entry__.REFERENCE, "code")])
        except Exception:
            return None
    if not os.path.exists(so):
        return None
    lib = ctypes.CDLL(so)
    with open(os.path.join(REF, "g3m3_ref.json")) as fh:
        meta = json.load(fh)
    _LIB = (lib, meta)
    return _LIB


def dummies(name):
    return load()[1]["subroutines"][name]["args"]


def call(name, *args):
    """CALL name(args) with Fortran by-reference semantics."""
    lib, meta = load()
    ds = meta["subroutines"][name]["args"]
    if len(args) != len(ds):
        raise TypeError(f"{name}: {len(args)} arguments for {len(ds)} dummies")
    keep, cargs = [], []
    for a, d in zip(args, ds):
        t = d["type"]
        if isinstance(a, np.ndarray):
            if t in _NP and a.dtype != _NP[t]:
                raise TypeError(f"{name}: {d['name']} wants {t}, got {a.dtype}")
            if not a.flags["C_CONTIGUOUS"]:
                raise TypeError(f"{name}: {d['name']} is not contiguous")
            cargs.append(ctypes.c_void_p(a.ctypes.data))
        elif isinstance(a, (ctypes._SimpleCData, ctypes.Array, ctypes.Structure)):
            cargs.append(ctypes.c_void_p(ctypes.addressof(a)))
        elif isinstance(a, (bytes, str)):
            buf = ctypes.create_string_buffer(a.encode() if isinstance(a, str) else a)
            keep.append(buf)
            cargs.append(ctypes.c_void_p(ctypes.addressof(buf)))
        else:
            if d["rank"]:
                raise TypeError(f"{name}: {d['name']} is an array")
            v = _CT[t](a)
            keep.append(v)
            cargs.append(ctypes.c_void_p(ctypes.addressof(v)))
    fn = getattr(lib, "ref_" + name)
    fn.restype = None
    fn.argtypes = [ctypes.c_void_p] * len(cargs)
    fn(*cargs)
    del keep


def set_common(block, **values):
    """Store values into a common block by member name (scalars or arrays)."""
    lib, meta = load()
    blk = meta["commons"][block]
    base = ctypes.addressof(ctypes.c_ubyte.in_dll(lib, "ref_common_" + block))
    members = {m["name"]: m for m in blk["members"]}
    for k, v in values.items():
        m = members[k]
        arr = np.ascontiguousarray(np.asarray(v, dtype=_NP[m["type"]]).ravel())
        if arr.size > m["count"]:
            raise ValueError(f"/{block}/ {k}: {arr.size} values for {m['count']}")
        ctypes.memmove(base + m["offset"], arr.ctypes.data, arr.nbytes)
