"""ctypes access to the CPU oracle (TEST INFRASTRUCTURE ONLY).

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg may
import this module.  It loads liboracle.so (serial, the parity reference) or
liboracle_omp.so (OpenMP, the timed baseline); both give identical bits.
Pinned to the reference's own routines and main loop: see g3m3_oracle.h.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

from g3m3_gb300.params import G3M3Params, NFIELDS, MAX_GRIDS

HERE = os.path.dirname(os.path.abspath(__file__))
_fp = ctypes.POINTER(ctypes.c_float)
_ip = ctypes.POINTER(ctypes.c_int32)
_dp = ctypes.POINTER(ctypes.c_double)


def build():
    subprocess.run(["make", "-s", "-C", HERE], check=True)


def fptr(a):
    assert a.dtype == np.float32 and a.flags["C_CONTIGUOUS"], (a.dtype, a.flags)
    return a.ctypes.data_as(_fp)


def _rptr(a):
    """A float64 array passed where the FP64 build's REAL pointers go."""
    assert a.dtype == np.float64 and a.flags["C_CONTIGUOUS"], (a.dtype, a.flags)
    return ctypes.cast(a.ctypes.data, _fp)


def iptr(a):
    assert a.dtype == np.int32 and a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(_ip)


class OracleState(ctypes.Structure):
    _fields_ = [
        ("cur", _fp * NFIELDS), ("old", _fp * NFIELDS), ("wrk", _fp * NFIELDS),
        ("b0", _fp * 3), ("resistive", _fp),
        ("ijsrf", _ip), ("ijmid", _ip), ("ijzero", _ip),
        ("numsrf", _ip), ("nummid", _ip), ("numzero", _ip),
        ("parm_srf", _fp), ("parm_mid", _fp), ("parm_zero", _fp),
        ("msrf", ctypes.c_int), ("mmid", ctypes.c_int), ("mzero", ctypes.c_int),
        ("efld", _fp * 3), ("curr", _fp * 3), ("bs", _fp * 3), ("btot", _fp),
        ("vv", _fp * 3), ("tv", _fp * 3), ("ev", _fp * 3),
        ("t", ctypes.c_double),
        ("t_old", ctypes.c_double * MAX_GRIDS), ("t_new", ctypes.c_double * MAX_GRIDS),
        ("t_step", ctypes.c_double * MAX_GRIDS), ("t_stepnew", ctypes.c_double * MAX_GRIDS),
        ("cell_updates", ctypes.c_int64), ("nsteps_done", ctypes.c_int32),
        ("last_cg_iters", ctypes.c_int32),
    ]


_LIBS = {}


def _dptr(a):
    """A complex128 array (value, tangent) passed where the forward-mode
    build's dual REAL pointers go."""
    assert a.dtype == np.complex128 and a.flags["C_CONTIGUOUS"], (a.dtype, a.flags)
    return ctypes.cast(a.ctypes.data, _fp)


def lib(omp: bool = False, real8: bool = False, dual: bool = False):
    name = ("liboracle_dual_omp" if dual else
            "liboracle" + ("_r8" if real8 else "") + ("_omp" if omp else "")) + ".so"
    if name not in _LIBS:
        path = os.path.join(HERE, name)
        if not os.path.exists(path):
            build()
        L = ctypes.CDLL(path)
        if real8 or dual:   # only the main-step entries (below) are used; their arguments are pointers
            _LIBS[name] = L
            return L
        from g3m3_gb300 import _lib as glib
        for fname, ret, params in glib.header_functions(os.path.join(HERE, "g3m3_oracle.h"), "oracle_"):
            fn = getattr(L, fname)
            fn.restype = glib.restype_of(ret)
            fn.argtypes = [glib.ctype_of(q) for q in params]
        _LIBS[name] = L
    return _LIBS[name]


class OracleModel:
    """Holds a full multi-box state in numpy arrays and steps it on the CPU
    with the oracle's restatement of the reference main loop.  With
    ``real8``, the FP64 build (every REAL in double precision, real8.h):
    the state is float64, started from the FP32 state's values.  With
    ``dual``, the FP64 build in forward-mode dual numbers (dual.h): the
    state is complex128, value in the real part and tangent in the
    imaginary part (zero to start), and ``wind_tangent`` (8) seeds the
    wind-face parameters' tangents."""

    def __init__(self, state, omp: bool = False, real8: bool = False, dual: bool = False):
        self.L = lib(omp, real8, dual)
        self.real8 = real8 or dual
        self.dual = dual
        self.p = state.params
        p = self.p
        ft = np.complex128 if dual else (np.float64 if real8 else np.float32)
        self.cur = state.cur.astype(ft)
        self.old = np.zeros_like(self.cur)
        self.wrk = self.cur.copy()   # wrkepres is read before it is written
        self.b0 = state.b0.astype(ft)
        self.resistive = state.resistive.astype(ft)
        self.lists = {k: np.ascontiguousarray(v) for k, v in state.lists.items()}
        if real8 or dual:
            for k in ("parm_srf", "parm_mid", "parm_zero"):
                self.lists[k] = np.ascontiguousarray(self.lists[k], ft)
        box = (p.nz, p.ny, p.nx)
        self.scr = np.zeros((19,) + box, ft)
        fptr = _dptr if dual else (_rptr if real8 else globals()["fptr"])
        s = OracleState()
        for q in range(NFIELDS):
            s.cur[q] = fptr(self.cur[q]); s.old[q] = fptr(self.old[q]); s.wrk[q] = fptr(self.wrk[q])
        for q in range(3):
            s.b0[q] = fptr(self.b0[q])
        s.resistive = fptr(self.resistive)
        for key in ("srf", "mid", "zero"):
            setattr(s, "ij" + key, iptr(self.lists["ij" + key]))
            setattr(s, "num" + key, iptr(self.lists["num" + key]))
            setattr(s, "parm_" + key, fptr(self.lists["parm_" + key]))
            setattr(s, "m" + key, self.lists["ij" + key].shape[0])
        names = ["efld"] * 3 + ["curr"] * 3 + ["bs"] * 3 + ["btot"] + ["vv"] * 3 + ["tv"] * 3 + ["ev"] * 3
        idx = {}
        for i, n in enumerate(names):
            k = idx.get(n, 0)
            if n == "btot":
                s.btot = fptr(self.scr[i])
            else:
                getattr(s, n)[k] = fptr(self.scr[i])
            idx[n] = k + 1
        self.s = s

    def set_wind_tangent(self, t):
        """The tangents of the eight wind-face parameters (forward-mode build)."""
        assert self.dual
        arr = (ctypes.c_double * 8).in_dll(self.L, "oracle_wind_tangent")
        for k in range(8):
            arr[k] = float(t[k])

    def init_steps(self):
        self.L.oracle_init_steps(ctypes.byref(self.p), ctypes.byref(self.s))

    def main_step(self):
        return self.L.oracle_main_step(ctypes.byref(self.p), ctypes.byref(self.s))

    def divb_all(self):
        self.L.oracle_divb_all(ctypes.byref(self.p), ctypes.byref(self.s))

    @property
    def t_stepnew(self):
        return np.array(self.s.t_stepnew[: self.p.n_grids])

    @property
    def cell_updates(self):
        return int(self.s.cell_updates)


def call(name, *args, omp=False):
    """oracle_<name>(*args) with numpy arrays / ctypes objects converted to
    addresses -- the same argument list as the library's g3m3_<name>."""
    from g3m3_gb300.api import addr
    L = lib(omp)
    fn = getattr(L, "oracle_" + name)
    conv = [addr(a) if t is ctypes.c_void_p else a for a, t in zip(args, fn.argtypes)]
    if len(conv) != len(fn.argtypes):
        raise TypeError(f"oracle_{name} takes {len(fn.argtypes)} arguments, got {len(args)}")
    return fn(*conv)
