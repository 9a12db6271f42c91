"""Python side of the G3M^3 GB300 library (ctypes over libg3m3_gpu.so).

``Context`` exposes the drop-in routines with the reference's argument
order: ``ctx.push_ion(qrho, ..., isotropic)`` takes exactly the arguments of
sub_push_ion.f90:4-17.  Arrays may be numpy arrays (mirrored on the device,
read back with ``ctx.sync_to_host``) or CUDA tensors (``data_ptr``).
``Model`` drives the step engine on a device-resident multi-box state.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib
from .params import G3M3Params, NFIELDS

_vp = ctypes.c_void_p


def addr(x):
    """Raw address of a numpy array, CUDA tensor, ctypes object or int."""
    if x is None:
        return None
    if isinstance(x, int):
        return x
    if isinstance(x, np.ndarray):
        if not x.flags["C_CONTIGUOUS"]:
            raise ValueError("arrays must be contiguous")
        return x.ctypes.data
    if hasattr(x, "data_ptr"):
        if not x.is_contiguous():
            raise ValueError("tensors must be contiguous")
        return x.data_ptr()
    if isinstance(x, ctypes.Array) or isinstance(x, ctypes.Structure):
        return ctypes.addressof(x)
    raise TypeError(f"cannot take the address of {type(x)}")


class G3M3Error(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"g3m3 error {code}: {msg}")
        self.code = code


def table(arrays):
    """A ctypes array of 34 addresses (the field tables of the C ABI)."""
    t = (ctypes.c_void_p * NFIELDS)()
    for i, a in enumerate(arrays):
        t[i] = addr(a)
    return t


class Context:
    def __init__(self, device: int = 0):
        self.L = _lib.load()
        h = ctypes.c_void_p()
        rc = self.L.g3m3_ctx_create(ctypes.byref(h), device)
        if rc:
            raise G3M3Error(rc, "context creation failed (no CUDA device?)")
        self.h = h
        self._keep = []
        self._models = []

    def close(self):
        if self.h:
            for m in list(self._models):   # models use the context's stream
                m.close()
            self._models = []
            self.L.g3m3_ctx_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def check(self, rc):
        if rc:
            msg = self.L.g3m3_last_error(self.h)
            raise G3M3Error(rc, msg.decode() if msg else "")
        return rc

    def sync_to_host(self, *arrays):
        for a in arrays:
            self.check(self.L.g3m3_sync_to_host(self.h, addr(a)))

    def sync_to_device(self, *arrays):
        for a in arrays:
            self.check(self.L.g3m3_sync_to_device(self.h, addr(a)))

    def synchronize(self):
        self.check(self.L.g3m3_synchronize(self.h))

    def call(self, name, *args, check=True):
        """Call g3m3_<name>(ctx, *args); arrays are converted to addresses."""
        fn = getattr(self.L, "g3m3_" + name)
        conv = []
        for a, t in zip(args, fn.argtypes[1:]):
            if t is ctypes.c_void_p:
                conv.append(addr(a))
            else:
                conv.append(a)
        if len(conv) != len(fn.argtypes) - 1:
            raise TypeError(f"g3m3_{name} takes {len(fn.argtypes) - 1} arguments, got {len(conv)}")
        rc = fn(self.h, *conv)
        return self.check(rc) if check else rc

    def __getattr__(self, name):
        if name.startswith("_") or name in ("L", "h"):
            raise AttributeError(name)
        return lambda *args, **kw: self.call(name, *args, **kw)


class Model:
    """A multi-box state on the device advanced by the step engine."""

    def __init__(self, ctx: Context, state, handle=None, params=None):
        """A new model for ``state``; with ``handle``, a view of a model the
        library already holds (an ensemble member), which this object loads
        with ``state`` but does not destroy.  With ``state`` None, an empty
        model for ``params`` (fill it with :meth:`init_state`)."""
        self.ctx = ctx
        self.L = ctx.L
        self.p = state.params if state is not None else params
        self.owned = handle is None
        if handle is None:
            h = ctypes.c_void_p()
            ctx.check(self.L.g3m3_model_create(ctx.h, ctypes.byref(self.p), ctypes.byref(h)))
            self.h = h
            ctx._models.append(self)
        else:
            self.h = handle
        if state is not None:
            self.upload(state)

    GRAPHING = (["bx_total", "by_total", "bz_total", "btot", "ex", "ey", "ez", "jx", "jy", "jz"]
                + [f"{s}{q}" for s in ("q", "h", "o")
                   for q in ("vx", "vy", "vz", "p_para", "p_perp", "p_cross", "rho")] + ["epres"])

    def graphing(self, box: int, plane: int, index: int):
        """One grid plane (0: x-y at k=index, 1: x-z at j=index, 2: y-z at
        i=index) of the graphing quantities of box ``box``, code units."""
        p = self.p
        na = p.ny if plane == 0 else p.nz
        nb = p.ny if plane == 2 else p.nx
        out = np.zeros((32, na, nb), np.float32)
        self.ctx.check(self.L.g3m3_model_graphing(self.h, box, plane, index, addr(out)))
        return dict(zip(self.GRAPHING, out))

    def init_state(self, alf_inner=-5.0, seed=20261203, noise=0.01, iono_lo=1.0, iono_hi=1.0):
        """The fresh-start state built on the device (dipole, plasma load,
        solar wind, speed clip, seeded perturbation, inner lists)."""
        self.ctx.check(self.L.g3m3_model_init_state(self.h, float(alf_inner), int(seed), float(noise),
                                                   float(iono_lo), float(iono_hi)))

    def upload(self, state):
        L, h = self.L, self.h
        cur = np.ascontiguousarray(state.cur, np.float32)
        self.ctx.check(L.g3m3_model_set_state(h, addr(cur)))
        # the wrk copy starts as the state (wrkepres is read before written)
        for q in range(NFIELDS):
            self.ctx.check(L.g3m3_model_set_field(h, 2, q, addr(cur[q])))
        b0 = np.ascontiguousarray(state.b0, np.float32)
        self.ctx.check(L.g3m3_model_set_b0(h, addr(b0[0]), addr(b0[1]), addr(b0[2])))
        li = state.lists
        self._keep = [li, cur, b0]
        rst = np.ascontiguousarray(state.resistive, np.float32)
        self.ctx.check(L.g3m3_model_set_inner(
            h, addr(rst),
            addr(li["ijsrf"]), addr(li["numsrf"]), addr(li["parm_srf"]), li["ijsrf"].shape[0],
            addr(li["ijmid"]), addr(li["nummid"]), addr(li["parm_mid"]), li["ijmid"].shape[0],
            addr(li["ijzero"]), addr(li["numzero"]), addr(li["parm_zero"]), li["ijzero"].shape[0]))
        self.ctx.synchronize()

    def record_fluxes(self, scale, capacity: int):
        """Record flux_counter of every box at the start of each main step
        (scale: one float per box)."""
        sc = np.ascontiguousarray(scale, np.float32)
        self._flux_scale = sc
        self.ctx.check(self.L.g3m3_model_record_fluxes(self.h, addr(sc), int(capacity)))
        self._flux_cap = int(capacity)

    def fluxes(self):
        """(steps, n_grids, 6) array: q in, q out, h in, h out, o in, o out."""
        cap = getattr(self, "_flux_cap", 0)
        out = np.zeros((max(cap, 1), self.p.n_grids, 6), np.float32)
        n = ctypes.c_int()
        self.ctx.check(self.L.g3m3_model_fluxes(self.h, addr(out), ctypes.byref(n)))
        return out[: n.value]

    def set_variant(self, kernel: int, variant: int):
        self.ctx.check(self.L.g3m3_model_set_variant(self.h, kernel, variant))

    def autotune(self):
        """Times the flux-correction variants (0: 32x8 tiles, 1: 32x16,
        2/3: 32x8 with two fields per block in FP32x2, 3/4 blocks per SM,
        4/5/6: the same with asynchronous plane copies and one barrier per
        plane, 3/3/4 blocks per SM, 7: that form on 32x16 tiles) on this
        model's box size and keeps the fastest; returns the chosen
        variant."""
        v = ctypes.c_int(-1)
        self.ctx.check(self.L.g3m3_model_autotune(self.h, ctypes.byref(v)))
        return v.value

    def init_steps(self):
        self.ctx.check(self.L.g3m3_model_init_steps(self.h))

    def run(self, nsteps: int, graph: bool = False):
        self.ctx.check(self.L.g3m3_model_run(self.h, nsteps, 1 if graph else 0))

    def divb_all(self):
        rc = self.L.g3m3_model_divb_all(self.h)
        if rc not in (0, 3):
            self.ctx.check(rc)
        return rc

    def state(self, out=None):
        p = self.p
        if out is None:
            out = np.empty((NFIELDS, p.n_grids, p.nz, p.ny, p.nx), np.float32)
        self.ctx.check(self.L.g3m3_model_get_state(self.h, addr(out)))
        return out

    def set_state(self, arr):
        self.ctx.check(self.L.g3m3_model_set_state(self.h, addr(arr)))

    def step_host(self, inp, out, graph: bool = False):
        """One main step from host state ``inp`` to host state ``out`` (the
        :meth:`state` layout; pinned buffers let the per-box uploads overlap
        the step)."""
        self.ctx.check(self.L.g3m3_model_step_host(self.h, addr(inp), addr(out), 1 if graph else 0))

    def field(self, which: int, q: int):
        p = self.p
        out = np.empty((p.n_grids, p.nz, p.ny, p.nx), np.float32)
        self.ctx.check(self.L.g3m3_model_get_field(self.h, which, q, addr(out)))
        return out

    def times(self):
        t = ctypes.c_double()
        tsn = (ctypes.c_double * self.p.n_grids)()
        cu = ctypes.c_int64()
        self.ctx.check(self.L.g3m3_model_times(self.h, ctypes.byref(t), tsn, ctypes.byref(cu)))
        return t.value, np.array(tsn[:]), cu.value

    def set_capture_after(self, n: int):
        """Capture a step plan's graph at its n-th occurrence (1: at once)."""
        self.ctx.check(self.L.g3m3_model_set_capture_after(self.h, int(n)))

    def clock(self):
        """(t, main steps done): the time and the count the div B cadence
        follows."""
        t = ctypes.c_double()
        n = ctypes.c_int()
        self.ctx.check(self.L.g3m3_model_get_clock(self.h, ctypes.byref(t), ctypes.byref(n)))
        return t.value, n.value

    def set_clock(self, t, nsteps_done):
        self.ctx.check(self.L.g3m3_model_set_clock(self.h, float(t), int(nsteps_done)))

    def stats(self):
        k = ctypes.c_int64()
        g = ctypes.c_int64()
        self.ctx.check(self.L.g3m3_model_stats(self.h, ctypes.byref(k), ctypes.byref(g)))
        return k.value, g.value

    @property
    def stream(self):
        return self.L.g3m3_model_stream(self.h)

    def close(self):
        if self.h and self.ctx.h and self.owned:
            self.L.g3m3_model_destroy(self.h)
        self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Ensemble:
    """Independent states (box sizes may differ) advanced together: with
    ``graph=True`` one main step of every member is one CUDA graph, the
    members' kernels overlapping on their own streams."""

    def __init__(self, ctx: Context, states):
        self.ctx = ctx
        self.L = ctx.L
        self._params = (G3M3Params * len(states))(*[st.params for st in states])
        h = ctypes.c_void_p()
        ctx.check(self.L.g3m3_ensemble_create(ctx.h, len(states), self._params, ctypes.byref(h)))
        self.h = h
        ctx._models.append(self)
        self.members = []
        for i, st in enumerate(states):
            mh = ctypes.c_void_p()
            ctx.check(self.L.g3m3_ensemble_member(h, i, ctypes.byref(mh)))
            self.members.append(Model(ctx, st, handle=mh))

    def init_steps(self):
        for m in self.members:
            m.init_steps()

    def autotune(self):
        """Picks the flux-correction form once per distinct box size (on the
        first member of that size) and gives it to every member of the size;
        returns {(nx, ny, nz): variant}."""
        chosen = {}
        for m in self.members:
            key = (m.p.nx, m.p.ny, m.p.nz)
            if key not in chosen:
                chosen[key] = m.autotune()
            else:
                m.set_variant(1, chosen[key])
        return chosen

    def run(self, nsteps: int, graph: bool = True, concurrent: bool = False):
        """graph: one CUDA graph per main step for all members; concurrent
        (without graph): every member launched at once on its own stream;
        both: every member's own step graph launched at once on its own
        stream; neither: members one after another."""
        mode = (3 if concurrent else 1) if graph else (2 if concurrent else 0)
        self.ctx.check(self.L.g3m3_ensemble_run(self.h, nsteps, mode))

    def stats(self):
        k, g, cu = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int64()
        self.ctx.check(self.L.g3m3_ensemble_stats(self.h, ctypes.byref(k), ctypes.byref(g), ctypes.byref(cu)))
        return k.value, g.value, cu.value

    @property
    def stream(self):
        return self.L.g3m3_ensemble_stream(self.h)

    def close(self):
        if self.h and self.ctx.h:
            for m in self.members:
                m.h = None
            self.L.g3m3_ensemble_destroy(self.h)
        self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
