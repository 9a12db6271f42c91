"""Shared test helpers: seeded inputs, the same argument list for the
oracle (oracle_<name>) and the library (g3m3_<name>), and comparisons.

Parity bar: the library reproduces the oracle's FP32 arithmetic operation
for operation, so the per-routine tests require bitwise equality (with
+0 == -0 and NaN == NaN); the div B solver accumulates its dot products in
FP64 where the oracle uses FP32, so it is compared at its convergence
tolerance.
"""
from __future__ import annotations

import ctypes
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

from g3m3_gb300.params import NFIELDS  # noqa: E402
from g3m3_gb300.state import make_config, perturbed  # noqa: E402


def has_gpu():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


def same_bits(a, b):
    """Element-wise equality treating NaN == NaN and +0 == -0."""
    a = np.asarray(a)
    b = np.asarray(b)
    return (a == b) | (np.isnan(a) & np.isnan(b))


def assert_same(got, want, what=""):
    eq = same_bits(got, want)
    if not eq.all():
        idx = np.argwhere(~eq)
        g, w = np.asarray(got), np.asarray(want)
        diff = np.abs(g.astype(np.float64) - w.astype(np.float64))
        first = tuple(idx[0])
        raise AssertionError(
            f"{what}: {int((~eq).sum())} of {eq.size} values differ; max |diff| {np.nanmax(diff):.3e}; "
            f"first at {first}: got {g[first]!r} want {w[first]!r}")


def rel_l2(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    den = np.linalg.norm(b)
    return np.linalg.norm(a - b) / (den if den > 0 else 1.0)


class Inputs:
    """cur/old/wrk copies of a seeded state plus per-box scratch inputs."""

    def __init__(self, name="tiny2", seed=7, **over):
        self.st = make_config(name, **over)
        self.p = self.st.params
        p = self.p
        self.cur = self.st.cur.copy()
        self.old = perturbed(self.st, seed + 1, 2e-3).cur
        self.wrk = perturbed(self.st, seed + 2, 2e-3).cur
        self.b0 = self.st.b0.copy()
        rng = np.random.default_rng(seed)
        box3 = (p.nz, p.ny, p.nx)
        # perturbation B is small compared to b0: give it structure
        for q in (31, 32, 33):
            for arr, sc in ((self.cur, 0.02), (self.old, 0.021), (self.wrk, 0.019)):
                arr[q] = (arr[q] + sc * rng.standard_normal(arr[q].shape)).astype(np.float32)
        self.rng = rng
        self.box3 = box3
        self.lists = self.st.lists
        self.resistive = self.st.resistive.copy()

    def crop(self, nx, ny, nz):
        """Keep the first nx x ny x nz cells of every box: an anisotropic box
        whose sizes leave ragged tiles in every direction.  Each box keeps
        its spacing; its upper extents follow.  The inner-boundary lists no
        longer apply."""
        p = self.p
        assert nx <= p.nx and ny <= p.ny and nz <= p.nz
        for name in ("cur", "old", "wrk", "b0"):
            setattr(self, name, np.ascontiguousarray(getattr(self, name)[:, :, :nz, :ny, :nx]))
        self.resistive = np.ascontiguousarray(self.resistive[:, :nz, :ny, :nx])
        for b in range(p.n_grids):
            for ax, n_old, n_new in (("x", p.nx, nx), ("y", p.ny, ny), ("z", p.nz, nz)):
                lo, hi = getattr(p, f"grd_{ax}min"), getattr(p, f"grd_{ax}max")
                hi[b] = lo[b] + (hi[b] - lo[b]) / (n_old - 1) * (n_new - 1)
        p.nx, p.ny, p.nz = nx, ny, nz
        self.box3 = (nz, ny, nx)
        self.lists = None
        return self

    def scratch(self, scale=1.0, n=1):
        return [(scale * self.rng.standard_normal(self.box3)).astype(np.float32) for _ in range(n)]

    def grid(self):
        p = self.p
        g = [np.array(getattr(p, k)[: p.n_grids], np.float32)
             for k in ("grd_xmin", "grd_xmax", "grd_ymin", "grd_ymax", "grd_zmin", "grd_zmax")]
        return g

    def dims(self, box):
        p = self.p
        return [p.nx, p.ny, p.nz, p.n_grids, box]


def copy_args(args):
    """Deep-copy the numpy arrays of an argument list (each side mutates its own)."""
    out = []
    for a in args:
        if isinstance(a, np.ndarray):
            out.append(a.copy())
        elif isinstance(a, list):
            out.append([x.copy() if isinstance(x, np.ndarray) else x for x in a])
        else:
            out.append(a)
    return out


def tables(args):
    """Turn list-of-array arguments into ctypes pointer tables (kept alive)."""
    from g3m3_gb300.api import addr
    out, keep = [], []
    for a in args:
        if isinstance(a, list):
            t = (ctypes.c_void_p * len(a))(*[addr(x) for x in a])
            keep.append(t)
            out.append(t)
        else:
            out.append(a)
    return out, keep


def run_both(name, args, gpu_name=None, gpu_extra=(), oracle_drop=()):
    """Run oracle_<name> and g3m3_<name> on separate copies of args and
    return (oracle_args, gpu_args) after the calls (arrays read back)."""
    from oracle import oracle
    from g3m3_gb300.api import Context
    oa = copy_args(args)
    oargs, okeep = tables(oa)
    oracle.call(name, *oargs)
    ga = copy_args(args)
    gl = [a for i, a in enumerate(ga) if i not in oracle_drop]
    gargs, gkeep = tables(gl)
    with Context() as ctx:
        ctx.call(gpu_name or name, *gargs, *gpu_extra)
        for a in ga:
            if isinstance(a, np.ndarray):
                ctx.sync_to_host(a)
            elif isinstance(a, list):
                for x in a:
                    if isinstance(x, np.ndarray):
                        ctx.sync_to_host(x)
        ctx.synchronize()
    return oa, ga
