"""ctypes access to oracle/_ref/libg3m3_ref_main_<tag>[_omp].so: the
reference's time-step set-up and main time loop (the body of ``do
while(t.lt.tmax)``, code/3d_main.f90), translated to C with all its routines
by oracle/fortran_to_c.py for one grid size.

TEST INFRASTRUCTURE ONLY: the tests use it as the parity reference of the
main step, and bench.py's CPU legs time it as the reference's own CPU path.

The main program's variables are globals ``ref_main_<name>``; this module
loads a state into them the way the reference's initialisation leaves it,
runs main steps, and reads the fields back.  Everything outside the hot path
stays off: no spacecraft, no fluid input, no tilting, no torus injection, no
graphing; fluid-file times control the div B pass.
"""
from __future__ import annotations

import ctypes
import json
import os

import numpy as np

from oracle.fortran_to_c import OUT as REF, main as _build_all
from g3m3_gb300.params import FIELD_NAMES

_CT = {"int": ctypes.c_int32, "logical": ctypes.c_int32, "float": ctypes.c_float,
       "double": ctypes.c_double}
_NP = {"int": np.int32, "logical": np.int32, "float": np.float32, "double": np.float64}
BIG = 1.0e30


class RefMain:
    def __init__(self, tag, omp=False, real8=False):
        stem = f"g3m3_ref_main_{tag}" + ("_r8" if real8 else "") + ("_omp" if omp else "")
        so = os.path.join(REF, f"lib{stem}.so")
        if not os.path.exists(so):
            _build_all(["fortran_to_c"])     # builds everything where the sources exist
        if not os.path.exists(so):
            raise FileNotFoundError(so)
        self.lib = ctypes.CDLL(so)
        with open(os.path.join(REF, f"{stem}.json")) as fh:
            self.meta = json.load(fh)
        self.vars = self.meta["main"]["variables"]
        self.keep = []
        # fluid files written at fluid-file times go to a scratch directory
        # unless set_unit_dir chooses one
        import tempfile
        self._tmp = tempfile.TemporaryDirectory(prefix="g3m3_ref_units_")
        self.set_unit_dir(self._tmp.name)

    # ---- variables ----
    def _sym(self, name, ctype):
        return ctype.in_dll(self.lib, "ref_main_" + name)

    def set(self, **values):
        for k, v in values.items():
            if k not in self.vars:           # a member of one of the main program's commons
                blk = next(b for b, d in self.meta["commons"].items()
                           if any(m["name"] == k for m in d["members"]))
                self.set_common(blk, **{k: v})
                continue
            m = self.vars[k]
            if m["dims"] is not None:
                raise TypeError(f"{k} is an array")
            self._sym(k, _CT[m["type"]]).value = v

    def get(self, name):
        m = self.vars[name]
        return self._sym(name, _CT[m["type"]]).value

    def array(self, name):
        """numpy view of a fixed-size array, C order (the Fortran dims reversed)."""
        m = self.vars[name]
        ptr = ctypes.c_void_p.in_dll(self.lib, "ref_main_" + name).value
        n = int(np.prod(m["dims"]))
        buf = (_CT[m["type"]] * n).from_address(ptr)
        return np.ctypeslib.as_array(buf).reshape(tuple(reversed(m["dims"])))

    def set_allocatable(self, name, arr, fdims):
        """Point an ALLOCATABLE array at `arr` (C order of Fortran dims `fdims`)."""
        m = self.vars[name]
        a = np.ascontiguousarray(arr, dtype=_NP[m["type"]])
        assert a.size == int(np.prod(fdims))
        self.keep.append(a)
        ctypes.c_void_p.in_dll(self.lib, "ref_main_" + name).value = a.ctypes.data
        for d, e in enumerate(fdims):
            ctypes.c_long.in_dll(self.lib, f"ref_main_{name}_lo{d}").value = 1
            ctypes.c_long.in_dll(self.lib, f"ref_main_{name}_ex{d}").value = int(e)

    def set_common(self, block, **values):
        blk = self.meta["commons"][block]
        base = ctypes.addressof(ctypes.c_ubyte.in_dll(self.lib, "ref_common_" + block))
        members = {m["name"]: m for m in blk["members"]}
        for k, v in values.items():
            m = members[k]
            a = np.ascontiguousarray(np.asarray(v, dtype=_NP[m["type"]]).ravel())
            ctypes.memmove(base + m["offset"], a.ctypes.data, a.nbytes)

    def set_unit_dir(self, path):
        """Directory where the loop's unformatted units (the fluid files,
        unit fluid_f) are written as fort.<unit>."""
        b = os.fsencode(path)[:511] + b"\0"
        buf = (ctypes.c_char * 512).in_dll(self.lib, "ref_unit_dir")
        ctypes.memmove(ctypes.addressof(buf), b, len(b))

    # ---- running ----
    def init_steps(self):
        """The reference's time-step set-up before its loop (density and
        speed checks of every box, first t_stepnew)."""
        self.lib.ref_main_init_steps()
        self._check()

    def steps(self, n):
        self.lib.ref_main_steps.argtypes = [ctypes.c_void_p]
        k = ctypes.c_int32(n)
        self.lib.ref_main_steps(ctypes.addressof(k))
        self._check()

    def fresh_start(self, p, consts, capacity=None):
        """The reference's fresh start (the ELSE branch of its
        ``if(.not.start)``, 3d_main.f90:1194-1634: dipole field, corotating
        ionospheric plasma, solar wind, speed clip, inner-boundary lists,
        resistivity) for the grid and constants of `p`, with the derived
        constants `consts` the reference computes before it (3d_main.f90:
        790-880): r_inner, zero/mid/srf_bndry, erho, b0, cs_inner, alpha_e,
        cs_wind, xdip; no rotation, tilt, moon or torus.  Returns the fields
        (34, n_grids, nz, ny, nx), b0 (3, ...), the resistivity and the
        inner-boundary lists as make_state's ``lists``."""
        ng, mb = p.n_grids, p.mbndry
        gmin, gmax = self.array("grid_minvals"), self.array("grid_maxvals")
        for b in range(ng):
            gmin[b] = [p.grd_xmin[b], p.grd_ymin[b], p.grd_zmin[b]]
            gmax[b] = [p.grd_xmax[b], p.grd_ymax[b], p.grd_zmax[b]]
        self.array("xspac")[...] = np.array(p.xspac[:ng], np.float32)
        for k in ("rmassq", "rmassh", "rmasso", "gamma", "resist", "re_equiv", "srho", "rho_frac", "spress",
                  "spx", "spy", "spz", "ti_te"):
            self.set(**{k: float(getattr(p, k))})
        for k in ("r_inner", "zero_bndry", "mid_bndry", "srf_bndry", "erho", "cs_inner", "alpha_e", "cs_wind"):
            self.set(**{k: float(consts[k])})
        self.set(t=0.0, utstart=0.0, t_equiv=1.0, tsave=BIG, tmax=BIG, deltg=BIG, deltinj=BIG, planet_per=1.0,
                 moon_per=1.0, moon_init_rot=0.0, moon_orbit_rad=0.0)
        self.set_common("rotation", v_rot=p.v_rot, r_rot=p.r_rot, xdip=consts["xdip"], ydip=0.0, zdip=0.0,
                        sin_tilt=0.0, cos_tilt=1.0, b0=consts["b0"])
        cap = capacity or p.nx * p.ny * p.nz
        lists = {}
        for key in ("srf", "mid", "zero"):
            ij = np.zeros((cap, 3, mb), np.int32)
            parm = np.zeros((cap, 7, mb), np.float32)
            self.set_allocatable("ij" + key, ij, (mb, 3, cap))
            self.set_allocatable("parm_" + key, parm, (mb, 7, cap))
            self.set(**{"m" + key: cap})
            lists[key] = (ij, parm)
        self.lib.ref_main_fresh_start()
        self._check()
        out = {"fields": self.fields().copy(),
               "b0": np.stack([self.array(f"b{c}0").copy() for c in "xyz"]),
               "resistive": self.array("resistive").copy()}
        for key, (ij, parm) in lists.items():
            num = self.array("num" + key).copy()
            m = int(num.max()) if num.size else 0
            out["ij" + key] = ij[:max(m, 1)].copy()
            out["parm_" + key] = parm[:max(m, 1)].copy()
            out["num" + key] = num
        return out

    def divb_pass(self, p):
        """One div B cleaning pass as the main loop makes it at a fluid-file
        time (3d_main.f90:3363-3408): divB_correct twice per box from the
        outermost in, flanks_synced of bx, by, bz from box n_grids-1 down,
        bndry_corer from box 1 up, each the reference's own routine called
        on the loop's arrays.  Returns the seconds it took."""
        import time
        nx, ny, nz, ng = p.nx, p.ny, p.nz, p.n_grids
        i32 = lambda v: ctypes.byref(ctypes.c_int32(v))
        pos = np.array([nx * ny, nx, 1, 0, -1, -nx, -nx * ny], np.int32)
        xs = np.ascontiguousarray(self.array("xspac"), np.float32)
        err = ctypes.c_float(p.divb_errlim)
        gmin, gmax = self.array("grid_minvals"), self.array("grid_maxvals")
        grids = [np.ascontiguousarray(a[:, q]) for q in range(3) for a in (gmin, gmax)]
        gptr = [g.ctypes.data_as(ctypes.c_void_p) for g in grids]
        b = [self.array(n).ctypes.data_as(ctypes.c_void_p) for n in ("bx", "by", "bz")]
        corer = [a["name"] for a in self.meta["subroutines"]["bndry_corer"]["args"]]
        fields = [self.array(n).ctypes.data_as(ctypes.c_void_p) for n in corer[:34]]
        t0 = time.perf_counter()
        for box in range(ng, 0, -1):
            for _ in range(2):
                self.lib.ref_divb_correct(i32(nx), i32(ny), i32(nz), i32(ng), i32(box), i32(7),
                                          pos.ctypes.data_as(ctypes.c_void_p), xs.ctypes.data_as(ctypes.c_void_p),
                                          ctypes.byref(err), *b)
        for box in range(ng - 1, 0, -1):
            for q in range(3):
                self.lib.ref_flanks_synced(b[q], i32(nx), i32(ny), i32(nz), i32(ng), i32(box), *gptr)
        for box in range(1, ng):
            self.lib.ref_bndry_corer(*fields, i32(nx), i32(ny), i32(nz), i32(ng), i32(box), *gptr)
        dt = time.perf_counter() - t0
        self._check()
        return dt

    def _check(self):
        if ctypes.c_int.in_dll(self.lib, "ref_main_stopped").value:
            raise RuntimeError("the reference's main loop executed STOP")
        calls = ctypes.c_int.in_dll(self.lib, "ref_untranslated_calls").value
        if calls:
            last = ctypes.c_char.in_dll(self.lib, "ref_untranslated_last")
            raise RuntimeError(f"{calls} calls to routines off the hot path "
                               f"(last {ctypes.string_at(ctypes.addressof(last)).decode()})")

    def load_state(self, p, cur, old, wrk, b0, resistive, lists, t, t_stepnew, divb_at=None):
        """The state the reference's initialisation builds: fields, dipole,
        resistivity, inner-boundary lists, grid, constants, times.  The div B
        pass runs in the main step at which t first reaches `divb_at`."""
        ng = p.n_grids
        for q, name in enumerate(FIELD_NAMES):
            self.array(name)[...] = cur[q]
            self.array("old" + name)[...] = old[q]
            self.array("wrk" + name)[...] = wrk[q]
        for q, c in enumerate("xyz"):
            self.array(f"b{c}0")[...] = b0[q]
        res = self.array("resistive")
        res[...] = resistive.reshape(res.shape)
        for key in ("srf", "mid", "zero"):
            ij = lists["ij" + key]            # C order (m, 3, mbndry) = Fortran (mbndry, 3, m)
            self.set_allocatable("ij" + key, ij, (p.mbndry, 3, ij.shape[0]))
            parm = lists["parm_" + key]
            self.set_allocatable("parm_" + key, parm, (p.mbndry, 7, parm.shape[0]))
            self.array("num" + key)[...] = lists["num" + key]
            self.set(**{"m" + key: int(ij.shape[0])})
        gmin, gmax = self.array("grid_minvals"), self.array("grid_maxvals")
        for b in range(ng):
            gmin[b] = [p.grd_xmin[b], p.grd_ymin[b], p.grd_zmin[b]]
            gmax[b] = [p.grd_xmax[b], p.grd_ymax[b], p.grd_zmax[b]]
        self.array("xspac")[...] = np.array(p.xspac[:ng], np.float32)
        for k in ("rmassq", "rmassh", "rmasso", "gamma", "gamma1", "reynolds", "resist", "grav", "re_equiv",
                  "chirho", "chipxyz", "chierg", "difrho", "diferg", "aniso_limit", "qvlim", "hvlim", "ovlim",
                  "qclim", "hclim", "oclim", "cslim", "stepsz", "t_step_max", "srho", "rho_frac", "o_conc",
                  "spress", "spx", "spy", "spz", "sbx_wind", "sby_wind", "sbz_wind", "ti_te", "erho", "epress",
                  "alpha_e", "r_inner"):
            self.set(**{k: float(getattr(p, k))})
        self.set(isotropic=int(p.isotropic))
        self.set_common("rotation", v_rot=p.v_rot, r_rot=p.r_rot)
        # off the hot path
        self.set(input_fluid=0, spacecraft=0, tilting=0, ringo=0, warp=0)
        self.set(tmax=BIG, tgraph=BIG, tinj=BIG, dtilt=0.0, tilt=0.0)
        self.set(t_equiv=1.0, planet_per=1.0, moon_per=1.0, moon_orbit_rad=0.0, moon_init_rot=0.0)
        self.set(rho_equiv=1.0, v_equiv=1.0, planet_rad=1.0)
        # fluid-file time: the div B pass runs there (3d_main.f90:3305-3408)
        if divb_at is None:
            self.set(ts1=BIG, divb_lores=0)
        else:
            self.set(ts1=float(divb_at), tsave=BIG, divb_lores=1, fluid_f=11, offset_f=0)
        self.set(t=float(t))
        self.array("t_stepnew")[...] = np.asarray(t_stepnew, np.float64)

    def box_steps(self):
        """Box-steps of box 1..n_grids in the last main step: box b steps
        every t_step(b) through the main step of length t_step(n_grids)
        (3d_main.f90:1954-1966)."""
        ts = self.array("t_step")
        return [int(round(ts[-1] / ts[b])) for b in range(len(ts))]

    def fields(self):
        return np.stack([self.array(n) for n in FIELD_NAMES])
