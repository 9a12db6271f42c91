"""Seeded synthetic G3M^3 states and run constants.

The reference reads its run constants from the namelist file ``input`` and
builds its initial state in the fresh-start block of code/3d_main.f90
(dipole :1268-1289, plasma load :1291-1367, inner-boundary index lists
:1374-1452, solar-wind fill :1466-1585, speed clip :1589-1625, set_resist
:1629).  This module restates those formulas in numpy (float64, rounded to
FP32 at the end) so that every test and benchmark starts from a physically
shaped state, and adds the seeded 1 % multiplicative Gaussian perturbation
on density and diagonal pressure that the benchmark configurations ask for.

No reference data are read: all inputs are synthetic.  Configurations:

* ``small``     -- 1 box 61x61x31 (the CPU-runnable case)
* ``nested``    -- 5 boxes 121x121x61, 2x refinement (production grid)
* ``tiny``/``tiny2``/``tiny3`` -- 17x17x9 grids with 1-3 boxes for tests
* any custom limit / n_grids via :func:`make_config`
"""
from __future__ import annotations

import dataclasses
import math

import numpy as np

from .params import G3M3Params, NFIELDS, F, F_EPRES, F_BX, F_BY, F_BZ

MU0 = 4.0e-7 * math.pi          # mod_astrometry.f90:21
M_PROT = 1.67262e-27            # mod_astrometry.f90:22
EARTH_RAD = 6378.14             # mod_astrometry.f90:158 (km)
EARTH_PER = 24.0                # hours
EARTH_R_ROT = 10.0              # planet radii
EV = 1.602176634e-19


@dataclasses.dataclass
class UpstreamWind:
    """Upstream solar wind in physical units."""
    n_cm3: float = 5.0
    speed_kms: float = 400.0
    clock_angle: float = math.pi     # IMF direction in the y-z plane (pi: -z)
    b_nT: float = 5.0
    t_ev: float = 10.0


@dataclasses.dataclass
class Setup:
    limit: int = 30
    n_grids: int = 1
    wind_adjust: float = 1.0
    r_inner: float = 3.0              # planet radius in finest-grid cells
    rmassq: float = 1.0
    rmassh: float = 1.0
    rmasso: float = 16.0
    wind: UpstreamWind = dataclasses.field(default_factory=UpstreamWind)
    v_equiv: float = 1000.0           # km/s
    rho_equiv: float = 1.0            # cm^-3
    chi: float = 0.1                  # Lapidus coefficient (chirho=chipxyz=chierg)
    difrho: float = 0.008
    diferg: float = 0.004
    divb_errlim: float = 1.0e-4
    divb_every: int = 0
    iono_lo: float = 1.0              # ionospheric inflow density range
    iono_hi: float = 1.0              # (log-uniform per list entry)
    mbndry: int = 1
    seed: int = 20261203
    noise: float = 0.01


def _fill_params(s: Setup) -> G3M3Params:
    p = G3M3Params()
    limit = float(s.limit)
    nx = ny = 2 * s.limit + 1
    nz = s.limit + 1
    p.nx, p.ny, p.nz, p.n_grids, p.mbndry = nx, ny, nz, s.n_grids, s.mbndry
    p.isotropic = 0
    p.divb_every = s.divb_every
    # grid set-up, 3d_main.f90:723-751
    for i in range(1, s.n_grids + 1):
        xs = float(2 ** (i - 1))
        xmin, xmax = -limit * xs, limit * xs
        zmin, zmax = -(limit / 2.0) * xs, (limit / 2.0) * xs
        if i == s.n_grids:
            diff = xmax * s.wind_adjust - xmax
            xmin, xmax = xmin + diff, xmax + diff
        p.xspac[i - 1] = xs
        p.grd_xmin[i - 1], p.grd_xmax[i - 1] = xmin, xmax
        p.grd_ymin[i - 1], p.grd_ymax[i - 1] = -limit * xs, limit * xs
        p.grd_zmin[i - 1], p.grd_zmax[i - 1] = zmin, zmax
        if (1 + round((xmax - xmin) / xs) != nx) or (1 + round((zmax - zmin) / xs) != nz):
            raise ValueError("grid spacing does not match the number of points")
    # physical constants (namelists of the reference's input file)
    gamma = 1.6666
    p.rmassq, p.rmassh, p.rmasso = s.rmassq, s.rmassh, s.rmasso
    p.gamma, p.gamma1 = gamma, gamma - 1.0
    p.reynolds, p.resist = 256.0, 64.0
    re_equiv = 1.0 / s.r_inner                       # planet radii per cell
    p.re_equiv = re_equiv
    gravity = 9.8
    p.grav = gravity * (EARTH_RAD * re_equiv * 1000.0) / (1000.0 * s.v_equiv) ** 2
    p.chirho = p.chipxyz = p.chierg = s.chi
    p.difrho, p.diferg = s.difrho, s.diferg
    p.smallbit, p.aniso_limit, p.vlim_factor = 1.0e-5, 0.9995, 0.6
    p.qvlim, p.hvlim, p.ovlim = 1.0, 1.4, 2.0
    p.qclim, p.hclim, p.oclim, p.cslim = 1.0, 1.0, 4.0, 1.0
    p.stepsz, p.t_step_max, p.t_step_min = 0.25, 20.0, 1.0e-6
    # solar wind, 3d_main.f90:907-943 unit conversions
    w = s.wind
    b_equiv = s.v_equiv * 1.0e3 * math.sqrt(MU0 * s.rho_equiv * 1.0e6 * M_PROT) * 1.0e9
    den_wind1 = w.n_cm3 / s.rho_equiv
    vx_wind1 = w.speed_kms / s.v_equiv                # flows +x from the i=1 face
    cs_wind = math.sqrt(gamma * w.t_ev * EV / M_PROT) / 1.0e3 / s.v_equiv
    rho_wind1 = den_wind1 * s.rmassq
    alfy = w.b_nT * math.sin(w.clock_angle) / (b_equiv * math.sqrt(rho_wind1))
    alfz = w.b_nT * math.cos(w.clock_angle) / (b_equiv * math.sqrt(rho_wind1))
    srho = rho_wind1
    spress = (cs_wind ** 2 * srho / gamma) / (gamma - 1.0)
    p.srho, p.spress = srho, spress
    p.spx, p.spy, p.spz = srho * vx_wind1, 0.0, 0.0
    p.sbx_wind = 0.0
    p.sby_wind = alfy * math.sqrt(rho_wind1)
    p.sbz_wind = alfz * math.sqrt(rho_wind1)
    p.rho_frac, p.o_conc, p.ti_te = 0.001, 0.125, 5.0
    # inner boundary
    denh_inner, alpha_e, cs_inner = 10.0, 6.0, 0.0163
    p.erho = denh_inner * s.rmassh
    p.epress = cs_inner ** 2 * p.erho / gamma
    p.alpha_e = alpha_e
    p.r_inner = s.r_inner
    p.v_rot = 2.0 * math.pi * EARTH_RAD / (EARTH_PER * 3600.0) / s.v_equiv
    p.r_rot = EARTH_R_ROT
    p.divb_errlim = s.divb_errlim
    return p


class State:
    """Host (numpy, FP32) copy of a full multi-box state.

    ``cur`` has shape (34, n_grids, nz, ny, nx): field q's slab is the
    reference's column-major A(nx,ny,nz,n_grids) array.
    """

    def __init__(self, params: G3M3Params):
        self.params = params
        p = params
        shape = (p.n_grids, p.nz, p.ny, p.nx)
        self.cur = np.zeros((NFIELDS,) + shape, np.float32)
        self.b0 = np.zeros((3,) + shape, np.float32)
        self.resistive = np.zeros((p.mbndry, p.nz, p.ny, p.nx), np.float32)
        self.lists = {}
        self.t_stepnew = None

    @property
    def shape(self):
        return self.cur.shape[1:]

    def copy(self):
        o = State(self.params)
        o.cur = self.cur.copy()
        o.b0 = self.b0.copy()
        o.resistive = self.resistive.copy()
        o.lists = {k: v.copy() for k, v in self.lists.items()}
        return o


def _dipole(b0, ax, ay, az, xdip):
    """sub_dipole.f90:4-52 with no rotation and no tilt."""
    x1, y1, z1 = ax - xdip, ay, az
    x2, y2, z2 = x1 * x1, y1 * y1, z1 * z1
    ar = np.sqrt(x2 + y2 + z2)
    bmag = -b0 / ar ** 5
    return -3.0 * bmag * x1 * z1, -3.0 * bmag * y1 * z1, bmag * (x2 + y2 - 2.0 * z2)


def make_state(s: Setup) -> State:
    p = _fill_params(s)
    st = State(p)
    rng = np.random.default_rng(s.seed)
    nx, ny, nz = p.nx, p.ny, p.nz
    xdip = 0.00001
    r_inner = s.r_inner
    zero_b, mid_b, srf_b = r_inner - 1.5, r_inner - 0.5, r_inner + 0.6
    erho = p.erho
    alf_inner1 = -5.0              # negative: moment along -z (3d_main.f90:901)
    b0c = alf_inner1 * math.sqrt(erho) * r_inner ** 3
    cs_inner, alpha_e, d_min = 0.0163, 6.0, 0.01
    ti_te, rq, rh, ro = p.ti_te, p.rmassq, p.rmassh, p.rmasso
    re_equiv, v_rot, r_rot = p.re_equiv, p.v_rot, p.r_rot

    lists = {"srf": [], "mid": [], "zero": []}
    parms = {"srf": [], "mid": [], "zero": []}
    for box in range(1, p.n_grids + 1):
        dx = (p.grd_xmax[box - 1] - p.grd_xmin[box - 1]) / (nx - 1.0)
        dy = (p.grd_ymax[box - 1] - p.grd_ymin[box - 1]) / (ny - 1.0)
        dz = (p.grd_zmax[box - 1] - p.grd_zmin[box - 1]) / (nz - 1.0)
        az = (p.grd_zmin[box - 1] + dz * np.arange(nz))[:, None, None]
        ay = (p.grd_ymin[box - 1] + dy * np.arange(ny))[None, :, None]
        ax = (p.grd_xmin[box - 1] + dx * np.arange(nx) - xdip)[None, None, :]
        ax, ay, az = np.broadcast_arrays(ax, ay, az)
        xp, yp, zp = ax, ay, az
        ar = np.sqrt(xp ** 2 + yp ** 2 + zp ** 2)
        bx0, by0, bz0 = _dipole(b0c, ax + xdip, ay, az, xdip)
        inside = ar < zero_b
        for q, b in enumerate((bx0, by0, bz0)):
            b = np.where(inside, 0.0, b)
            st.b0[q, box - 1] = b
        # corotation (3d_main.f90:1296-1308)
        rx, ry = ax * re_equiv, ay * re_equiv
        rd = np.sqrt(rx ** 2 + ry ** 2)
        vfrac = np.where(rd < r_rot, 1.0, ((2.0 * r_rot ** 2) / (r_rot ** 2 + rd ** 2)) ** 2)
        rvy, rvx = rx * v_rot * vfrac, -ry * v_rot * vfrac
        # plasma load (3d_main.f90:1310-1367)
        ar_iono = np.maximum(np.sqrt(xp ** 2 + ay ** 2 + 1.25 * zp ** 2), 0.0001)
        ra = ((ar_iono + 0.5 * r_inner) / (1.5 * r_inner)) ** (-alpha_e)
        zheight = np.maximum(1.0, (zp ** 2 + (1.5 * r_inner) ** 2) / (3.0 * r_inner) ** 2)
        ra = ra / zheight ** 2
        rho_iono = np.maximum(erho * ra, d_min)
        arho = np.maximum(rho_iono, d_min)
        vt = np.maximum(np.sqrt(rvy ** 2 + rvx ** 2), cs_inner)
        qrho = arho * rq / zheight
        qpres = arho * vt
        hrho = 0.05 * qrho * rh / rq
        hpres = 0.05 * qpres
        orho = qrho * ro / rq
        opres = qpres.copy()
        sp = {"q": [qrho, qrho * rvx, qrho * rvy, 0.0 * qrho, qpres],
              "h": [hrho, hrho * rvx, hrho * rvy, 0.0 * hrho, hpres],
              "o": [orho, orho * rvx, orho * rvy, 0.0 * orho, opres]}
        epres = (qpres + hpres + opres) / ti_te
        # solar wind (3d_main.f90:1466-1585)
        wind_bnd = r_rot / re_equiv
        ar0 = np.sqrt(ax ** 2 + ay ** 2 + az ** 2)
        full = (ar0 >= 1.5 * wind_bnd) & (ax < 0.0)
        ramp = (ar0 > wind_bnd) & (ar0 < 1.5 * wind_bnd) & (ax < 0.0)
        dfrac = np.where(full, 1.0, np.where(ramp, (ar0 - wind_bnd) / (0.5 * wind_bnd), 0.0))
        gamma = p.gamma
        cs_wind2 = p.spress * (gamma - 1.0) * gamma / p.srho
        qr = sp["q"][0] + p.srho * dfrac
        qpx = sp["q"][1] + p.spx * dfrac
        qpy = sp["q"][2] + p.spy * dfrac
        qpz = sp["q"][3] + p.spz * dfrac
        avx, avy, avz = qpx / qr, qpy / qr, qpz / qr
        apres = cs_wind2 * qr / gamma
        wind = dfrac > 0
        sp["q"] = [qr, qpx, qpy, qpz, np.where(wind, 0.5 * apres * dfrac + qpres, qpres)]
        epres = np.where(wind, 0.5 * apres / ti_te * dfrac + epres, epres)
        hr = hrho + p.srho * p.rho_frac * rh / rq * dfrac
        sp["h"] = [hr, np.where(wind, avx * hr, sp["h"][1]), np.where(wind, avy * hr, sp["h"][2]),
                   np.where(wind, avz * hr, 0.0 * hr),
                   hpres + 0.5 * p.spress * p.rho_frac * dfrac]
        orr = orho + p.srho * p.rho_frac * ro / rq * dfrac
        sp["o"] = [orr, np.where(wind, avx * orr, sp["o"][1]), np.where(wind, avy * orr, sp["o"][2]),
                   np.where(wind, avz * orr, 0.0 * orr),
                   opres + 0.5 * p.spress * p.rho_frac * dfrac]
        # speed clip (3d_main.f90:1589-1625)
        for key in ("q", "h", "o"):
            r, mx, my, mz, pr = sp[key]
            spd = np.sqrt((mx / r) ** 2 + (my / r) ** 2 + (mz / r) ** 2)
            bad = spd > 1.0
            sp[key] = [r, np.where(bad, 0.0, mx), np.where(bad, 0.0, my), np.where(bad, 0.0, mz), pr]
        # seeded perturbation of density and diagonal pressure
        for si, key in enumerate(("q", "h", "o")):
            r, mx, my, mz, pr = sp[key]
            nr = 1.0 + s.noise * rng.standard_normal(r.shape)
            base = 10 * si
            st.cur[base + 0, box - 1] = r * nr
            st.cur[base + 1, box - 1] = mx
            st.cur[base + 2, box - 1] = my
            st.cur[base + 3, box - 1] = mz
            for d in range(3):
                st.cur[base + 4 + d, box - 1] = pr * (1.0 + s.noise * rng.standard_normal(r.shape))
        st.cur[F_EPRES, box - 1] = epres
        # inner boundary lists for boxes <= mbndry (3d_main.f90:1374-1452)
        if box <= p.mbndry:
            sel = ar <= srf_b
            kk, jj, ii = np.nonzero(sel)          # k slowest: the reference's loop order
            for k, j, i in zip(kk, jj, ii):
                a = ar[k, j, i]
                key = "zero" if a < zero_b else ("mid" if a < mid_b else "srf")
                lists[key].append((box, i + 1, j + 1, k + 1))
                c = (slice(None), box - 1, k, j, i)
                vals = [st.cur[0, box - 1, k, j, i], st.cur[10, box - 1, k, j, i],
                        st.cur[20, box - 1, k, j, i], st.cur[4, box - 1, k, j, i],
                        st.cur[14, box - 1, k, j, i], st.cur[24, box - 1, k, j, i],
                        st.cur[F_EPRES, box - 1, k, j, i]]
                del c
                parms[key].append(vals)
    # ionospheric inflow densities drawn log-uniform per list entry
    for key in ("srf", "mid", "zero"):
        for v in parms[key]:
            f = math.exp(rng.uniform(math.log(s.iono_lo), math.log(s.iono_hi))) if s.iono_hi > s.iono_lo else 1.0
            v[0] *= f; v[1] *= f; v[2] *= f
    mb = p.mbndry
    for key in ("srf", "mid", "zero"):
        m = max(1, max([sum(1 for e in lists[key] if e[0] == b) for b in range(1, mb + 1)] + [0]))
        ij = np.zeros((m, 3, mb), np.int32)          # Fortran (mbndry,3,m)
        parm = np.zeros((m, 7, mb), np.float32)      # Fortran (mbndry,7,m)
        num = np.zeros(mb, np.int32)
        for e, v in zip(lists[key], parms[key]):
            b = e[0]
            n = num[b - 1]
            ij[n, :, b - 1] = e[1:]
            parm[n, :, b - 1] = v
            num[b - 1] = n + 1
        st.lists["ij" + key] = ij
        st.lists["parm_" + key] = parm
        st.lists["num" + key] = num
    # set_resist with b0 = 1 (sub_set_resist.f90:10-63; 3d_main.f90:1629)
    rst = st.resistive
    for key, val in (("zero", 1.0 / p.resist), ("mid", 0.5 / p.resist), ("srf", 0.125 / p.resist)):
        ij, num = st.lists["ij" + key], st.lists["num" + key]
        for b in range(1, mb + 1):
            for n in range(num[b - 1]):
                i, j, k = ij[n, :, b - 1]
                rst[b - 1, k - 1, j - 1, i - 1] = val
    return st


CONFIGS = {
    "small": dict(limit=30, n_grids=1, wind_adjust=1.0, divb_errlim=1.0e-6, divb_every=5),
    "nested": dict(limit=60, n_grids=5, wind_adjust=1.25, divb_errlim=1.0e-4, divb_every=10,
                   iono_lo=1.0, iono_hi=100.0),
    "tiny": dict(limit=8, n_grids=1, wind_adjust=1.0, divb_errlim=1.0e-4),
    "tiny2": dict(limit=8, n_grids=2, wind_adjust=1.0, divb_errlim=1.0e-4),
    "tiny3": dict(limit=8, n_grids=3, wind_adjust=1.25, divb_errlim=1.0e-4, iono_lo=1.0, iono_hi=100.0),
    "mid3": dict(limit=24, n_grids=3, wind_adjust=1.25, divb_errlim=1.0e-4, iono_lo=1.0, iono_hi=100.0),
}


def make_config(name: str = "small", **over) -> State:
    kw = dict(CONFIGS[name]) if name in CONFIGS else {}
    kw.update(over)
    return make_state(Setup(**kw))


ENSEMBLE_LIMITS = (60, 48, 40)   # boxes of 121x121x61, 97x97x49, 81x81x41


def ensemble_member(i: int, seed: int = 20261203, n_grids: int = 5, limits=ENSEMBLE_LIMITS, **over) -> State:
    """Member i of the upstream-condition ensemble: box size cycling through
    ``limits``, upstream wind drawn from the seed (n in [1,20] cm^-3, |v| in
    [300,800] km/s, IMF clock angle in [0, 2 pi), |B| in [2,15] nT), the
    nested-grid settings otherwise, and its own perturbation seed."""
    rng = np.random.default_rng([seed, i])
    wind = UpstreamWind(n_cm3=float(rng.uniform(1.0, 20.0)), speed_kms=float(rng.uniform(300.0, 800.0)),
                        clock_angle=float(rng.uniform(0.0, 2.0 * math.pi)), b_nT=float(rng.uniform(2.0, 15.0)))
    kw = dict(CONFIGS["nested"])
    kw.update(limit=limits[i % len(limits)], n_grids=n_grids, wind=wind, seed=seed + 1000 + i)
    kw.update(over)
    return make_state(Setup(**kw))


def perturbed(state: State, seed: int, scale: float = 1e-3) -> State:
    """A copy with every field multiplied by (1 + scale*N(0,1)) -- used to
    fill the old/wrk copies with data distinct from cur in kernel tests."""
    rng = np.random.default_rng(seed)
    o = state.copy()
    o.cur = (o.cur * (1.0 + scale * rng.standard_normal(o.cur.shape))).astype(np.float32)
    return o
