"""The per-cell arithmetic of the step's kernels, stated for the reverse-mode
generator (adgen.py), which writes csrc/adj_cells.cuh from it.

Each function restates, operation for operation, what one thread of the
forward kernel computes for one cell; it is parsed, not run.  Inputs are the
values the thread loads (stencil points named by suffix: c the cell, xp/xm
its +x/-x neighbours, and so on), parameters are per-launch or per-cell
constants that are not differentiated, outputs are what it stores.
"""
from .adgen import cell

P7 = ["c", "xp", "xm", "yp", "ym", "zp", "zm"]
PUSH_FIELDS = ["rho", "px", "py", "pz", "xx", "yy", "zz", "xy", "xz", "yz", "bx", "by", "bz"]
PUSH_STENCIL = [f"{f}_{p}" for f in PUSH_FIELDS for p in P7]
PUSH_CENTRE = [f"old{i}" for i in range(10)] + ["bt", "e0", "e1", "e2", "tvx", "tvy", "tvz"]
PUSH_PARAMS = ["delt", "dxt", "dyt", "dzt", "rmass", "rey", "bmax", "grav", "rr2", "radius", "ax", "ay", "az"]
PUSH_OUT = ["o_rho", "o_px", "o_py", "o_pz", "o_xx", "o_yy", "o_zz", "o_xy", "o_xz", "o_yz"]


@cell(inputs=PUSH_STENCIL + PUSH_CENTRE, params=PUSH_PARAMS, outputs=PUSH_OUT)
def push_ion_cell():
    """push_ion at one interior cell (sub_push_ion.f90:107-356; k_push_tiled.cu push_cell).
    Source state (rho, p, pressure tensor) and bs on the 7-point stencil;
    old state, btot, E and the mass-averaged velocity tv at the cell."""
    # species velocity v = p / max(rho, 1e-6) at the stencil points (:67-81)
    r_c = amax1(rho_c, 1e-06)
    vx_c = px_c / r_c
    vy_c = py_c / r_c
    vz_c = pz_c / r_c
    r_xp = amax1(rho_xp, 1e-06)
    vx_xp = px_xp / r_xp
    vy_xp = py_xp / r_xp
    vz_xp = pz_xp / r_xp
    r_xm = amax1(rho_xm, 1e-06)
    vx_xm = px_xm / r_xm
    vy_xm = py_xm / r_xm
    vz_xm = pz_xm / r_xm
    r_yp = amax1(rho_yp, 1e-06)
    vx_yp = px_yp / r_yp
    vy_yp = py_yp / r_yp
    vz_yp = pz_yp / r_yp
    r_ym = amax1(rho_ym, 1e-06)
    vx_ym = px_ym / r_ym
    vy_ym = py_ym / r_ym
    vz_ym = pz_ym / r_ym
    r_zp = amax1(rho_zp, 1e-06)
    vx_zp = px_zp / r_zp
    vy_zp = py_zp / r_zp
    vz_zp = pz_zp / r_zp
    r_zm = amax1(rho_zm, 1e-06)
    vx_zm = px_zm / r_zm
    vy_zm = py_zm / r_zm
    vz_zm = pz_zm / r_zm
    # continuity and momentum flux (sub_push_ion.f90:107-134)
    o_rho = old0 - delt * (((px_xp - px_xm) / dxt + (py_yp - py_ym) / dyt) + (pz_zp - pz_zm) / dzt)
    fd1 = ((px_xp * vx_xp - px_xm * vx_xm) / dxt + (px_yp * vy_yp - px_ym * vy_ym) / dyt) + (px_zp * vz_zp - px_zm * vz_zm) / dzt
    fd2 = ((py_xp * vx_xp - py_xm * vx_xm) / dxt + (py_yp * vy_yp - py_ym * vy_ym) / dyt) + (py_zp * vz_zp - py_zm * vz_zm) / dzt
    fd3 = ((pz_xp * vx_xp - pz_xm * vx_xm) / dxt + (pz_yp * vy_yp - pz_ym * vy_ym) / dyt) + (pz_zp * vz_zp - pz_zm * vz_zm) / dzt
    fd4 = ((xx_xp * vx_xp - xx_xm * vx_xm) / dxt + (xx_yp * vy_yp - xx_ym * vy_ym) / dyt) + (xx_zp * vz_zp - xx_zm * vz_zm) / dzt
    fd5 = ((yy_xp * vx_xp - yy_xm * vx_xm) / dxt + (yy_yp * vy_yp - yy_ym * vy_ym) / dyt) + (yy_zp * vz_zp - yy_zm * vz_zm) / dzt
    fd6 = ((zz_xp * vx_xp - zz_xm * vx_xm) / dxt + (zz_yp * vy_yp - zz_ym * vy_ym) / dyt) + (zz_zp * vz_zp - zz_zm * vz_zm) / dzt
    fd7 = ((xy_xp * vx_xp - xy_xm * vx_xm) / dxt + (xy_yp * vy_yp - xy_ym * vy_ym) / dyt) + (xy_zp * vz_zp - xy_zm * vz_zm) / dzt
    fd8 = ((xz_xp * vx_xp - xz_xm * vx_xm) / dxt + (xz_yp * vy_yp - xz_ym * vy_ym) / dyt) + (xz_zp * vz_zp - xz_zm * vz_zm) / dzt
    fd9 = ((yz_xp * vx_xp - yz_xm * vx_xm) / dxt + (yz_yp * vy_yp - yz_ym * vy_ym) / dyt) + (yz_zp * vz_zp - yz_zm * vz_zm) / dzt
    aqpx = old1 - delt * fd1
    aqpy = old2 - delt * fd2
    aqpz = old3 - delt * fd3
    # E + v x B and the skin-depth Hall terms (:138-188)
    weight = amax1(1.0, bt / bmax)
    skin_depth = rey / weight
    tcx = tvy * bz_c - tvz * by_c
    tcy = -(tvx * bz_c - tvz * bx_c)
    tcz = tvx * by_c - tvy * bx_c
    qcx = vy_c * bz_c - vz_c * by_c
    qcy = -(vx_c * bz_c - vz_c * bx_c)
    qcz = vx_c * by_c - vy_c * bx_c
    gpx = (xx_xp - xx_xm) / dxt + (xy_yp - xy_ym) / dxt + (xz_zp - xz_zm) / dxt
    gpy = (xy_xp - xy_xm) / dxt + (yy_yp - yy_ym) / dyt + (yz_zp - yz_zm) / dxt
    gpz = (xz_xp - xz_xm) / dxt + (yz_yp - yz_ym) / dyt + (zz_zp - zz_zm) / dzt
    dex = (e0 + tcx) * rey
    dey = (e1 + tcy) * rey
    dez = (e2 + tcz) * rey
    dvx = (qcx - tcx) * skin_depth
    dvy = (qcy - tcy) * skin_depth
    dvz = (qcz - tcz) * skin_depth
    qden = rho_c / rmass
    npx = aqpx + delt * (qden * (dex + dvx) - gpx)
    npy = aqpy + delt * (qden * (dey + dvy) - gpy)
    npz = aqpz + delt * (qden * (dez + dvz) - gpz)
    # gravity (:202-206); ax, ay, az, rr2 = (re_equiv * radius)**2 and radius are per-cell constants
    g = delt * rho_c * grav / rr2
    o_px = npx - g * ax / radius
    o_py = npy - g * ay / radius
    o_pz = npz - g * az / radius
    # diagonal pressures (:210-238) with the 12-point smoothed B gyro term (:242-281)
    t2 = 2.0 * delt
    px_ = old4 - delt * fd4 - t2 * xx_c * (vx_xp - vx_xm) / dxt
    py_ = old5 - delt * fd5 - t2 * yy_c * (vy_yp - vy_ym) / dyt
    pz_ = old6 - delt * fd6 - t2 * zz_c * (vz_zp - vz_zm) / dzt
    abx = (6.0 * bx_c + bx_xp + bx_xm + bx_yp + bx_ym + bx_zp + bx_zm) / 12.0
    aby = (6.0 * by_c + by_xp + by_xm + by_yp + by_ym + by_zp + by_zm) / 12.0
    abz = (6.0 * bz_c + bz_xp + bz_xm + bz_yp + bz_ym + bz_zp + bz_zm) / 12.0
    bmag = sqrt(abx * abx + aby * aby + abz * abz)
    skin = rey * (bmax / bmag) if bmag > bmax else rey
    gy2 = t2 * skin / rmass
    o_xx = px_ - t2 * xy_c * (vx_yp - vx_ym) / dyt - t2 * xz_c * (vx_zp - vx_zm) / dzt + gy2 * (xy_c * abz - xz_c * aby)
    o_yy = py_ - t2 * xy_c * (vy_xp - vy_xm) / dxt - t2 * yz_c * (vy_zp - vy_zm) / dzt + gy2 * (yz_c * abx - xy_c * abz)
    o_zz = pz_ - t2 * xz_c * (vz_xp - vz_xm) / dxt - t2 * yz_c * (vz_yp - vz_ym) / dyt + gy2 * (xz_c * aby - yz_c * abx)
    # off-diagonal pressures (:285-356)
    gy1 = delt * skin / rmass
    o_xy = (old7 - delt * fd7 - delt * xy_c * ((vx_xp - vx_xm) / dxt + (vy_yp - vy_ym) / dyt) - delt * yy_c * (vx_yp - vx_ym) / dyt - delt * xx_c * (vy_xp - vy_xm) / dxt - delt * yz_c * (vx_zp - vx_zm) / dzt - delt * xz_c * (vy_zp - vy_zm) / dzt + gy1 * (abz * (yy_c - xx_c) - aby * yz_c + abx * xz_c))
    o_xz = (old8 - delt * fd8 - delt * xz_c * ((vx_xp - vx_xm) / dxt + (vz_zp - vz_zm) / dzt) - delt * zz_c * (vx_zp - vx_zm) / dzt - delt * xx_c * (vz_xp - vz_xm) / dxt - delt * yz_c * (vx_yp - vx_ym) / dyt - delt * xy_c * (vz_yp - vz_ym) / dyt + gy1 * (aby * (xx_c - zz_c) - abx * xy_c + abz * yz_c))
    o_yz = (old9 - delt * fd9 - delt * yz_c * ((vy_yp - vy_ym) / dyt + (vz_zp - vz_zm) / dzt) - delt * yy_c * (vz_yp - vz_ym) / dyt - delt * zz_c * (vy_zp - vy_zm) / dzt - delt * xy_c * (vz_xp - vz_xm) / dxt - delt * xz_c * (vy_xp - vy_xm) / dxt + gy1 * (abx * (zz_c - yy_c) - abz * xz_c + aby * xy_c))
    return o_rho, o_px, o_py, o_pz, o_xx, o_yy, o_zz, o_xy, o_xz, o_yz


@cell(inputs=["w_xp", "w_xm", "w_yp", "w_ym", "w_zp", "w_zm", "evx_xp", "evx_xm", "evy_yp", "evy_ym",
              "evz_zp", "evz_zm", "evx_c", "evy_c", "evz_c", "old"],
      params=["delt", "gamma", "gamma1", "dxt", "dyt", "dzt"], outputs=["e"])
def push_elec_cell():
    """push_elec at one interior cell (sub_push_elec.f90:37-47): w is the
    source pressure (argument 1), ev the electron velocity."""
    gx = (w_xp - w_xm) / dxt
    gy = (w_yp - w_ym) / dyt
    gz = (w_zp - w_zm) / dzt
    e0 = old - delt * gamma * (((w_xp * evx_xp - w_xm * evx_xm) / dxt + (w_yp * evy_yp - w_ym * evy_ym) / dyt)
                               + (w_zp * evz_zp - w_zm * evz_zm) / dzt)
    e = e0 + delt * gamma1 * (evx_c * gx + evy_c * gy + evz_c * gz)
    return e


@cell(inputs=["obx", "oby", "obz", "ex_yp", "ex_ym", "ex_zp", "ex_zm", "ey_xp", "ey_xm", "ey_zp", "ey_zm",
              "ez_xp", "ez_xm", "ez_yp", "ez_ym"],
      params=["delt", "dxt", "dyt", "dzt"], outputs=["bx", "by", "bz"])
def push_bfld_cell():
    """push_bfld at one interior cell (sub_push_bfld.f90:20-47): B = B_old -/+ dt curl E."""
    bx = obx - delt * ((ez_yp - ez_ym) / dyt - (ey_zp - ey_zm) / dzt)
    by = oby + delt * ((ez_xp - ez_xm) / dxt - (ex_zp - ex_zm) / dzt)
    bz = obz - delt * ((ey_xp - ey_xm) / dxt - (ex_yp - ex_ym) / dyt)
    return bx, by, bz


@cell(inputs=["bx_yp", "bx_ym", "bx_zp", "bx_zm", "by_xp", "by_xm", "by_zp", "by_zm",
              "bz_xp", "bz_xm", "bz_yp", "bz_ym"],
      params=["dxt", "dyt", "dzt"], outputs=["cx", "cy", "cz"])
def curl_cell():
    """calcur at one interior point (sub_calcur.f90:30-44); faces, edges and
    corners take the value of the clamped interior point."""
    cx = (bz_yp - bz_ym) / dyt - (by_zp - by_zm) / dzt
    cy = (bx_zp - bx_zm) / dzt - (bz_xp - bz_xm) / dxt
    cz = (by_xp - by_xm) / dxt - (bx_yp - bx_ym) / dyt
    return cx, cy, cz


@cell(inputs=["bx", "by", "bz"], params=["b0x", "b0y", "b0z", "smallbit"], outputs=["sx", "sy", "sz", "bt"])
def total_b_cell():
    """bs = b0 + b, btot = max(|bs|, smallbit) (3d_main.f90:2248-2254)."""
    sx = b0x + bx
    sy = b0y + by
    sz = b0z + bz
    bt = amax1(sqrt(sx * sx + sy * sy + sz * sz), smallbit)
    return sx, sy, sz, bt


@cell(inputs=["rq", "rh", "ro", "qpx", "qpy", "qpz", "hpx", "hpy", "hpz", "opx", "opy", "opz", "jx", "jy", "jz"],
      params=["mq", "mh", "mo", "reynolds"], outputs=["evx", "evy", "evz", "tvx", "tvy", "tvz"])
def evel_cell():
    """fnd_evel at one cell (sub_fnd_evel.f90:20-54): tv = sum p / sum rho,
    ev = tv - J / (number density) / reynolds."""
    tden = rq + rh + ro
    tvx = (qpx + hpx + opx) / tden
    tvy = (qpy + hpy + opy) / tden
    tvz = (qpz + hpz + opz) / tden
    qden = (rq + 1e-06) / mq
    hden = (rh + 1e-06) / mh
    oden = (ro + 1e-06) / mo
    tot = qden + hden + oden
    evx = tvx - jx / tot / reynolds
    evy = tvy - jy / tot / reynolds
    evz = tvz - jz / tot / reynolds
    return evx, evy, evz, tvx, tvy, tvz


@cell(inputs=["rq", "rh", "ro", "qpx", "qpy", "qpz", "hpx", "hpy", "hpz", "opx", "opy", "opz"],
      params=[], outputs=["tvx", "tvy", "tvz"])
def vtot_cell():
    """fnd_vtot at one cell (sub_fnd_vtot.f90:20-38)."""
    tden = rq + rh + ro
    tvx = (qpx + hpx + opx) / tden
    tvy = (qpy + hpy + opy) / tden
    tvz = (qpz + hpz + opz) / tden
    return tvx, tvy, tvz


@cell(inputs=["evx", "evy", "evz", "bsx", "bsy", "bsz", "rq", "rh", "ro",
              "ep_xp", "ep_xm", "ep_yp", "ep_ym", "ep_zp", "ep_zm", "jx", "jy", "jz"],
      params=["mq", "mh", "mo", "reynolds", "dxt", "dyt", "dzt", "rst"], outputs=["ex", "ey", "ez"])
def bande_cell():
    """BandE at one interior point (sub_BandE.f90:32-116): -ev x bs, the
    electron pressure gradient, and the resistive term rst J / n (zero where
    rst is zero); faces take the value of the clamped interior point."""
    e1x = -(evy * bsz - evz * bsy)
    e1y = -(evz * bsx - evx * bsz)
    e1z = -(evx * bsy - evy * bsx)
    arho = (rq / mq + rh / mh + ro / mo) * reynolds
    e2x = e1x - (ep_xp - ep_xm) / dxt / arho
    e2y = e1y - (ep_yp - ep_ym) / dyt / arho
    e2z = e1z - (ep_zp - ep_zm) / dzt / arho
    eden = rq / mq + rh / mh + ro / mo
    ex = e2x + rst * jx / eden
    ey = e2y + rst * jy / eden
    ez = e2z + rst * jz / eden
    return ex, ey, ez


@cell(inputs=["rho_c", "rho_xp", "rho_xm", "rho_yp", "rho_ym", "rho_zp", "rho_zm",
              "px_c", "px_xp", "px_xm", "py_c", "py_yp", "py_ym", "pz_c", "pz_zp", "pz_zm"],
      params=["vfloor"], outputs=["uxp", "uxm", "uyp", "uym", "uzp", "uzm"])
def lap_speed_cell():
    """The Lapidus velocity jumps of one species at one cell: v = p /
    max(rho, floor) (3d_main.f90:2698-2703), |v(+1) - v(0)|, |v(0) - v(-1)|
    per axis (sub_lap_plasma.f90:33-47)."""
    r0 = amax1(rho_c, vfloor)
    vx0 = px_c / r0
    vy0 = py_c / r0
    vz0 = pz_c / r0
    vxp = px_xp / amax1(rho_xp, vfloor)
    vxm = px_xm / amax1(rho_xm, vfloor)
    vyp = py_yp / amax1(rho_yp, vfloor)
    vym = py_ym / amax1(rho_ym, vfloor)
    vzp = pz_zp / amax1(rho_zp, vfloor)
    vzm = pz_zm / amax1(rho_zm, vfloor)
    uxp = fabs(vxp - vx0)
    uxm = fabs(vx0 - vxm)
    uyp = fabs(vyp - vy0)
    uym = fabs(vy0 - vym)
    uzp = fabs(vzp - vz0)
    uzm = fabs(vz0 - vzm)
    return uxp, uxm, uyp, uym, uzp, uzm


@cell(inputs=["vx_c", "vx_xp", "vx_xm", "vy_c", "vy_yp", "vy_ym", "vz_c", "vz_zp", "vz_zm"],
      params=[], outputs=["uxp", "uxm", "uyp", "uym", "uzp", "uzm"])
def lap_jump_cell():
    """The Lapidus velocity jumps from a given velocity field (tv, for
    lap_elec and lap_bfld, sub_lap_elec.f90:20-32)."""
    uxp = fabs(vx_xp - vx_c)
    uxm = fabs(vx_c - vx_xm)
    uyp = fabs(vy_yp - vy_c)
    uym = fabs(vy_c - vy_ym)
    uzp = fabs(vz_zp - vz_c)
    uzm = fabs(vz_c - vz_zm)
    return uxp, uxm, uyp, uym, uzp, uzm


@cell(inputs=["f_c", "f_xp", "f_xm", "f_yp", "f_ym", "f_zp", "f_zm", "uxp", "uxm", "uyp", "uym", "uzp", "uzm"],
      params=["chi", "delt"], outputs=["out"])
def lap_field_cell():
    """Lapidus smoothing of one field at one interior cell
    (sub_lap_plasma.f90:50-140)."""
    out = f_c + chi * (delt * (uxp * (f_xp - f_c) - uxm * (f_c - f_xm))
                       + delt * (uyp * (f_yp - f_c) - uym * (f_c - f_ym))
                       + delt * (uzp * (f_zp - f_c) - uzm * (f_c - f_zm)))
    return out


@cell(inputs=["pm1", "p0", "pa", "pb", "w0", "wp"], params=["chi"], outputs=["fn"])
def fcs_flux_cell():
    """The flux-correction limiter flux at one face (sub_fcsmooth.f90:87-239):
    with the diffused field P1 and the undiffused w, dw = w(m+1) - w(m),
    fn = s max(0, min(s (P1(m) - P1(m-1)), chi |dw|, s (P1(q+1) - P1(q))))
    where s = sign(dw) and q = min(m+1, n-1)."""
    dw = wp - w0
    sg = 1.0 if dw >= 0.0 else -1.0
    d1m = p0 - pm1
    d1p = pb - pa
    fn = sg * amax1(0.0, amin1(amin1(sg * d1m, chi * fabs(dw)), sg * d1p))
    return fn
