"""Whole-step parity: the step engine (g3m3_model_*) against the oracle's
restatement of the reference main loop (3d_main.f90:1925-3095) on nested,
sub-cycled boxes -- after 1 and after N main steps, host-loop launches and
CUDA-graph replay alike.  Bitwise: the engine performs the reference's FP32
operations in the reference's order."""
import ctypes

import numpy as np
import pytest

from _support import assert_same, rel_l2
from g3m3_gb300.state import make_config

pytestmark = pytest.mark.gpu


def run_pair(cfg, nsteps, graph=False, variant=None, autotune=False, **over):
    from oracle.oracle import OracleModel
    from g3m3_gb300.api import Context, Model
    st = make_config(cfg, **over)
    om = OracleModel(st, omp=True)
    om.init_steps()
    with Context() as ctx:
        m = Model(ctx, st)
        if variant is not None:
            m.set_variant(1, variant)
        if autotune:
            assert m.autotune() in range(8)
        m.init_steps()
        assert np.array_equal(m.times()[1], om.t_stepnew), (m.times()[1], om.t_stepnew)
        for _ in range(nsteps):
            assert om.main_step() == 0
        m.run(nsteps, graph=graph)
        g = m.state()
        t, tsn, cu = m.times()
        k, gl = m.stats()
        m.close()
    return om, g, (t, tsn, cu, k, gl)


@pytest.mark.parametrize("cfg", ["tiny", "tiny2", "tiny3"])
def test_one_step(cfg):
    om, g, (t, tsn, cu, k, gl) = run_pair(cfg, 1)
    for q in range(34):
        assert_same(g[q], om.cur[q], f"{cfg} field {q}")
    assert t == om.s.t
    assert np.array_equal(tsn, om.t_stepnew)
    assert cu == om.cell_updates
    assert k > 0


@pytest.mark.parametrize("cfg,n", [("tiny3", 6), ("mid3", 2)])
def test_n_steps(cfg, n):
    om, g, (t, tsn, cu, k, gl) = run_pair(cfg, n)
    for q in range(34):
        assert_same(g[q], om.cur[q], f"{cfg} field {q} after {n} steps")
    assert np.array_equal(tsn, om.t_stepnew)
    assert cu == om.cell_updates


def test_graph_replay_matches():
    om, g, (t, tsn, cu, k, gl) = run_pair("tiny3", 5, graph=True)
    assert gl == 5
    for q in range(34):
        assert_same(g[q], om.cur[q], f"graph field {q}")
    assert np.array_equal(tsn, om.t_stepnew)


def test_divb_all():
    """div B cleaning of every box + flanks_synced + bndry_corer; the CG
    dots are FP64 on the GPU, FP32 in the oracle: B compared with the FP64
    build (as close as the reference's FP32 solve), the rest bitwise."""
    from oracle.oracle import OracleModel
    from g3m3_gb300.api import Context, Model
    st = make_config("tiny3", divb_errlim=1e-5)
    rng = np.random.default_rng(5)
    for q in (31, 32, 33):
        st.cur[q] += (0.05 * rng.standard_normal(st.cur[q].shape)).astype(np.float32)
    om = OracleModel(st)
    om.divb_all()
    with Context() as ctx:
        m = Model(ctx, st)
        m.divb_all()
        g = m.state()
        m.close()
    import _divb_parity as D
    r8 = D.divb_all_r8(st)
    for q in (31, 32, 33):
        eg, er = D.rel(g[q], r8[q]), D.rel(om.cur[q], r8[q])
        assert eg <= D.SLACK * er + D.FLOOR, (q, eg, er)
    for q in range(31):
        assert_same(g[q], om.cur[q], f"divb untouched field {q}")


@pytest.mark.parametrize("host_fed", [False, True])
def test_divb_inside_steps(host_fed):
    """Two main steps with div B due after the second (all boxes solved side
    by side): the fields div B does not touch are the oracle's bits, B is as
    close to the FP64 build's as the reference's FP32 solve, host-fed
    (graph) or not."""
    import torch
    from oracle.oracle import OracleModel
    from g3m3_gb300.api import Context, Model
    st = make_config("mid3", divb_every=2, divb_errlim=1e-5)
    om = OracleModel(st, omp=True)     # its second main step ends with div B
    om.init_steps()
    o8 = OracleModel(st, omp=True, real8=True)
    o8.init_steps()
    for _ in range(2):
        assert om.main_step() == 0
        assert o8.main_step() == 0
    with Context() as ctx:
        m = Model(ctx, st)
        m.init_steps()
        if host_fed:
            buf = torch.empty(st.cur.shape, dtype=torch.float32, pin_memory=True).numpy()
            m.state(out=buf)
            for _ in range(2):
                m.step_host(buf, buf, graph=True)
            g = buf
        else:
            m.run(2, graph=False)
            g = m.state()
        m.close()
    for q in range(31):
        assert_same(g[q], om.cur[q], f"field {q}")
    import _divb_parity as D
    for q in (31, 32, 33):
        eg, er = D.rel(g[q], o8.cur[q]), D.rel(om.cur[q], o8.cur[q])
        assert eg <= D.SLACK * er + D.FLOOR, (q, eg, er)


@pytest.mark.parametrize("cfg,nsteps,variant", [("tiny3", 2, 1), ("mid3", 2, 1), ("tiny3", 2, 2), ("mid3", 2, 2),
                                               ("mid3", 2, 3), ("tiny3", 2, 4), ("mid3", 2, 4), ("tiny3", 2, 5),
                                               ("mid3", 2, 5), ("tiny3", 2, 6), ("mid3", 2, 6), ("tiny3", 2, 7),
                                               ("mid3", 2, 7)])
def test_fcsmooth_variants(cfg, nsteps, variant):
    """The 32x16-tile and the two-field packed FP32x2 flux corrections
    (planes staged through registers with two barriers per plane, 2-3;
    copied asynchronously with one barrier per plane, 4-7)
    give the same bits as the oracle."""
    om, g, (t, tsn, cu, k, gl) = run_pair(cfg, nsteps, variant=variant)
    for q in range(34):
        assert_same(g[q], om.cur[q], f"{cfg} field {q}")
    assert np.array_equal(tsn, om.t_stepnew)


@pytest.mark.parametrize("limit", [22, 14])
@pytest.mark.parametrize("variant", range(8))
def test_ragged_grids_every_variant(limit, variant):
    """Three nested boxes of 45x45x23 or 29x29x15 (remainders 13 and 29
    against the 32-wide tile rows, 5 and 13 against 8- and 16-row tiles,
    where the other grids leave 1): two main steps with each flux-correction
    form, every kernel of the step on ragged tiles, bitwise."""
    om, g, (t, tsn, cu, k, gl) = run_pair("tiny3", 2, variant=variant, limit=limit)
    for q in range(34):
        assert_same(g[q], om.cur[q], f"limit {limit} variant {variant} field {q}")
    assert np.array_equal(tsn, om.t_stepnew)
    assert cu == om.cell_updates


def test_capture_after_second_occurrence():
    """With g3m3_model_set_capture_after(2) a step plan runs host-launched
    at its first occurrence and from a graph afterwards: the same bits."""
    from oracle.oracle import OracleModel
    from g3m3_gb300.api import Context, Model
    st = make_config("tiny3")
    om = OracleModel(st, omp=True)
    om.init_steps()
    for _ in range(6):
        assert om.main_step() == 0
    with Context() as ctx:
        m = Model(ctx, st)
        m.set_capture_after(2)
        m.init_steps()
        m.run(6, graph=True)
        g = m.state()
        k, gl = m.stats()
        m.close()
    assert 0 < gl < 6, gl
    for q in range(34):
        assert_same(g[q], om.cur[q], f"field {q}")


@pytest.mark.parametrize("graph,pin", [(False, True), (True, True), (False, False)])
def test_step_host(graph, pin):
    """Host-fed main steps (per-box uploads overlapping the step, result
    read back, fed in again) give the oracle's bits after two steps, with
    pinned buffers (graph or host launches) and with pageable ones."""
    import torch
    from oracle.oracle import OracleModel
    from g3m3_gb300.api import Context, Model
    st = make_config("mid3")
    om = OracleModel(st, omp=True)
    om.init_steps()
    for _ in range(2):
        assert om.main_step() == 0
    with Context() as ctx:
        m = Model(ctx, st)
        m.init_steps()
        if pin:
            buf_t = torch.empty(st.cur.shape, dtype=torch.float32, pin_memory=True)
            buf = buf_t.numpy()
        else:
            buf = np.empty(st.cur.shape, np.float32)
        m.state(out=buf)   # the state init_steps prepared
        for _ in range(2):
            m.step_host(buf, buf, graph=graph)
        tsn = m.times()[1]
        m.close()
    for q in range(34):
        assert_same(buf[q], om.cur[q], f"field {q}")
    assert np.array_equal(tsn, om.t_stepnew)


def test_autotuned_steps():
    """Autotuning picks a tile shape on scratch copies: the state it leaves
    and the steps after it are the oracle's."""
    om, g, (t, tsn, cu, k, gl) = run_pair("mid3", 2, graph=True, autotune=True)
    for q in range(34):
        assert_same(g[q], om.cur[q], f"mid3 field {q}")
    assert np.array_equal(tsn, om.t_stepnew)


@pytest.mark.parametrize("graph", [False, True])
def test_flux_history(graph):
    """The engine records flux_counter of every box at the start of each
    main step; the history matches the oracle applied to the oracle's state
    at the same points."""
    import ctypes
    from oracle import oracle
    from oracle.oracle import OracleModel
    from g3m3_gb300.api import Context, Model
    st = make_config("tiny3")
    p = st.params
    scale = np.array([1.0e3 * (b + 1) for b in range(p.n_grids)], np.float32)
    om = OracleModel(st, omp=True)
    om.init_steps()
    nsteps = 3
    want = np.zeros((nsteps, p.n_grids, 6), np.float32)
    for n in range(nsteps):
        for b in range(1, p.n_grids + 1):
            oo = [ctypes.c_float() for _ in range(6)]
            moms = [np.ascontiguousarray(om.cur[10 * s + 1 + q]) for s in range(3) for q in range(3)]
            oracle.call("flux_counter", *moms, p.nx, p.ny, p.nz, p.n_grids, b, p.rmassq, p.rmassh, p.rmasso,
                        float(scale[b - 1]), *[ctypes.addressof(x) for x in oo])
            want[n, b - 1] = [x.value for x in oo]
        assert om.main_step() == 0
    with Context() as ctx:
        m = Model(ctx, st)
        m.record_fluxes(scale, 8)
        m.init_steps()
        m.run(nsteps, graph=graph)
        got = m.fluxes()
        m.close()
    assert got.shape == want.shape
    assert_same(got, want, "flux history")


def _oracle_sample(field, xyz, p):
    """findgrid + trilin_interp of the oracle at one point (field: (n_grids, nz, ny, nx))."""
    import ctypes
    from oracle import oracle
    gmin = np.array([[p.grd_xmin[b], p.grd_ymin[b], p.grd_zmin[b]] for b in range(p.n_grids)], np.float32)
    gmax = np.array([[p.grd_xmax[b], p.grd_ymax[b], p.grd_zmax[b]] for b in range(p.n_grids)], np.float32)
    xs = np.array(p.xspac[: p.n_grids], np.float32)
    gp = (ctypes.c_int * 4)()
    pt = np.ascontiguousarray(xyz, np.float32)
    oracle.call("findgrid", pt, p.n_grids, gmin, gmax, xs, gp, p.re_equiv)
    i, j, k, b = gp[0], gp[1], gp[2], gp[3]
    cube = np.zeros((2, 3), np.float32)
    for a in range(3):
        cube[0, a] = (gmin[b - 1, a] + np.float32(gp[a] - 1) * xs[b - 1]) * np.float32(p.re_equiv)
        cube[1, a] = cube[0, a] + xs[b - 1] * np.float32(p.re_equiv)
    q = np.ascontiguousarray(field[b - 1, k - 1:k + 1, j - 1:j + 1, i - 1:i + 1])
    v = ctypes.c_float()
    oracle.call("trilin_interp", pt, cube, q, ctypes.addressof(v))
    return v.value


@pytest.mark.parametrize("graph", [False, True])
def test_craft_records(graph):
    """Virtual spacecraft recorded on the device at the end of each main
    step: positions interpolated along the trajectories (FP32, as linterp),
    values equal to the oracle's findgrid + trilin_interp on the model's
    state of that step; a craft outside its time range records NaN."""
    from g3m3_gb300.api import Context, Model
    st = make_config("tiny3")
    p = st.params
    f32 = np.float32
    # three trajectories in planet radii: through the inner box, across the
    # middle box, and one that starts only after the second step
    tr = [np.array([[-2.0, -1.5, 0.3, 0.0], [2.5, 1.0, -0.4, 50.0]], np.float32),
          np.array([[5.0, -4.0, 1.0, 0.0], [0.0, 0.0, 0.0, 1.0], [-6.0, 3.0, -1.0, 60.0]], np.float32),
          np.array([[1.0, 1.0, 0.5, 1e6], [1.5, 1.0, 0.5, 2e6]], np.float32)]
    npts = np.array([len(t) for t in tr], np.int32)
    traj = np.ascontiguousarray(np.concatenate(tr).reshape(-1), np.float32)
    fields = np.array([31, 32, 33, 0], np.int32)
    nsteps = 3
    states, times = [], []
    with Context() as ctx:
        m = Model(ctx, st)
        ctx.check(ctx.L.g3m3_model_record_craft(m.h, len(tr), npts.ctypes.data, traj.ctypes.data, len(fields),
                                                fields.ctypes.data, 8))
        m.init_steps()
        for _ in range(nsteps):
            m.run(1, graph=graph)
            states.append(m.state())
            times.append(m.times()[0])
        rec = np.zeros((8, len(tr), 4 + len(fields)), np.float32)
        n = ctypes.c_int()
        ctx.check(ctx.L.g3m3_model_craft_records(m.h, rec.ctypes.data, ctypes.byref(n)))
        m.close()
    assert n.value == nsteps
    for s_ in range(nsteps):
        t = f32(times[s_])
        for c, T in enumerate(tr):
            r = rec[s_, c]
            assert r[0] == t
            seg = [i for i in range(len(T) - 1) if T[i, 3] <= t < T[i + 1, 3]]
            if not seg:
                assert np.isnan(r[1:]).all()
                continue
            x1, x2 = T[seg[0]], T[seg[0] + 1]
            xyz = np.array([x1[q] + (x2[q] - x1[q]) / (x2[3] - x1[3]) * (t - x1[3]) for q in range(3)], np.float32)
            assert np.array_equal(r[1:4], xyz), (s_, c, r[1:4], xyz)
            for fi, fq in enumerate(fields):
                want = _oracle_sample(states[s_][fq], xyz, p)
                assert r[4 + fi] == want, (s_, c, fq, r[4 + fi], want)


@pytest.mark.parametrize("plane", [0, 1, 2])
def test_graphing_planes(plane):
    """The graphing plane of box 1 after a step equals the oracle's calcur,
    total B, fnd_evel, BandE and fnd_pres of the same state, cut the same
    way."""
    from oracle import oracle
    from g3m3_gb300.api import Context, Model
    st = make_config("tiny3")
    p = st.params
    box = 1
    index = {0: p.nz // 2 + 1, 1: p.ny // 2 + 1, 2: p.nx // 2 + 1}[plane]
    na = p.ny if plane == 0 else p.nz
    nb = p.ny if plane == 2 else p.nx
    with Context() as ctx:
        m = Model(ctx, st)
        m.init_steps()
        m.run(1)
        s = m.state()
        got = np.zeros((32, na, nb), np.float32)
        ctx.check(ctx.L.g3m3_model_graphing(m.h, box, plane, index, got.ctypes.data))
        m.close()
    F = [np.ascontiguousarray(s[q]) for q in range(34)]
    b0 = [np.ascontiguousarray(st.b0[q]) for q in range(3)]
    dims = [p.nx, p.ny, p.nz, p.n_grids, box]
    rx = float(p.xspac[box - 1])
    box3 = (p.nz, p.ny, p.nx)
    z = lambda: np.zeros(box3, np.float32)
    cur = [z(), z(), z()]
    oracle.call("calcur", F[31], F[32], F[33], *dims, *cur, rx, rx, rx)
    bs = [z(), z(), z()]
    btot = z()
    oracle.call("total_b", F[31], F[32], F[33], *b0, *dims, p.smallbit, *bs, btot)
    ev, tv = [z(), z(), z()], [z(), z(), z()]
    sp = []
    for q in (0, 10, 20):
        sp += [F[q + 1], F[q + 2], F[q + 3], F[q]]
    oracle.call("fnd_evel", *sp, *cur, *ev, *tv, *dims, p.rmassq, p.rmassh, p.rmasso, p.reynolds)
    L = st.lists
    ef = [z(), z(), z()]
    oracle.call("bande", *ef, *bs, *cur, *ev, btot, F[30], F[0], F[10], F[20], np.ascontiguousarray(st.resistive),
                p.resist, p.reynolds, *dims, p.rmassq, p.rmassh, p.rmasso, L["ijmid"], L["nummid"], L["ijzero"],
                p.mbndry, L["numzero"], L["ijmid"].shape[0], L["ijzero"].shape[0], rx, rx, rx)
    want = [bs[0], bs[1], bs[2], btot, ef[0], ef[1], ef[2], cur[0], cur[1], cur[2]]
    for q in (0, 10, 20):
        r = np.maximum(F[q][box - 1], np.float32(p.smallbit))
        v = [(F[q + 1 + c][box - 1] / r).astype(np.float32) for c in range(3)]
        par, perp, cross = (np.zeros_like(F[0]) for _ in range(3))
        oracle.call("fnd_pres", F[q + 4], F[q + 5], F[q + 6], F[q + 7], F[q + 8], F[q + 9], par, perp, cross,
                    *[np.ascontiguousarray(x) for x in v], *bs, *dims)
        want += v + [par[box - 1], perp[box - 1], cross[box - 1], F[q][box - 1]]
    want.append(F[30][box - 1])
    for qi, w in enumerate(want):
        w = w[box - 1] if w.ndim == 4 else w
        cutw = w[index - 1, :, :] if plane == 0 else (w[:, index - 1, :] if plane == 1 else w[:, :, index - 1])
        assert_same(got[qi], cutw, f"plane {plane} quantity {qi}")
