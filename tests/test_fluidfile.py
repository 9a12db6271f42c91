"""Fluid (restart) files: the library writes the reference's record layout
(3d_main.f90:3305-3349) byte for byte as an independent numpy writer does,
reads it back, and a model restarted from its own file continues with the
same bits."""
import ctypes
import struct

import numpy as np
import pytest

from _support import assert_same
from g3m3_gb300.params import NFIELDS

FILE_ORDER = list(range(30)) + [31, 32, 33, 30]   # file records: species, bx, by, bz, epres


def numpy_fluid_bytes(t, state, b0, lists, mb):
    """The format written out independently of the library."""
    out = bytearray()

    def rec(*parts):
        body = b"".join(np.ascontiguousarray(p).tobytes() for p in parts)
        out.extend(struct.pack("<i", len(body)) + body + struct.pack("<i", len(body)))

    rec(np.array([t], np.float64))
    for q in FILE_ORDER:
        rec(state[q])
    for q in range(3):
        rec(b0[q])
    rec(lists["parm_srf"], lists["parm_mid"], lists["parm_zero"], lists["ijzero"], lists["numzero"],
        lists["ijmid"], lists["nummid"], lists["ijsrf"], lists["numsrf"])
    return bytes(out)


def _write_args(p, t, state, b0, li):
    from g3m3_gb300.api import addr
    return [ctypes.byref(p), ctypes.c_double(t), addr(state), addr(b0),
            addr(li["parm_srf"]), addr(li["parm_mid"]), addr(li["parm_zero"]),
            addr(li["ijzero"]), addr(li["numzero"]), addr(li["ijmid"]), addr(li["nummid"]),
            addr(li["ijsrf"]), addr(li["numsrf"]),
            li["ijsrf"].shape[0], li["ijmid"].shape[0], li["ijzero"].shape[0]]


def test_fluid_file_layout_and_round_trip(tmp_path):
    from g3m3_gb300 import _lib
    from g3m3_gb300.state import make_config
    L = _lib.load()
    st = make_config("tiny2")
    p = st.params
    li = {k: np.ascontiguousarray(v) for k, v in st.lists.items()}
    t = 123.456789012345
    path = str(tmp_path / "fluid11")
    rc = L.g3m3_fluid_write(None, path.encode(), *_write_args(p, t, st.cur, st.b0, li))
    assert rc == 0
    data = open(path, "rb").read()
    assert data == numpy_fluid_bytes(t, st.cur, st.b0, li, p.mbndry)
    # read back
    from g3m3_gb300.api import addr
    state = np.zeros_like(st.cur)
    b0 = np.zeros_like(st.b0)
    back = {k: np.zeros_like(v) for k, v in li.items()}
    tt = ctypes.c_double()
    rc = L.g3m3_fluid_read(None, path.encode(), ctypes.byref(p), ctypes.byref(tt), addr(state), addr(b0),
                           addr(back["parm_srf"]), addr(back["parm_mid"]), addr(back["parm_zero"]),
                           addr(back["ijzero"]), addr(back["numzero"]), addr(back["ijmid"]), addr(back["nummid"]),
                           addr(back["ijsrf"]), addr(back["numsrf"]),
                           li["ijsrf"].shape[0], li["ijmid"].shape[0], li["ijzero"].shape[0])
    assert rc == 0 and tt.value == t
    assert np.array_equal(state.view(np.uint32), st.cur.view(np.uint32))
    assert np.array_equal(b0.view(np.uint32), st.b0.view(np.uint32))
    for k in li:
        assert np.array_equal(back[k], li[k]), k
    # a file of other dimensions is refused
    q = make_config("tiny3").params
    rc = L.g3m3_fluid_read(None, path.encode(), ctypes.byref(q), ctypes.byref(tt), addr(np.zeros((34, 3, 9, 17, 17), np.float32)),
                           addr(np.zeros((3, 3, 9, 17, 17), np.float32)), None, None, None, None, None, None, None,
                           None, None, 1, 1, 1)
    assert rc != 0


@pytest.mark.gpu
def test_restart_from_fluid_file(tmp_path):
    """A stepped model written to a fluid file and read into a new model
    holds the same state, b0, tables and time: writing the new model gives
    the same file, byte for byte; the read model then steps like the
    oracle started from the file's contents."""
    from g3m3_gb300.api import Context, Model
    from g3m3_gb300.state import make_config
    from oracle.oracle import OracleModel
    st = make_config("tiny3")
    li = st.lists
    m3 = (li["ijsrf"].shape[0], li["ijmid"].shape[0], li["ijzero"].shape[0])
    p1 = str(tmp_path / "fluid11").encode()
    p2 = str(tmp_path / "fluid12").encode()
    with Context() as ctx:
        a = Model(ctx, st)
        a.init_steps()
        a.run(2)
        ctx.check(ctx.L.g3m3_model_write_fluid(a.h, p1))
        b = Model(ctx, make_config("tiny3", seed=99))   # different contents before the read
        ctx.check(ctx.L.g3m3_model_read_fluid(b.h, p1, *m3))
        ctx.check(ctx.L.g3m3_model_write_fluid(b.h, p2))
        assert open(p1, "rb").read() == open(p2, "rb").read()
        sb = b.state()
        tb = b.times()[0]
        b.init_steps()
        b.run(2)
        got = b.state()
    ref = make_config("tiny3")
    ref.cur = np.ascontiguousarray(sb)
    om = OracleModel(ref, omp=True)
    om.s.t = tb   # a restart keeps the file's time (t_old, t_new restart at 0, 3d_main.f90:1864-1865)
    om.init_steps()
    for _ in range(2):
        assert om.main_step() == 0
    for q in range(NFIELDS):
        assert_same(got[q], om.cur[q], f"restarted field {q}")


@pytest.mark.gpu
def test_diff_fields_matches_numpy():
    from g3m3_gb300.api import Context, addr, table
    from g3m3_gb300.state import make_config
    st = make_config("tiny2")
    p = st.params
    a = st.cur.copy()
    b = st.cur.copy()
    rng = np.random.default_rng(3)
    for q in (0, 5, 31):
        idx = rng.integers(0, b[q].size, 40)
        b[q].reshape(-1)[idx] += rng.standard_normal(40).astype(np.float32)
    b[7].reshape(-1)[:5] = -b[7].reshape(-1)[:5] * 0.0   # -0 vs +0 counts as equal where a is zero
    nf = 34
    stats = np.zeros((nf, p.n_grids, 4), np.float64)
    with Context() as ctx:
        ta, tb = table(list(a)), table(list(b))
        ctx.check(ctx.L.g3m3_diff_fields(ctx.h, nf, ctypes.addressof(ta), ctypes.addressof(tb), p.nx, p.ny, p.nz,
                                         p.n_grids, addr(stats)))
    for q in range(nf):
        for bx in range(p.n_grids):
            x = a[q, bx].astype(np.float64)
            y = b[q, bx].astype(np.float64)
            d = x - y
            cnt = int(np.sum((a[q, bx] != b[q, bx]) & ~(np.isnan(a[q, bx]) & np.isnan(b[q, bx]))))
            assert stats[q, bx, 3] == cnt, (q, bx)
            assert stats[q, bx, 0] == (np.max(np.abs(d)) if cnt else 0.0)
            assert abs(stats[q, bx, 1] - np.sum(d * d)) <= 1e-9 * max(1.0, np.sum(d * d))
            assert abs(stats[q, bx, 2] - np.sum(x * x)) <= 1e-9 * np.sum(x * x)
