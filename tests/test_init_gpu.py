"""The fresh-start state built on the device equals the host restatement of
the reference's initial conditions (g3m3_gb300/state.py) with the random
parts switched off: FP64 arithmetic rounded to FP32 on both sides, so the
values agree to 1 ulp (transcendentals may differ in the last FP64 bit) and
the inner-boundary lists exactly; the device-built state then steps like
the oracle started from it."""
import numpy as np
import pytest

from _support import assert_same

pytestmark = pytest.mark.gpu


def _read_fluid(path, p, li_shapes):
    data = open(path, "rb").read()
    pos = 0

    def rec():
        nonlocal pos
        n = int.from_bytes(data[pos:pos + 4], "little")
        body = data[pos + 4:pos + 4 + n]
        pos += 8 + n
        return body
    t = np.frombuffer(rec(), np.float64)[0]
    shape = (p.n_grids, p.nz, p.ny, p.nx)
    recs = [np.frombuffer(rec(), np.float32).reshape(shape) for _ in range(37)]
    file_order = list(range(30)) + [31, 32, 33, 30]   # library field held by each file record
    state = np.zeros((34,) + shape, np.float32)
    for r in range(34):
        state[file_order[r]] = recs[r]
    b0 = np.stack(recs[34:37])
    tail = rec()
    return t, state, b0, tail


@pytest.mark.parametrize("cfg", ["tiny3", "mid3"])
def test_device_init_matches_host(cfg, tmp_path):
    from g3m3_gb300.api import Context, Model
    from g3m3_gb300.state import make_config
    from oracle.oracle import OracleModel
    host = make_config(cfg, noise=0.0, iono_lo=1.0, iono_hi=1.0)
    p = host.params
    path = str(tmp_path / "fluid_dev").encode()
    with Context() as ctx:
        m = Model(ctx, None, params=p)
        m.init_state(alf_inner=-5.0, noise=0.0)
        ctx.check(ctx.L.g3m3_model_write_fluid(m.h, path))
        m.init_steps()
        m.run(2)
        stepped = m.state()
        m.close()
    t, state, b0, tail = _read_fluid(path, p, None)
    tol = lambda a, b: np.abs(a.astype(np.float64) - b) <= 1.2e-7 * np.abs(b.astype(np.float64)) + 1e-30
    assert tol(state, host.cur).all(), int((~tol(state, host.cur)).sum())
    assert tol(b0, host.b0).all(), int((~tol(b0, host.b0)).sum())
    li = host.lists
    want = b"".join(np.ascontiguousarray(li[k]).tobytes() for k in
                    ("parm_srf", "parm_mid", "parm_zero", "ijzero", "numzero", "ijmid", "nummid", "ijsrf", "numsrf"))
    assert len(tail) == len(want)
    # the integer tables exactly; the parm values to 1 ulp
    off = 0
    for k in ("parm_srf", "parm_mid", "parm_zero", "ijzero", "numzero", "ijmid", "nummid", "ijsrf", "numsrf"):
        a = np.ascontiguousarray(li[k])
        got = np.frombuffer(tail[off:off + a.nbytes], a.dtype).reshape(a.shape)
        off += a.nbytes
        if a.dtype == np.int32:
            assert np.array_equal(got, a), k
        else:
            assert tol(got, a).all(), k
    # the device-built state steps like the oracle started from it
    ref = make_config(cfg, noise=0.0, iono_lo=1.0, iono_hi=1.0)
    ref.cur = np.ascontiguousarray(state)
    ref.b0 = np.ascontiguousarray(b0)
    om = OracleModel(ref, omp=True)
    om.init_steps()
    for _ in range(2):
        assert om.main_step() == 0
    for q in range(34):
        assert_same(stepped[q], om.cur[q], f"{cfg} field {q} after 2 steps")
