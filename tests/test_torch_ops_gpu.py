"""torch.ops.g3m3 on CUDA tensors against the oracle, bitwise: the ops
take the same arguments as the drop-in entries (tests/test_routines_gpu.py)
with arrays as CUDA tensors, tables as lists of tensors, integer lists and
real(dp) times as int32 / float64 tensors and the parameter block as bytes;
scalar results come back as return values."""
import ctypes

import numpy as np
import pytest

import test_routines_gpu as R
from _support import Inputs, assert_same, run_both

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def to_torch(args):
    import g3m3_gb300.torch_ops as T
    from g3m3_gb300.params import G3M3Params
    out = []
    for a in args:
        if isinstance(a, np.ndarray):
            out.append(torch.from_numpy(a.copy()).cuda())
        elif isinstance(a, list):
            out.append([torch.from_numpy(x.copy()).cuda() for x in a])
        elif isinstance(a, G3M3Params):
            out.append(T.params_tensor(a))
        elif isinstance(a, ctypes.Array):
            out.append(torch.from_numpy(np.ctypeslib.as_array(a).copy()))
        else:
            out.append(a)
    return out


def back(t):
    if isinstance(t, list):
        return [x.cpu().numpy() for x in t]
    return t.cpu().numpy() if isinstance(t, torch.Tensor) else t


def test_push_ion_op():
    I = Inputs("tiny2")
    args = R.push_ion_args(I, "h", 2)
    oa, _ = run_both("push_ion", args)
    ta = to_torch(args)
    assert torch.ops.g3m3.push_ion(*ta) is None
    torch.cuda.synchronize()
    for k in list(range(7)) + [21, 22, 23, 38, 39, 40]:
        assert_same(back(ta[k]), oa[k], f"push_ion arg {k}")


def test_flux_correct_and_bndry_outer_ops():
    I = Inputs("tiny2")
    p = I.p
    vv = I.scratch(1.0, 3)
    args = [list(I.cur), list(I.wrk), list(I.old)] + vv + I.dims(2) + [p.difrho, p.diferg]
    oa, _ = run_both("flux_correct", args, oracle_drop=(3, 4, 5))
    ta = to_torch([a for i, a in enumerate(args) if i not in (3, 4, 5)])
    torch.ops.g3m3.flux_correct(*ta)
    for q in range(34):
        assert_same(back(ta[0][q]), oa[0][q], f"flux_correct field {q}")
    args = [list(I.wrk), I.b0[0], I.b0[1], I.b0[2], p]
    oa, _ = run_both("bndry_outer", args)
    ta = to_torch(args)
    torch.ops.g3m3.bndry_outer(*ta)
    for q in range(34):
        assert_same(back(ta[0][q]), oa[0][q], f"bndry_outer field {q}")


def test_flanks_op_with_fp64_times():
    I = Inputs("tiny3")
    p = I.p
    g = I.grid()
    t_old = np.zeros(p.n_grids, np.float64)
    t_new = np.full(p.n_grids, 0.2, np.float64)
    work = np.zeros(I.box3, np.float32)
    args = [I.wrk[7], I.cur[7], I.old[7]] + I.dims(1) + [(ctypes.c_double * p.n_grids)(*t_new),
                                                         (ctypes.c_double * p.n_grids)(*t_old), 0.074, work] + g
    oa, _ = run_both("flanks", args)
    ta = to_torch(args)
    torch.ops.g3m3.flanks(*ta)
    assert_same(back(ta[0]), oa[0], "flanks")


def test_set_speed_agrd_op_returns_the_maxima():
    I = Inputs("tiny2")
    R.guard_inputs(I, 1)
    p = I.p
    f = I.cur
    args = (I.dims(1)[:4] + [1, p.rmassq, p.rmassh, p.rmasso, 0, p.smallbit, p.aniso_limit, p.vlim_factor, p.qvlim,
                             p.hvlim, p.ovlim, p.qclim, p.hclim, p.oclim, p.cslim,
                             f[31], f[32], f[33], I.b0[0], I.b0[1], I.b0[2]]
            + [f[q] for q in range(30)] + [f[30], np.zeros(I.box3, np.float32)])
    from _support import copy_args
    from oracle import oracle
    oa = copy_args(args)
    oo = [ctypes.c_float() for _ in range(6)]
    oracle.call("set_speed_agrd", *oa, *[ctypes.addressof(x) for x in oo])
    ta = to_torch(args)
    got = torch.ops.g3m3.set_speed_agrd(*ta)
    for k in range(25, 57):
        assert_same(back(ta[k]), oa[k], f"set_speed_agrd arg {k}")
    assert [np.float32(x) for x in got] == [np.float32(x.value) for x in oo]


def test_divb_correct_op_returns_iterations():
    I = Inputs("tiny2")
    p = I.p
    pos = np.array([p.nx * p.ny, p.nx, 1, 0, -1, -p.nx, -p.nx * p.ny], np.int32)
    xs = np.array(p.xspac[: p.n_grids], np.float32)
    b = [I.cur[31].copy(), I.cur[32].copy(), I.cur[33].copy()]
    from g3m3_gb300.api import Context
    gb = [x.copy() for x in b]
    it = ctypes.c_int()
    with Context() as ctx:
        ctx.call("divb_correct", *I.dims(1), 7, pos, xs, 1e-4, *gb, ctypes.addressof(it))
        ctx.sync_to_host(*gb)
    ta = to_torch([pos, xs] + b)
    iters = torch.ops.g3m3.divb_correct(*I.dims(1), 7, ta[0], ta[1], 1e-4, ta[2], ta[3], ta[4])
    # the same library solve, up to the order of its FP64 atomic sums
    assert isinstance(iters, int) and abs(iters - it.value) <= 1, (iters, it.value)
    for q in range(3):
        rel = np.linalg.norm(back(ta[2 + q]) - gb[q]) / np.linalg.norm(gb[q])
        assert rel <= 1e-5, (q, rel)
