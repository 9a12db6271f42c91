"""Failure handling of the C ABI, made on the host (no GPU fault):

* every drop-in entry returns G3M3_ERR_ARG for bad dimensions, before it
  touches an array or launches anything (its arrays here are valid host
  buffers, so nothing could fault even if a check were missing);
* a div B solve that reaches the iteration cap returns G3M3_ERR_NOCONV (the
  reference's "too many iterations" warning, sub_sparse_solver.f90:93,157),
  through the drop-in routine and through the engine;
* with the finite check on, NaN or Inf in host-staged inputs returns
  G3M3_ERR_NONFINITE before any upload;
* an allocation budget below what a call needs makes it fail with
  G3M3_ERR_ALLOC, as a full device would, and the context stays usable.
"""
import ctypes

import numpy as np
import pytest

from _support import Inputs

pytestmark = pytest.mark.gpu

ERR_ARG, ERR_NOCONV, ERR_NONFINITE, ERR_ALLOC = 1, 3, 4, 5

NOT_DROPIN = {"g3m3_ctx_create", "g3m3_ctx_destroy", "g3m3_ctx_set_cg_maxit", "g3m3_ctx_set_finite_check",
              "g3m3_ctx_set_alloc_limit", "g3m3_ctx_allocated", "g3m3_ctx_stream", "g3m3_last_error",
              "g3m3_sync_to_host", "g3m3_sync_to_device", "g3m3_release_mirrors", "g3m3_synchronize",
              "g3m3_model_create", "g3m3_ensemble_create"}


def dropin_entries():
    from g3m3_gb300 import _lib
    out = []
    for name, _ret, params in _lib.header_functions():
        if name in NOT_DROPIN or not params or not params[0].replace(" ", "").startswith("g3m3_ctx*"):
            continue
        out.append((name, params[1:]))
    return out


def test_every_dropin_rejects_bad_dimensions():
    from g3m3_gb300 import _lib
    from g3m3_gb300.api import Context

    entries = dropin_entries()
    assert len(entries) >= 30, [n for n, _ in entries]
    buf = np.zeros(1 << 16, np.float32)   # zero dims in any params struct, empty path strings
    tab = (ctypes.c_void_p * 64)(*([buf.ctypes.data] * 64))
    with Context() as ctx:
        for name, params in entries:
            fn = getattr(ctx.L, name)
            args = []
            for p, t in zip(params, fn.argtypes[1:]):
                if t is ctypes.c_void_p:
                    args.append(ctypes.addressof(tab) if "const*" in p.replace(" ", "") or "[" in p
                                else buf.ctypes.data)
                elif t in (ctypes.c_float, ctypes.c_double):
                    args.append(1.0)
                else:
                    args.append(0)   # nx = ny = nz = n_grids = box = npts = nbands = 0
            rc = fn(ctx.h, *args)
            assert rc == ERR_ARG, (name, rc, ctx.L.g3m3_last_error(ctx.h))
        ctx.synchronize()


def _divb_case(seed=5):
    I = Inputs("small", seed)
    p = I.p
    pos = (ctypes.c_int * 7)(p.nx * p.ny, p.nx, 1, 0, -1, -p.nx, -p.nx * p.ny)
    xs = np.array(p.xspac[: p.n_grids], np.float32)
    return I, pos, xs


def test_divb_iteration_cap_returns_noconv():
    import torch
    from g3m3_gb300.api import Context, G3M3Error

    I, pos, xs = _divb_case()
    p = I.p
    dims = [p.nx, p.ny, p.nz, p.n_grids, 1]
    with Context() as ctx:
        b = [torch.from_numpy(I.cur[31 + q].copy()).cuda() for q in range(3)]
        torch.cuda.synchronize()
        it = ctypes.c_int(-1)
        ctx.ctx_set_cg_maxit(2)
        with pytest.raises(G3M3Error) as e:
            ctx.divb_correct(*dims, 7, pos, xs, 1e-9, *b, ctypes.addressof(it))
        assert e.value.code == ERR_NOCONV and "too many iterations" in str(e.value)
        assert it.value == 2
        assert all(torch.isfinite(x).all() for x in b)
        # the same solve without the cap converges
        ctx.ctx_set_cg_maxit(0)
        b2 = [torch.from_numpy(I.cur[31 + q].copy()).cuda() for q in range(3)]
        torch.cuda.synchronize()
        ctx.divb_correct(*dims, 7, pos, xs, 1e-4, *b2, ctypes.addressof(it))
        ctx.synchronize()
        assert it.value > 2


def test_engine_divb_cap_returns_noconv():
    from g3m3_gb300.api import Context, G3M3Error, Model
    from g3m3_gb300.state import make_config

    st = make_config("tiny3")
    rng = np.random.default_rng(3)
    for q in (31, 32, 33):   # a B with divergence for the solver to remove
        st.cur[q] = (st.cur[q] + 0.02 * rng.standard_normal(st.cur[q].shape)).astype(np.float32)
    with Context() as ctx:
        m = Model(ctx, st)
        ctx.ctx_set_cg_maxit(1)
        with pytest.raises(G3M3Error) as e:
            ctx.check(ctx.L.g3m3_model_divb_all(m.h))
        assert e.value.code == ERR_NOCONV
        ctx.ctx_set_cg_maxit(0)
        ctx.check(ctx.L.g3m3_model_divb_all(m.h))
        assert np.isfinite(m.state()).all()
        m.close()


def test_finite_check_rejects_nan_and_inf():
    from g3m3_gb300.api import Context, G3M3Error, Model
    from g3m3_gb300.state import make_config

    I = Inputs("tiny2")
    p = I.p
    ev = I.scratch(0.1, 3)
    wrk = I.wrk[30].copy()
    wrk.flat[17] = np.nan
    args = [wrk, I.old[30].copy(), I.cur[30].copy()] + ev + [p.gamma, p.gamma1] + I.dims(1) + [0.02, 1.0, 1.0, 1.0]
    with Context() as ctx:
        ctx.ctx_set_finite_check(1)
        with pytest.raises(G3M3Error) as e:
            ctx.push_elec(*args)
        assert e.value.code == ERR_NONFINITE
        # a mirrored array refreshed with an Inf is refused too
        good = [I.wrk[30].copy(), I.old[30].copy(), I.cur[30].copy()] + ev
        ctx.push_elec(*good, p.gamma, p.gamma1, *I.dims(1), 0.02, 1.0, 1.0, 1.0)
        good[1].flat[3] = np.inf
        with pytest.raises(G3M3Error) as e:
            ctx.sync_to_device(good[1])
        assert e.value.code == ERR_NONFINITE
        st = make_config("tiny3")
        st.cur[4].flat[11] = -np.inf
        with pytest.raises(G3M3Error) as e:
            Model(ctx, st)
        assert e.value.code == ERR_NONFINITE
        # with the check off the same call goes through (the reference would
        # carry the NaN along)
        ctx.ctx_set_finite_check(0)
        ctx.push_elec(*args)
        ctx.synchronize()


def test_allocation_budget_fails_cleanly():
    from g3m3_gb300.api import Context, G3M3Error, Model
    from g3m3_gb300.state import make_config

    st = make_config("tiny3")
    with Context() as ctx:
        used = ctx.L.g3m3_ctx_allocated(ctx.h)
        ctx.ctx_set_alloc_limit(used + (64 << 10))
        with pytest.raises(G3M3Error) as e:
            Model(ctx, st)
        assert e.value.code == ERR_ALLOC
        I = Inputs("small")
        p = I.p
        ev = I.scratch(0.1, 3)
        with pytest.raises(G3M3Error) as e:
            ctx.push_elec(I.wrk[30], I.old[30], I.cur[30], *ev, p.gamma, p.gamma1, *I.dims(1), 0.02, 1.0, 1.0, 1.0)
        assert e.value.code == ERR_ALLOC
        ctx.ctx_set_alloc_limit(0)
        m = Model(ctx, st)
        m.init_steps()
        m.run(1, graph=False)
        assert np.isfinite(m.state()).all()
        m.close()
