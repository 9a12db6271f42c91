"""Gradients of a virtual-spacecraft misfit through the step engine
(g3m3_adjoint_* of libg3m3_gpu.so), and their torch.autograd binding.

``Adjoint`` wraps the C ABI: a forward run of N main steps from a model's
state (time steps recorded, state checkpointed every K steps, the misfit of
samples taken at the end of their main steps), then the hand-written
reverse of every kernel, checkpoint segment by checkpoint segment, which
gives dL/d(upstream parameters of the wind face) and dL/d(state before the
first step).

``upstream_wind`` maps the physical upstream conditions (n in cm^-3,
v in km/s, IMF in nT; 3d_main.f90:907-943) to the eight wind-face
parameters as torch operations, and ``WindMisfit`` is a
torch.autograd.Function of those eight parameters whose backward is the
CUDA adjoint, so

    loss = WindMisfit.apply(upstream_wind(u, setup), run)
    loss.backward()            # u.grad = dL/d(n, vx, vy, vz, bx, by, bz)

``EnsembleWindMisfit`` is the batched form over the members of an
``Ensemble`` (``EnsembleMisfit``): one loss per member, each member's
gradient from its own adjoint.
"""
from __future__ import annotations

import ctypes
import math

import numpy as np

from .api import Model, addr
from .params import NFIELDS
from .state import EV, M_PROT, MU0

WIND = ("srho", "spx", "spy", "spz", "spress", "sbx_wind", "sby_wind", "sbz_wind")



class Adjoint:
    def __init__(self, model: Model, nsteps: int, checkpoint_every: int = 10, cg_errlim: float = 0.0):
        self.model = model
        self.L = model.L
        self.ctx = model.ctx
        self.nsteps = int(nsteps)
        h = ctypes.c_void_p()
        self.ctx.check(self.L.g3m3_adjoint_create(model.h, self.nsteps, int(checkpoint_every), float(cg_errlim),
                                                  ctypes.byref(h)))
        self.h = h
        self._keep = []
        self.ctx._models.insert(0, self)   # closed before the models when the context closes

    def set_samples(self, xyz, step, target):
        """xyz (n, 3) planet radii; step (n,) main step (1-based) at whose end
        the sample is taken, non-decreasing; target (n, 4): bx, by, bz, rho."""
        xyz = np.ascontiguousarray(xyz, np.float32)
        step = np.ascontiguousarray(step, np.int32)
        target = np.ascontiguousarray(target, np.float32)
        self.ctx.check(self.L.g3m3_adjoint_set_samples(self.h, int(len(step)), addr(xyz), addr(step), addr(target)))

    def forward(self, schedule=None):
        """Run the N main steps from the model's state; returns the misfit.
        With ``schedule`` ((N, n_grids) t_stepnew), the time steps are those."""
        loss = ctypes.c_double()
        sch = None
        if schedule is not None:
            sch = np.ascontiguousarray(schedule, np.float64)
            self._keep = [sch]
        self.ctx.check(self.L.g3m3_adjoint_forward(self.h, addr(sch) if sch is not None else None,
                                                   ctypes.byref(loss)))
        return loss.value

    def schedule(self):
        out = np.empty((self.nsteps, self.model.p.n_grids), np.float64)
        self.ctx.check(self.L.g3m3_adjoint_schedule(self.h, addr(out)))
        return out

    def backward(self, state=True):
        """dL/d(wind parameters) (8, float64), and with ``state`` dL/d(state
        before the first step) (34, n_grids, nz, ny, nx) and dL/d(wrk epres)."""
        p = self.model.p
        gp = np.zeros(8, np.float64)
        gs = np.zeros((NFIELDS, p.n_grids, p.nz, p.ny, p.nx), np.float32) if state else None
        gw = np.zeros((p.n_grids, p.nz, p.ny, p.nx), np.float32) if state else None
        rc = self.L.g3m3_adjoint_backward(self.h, addr(gp), addr(gs) if state else None, addr(gw) if state else None)
        if rc not in (0, 3):   # 3: an adjoint div B solve hit its iteration cap (a warning)
            self.ctx.check(rc)
        return dict(params=gp, state=gs, wrk_epres=gw, noconv=rc == 3)

    def phases(self):
        """Seconds of the last backward: re-run with snapshots, reverse
        kernels, reversed div B passes; then the host time spent issuing
        each of the three."""
        out = (ctypes.c_double * 6)()
        self.ctx.check(self.L.g3m3_adjoint_phases(self.h, out))
        return list(out)

    def tape_bytes(self):
        return int(self.L.g3m3_adjoint_tape_bytes(self.h))

    def close(self):
        if self.h and self.model.h and self.ctx.h:
            self.L.g3m3_adjoint_destroy(self.h)
        self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def sample_state(p, cur, xyz):
    """(n, 4) trilinear values of bx, by, bz and the total density
    qrho + hrho + orho at xyz (n, 3) [planet radii] in the smallest box
    whose open extent holds the point (the library's misfit samples,
    cft_findgrid.f90:70-126, cft_trilin_interp.f90:34-54); NaN where no
    box holds it.  cur: (34, n_grids, nz, ny, nx) on the host."""
    out = np.full((len(xyz), 4), np.nan)
    for n, X in enumerate(np.asarray(xyz, np.float64)):
        v = X / p.re_equiv
        box = 0
        for b in range(1, p.n_grids + 1):
            mn = np.array([p.grd_xmin[b - 1], p.grd_ymin[b - 1], p.grd_zmin[b - 1]])
            mx = np.array([p.grd_xmax[b - 1], p.grd_ymax[b - 1], p.grd_zmax[b - 1]])
            if (v > mn).all() and (v < mx).all():
                box = b
                break
        if box == 0:
            continue
        mn = np.array([p.grd_xmin[box - 1], p.grd_ymin[box - 1], p.grd_zmin[box - 1]])
        sp = p.xspac[box - 1]
        g = 1 + ((v - mn) / sp).astype(int)
        if (g < 1).any() or g[0] >= p.nx or g[1] >= p.ny or g[2] >= p.nz:
            continue
        c0 = (mn + (g - 1) * sp) * p.re_equiv
        w = (X - c0) / (sp * p.re_equiv)
        i, j, k = g - 1
        val = np.zeros(4)
        for dk in (0, 1):
            for dj in (0, 1):
                for di in (0, 1):
                    wt = (w[0] if di else 1 - w[0]) * (w[1] if dj else 1 - w[1]) * (w[2] if dk else 1 - w[2])
                    c = (box - 1, k + dk, j + dj, i + di)
                    for q in range(3):
                        val[q] += wt * cur[31 + q][c]
                    val[3] += wt * (cur[0][c] + cur[10][c] + cur[20][c])
        out[n] = val
    return out


def line_samples(state, nsteps, n=200, seed=20261205, scale=0.1, x_end=0.4):
    """A virtual spacecraft on a straight line: n samples through the
    outermost box, from 2 % of its x extent (next to the inflow face) to
    x_end, y and z drawn from the seed between 15 and 30 % (beside the
    planet), spread evenly over the N main steps; targets are the initial
    state's values there times (1 + scale N(0,1)), drawn from the seed."""
    p = state.params
    rng = np.random.default_rng(seed)
    ng = p.n_grids
    lo = np.array([p.grd_xmin[ng - 1], p.grd_ymin[ng - 1], p.grd_zmin[ng - 1]]) * p.re_equiv
    hi = np.array([p.grd_xmax[ng - 1], p.grd_ymax[ng - 1], p.grd_zmax[ng - 1]]) * p.re_equiv
    span = hi - lo
    a = lo + span * np.array([0.02, 0.15 + 0.15 * rng.random(), 0.15 + 0.15 * rng.random()])
    b = lo + span * np.array([x_end, 0.15 + 0.15 * rng.random(), 0.15 + 0.15 * rng.random()])
    t = np.linspace(0.0, 1.0, n)
    xyz = (a[None, :] + t[:, None] * (b - a)[None, :]).astype(np.float32)
    step = (1 + (np.arange(n) * nsteps) // n).astype(np.int32)
    v0 = sample_state(p, state.cur.astype(np.float64), xyz)
    v0[np.isnan(v0)] = 0.0
    target = (v0 * (1.0 + scale * rng.standard_normal(v0.shape))).astype(np.float32)
    return xyz, step, target


def wind_of(params):
    """The eight wind-face parameters of a parameter block."""
    return np.array([getattr(params, k) for k in WIND], np.float64)


def wind_scales(setup):
    """Constants of the upstream conversion for a state.Setup: (1/rho_equiv *
    rmassq, 1/v_equiv, spress per unit srho, 1/b_equiv)."""
    gamma = 1.6666   # the value state.py (3d_main.f90's gamma) uses
    b_equiv = setup.v_equiv * 1.0e3 * math.sqrt(MU0 * setup.rho_equiv * 1.0e6 * M_PROT) * 1.0e9
    cs_wind = math.sqrt(gamma * setup.wind.t_ev * EV / M_PROT) / 1.0e3 / setup.v_equiv
    return setup.rmassq / setup.rho_equiv, 1.0 / setup.v_equiv, (cs_wind ** 2 / gamma) / (gamma - 1.0), 1.0 / b_equiv


def upstream_wind(u, setup):
    """The eight wind-face parameters from u = (n [cm^-3], vx, vy, vz [km/s],
    bx, by, bz [nT]) as torch operations (differentiable): srho = n m_q /
    rho_equiv, sp = srho v / v_equiv, spress = srho cs^2 / (gamma (gamma-1)),
    sb = B / b_equiv (state.py's conversion with the temperature held)."""
    import torch
    kr, kv, kp, kb = wind_scales(setup)
    srho = u[0] * kr
    return torch.stack([srho, srho * u[1] * kv, srho * u[2] * kv, srho * u[3] * kv, srho * kp,
                        u[4] * kb, u[5] * kb, u[6] * kb])


class MisfitRun:
    """A fixed experiment: the model's initial state, N main steps, the
    samples and (after the first call) the time-step schedule; ``loss(w)``
    runs it with wind parameters w and keeps the adjoint ready."""

    def __init__(self, model: Model, state, nsteps, samples, checkpoint_every=10, cg_errlim=0.0, schedule=None,
                 clock=None):
        self.model = model
        self.state = state
        self.adj = Adjoint(model, nsteps, checkpoint_every, cg_errlim)
        self.adj.set_samples(*samples)
        self.schedule = schedule
        # every run starts from this clock (t, main steps done: the div B cadence)
        self.clock = model.clock() if clock is None else clock

    def reset(self):
        self.model.upload(self.state)
        self.model.set_clock(*self.clock)
        self.model.init_steps()

    def loss(self, wind):
        w = np.ascontiguousarray(np.asarray(wind, np.float64).astype(np.float32))
        self.model.ctx.check(self.model.L.g3m3_model_set_wind(self.model.h, addr(w)))
        self.reset()
        val = self.adj.forward(self.schedule)
        if self.schedule is None:
            self.schedule = self.adj.schedule()
        return val


def ensemble_gradients(ensemble, states, nsteps, samples_of, checkpoint_every=1, cg_errlim=0.0, timer=None):
    """Batched + adjoint: every member of an ``Ensemble`` with its own
    virtual-spacecraft misfit and its gradient.  The members' gradients are
    taken one after another on their own models, each adjoint created,
    run (forward with checkpoints, backward) and destroyed before the next,
    so the members share the memory of one tape (one checkpoint interval
    of a 5-box 121x121x61 member is about 30 GB per main step).  Returns
    one dict per member: loss, dL/d(wind parameters), tape bytes, the
    backward's phases, and, with ``timer`` (timer(model, fn) runs fn and
    returns its milliseconds on the model's stream), the forward's and
    backward's times."""
    out = []
    for m, st in zip(ensemble.members, states):
        run = MisfitRun(m, st, nsteps, samples_of(st), checkpoint_every, cg_errlim)
        w = wind_of(st.params)
        rec = {}
        if timer is None:
            rec["loss"] = run.loss(w)
            g = run.adj.backward(state=False)
        else:
            box = {}
            rec["forward_ms"] = timer(m, lambda: box.setdefault("loss", run.loss(w)))
            rec["loss"] = box["loss"]
            rec["backward_ms"] = timer(m, lambda: box.setdefault("g", run.adj.backward(state=False)))
            g = box["g"]
        rec["grad_wind"] = g["params"]
        rec["tape_bytes"] = run.adj.tape_bytes()
        rec["phases_s"] = run.adj.phases()[:3]
        run.adj.close()
        out.append(rec)
    return out


class EnsembleMisfit:
    """The batched experiment: the members of an ``Ensemble``, each from
    its own state and its clock at construction, N main steps, each with its
    own samples (``samples_of(state)``); the time-step schedules of the
    first run are kept and reused."""

    def __init__(self, ensemble, states, nsteps, samples_of, checkpoint_every=1, cg_errlim=0.0):
        self.ensemble = ensemble
        self.states = list(states)
        self.nsteps = nsteps
        self.samples = [samples_of(st) for st in self.states]
        self.every = checkpoint_every
        self.errlim = cg_errlim
        self.schedules = [None] * len(self.states)
        self.clocks = [m.clock() for m in ensemble.members]

    def member(self, i):
        """A MisfitRun of member i (its adjoint holds a tape until closed)."""
        return MisfitRun(self.ensemble.members[i], self.states[i], self.nsteps, self.samples[i], self.every,
                         self.errlim, schedule=self.schedules[i], clock=self.clocks[i])

    def losses(self, winds):
        out = []
        for i in range(len(self.states)):
            run = self.member(i)
            out.append(run.loss(winds[i]))
            self.schedules[i] = run.schedule
            run.adj.close()
        return out

    def gradients(self, winds):
        out = []
        for i in range(len(self.states)):
            run = self.member(i)
            run.loss(winds[i])
            out.append(run.adj.backward(state=False)["params"])
            run.adj.close()
        return out


def _function():
    import torch

    class WindMisfit(torch.autograd.Function):
        """loss = misfit of a MisfitRun with the given wind parameters (8);
        backward: the hand-written CUDA adjoint."""

        @staticmethod
        def forward(ctx, wind, run):
            ctx.run = run
            val = run.loss(wind.detach().cpu().numpy())
            return torch.tensor(val, dtype=torch.float64)

        @staticmethod
        def backward(ctx, g):
            grads = ctx.run.adj.backward(state=False)
            return torch.from_numpy(grads["params"]) * g, None

    class EnsembleWindMisfit(torch.autograd.Function):
        """losses[m] = member m's misfit with wind parameters winds[m]
        (winds: members x 8) over an EnsembleMisfit; backward: each
        member's hand-written CUDA adjoint, the members one after another.
        The forward keeps no tape: backward runs each member's forward
        again with checkpoints before its reverse, so the members share the
        memory of one tape."""

        @staticmethod
        def forward(ctx, winds, experiment):
            w = winds.detach().cpu().numpy()
            ctx.experiment = experiment
            ctx.w = w
            return torch.tensor(experiment.losses(w), dtype=torch.float64)

        @staticmethod
        def backward(ctx, g):
            grads = np.stack(ctx.experiment.gradients(ctx.w))
            return torch.from_numpy(grads) * g.reshape(-1, 1), None

    return WindMisfit, EnsembleWindMisfit


class _Lazy:
    fns = None


def WindMisfit():
    if _Lazy.fns is None:
        _Lazy.fns = _function()
    return _Lazy.fns[0]


def EnsembleWindMisfit():
    """The batched form of WindMisfit (see _function)."""
    if _Lazy.fns is None:
        _Lazy.fns = _function()
    return _Lazy.fns[1]
