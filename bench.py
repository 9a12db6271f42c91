"""Benchmark of the G3M^3 multifluid step on GB300.

Workload (default): the production nested grid -- 5 boxes of 121x121x61,
2x refined, FP32 state, 34 fields per box, sub-cycled (box b steps up to
2^(5-b) times per main step), div B cleaning every 10 main steps.  A "step"
is one main step of the reference time loop (3d_main.f90:1925-3095).
Metric: multifluid cell-updates/s (cells x executed box-steps / time).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

--impl reference times the reference's own main loop on the host cores: its
Fortran translated to C and compiled by oracle/fortran_to_c.py (there is no
Fortran compiler in the image), its OpenMP loops on every host thread with
each parallel loop's temporaries private (the build is checked bit for bit
against the serial one).  Where that build is absent, the oracle's
restatement (OpenMP) stands in and the line says "port".
With N>1 (torchrun) every rank advances its own replica: the path has no
data exchange between members.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

METRIC = "multifluid cell-updates/s"
WORKLOAD = "nested grid, 5 boxes 121x121x61, 2x refinement, sub-cycled, FP32, divB CG every 10 steps"


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def replica_reduce(max_vals, sum_vals):
    """Whole-job figures of N independent replicas (one per rank): the
    slowest rank's times (max) and the work of all ranks (sum).  Without an
    initialised process group the values are returned unchanged."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return [float(x) for x in max_vals], [float(x) for x in sum_vals]
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(x) for x in max_vals], dtype=torch.float64, device=dev)
    u = torch.tensor([float(x) for x in sum_vals], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    dist.all_reduce(u, op=dist.ReduceOp.SUM)
    return [float(x) for x in t.tolist()], [float(x) for x in u.tolist()]


class Clocks:
    """nvidia-smi samples while the timed region runs."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu):
        self.gpu = gpu
        self.proc = None
        self.lines = []

    def start(self):
        """Starts the sampler and returns once its first sample is in (at
        most 10 s), so that samples cover the timed region from its start;
        only samples taken after this returns are counted."""
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            threading.Thread(target=self._read, daemon=True).start()
        except Exception:
            self.proc = None
            return
        t0 = time.time()
        while not self.lines and self.proc.poll() is None and time.time() - t0 < 10.0:
            time.sleep(0.01)
        self.first = len(self.lines)

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
        self.lines = self.lines[getattr(self, "first", 0):]
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(sm)}


def peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


# ------------------------------------------------------------------ our arm
def run_ours(args):
    import torch
    ws, rank, local = dist_env()
    torch.cuda.set_device(local)
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    from g3m3_gb300.api import Context, Model, addr
    from g3m3_gb300.state import make_config

    st = make_config("nested", seed=20261203 + rank)
    p = st.params
    ctx = Context(local)
    m = Model(ctx, st)
    fcs_variant = m.autotune()   # tile shapes, timed on scratch copies (untimed setup)
    # a step plan (the boxes' sub-cycling schedule) is captured as a graph at
    # its second occurrence; one that occurs once runs host-launched
    m.set_capture_after(2)
    m.init_steps()
    stream = torch.cuda.ExternalStream(m.stream)

    def barrier():
        torch.cuda.synchronize()
        if ws > 1:
            torch.distributed.barrier()

    def timed(nsteps, graph):
        t0c, _, cu0 = m.times()
        k0 = 0
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        barrier()
        e0.record(stream)
        m.run(nsteps, graph=graph)
        e1.record(stream)
        barrier()
        ms = e0.elapsed_time(e1)
        _, tsn, cu1 = m.times()
        k, g = m.stats()
        return ms, cu1 - cu0, k

    # warm-up (captures the graphs for the schedule shapes seen), then a
    # four-step trial of each launch mode -- one CUDA graph per main step, or
    # kernels launched from the host on the model's streams -- kept clear of
    # the div B step (every 10th); the timed region runs the faster mode
    done = 0
    m.run(max(args.warmup, 3), graph=True)
    m.divb_all()          # warm-up of the div B pass too (captures its iteration graphs)
    m.run(1, graph=False)
    done += max(args.warmup, 3) + 1
    TRIAL = 4
    while any((done + i) % 10 == 0 for i in range(1, 2 * TRIAL + 1)):
        m.run(1, graph=True)
        done += 1
    trial = {}
    for graph in (True, False):
        ms_t, cu_t, _ = timed(TRIAL, graph)
        trial[graph] = cu_t / ms_t
    done += 2 * TRIAL
    use_graph = trial[True] >= trial[False]
    mode_name = {True: "one CUDA graph per main step", False: "kernels launched from the host on the model's streams"}
    clocks = Clocks(local)
    clocks.start()
    ms_g, cu_g, k_g = timed(args.steps, use_graph)
    clk = clocks.stop()
    ms_p, cu_p, k_p = timed(args.steps, not use_graph)

    # the contracted flavour of push_ion (FMA contraction, reciprocal
    # products; within 1e-5 relative L2 per field per main step of the FP32
    # bits), same mode, then back to the bitwise build for the e2e leg
    m.L.g3m3_model_set_contracted(m.h, 1)
    m.run(2, graph=use_graph)                  # recaptures the step graphs
    ms_c, cu_c, _ = timed(args.steps, use_graph)
    m.L.g3m3_model_set_contracted(m.h, 0)
    m.run(2, graph=use_graph)

    # e2e: state from pinned host memory every step, result read back
    n4 = p.n_grids * p.nz * p.ny * p.nx
    host = torch.empty((34 * n4,), dtype=torch.float32, pin_memory=True)
    host_np = host.numpy()
    m.state(out=host_np.reshape(34, p.n_grids, p.nz, p.ny, p.nx))
    # one call per main step: g3m3_model_step_host uploads each box on a copy
    # stream (the step waits for a box only before touching it), steps, and
    # reads the state back.  Untimed warm-up first, one div B period of
    # steps: the graphs of this host buffer for the schedule shapes a long
    # run repeats (the buffer roles alternate; a shape first seen later is
    # captured inside the window, about 23 ms once: e2e.ms_per_call).
    for _ in range(10):
        m.step_host(host_np, host_np, graph=use_graph)
    # as many main steps as the device-timed region, so both hold the same
    # share of div B passes (one every 10th main step)
    e2e_steps = max(2, args.steps)
    barrier()
    t0 = time.perf_counter()
    cu_e0 = m.times()[2]
    call_ms = []
    for _ in range(e2e_steps):
        tc = time.perf_counter()
        m.step_host(host_np, host_np, graph=use_graph)
        call_ms.append(round((time.perf_counter() - tc) * 1e3, 2))
    barrier()
    e2e_s = time.perf_counter() - t0
    cu_e = m.times()[2] - cu_e0
    # the host link on its own: the whole state up and down (best of 3)
    up_s = down_s = 1e30
    for _ in range(3):
        t0 = time.perf_counter()
        m.set_state(host_np.reshape(34, p.n_grids, p.nz, p.ny, p.nx))
        torch.cuda.synchronize(local)   # the upload is asynchronous
        up_s = min(up_s, time.perf_counter() - t0)
        t0 = time.perf_counter()
        m.state(out=host_np.reshape(34, p.n_grids, p.nz, p.ny, p.nx))
        down_s = min(down_s, time.perf_counter() - t0)

    # one div B cleaning pass over all boxes (the main-step loop runs one
    # inside every 10th main step, so the timed region above holds one)
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    barrier()
    e0.record(stream)
    m.divb_all()
    e1.record(stream)
    barrier()
    divb_ms = e0.elapsed_time(e1)

    # per-kernel times (CUDA events on the engine's stream) for the roofline;
    # this overwrites the wrk/old copies, so it runs after the timed legs
    rows = kernel_table(m)
    roof = roofline_from(rows)
    m.L.g3m3_model_set_contracted(m.h, 1)
    contracted_push = kernel_table(m, only=0)
    m.L.g3m3_model_set_contracted(m.h, 0)
    (ms_g, ms_p, e2e_s, ms_c), (cu_g, cu_p, cu_e, k_g, cu_c) = replica_reduce([ms_g, ms_p, e2e_s, ms_c],
                                                                              [cu_g, cu_p, cu_e, k_g, cu_c])
    m.close()
    ctx.close()
    if rank != 0:
        return None
    value = cu_g / (ms_g / 1e3)
    line = {
        "metric": METRIC, "value": value, "unit": "cell-updates/s", "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_g / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded state from the "
        "reference's initial-condition formulas + 1% noise)",
        "config": {"workload": WORKLOAD, "boxes": p.n_grids, "box": [p.nx, p.ny, p.nz],
                   "cells_per_box": p.nx * p.ny * p.nz, "cell_updates_per_step": cu_g / args.steps / ws,
                   "mode": mode_name[use_graph], "graph_capture": "at a step plan's second occurrence",
                   "l2": "working set (>400 MB per box) exceeds L2",
                   "parallelism": f"replicas x{ws}",
                   "autotuned": {"fcsmooth": {0: "32x8 tiles", 1: "32x16 tiles",
                                              2: "32x8 tiles, two fields per block, FP32x2, 3 blocks/SM",
                                              3: "32x8 tiles, two fields per block, FP32x2, 4 blocks/SM",
                                              4: "32x8 tiles, two fields per block, FP32x2, cp.async planes, one barrier per plane, 80 registers",
                                              5: "32x8 tiles, two fields per block, FP32x2, cp.async planes, one barrier per plane, registers unbounded",
                                              6: "32x8 tiles, two fields per block, FP32x2, cp.async planes, one barrier per plane, 55 KB rings, 4 blocks/SM",
                                              7: "32x16 tiles, two fields per block, FP32x2, cp.async planes, one barrier per plane, 92 KB rings, 2 blocks/SM",
                                              }[fcs_variant]}},
        "other_mode": {"value": cu_p / (ms_p / 1e3), "ms_per_step": ms_p / args.steps,
                       "mode": mode_name[not use_graph]},
        "contracted": {"value": cu_c / (ms_c / 1e3), "ms_per_step": ms_c / args.steps,
                       "accuracy": "push_ion with FMA contraction and reciprocal products: within 1e-5 relative "
                                   "L2 per field per main step of the reference's FP32 bits "
                                   "(tests/test_contracted_gpu.py)",
                       "push_ion": contracted_push.get("push_ion")},
        "mode_trial": {"graph": trial[True] * 1e3, "streams": trial[False] * 1e3, "unit": "cell-updates/s",
                       "steps": TRIAL},
        "e2e": {"value": cu_e / e2e_s, "unit": "cell-updates/s", "h2d_bytes_per_step": 34 * n4 * 4,
                "d2h_bytes_per_step": 34 * n4 * 4,
                "path": "g3m3_model_step_host (pinned host state in, per-box uploads overlapping the step, state out)",
                "ms_per_call": call_ms,
                "state_copy_ms": {"h2d": up_s * 1e3, "d2h": down_s * 1e3,
                                  "note": "the whole state alone, best of 3: the read-back follows the step's last "
                                          "kernels, and the step waits for the coarsest box's upload"}},
        "gpu_launches": int(k_g),
        "divb_all_ms": divb_ms,
        "roofline": roof,
        "kernels": rows,
        "clocks": clk,
    }
    if not args.no_batched:
        line["batched"] = run_batched(args, local)
    if not args.no_adjoint:
        line["adjoint"] = run_adjoint(local)
        line["batched_adjoint"] = run_batched_adjoint(local)
    if not args.no_cpu and ws == 1:
        line["cpu_baseline"] = cpu_baseline()
    return line


def run_batched(args, device, members=16):
    """The upstream-condition ensemble: 16 nested grids (5 boxes each, box
    sizes cycling 121x121x61, 97x97x49, 81x81x41; wind from the seed),
    advanced with one CUDA graph per main step for all members, and plain
    (members one after another, kernels launched from the host loop)."""
    import torch
    from g3m3_gb300.api import Context, Ensemble
    from g3m3_gb300.state import ensemble_member
    ctx = Context(device)
    states = [ensemble_member(i) for i in range(members)]
    ens = Ensemble(ctx, states)
    cells = sorted({(st.params.nx, st.params.ny, st.params.nz) for st in states}, reverse=True)
    del states
    tuned = ens.autotune()
    ens.init_steps()
    stream = torch.cuda.ExternalStream(ens.stream)

    def timed(nsteps, mode):
        cu0 = ens.stats()[2]
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record(stream)
        ens.run(nsteps, graph=mode in ("graph", "member_graphs"), concurrent=mode in ("streams", "member_graphs"))
        e1.record(stream)
        torch.cuda.synchronize()
        k, _, cu1 = ens.stats()
        return e0.elapsed_time(e1), cu1 - cu0, k

    ens.run(max(args.warmup, 2), graph=True)   # captures the step graphs
    for mm in ens.members:                     # and the div B iteration graphs
        mm.divb_all()
    ens.run(2, graph=True, concurrent=True)    # and every member's own graphs
    ens.run(1, graph=False, concurrent=True)
    ms_g, cu_g, k_g = timed(args.steps, "graph")
    ms_m, cu_m, k_m = timed(args.steps, "member_graphs")
    ms_c, cu_c, _ = timed(args.steps, "streams")
    n_p = max(2, args.steps // 2)
    ms_p, cu_p, _ = timed(n_p, "sequential")
    ens.close()
    ctx.close()
    vg, vc, vp = cu_g / (ms_g / 1e3), cu_c / (ms_c / 1e3), cu_p / (ms_p / 1e3)
    vm = cu_m / (ms_m / 1e3)
    return {"workload": f"ensemble of {members} nested grids, 5 boxes each, box sizes "
                        + ", ".join(f"{a}x{b}x{c}" for a, b, c in cells) + " cycling; upstream n, |v|, IMF "
                        "clock angle and |B| drawn from the seed",
            "members": members,
            "autotuned_fcsmooth": {f"{a}x{b}x{c}": v for (a, b, c), v in tuned.items()},
            "graph": {"value": vg, "unit": "cell-updates/s", "ms_per_step": ms_g / args.steps, "steps": args.steps,
                      "gpu_launches": int(k_g), "mode": "one CUDA graph per main step for all members, "
                      "members on their own streams"},
            "member_graphs": {"value": vm, "unit": "cell-updates/s", "ms_per_step": ms_m / args.steps,
                              "steps": args.steps, "gpu_launches": int(k_m),
                              "mode": "every member's own step graph launched at once on its own stream"},
            "streams": {"value": vc, "unit": "cell-updates/s", "ms_per_step": ms_c / args.steps,
                        "steps": args.steps,
                        "mode": "every member launched at once from the host on its own streams"},
            "plain": {"value": vp, "unit": "cell-updates/s", "ms_per_step": ms_p / n_p, "steps": n_p,
                      "mode": "members one after another, kernels launched from the host loop"},
            "graph_over_plain": vg / vp, "member_graphs_over_plain": vm / vp, "streams_over_plain": vc / vp}


ADJOINT_WORKLOAD = ("adjoint of 50 main steps on 3 nested boxes of 97x97x49 (2x refinement, sub-cycled, FP32 state, "
                    "FP64 CG reductions, div B every 10 steps), checkpointed every 10 steps; misfit of B and density "
                    "at 200 samples along a seeded straight line, gradient w.r.t. the 8 upstream wind-face parameters "
                    "and the initial state")


def run_adjoint(device, nsteps=50, every=10, nsamp=200):
    """The adjoint of 50 main steps of 3 nested 97x97x49
    boxes, checkpointed every 10 steps.  Times (CUDA events on the model's
    stream): the plain forward (the engine's step, graph-replayed), the
    adjoint's forward (host-launched, with checkpoints and the misfit), and
    the backward (each checkpoint interval re-run with snapshots, then every
    kernel reversed).  adjoint_over_forward = backward / plain forward, per
    main step."""
    import torch
    from g3m3_gb300.adjoint import MisfitRun, line_samples, wind_of
    from g3m3_gb300.api import Context, Model
    from g3m3_gb300.state import make_config
    st = make_config("nested", limit=48, n_grids=3)
    p = st.params
    ctx = Context(device)
    m = Model(ctx, st)
    m.autotune()
    stream = torch.cuda.ExternalStream(m.stream)

    def ev_time(fn):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record(stream)
        fn()
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1)

    # the plain forward: the same 50 main steps from the same state, graph-replayed
    m.init_steps()
    m.run(3, graph=True)                       # warm-up (graph captures)
    m.upload(st)
    m.init_steps()
    cu0 = m.times()[2]
    fwd_ms = ev_time(lambda: m.run(nsteps, graph=True))
    cu = m.times()[2] - cu0
    samples = line_samples(st, nsteps, n=nsamp)
    run = MisfitRun(m, st, nsteps, samples, checkpoint_every=every)
    w = wind_of(p)
    run.loss(w)                                 # warm-up: records the schedule, allocates
    run.adj.backward(state=False)
    loss_box = {}
    afwd_ms = ev_time(lambda: loss_box.setdefault("loss", run.loss(w)))
    grads = {}
    bwd_ms = ev_time(lambda: grads.update(run.adj.backward(state=False)))
    tape = run.adj.tape_bytes()
    phases = run.adj.phases()
    run.adj.close()
    m.close()
    ctx.close()
    return {"workload": ADJOINT_WORKLOAD, "boxes": p.n_grids, "box": [p.nx, p.ny, p.nz], "main_steps": nsteps,
            "checkpoint_every": every, "samples": nsamp, "cell_updates": cu,
            "forward_ms_per_step": fwd_ms / nsteps,
            "adjoint_forward_ms_per_step": afwd_ms / nsteps,
            "backward_ms_per_step": bwd_ms / nsteps,
            "adjoint_over_forward": bwd_ms / fwd_ms,
            "gradient_over_forward": (afwd_ms + bwd_ms) / fwd_ms,
            "loss": loss_box["loss"], "grad_wind": [float(x) for x in grads["params"]],
            "tape_bytes": tape,
            "backward_phases_s": {"rerun_with_snapshots": phases[0], "reverse_kernels": phases[1],
                                  "divb_reverse": phases[2]},
            "backward_issue_s": {"rerun_with_snapshots": phases[3], "reverse_kernels": phases[4],
                                 "divb_reverse": phases[5]},
            "note": "forward: the engine's graph-replayed main steps; backward: per checkpoint interval the steps "
                    "re-run with snapshots, then the reverse kernels"}


def run_batched_adjoint(device, members=8, nsteps=10, every=1, nsamp=200):
    """Batched + adjoint: 8 ensemble members on nested grids of 5 boxes of
    121x121x61 (upstream conditions from the seed), the forward of all
    members as one CUDA graph per main step, then each member's adjoint of
    the same 10 main steps (checkpoints every step: one step's tape, about
    30 GB, is what one member's backward holds) for the misfit of its own
    200 line samples; members' gradients one after another, sharing the
    tape's memory.  adjoint_over_forward = the members' backward time /
    the batched forward's, per main step."""
    import torch
    from g3m3_gb300.adjoint import ensemble_gradients, line_samples
    from g3m3_gb300.api import Context, Ensemble
    from g3m3_gb300.state import ensemble_member
    ctx = Context(device)
    states = [ensemble_member(i, limits=(60,)) for i in range(members)]
    ens = Ensemble(ctx, states)
    ens.autotune()
    ens.init_steps()
    stream = torch.cuda.ExternalStream(ens.stream)

    def ev_time(fn, s=stream):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record(s)
        fn()
        e1.record(s)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1)

    ens.run(2, graph=True)                     # warm-up: graph captures
    for m, st in zip(ens.members, states):
        m.upload(st)
    ens.init_steps()
    cu0 = ens.stats()[2]
    fwd_ms = ev_time(lambda: ens.run(nsteps, graph=True))
    cu = ens.stats()[2] - cu0
    # each member's gradient: CUDA events on that member's stream
    recs = ensemble_gradients(ens, states, nsteps, lambda st: line_samples(st, nsteps, n=nsamp),
                              checkpoint_every=every,
                              timer=lambda m, fn: ev_time(fn, torch.cuda.ExternalStream(m.stream)))
    p = states[0].params
    ens.close()
    ctx.close()
    bwd_ms = sum(r["backward_ms"] for r in recs)
    afwd_ms = sum(r["forward_ms"] for r in recs)
    return {"workload": f"{members} ensemble members, nested grids of 5 boxes of 121x121x61 (upstream conditions "
                        f"from the seed), {nsteps} main steps; forward: all members in one CUDA graph per main "
                        f"step; gradient: each member's adjoint (checkpoints every {every} step(s), {nsamp} line "
                        f"samples of its own), members one after another sharing the tape's memory",
            "members": members, "box": [p.nx, p.ny, p.nz], "boxes": p.n_grids, "main_steps": nsteps,
            "checkpoint_every": every,
            "forward": {"value": cu / (fwd_ms / 1e3), "unit": "cell-updates/s", "ms_per_step": fwd_ms / nsteps},
            "gradient": {"value": cu / ((afwd_ms + bwd_ms) / 1e3), "unit": "cell-updates/s (forward with "
                         "checkpoints + backward, all members)", "ms_per_step": (afwd_ms + bwd_ms) / nsteps},
            "adjoint_forward_ms_per_step": afwd_ms / nsteps, "backward_ms_per_step": bwd_ms / nsteps,
            "adjoint_over_forward": bwd_ms / fwd_ms, "gradient_over_forward": (afwd_ms + bwd_ms) / fwd_ms,
            "tape_bytes_per_member": max(r["tape_bytes"] for r in recs),
            "losses": [r["loss"] for r in recs],
            "grad_wind_norms": [float(np.linalg.norm(r["grad_wind"])) for r in recs]}


KERNELS = {  # id: (name, launches per box-step)
    0: ("push_ion", 6), 1: ("fcsmooth x34", 1), 2: ("set_rho+set_speed_agrd", 4),
    3: ("lapidus (10 fields)", 3), 4: ("flanks x34", 4), 5: ("calcur+bs/btot", 2), 6: ("BandE", 2),
}


def kernel_table(m, reps=20, only=None):
    """Each engine kernel (or kernel `only`) on box 1 of the nested grid,
    CUDA events on the engine's stream; share = launches per box-step x
    time per launch."""
    import ctypes
    rows = {}
    for kid, (name, per_step) in KERNELS.items():
        if only is not None and kid != only:
            continue
        ms = ctypes.c_float()
        by = ctypes.c_double()
        rc = m.L.g3m3_model_time_kernel(m.h, kid, 1, reps, ctypes.byref(ms), ctypes.byref(by))
        if rc:
            continue
        rows[name] = {"ms_per_launch": ms.value, "launches_per_box_step": per_step,
                      "algorithmic_bytes_per_launch": by.value,
                      "achieved_gbs": by.value / (ms.value / 1e3) / 1e9}
    tot = sum(r["ms_per_launch"] * r["launches_per_box_step"] for r in rows.values())
    for r in rows.values():
        r["share_of_timed_kernels"] = r["ms_per_launch"] * r["launches_per_box_step"] / tot if tot else None
    return rows


# DRAM bytes (read + write) per launch from one ncu capture of each kernel
# on a 121x121x61 box (profiles/*_121x121x61.md); push_ion's is the mean of
# the 9 corrector-form launches (30 arrays read, the form the kernel timer
# runs) of the two-box capture (profiles/hbm_per_kernel_2x121x121x61.md)
NCU_TRAFFIC = {
    "fcsmooth x34": 243.07e6 + 95.59e6,
    "push_ion": 113.55e6 + 10.35e6,
    "set_rho+set_speed_agrd": 100.11e6 + 4.78e6,
    "flanks x34": 82.79e6 + 4.61e6,
}


def roofline_from(rows):
    name = max(rows, key=lambda k: rows[k]["ms_per_launch"] * rows[k]["launches_per_box_step"])
    r = rows[name]
    peak, kind = peaks()
    return {"kernel": name + " (121x121x61 box)", "bound": "hbm", "achieved": r["achieved_gbs"], "peak": peak,
            "unit": "GB/s", "frac": r["achieved_gbs"] / peak, "peak_source": kind,
            "ms_per_launch": r["ms_per_launch"], "algorithmic_bytes_per_launch": r["algorithmic_bytes_per_launch"],
            "traffic": NCU_TRAFFIC.get(name),
            "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum, one launch" if name in NCU_TRAFFIC
            else None}


def _reference_steps(nsteps, warmup):
    """Time `nsteps` main steps of the nested grid on the CPU after `warmup`
    untimed ones, then one div B pass, charged at the GPU arm's cadence
    (one pass per `divb_every` main steps, as the timed GPU steps hold):
    the reference's own main loop and its own div B routines where its
    translated build exists ("reference"), else the oracle's restatement
    ("port"); the steps with OpenMP on every host thread, the pass as the
    reference runs it (serial).  Returns (cell-updates/s, seconds per step
    with the pass's share, kind, threads, seconds of the pass)."""
    from g3m3_gb300.state import make_config
    every = make_config("nested").params.divb_every
    st = make_config("nested", divb_every=0)
    p = st.params
    cells = p.nx * p.ny * p.nz
    threads = int(os.environ.get("OMP_NUM_THREADS", os.cpu_count()))
    try:
        from oracle.refmain import RefMain
        rm = RefMain("nested", omp=True)
    except (FileNotFoundError, OSError):
        rm = None
    if rm is not None:
        # the state the reference's initialisation leaves: old zeroed, wrk = cur
        rm.load_state(p, st.cur, np.zeros_like(st.cur), st.cur.copy(), st.b0, st.resistive, st.lists,
                      0.0, np.zeros(p.n_grids))
        rm.init_steps()
        for _ in range(warmup):
            rm.steps(1)
        cu, t0 = 0, time.perf_counter()
        for _ in range(nsteps):
            rm.steps(1)
            cu += sum(rm.box_steps()) * cells
        dt = time.perf_counter() - t0
        pass_s = rm.divb_pass(p)
        dt += pass_s * nsteps / every
        return cu / dt, dt / nsteps, "reference", threads, pass_s
    from oracle.oracle import OracleModel
    om = OracleModel(st, omp=True)
    om.init_steps()
    for _ in range(warmup):
        om.main_step()
    cu0, t0 = om.cell_updates, time.perf_counter()
    for _ in range(nsteps):
        om.main_step()
    dt = time.perf_counter() - t0
    t1 = time.perf_counter()
    om.divb_all()
    pass_s = time.perf_counter() - t1
    dt += pass_s * nsteps / every
    return (om.cell_updates - cu0) / dt, dt / nsteps, "port", threads, pass_s


def cpu_baseline():
    """The reference's CPU path on a bounded sample: one main step of the
    same nested grid (about 27.7 M cell-updates) after one untimed step
    (the first touches the 1.9 GB of state)."""
    v, sec, kind, threads, pass_s = _reference_steps(1, 1)
    what = ("the reference's main loop (translated Fortran, OpenMP)" if kind == "reference"
            else "the oracle's restatement (OpenMP)")
    return {"value": v, "unit": "cell-updates/s", "cores": threads, "kind": kind,
            "sample": f"1 main step of the nested 5-box grid after 1 untimed, {what}, plus one div B pass "
                      f"({pass_s:.1f} s, charged as 1/10 per main step, the GPU arm's cadence): {sec:.1f} s per step"}


# ------------------------------------------------------------ reference arm
def run_reference(args):
    ws, rank, _ = dist_env()
    if rank != 0:
        return None
    from g3m3_gb300.state import make_config
    st = make_config("nested", divb_every=0)
    steps, warmup = min(args.steps, 2), min(args.warmup, 1)
    v, sec, kind, threads, pass_s = _reference_steps(steps, warmup)
    what = ("the reference's main loop (its Fortran translated to C, OpenMP loops with private temporaries)"
            if kind == "reference" else "the oracle's restatement of the reference (OpenMP)")
    sample = (f"{steps} main step(s) of the nested 5-box grid after {warmup} warm-up, {what}, plus one div B "
              f"pass of the reference's own routines ({pass_s:.1f} s, charged as 1/10 per main step: the GPU "
              f"arm's div B cadence, so both arms run the same work per step)")
    return {"impl": "reference", "metric": METRIC, "value": v, "unit": "cell-updates/s", "n_gpus": ws,
            "steps": steps, "warmup": warmup, "ms_per_step": sec * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic", "config": {"workload": WORKLOAD, "boxes": st.params.n_grids,
                                            "box": [st.params.nx, st.params.ny, st.params.nz],
                                            "cells_per_box": st.params.nx * st.params.ny * st.params.nz,
                                            "divb_every": make_config("nested").params.divb_every,
                                            "parallelism": f"host OpenMP, {threads} threads"},
            "cpu_baseline": {"value": v, "unit": "cell-updates/s", "cores": threads, "kind": kind,
                             "sample": sample},
            "e2e": {"value": v, "unit": "cell-updates/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def run_adjoint_profile():
    """The small case of the adjoint's ncu captures: 10 main steps of 3
    nested 65x65x33 boxes (a 2.6 GB tape), checkpoints every 2, 50
    samples; one forward, one backward."""
    from g3m3_gb300.adjoint import MisfitRun, line_samples, wind_of
    from g3m3_gb300.api import Context, Model
    from g3m3_gb300.state import make_config
    st = make_config("nested", limit=32, n_grids=3)
    with Context(0) as ctx:
        m = Model(ctx, st)
        run = MisfitRun(m, st, 10, line_samples(st, 10, n=50), checkpoint_every=2)
        loss = run.loss(wind_of(st.params))
        run.adj.backward(state=False)
        print(json.dumps({"adjoint_profile_case": "3 nested boxes 65x65x33, 10 main steps, checkpoints every 2",
                          "loss": loss, "backward_phases_s": run.adj.phases()[:3]}))
        run.adj.close()
        m.close()


def run_profile(args):
    """One 121x121x61 box (state > L2, < 1 GB on the device), or the first
    --profile-boxes of the nested grid (2: about 1.5 GB, with flanks and
    corer), stepped with host-loop launches; the small case of the ncu
    captures."""
    from g3m3_gb300.api import Context, Model
    from g3m3_gb300.state import make_config
    st = make_config("nested", n_grids=args.profile_boxes, divb_every=0)
    with Context(0) as ctx:
        m = Model(ctx, st)
        variant = m.autotune()   # 24 flux-correction launches, as in the benchmark
        if args.contracted:
            m.ctx.check(m.L.g3m3_model_set_contracted(m.h, 1))
        m.init_steps()
        m.run(args.warmup + args.steps, graph=False)
        k, _ = m.stats()
        print(json.dumps({"profile_case": f"{args.profile_boxes} box(es) 121x121x61", "main_steps": args.warmup + args.steps,
                          "kernel_launches": k, "fcsmooth_variant": variant, "contracted": bool(args.contracted)}))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--no-batched", action="store_true", help="skip the 16-member ensemble leg")
    ap.add_argument("--no-adjoint", action="store_true", help="skip the adjoint legs (3 x 97x97x49 boxes; 8 members of 5 x 121x121x61)")
    ap.add_argument("--adjoint-only", action="store_true", help="run only the adjoint leg and print its block")
    ap.add_argument("--profile", action="store_true",
                    help="profiling case for ncu: one 121x121x61 box, warmup+steps main steps, host-loop launches")
    ap.add_argument("--adjoint-profile", action="store_true",
                    help="profiling case for ncu: the adjoint of 10 main steps on 3 nested 65x65x33 boxes, "
                         "checkpoints every 2, one forward and one backward")
    ap.add_argument("--contracted", action="store_true",
                    help="with --profile: the contracted flavour of push_ion")
    ap.add_argument("--profile-boxes", type=int, default=1,
                    help="nested 121x121x61 boxes of the profiling case (2: flanks and corer run too)")
    args = ap.parse_args()
    if args.profile:
        return run_profile(args)
    if args.adjoint_profile:
        return run_adjoint_profile()
    if args.adjoint_only:
        print(json.dumps({"adjoint": run_adjoint(0)}), flush=True)
        return None
    line = run_reference(args) if args.impl == "reference" else run_ours(args)
    if line is not None:
        print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
