"""FP64 central differences of the virtual-spacecraft misfit of BASELINE
config 3 (TEST INFRASTRUCTURE): 50 main steps of 3 nested boxes of
97x97x49, div B every 10 steps, 200 samples along the seeded line of
g3m3_gb300.adjoint.line_samples.  The time-step schedule is the oracle's
FP32 run's (the reference's FP32 bits); the misfit is evaluated with the
oracle's FP64 build under that schedule and differenced with respect to
the seven upstream conditions u = (n, vx, vy, vz, bx, by, bz) at
h = 1e-4 relative to the magnitude of u's density, speed and field.
Writes adjoint_fd_config3.json beside this file; the GPU test
tests/test_adjoint_gpu.py::test_config3_gradient compares the library's
adjoint with it.

    python tests/golden/make_adjoint_fd.py
"""
import json
import math
import os
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path[:0] = [ROOT, os.path.join(ROOT, "tests")]

import numpy as np  # noqa: E402

import _adjoint_ref as R  # noqa: E402

NSTEPS = 50


def config3(**over):
    from g3m3_gb300.state import make_config
    return make_config("nested", limit=48, n_grids=3, **over)


def main(argv=()):
    """Options (diagnostics; the fixture is made without them):
    --divb-every N, --errlim E, --params 0,1,.. (components of u), --out NAME."""
    opts = dict(a.split("=", 1) for a in argv if a.startswith("--"))
    over = {}
    if "--divb-every" in opts:
        over["divb_every"] = int(opts["--divb-every"])
    if "--errlim" in opts:
        over["divb_errlim"] = float(opts["--errlim"])
    comps = [int(x) for x in opts["--params"].split(",")] if "--params" in opts else list(range(7))
    name = opts.get("--out", "adjoint_fd_config3.json")
    import torch
    from g3m3_gb300.adjoint import line_samples, upstream_wind
    from g3m3_gb300.state import CONFIGS, Setup
    from oracle.oracle import OracleModel
    st = config3(**over)
    setup = Setup(**dict(CONFIGS["nested"], limit=48, n_grids=3, **over))
    samples = line_samples(st, NSTEPS, n=200)
    om = OracleModel(st, omp=True)
    om.init_steps()
    sch = []
    t0 = time.time()
    for _ in range(NSTEPS):
        sch.append([float(om.s.t_stepnew[b]) for b in range(st.params.n_grids)])
        assert om.main_step() == 0
    print(f"schedule: {time.time() - t0:.0f} s", flush=True)
    w = setup.wind
    u0 = np.array([w.n_cm3, w.speed_kms, 0.0, 0.0, 0.0, w.b_nT * math.sin(w.clock_angle),
                   w.b_nT * math.cos(w.clock_angle)])
    scale = np.array([abs(u0[0])] + [np.linalg.norm(u0[1:4])] * 3 + [np.linalg.norm(u0[4:7])] * 3)
    wind = lambda u: upstream_wind(torch.tensor(u, dtype=torch.float64), setup).numpy()
    L0 = R.oracle_loss(st, wind(u0), sch, samples)
    print(f"loss {L0:.10e}", flush=True)
    fd = []
    for k in comps:
        h = 1e-4 * scale[k]
        up, um = u0.copy(), u0.copy()
        up[k] += h
        um[k] -= h
        t0 = time.time()
        g = (R.oracle_loss(st, wind(up), sch, samples) - R.oracle_loss(st, wind(um), sch, samples)) / (2 * h)
        fd.append(g)
        print(f"u[{k}]: {g:.8e} ({time.time() - t0:.0f} s)", flush=True)
    out = {"config": "3 nested boxes 97x97x49, 50 main steps, div B every %d (errlim %g), 200 line samples"
                     % (st.params.divb_every, st.params.divb_errlim), "components": comps,
           "u": u0.tolist(), "h_rel": 1e-4, "h": (1e-4 * scale).tolist(), "loss_fp64": L0,
           "grad_u_fd_fp64": fd, "schedule": sch}
    with open(os.path.join(HERE, name), "w") as fh:
        json.dump(out, fh, indent=1)
    print("written")


if __name__ == "__main__":
    main(sys.argv[1:])
