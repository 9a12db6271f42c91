"""FP64 central differences of the virtual-spacecraft misfit of the adjoint
benchmark (TEST INFRASTRUCTURE): 50 main steps of 3 nested boxes of
97x97x49, div B every 10 steps, 200 samples along the seeded line of
g3m3_gb300.adjoint.line_samples.  The time-step schedule is the oracle's
FP32 run's (the reference's FP32 bits); the misfit is evaluated with the
oracle's FP64 build under that schedule.

The differences are taken in the eight wind-face parameters w (srho, spx,
spy, spz, spress, sbx/sby/sbz_wind), which the reference holds in FP32:
w_k +- h_k rounded to FP32, divided by the rounded difference, so that the
step is exact.  h_k = h_rel * scale_k, scale_k the magnitude of the
parameter's group (srho; |sp|; spress; |sb|).  The gradient with respect
to the upstream conditions u = (n, v, B) follows by the chain rule through
the exact Jacobian of g3m3_gb300.adjoint.upstream_wind.  Two steps are
taken: h_rel = 1e-4 (the benchmark's stated step) and 1e-5; the misfit has kinks
(limiter and guard branches), and the difference quotients of the two
steps differ by more than the smaller one differs from the adjoint.

With --jvp, the existing file's schedule is kept and the exact directional
derivatives of the same FP64 misfit along each parameter are added to it
("grad_wind_jvp_fp64"), from the FP64 build run in forward-mode dual
numbers (oracle/dual.h): the derivative the difference quotients
approximate, with no step.

Writes adjoint_fd_3x97x97x49.json beside this file; the GPU test
tests/test_adjoint_gpu.py::test_nested_97_gradient compares the library's
adjoint with it.

    python tests/golden/make_adjoint_fd.py [--params 0,1,..] [--hrel 1e-4,1e-5]
                                           [--divb-every N] [--errlim E] [--out NAME] [--jvp]
"""
import json
import os
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path[:0] = [ROOT, os.path.join(ROOT, "tests")]

import numpy as np  # noqa: E402

import _adjoint_ref as R  # noqa: E402

NSTEPS = 50


def adjoint_grid(**over):
    from g3m3_gb300.state import make_config
    return make_config("nested", limit=48, n_grids=3, **over)


def wind_steps(w, h_rel):
    """The FP32-exact pairs (w_k + h, w_k - h) of every parameter."""
    sp = np.linalg.norm(w[1:4])
    sb = np.linalg.norm(w[5:8])
    scale = np.array([abs(w[0]), sp, sp, sp, abs(w[4]), sb, sb, sb])
    out = []
    for k in range(8):
        h = h_rel * scale[k]
        out.append((float(np.float32(w[k] + h)), float(np.float32(w[k] - h))))
    return out


def main(argv=()):
    opts = dict(a.split("=", 1) for a in argv if a.startswith("--") and "=" in a)
    over = {}
    if "--divb-every" in opts:
        over["divb_every"] = int(opts["--divb-every"])
    if "--errlim" in opts:
        over["divb_errlim"] = float(opts["--errlim"])
    comps = [int(x) for x in opts["--params"].split(",")] if "--params" in opts else list(range(8))
    hrels = [float(x) for x in opts["--hrel"].split(",")] if "--hrel" in opts else [1e-4, 1e-5]
    name = opts.get("--out", "adjoint_fd_3x97x97x49.json")
    if "--jvp" in argv:
        return add_jvp(name, comps)
    from g3m3_gb300.adjoint import line_samples, wind_of
    from oracle.oracle import OracleModel
    st = adjoint_grid(**over)
    samples = line_samples(st, NSTEPS, n=200)
    om = OracleModel(st, omp=True)
    om.init_steps()
    sch = []
    t0 = time.time()
    for _ in range(NSTEPS):
        sch.append([float(om.s.t_stepnew[b]) for b in range(st.params.n_grids)])
        assert om.main_step() == 0
    print(f"schedule: {time.time() - t0:.0f} s", flush=True)
    w0 = wind_of(st.params)
    L0 = R.oracle_loss(st, w0, sch, samples)
    print(f"loss {L0:.10e}", flush=True)
    grads = {}
    for hr in hrels:
        pairs = wind_steps(w0, hr)
        g = {}
        for k in comps:
            wp, wm = w0.copy(), w0.copy()
            wp[k], wm[k] = pairs[k]
            t0 = time.time()
            g[k] = (R.oracle_loss(st, wp, sch, samples) - R.oracle_loss(st, wm, sch, samples)) / (wp[k] - wm[k])
            print(f"h_rel {hr:g} w[{k}]: {g[k]:.10e} ({time.time() - t0:.0f} s)", flush=True)
        grads[f"{hr:g}"] = [g.get(k) for k in range(8)]
    out = {"config": "3 nested boxes 97x97x49, 50 main steps, div B every %d (errlim %g), 200 line samples"
                     % (st.params.divb_every, st.params.divb_errlim),
           "wind": w0.tolist(), "loss_fp64": L0, "grad_wind_fd_fp64": grads, "schedule": sch}
    with open(os.path.join(HERE, name), "w") as fh:
        json.dump(out, fh, indent=1)
    print("written")


def add_jvp(name, comps):
    from g3m3_gb300.adjoint import line_samples, wind_of
    path = os.path.join(HERE, name)
    fx = json.load(open(path))
    st = adjoint_grid()
    samples = line_samples(st, NSTEPS, n=200)
    w0 = wind_of(st.params)
    assert np.array_equal(w0, np.array(fx["wind"]))
    jvp = fx.get("grad_wind_jvp_fp64", [None] * 8)
    for k in comps:
        e = np.zeros(8)
        e[k] = 1.0
        t0 = time.time()
        loss, jvp[k] = R.oracle_jvp(st, w0, fx["schedule"], samples, wind_tangent=e)
        print(f"w[{k}]: {jvp[k]:.10e} (loss {loss:.10e}, {time.time() - t0:.0f} s)", flush=True)
        fx["grad_wind_jvp_fp64"] = jvp
        with open(path, "w") as fh:
            json.dump(fx, fh, indent=1)
    print("written")


if __name__ == "__main__":
    main(sys.argv[1:])
