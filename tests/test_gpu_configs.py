"""GPU parity on the benchmark scenes, with the production solver.

The other parity tests solve the pressure to convergence on both sides.  Here
both sides run the solver the benchmark runs: fp32 Jacobi PCG to relative
residual 1e-5 (common/solver.cc:263-366, the loop of
common/solver_driver.cc:14-69 with a relative stopping rule), and dt from the
CFL rule of FlipDriver::WhileAndComputeDt (common/flip_app_sim.cc:357-428).

Replay: every step, the oracle's particle state is uploaded to the GPU, and
both sides run one RunOneStep (common/flip_app_sim.cc:211-254) with the same
dt.  Binning, positions, leaf topology and markers must be bit-exact.

Two fp32 solves that stop at a 1e-5 residual differ from the exact solution
by the solver's own error, and from each other by up to the sum of the two.
The GPU sums its dot products in a fixed tree order, the oracle in 100
serial chunks (r.r, r.z) and four serial lanes (p.Ap), so their CG iterates
drift apart by rounding (and the GPU, with the more accurate sums, stops in
fewer iterations).  Each step is therefore
also run with the pressure solved in fp64 to relative residual 1e-13 (the
converged step, "64"), and every field f (pressure, grid velocity, particle
velocity and PIC velocity) reports
  e_gpu = |f_gpu - f_64| / |f_64|,  e_orc = |f_orc - f_64| / |f_64|,
  d     = |f_gpu - f_orc| / |f_orc|.
The bars: e_gpu <= max(1e-5, 1.5 e_orc) -- the GPU step is within 1e-5 of
the converged step, or no further from it than the reference solver's own
fp32 step (1.5 leaves room for two different summation orders) -- and
d <= 1e-5 + e_gpu + e_orc.  The velocities right after the first steps are
a small difference of gravity and the pressure gradient (the pool is nearly
hydrostatic), so there a pressure error of a few 1e-6 shows as a few 1e-5 in
the velocities on both sides alike.
"""
import json
import os

import numpy as np
import pytest

import fsim
from _util import FIELD_RTOL, assert_marker, make_gpu, make_oracle, rel_l2
from oracle import oracle as O
from oracle.oracle import OracleSim, compute_dt

pytestmark = pytest.mark.gpu

FRAME_STEP = float(np.float32(1.0) / np.float32(30.0))


def _next_dt(inv, t_in):
    dt, t = compute_dt(inv, 1, FRAME_STEP, t_in)
    if t + 1e-5 >= FRAME_STEP:  # the frame's While loop ends; ResetDt
        t = 0.0
    return dt, t


def _replay(n, scene, steps, max_iterations, gpu_ref=False):
    """Per-step figures (module docstring) of the GPU step and the oracle
    step against the converged step.  The converged step comes from the
    oracle with the FP64 solver, or with gpu_ref from the GPU with its FP64
    solver (checked against the oracle's fp64 solve in tests/test_gpu_pcg.py),
    which keeps the large cases within minutes.  The oracle runs on every
    host thread (its results do not depend on the thread count)."""
    O.set_threads(os.cpu_count() or 1)
    try:
        return _replay_steps(n, scene, steps, max_iterations, gpu_ref)
    finally:
        O.set_threads(1)


def _replay_steps(n, scene, steps, max_iterations, gpu_ref):
    orc = make_oracle(n, scene)
    sim = make_gpu(orc)
    g, f = fsim.physical_gravity(n)
    if gpu_ref:
        ref = fsim.Simulation((n, n, n), fsim.BOUNDARY_BOX, g, f, 0.95, 8)
    else:
        ref = OracleSim((n, n, n), fsim.BOUNDARY_BOX, g, f, 0.95, 8)
    prm = fsim.pcg_params(fsim.PCG_RELATIVE, fsim.PREC_FP32, max_iterations, tolerance=1e-5)
    prm64 = fsim.pcg_params(fsim.PCG_RELATIVE, fsim.PREC_FP64, 40000, tolerance=1e-13)
    t_in = 0.0
    rows = []
    for k in range(steps):
        dt, t_in = _next_dt(orc.cfl(), t_in)
        p0, v0, g0 = orc.particles()
        sim.upload_particles(p0, v0, g0)
        if gpu_ref:
            ref.upload_particles(p0, v0, g0)
            s64 = ref.step(dt, prm64).pcg
        else:
            ref.set_particles(p0, v0, g0)
            s64 = ref.step(dt, mode=1, precision=2, max_iterations=40000, tol=1e-13)
        st = sim.step(dt, prm)
        ost = orc.step(dt, mode=1, precision=0, max_iterations=max_iterations, tol=1e-5)
        assert st.pcg.status == 0 and ost.status == 0 and s64.status == 0, k
        p1, v1, g1 = sim.download_particles()
        p0, v0, g0 = orc.particles()
        p2, v2, g2 = (ref.download_particles() if gpu_ref else ref.particles())
        assert p1.shape == p0.shape and st.particles == p0.shape[0], k
        assert np.array_equal(p1, p0), f"step {k}: positions differ"
        assert np.array_equal(p2, p0), f"step {k}: positions of the converged step differ"
        assert np.array_equal(sim.leaves(), orc.leaves()), f"step {k}: leaves differ"
        assert_marker(sim, orc, f"step {k} marker")
        row = dict(step=k, dt=float(dt), particles=int(p0.shape[0]),
                   unknowns=int(st.pcg.n_rows), iters_gpu=int(st.pcg.iterations),
                   iters_orc=int(ost.iterations), iters_64=int(s64.iterations))
        fields = {}
        for name, which in (("p", fsim.FIELD_PRESSURE), ("u", fsim.FIELD_VELOCITY)):
            a, aa = sim.field(which)
            b, ba = orc.field(which)
            c, _ = ref.field(which)
            assert np.array_equal(aa, ba), f"step {k}: {name} active set differs"
            fields[name] = (a, b, c)
        fields["vel"] = (v1, v0, v2)
        fields["gvel"] = (g1, g0, g2)
        for name, (a, b, c) in fields.items():
            row[name] = dict(d=rel_l2(a, b), e_gpu=rel_l2(a, c), e_orc=rel_l2(b, c))
        rows.append(row)
    sim.close()
    orc.close()
    ref.close()
    return rows


def _check(rows, label):
    out = os.environ.get("FSIM_PARITY_REPORT")
    if out:
        with open(out, "a") as fh:
            fh.write(json.dumps({"case": label, "rows": rows}) + "\n")
    for r in rows:
        print(label, json.dumps(r))
    for r in rows:
        # the GPU's tree-ordered sums converge at least as fast as the chunked ones
        assert r["iters_gpu"] <= 1.1 * r["iters_orc"] + 2, r
        for name in ("p", "u", "vel", "gvel"):
            e = r[name]
            assert e["e_gpu"] <= max(FIELD_RTOL, 1.5 * e["e_orc"]), (name, r)
            assert e["d"] <= FIELD_RTOL + e["e_gpu"] + e["e_orc"], (name, r)


def test_sphere_drop_64_twenty_steps():
    """The 64^3 sphere drop (r 0.15 at (0.5, 0.7, 0.5) over a pool y < 0.2),
    8 particles per cell from seed 0, walls, 20 steps, PCG relative 1e-5 with
    at most 200 iterations."""
    _check(_replay(64, "sphere_drop", 20, 200), "sphere_drop_64")


def test_dam_break_256_three_steps():
    """The 256^3 dam break (x < 0.4, y < 0.6), 32.2 M particles, the
    first three steps, PCG relative 1e-5 (max 1500)."""
    _check(_replay(256, "dam_break", 3, 1500, gpu_ref=True), "dam_break_256")


def test_multidam_512_one_step():
    """The 512^3 multi-dam of the mixed-precision comparison (four
    0.2 x 0.5 x 0.2 blocks at the x/z quadrant corners over a pool
    y < 0.05), 131 M particles, about 14% of the leaves active, first step,
    with the benchmark's fp32 solver (PCG relative 1e-5, max 1500)."""
    _check(_replay(512, "multidam", 1, 1500, gpu_ref=True), "multidam_512")
