"""Generates the regression fixtures in this folder from the oracle.

The reference publishes no golden vectors and cannot be built here, so these
fixtures pin the oracle itself: a change to the CPU restatement that moves any
of these numbers shows up as a failing test.  Each fixture is a small seeded
scene stepped through the reference's RunOneStep order on the oracle:

  sphere_drop_16.npz  16^3 sphere drop (walls), 8 particles per cell from
                      seed 0, velocities perturbed by N(0, 1.6^2) from seed 1
                      (the oracle's generator); 2 steps of dt = 1/120 with
                      fp32 Jacobi PCG to relative residual 1e-5
  dam_tank_16.npz     16^3 dam break in a tank (open top) with one interior
                      cuboid solid; 2 steps of dt = 1/100, same solver

Stored: the initial particles, the particles after the last step (positions,
velocities, grid velocities) and their keys, the pressure and velocity fields
and markers after the last step, and the PCG iterations of each step.

Run:  python tests/golden/make_golden.py
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parents[1]
sys.path.insert(0, str(ROOT / "fluid-sim-lb_gb300"))
sys.path.insert(0, str(ROOT))

import fsim  # noqa: E402
from oracle.oracle import OracleSim  # noqa: E402

CASES = {
    "sphere_drop_16": dict(n=16, scene="sphere_drop", boundary=fsim.BOUNDARY_BOX, solids=(),
                           sigma=1.6, dt=1.0 / 120.0, steps=2),
    "dam_tank_16": dict(n=16, scene="dam_break", boundary=fsim.BOUNDARY_TANK,
                        solids=(((9, 0, 5), (10, 4, 10)),), sigma=0.0, dt=1.0 / 100.0, steps=2),
}


def build(case: dict) -> OracleSim:
    n = case["n"]
    g, f = fsim.physical_gravity(n)
    orc = OracleSim((n, n, n), case["boundary"], g, f, 0.95, 8)
    for lo, hi in case["solids"]:
        orc.add_solid_cuboid(lo, hi)
    orc.seed(fsim.scene_passes(case["scene"], n), seed=0)
    if case["sigma"]:
        orc.perturb_velocities(case["sigma"], 1)
    return orc


def run(case: dict) -> dict:
    orc = build(case)
    out = {}
    pos, vel, gvel = orc.particles()
    out["pos0"], out["vel0"], out["gvel0"] = pos, vel, gvel
    iters = []
    for k in range(case["steps"]):
        st = orc.step(case["dt"], mode=fsim.PCG_RELATIVE, precision=fsim.PREC_FP32,
                      max_iterations=1500, tol=1e-5)
        iters.append(st.iterations)
    pos, vel, gvel = orc.particles()
    out["pos"], out["vel"], out["gvel"] = pos, vel, gvel
    out["keys"] = orc.keys()
    out["pressure"], out["pressure_active"] = orc.field(fsim.FIELD_PRESSURE)
    out["velocity"], out["velocity_active"] = orc.field(fsim.FIELD_VELOCITY)
    out["marker"], _ = orc.marker()
    out["pcg_iterations"] = np.array(iters, np.int32)
    orc.close()
    return out


def main():
    for name, case in CASES.items():
        np.savez_compressed(HERE / f"{name}.npz", **run(case))
        print("wrote", name)


if __name__ == "__main__":
    main()
