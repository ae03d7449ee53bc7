"""Regression fixtures (tests/golden/*.npz, made by tests/golden/make_golden.py).

The reference ships no golden vectors and cannot be built here; these
fixtures pin the oracle: the CPU test re-runs each case on the oracle and
requires every stored array bit for bit.  The GPU test runs the tank case on
the CUDA path from the same seed and checks it against the fixture.
"""
import sys
from pathlib import Path

import numpy as np
import pytest

import fsim
from _util import rel_l2

HERE = Path(__file__).resolve().parent / "golden"
sys.path.insert(0, str(HERE))
import make_golden  # noqa: E402


@pytest.mark.parametrize("name", sorted(make_golden.CASES))
def test_oracle_reproduces_fixture(name):
    ref = np.load(HERE / f"{name}.npz")
    got = make_golden.run(make_golden.CASES[name])
    assert sorted(got) == sorted(ref.files)
    for k in ref.files:
        assert np.array_equal(got[k], ref[k]), f"{name}: {k} differs from the fixture"


@pytest.mark.gpu
def test_gpu_tank_case_against_fixture():
    case = make_golden.CASES["dam_tank_16"]
    ref = np.load(HERE / "dam_tank_16.npz")
    n = case["n"]
    g, f = fsim.physical_gravity(n)
    sim = fsim.Simulation((n, n, n), case["boundary"], g, f, 0.95, 8)
    for lo, hi in case["solids"]:
        sim.add_solid_cuboid(lo, hi)
    sim.seed(fsim.scene_passes(case["scene"], n), seed=0)
    pos, vel, gvel = sim.download_particles()
    assert np.array_equal(pos, ref["pos0"]) and np.array_equal(vel, ref["vel0"])
    prm = fsim.pcg_params(fsim.PCG_RELATIVE, fsim.PREC_FP32, 1500, tolerance=1e-5)
    iters = [sim.step(case["dt"], prm).pcg.iterations for _ in range(case["steps"])]
    assert all(abs(a - b) <= 2 for a, b in zip(iters, ref["pcg_iterations"]))
    pos, vel, gvel = sim.download_particles()
    assert pos.shape == ref["pos"].shape
    assert rel_l2(pos, ref["pos"]) <= 1e-6
    # The GPU's fp32 solves stop at relative residual 1e-5 after other iteration counts
    # than the fixture's (different dot-product summation orders), so each differs from
    # the converged solve by the solver's own error; two such solves differ by up to the
    # sum of the two (tests/test_gpu_configs.py measures both errors).  1e-4 bounds that
    # sum here; bitwise topology is asserted above.
    assert rel_l2(vel, ref["vel"]) <= 1e-4
    p, pa = sim.field(fsim.FIELD_PRESSURE)
    assert np.array_equal(pa, ref["pressure_active"])
    assert rel_l2(p, ref["pressure"]) <= 1e-4
    sim.close()
