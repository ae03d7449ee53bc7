"""Water sources and init-file scenes on the CUDA path, against the oracle.

Per-step replay as in test_gpu_parity: the same state goes into fsim_step
and the oracle's RunOneStep (AddSources before the move, DeleteSources after
it, time += dt); particles, their order and keys must match bit for bit
(source draws come from the shared counter-based generator), fields within
the 1e-5 bar.
"""
from pathlib import Path

import numpy as np
import pytest

import fsim
from _util import FIELD_RTOL, assert_marker, assert_vec_field, rel_l2
from oracle.oracle import OracleSim

pytestmark = pytest.mark.gpu

SCENE = (Path(__file__).resolve().parent / "scenes" / "reservoir_sources.txt").read_text()
OSC = """fluid : 0
boundary : 0
fluid-cube : 0.0 0.0 0.0, 1.0 0.25 1.0, 0 0 0
source-oscillating : 0.25 0.5 0.25, 0.5 0.75 0.5, 0.5 0.5 0.5, 0.75 0.75 0.75, 0.02, 1 -1 0, -1 -1 1, 0.05
"""


def _pair(text, n):
    dims = (n, n, n)
    sim, sc = fsim.Simulation.from_scene(text, dims, seed=3)
    orc = OracleSim(dims, sc.boundary, sc.gravity, tuple(sc.force), 0.95, 8)
    for q in range(sc.nsolids):
        orc.add_solid_cuboid(tuple(sc.solid_lo[q]), tuple(sc.solid_hi[q]))
    for q in range(sc.nsources):
        orc.add_source(sc.sources[q])
    orc.seed_scene(sc, 3)
    return sim, orc


@pytest.mark.parametrize("text", [SCENE, OSC], ids=["static+timed", "oscillating"])
def test_scene_step_replay_with_sources(text):
    sim, orc = _pair(text, 32)
    p1, v1, g1 = sim.download_particles()
    p0, v0, g0 = orc.particles()
    assert np.array_equal(p1, p0) and np.array_equal(v1, v0)
    prm = fsim.pcg_params(fsim.PCG_RELATIVE, fsim.PREC_MIXED, 2000, tolerance=1e-10,
                          inner_tolerance=1e-4)
    counts = []
    for k in range(4):
        dt = 0.01
        st = sim.step(dt, prm)
        orc.step(dt, mode=1, precision=2, max_iterations=20000, tol=1e-13)
        assert sim.time == pytest.approx(orc.time)
        p1, v1, g1 = sim.download_particles()
        p0, v0, g0 = orc.particles()
        assert p1.shape == p0.shape and st.particles == p0.shape[0], k
        assert np.array_equal(p1, p0), f"step {k}: positions / order differ"
        assert rel_l2(v1, v0) <= FIELD_RTOL and rel_l2(g1, g0) <= FIELD_RTOL
        assert_marker(sim, orc, f"step {k} marker")
        assert_vec_field(sim, orc, fsim.FIELD_VELOCITY, FIELD_RTOL, label=f"step {k} velocity")
        a, _ = sim.field(fsim.FIELD_PRESSURE)
        b, _ = orc.field(4)
        assert rel_l2(a, b) <= FIELD_RTOL
        counts.append(p0.shape[0])
        sim.upload_particles(p0, v0, g0)
    assert counts[-1] != counts[0] or len(set(counts)) > 1  # the sources changed the fluid
    sim.close()


def test_per_stage_sources_match_oracle():
    sim, orc = _pair(SCENE, 32)
    sim.add_contribution_from_sources(0.0)
    orc.add_contribution_from_sources(0.0)
    sim.move_particles(0.01)
    orc.move_particles(0.01)
    sim.delete_fluid_in_sources(0.0)
    orc.delete_fluid_in_sources(0.0)
    p1, v1, g1 = sim.download_particles()
    p0, v0, g0 = orc.particles()
    assert np.array_equal(p1, p0) and np.array_equal(v1, v0) and np.array_equal(g1, g0)
    sim.close()
