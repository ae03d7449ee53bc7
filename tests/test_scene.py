"""Init-file scenes: the reference's configuration format, scaled as its
driver scales it (FlipApp::ParseSimulationConfiguration, common/flip_app.cc:
159-251; FlipDriver::Initialize, common/flip_app_sim.cc:70-183), and the
water sources of the step (common/flip_simulation.cc:1207-1281) on the
oracle.  The GPU path of the same scenes is checked against the oracle in
tests/test_gpu_sources.py.
"""
from pathlib import Path

import numpy as np
import pytest

import fsim
from oracle.oracle import OracleSim

SCENE = (Path(__file__).resolve().parent / "scenes" / "reservoir_sources.txt").read_text()


def test_defaults():
    sc = fsim.parse_scene("", (64, 64, 64))
    assert (sc.fluid, sc.boundary, sc.nsolids, sc.nsources) == (1, 0, 0, 0)
    # scaled gravity = 9.8 * 64 / 128, force (0,1,0) * scaled gravity
    g = np.float32(np.float64(np.float32(9.8)) * (64.0 / 128.0))
    assert sc.gravity == g and tuple(sc.force) == (0.0, g, 0.0)
    # the sphere-drop preset: pool at N1/4 and a sphere at (N0/2, 3N1/4, 5N2/8), r = (N0/4)*0.8
    p = sc.passes[0]
    assert sc.npasses == 1 and p.nshapes == 2
    assert p.shapes[0].kind == fsim.SHAPE_POOL and p.shapes[0].a[1] == 16.0
    assert p.shapes[1].kind == fsim.SHAPE_SPHERE
    assert tuple(p.shapes[1].a) == (32.0, 48.0, 40.0)
    assert p.shapes[1].r == np.float32(16 * 0.8)


def test_dam_preset():
    sc = fsim.parse_scene("fluid : 2", (32, 64, 16))
    sh = sc.passes[0].shapes[0]
    assert sc.npasses == 1 and sh.kind == fsim.SHAPE_CUBOID
    assert tuple(sh.a) == (0.0, 0.0, 0.0) and tuple(sh.b) == (7.0, 47.0, 15.0)


def test_scene_file_is_scaled_as_the_driver_does():
    sc = fsim.parse_scene(SCENE, (32, 32, 32))
    g = np.float32(np.float64(np.float32(4.0)) * (32.0 / 128.0))
    assert sc.boundary == 1 and sc.fluid == 0 and sc.gravity == g
    assert sc.npasses == 2 and sc.nsolids == 1 and sc.nsources == 2
    cube, sphere = sc.passes[0].shapes[0], sc.passes[1].shapes[0]
    # additional cube: scaled, end lowered by 1
    assert tuple(cube.a) == (16.0, 4.0, 16.0) and tuple(cube.b) == (31.0, 11.0, 31.0)
    assert tuple(sphere.a) == (8.0, np.float32(0.7) * 32, 8.0) and sphere.r == 4.0
    assert tuple(sc.passes[1].velocity) == (0.0, np.float32(-0.5) * g, 0.0)
    # solid: get_coord_bbox of the scaled cube
    assert tuple(sc.solid_lo[0]) == (16, 3, 16) and tuple(sc.solid_hi[0]) == (31, 3, 31)
    s0, s1 = sc.sources[0], sc.sources[1]
    assert tuple(s0.lo) == (0.0, 24.0, 12.0) and tuple(s0.hi) == (4.0, 28.0, 16.0)
    assert tuple(s0.velocity) == (np.float32(2.0) * g, 0.0, 0.0) and s0.timed == 0
    assert s1.timed == 1 and s1.start_time == 0.0 and s1.end_time == np.float32(0.05)


def test_oscillating_source_line():
    sc = fsim.parse_scene("source-oscillating : 0 0 0, .25 .25 .25, .5 .5 .5, 1 1 1, 2.0, "
                          "1 0 0, 0 1 0, 3.0", (16, 16, 16))
    s = sc.sources[0]
    assert s.box_oscillating == 1 and s.velocity_oscillating == 1
    assert s.box_period == 2.0 and s.velocity_period == 3.0
    assert tuple(s.lo2) == (8.0, 8.0, 8.0) and tuple(s.hi2) == (16.0, 16.0, 16.0)


@pytest.mark.parametrize("text, code", [("fluid-cube : 0 0 0, 1 1", 1), ("boundary : 3", 1),
                                        ("solid : 0.01 0 0, 0.5 0.5 0.5", 1)])
def test_rejects(text, code):
    with pytest.raises(fsim.FsimError) as e:
        fsim.parse_scene(text, (32, 32, 32))
    assert e.value.code == code


def _oracle(sc, dims, seed=0):
    orc = OracleSim(dims, sc.boundary, sc.gravity, tuple(sc.force), 0.95, 8)
    for q in range(sc.nsolids):
        orc.add_solid_cuboid(tuple(sc.solid_lo[q]), tuple(sc.solid_hi[q]))
    for q in range(sc.nsources):
        orc.add_source(sc.sources[q])
    orc.seed_scene(sc, seed)
    return orc


def test_oracle_sources_add_and_delete():
    dims = (32, 32, 32)
    sc = fsim.parse_scene("fluid : 0\nsource-static : 0.25 0.5 0.25, 0.5 0.75 0.5, 0 -1 0",
                          dims)
    orc = _oracle(sc, dims)
    assert orc.particle_count() == 0
    orc.add_contribution_from_sources(0.0)
    pos, vel, gvel = orc.particles()
    # get_box: [8,16] x [16,24] x [8,16] with the end lowered by 1 -> [8,15]..; kept draws lie inside
    assert len(pos) > 0
    assert (pos >= [8, 16, 8]).all() and (pos <= [15, 23, 15]).all()
    assert np.all(vel == np.float32(-1.0) * sc.gravity * np.array([0, 1, 0], np.float32) + 0)
    assert np.array_equal(vel, gvel)
    keys = orc.keys()
    assert np.all(np.diff(keys.astype(np.int64)) >= 0)  # cell lists in iteration order
    n0 = len(pos)
    orc.delete_fluid_in_sources(0.0)
    assert orc.particle_count() == 0 and n0 > 0


def test_oracle_timed_source_and_time():
    dims = (32, 32, 32)
    sc = fsim.parse_scene(SCENE, dims)
    orc = _oracle(sc, dims)
    n_seed = orc.particle_count()
    assert orc.time == 0.0
    orc.step(0.01, mode=1, tol=1e-5)
    assert orc.time == pytest.approx(0.01)
    n1 = orc.particle_count()
    assert n1 > n_seed  # both sources poured in (the timed one is active until 0.05)
    orc.time = 1.0      # the timed source is off now; the static one keeps pouring
    orc.step(0.01, mode=1, tol=1e-5)
    assert orc.particle_count() > 0
