"""Shared helpers for the parity tests (CUDA path vs the CPU oracle)."""
from __future__ import annotations

import numpy as np

import fsim
from oracle.oracle import OracleSim

# Tolerance of the bar: velocities and pressures within 1e-5 relative L2.
FIELD_RTOL = 1e-5


def rel_l2(a, b) -> float:
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    den = np.linalg.norm(b)
    return float(np.linalg.norm(a - b) / (den if den > 0 else 1.0))


def make_oracle(n, scene="sphere_drop", boundary=fsim.BOUNDARY_BOX, solids=(), noise=0.0,
                seed=0, nppc=8, flip=0.95):
    dims = (n, n, n) if np.isscalar(n) else tuple(n)
    g, f = fsim.physical_gravity(dims[1])
    orc = OracleSim(dims, boundary, g, f, flip, nppc)
    for lo, hi in solids:
        orc.add_solid_cuboid(lo, hi)
    orc.seed(fsim.scene_passes(scene, dims[1]), seed=seed)
    if noise:
        pos, vel, gvel = orc.particles()
        rng = np.random.default_rng(seed + 1)
        vel = (vel + rng.normal(0.0, noise, vel.shape)).astype(np.float32)
        orc.set_particles(pos, vel, vel.copy())
    return orc


def make_gpu(orc: OracleSim, boundary=fsim.BOUNDARY_BOX, solids=(), nppc=8, flip=0.95):
    dims = orc.dims
    g, f = fsim.physical_gravity(dims[1])
    sim = fsim.Simulation(dims, boundary, g, f, flip, nppc)
    for lo, hi in solids:
        sim.add_solid_cuboid(lo, hi)
    pos, vel, gvel = orc.particles()
    sim.upload_particles(pos, vel, gvel)
    return sim


def assert_vec_field(sim, orc, which, rtol=FIELD_RTOL, exact_mask=True, label=""):
    a, aa = sim.field(which)
    b, ba = orc.field(which)
    if exact_mask:
        diff = np.argwhere(aa != ba)
        assert diff.size == 0, f"{label} active mask differs at {diff[:5]} (n={len(diff)})"
    e = rel_l2(a, b)
    assert e <= rtol, f"{label} rel L2 {e:.3e} > {rtol}"
    return e


def assert_marker(sim, orc, label=""):
    a, aa = sim.marker()
    b, ba = orc.marker()
    diff = np.argwhere(a != b)
    assert diff.size == 0, f"{label} marker differs at {diff[:5]} (n={len(diff)})"
    assert np.array_equal(aa, ba), f"{label} marker active mask differs"
