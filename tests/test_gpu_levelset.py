"""Particles to a narrow-band level set (fsim_particles_to_level_set) against
a NumPy restatement of the same method in the same float32 arithmetic:
phi = clamp(min_p |x - p| - R, -w, w) at the voxel points, then mean-filter
passes of the 3^3 neighbourhood over the band (the method of the reference's
projects/particles-to-levelset/convert.cc)."""
import numpy as np
import pytest

import fsim

pytestmark = pytest.mark.gpu


def _reference(pos, n, radius, w, iters):
    f32 = np.float32
    g = np.arange(-1, n + 1, dtype=f32)
    X, Y, Z = np.meshgrid(g, g, g, indexing="ij")
    phi = np.full(X.shape, np.inf, f32)
    for p in pos:
        dx, dy, dz = X - p[0], Y - p[1], Z - p[2]
        d2 = (dx * dx + dy * dy) + dz * dz
        phi = np.minimum(phi, np.sqrt(d2) - f32(radius))
    phi = np.clip(phi, -f32(w), f32(w))
    for _ in range(iters):
        pad = np.pad(phi, 1, constant_values=f32(w))
        s = np.zeros_like(phi)
        for a in range(3):
            for b in range(3):
                for c in range(3):
                    s = s + pad[a:a + phi.shape[0], b:b + phi.shape[1], c:c + phi.shape[2]]
        out = np.clip(s / f32(27.0), -f32(w), f32(w))
        phi = np.where(np.abs(phi) < f32(w), out, phi)
    return phi


@pytest.mark.parametrize("iters", [0, 1, 2])
def test_level_set_matches_restatement(iters):
    n = 16
    g, f = fsim.physical_gravity(n)
    sim = fsim.Simulation((n, n, n), fsim.BOUNDARY_BOX, g, f)
    sim.seed(fsim.scene_passes("sphere_drop", n), seed=0)
    pos, _, _ = sim.download_particles()
    phi, act = sim.level_set(3.0, 3.0, iters)
    ref = _reference(pos, n, 3.0, 3.0, iters)
    assert np.array_equal(phi, ref)
    assert np.array_equal(act, (np.abs(ref) < 3.0).astype(np.uint8))
    assert (phi < 0).any() and (phi == 3.0).any()
    sim.close()
