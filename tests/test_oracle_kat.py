"""Known-answer tests that pin the CPU oracle (no GPU).

The reference ships no tests or golden data and cannot be built here, so the
oracle's restatement is pinned against answers derived by hand from the
reference's code (file:line cited per test).
"""
import math

import numpy as np
import pytest

import fsim
from oracle.oracle import OracleSim, compute_dt, seed_uniform

N = 16


def _sim(n=N, boundary=0, g=None, force=None, flip=0.95):
    gg, ff = fsim.physical_gravity(n)
    return OracleSim((n, n, n), boundary, gg if g is None else g, ff if force is None else force,
                     flip, 8)


def _ix(n, i, j, k):
    return (i + 1, j + 1, k + 1)


def test_single_particle_p2g_weights():
    """ScatterWeight<D> (flip_simulation.cc:927-1009): for a particle at
    c + (0.25, 0.75, 0.5) the x-component's lower node is (c.x, c.y, c.z)
    (y: 0.75 >= 0.5; z: 0.5 >= 0.5, no shift) with fractions (0.25, 0.25, 0),
    so the weights are (1-x)(1-y)(1-z)... and sum to 1."""
    o = _sim()
    c = (5, 6, 7)
    pos = np.array([[c[0] + 0.25, c[1] + 0.75, c[2] + 0.5]], np.float32)
    vel = np.array([[1.5, -2.0, 3.0]], np.float32)
    o.set_particles(pos, vel, vel.copy())
    o.transfer_particles_to_grid()
    w, wa = o.field(2)
    v, va = o.field(0)
    for D in range(3):
        assert w[..., D].sum() == pytest.approx(1.0, abs=1e-6)
    # x component: nodes x in {5,6}, y in {6,7}, z in {7,8}; fractions 0.25,0.25,0
    wx = {(5, 6, 7): 0.75 * 0.75, (6, 6, 7): 0.25 * 0.75, (5, 7, 7): 0.75 * 0.25,
          (6, 7, 7): 0.25 * 0.25}
    for node, ww in wx.items():
        assert w[_ix(N, *node) + (0,)] == pytest.approx(ww, abs=1e-7)
    assert w[_ix(N, 5, 6, 8) + (0,)] == 0.0 and wa[_ix(N, 5, 6, 8)] == 1  # touched, weight 0
    # normalised velocity equals the particle's wherever the weight >= 1e-5
    for D in range(3):
        m = (wa == 1) & (w[..., D] > 1e-5)
        assert np.allclose(v[..., D][m], vel[0, D])
        assert np.all(v[..., D][(wa == 1) & (w[..., D] <= 1e-5)] == 0.0)
    # 3 components x 8 nodes, activation per voxel: 2x2x2 blocks overlap
    assert wa.sum() == (va == 1).sum()
    m, ma = o.marker()
    assert m[_ix(N, *c)] == fsim.FLUID and ma.sum() == 1


def test_p2g_normalisation_threshold_is_double_literal():
    """THRESH is the double 1e-5 (flip_simulation.cc:14,906-920): a weight sum
    of exactly float(1e-5) is below it, so that face velocity is zero."""
    assert float(np.float32(1e-5)) < 1e-5  # the float rounds below the double
    o = _sim()
    # x-component weight of node (1, 4, 4) for a particle at (x, 4.5, 4.5)
    # (cell (0,4,4), tangential fractions 0) is exactly x = float32(1e-5)
    x = np.float32(1e-5)
    pos = np.array([[x, 4.5, 4.5]], np.float32)
    vel = np.array([[2.0, 0.0, 0.0]], np.float32)
    o.set_particles(pos, vel, vel.copy())
    o.transfer_particles_to_grid()
    w, _ = o.field(2)
    v, _ = o.field(0)
    assert w[_ix(N, 1, 4, 4) + (0,)] == x
    assert v[_ix(N, 1, 4, 4) + (0,)] == 0.0
    assert v[_ix(N, 0, 4, 4) + (0,)] == pytest.approx(2.0)


def test_seeding_loop_semantics():
    """InitializePhiAndParticles (flip_simulation.cc:139-188): a draw is kept
    when phi(p) <= 0; a kept draw advances num_attempts twice; at most
    nparticles_per_cell per pass.  Re-derived here from the exported draw."""
    n = 12
    o = _sim(n)
    r = 3.3
    ctr = (6.0, 6.0, 6.0)
    passes = [fsim.SeedPass([fsim.SceneShape(fsim.SHAPE_SPHERE, a=ctr, r=r)])]
    o.seed(passes, seed=7)
    pos, _, _ = o.particles()

    def phi(p):
        d = np.array(p, np.float32) - np.array(ctr, np.float32)
        l2 = np.float32(np.float32(d[0] * d[0] + d[1] * d[1]) + d[2] * d[2])
        return np.float32(np.sqrt(l2)) - np.float32(r)

    expect = []
    for i in range(n):
        for j in range(n):
            for k in range(n):
                org = np.array([i, j, k], np.float32)
                if not phi(org + np.float32(0.5)) < 0:
                    continue
                cell = (i * n + j) * n + k
                att, draw, pi = 0, 0, 0
                while att < 32 and pi < 8:
                    p = [org[d] + np.float32(seed_uniform(7, 0, cell, draw, d)) for d in range(3)]
                    if not phi(p) > 0:
                        expect.append(p)
                        pi += 1
                        att += 1
                    att += 1
                    draw += 1
    expect = np.array(expect, np.float32)
    assert pos.shape == expect.shape
    key = lambda a: np.lexsort(a.T)
    assert np.array_equal(pos[key(pos)], expect[key(expect)])
    assert np.all([phi(p) <= 0 for p in pos[:200]])


def test_move_particles_clamping_and_deletion():
    """StepInGrid (particles.cc:512-545): below 0 -> pos 0, cell 0 (kept);
    at or above N -> pos N, cell N, which is solid under box walls and
    deleted (DeleteParticlesInSolids, :202-219); under the tank boundary the
    top cell N survives until DeleteOutsideParticles (:273-293)."""
    for boundary, kept_top in ((0, False), (1, True)):
        o = _sim(boundary=boundary)
        pos = np.array([[0.2, 5.5, 5.5], [8.5, N - 0.1, 8.5], [3.5, 3.5, 15.9]], np.float32)
        gv = np.array([[-10.0, 0.0, 0.0], [0.0, 10.0, 0.0], [0.0, 0.0, 10.0]], np.float32)
        o.set_particles(pos, gv, gv)
        o.move_particles(0.1)
        p, _, _ = o.particles()
        assert any((q[0] == 0.0 and q[1] == 5.5) for q in p)
        assert not any(q[2] == N for q in p)  # z wall is solid in both boundaries
        assert any(q[1] == N for q in p) == kept_top
        if kept_top:
            o.delete_outside_particles()
            p, _, _ = o.particles()
            assert not any(q[1] == N for q in p)


def test_iteration_key_order():
    """OpenVDB Tree3<T,3,3> iteration: root children (64^3 blocks) ordered
    lexicographically by origin, then x-major leaves, then x-major voxels."""
    n = 128
    o = _sim(n)
    cells = [(0, 0, 1), (0, 1, 0), (1, 0, 0), (0, 0, 8), (0, 8, 0), (8, 0, 0), (0, 0, 64),
             (0, 64, 0), (64, 0, 0), (63, 63, 63), (7, 7, 7), (9, 0, 0)]
    pos = np.array([[c[0] + 0.5, c[1] + 0.5, c[2] + 0.5] for c in cells], np.float32)
    o.set_particles(pos, np.zeros_like(pos), np.zeros_like(pos))
    got = [tuple(int(x) for x in np.floor(p)) for p in o.particles()[0]]

    def vdb_key(c):
        return (tuple(x // 64 for x in c), tuple((x // 8) % 8 for x in c), tuple(x % 8 for x in c))

    assert got == sorted(cells, key=vdb_key)


def _laplacian(marker):
    """Dense matrix of Solver::CreateLaplacianMatrix (solver.cc:198-233)."""
    idx = {}
    shp = marker.shape
    for i in range(shp[0]):
        for j in range(shp[1]):
            for k in range(shp[2]):
                if marker[i, j, k] == 1:
                    idx[(i, j, k)] = len(idx)
    A = np.zeros((len(idx), len(idx)))
    for c, r in idx.items():
        for d in ((-1, 0, 0), (1, 0, 0), (0, -1, 0), (0, 1, 0), (0, 0, -1), (0, 0, 1)):
            nb = tuple(c[a] + d[a] for a in range(3))
            m = marker[nb] if all(0 <= nb[a] < shp[a] for a in range(3)) else 0
            if m != 2:
                A[r, r] += 1
            if m == 1:
                A[r, idx[nb]] = -1
    return A, idx


def test_pcg_matches_dense_solve():
    n = 10
    o = _sim(n)
    rng = np.random.default_rng(0)
    shp = (n + 2,) * 3
    marker = np.zeros(shp, np.int32)
    inner = rng.random((n, n, n)) < 0.55
    marker[1:-1, 1:-1, 1:-1] = np.where(inner, 1, 0)
    marker[1:-1, 1:4, 1:-1] = 1  # a connected pool touching walls
    marker[0, :, :] = marker[-1, :, :] = 2
    marker[:, 0, :] = marker[:, -1, :] = 2
    marker[:, :, 0] = marker[:, :, -1] = 2
    marker[4:6, 3, 4:6] = 2  # interior solid cells
    div = np.where(marker == 1, rng.normal(size=shp), 0).astype(np.float32)
    o.set_marker(marker)
    o.set_divergence(div)
    st = o.pcg_solve(mode=1, precision=2, max_iterations=10000, tol=1e-14)
    assert st.status == 0
    A, idx = _laplacian(marker)
    b = np.array([div[c] for c in idx], np.float64)
    x = np.linalg.lstsq(A, b, rcond=None)[0] if np.linalg.matrix_rank(A) < len(b) else \
        np.linalg.solve(A, b)
    got = o.pressure_f64()
    xs = np.array([got[c] for c in idx])
    assert np.linalg.norm(A @ xs - b) <= 1e-10 * np.linalg.norm(b)
    assert np.allclose(xs, x, rtol=1e-8, atol=1e-8 * np.abs(x).max())
    assert st.n_rows == len(idx)


def test_pcg_reference_stop_rule_and_fixed_mode():
    """Loop test at the head (solver_driver.cc:319-337): stop when
    iterations >= max or r.r < threshold; fixed mode runs exactly max."""
    n = 10
    o = _sim(n)
    shp = (n + 2,) * 3
    marker = np.zeros(shp, np.int32)
    marker[1:-1, 1:6, 1:-1] = 1
    for s in (0, -1):
        marker[s, :, :] = 2
        marker[:, s, :] = 2
        marker[:, :, s] = 2
    rng = np.random.default_rng(1)
    div = np.where(marker == 1, rng.normal(size=shp), 0).astype(np.float32)
    o.set_marker(marker)
    o.set_divergence(div)
    st = o.pcg_solve(mode=2, precision=0, max_iterations=7)
    assert st.iterations == 7
    big = o.pcg_solve(mode=0, precision=0, max_iterations=1500, threshold=1e30)
    assert big.iterations == 0  # r.r < threshold before the first iteration
    st = o.pcg_solve(mode=0, precision=0, max_iterations=1500, threshold=1e-3)
    assert st.rr < 1e-3 and st.iterations > 0


def _one_step(o, dt):
    return o.step(dt, mode=1, precision=2, max_iterations=20000, tol=1e-12)


def test_hydrostatic_pool_stays_at_rest():
    """A flat pool at rest: gravity is cancelled by the pressure projection,
    so faces between two fluid cells keep (near) zero velocity."""
    n = 16
    o = _sim(n)
    o.seed([fsim.SeedPass([fsim.SceneShape(fsim.SHAPE_POOL, a=(0, 6.0, 0))])], seed=3)
    dt = 0.01
    _one_step(o, dt)
    v, _ = o.field(0)
    m, _ = o.marker()
    fl = m == 1
    both = fl[1:, :, :] & fl[:-1, :, :]
    gdt = 9.8 * n * dt
    vy = v[:, 1:, :, 1]
    inner = fl[:, 1:, :] & fl[:, :-1, :]
    assert np.abs(vy[inner]).max() < 1e-6 * gdt * 1e3
    assert both.sum() > 0


def test_projection_is_divergence_free():
    n = 16
    o = _sim(n)
    o.seed(fsim.scene_passes("sphere_drop", n), seed=0)
    pos, vel, _ = o.particles()
    rng = np.random.default_rng(2)
    vel = (vel + rng.normal(0, 5.0, vel.shape)).astype(np.float32)
    o.set_particles(pos, vel, vel.copy())
    st = _one_step(o, 0.01)
    o2 = o  # fields after the step (vel extrapolated into ghosts only)
    v, _ = o2.field(0)
    m, _ = o2.marker()
    u, w, z = v[..., 0], v[..., 1], v[..., 2]
    div = (u[2:, 1:-1, 1:-1] - u[1:-1, 1:-1, 1:-1]) + (w[1:-1, 2:, 1:-1] - w[1:-1, 1:-1, 1:-1]) + \
        (z[1:-1, 1:-1, 2:] - z[1:-1, 1:-1, 1:-1])
    fl = m[1:-1, 1:-1, 1:-1] == 1
    assert np.abs(div[fl]).max() < 1e-6 * math.sqrt(st.bb)


def test_cfl_and_dt_rules():
    """CFL (flip_simulation.cc:460-488) and WhileAndComputeDt
    (flip_app_sim.cc:357-428)."""
    g = 9.8 * 64
    o = _sim(64, g=g)
    inv = o.cfl()  # empty grid: 1/sqrt(0.5 g)
    assert inv == np.float32(1.0 / np.float32(math.sqrt(0.5 * np.float64(np.float32(g)))))
    fs = float(np.float32(1) / np.float32(30))
    dt, t = compute_dt(0.5, 1, fs, 0.0)
    assert dt == np.float32(fs) and t == 0.0 or dt == np.float32(fs)
    dt, t = compute_dt(1e-4, 1, fs, 0.0)  # floored at frame_step/10
    assert dt == pytest.approx(fs / 10, rel=1e-6)
    dt, t = compute_dt(0.02, 1, fs, 0.0)  # 0.02 + 0 <= 0.9 frame
    assert dt == pytest.approx(0.02, rel=1e-6)
    dt2, t2 = compute_dt(0.02, 1, fs, t)  # would pass 0.9 frame: clipped to end
    assert t2 == pytest.approx(fs, rel=1e-6)


def test_velocity_update_ghost_quirk():
    """GetVelocityUpdate loops faces [0,N]^3 only (flip_simulation.cc:781-801),
    so a ghost face at -1 keeps the saved velocity instead of the difference."""
    n = 16
    o = _sim(n)
    pos = np.array([[0.2, 8.5, 0.2]], np.float32)
    vel = np.array([[0.0, 3.0, 0.0]], np.float32)
    o.set_particles(pos, vel, vel.copy())
    dt = 0.01
    o.transfer_particles_to_grid()
    o.apply_boundary_conditions()
    o.save_grid_velocities()
    saved, _ = o.field(1)
    o.add_gravity(dt)
    o.apply_boundary_conditions()
    o.compute_divergence()
    o.pcg_solve(mode=1, precision=2, max_iterations=1000, tol=1e-12)
    o.update_velocity_from_pressure()
    assert o.get_velocity_update() == 0
    dv, _ = o.field(1)
    # y-component at (-1, 8, -1): never overwritten by the update or the
    # extrapolation (edge of two ghost layers)
    c = _ix(n, -1, 8, -1) + (1,)
    assert dv[c] == saved[c] and saved[c] != 0.0
