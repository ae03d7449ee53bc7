"""The allocation-free CFL entry point (fsim_cfl_noalloc) against the
handle-based fsim_cfl, through the C ABI.

fsim_cfl_noalloc is for callers that cannot call cudaMalloc while stepping
(engines that hand the solver buffers from a pre-reserved pool and forbid
allocation in their frame loop).  Here the test itself allocates the device
buffers (it plays the part of that engine) and checks that two calls in a
row reproduce fsim_cfl exactly (a maximum and the same scalar formula, so
the results are bit-equal), and that a grid larger than the scratch's 1024
blocks x 256 threads reproduces a NumPy restatement of CFL() exactly.  This
file is collected last on purpose.
"""
import ctypes as C

import numpy as np
import pytest

import fsim

pytestmark = pytest.mark.gpu


def _simulated_field(n=32):
    g, f = fsim.physical_gravity(n)
    sim = fsim.Simulation((n, n, n), fsim.BOUNDARY_BOX, g, f)
    sim.seed(fsim.scene_passes("sphere_drop", n), seed=0)
    pos, vel, gvel = sim.download_particles()
    rng = np.random.default_rng(11)
    vel = (vel + rng.normal(0, 2.0 * n, vel.shape)).astype(np.float32)
    sim.upload_particles(pos, vel, vel.copy())
    sim.step(0.005, fsim.pcg_params(fsim.PCG_RELATIVE, fsim.PREC_FP32, 500, tolerance=1e-5))
    return sim, g


def test_noalloc_cfl_matches_handle_cfl_twice():
    torch = pytest.importorskip("torch")
    sim, g = _simulated_field()
    expect = sim.cfl()
    vel, act = sim.field(fsim.FIELD_VELOCITY)
    dims = (C.c_int32 * 3)(*sim.dims)
    sim.close()
    d_vel = torch.from_numpy(np.ascontiguousarray(vel)).cuda()
    d_act = torch.from_numpy(np.ascontiguousarray(act)).cuda()
    lib = fsim.load_library()
    stream = torch.cuda.current_stream()
    for _ in range(2):
        d_out = torch.full((1,), -1.0, dtype=torch.float32, device="cuda")
        rc = lib.fsim_cfl_noalloc(C.c_void_p(d_vel.data_ptr()), C.c_void_p(d_act.data_ptr()),
                                  dims, C.c_float(g), C.c_void_p(d_out.data_ptr()),
                                  C.c_void_p(stream.cuda_stream))
        assert rc == fsim.OK
        torch.cuda.synchronize()
        got = float(d_out.item())
        assert got == expect, (got, expect)
    # the velocity field is not trivially the gravity floor
    assert expect < 1.0 / np.sqrt(0.5 * g)


def _cfl_numpy(vel, act, dims, g):
    """FlipSimulation::CFL (common/flip_simulation.cc:460-488) on a dense
    field: max |v_d| over active in-box faces, leaving out the last index on
    the two tangential axes, then v = max(sqrt(0.5 g), v_inf) >= 1e-2."""
    n0, n1, n2 = dims
    a = act[1:n0 + 1, 1:n1 + 1, 1:n2 + 1].astype(bool)
    v = np.abs(vel[1:n0 + 1, 1:n1 + 1, 1:n2 + 1])
    m = np.float32(0.0)
    for d, (p, q) in enumerate(((1, 2), (0, 2), (0, 1))):
        keep = a.copy()
        for ax in (p, q):
            idx = [slice(None)] * 3
            idx[ax] = -1
            keep[tuple(idx)] = False
        if keep.any():
            m = max(m, np.float32(v[..., d][keep].max()))
    vv = np.float32(max(np.sqrt(0.5 * np.float64(np.float32(g))), np.float64(m)))
    if vv < 1e-2:
        vv = np.float32(1e-2)
    return np.float32(1.0 / np.float64(vv))


def test_noalloc_cfl_grid_beyond_scratch_blocks():
    """72 x 64 x 80 cells (368,640 > 1024 x 256): the grid is capped at the
    scratch's 1024 blocks and the grid-stride loop covers the rest; the
    largest speed is planted near the end of the loop's range, in a cell
    only the second sweep of the loop visits."""
    torch = pytest.importorskip("torch")
    dims = (72, 64, 80)
    rng = np.random.default_rng(5)
    shape = tuple(d + 2 for d in dims)
    vel = rng.normal(0.0, 40.0, shape + (3,)).astype(np.float32)
    act = (rng.random(shape) < 0.7).astype(np.uint8)
    i, j, k = dims[0], dims[1] - 1, dims[2] - 1  # cell (n0-1, n1-2, n2-2), in-box for v_x
    act[i, j, k] = 1
    vel[i, j, k, 0] = -9.0e3
    g = 9.8 * 64
    expect = _cfl_numpy(vel, act, dims, g)
    assert expect == np.float32(1.0 / 9.0e3)
    d_vel = torch.from_numpy(vel).cuda()
    d_act = torch.from_numpy(act).cuda()
    lib = fsim.load_library()
    stream = torch.cuda.current_stream()
    cd = (C.c_int32 * 3)(*dims)
    for _ in range(2):
        d_out = torch.full((1,), -1.0, dtype=torch.float32, device="cuda")
        rc = lib.fsim_cfl_noalloc(C.c_void_p(d_vel.data_ptr()), C.c_void_p(d_act.data_ptr()), cd,
                                  C.c_float(g), C.c_void_p(d_out.data_ptr()),
                                  C.c_void_p(stream.cuda_stream))
        assert rc == fsim.OK
        torch.cuda.synchronize()
        assert np.float32(d_out.item()) == expect


def test_noalloc_cfl_rejects_sizes_beyond_maximum():
    lib = fsim.load_library()
    big = (C.c_int32 * 3)(2048, 64, 64)
    dummy = C.c_void_p(16)  # never dereferenced: the size check comes first
    assert lib.fsim_cfl_noalloc(dummy, dummy, big, C.c_float(9.8), dummy, None) == fsim.ERR_CAPACITY
    small = (C.c_int32 * 3)(4, 64, 64)
    assert lib.fsim_cfl_noalloc(dummy, dummy, small, C.c_float(9.8), dummy, None) == fsim.ERR_INVALID
