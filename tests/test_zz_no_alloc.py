"""The allocation-free CFL entry point (fsim_cfl_noalloc) against the
handle-based fsim_cfl, through the C ABI.

fsim_cfl_noalloc is for callers that cannot call cudaMalloc while stepping
(engines that hand the solver buffers from a pre-reserved pool and forbid
allocation in their frame loop).  Here the test itself allocates the device
buffers (it plays the part of that engine) and checks that two calls in a
row reproduce fsim_cfl exactly.  This file is collected last on purpose.
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
        assert got == pytest.approx(expect, rel=1e-6), (got, expect)
    # the velocity field is not trivially the gravity floor
    assert expect < 1.0 / np.sqrt(0.5 * g)


def test_noalloc_cfl_rejects_sizes_beyond_maximum():
    lib = fsim.load_library()
    big = (C.c_int32 * 3)(2048, 64, 64)
    dummy = C.c_void_p(16)  # never dereferenced: the size check comes first
    assert lib.fsim_cfl_noalloc(dummy, dummy, big, C.c_float(9.8), dummy, None) == fsim.ERR_CAPACITY
    small = (C.c_int32 * 3)(4, 64, 64)
    assert lib.fsim_cfl_noalloc(dummy, dummy, small, C.c_float(9.8), dummy, None) == fsim.ERR_INVALID
