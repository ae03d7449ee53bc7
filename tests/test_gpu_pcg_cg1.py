"""The single-reduction (Chronopoulos-Gear) PCG loop.

fp32 solves take it with FSIM_PCG_CG1=1 (the pair of kernels is the
default).  It runs the iterates of PCGSolver
(common/solver.cc:297-366) with one reduction per iteration: alpha from
gamma = r.z and delta = (A z).z, and A p carried by a recurrence instead of
formed from p.  In exact arithmetic the iterates are the reference's; in
fp32 the rounding differs, so the bars are the solver's own: after a fixed
number of iterations it tracks the oracle as closely as the pair of kernels
does, and a relative-1e-5 solve is no further from the converged (FP64,
1e-13) solution than the oracle's fp32 solve.
"""
import numpy as np
import pytest

import fsim
from _util import rel_l2
from test_gpu_pcg import _pressures, _prepared

pytestmark = pytest.mark.gpu


def _prepared_cg1(monkeypatch, n=32, scene="dam_break", env=()):
    with monkeypatch.context() as m:
        m.setenv("FSIM_PCG_CG1", "1")
        for k, v in env:
            m.setenv(k, v)
        return _prepared(n=n, scene=scene)


def test_fixed_iterations_track_oracle(monkeypatch):
    orc, sim = _prepared_cg1(monkeypatch)
    for it in (1, 5, 25):
        st = sim.pcg_solve(fsim.pcg_params(fsim.PCG_FIXED, fsim.PREC_FP32, it))
        ost = orc.pcg_solve(mode=2, precision=0, max_iterations=it)
        assert st.status == 0 and st.iterations == it and ost.iterations == it
        a, b = _pressures(sim, orc)
        assert rel_l2(a, b) <= 1e-5, it
        assert abs(st.rr - ost.rr) <= 1e-3 * ost.rr + 1e-30, it
    sim.close()


@pytest.mark.parametrize("n,scene", [(32, "dam_break"), (64, "sphere_drop")])
def test_relative_solve_against_converged(monkeypatch, n, scene):
    """Relative 1e-5: iteration count within 10% (+2) of the oracle's, and
    the solution within max(1e-5, 1.5 x the oracle's own error) of the
    converged solve."""
    orc, sim = _prepared_cg1(monkeypatch, n=n, scene=scene)
    st = sim.pcg_solve(fsim.pcg_params(fsim.PCG_RELATIVE, fsim.PREC_FP32, 3000, tolerance=1e-5))
    ost = orc.pcg_solve(mode=1, precision=0, max_iterations=3000, tol=1e-5)
    assert st.status == 0 and ost.status == 0
    assert st.iterations <= 1.1 * ost.iterations + 2, (st.iterations, ost.iterations)
    assert st.rr <= 1e-10 * st.bb
    a, b = _pressures(sim, orc)
    orc.pcg_solve(mode=1, precision=2, max_iterations=20000, tol=1e-13)
    x64 = orc.pressure_f64()
    e_gpu, e_orc = rel_l2(a, x64), rel_l2(b, x64)
    assert e_gpu <= max(1e-5, 1.5 * e_orc), (e_gpu, e_orc)
    sim.close()


def test_reference_absolute_rule(monkeypatch):
    orc, sim = _prepared_cg1(monkeypatch)
    prm = sim.default_pcg_params()
    st = sim.pcg_solve(prm)
    ost = orc.pcg_solve(mode=0, precision=0, max_iterations=1500, threshold=prm.threshold)
    assert st.status == 0 and st.rr < prm.threshold
    assert abs(st.iterations - ost.iterations) <= 2 + ost.iterations // 20
    a, b = _pressures(sim, orc)
    orc.pcg_solve(mode=1, precision=2, max_iterations=20000, tol=1e-13)
    x64 = orc.pressure_f64()
    assert rel_l2(a, x64) <= max(1e-5, 1.5 * rel_l2(b, x64))
    sim.close()


def test_loop_forms_agree(monkeypatch):
    """Graph loop with programmatic or plain edges, and host-polled launches:
    the same launches in the same order, so bitwise equal solves; and a
    second solve on the same handle repeats the first bit for bit."""
    prm = fsim.pcg_params(fsim.PCG_RELATIVE, fsim.PREC_FP32, 3000, tolerance=1e-5)
    got = {}
    for name, env in (("graph", ()), ("plain_edges", (("FSIM_PCG_PDL", "0"),)),
                      ("host", (("FSIM_PCG_GRAPH", "0"),))):
        orc, sim = _prepared_cg1(monkeypatch, env=env)
        runs = []
        for _ in range(2):
            st = sim.pcg_solve(prm)
            assert st.status == 0, name
            runs.append((st.iterations, st.rr, sim.field(fsim.FIELD_PRESSURE)[0]))
        assert runs[0][:2] == runs[1][:2] and np.array_equal(runs[0][2], runs[1][2]), name
        got[name] = runs[0]
        sim.close()
    it, rr, x = got["graph"]
    for name in ("plain_edges", "host"):
        assert got[name][:2] == (it, rr) and np.array_equal(got[name][2], x), name


def test_status_and_empty_system(monkeypatch):
    orc, sim = _prepared_cg1(monkeypatch)
    st = sim.pcg_solve(fsim.pcg_params(fsim.PCG_RELATIVE, fsim.PREC_FP32, 3, tolerance=1e-12))
    assert st.status == fsim.ERR_NOT_CONVERGED and st.iterations == 3
    # the other precisions keep their own loops on a handle with the option set
    st = sim.pcg_solve(fsim.pcg_params(fsim.PCG_RELATIVE, fsim.PREC_MIXED, 3000, tolerance=1e-7,
                                       max_refinements=20))
    assert st.status == 0
    sim.close()
    n = 16
    g, f = fsim.physical_gravity(n)
    with monkeypatch.context() as m:
        m.setenv("FSIM_PCG_CG1", "1")
        sim = fsim.Simulation((n, n, n), fsim.BOUNDARY_BOX, g, f)
    with sim:
        pos = np.array([[8.5, 8.5, 8.5]], np.float32)
        z = np.zeros_like(pos)
        sim.upload_particles(pos, z, z)
        sim.transfer_particles_to_grid()
        sim.apply_boundary_conditions()
        sim.compute_divergence()
        assert sim.pcg_solve(sim.default_pcg_params()).status == 0


def _loop_kernels(sim, prm):
    sim.set_profiling(True)
    sim.reset_kernel_times()
    sim.pcg_solve(prm)
    names = {k for k in sim.kernel_times() if k.startswith("pcg_")}
    sim.set_profiling(False)
    return names


def test_off_by_default(monkeypatch):
    """Without FSIM_PCG_CG1 every solve runs the spmv / update pair."""
    monkeypatch.delenv("FSIM_PCG_CG1", raising=False)
    orc, sim = _prepared()
    for prec in (fsim.PREC_FP32, fsim.PREC_MIXED):
        names = _loop_kernels(sim, fsim.pcg_params(fsim.PCG_RELATIVE, prec, 500, tolerance=1e-5))
        assert "pcg_cg1" not in names and any(k.startswith("pcg_spmv") for k in names), names
    sim.close()
    orc, sim = _prepared_cg1(monkeypatch)
    assert "pcg_cg1" in _loop_kernels(sim, fsim.pcg_params(fsim.PCG_FIXED, fsim.PREC_FP32, 4))
    sim.close()
