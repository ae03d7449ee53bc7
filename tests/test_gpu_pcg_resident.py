"""The resident PCG loop: one persistent CTA per SM keeps r,
p and the flags of its particle leaves on chip and runs every iteration of
PCGSolver (common/solver.cc:297-366) in one cooperative launch, with two
bounded grid barriers per iteration.  The arithmetic is the pair's, summed per
thread in another order, so the bars are the solver's own: after a fixed
number of iterations it tracks the oracle as closely as the pair does, and a
relative-1e-5 solve is no further from the converged (FP64) solution than the
oracle's fp32 solve.  By default it takes the fp32 solves of systems with
2 to 56 particle leaves per SM; FSIM_PCG_RES=1 forces it wherever it fits,
=0 turns it off."""
import numpy as np
import pytest

import fsim
from _util import rel_l2
from test_gpu_pcg import _pressures, _prepared

pytestmark = pytest.mark.gpu


def _prepared_res(monkeypatch, n=32, scene="dam_break"):
    with monkeypatch.context() as m:
        m.setenv("FSIM_PCG_RES", "1")
        return _prepared(n=n, scene=scene)


def _loop_kernels(sim, prm):
    sim.set_profiling(True)
    sim.reset_kernel_times()
    st = sim.pcg_solve(prm)
    names = {k for k in sim.kernel_times() if k.startswith("pcg_")}
    sim.set_profiling(False)
    return st, names


def test_fixed_iterations_track_oracle(monkeypatch):
    orc, sim = _prepared_res(monkeypatch)
    for it in (1, 5, 25):
        st, names = _loop_kernels(sim, fsim.pcg_params(fsim.PCG_FIXED, fsim.PREC_FP32, it))
        assert "pcg_resident" in names, names
        ost = orc.pcg_solve(mode=2, precision=0, max_iterations=it)
        assert st.status == 0 and st.iterations == it and ost.iterations == it
        a, b = _pressures(sim, orc)
        assert rel_l2(a, b) <= 1e-5, it
        assert abs(st.rr - ost.rr) <= 1e-3 * ost.rr + 1e-30, it
    sim.close()


@pytest.mark.parametrize("n,scene", [(32, "dam_break"), (64, "sphere_drop")])
def test_relative_solve_against_converged(monkeypatch, n, scene):
    orc, sim = _prepared_res(monkeypatch, n=n, scene=scene)
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


def test_reference_absolute_rule_and_repeat(monkeypatch):
    """The reference's absolute rule; a second solve on the handle repeats
    the first bit for bit (fixed-order sums)."""
    orc, sim = _prepared_res(monkeypatch)
    prm = sim.default_pcg_params()
    st = sim.pcg_solve(prm)
    x1 = sim.field(fsim.FIELD_PRESSURE)[0]
    st2 = sim.pcg_solve(prm)
    assert (st2.iterations, st2.rr) == (st.iterations, st.rr)
    assert np.array_equal(sim.field(fsim.FIELD_PRESSURE)[0], x1)
    ost = orc.pcg_solve(mode=0, precision=0, max_iterations=1500, threshold=prm.threshold)
    assert st.status == 0 and st.rr < prm.threshold
    assert abs(st.iterations - ost.iterations) <= 2 + ost.iterations // 20
    a, b = _pressures(sim, orc)
    orc.pcg_solve(mode=1, precision=2, max_iterations=20000, tol=1e-13)
    x64 = orc.pressure_f64()
    assert rel_l2(a, x64) <= max(1e-5, 1.5 * rel_l2(b, x64))
    sim.close()


def test_status_other_precisions_and_default(monkeypatch):
    orc, sim = _prepared_res(monkeypatch)
    st = sim.pcg_solve(fsim.pcg_params(fsim.PCG_RELATIVE, fsim.PREC_FP32, 3, tolerance=1e-12))
    assert st.status == fsim.ERR_NOT_CONVERGED and st.iterations == 3
    st, names = _loop_kernels(sim, fsim.pcg_params(fsim.PCG_RELATIVE, fsim.PREC_MIXED, 3000,
                                                   tolerance=1e-7, max_refinements=20))
    assert st.status == 0 and "pcg_resident" not in names
    sim.close()
    monkeypatch.delenv("FSIM_PCG_RES", raising=False)
    orc, sim = _prepared()
    st, names = _loop_kernels(sim, fsim.pcg_params(fsim.PCG_FIXED, fsim.PREC_FP32, 4))
    assert "pcg_resident" not in names
    sim.close()


def test_chosen_by_system_size(monkeypatch):
    """Without FSIM_PCG_RES the 256^3 dam break (8,320 particle leaves, 55 per
    SM) and the 128^3 sphere drop (1,148, 7.6 per SM) take the resident loop,
    the 64^3 sphere drop (156, about one per SM) and a 32^3 system the pair;
    with FSIM_PCG_RES=0 the 256^3 system takes the pair."""
    import torch

    monkeypatch.delenv("FSIM_PCG_RES", raising=False)
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    prm = fsim.pcg_params(fsim.PCG_FIXED, fsim.PREC_FP32, 4)
    orc, sim = _prepared()
    assert "pcg_resident" not in _loop_kernels(sim, prm)[1]
    sim.close()
    for n, scene, env, want in ((64, "sphere_drop", None, False), (128, "sphere_drop", None, True),
                                (256, "dam_break", None, True), (256, "dam_break", "0", False)):
        g, f = fsim.physical_gravity(n)
        with monkeypatch.context() as m:
            if env is not None:
                m.setenv("FSIM_PCG_RES", env)
            big = fsim.Simulation((n, n, n), fsim.BOUNDARY_BOX, g, f)
        with big:
            big.seed(fsim.scene_passes(scene, n), seed=0)
            big.transfer_particles_to_grid()
            big.apply_boundary_conditions()
            big.compute_divergence()
            nl = big.leaves().shape[0]
            assert (2 * sms <= nl <= 56 * sms) == (want or env == "0"), (n, nl, sms)
            names = _loop_kernels(big, prm)[1]
            assert ("pcg_resident" in names) == want, (n, env, names)


def test_barrier_wait_gives_up_and_recovers(monkeypatch):
    """The grid-barrier waits are bounded.  With FSIM_PCG_RES_WITHHOLD=1 CTA 0
    of the first solve does not arrive at its first barrier (and the limit is
    256 polls), so every CTA's wait gives up without a fault: each leaves the
    loop, frees its tensor memory, and the solve reports FSIM_ERR_TIMEOUT.
    The handle's next solve runs normally, bit for bit as a handle that never
    timed out."""
    prm = fsim.pcg_params(fsim.PCG_RELATIVE, fsim.PREC_FP32, 3000, tolerance=1e-5)
    orc, ref = _prepared_res(monkeypatch)
    st_ref = ref.pcg_solve(prm)
    x_ref = ref.field(fsim.FIELD_PRESSURE)[0]
    ref.close()
    with monkeypatch.context() as m:
        m.setenv("FSIM_PCG_RES", "1")
        m.setenv("FSIM_PCG_RES_WITHHOLD", "1")
        orc, sim = _prepared()
    with pytest.raises(fsim.FsimError) as err:
        sim.pcg_solve(prm)
    assert err.value.code == fsim.ERR_TIMEOUT
    st = sim.pcg_solve(prm)  # the withheld arrival applied to one solve only
    assert st.status == 0 and (st.iterations, st.rr) == (st_ref.iterations, st_ref.rr)
    assert np.array_equal(sim.field(fsim.FIELD_PRESSURE)[0], x_ref)
    sim.close()
