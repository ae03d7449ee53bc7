"""Adjoint of the FLIP rollout (fsim_rollout_*) against finite differences.

The gradient of L = 0.5 ||u_K - u_target||^2 w.r.t. the initial particle
velocity is taken along the fp32 forward (the production step) with the
discrete choices frozen (bins, clamps, stencil sides, markers, active
faces, the 1e-5 weight cut).  Central differences use the fp64 replay of that same frozen
map, so they see no binning jumps; the fp64 reference gradient is the same
adjoint linearised along the replay.  A torch.autograd.Function wraps the
rollout here, and only here.
"""
import numpy as np
import pytest

import fsim
from _util import rel_l2

pytestmark = pytest.mark.gpu

N, STEPS, EVERY = 32, 6, 2
DT = 1.0 / 300.0
# The frozen map keeps every discrete choice of the recorded forward,
# including the side of the cell centre each particle's trilinear stencil
# starts on, so it is smooth (polynomial up to the normalisation's division)
# around the recorded state, and central differences converge to the fp64
# adjoint at O(eps^2) (Richardson-combined, O(eps^4)).  eps = 1e-3 is the
# differentiable-rollout configuration's step.  The fp32-trajectory gradient differs from the
# fp64-trajectory one by the trajectory's sensitivity (~1e-4 here).
EPS = 1e-3
FP64_RTOL = 1e-5
FP32_RTOL = 1e-3


def _adj_params():
    return fsim.pcg_params(fsim.PCG_RELATIVE, fsim.PREC_FP64, 20000, tolerance=1e-12)


@pytest.fixture(scope="module")
def case():
    sim, ro, target, pcg = fsim.rollout_case(N, STEPS, EVERY, DT)
    loss = ro.forward(DT, pcg, target)
    yield sim, ro, target, pcg, loss
    ro.close()
    sim.close()


@pytest.fixture(scope="module")
def grads(case):
    sim, ro, target, pcg, loss = case
    gv, gg = ro.backward(_adj_params(), tape=0)
    return gv, gg


@pytest.fixture(scope="module")
def fd(case):
    """Central differences of the fp64 replay loss along seeded directions
    (the same perturbation of vel and gvel, which the scene seeds equal), at
    EPS and EPS/2, combined by Richardson extrapolation: the map is smooth,
    but v = m / w at faces whose weight is near the 1e-5 cut curves it
    strongly, and (4 D(EPS/2) - D(EPS)) / 3 cancels the EPS^2 term."""
    sim, ro, target, pcg, loss = case
    theta, gtheta = ro.initial_velocity()
    assert np.array_equal(theta, gtheta)
    rng = np.random.default_rng(7)

    def central(d, eps):
        lp = ro.replay_loss(theta + eps * d, theta + eps * d)
        lm = ro.replay_loss(theta - eps * d, theta - eps * d)
        return (lp - lm) / (2 * eps)

    out = []
    for _ in range(4):
        d = rng.standard_normal(theta.shape)
        out.append((d, (4.0 * central(d, EPS / 2) - central(d, EPS)) / 3.0))
    return out


def test_forward_loss_matches_fp64_replay(case):
    sim, ro, target, pcg, loss = case
    assert loss > 0.0
    l64 = ro.replay_loss()
    assert abs(l64 - loss) <= 1e-4 * loss, (loss, l64)


def test_gradient_matches_central_differences(case, grads, fd):
    gv, gg = grads
    g = gv + gg
    assert np.isfinite(g).all() and np.abs(g).max() > 0.0
    for k, (d, f) in enumerate(fd):
        ad = float(np.sum(g * d))
        assert abs(ad - f) <= FP32_RTOL * abs(f), f"direction {k}: adjoint {ad} vs FD {f}"


def test_fp64_reference_gradient(case, grads, fd):
    sim, ro, target, pcg, loss = case
    gv, gg = grads
    gv64, gg64 = ro.backward(_adj_params(), tape=1)
    # the fp64 adjoint is the exact transpose of the replay the differences see
    for k, (d, f) in enumerate(fd):
        ad = float(np.sum((gv64 + gg64) * d))
        assert abs(ad - f) <= FP64_RTOL * abs(f), f"direction {k}: fp64 adjoint {ad} vs FD {f}"
    assert rel_l2(gv, gv64) <= FP32_RTOL
    assert rel_l2(gg, gg64) <= FP32_RTOL


def test_checkpoint_interval_does_not_change_the_gradient(case, grads):
    sim, ro, target, pcg, loss = case
    gv, gg = grads
    sim2, ro2, target2, pcg2 = fsim.rollout_case(N, STEPS, 1, DT)
    l2 = ro2.forward(DT, pcg2, target2)
    # the production forward is deterministic (only the loss sum's order is not)
    assert abs(l2 - loss) <= 1e-12 * loss
    gv2, gg2 = ro2.backward(_adj_params(), tape=0)
    assert rel_l2(gv2, gv) <= 1e-10 and rel_l2(gg2, gg) <= 1e-10
    ro2.close()
    sim2.close()


def test_mixed_precision_adjoint_solves(case, grads):
    sim, ro, target, pcg, loss = case
    gv, gg = grads
    mixed = fsim.pcg_params(fsim.PCG_RELATIVE, fsim.PREC_MIXED, 20000, tolerance=1e-10,
                            inner_tolerance=1e-3, max_refinements=30)
    gvm, ggm = ro.backward(mixed, tape=0)
    assert rel_l2(gvm + ggm, gv + gg) <= 1e-6


def test_torch_autograd_wrapper(case, grads):
    torch = pytest.importorskip("torch")
    sim, ro, target, pcg, loss = case
    gv, gg = grads
    adj = _adj_params()

    class RolloutLoss(torch.autograd.Function):
        @staticmethod
        def forward(ctx, v0):
            ro.set_initial_velocity(v0.detach().cpu().numpy())
            return v0.new_tensor(ro.forward(DT, pcg, target))

        @staticmethod
        def backward(ctx, gout):
            a, b = ro.backward(adj, tape=0)
            return torch.from_numpy(a + b).to(gout.dtype) * gout

    theta, _ = ro.initial_velocity()
    v0 = torch.tensor(theta, dtype=torch.float64, requires_grad=True)
    out = RolloutLoss.apply(v0)
    assert abs(float(out.detach()) - loss) <= 1e-12 * loss
    out.backward()
    assert rel_l2(v0.grad.numpy(), gv + gg) <= 1e-10
