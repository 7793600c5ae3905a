"""Differentiation form: the hand-written adjoint (sph_adjoint_step behind
sph.adjoint.WallLoadLoss) against torch autograd through an unfused FP64
torch restatement of the step, and against central finite differences in
FP64 (eps = 1e-6)."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def case():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from sph import build
    build.build()
    from sph import adjoint, scenarios
    dx = 0.02
    pa = scenarios.dam_break(0.2, 0.4, dx, 0.8, 0.6, side="right")
    return adjoint.WallLoadCase(pa, height=0.4, r0=dx, h=1.3 * dx, dt=1e-4, nsteps=40, wall_x=0.8, checkpoint=10)


def _rel(a, b):
    a, b = torch.as_tensor(a, dtype=torch.float64), torch.as_tensor(b, dtype=torch.float64)
    return (torch.linalg.norm(a - b) / torch.linalg.norm(b)).item()


def test_wall_is_loaded_and_forward_matches_torch(case):
    import adjoint_ref
    pos, vel = case.positions(), case.velocities()
    loss = case.loss(0.01, pos, vel).item()
    with torch.no_grad():
        ref = adjoint_ref.reference_loss(case, torch.tensor(0.01, dtype=torch.float64, device="cuda"), pos, vel)
    assert loss > 0.0
    assert loss == pytest.approx(ref.item(), rel=1e-11)


def test_checkpointing_does_not_change_the_loss(case):
    from sph import adjoint
    pos, vel = case.positions(), case.velocities()
    a = torch.tensor(0.01, dtype=torch.float64, device="cuda")
    l1 = adjoint.WallLoadLoss.apply(a, pos, vel, case).item()
    assert l1 == case.loss(0.01, pos, vel).item()


def test_adjoint_matches_torch_autograd(case):
    import adjoint_ref
    from sph import adjoint
    torch.manual_seed(0)
    pos = case.positions()
    vel = case.velocities() + 0.05 * torch.randn_like(case.velocities())
    loss, ga, gp, gv = adjoint.gradients(case, 0.01, pos, vel)
    a = torch.tensor(0.01, dtype=torch.float64, device="cuda", requires_grad=True)
    p = pos.clone().requires_grad_(True)
    v = vel.clone().requires_grad_(True)
    ref = adjoint_ref.reference_loss(case, a, p, v)
    ra, rp, rv = torch.autograd.grad(ref, (a, p, v))
    assert loss.item() == pytest.approx(ref.item(), rel=1e-11)
    assert _rel(ga, ra) <= 1e-8
    assert _rel(gp, rp) <= 1e-8
    assert _rel(gv, rv) <= 1e-8


def test_adjoint_matches_central_differences(case):
    from sph import adjoint
    torch.manual_seed(1)
    pos, vel = case.positions(), case.velocities()
    loss, ga, gp, gv = adjoint.gradients(case, 0.01, pos, vel)
    fd_a = adjoint.central_difference(case, 0.01, pos, vel, eps=1e-6, d_alpha=1.0)
    assert ga.item() == pytest.approx(fd_a, rel=1e-4)
    for _ in range(2):
        dpos = torch.randn_like(pos)
        dpos /= torch.linalg.norm(dpos)
        fd = adjoint.central_difference(case, 0.01, pos, vel, eps=1e-6, d_pos=dpos)
        assert (gp * dpos).sum().item() == pytest.approx(fd, rel=1e-4)
        dvel = torch.randn_like(vel)
        dvel /= torch.linalg.norm(dvel)
        fd = adjoint.central_difference(case, 0.01, pos, vel, eps=1e-6, d_vel=dvel)
        assert (gv * dvel).sum().item() == pytest.approx(fd, rel=1e-4)
