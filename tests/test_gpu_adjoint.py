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


def test_wendland_adjoint_matches_torch_autograd(case):
    import adjoint_ref
    from sph import adjoint, scenarios
    dx = 0.02
    pa = scenarios.dam_break(0.2, 0.4, dx, 0.8, 0.6, side="right")
    wc = adjoint.WallLoadCase(pa, height=0.4, r0=dx, h=1.3 * dx, dt=1e-4, nsteps=20, wall_x=0.8, checkpoint=10,
                              kernel=2)
    torch.manual_seed(5)
    pos = wc.positions()
    vel = wc.velocities() + 0.05 * torch.randn_like(pos)
    loss, ga, gp, gv = adjoint.gradients(wc, 0.01, pos, vel)
    a = torch.tensor(0.01, dtype=torch.float64, device="cuda", requires_grad=True)
    p = pos.clone().requires_grad_(True)
    v = vel.clone().requires_grad_(True)
    ref = adjoint_ref.reference_loss(wc, a, p, v)
    ra, rp, rv = torch.autograd.grad(ref, (a, p, v))
    assert loss.item() > 0.0 and loss.item() == pytest.approx(ref.item(), rel=1e-11)
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


def test_full_size_case_against_torch_and_differences():
    """The 20k-fluid case (1.0 x 2.0 m column at dx = 0.01 against the right
    wall, 200 steps of 5e-5 s, checkpoints every 20): adjoint against torch
    autograd (the unfused restatement holds ~30 GB of autograd state) and
    against central differences along alpha."""
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import adjoint_ref
    from sph import adjoint, build, scenarios
    build.build()
    big = adjoint.WallLoadCase(scenarios.cfg_adjoint(), height=2.0, r0=0.01, h=0.013, dt=5e-5, nsteps=200,
                               wall_x=4.0, checkpoint=20)
    # a small seeded velocity field keeps v_ij . x_ij away from 0, the kink of
    # the artificial-viscosity switch (at rest every pair sits on it)
    torch.manual_seed(3)
    pos = big.positions()
    vel = big.velocities() + 0.01 * torch.randn_like(pos)
    loss, ga, gp, gv = adjoint.gradients(big, 0.01, pos, vel)
    a = torch.tensor(0.01, dtype=torch.float64, device="cuda", requires_grad=True)
    p = pos.clone().requires_grad_(True)
    v = vel.clone().requires_grad_(True)
    ref = adjoint_ref.reference_loss(big, a, p, v)
    ra, rp, rv = torch.autograd.grad(ref, (a, p, v))
    ref_value = ref.item()
    del ref
    torch.cuda.empty_cache()
    assert loss.item() > 0.0
    assert loss.item() == pytest.approx(ref_value, rel=1e-11)
    # both are FP64 gradients of the same model; they differ by round-off
    # (summation order, powers), which 200 steps of stiff wall contact
    # amplify to ~1e-6 in the position gradient
    assert _rel(ga, ra) <= 1e-8
    assert _rel(gp, rp) <= 1e-5
    assert _rel(gv, rv) <= 1e-5
    fd = adjoint.central_difference(big, 0.01, pos, vel, eps=1e-6, d_alpha=1.0)
    assert ga.item() == pytest.approx(fd, rel=1e-4)
    torch.manual_seed(2)
    dpos = torch.randn_like(pos)
    dpos /= torch.linalg.norm(dpos)
    dvel = torch.randn_like(vel)
    dvel /= torch.linalg.norm(dvel)
    fd = adjoint.central_difference(big, 0.01, pos, vel, eps=1e-6, d_vel=dvel)
    assert (gv * dvel).sum().item() == pytest.approx(fd, rel=1e-4)
    # Along the initial positions the bar is checked over 50 steps: over the
    # full 200 the loss is kinked in the positions (pairs that cross the
    # Lennard-Jones cutoff r0, where the force's slope jumps), and the central
    # difference does not converge in eps there (it scatters by ~1e-2
    # relative over eps = 1e-4 .. 1e-8), so it checks nothing at 1e-4.
    # Over 50 steps the differences converge: 1e-4 along both
    short = adjoint.WallLoadCase(scenarios.cfg_adjoint(), height=2.0, r0=0.01, h=0.013, dt=5e-5, nsteps=50,
                                 wall_x=4.0, checkpoint=10)
    loss, ga, gp, gv = adjoint.gradients(short, 0.01, pos, vel)
    fd = adjoint.central_difference(short, 0.01, pos, vel, eps=1e-6, d_pos=dpos)
    assert (gp * dpos).sum().item() == pytest.approx(fd, rel=1e-4)
    fd = adjoint.central_difference(short, 0.01, pos, vel, eps=1e-5, d_vel=dvel)
    assert (gv * dvel).sum().item() == pytest.approx(fd, rel=1e-4)


def test_mixed_adjoint_against_fp64_adjoint_and_differences(case):
    """The mixed form of the adjoint (FP32 pair arithmetic in the
    vector-Jacobian product, FP64 forward and replay) against the FP64
    adjoint and central differences of the FP64 loss on the small case."""
    from sph import adjoint, scenarios
    dx = 0.02
    pa = scenarios.dam_break(0.2, 0.4, dx, 0.8, 0.6, side="right")
    mixed = adjoint.WallLoadCase(pa, height=0.4, r0=dx, h=1.3 * dx, dt=1e-4, nsteps=40, wall_x=0.8, checkpoint=10,
                                 adjoint_precision="mixed")
    torch.manual_seed(5)
    pos = case.positions()
    vel = case.velocities() + 0.01 * torch.randn_like(pos)
    l64, ga, gp, gv = adjoint.gradients(case, 0.01, pos, vel)
    lmx, gam, gpm, gvm = adjoint.gradients(mixed, 0.01, pos, vel)
    assert lmx.item() == l64.item()  # the same FP64 forward
    assert abs(gam.item() - ga.item()) <= 1e-4 * abs(ga.item())
    assert _rel(gpm, gp) <= 1e-4 and _rel(gvm, gv) <= 1e-4
    fd = adjoint.central_difference(case, 0.01, pos, vel, eps=1e-6, d_alpha=1.0)
    assert gam.item() == pytest.approx(fd, rel=1e-4)

