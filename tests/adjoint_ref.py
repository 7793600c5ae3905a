"""Unfused FP64 torch restatement of the differentiated step, for checking the
hand-written adjoint against torch autograd.

Test infrastructure only.  Each evaluation takes its neighbour pairs from the
device neighbour export at the half state (indices carry no gradient); the
physics is plain torch arithmetic in FP64, following the reference:
continuity (src/Equations/Continuity.py), momentum with artificial viscosity
and gravity (src/Equations/Momentum.py, src/Methods/WCSPH.py:151-169), the
Tait EOS (src/Equations/TaitEOS.py), the Lennard-Jones boundary force
(src/Equations/BoundaryForce.py), the cubic spline or Wendland C4 gradient
and PEC with a fixed dt
(src/Integrators/PEC.py:32-89).
"""
import math

import torch


def _pairs(case, x, y):
    """Neighbour pairs (i, j), i fluid, j != i, of the state with positions
    (x, y) on the reference's cell grid (the device export)."""
    from sph import core
    from sph.state import DeviceParticles
    dp = DeviceParticles(case.n)
    dp._buf.copy_(case.base._buf)
    dp.label.copy_(case.base.label)
    dp.x.copy_(x.detach())
    dp.y.copy_(y.detach())
    core.nn_update(dp, case.cfg, case.ws)
    off, idx = core.nn_export(dp, case.cfg, case.ws)
    off = torch.from_numpy(off).to(x.device)
    idx = torch.from_numpy(idx).to(x.device)
    counts = off[1:] - off[:-1]
    i = torch.repeat_interleave(torch.arange(case.n, device=x.device), counts)
    keep = (i != idx) & case.fluid[i]
    return i[keep], idx[keep]


def _evaluate(case, wc, alpha, x, y, vx, vy, rho, i, j):
    f = case.fluid
    m, h = case.base.m, case.base.h
    n = case.n
    rho_s = torch.where(f, rho, torch.ones_like(rho))
    t = rho_s / wc.rho0
    p = torch.where(f, wc.B * (t ** 7 - 1.0) + wc.Pb, torch.zeros_like(rho))
    othr = torch.where(f, p / (rho_s * rho_s), torch.zeros_like(rho))
    dx = x[i] - x[j]
    dy = y[i] - y[j]
    r = torch.sqrt(dx * dx + dy * dy)
    hij = 0.5 * (h[i] + h[j])
    q = r / hij
    jf = f[j]
    if case.cfg.kernel == 2:
        # Wendland C4 gradient factor (src/Kernels/Wendland.py:36-64)
        al = 9.0 / (4.0 * math.pi) / (hij * hij)
        inner = torch.clamp(1.0 - 0.5 * q, min=0.0)
        g = inner ** 5 * (-14.0 / 3.0) * q * (1.0 + 2.5 * q)
        inside = (q < 2.0) & (r >= 1e-10) & jf
    else:
        # cubic spline gradient factor (src/Kernels/CubicSpline.py:40-70)
        al = 10.0 / (7.0 * math.pi) / (hij * hij)
        g = torch.where(q > 1.0, -0.75 * (2.0 - q) ** 2, -3.0 * q * (1.0 - 0.75 * q))
        inside = (q <= 2.0) & (r >= 1e-10) & jf
    coef = torch.where(inside, al * g / (hij * r), torch.zeros_like(r))
    dWx, dWy = coef * dx, coef * dy
    vxij = vx[i] - vx[j]
    vyij = vy[i] - vy[j]
    dot = vxij * dx + vyij * dy
    hb = 0.5 * (h[i] + hij)
    den = r * r + 0.01 * hb * hb
    mu = hb * dot / den
    rbar = 0.5 * (rho_s[i] + rho_s[j])
    cbar = 0.5 * wc.co
    Pi = torch.where(dot < 0.0, mu * (wc.beta * mu - alpha * cbar) / rbar, torch.zeros_like(r))
    S = othr[i] + othr[j] + Pi
    mj = m[j]
    ax = torch.zeros(n, dtype=torch.float64, device=x.device).index_add(0, i, torch.where(inside, -mj * S * dWx, 0.0))
    ay = torch.zeros(n, dtype=torch.float64, device=x.device).index_add(0, i, torch.where(inside, -mj * S * dWy, 0.0))
    drho = torch.zeros(n, dtype=torch.float64, device=x.device).index_add(
        0, i, torch.where(inside, mj * (vxij * dWx + vyij * dWy), 0.0))
    # Lennard-Jones boundary force (no mass factor)
    lj = (~jf) & (r <= wc.r0) & (r > 1e-12)
    r_s = torch.where(lj, r, torch.ones_like(r))
    s2 = (wc.r0 / r_s) ** 2
    fac = torch.where(lj, wc.D * (s2 * s2 - s2) / (r_s * r_s), torch.zeros_like(r))
    bx, by = fac * dx, fac * dy
    ax = ax.index_add(0, i, bx)
    ay = ay.index_add(0, i, by) - 9.81
    wall = lj & (x[j] >= case.wall_x)
    load = -(m[i] * torch.where(wall, bx, torch.zeros_like(bx))).sum()
    return ax, ay, drho, load


def reference_loss(case, alpha, pos, vel):
    """The loss of sph.adjoint.WallLoadLoss as a differentiable torch graph."""
    f = case.fluid
    fi = torch.nonzero(f).squeeze(1)
    wc = case.wcsph(0.0)
    dt = case.dt
    x = case.base.x.detach().clone().index_put((fi,), pos[:, 0])
    y = case.base.y.detach().clone().index_put((fi,), pos[:, 1])
    vx = torch.zeros_like(x).index_put((fi,), vel[:, 0])
    vy = torch.zeros_like(x).index_put((fi,), vel[:, 1])
    rho = case.rho_init.clone()
    ax = torch.zeros_like(x)
    ay = torch.zeros_like(x)
    drho = torch.zeros_like(x)
    ff = f.to(torch.float64)
    loss = torch.zeros((), dtype=torch.float64, device=x.device)
    for _ in range(case.nsteps):
        xh = x + 0.5 * dt * vx * ff
        yh = y + 0.5 * dt * vy * ff
        vxh = vx + 0.5 * dt * ax * ff
        vyh = vy + 0.5 * dt * ay * ff
        rhoh = rho + 0.5 * dt * drho * ff
        i, j = _pairs(case, xh, yh)
        A_x, A_y, D, load = _evaluate(case, wc, alpha, xh, yh, vxh, vyh, rhoh, i, j)
        x = x + dt * vxh * ff
        y = y + dt * vyh * ff
        vx = vx + dt * A_x * ff
        vy = vy + dt * A_y * ff
        rho = rho + dt * D * ff
        ax, ay, drho = A_x * ff, A_y * ff, D * ff
        loss = loss + dt * load
    return loss
