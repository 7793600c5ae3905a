"""Differentiation form of the WCSPH step.

Gradients of a wall-load loss with respect to the artificial-viscosity
``alpha`` (``WCSPH.alpha``, src/Methods/WCSPH.py:35-79), the initial fluid
velocities and the initial fluid positions, through ``nsteps`` PEC steps with
a fixed dt (src/Solver.py:370-372) and fixed h.

Loss: L = sum over steps of omega_s * load_s, with omega_s = dt (a time
integral) and load_s = -sum_i m_i b_x,i, where b_i is the Lennard-Jones
boundary acceleration (src/Equations/BoundaryForce.py:6-42) that the boundary
particles at x >= wall_x (the right wall) exert on fluid particle i at the
step's evaluation.  The reference has no such diagnostic; it is the
horizontal force the fluid exerts on that wall.

The forward pass runs the device step (``sph_run_wall_load``) and keeps a
checkpoint of the state every ``checkpoint`` steps.  The backward pass
replays each segment from its checkpoint, keeping a copy of the workspace
after every replayed step (its neighbour build and FP64 records), and walks
the segment in reverse with the hand-written adjoint step
(``sph_adjoint_step``: the vector-Jacobian product of the fused pair
evaluation and of PEC), which reuses those builds.  The replay of the
segment before runs on a second stream while the walk runs, into the other
of two sets of workspace copies.  ``adjoint_precision``
"mixed" runs that product's pair arithmetic in FP32 (the mixed form); the
forward, the checkpoints and the replay stay FP64, so the loss and its
finite differences are the FP64 ones.
The initial density is an input held fixed (it is not recomputed from
perturbed positions), as are h and the boundary particles.
"""
import ctypes as C

import numpy as np
import torch

from . import _lib as L
from . import core
from .Common import FLOAT_FIELDS
from .state import DeviceParticles, DeviceWorkspace, current_stream

#: the state of a step: what sph_run leaves and the next step reads
STATE_FIELDS = ("x", "y", "vx", "vy", "rho", "ax", "ay", "drho")
_STATE_ROWS = [FLOAT_FIELDS.index(k) for k in STATE_FIELDS]


class WallLoadCase:
    """A scenario for the differentiation form.

    pa: particle_dtype array (fluid and boundary); height, r0: WCSPH
    constructor arguments; h: the fixed h; dt: the fixed time step;
    wall_x: boundary particles at x >= wall_x form the loaded wall.
    """

    def __init__(self, pa, height, r0, h, dt, nsteps, wall_x, checkpoint=20, kernel=L.KERNEL_CUBIC,
                 rho0=1000.0, device="cuda", adjoint_precision="fp64"):
        self.n = len(pa)
        self.nsteps = int(nsteps)
        self.checkpoint = int(checkpoint)
        self.dt = float(dt)
        self.wall_x = float(wall_x)
        self.height, self.r0, self.rho0 = float(height), float(r0), float(rho0)
        self.cfg = core.config_struct(kernel=kernel, precision="fp64", h_fixed=h, dt_fixed=dt, cfl_c=0.3)
        # the adjoint step's own form: "fp64", or "mixed" (FP32 pair arithmetic
        # in the vector-Jacobian product; the forward stays FP64)
        self.cfg_adj = core.config_struct(kernel=kernel, precision=adjoint_precision, h_fixed=h, dt_fixed=dt,
                                          cfl_c=0.3)
        self.fluid = torch.from_numpy(pa["label"] == 0).to(device)
        self.nf = int(self.fluid.sum().item())
        # base state: hydrostatic density and pressure (WCSPH.initialize), fixed h
        base = DeviceParticles.from_array(pa, device)
        core.initialize(base, self.wcsph(0.01), self.cfg)
        self.base = base
        self.rho_init = base.rho.clone()
        self.ws = DeviceWorkspace(self.n, device=device)
        self.dp = DeviceParticles(self.n, device)
        self.half = DeviceParticles(self.n, device)
        self.fr = torch.zeros(self.n, dtype=torch.float64, device=device)
        self._rows = torch.tensor(_STATE_ROWS, dtype=torch.int64, device=device)
        # the backward's replays run here, beside the adjoint walk
        self.replay_stream = torch.cuda.Stream(device=device)

    def wcsph(self, alpha):
        return core.wcsph_struct(self.height, self.r0, self.rho0, alpha=float(alpha))

    def positions(self):
        return torch.stack((self.base.x[self.fluid], self.base.y[self.fluid]), 1).clone()

    def velocities(self):
        return torch.stack((self.base.vx[self.fluid], self.base.vy[self.fluid]), 1).clone()

    def _start(self, pos, vel):
        dp = self.dp
        dp._buf.copy_(self.base._buf)
        dp.label.copy_(self.base.label)
        f = self.fluid
        dp.x[f] = pos[:, 0]
        dp.y[f] = pos[:, 1]
        dp.vx[f] = vel[:, 0]
        dp.vy[f] = vel[:, 1]
        dp.rho.copy_(self.rho_init)
        for k in ("ax", "ay", "drho"):
            dp.fields[k].zero_()
        return dp

    def _run(self, dp, wc, nsteps, hist):
        L.check(L.load().sph_run_wall_load(core._P(dp), C.byref(wc), C.byref(self.cfg), C.byref(self.ws.ws),
                                           int(nsteps), self.wall_x, self.fr.data_ptr(), hist.data_ptr(),
                                           current_stream()), "sph_run_wall_load")

    def loss(self, alpha, pos, vel):
        """The loss without gradients (FP64 forward on the device)."""
        with torch.no_grad():
            wc = self.wcsph(alpha)
            dp = self._start(pos, vel)
            hist = torch.empty(self.nsteps, dtype=torch.float64, device=pos.device)
            self._run(dp, wc, self.nsteps, hist)
            self.ws.check()
            return self.dt * hist.sum()

    def snapshot(self, dp):
        return dp._buf[self._rows, :self.n]

    def restore(self, dp, snap):
        dp._buf[self._rows, :self.n] = snap


class WallLoadLoss(torch.autograd.Function):
    """loss = WallLoadLoss.apply(alpha, pos, vel, case): alpha a 0-d float64
    tensor, pos and vel (n_fluid, 2) float64 CUDA tensors."""

    @staticmethod
    def forward(ctx, alpha, pos, vel, case):
        wc = case.wcsph(alpha.item())
        dp = case._start(pos, vel)
        hist = torch.empty(case.nsteps, dtype=torch.float64, device=pos.device)
        ckpts = []
        K = case.checkpoint
        for s0 in range(0, case.nsteps, K):
            ckpts.append(case.snapshot(dp))
            case._run(dp, wc, min(K, case.nsteps - s0), hist[s0:])
        case.ws.check()
        ctx.case = case
        ctx.ckpts = ckpts
        ctx.alpha = alpha.item()
        return case.dt * hist.sum()

    @staticmethod
    def backward(ctx, g):
        case = ctx.case
        wc = case.wcsph(ctx.alpha)
        n, dev = case.n, case.fluid.device
        adj = torch.zeros((len(L.ADJOINT_ARRAYS), n), dtype=torch.float64, device=dev)
        A = {k: adj[j] for j, k in enumerate(L.ADJOINT_ARRAYS)}
        cs = L.Adjoint(**{k: A[k].data_ptr() for k in L.ADJOINT_ARRAYS})
        cs.omega = case.dt * float(g.item())
        cs.wall_x = case.wall_x
        cs.reuse_build = 1
        dp, half = case.dp, case.half
        lib = L.load()
        K = case.checkpoint
        w0 = case.ws.ws
        nseg = len(ctx.ckpts)
        main, side = torch.cuda.current_stream(dev), case.replay_stream
        side.wait_stream(main)
        # Two sets of K workspace copies: while the adjoint walks segment seg
        # on the main stream (reading set seg % 2), the side stream replays
        # segment seg - 1 into the other set.  walked[seg]: the main stream
        # has finished reading segment seg's set.
        sets = [[torch.empty_like(case.ws.buf) for _ in range(K)] for _ in range(min(2, nseg))]
        walked = [None] * nseg

        def replay(seg):
            # after each step the workspace holds that step's neighbour build
            # and FP64 records, which its adjoint reuses; the same step as the
            # forward's without the wall-load output (the state is identical)
            bufs = sets[seg % 2]
            with torch.cuda.stream(side):
                if seg + 2 < nseg:
                    side.wait_event(walked[seg + 2])
                dp._buf.copy_(case.base._buf)
                case.restore(dp, ctx.ckpts[seg])
                for s in range(min(K, case.nsteps - seg * K)):
                    core.run(dp, wc, case.cfg, case.ws, 1)
                    bufs[s].copy_(case.ws.buf)
                return side.record_event()

        ready = replay(nseg - 1)
        for seg in reversed(range(nseg)):
            main.wait_event(ready)
            if seg > 0:
                ready = replay(seg - 1)
            bufs = sets[seg % 2]
            for s in reversed(range(min(K, case.nsteps - seg * K))):
                ws_s = L.Workspace(ptr=bufs[s].data_ptr(), bytes=w0.bytes, n_cap=w0.n_cap, max_cells=w0.max_cells)
                L.check(lib.sph_adjoint_step(core._P(case.base), core._P(half), C.byref(wc), C.byref(case.cfg_adj),
                                             C.byref(ws_s), C.byref(cs), current_stream()), "sph_adjoint_step")
            walked[seg] = main.record_event()
        main.wait_stream(side)
        case.ws.check()
        del sets
        f = case.fluid
        galpha = A["alphab"].sum().reshape(())
        gpos = torch.stack((A["xb"][f], A["yb"][f]), 1)
        gvel = torch.stack((A["vxb"][f], A["vyb"][f]), 1)
        return galpha, gpos, gvel, None


def gradients(case, alpha, pos=None, vel=None):
    """(loss, dL/dalpha, dL/dpos, dL/dvel) through the adjoint."""
    pos = case.positions() if pos is None else pos
    vel = case.velocities() if vel is None else vel
    a = torch.tensor(float(alpha), dtype=torch.float64, device=pos.device, requires_grad=True)
    p = pos.clone().requires_grad_(True)
    v = vel.clone().requires_grad_(True)
    loss = WallLoadLoss.apply(a, p, v, case)
    ga, gp, gv = torch.autograd.grad(loss, (a, p, v))
    return loss.detach(), ga, gp, gv


def central_difference(case, alpha, pos, vel, eps=1e-6, d_alpha=0.0, d_pos=None, d_vel=None):
    """Central finite difference of the loss along (d_alpha, d_pos, d_vel)."""
    dp_ = torch.zeros_like(pos) if d_pos is None else d_pos
    dv_ = torch.zeros_like(vel) if d_vel is None else d_vel
    lp = case.loss(alpha + eps * d_alpha, pos + eps * dp_, vel + eps * dv_)
    lm = case.loss(alpha - eps * d_alpha, pos - eps * dp_, vel - eps * dv_)
    return ((lp - lm) / (2.0 * eps)).item()
