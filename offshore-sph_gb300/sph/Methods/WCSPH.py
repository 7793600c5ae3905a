"""WCSPH method (src/Methods/WCSPH.py:33-203) on the GB300 path.

Same constructor and attributes as the reference (height, rho0, useXSPH,
useSummationDensity, epsilon, gamma, co, B, Pb, alpha, beta, r0, D, p1, p2);
the attributes stay assignable, as on the reference's jitclass, and are read
at every device call.  The per-particle methods run on the device.  The
per-neighbour-block methods (compute_density_change, compute_acceleration,
compute_velocity) take the reference's arguments -- one particle and its
neighbours as a computed_dtype block -- and evaluate the block on the device
(sph_block_equations); the step itself runs the same equations fused in its
pair kernels.
"""
import math

import numpy as np

from .. import core
from ..Common import ParticleType
from .Method import Method


class WCSPH(Method):
    def __init__(self, height: float, r0: float, rho0: float, useXSPH: bool, Pb: float,
                 useSummationDensity: bool = False):
        self.height = height
        self.rho0 = rho0
        self.useXSPH = useXSPH
        self.useSummationDensity = useSummationDensity
        self.epsilon = 0.5
        self.gamma = 7.0
        self.co = 10.0 * math.sqrt(2 * 9.81 * self.height)  # TaitEOS_co (TaitEOS.py:40-44)
        self.B = self.co * self.co * self.rho0 / self.gamma  # TaitEOS_B (TaitEOS.py:33-38)
        self.Pb = Pb
        self.alpha = 0.01
        self.beta = 0.0
        self.r0 = r0
        self.D = 5 * 9.81 * self.height
        self.p1 = 4
        self.p2 = 2

    def wcsph_struct(self):
        """The sph_wcsph_t of the current attribute values."""
        return core.wcsph_struct(self.height, self.r0, self.rho0, use_xsph=self.useXSPH, Pb=self.Pb,
                                 use_summation_density=self.useSummationDensity, alpha=self.alpha,
                                 beta=self.beta, epsilon=self.epsilon, gamma=self.gamma, co=self.co, B=self.B,
                                 D=self.D, p1=float(self.p1), p2=float(self.p2))

    def initialize(self, pA):
        """Hydrostatic density of the given (fluid) particles
        (WCSPH.py:82-108, TaitEOS_height)."""
        def op(dp):
            cfg = core.config_struct(h_fixed=0.0)
            # sph_initialize also sets h, p and c; keep the caller's h, p, c
            h, p, c = dp.h.clone(), dp.p.clone(), dp.c.clone()
            core.initialize(dp, self.wcsph_struct(), cfg)
            dp.h.copy_(h)
            dp.p.copy_(p)
            dp.c.copy_(c)
        return core.on_device(pA, op, fields=("rho",), as_fluid=True)

    def compute_pressure(self, pA):
        """Tait EOS + Pb for every particle (WCSPH.py:131-149)."""
        out = {}

        def op(dp):
            core.eos(dp, self.wcsph_struct())
            out["p"] = dp.p.cpu().numpy()
        core.on_device(pA, op, fields=())
        return out["p"]

    def compute_speed_of_sound(self, pA):
        """co for every particle (WCSPH.py:110-129)."""
        return np.full(len(pA), self.co, dtype=np.float64)

    def _block(self, p, comp):
        return core.block_equations(comp, p, self.wcsph_struct())

    def compute_acceleration(self, p, comp):
        """Momentum with artificial viscosity, then gravity (WCSPH.py:151-169,
        src/Equations/Momentum.py:5-57): [a_x, a_y - 9.81]."""
        out = self._block(p, comp)
        return [float(out[1]), float(out[2]) - 9.81]

    def compute_velocity(self, p, comp):
        """XSPH (WCSPH.py:171-189, src/Equations/XSPH.py:5-31):
        [vx, vy, vx + xsph_x, vy + xsph_y] with XSPH, else [vx, vy, 0, 0]."""
        if self.useXSPH:
            out = self._block(p, comp)
            return [float(p["vx"]), float(p["vy"]), float(p["vx"]) + float(out[5]), float(p["vy"]) + float(out[6])]
        return [float(p["vx"]), float(p["vy"]), 0.0, 0.0]

    def compute_density_change(self, p, comp):
        """Continuity (WCSPH.py:191-203, src/Equations/Continuity.py:4-16), or
        0 with summation density."""
        if self.useSummationDensity:
            return 0.0
        return float(self._block(p, comp)[0])
