"""Monaghan's symplectic Verlet, drift-kick-drift (src/Integrators/Verlet.py:7-53),
on the device.

predict drifts the positions by half a step; correct kicks the velocities by
the new accelerations and drifts the second half with the new velocity (or
XSPH).  As in the reference, the density is not integrated.  Inside
Solver.run the corrector of one step and the predictor of the next are fused
into one device pass."""
import torch

from .. import _lib, core
from .Integrator import Integrator


class Verlet(Integrator):
    integrator_id = _lib.INTEGRATOR_VERLET

    def __init__(self, useXSPH: bool):
        self.useXSPH = useXSPH

    def isMultiStage(self) -> bool:
        return False

    def _cfg(self):
        return core.config_struct(integrator=_lib.INTEGRATOR_VERLET, pec_use_xsph=self.useXSPH)

    def predict(self, dt: float, pA, damping: float = 0.0):
        dtd = torch.tensor([dt], dtype=torch.float64, device="cuda")
        return core.on_device(pA, lambda dp: core.predict(dp, self._cfg(), dtd), fields=("x", "y"), as_fluid=True)

    def correct(self, dt: float, pA, damping: float = 0.0):
        dtd = torch.tensor([dt], dtype=torch.float64, device="cuda")
        return core.on_device(pA, lambda dp: core.correct(dp, self._cfg(), dtd), fields=("x", "y", "vx", "vy"),
                              as_fluid=True)
