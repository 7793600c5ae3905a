"""Predictor-corrector (src/Integrators/PEC.py:11-89) on the device.

predict / correct take and return a particle_dtype array like the
reference's jitclass methods, applying the update to the particles passed
(the Solver passes the fluid ones); they run as sph_predict / sph_correct.
Inside Solver.run the corrector of one step and the predictor of the next
are fused into one device pass."""
import torch

from .. import _lib, core
from .Integrator import Integrator


class PEC(Integrator):
    integrator_id = _lib.INTEGRATOR_PEC

    def __init__(self, useXSPH: bool = True, strict: bool = True):
        self.useXSPH = useXSPH
        self.strict = strict

    def isMultiStage(self) -> bool:
        return False

    def _cfg(self, damping):
        return core.config_struct(integrator=_lib.INTEGRATOR_PEC, pec_use_xsph=self.useXSPH, pec_strict=self.strict,
                                  damping=damping)

    def predict(self, dt: float, pA, damping: float):
        dtd = torch.tensor([dt], dtype=torch.float64, device="cuda")
        return core.on_device(pA, lambda dp: core.predict(dp, self._cfg(damping), dtd),
                              fields=("x", "y", "vx", "vy", "rho", "x0", "y0", "vx0", "vy0", "rho0"),
                              as_fluid=True)

    def correct(self, dt: float, pA, damping: float):
        dtd = torch.tensor([dt], dtype=torch.float64, device="cuda")
        return core.on_device(pA, lambda dp: core.correct(dp, self._cfg(damping), dtd),
                              fields=("x", "y", "vx", "vy", "rho"), as_fluid=True)
