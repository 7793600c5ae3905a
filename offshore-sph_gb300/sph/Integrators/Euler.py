"""Explicit Euler (src/Integrators/Euler.py:6-27) on the device."""
import torch

from .. import _lib, core
from .Integrator import Integrator


class Euler(Integrator):
    integrator_id = _lib.INTEGRATOR_EULER

    def isMultiStage(self) -> bool:
        return False

    def predict(self, dt: float, pA, damping: float = 0.0):
        """Euler.predict does nothing (Euler.py:13-15)."""
        return pA

    def correct(self, dt: float, pA, damping: float = 0.0):
        dtd = torch.tensor([dt], dtype=torch.float64, device="cuda")
        cfg = core.config_struct(integrator=_lib.INTEGRATOR_EULER)
        return core.on_device(pA, lambda dp: core.correct(dp, cfg, dtd), fields=("x", "y", "vx", "vy", "rho"),
                              as_fluid=True)
