"""TimeStep (src/Equations/TimeStep.py:7-91) on the device."""
from .. import core, state
from ..Common import ParticleType


class TimeStep:
    def compute(self, J, pA, gamma_c: float = 0.25, gamma_f: float = 0.25):
        """(dt, dt_courant, dt_force) over the fluid particles of pA (J is
        kept for the reference's signature; pA holds the particles)."""
        cfg = core.config_struct(cfl_c=gamma_c, cfl_f=gamma_f)
        wc = core.wcsph_struct(1.0, 1.0, 1000.0)
        dp = state.DeviceParticles.from_array(pA)
        ws = state.DeviceWorkspace(dp.n, 1)
        dt3 = core.timestep(dp, wc, cfg, ws).cpu().numpy()
        return float(dt3[0]), float(dt3[1]), float(dt3[2])
