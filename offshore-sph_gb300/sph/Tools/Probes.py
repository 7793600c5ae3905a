"""Field probes at arbitrary points on the device.

pressure_SPH is the interpolation the reference's ice-coupling example
builds from the neighbour finder (examples/IceBreak.py:253-285): the nearPos
set of (x, y - hh) with smoothing length h, the kernel value W(r, h), the
Shepard normalisation (src/Equations/Shepard.py), summation density
(src/Equations/SummationDensity.py) and the Tait EOS.  Here it takes many
points at once and runs on the solver's device state and the table of its
last neighbour build."""
import numpy as np

from .. import core


def pressure_SPH(x, y, solver, h, hh=0.0):
    """(rho, p) as numpy arrays at the points (x, y - hh) of the solver's
    current state."""
    x = np.atleast_1d(np.asarray(x, dtype=np.float64))
    y = np.atleast_1d(np.asarray(y, dtype=np.float64)) - hh
    hs = np.full(x.shape, float(h))
    rho, p = core.probe_density(solver._dp, solver.method.wcsph_struct(), solver.kernel.kernel_id, solver._ws, x, y,
                                hs, hs)
    return rho.cpu().numpy(), p.cpu().numpy()
