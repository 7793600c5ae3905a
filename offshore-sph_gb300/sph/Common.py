"""Particle data ABI shared with Offshore-SPH.

``particle_dtype`` is field-for-field the reference's record
(``src/Common.py:26-57``): the same names, order and types (154 bytes, packed),
so that arrays built for the reference load here unchanged and results can be
handed back in the reference's format.  ``ParticleType`` mirrors
``src/Common.py:8-12``; ``computed_dtype`` is the reference's per-neighbour
block record (``src/Common.py:60-98``) that the per-block plugin methods of a
Method take.
"""
import enum

import numpy as np


class ParticleType(enum.IntEnum):
    Fluid = 0
    Boundary = 1
    TempBoundary = 2
    Coupled = 3


def get_label_code(label: str):
    codes = {"fluid": ParticleType.Fluid, "boundary": ParticleType.Boundary,
             "temp-boundary": ParticleType.TempBoundary, "coupled": ParticleType.Coupled}
    if label not in codes:
        raise Exception("Argument out of range")
    return codes[label]


#: the f64 fields of particle_dtype, in record order
FLOAT_FIELDS = ("m", "rho", "p", "c", "drho", "h", "x", "y", "vx", "vy", "ax", "ay",
                "xsphx", "xsphy", "x0", "y0", "vx0", "vy0", "rho0")

particle_dtype = np.dtype({
    "names": ["deleted", "label"] + list(FLOAT_FIELDS),
    "formats": [np.bool_, np.int8] + [np.float64] * len(FLOAT_FIELDS),
})

assert particle_dtype.itemsize == 154

#: one neighbour of a particle as _assignProps fills it
#: (src/Tools/SolverTools.py:74-104): the argument of Method.compute_* per block
computed_dtype = np.dtype({
    "names": ["label", "m", "p", "rho", "h", "q", "c", "r", "w", "dw_x", "dw_y", "x", "y", "vx", "vy"],
    "formats": [np.int8] + [np.float64] * 14,
})
