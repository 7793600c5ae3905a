"""Wendland C4 kernel (src/Kernels/Wendland.py:6-64) on the device.

evaluate / gradient take and return numpy arrays like the reference's static
functions; they run as elementwise maps in libsph_gb300 (sph_kernel_eval,
sph_kernel_grad).  The Solver uses kernel_id to select the kernel inside the
fused pair kernel.  Support 2h, like the cubic spline."""
import math

import numpy as np

from .. import _lib, core
from .Kernel import Kernel


class Wendland(Kernel):
    kernel_id = _lib.KERNEL_WENDLAND

    def __init__(self):
        self.alpha = 9.0 / (4.0 * math.pi)

    @staticmethod
    def evaluate(r, h):
        r, h = np.asarray(r, np.float64), np.asarray(h, np.float64)
        return core.kernel_eval(_lib.KERNEL_WENDLAND, r.ravel(), h.ravel()).cpu().numpy().reshape(r.shape)

    @staticmethod
    def gradient(x, r, h):
        x, r, h = np.asarray(x, np.float64), np.asarray(r, np.float64), np.asarray(h, np.float64)
        return core.kernel_grad(_lib.KERNEL_WENDLAND, x.ravel(), r.ravel(), h.ravel()).cpu().numpy().reshape(r.shape)
