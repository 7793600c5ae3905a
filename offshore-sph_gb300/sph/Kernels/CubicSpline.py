"""Cubic spline kernel (src/Kernels/CubicSpline.py:6-70) on the device.

evaluate / gradient take and return numpy arrays like the reference's static
functions; they run as elementwise maps in libsph_gb300 (sph_kernel_eval,
sph_kernel_grad).  The Solver uses kernel_id to select the kernel inside the
fused pair kernel."""
import math

import numpy as np

from .. import _lib, core
from .Kernel import Kernel


class CubicSpline(Kernel):
    kernel_id = _lib.KERNEL_CUBIC

    def __init__(self):
        self.alpha = 10 / (7 * math.pi)

    @staticmethod
    def evaluate(r, h):
        return core.kernel_eval(_lib.KERNEL_CUBIC, np.asarray(r, np.float64), np.asarray(h, np.float64)).cpu().numpy()

    @staticmethod
    def gradient(x, r, h):
        return core.kernel_grad(_lib.KERNEL_CUBIC, np.asarray(x, np.float64), np.asarray(r, np.float64),
                                np.asarray(h, np.float64)).cpu().numpy()
