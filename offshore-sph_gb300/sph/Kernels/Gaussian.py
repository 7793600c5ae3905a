"""Gaussian kernel truncated at q = 3 (src/Kernels/Gaussian.py:6-59) on the
device; evaluate / derivative / gradient as elementwise maps in
libsph_gb300."""
import numpy as np

from .. import _lib, core
from .Kernel import Kernel


class Gaussian(Kernel):
    kernel_id = _lib.KERNEL_GAUSSIAN

    @staticmethod
    def evaluate(r, h):
        r, h = np.broadcast_arrays(np.asarray(r, np.float64), np.asarray(h, np.float64))
        return core.kernel_eval(_lib.KERNEL_GAUSSIAN, r.ravel(), h.ravel()).cpu().numpy().reshape(r.shape)

    @staticmethod
    def derivative(r, h):
        r, h = np.broadcast_arrays(np.asarray(r, np.float64), np.asarray(h, np.float64))
        return core.gauss_deriv(r.ravel(), h.ravel()).cpu().numpy().reshape(r.shape)

    @staticmethod
    def gradient(x, r, h):
        x, r, h = np.broadcast_arrays(np.asarray(x, np.float64), np.asarray(r, np.float64),
                                      np.asarray(h, np.float64))
        return core.kernel_grad(_lib.KERNEL_GAUSSIAN, x.ravel(), r.ravel(), h.ravel()).cpu().numpy().reshape(r.shape)
