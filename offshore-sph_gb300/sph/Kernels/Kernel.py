"""The Kernel plugin contract (src/Kernels/Kernel.py:5-12)."""
import abc


class Kernel(metaclass=abc.ABCMeta):
    #: id of the kernel in the C ABI (SPH_KERNEL_*)
    kernel_id = None

    @abc.abstractstaticmethod
    def evaluate(r, h):
        pass

    @abc.abstractstaticmethod
    def gradient(x, r, h):
        pass
