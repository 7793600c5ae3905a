"""The Integrator plugin contract (src/Integrators/Integrator.py:4-37)."""
import abc


class Integrator:
    #: SPH_INTEGRATOR_* of the C ABI
    integrator_id = None
    useXSPH = False
    strict = False

    @abc.abstractmethod
    def isMultiStage(self) -> bool:
        pass

    @abc.abstractmethod
    def predict(self, dt, pA, damping):
        pass

    @abc.abstractmethod
    def correct(self, dt, pA, damping):
        pass
