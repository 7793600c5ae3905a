"""The Method plugin contract (src/Methods/Method.py:5-37)."""
import abc


class Method:
    """Generic SPH method: the Solver calls these to initialise particles and
    to evaluate pressure and speed of sound; the per-pair terms run inside the
    fused device pair kernel."""

    @abc.abstractmethod
    def initialize(self, pA):
        raise Exception("Not implemented!")

    @abc.abstractmethod
    def compute_speed_of_sound(self, pA):
        raise Exception("Not implemented!")

    @abc.abstractmethod
    def compute_pressure(self, pA):
        raise Exception("Not implemented!")

    @abc.abstractmethod
    def compute_density_change(self, p, comp):
        raise Exception("Not implemented!")

    @abc.abstractmethod
    def compute_acceleration(self, p, comp):
        raise Exception("Not implemented!")

    @abc.abstractmethod
    def compute_velocity(self, p, comp):
        raise Exception("Not implemented!")
