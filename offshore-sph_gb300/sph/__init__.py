"""GB300-native WCSPH step behind Offshore-SPH's plugin surface.

Drop-in classes with the reference's names and constructors:

    from sph import Solver, WCSPH, CubicSpline, Gaussian, PEC, Euler
    solver = Solver(WCSPH(height, r0, rho0, useXSPH, Pb), PEC(useXSPH, strict), CubicSpline(), duration, h=...)
    solver.addParticles(particles)      # a particle_dtype array
    solver.setup(); solver.run()

Every stage of the step runs in libsph_gb300.so (CUDA, sm_103a) through its C
ABI (include/sph_gb300.h); there is no CPU fallback.
"""
from .Common import ParticleType, computed_dtype, particle_dtype, get_label_code
from .Methods.WCSPH import WCSPH
from .Kernels.CubicSpline import CubicSpline
from .Kernels.Gaussian import Gaussian
from .Kernels.Wendland import Wendland
from .Integrators.PEC import PEC
from .Integrators.Euler import Euler
from .Integrators.Verlet import Verlet
from .Integrators.NewmarkBeta import NewmarkBeta
from .Tools.NNLinkedList import NNLinkedList
from .Equations.TimeStep import TimeStep
from .Solver import Solver

__all__ = ["ParticleType", "computed_dtype", "particle_dtype", "get_label_code", "WCSPH", "CubicSpline", "Gaussian", "Wendland", "PEC",
           "Euler", "Verlet", "NewmarkBeta", "NNLinkedList", "TimeStep", "Solver"]
