"""GB300-native bond-based peridynamics time step.

A drop-in for the integrators of PeriPy (``peripy.integrators``: the
OpenCL ones and the Cython CPU ``Euler``) under PeriPy's
``Model(...).simulate(...)`` API: the step runs as hand-written sm_103a
CUDA kernels behind the C ABI of ``include/pp_gb300.h``.
"""
from .integrators import (  # noqa: F401
    Integrator, Euler, EulerCUDA, EulerCromerCUDA, VelocityVerletCUDA, EulerCL,
    EulerCromerCL, VelocityVerletCL, CUDAContext, ContextError, get_context)
from .model import (  # noqa: F401
    Model, initial_crack_helper, create_crack, DimensionalityError,
    FamilyError, DamageModelError, InvalidIntegrator)

__version__ = "0.1.0"
