"""GB300-native (sm_103a) D2Q9 BGK lattice Boltzmann hot path.

Drop-in modules with the reference's names and call signatures:

  lattice_boltzmann_method  streaming, collision, moments, equilibrium, step
  boundary_conditions       rigid_wall, moving_wall, rigid_object, inlet,
                            outlet, periodic_with_pressure_variations
  boundary_utils            Couette / Poiseuille / von Karman compositions,
                            cavity, the halo hook
  initial_values            initial density and velocity fields

plus ``Lattice``, the device-resident hot loop.  All arithmetic runs in the
CUDA kernels of ``liblbm_gb300.so`` (built by ``_build.build()``); there is
no CPU path.
"""
from . import _lib  # noqa: F401
from . import boundary_conditions, boundary_utils, initial_values, lattice_boltzmann_method  # noqa: F401
from . import analysis, batch, scenarios, serving, sweeps  # noqa: F401
from .boundary_utils import Boundary  # noqa: F401
from .lattice import Lattice  # noqa: F401

__all__ = ["Lattice", "Boundary", "lattice_boltzmann_method", "boundary_conditions", "boundary_utils",
           "initial_values"]
