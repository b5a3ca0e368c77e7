"""GB300-native ePIC2D time-step loop: deposit, Poisson solve, E-field, gather +
push and MCC as CUDA kernels for sm_103a behind the C ABI of include/epic2d.h."""
from .api import (Conductor, Config, EpicError, Simulation, SpeciesDesc, conductors_from_ini, config_from_ini,  # noqa: F401
                  default_config, lib)
