"""GB300-native ePIC2D time-step loop: deposit, Poisson solve, E-field, gather +
push and MCC as CUDA kernels for sm_103a behind the C ABI of include/epic2d.h."""
from .api import (Conductor, Config, Emitter, EpicError, Simulation, SpeciesDesc, conductors_from_ini,  # noqa: F401
                  config_from_ini, default_config, emitters_from_ini, lib)
