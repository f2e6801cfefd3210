"""GB300-native clump-DEM engine: a drop-in for the step loop of AvalancheFlume3D.

The compute path is hand-written CUDA for sm_103a behind the C ABI of ``include/af3d.h``
(``libaf3d.so``, built in-tree by :mod:`avalancheflume3d_gb300.build`); this package is the
host-side mirror of the reference's step interface.  Importing it does not touch the GPU.
"""
from ._lib import (CELL_PAR, FP_EXACT, FP_FAST, FRICTION_DEV, FRICTION_HST, FUNNEL, INPUTS, PARTICLE,
                   PHASE_AVALANCHE, PHASE_FILL, SYSTEM_PAR, EngineError, LIB_PATH, lib)
from .engine import (Engine, Rannew64, calculate_particle_parameters, derive_system, error_check,
                     generate_particles, lattice_block, load_datainput, place_particles,
                     read_last_config, set_initial_velocity, sphere_centres, write_last_config,
                     append_snapshot)

__all__ = [
    "Engine", "EngineError", "lib", "LIB_PATH", "PARTICLE", "SYSTEM_PAR", "FUNNEL", "CELL_PAR",
    "INPUTS", "FRICTION_HST", "FRICTION_DEV", "PHASE_FILL", "PHASE_AVALANCHE", "FP_EXACT", "FP_FAST",
    "load_datainput",
    "derive_system", "error_check", "write_last_config", "read_last_config", "append_snapshot", "Rannew64",
    "generate_particles", "calculate_particle_parameters", "place_particles",
    "set_initial_velocity", "sphere_centres", "lattice_block",
]
