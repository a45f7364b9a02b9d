"""GB300 (sm_103a) midpoint Lennard-Jones force path: a drop-in for exaMD's
exaMD_forces_midpoint_all, plus velocity-Verlet and batched ensembles.

The compute path is the CUDA library examd_gb300/_lib/libexamd_gb300.so
(C ABI: include/examd_gb300.h); this package is its Python front end.
"""
from .api import (FP64, MIXED, ExamdError, MidpointLJ, autotune, forces_midpoint_all, gen_fcc, gen_jittered_sc, gen_random,
                  gen_velocities, own_table, pinned_empty, read_particles, tile_split, write_particles)

__all__ = ["FP64", "MIXED", "ExamdError", "MidpointLJ", "autotune", "forces_midpoint_all", "gen_fcc", "gen_jittered_sc",
           "gen_random", "gen_velocities", "own_table", "pinned_empty", "read_particles", "tile_split", "write_particles"]
