"""GB300-native transient solve-and-sensitivity path of TopOpt_in_PETSc_Transient.

The compute backend is libtopopt_gb300.so (sm_103a CUDA kernels behind the C
ABI in include/topopt_gb300.h).  Importing the package does not load it; the
first object construction does, and fails loudly if it is missing.
"""
from ._lib import TopoError, load  # noqa: F401
from .topopt import (MMA, MPIIO, SOMMG, Filter, LinearElasticity, PDEFilt, VecScale,  # noqa: F401
                     read_petsc_vecs, write_petsc_vecs)
from .design import TopOpt, design_iteration, final_physics_output, load_restart, write_restart_files  # noqa: F401

__all__ = ["LinearElasticity", "PDEFilt", "Filter", "MMA", "MPIIO", "SOMMG", "TopOpt", "design_iteration", "TopoError", "load"]
