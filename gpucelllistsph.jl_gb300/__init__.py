"""GB300-native (sm_103a) hot path of GPUCellListSPH.jl.

Host-side mirror of the reference's Julia API over the C-ABI library
libgcsph.so (include/gcsph.h): GPUCellList / update / partialupdate /
neighborlist / neighborlistview (src/celllist.jl), SPHProblem / stepsolve /
timesolve and the getters (src/sphproblem.jl), and the exported kernel
functions (src/gpukernels_sph.jl).  All compute runs in the CUDA library;
there is no CPU fallback.
"""
from ._lib import GcsphError, launch_count, load as load_library, lib_path
from .celllist import GPUCellList, update, partialupdate, neighborlist, neighborlistview
from .sphproblem import (SPHProblem, WendlandC2, stepsolve, timesolve, get_points, get_velocity, get_density,
                         get_pressure, get_acceleration, get_dpccorr, get_simtime, get_dt, get_sumw, get_sumgradw,
                         get_ptype)
from . import kernels, workloads, ensemble, serving, vtkio, diagnostics
from .vtkio import writevtk, writecsv
from .ensemble import Ensemble, InstanceSpec, spec_from_case

__all__ = ["GcsphError", "GPUCellList", "update", "partialupdate", "neighborlist", "neighborlistview",
           "SPHProblem", "WendlandC2", "stepsolve", "timesolve", "get_points", "get_velocity", "get_density",
           "get_pressure", "get_acceleration", "get_dpccorr", "get_simtime", "get_dt", "get_sumw", "get_sumgradw",
           "get_ptype", "kernels", "workloads", "launch_count", "load_library", "lib_path", "ensemble", "Ensemble",
           "InstanceSpec", "spec_from_case", "serving", "vtkio", "writevtk", "writecsv", "diagnostics"]
