"""GB300-native explicit finite-volume step of BlackSiberian/HyperelasticSolver.

The compute path is libhyperelastic_cuda.so (CUDA C++ for sm_103a, C ABI in
include/hyperelastic.h). The modules named after the reference's Julia modules
(`Strains`, `EquationsOfState`, `Hyperelasticity`, `HyperelasticityMPh`,
`NumFluxes`) and `solver` (the main.jl time loop) are thin ctypes mirrors of that
ABI. There is no CPU fallback: without the built library or a CUDA device every
call raises.
"""
from . import _lib
from .build import build as build_library
from . import EquationsOfState, Strains, Hyperelasticity, HyperelasticityMPh, NumFluxes, solver, _cases, adjoint
from .EquationsOfState import Barton2009
from .solver import Solver, Batch

__all__ = ["Barton2009", "Solver", "Batch", "EquationsOfState", "Strains", "Hyperelasticity", "HyperelasticityMPh",
           "NumFluxes", "solver", "build_library"]
