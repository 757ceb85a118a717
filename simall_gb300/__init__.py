"""GB300 (sm_103a) pressure-correction path for SimAll.

The face-loop assembly of the pressure-correction Laplacian and the
preconditioned CG solve on it, as hand-written CUDA kernels behind a C ABI
(include/simall_gpu.h, libsimall_gpu.so).  This package is the Python-side
mirror of the reference's solver interface plus the mesh/assembly wrappers.
"""
from . import build
from .batch import BatchedSolver
from ._lib import MEM_DEVICE, MEM_HOST, SimallError, load
from .fields import DeviceFieldRegistry, checkpoint_read, checkpoint_write
from .mesh import BCType, MeshSoA, PressureSystem, cartesian, rcm
from .simple import GpuSimpleAlgorithm, PimpleOptions, PisoOptions, SimpleOptions, SimpleResiduals
from .topology import GpuSimpTopology, SimpConfig
from .solver import (CgGpu, Context, CSRMatrix, GpuCGSolver, GpuPreconditioner, GpuSolverConfig, GpuSolverStats, GpuLinearSolver, LinearSolverConfig, LinearSolverKind,
                     Precision, PreconditionerKind, default_context, make_bicgstab, make_cg, make_gmres,
                     make_linear_solver, make_tfqmr)

__all__ = ["build", "BatchedSolver", "load", "MEM_HOST", "MEM_DEVICE", "SimallError", "BCType", "MeshSoA", "PressureSystem",
           "cartesian", "rcm", "Context", "CSRMatrix", "GpuCGSolver", "LinearSolverConfig", "LinearSolverKind",
           "Precision", "PreconditionerKind", "default_context", "make_cg", "make_linear_solver", "GpuLinearSolver",
           "make_gmres", "make_bicgstab", "make_tfqmr", "GpuSimpleAlgorithm", "SimpleOptions", "SimpleResiduals", "PisoOptions",
           "PimpleOptions",
           "DeviceFieldRegistry", "checkpoint_read", "checkpoint_write", "GpuSimpTopology", "SimpConfig",
           "CgGpu", "GpuPreconditioner", "GpuSolverConfig", "GpuSolverStats"]
