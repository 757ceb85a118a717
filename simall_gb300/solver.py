"""Python mirror of SimAll's linear-solver interface for the pressure path.

Same names and semantics as the reference (src/solver/Solver.hpp:67-102,
src/solver/LinearSolvers.hpp:28-43, src/solver/CSRMatrix.hpp:16-36):
`LinearSolverConfig`, `PreconditionerKind`, `CSRMatrix`, and an
`ILinearSolver`-shaped `GpuCGSolver` whose `solve(A, b, x)` overwrites x from
zero and returns the iteration count exactly as CGSolver::solve does
(LinearSolvers.cpp:420-451), with `last_residual()` the relative residual.
Every call goes through libsimall_gpu.so; there is no CPU path.
"""
from __future__ import annotations

import atexit
import ctypes as C
import weakref
from dataclasses import dataclass, field
from enum import IntEnum

import numpy as np

from . import _lib
from ._lib import MEM_DEVICE, MEM_HOST, SimallError, check


class LinearSolverKind(IntEnum):
    GMRES = 0
    BiCGSTAB = 1
    CG = 2
    TFQMR = 3


class PreconditionerKind(IntEnum):
    Jacobi = 0
    ILU = 1
    SSOR = 2
    AMG = 3
    None_ = 4


class Precision(IntEnum):
    FP64 = 0
    MIXED = 1


@dataclass
class LinearSolverConfig:
    """LinearSolverConfig (src/solver/Solver.hpp:83-90), same defaults."""

    kind: LinearSolverKind = LinearSolverKind.GMRES
    preconditioner: PreconditionerKind = PreconditionerKind.ILU
    tolerance: float = 1.0e-8
    maxIterations: int = 1000
    restart: int = 30


@dataclass
class CSRMatrix:
    """CSRMatrix (src/solver/CSRMatrix.hpp:16-36): int32 rowPtr/colIdx, FP64 values."""

    rowPtr: np.ndarray = field(default_factory=lambda: np.zeros(0, np.int32))
    colIdx: np.ndarray = field(default_factory=lambda: np.zeros(0, np.int32))
    values: np.ndarray = field(default_factory=lambda: np.zeros(0, np.float64))

    def rows(self) -> int:
        return 0 if len(self.rowPtr) == 0 else len(self.rowPtr) - 1

    def nnz(self) -> int:
        return len(self.colIdx)


def _is_torch(a) -> bool:
    return type(a).__module__.startswith("torch")


def ptr_and_mem(a):
    """(address, memory kind) of a numpy array or a torch tensor."""
    if a is None:
        return None, MEM_HOST
    if _is_torch(a):
        if not a.is_contiguous():
            raise ValueError("tensor must be contiguous")
        return a.data_ptr(), (MEM_DEVICE if a.is_cuda else MEM_HOST)
    if not a.flags["C_CONTIGUOUS"]:
        raise ValueError("array must be C-contiguous")
    return a.ctypes.data, MEM_HOST


# Every live library object, so that interpreter shutdown releases children
# (solvers, pressure systems) before the contexts they point into, while the
# CUDA runtime is still up.  Finalizer order at shutdown is otherwise
# arbitrary.
_live_children: "weakref.WeakSet" = weakref.WeakSet()
_live_contexts: "weakref.WeakSet" = weakref.WeakSet()


def register_child(obj) -> None:
    _live_children.add(obj)


@atexit.register
def _release_all() -> None:
    for o in list(_live_children):
        try:
            o.close()
        except Exception:
            pass
    for c in list(_live_contexts):
        try:
            c.close()
        except Exception:
            pass


class Context:
    """A device + stream (simall_context)."""

    def __init__(self, device: int = 0, stream=None):
        self.L = _lib.load()
        h = C.c_void_p()
        s = None
        if stream is not None:
            s = stream.cuda_stream if hasattr(stream, "cuda_stream") else int(stream)
        st = self.L.simall_context_create(int(device), s, C.byref(h))
        if st != 0:
            raise SimallError(st, "simall_context_create")
        self.handle = h.value
        self.device = device
        self.children: "weakref.WeakSet" = weakref.WeakSet()
        _live_contexts.add(self)

    @property
    def stream(self) -> int:
        return self.L.simall_context_stream(self.handle) or 0

    @property
    def kernel_launches(self) -> int:
        return int(self.L.simall_context_kernel_launches(self.handle))

    def synchronize(self):
        check(self.L.simall_context_synchronize(self.handle), self.handle)

    def last_error(self) -> str:
        return (self.L.simall_context_last_error(self.handle) or b"").decode()

    def close(self):
        if getattr(self, "handle", None):
            for ch in list(self.children):
                ch.close()
            self.L.simall_context_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


_default_ctx: Context | None = None


def default_context() -> Context:
    global _default_ctx
    if _default_ctx is None:
        _default_ctx = Context(0)
    return _default_ctx


class GpuCGSolver:
    """ILinearSolver (src/solver/Solver.hpp:92-100) backed by the device PCG.

    precision=Precision.MIXED selects the FP32-inner / FP64-refined solver
    (Jacobi only).  `stats` holds the SolverStats of the last solve.
    """

    def __init__(self, cfg: LinearSolverConfig | None = None, precision: Precision = Precision.FP64,
                 ctx: Context | None = None, reliable_delta: float = 0.1, check_interval: int = 0,
                 engine: int = 0, _kind: LinearSolverKind = LinearSolverKind.CG):
        """engine: 0 automatic (one thread-block cluster for systems that fit),
        1 per-iteration kernels only."""
        cfg = cfg or LinearSolverConfig(kind=LinearSolverKind.CG)
        self.cfg = cfg
        self.ctx = ctx or default_context()
        self.L = self.ctx.L
        c = _lib.SolverConfig()
        self.L.simall_solver_config_default(C.byref(c))
        c.preconditioner = int(cfg.preconditioner)
        c.tolerance = float(cfg.tolerance)
        c.max_iterations = int(cfg.maxIterations)
        c.precision = int(precision)
        c.reliable_delta = float(reliable_delta)
        c.check_interval = int(check_interval)
        c.engine = int(engine)
        c.kind = int(_kind)
        c.restart = int(cfg.restart)
        h = C.c_void_p()
        check(self.L.simall_solver_create(self.ctx.handle, C.byref(c), C.byref(h)), self.ctx.handle)
        self.handle = h.value
        self.stats = _lib.SolverStats()
        self._keep = None  # device arrays referenced by set_matrix
        register_child(self)
        self.ctx.children.add(self)

    # -- ILinearSolver -------------------------------------------------------
    def solve(self, A: CSRMatrix, b, x) -> int:
        """CGSolver::solve: preconditioner set up again, x overwritten from 0."""
        n = A.rows()
        rp = np.ascontiguousarray(A.rowPtr, np.int32)
        ci = np.ascontiguousarray(A.colIdx, np.int32)
        va = np.ascontiguousarray(A.values, np.float64)
        bb = np.ascontiguousarray(b, np.float64)
        if len(bb) != n:
            raise SimallError(8, "b size")
        # the library writes x directly when the caller's array can take it (no temporary, no copy)
        direct = (isinstance(x, np.ndarray) and x.dtype == np.float64 and x.shape == (n,)
                  and x.flags["C_CONTIGUOUS"] and x.flags["WRITEABLE"])
        out = x if direct else np.empty(n, np.float64)
        st = self.L.simall_solver_solve_csr(self.handle, n, len(ci), rp.ctypes.data, ci.ctypes.data,
                                            va.ctypes.data, bb.ctypes.data, out.ctypes.data, C.byref(self.stats))
        check(st, self.ctx.handle)
        if not direct:
            if isinstance(x, np.ndarray) and x.shape == out.shape:
                x[...] = out
            elif isinstance(x, list):
                x[:] = out.tolist()
        return int(self.stats.iterations)

    def last_residual(self) -> float:
        return float(self.L.simall_solver_last_residual(self.handle))

    # -- device-resident use ---------------------------------------------------
    def set_matrix(self, rowPtr, colIdx, values):
        """Upload (numpy) or reference (CUDA tensors) a CSR matrix."""
        p0, m0 = ptr_and_mem(rowPtr)
        p1, _ = ptr_and_mem(colIdx)
        p2, _ = ptr_and_mem(values)
        n = len(rowPtr) - 1
        check(self.L.simall_solver_set_matrix(self.handle, n, len(colIdx), p0, p1, p2, m0), self.ctx.handle)
        self._keep = (rowPtr, colIdx, values) if m0 == MEM_DEVICE else None
        self.n = n

    def update_values(self, values):
        p, m = ptr_and_mem(values)
        check(self.L.simall_solver_update_values(self.handle, p, m), self.ctx.handle)

    def solve_into(self, b, x) -> int:
        """Solve with the current matrix; b and x both numpy or both CUDA tensors."""
        pb, mb = ptr_and_mem(b)
        px, mx = ptr_and_mem(x)
        if mb != mx:
            raise ValueError("b and x must live in the same memory")
        check(self.L.simall_solver_solve(self.handle, pb, px, mb, C.byref(self.stats)), self.ctx.handle)
        return int(self.stats.iterations)

    def spmv(self, x, y):
        px, mx = ptr_and_mem(x)
        py, _ = ptr_and_mem(y)
        check(self.L.simall_solver_spmv(self.handle, px, py, mx), self.ctx.handle)

    def precond_apply(self, r, z):
        """z = M^-1 r with the preconditioner set up for the current matrix
        (IPreconditioner::apply, src/solver/LinearSolvers.hpp:33-34)."""
        pr, mr = ptr_and_mem(r)
        pz, _ = ptr_and_mem(z)
        check(self.L.simall_solver_precond_apply(self.handle, pr, pz, mr), self.ctx.handle)

    def amg_levels(self) -> list[int]:
        """Rows of each level of the AMG hierarchy of the current matrix."""
        n = C.c_int(0)
        rows = np.zeros(16, np.int32)
        check(self.L.simall_solver_amg_levels(self.handle, C.byref(n), rows.ctypes.data_as(C.c_void_p), 16),
              self.ctx.handle)
        return [int(v) for v in rows[:n.value]]

    def close(self):
        if getattr(self, "handle", None) and getattr(self.ctx, "handle", None):
            self.L.simall_solver_destroy(self.handle)
        self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class GpuPreconditioner(IntEnum):
    """gpu::GpuPreconditioner (src/gpu/CgGpu.hpp:52-57)."""
    None_ = 0
    Jacobi = 1
    ILU0 = 2


_GPU_PRECOND_TO_C = {GpuPreconditioner.None_: 4, GpuPreconditioner.Jacobi: 0, GpuPreconditioner.ILU0: 1}
_C_TO_GPU_PRECOND = {v: k for k, v in _GPU_PRECOND_TO_C.items()}


@dataclass
class GpuSolverConfig:
    """gpu::GpuSolverConfig (src/gpu/CgGpu.hpp:59-66)."""
    preconditioner: GpuPreconditioner = GpuPreconditioner.Jacobi
    tolerance: float = 1.0e-8
    maxIterations: int = 1000
    relativeOrders: float = 0.0


@dataclass
class GpuSolverStats:
    """gpu::GpuSolverStats (src/gpu/CgGpu.hpp:68-75)."""
    iterations: int = 0
    finalResidual: float = 0.0
    initialResidual: float = 0.0
    converged: bool = False
    timeSeconds: float = 0.0


class CgGpu:
    """gpu::CgGpu (src/gpu/CgGpu.hpp:49-124) on the device: the FP64 PCG of
    this library with CgGpu::solve's conventions (SIMALL_SEMANTICS_CGGPU):
    x is the initial guess and the solution, stop on ||r||/bRef <= tolerance
    or the relativeOrders drop, None = no preconditioner, ILU0 falls back to
    Jacobi for good when its factor meets a zero pivot."""

    def __init__(self, cfg: GpuSolverConfig | None = None, ctx: Context | None = None):
        self.ctx = ctx or default_context()
        self.L = self.ctx.L
        self._cfg = cfg or GpuSolverConfig()
        self.handle = None
        self._make()
        self._last = 0.0
        self.n = 0
        register_child(self)
        self.ctx.children.add(self)

    def _make(self):
        if self.handle:
            self.L.simall_solver_destroy(self.handle)
        c = _lib.SolverConfig()
        self.L.simall_solver_config_default(C.byref(c))
        c.preconditioner = _GPU_PRECOND_TO_C[GpuPreconditioner(self._cfg.preconditioner)]
        c.tolerance = float(self._cfg.tolerance)
        c.max_iterations = int(self._cfg.maxIterations)
        c.semantics = 1
        c.relative_orders = float(self._cfg.relativeOrders)
        h = C.c_void_p()
        check(self.L.simall_solver_create(self.ctx.handle, C.byref(c), C.byref(h)), self.ctx.handle)
        self.handle = h.value

    def config(self) -> GpuSolverConfig:
        return self._cfg

    def set_config(self, cfg: GpuSolverConfig):
        """Takes effect at the next set_matrix, as in the reference (the
        preconditioner data is built there)."""
        self._cfg = cfg
        self._make()

    def set_matrix(self, rowPtr, colIdx, values):
        p0, m0 = ptr_and_mem(rowPtr)
        p1, _ = ptr_and_mem(colIdx)
        p2, _ = ptr_and_mem(values)
        self.n = len(rowPtr) - 1
        check(self.L.simall_solver_set_matrix(self.handle, self.n, len(colIdx), p0, p1, p2, m0), self.ctx.handle)
        # the preconditioner after CgGpu::set_matrix's ILU0 -> Jacobi fall-back
        self._cfg.preconditioner = self._precond_now()

    def _precond_now(self) -> GpuPreconditioner:
        pc = C.c_int(-1)
        check(self.L.simall_solver_preconditioner(self.handle, C.byref(pc)), self.ctx.handle)
        return _C_TO_GPU_PRECOND[pc.value]

    def solve(self, b, x) -> GpuSolverStats:
        """Solve A x = b; x (numpy array, or a CUDA tensor with b one too) is
        the initial guess on entry and the solution on exit."""
        pb, mb = ptr_and_mem(b)
        px, mx = ptr_and_mem(x)
        if mb != mx:
            raise ValueError("b and x must live in the same memory")
        st = _lib.SolverStats()
        check(self.L.simall_solver_solve(self.handle, pb, px, mb, C.byref(st)), self.ctx.handle)
        self.stats = st
        self._last = float(st.residual_norm)
        return GpuSolverStats(int(st.iterations), float(st.residual_norm), float(st.initial_residual),
                              bool(st.converged), float(st.seconds))

    def last_residual(self) -> float:
        return self._last

    def close(self):
        if getattr(self, "handle", None) and getattr(self.ctx, "handle", None):
            self.L.simall_solver_destroy(self.handle)
        self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class GpuLinearSolver(GpuCGSolver):
    """ILinearSolver of the kind cfg.kind names: GMRES(cfg.restart), BiCGSTAB
    or TFQMR (GMRESmSolver / BiCGSTABSolver / TfqmrSolver,
    src/solver/LinearSolvers.cpp:268-405, :497-609) in FP64 with the Jacobi,
    ILU(0) or SSOR preconditioner, or CG."""

    def __init__(self, cfg: LinearSolverConfig | None = None, ctx: Context | None = None, check_interval: int = 0,
                 **kw):
        cfg = cfg or LinearSolverConfig()
        super().__init__(cfg, ctx=ctx, check_interval=check_interval, _kind=cfg.kind, **kw)


def make_cg(cfg: LinearSolverConfig, **kw) -> GpuCGSolver:
    return GpuCGSolver(cfg, **kw)


def make_gmres(cfg: LinearSolverConfig, **kw) -> GpuLinearSolver:
    return GpuLinearSolver(LinearSolverConfig(LinearSolverKind.GMRES, cfg.preconditioner, cfg.tolerance,
                                              cfg.maxIterations, cfg.restart), **kw)


def make_bicgstab(cfg: LinearSolverConfig, **kw) -> GpuLinearSolver:
    return GpuLinearSolver(LinearSolverConfig(LinearSolverKind.BiCGSTAB, cfg.preconditioner, cfg.tolerance,
                                              cfg.maxIterations, cfg.restart), **kw)


def make_tfqmr(cfg: LinearSolverConfig, **kw) -> GpuLinearSolver:
    return GpuLinearSolver(LinearSolverConfig(LinearSolverKind.TFQMR, cfg.preconditioner, cfg.tolerance,
                                              cfg.maxIterations, cfg.restart), **kw)


def make_linear_solver(cfg: LinearSolverConfig, **kw) -> GpuCGSolver:
    """make_linear_solver (src/solver/Solver.cpp:25-39): CG, GMRES(m),
    BiCGSTAB and TFQMR all run on the device."""
    if cfg.kind == LinearSolverKind.CG:
        return GpuCGSolver(cfg, **kw)
    return GpuLinearSolver(cfg, **kw)
