"""Batched pressure solves (simall_batch_* in include/simall_gpu.h).

Many independent SPD systems solved in one persistent launch, each with the
mixed-precision Jacobi-PCG; the Python side only concatenates the systems.
The launch shape comes from the autotuner (timed on the batch, or read from
its JSON cache, autotune_cache_lookup / autotune_cache_store).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from ._lib import check
from .solver import Context, LinearSolverConfig, LinearSolverKind, PreconditionerKind, default_context, ptr_and_mem, \
    register_child


class BatchedSolver:
    def __init__(self, cfg: LinearSolverConfig | None = None, ctx: Context | None = None, reliable_delta: float = 0.1):
        cfg = cfg or LinearSolverConfig(kind=LinearSolverKind.CG, preconditioner=PreconditionerKind.Jacobi)
        self.ctx = ctx or default_context()
        self.L = self.ctx.L
        c = _lib.SolverConfig()
        self.L.simall_solver_config_default(C.byref(c))
        c.preconditioner = int(cfg.preconditioner)
        c.tolerance = float(cfg.tolerance)
        c.max_iterations = int(cfg.maxIterations)
        c.precision = 1
        c.reliable_delta = float(reliable_delta)
        h = C.c_void_p()
        check(self.L.simall_batch_create(self.ctx.handle, C.byref(c), C.byref(h)), self.ctx.handle)
        self.handle = h.value
        register_child(self)
        self.ctx.children.add(self)
        self.n_systems = 0
        self.total = _lib.BatchStats()

    def set_systems(self, systems):
        """systems: iterable of (rowPtr, colIdx, values) with local indices."""
        systems = list(systems)
        rows = np.zeros(len(systems) + 1, np.int64)
        nnzs = np.zeros(len(systems) + 1, np.int64)
        for i, (rp, ci, va) in enumerate(systems):
            rows[i + 1] = rows[i] + len(rp) - 1
            nnzs[i + 1] = nnzs[i] + len(ci)
        rowPtr = np.concatenate([np.asarray(rp, np.int32) for rp, _, _ in systems])
        colIdx = np.concatenate([np.asarray(ci, np.int32) for _, ci, _ in systems])
        values = np.concatenate([np.asarray(va, np.float64) for _, _, va in systems])
        check(self.L.simall_batch_set_systems(self.handle, len(systems), rows.ctypes.data, nnzs.ctypes.data,
                                              rowPtr.ctypes.data, colIdx.ctypes.data, values.ctypes.data),
              self.ctx.handle)
        self.n_systems = len(systems)
        self.row_offsets = rows
        self.nnz_offsets = nnzs
        return rows

    def launch_shape(self, block_threads: int, ctas_per_sm: int = 1):
        check(self.L.simall_batch_launch_shape(self.handle, int(block_threads), int(ctas_per_sm)))

    def cluster_route(self, cluster_rows: int, cluster_ctas: int = 8, clusters: int = 4):
        """Systems (diagonal storage) of at least cluster_rows rows on one cluster each (0: none), on
        `clusters` clusters of cluster_ctas CTAs."""
        check(self.L.simall_batch_cluster_route(self.handle, int(cluster_rows), int(cluster_ctas), int(clusters)))

    def autotune_cache(self, path: str | None):
        """Autotuner cache file of this batch (None or "": none)."""
        check(self.L.simall_batch_autotune_cache(self.handle, (path or "").encode()))

    def solve(self, b, x=None, per_system: bool = True):
        """b: concatenated rhs (numpy, or a CUDA tensor with x also a CUDA tensor)."""
        if x is None:
            x = np.empty(len(b))
        pb, mb = ptr_and_mem(b)
        px, mx = ptr_and_mem(x)
        if mb != mx:
            raise ValueError("b and x must live in the same memory")
        stats = np.zeros(self.n_systems, dtype=[("iterations", np.int32), ("reliable_updates", np.int32),
                                                ("converged", np.int32), ("status", np.int32),
                                                ("true_residual", np.float64), ("b_norm", np.float64)])
        check(self.L.simall_batch_solve(self.handle, pb, px, mb, stats.ctypes.data if per_system else None,
                                        C.byref(self.total)), self.ctx.handle)
        return x, stats

    def close(self):
        if getattr(self, "handle", None) and getattr(self.ctx, "handle", None):
            self.L.simall_batch_destroy(self.handle)
        self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def autotune_cache_lookup(path: str, key: str):
    """(block_threads, ctas_per_sm, rows_per_pass, cluster_rows, cluster_ctas, clusters) stored under key, or None."""
    L = _lib.load()
    v = (C.c_int * 6)()
    st = L.simall_autotune_cache_lookup(path.encode(), key.encode(), v)
    return tuple(v) if st == 0 else None


def autotune_cache_store(path: str, key: str, values, ms: float = 0.0) -> int:
    L = _lib.load()
    v = (C.c_int * 6)(*[int(t) for t in values])
    return int(L.simall_autotune_cache_store(path.encode(), key.encode(), v, float(ms)))
