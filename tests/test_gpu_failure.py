"""Failure detection without a GPU fault: a device-side wait that runs out is
reported to the host, and the context stays usable afterwards."""
import ctypes as C

import numpy as np
import pytest

from helpers import oracle_system

pytestmark = pytest.mark.gpu


def test_bounded_wait_times_out_and_context_survives(sg, ctx, oracle):
    L = sg.load()
    timed_out = C.c_int(-1)
    secs = C.c_double(0.0)
    assert L.simall_diagnose_bounded_wait(ctx.handle, C.byref(timed_out), C.byref(secs)) == 0
    assert timed_out.value == 1
    assert 0.0 < secs.value < 10.0
    # the same context solves afterwards
    m, rp, ci, v, rhs, aP, phi = oracle_system(oracle, 6)
    s = sg.GpuCGSolver(sg.LinearSolverConfig(kind=sg.LinearSolverKind.CG, preconditioner=sg.PreconditionerKind.ILU,
                                             tolerance=1e-10, maxIterations=500), ctx=ctx)
    x = np.zeros(len(rhs))
    s.solve(sg.CSRMatrix(rp, ci, v), rhs, x)
    assert s.stats.converged
