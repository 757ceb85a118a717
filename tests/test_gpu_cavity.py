"""The 128x128 lid-driven cavity at full size (Re 100, SIMPLE with urfP 0.3
and urfU 0.7, 200 outer iterations): the reference's first and last pressure
systems, assembled on the device from the recorded aP and phi and solved
there.  Fixture: tests/golden/cavity_simple_128.npz (the reference's own
SIMPLE loop, tests/golden/make_golden.py)."""
import hashlib
import os

import numpy as np
import pytest

from helpers import rel

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _digest(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


@pytest.fixture(scope="module")
def cavity():
    return np.load(os.path.join(GOLD, "cavity_simple_128.npz"))


def _system(sg, ctx, c):
    from simall_gb300 import workloads as W

    N = int(c["N"])
    m = sg.cartesian(N, N, 1, 1.0, 1.0, 1.0 / N)
    return sg.PressureSystem(m, W.CAVITY, ctx=ctx)


def test_cavity_128_assembly_is_the_reference_bytes(sg, ctx, cavity):
    ps = _system(sg, ctx, cavity)
    rp, ci = ps.pattern()
    assert _digest(rp) + _digest(ci) == str(cavity["pattern_sha256"])
    for k in range(len(cavity["recorded"])):
        ps.assemble(1.0, cavity["aP"][k], cavity["phi"][k])
        v, rhs = ps.download()
        assert _digest(v) == str(cavity["values_sha256"][k])
        assert _digest(rhs) == str(cavity["rhs_sha256"][k])
    ps.close()


def _cfg(sg, tol, maxit=1000):
    return sg.LinearSolverConfig(kind=sg.LinearSolverKind.CG, preconditioner=sg.PreconditionerKind.Jacobi,
                                 tolerance=tol, maxIterations=maxit)


@pytest.mark.parametrize("interval", [0, 8])
def test_cavity_128_pressure_solves(sg, ctx, cavity, interval):
    """FP64 Jacobi-PCG: the reference's iteration count and p' within 1e-10.
    Mixed precision within the reference's own maxIterations (1000): FP64 true
    residual below 1e-8."""
    ps = _system(sg, ctx, cavity)
    s64 = sg.GpuCGSolver(_cfg(sg, 1e-8), ctx=ctx, check_interval=interval)
    smx = sg.GpuCGSolver(_cfg(sg, 1e-8), precision=sg.Precision.MIXED, ctx=ctx, check_interval=interval)
    for k, it in enumerate(cavity["recorded"]):
        ps.assemble(1.0, cavity["aP"][k], cavity["phi"][k])
        x = ps.solve(s64)
        assert abs(int(s64.stats.iterations) - int(cavity["iters"][it])) <= 1
        assert rel(x, cavity["x"][k]) <= 1e-10
        xm = ps.solve(smx)
        assert smx.stats.converged and smx.stats.true_residual < 1e-8
        assert smx.stats.iterations <= 1.10 * int(cavity["iters"][it])  # 783 vs 737, 777 vs 775
        # At an equal residual the FP32 inner iteration leaves more error along
        # the pinned system's slowest mode than FP64 CG does: ~1e-6 against
        # ~2.7e-9 for the reference's p'.
        assert rel(xm, cavity["x"][k]) <= 5e-6
    ps.close()


def test_cavity_128_mixed_error_at_tighter_tolerance(sg, ctx, cavity):
    """Solved to 1e-10, the mixed solution is within 1e-9 of an FP64 solve to
    1e-12 (the FP64 oracle error the mixed solver reaches)."""
    ps = _system(sg, ctx, cavity)
    ps.assemble(1.0, cavity["aP"][1], cavity["phi"][1])
    xt = ps.solve(sg.GpuCGSolver(_cfg(sg, 1e-12, 5000), ctx=ctx))
    smx = sg.GpuCGSolver(_cfg(sg, 1e-10, 5000), precision=sg.Precision.MIXED, ctx=ctx)
    xm = ps.solve(smx)
    assert smx.stats.converged and smx.stats.true_residual < 1e-10
    assert rel(xm, xt) <= 1e-9
    ps.close()
