"""SSOR on the device (SsorPreconditioner with make_preconditioner's w = 1,
src/solver/LinearSolvers.cpp:163-231, :247-248) and the solver's
preconditioner apply (IPreconditioner::apply) for all three FP64
preconditioners, against the oracle: the sweeps bit-identical on the
single-CTA path (up to 24,576 rows) and on the free-running sweep kernels
(larger systems), and CG + SSOR against the oracle's CG and the reference's
known answers (tests/unit/solver/test_ssor_preconditioner.cpp)."""
import numpy as np
import pytest

from helpers import bits_equal, oracle_system, rel, tridiag

pytestmark = pytest.mark.gpu


def _solver(sg, ctx, pc, tol=1e-8, maxit=1000):
    cfg = sg.LinearSolverConfig(kind=sg.LinearSolverKind.CG, preconditioner=pc, tolerance=tol, maxIterations=maxit)
    return sg.GpuCGSolver(cfg, ctx=ctx)


def _oracle_apply(oracle, pc, rp, ci, v, r):
    if pc == 2:
        return oracle.ssor_apply(rp, ci, v, r)
    if pc == 1:
        lu, dp = oracle.ilu0_setup(rp, ci, v)
        return oracle.ilu0_apply(rp, ci, lu, dp, r)
    diag = np.array([v[rp[i] + np.flatnonzero(ci[rp[i]:rp[i + 1]] == i)[0]] for i in range(len(rp) - 1)])
    inv = np.where(diag != 0.0, 1.0 / np.where(diag != 0.0, diag, 1.0), 1.0)
    return inv * r


@pytest.mark.parametrize("pc", [0, 1, 2])
@pytest.mark.parametrize("dims", [(12, 11, 10), (34, 33, 32)])
def test_precond_apply_bit_exact(sg, ctx, oracle, pc, dims):
    """1,320 rows take the single-CTA sweeps, 35,904 the free-running ones."""
    m, rp, ci, v, rhs, aP, phi = oracle_system(oracle, 0, seed=11, dims=dims)
    s = _solver(sg, ctx, pc)
    s.set_matrix(rp, ci, v)
    for seed in (1, 2):
        r = np.random.default_rng(seed).standard_normal(len(rp) - 1)
        z = np.empty_like(r)
        s.precond_apply(r, z)
        assert bits_equal(z, _oracle_apply(oracle, pc, rp, ci, v, r)), (pc, dims, seed)
    s.close()


def test_ssor_identity_known_answer(sg, ctx):
    """tests/unit/solver/test_ssor_preconditioner.cpp:40-62: SSOR(1) of the
    5x5 identity returns r."""
    rp = np.arange(6, dtype=np.int32)
    ci = np.arange(5, dtype=np.int32)
    s = _solver(sg, ctx, sg.PreconditionerKind.SSOR)
    s.set_matrix(rp, ci, np.ones(5))
    r = np.arange(1.0, 6.0)
    z = np.empty(5)
    s.precond_apply(r, z)
    s.close()
    assert z.tolist() == r.tolist()


def test_cg_ssor_1d_laplacian_known_answer(sg, ctx):
    """tests/unit/solver/test_ssor_preconditioner.cpp:65-88: CG + SSOR on the
    50-point 1-D Laplacian, b = 1, tol 1e-10: |Ax - b| < 1e-7, iters > 0."""
    rp, ci, va = tridiag(50, -1.0, 2.0, -1.0)
    s = _solver(sg, ctx, sg.PreconditionerKind.SSOR, tol=1e-10, maxit=200)
    x = np.zeros(50)
    it = s.solve(sg.CSRMatrix(rp, ci, va), np.ones(50), x)
    s.close()
    ax = np.array([sum(va[k] * x[ci[k]] for k in range(rp[i], rp[i + 1])) for i in range(50)])
    assert it > 0 and np.linalg.norm(ax - 1.0) < 1e-7


@pytest.mark.parametrize("dims", [(12, 11, 10), (34, 33, 32)])
def test_cg_ssor_matches_oracle(sg, ctx, oracle, dims):
    """FP64 CG + SSOR on a distorted, RCM-renumbered pressure system: the
    oracle's iteration count (within one) and x within 1e-10 relative."""
    m, rp, ci, v, rhs, aP, phi = oracle_system(oracle, 0, seed=5, dims=dims)
    ox, oit, olast = oracle.cg(rp, ci, v, rhs, 2, 1e-8, 2000)
    s = _solver(sg, ctx, sg.PreconditionerKind.SSOR, maxit=2000)
    x = np.zeros(len(rhs))
    it = s.solve(sg.CSRMatrix(rp, ci, v), rhs, x)
    st = s.stats
    s.close()
    assert abs(it - oit) <= 1, (it, oit)
    assert st.converged and st.true_residual < 1e-8
    assert rel(x, ox) <= 1e-10


@pytest.mark.parametrize("pc", [1, 2, 3])
def test_zero_diagonals_and_tiny_systems(sg, ctx, oracle, pc):
    """Rows whose diagonal entry is an explicit 0 (SSOR: invD = 1 and
    a_ii y_i = 0; ILU(0): the sweep keeps the sum; AMG: Gauss-Seidel keeps
    the old value), and systems of 1 and 2 rows: the device apply is the
    oracle's bit for bit."""
    rp, ci, va = tridiag(40, -1.0, 2.5, -1.2)
    va = va.copy()
    for i in (0, 7, 23):
        va[rp[i] + (0 if i == 0 else 1)] = 0.0  # the diagonal of rows 0, 7, 23
    cases = [(rp, ci, va), (np.array([0, 1], np.int32), np.array([0], np.int32), np.array([3.0])),
             (np.array([0, 2, 4], np.int32), np.array([0, 1, 0, 1], np.int32), np.array([2.0, -1.0, -0.5, 4.0]))]
    for rp_, ci_, va_ in cases:
        n = len(rp_) - 1
        r = np.linspace(-1.0, 1.5, n)
        s = _solver(sg, ctx, pc)
        s.set_matrix(rp_, ci_, va_)
        z = np.empty(n)
        s.precond_apply(r, z)
        s.close()
        if pc == 3:
            oz = oracle.amg_apply(rp_, ci_, va_, r)[0]
        elif pc == 1:
            lu, dp = oracle.ilu0_setup(rp_, ci_, va_)
            oz = oracle.ilu0_apply(rp_, ci_, lu, dp, r)
        else:
            oz = oracle.ssor_apply(rp_, ci_, va_, r)
        assert bits_equal(z, oz), (pc, n)
