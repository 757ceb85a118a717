"""GMRES(m), BiCGSTAB and TFQMR on the device (GMRESmSolver / BiCGSTABSolver /
TfqmrSolver, src/solver/LinearSolvers.cpp:268-405, :497-609) with Jacobi,
ILU(0) and SSOR, against the oracle's restatement and the reference's own
results (tests/golden/momentum_7x6x5_rcm_bdf2.npz): the same iteration count
(within one, the FP64 dot products are summed in another order), a solution
within the solve's own accuracy, and the reference's return values on the
edge cases (b = 0, maxIterations reached mid-cycle, maxIterations = 0).

The reference's TFQMR often breaks down or diverges (Jacobi on the
convection-diffusion matrix, most momentum systems); the parity cases below
are the ones where its own run converges."""
import os

import numpy as np
import pytest

from helpers import rel

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
MOM_BCS = [(1, 4, (0.7, -0.2, 0.1)), (2, 7), (3, 1), (4, 2, (1.0, 0.3, 0.0)), (5, 9), (6, 3)]


def _conv_diff(n, pe=5.0):
    """Upwind convection-diffusion, tests/unit/solver/test_tfqmr_solver.cpp:43-62."""
    rp, ci, v = [0], [], []
    for i in range(n):
        if i > 0:
            ci.append(i - 1)
            v.append(-1.0 - pe)
        ci.append(i)
        v.append(2.0 + pe)
        if i < n - 1:
            ci.append(i + 1)
            v.append(-1.0)
        rp.append(len(ci))
    return np.array(rp, np.int32), np.array(ci, np.int32), np.array(v)


def _momentum_system(oracle, dims, seed=5, mu=0.01, urf=0.7):
    from simall_gb300 import workloads as W

    m = oracle.cartesian_mesh(*dims, node_shift=W.interior_node_shift(*dims, amp=0.2, seed=seed))
    oracle.rcm(m)
    rp, ci = oracle.build_sparsity(m)
    rng = np.random.default_rng(seed)
    U = rng.standard_normal((3, m.nC))
    phi = oracle.face_fluxes(m, MOM_BCS, 1.0, U)
    gp = oracle.lsq_gradient(m, rng.standard_normal(m.nC))
    v, rhs, _ = oracle.assemble_momentum(m, rp, ci, MOM_BCS, (1.0, mu, urf, 0.0), 0, phi, gp[0], U[0])
    return rp, ci, v, rhs


def _solver(sg, ctx, kind, pc, tol, maxit, restart=30):
    cfg = sg.LinearSolverConfig(kind=kind, preconditioner=pc, tolerance=tol, maxIterations=maxit, restart=restart)
    return sg.make_linear_solver(cfg, ctx=ctx)


def _oracle_solve(oracle, kind, rp, ci, v, b, pc, tol, maxit, restart):
    if kind == 0:
        return oracle.gmres(rp, ci, v, b, pc, tol, maxit, restart)
    if kind == 3:
        return oracle.tfqmr(rp, ci, v, b, pc, tol, maxit)
    return oracle.bicgstab(rp, ci, v, b, pc, tol, maxit)


def _device_solve(sg, ctx, kind, rp, ci, v, b, pc, tol, maxit, restart):
    s = _solver(sg, ctx, kind, pc, tol, maxit, restart)
    x = np.zeros(len(b))
    it = s.solve(sg.CSRMatrix(rp, ci, v), b, x)
    st = s.stats
    s.close()
    return x, it, st


@pytest.mark.parametrize("kind", [0, 1])
@pytest.mark.parametrize("pc", [0, 1, 2])
@pytest.mark.parametrize("case", ["conv_diff", "momentum_small", "momentum_64"])
def test_matches_oracle(sg, ctx, oracle, kind, pc, case):
    if case == "conv_diff":
        rp, ci, v = _conv_diff(40)
        b, tol, maxit, restart = np.ones(40), 1e-8, 500, 30
    elif case == "momentum_small":
        rp, ci, v, b = _momentum_system(oracle, (9, 8, 3))
        tol, maxit, restart = 1e-10, 200, 5
    else:
        rp, ci, v, b = _momentum_system(oracle, (64, 64, 64), mu=0.002)
        tol, maxit, restart = 1e-8, 300, 30
    ox, oit, olast = _oracle_solve(oracle, kind, rp, ci, v, b, pc, tol, maxit, restart)
    x, it, st = _device_solve(sg, ctx, kind, rp, ci, v, b, pc, tol, maxit, restart)
    assert abs(it - oit) <= 1, (it, oit)
    assert st.converged and st.final_residual < tol
    # GMRES stops on the preconditioned residual and BiCGSTAB on its recursive
    # one, so the true residual may exceed tol -- by as much as the
    # reference's own (BiCGSTAB + Jacobi on the convection-diffusion matrix:
    # 3.8e-4 at tol 1e-8)
    otrue = np.linalg.norm(b - oracle.spmv(rp, ci, v, ox)) / np.linalg.norm(b)
    assert st.true_residual <= 2.0 * otrue + 10 * tol, (st.true_residual, otrue)
    assert rel(x, ox) <= 1e4 * max(tol, otrue)


def test_reference_results_fixture(sg, ctx):
    """The reference's GMRES(5)+ILU(0) and BiCGSTAB+Jacobi on its own BDF2
    momentum system."""
    g = np.load(os.path.join(GOLD, "momentum_7x6x5_rcm_bdf2.npz"))
    args = (g["rowPtr"], g["colIdx"], g["values"][0], g["rhs"][0])
    x, it, st = _device_solve(sg, ctx, 0, *args, 1, 1e-10, 200, 5)
    assert abs(it - int(g["it_gmres"])) <= 1 and rel(x, g["x_gmres"]) <= 1e-8
    x, it, st = _device_solve(sg, ctx, 1, *args, 0, 1e-10, 200, 30)
    assert abs(it - int(g["it_bicgstab"])) <= 1 and rel(x, g["x_bicgstab"]) <= 1e-8


@pytest.mark.parametrize("case,pc,tol", [("conv_diff", 1, 1e-8), ("momentum_small", 1, 1e-6),
                                         ("momentum_small", 1, 1e-8), ("momentum_small", 1, 1e-10),
                                         ("momentum_small", 2, 1e-6), ("momentum_small", 2, 1e-8),
                                         ("momentum_16", 1, 1e-6)])
def test_tfqmr_matches_oracle(sg, ctx, oracle, case, pc, tol):
    """TFQMR with ILU(0) or SSOR where the reference's run converges: its
    count within one, the true residual below tol (TFQMR stops on it), x
    within the solve's accuracy."""
    if case == "conv_diff":
        rp, ci, v = _conv_diff(40)
        b = np.ones(40)
    elif case == "momentum_small":
        rp, ci, v, b = _momentum_system(oracle, (9, 8, 3))
    else:
        rp, ci, v, b = _momentum_system(oracle, (16, 16, 16), mu=0.002)
    ox, oit, olast = oracle.tfqmr(rp, ci, v, b, pc, tol, 300)
    assert oit < 300 and olast < tol  # the reference converges here
    x, it, st = _device_solve(sg, ctx, 3, rp, ci, v, b, pc, tol, 300, 30)
    assert abs(it - oit) <= 1, (it, oit)
    assert st.converged and st.final_residual < tol and st.true_residual < tol
    assert rel(x, ox) <= 1e4 * tol


@pytest.mark.parametrize("kind", [0, 1, 3])
def test_edge_cases(sg, ctx, oracle, kind):
    rp, ci, v = _conv_diff(40)
    # b = 0: no iteration, x = 0
    x, it, st = _device_solve(sg, ctx, kind, rp, ci, v, np.zeros(40), 0, 1e-8, 100, 30)
    assert it == 0 and not np.any(x)
    # maxIterations reached (GMRES: mid-cycle, restart 3): the reference's count and x
    # (TFQMR: its residual bound is still far above tol after seven steps)
    b = np.linspace(1.0, 2.0, 40)
    ox, oit, olast = _oracle_solve(oracle, kind, rp, ci, v, b, 0, 1e-14, 7, 3)
    x, it, st = _device_solve(sg, ctx, kind, rp, ci, v, b, 0, 1e-14, 7, 3)
    assert it == oit == 7 and not st.converged
    # seven unconverged steps (BiCGSTAB's residual grows here) amplify the
    # rounding differences of the dot products
    assert rel(x, ox) <= 1e-6
    assert abs(st.final_residual - olast) <= 1e-6 * olast
    # maxIterations = 0
    x, it, st = _device_solve(sg, ctx, kind, rp, ci, v, b, 0, 1e-8, 0, 3)
    assert it == 0 and not np.any(x)


def test_ilu_gmres_one_step_exact(sg, ctx, oracle):
    """ILU(0) of a tridiagonal matrix is exact: GMRES stops inside its first
    Arnoldi step and returns 0, as the reference's loop does."""
    rp, ci, v = _conv_diff(40)
    b = np.ones(40)
    ox, oit, _ = oracle.gmres(rp, ci, v, b, 1, 1e-8, 500, 30)
    x, it, st = _device_solve(sg, ctx, 0, rp, ci, v, b, 1, 1e-8, 500, 30)
    assert oit == 0 and it == 0 and rel(x, ox) <= 1e-12


def test_tfqmr_make_linear_solver(sg, ctx, oracle):
    """make_linear_solver hands TFQMR to the device: the reference's ILU(0)
    known answer (tests/unit/solver/test_tfqmr_solver.cpp:91-111)."""
    rp, ci, v = _conv_diff(40)
    cfg = sg.LinearSolverConfig(kind=sg.LinearSolverKind.TFQMR, preconditioner=sg.PreconditionerKind.ILU,
                                tolerance=1e-8, maxIterations=500)
    s = sg.make_linear_solver(cfg, ctx=ctx)
    x = np.zeros(40)
    s.solve(sg.CSRMatrix(rp, ci, v), np.ones(40), x)
    s.close()
    assert np.linalg.norm(oracle.spmv(rp, ci, v, x) - 1.0) < 1e-4
