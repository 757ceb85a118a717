"""The AMG preconditioner on the device (AMGPreconditioner,
src/solver/AMGPreconditioner.cpp, make_preconditioner's defaults) against the
oracle's restatement: the same hierarchy (levels and their sizes), the V-cycle
bit-identical (its Gauss-Seidel sweeps run on the free-running level schedule
of every level, the coarsest level by the dense LU), and CG / BiCGSTAB /
GMRES with AMG within one iteration of the oracle's count."""
import numpy as np
import pytest

from helpers import bits_equal, oracle_system, rel, tridiag

pytestmark = pytest.mark.gpu

AMG = 3


def _solver(sg, ctx, kind=2, tol=1e-8, maxit=1000, restart=30):
    cfg = sg.LinearSolverConfig(kind=kind, preconditioner=AMG, tolerance=tol, maxIterations=maxit, restart=restart)
    return sg.make_linear_solver(cfg, ctx=ctx)


SYSTEMS = {
    # name: dims of a distorted, RCM-renumbered pressure system
    "box_6x5x4": (6, 5, 4),
    "box_12x11x10": (12, 11, 10),
    "plate_20x20": (20, 20, 1),
    "box_16": (16, 16, 16),
    "cavity_128": (128, 128, 1),
    "box_32": (32, 32, 32),
}


@pytest.mark.parametrize("name", sorted(SYSTEMS))
def test_amg_apply_bit_exact(sg, ctx, oracle, name):
    m, rp, ci, v, rhs, aP, phi = oracle_system(oracle, 0, seed=3, dims=SYSTEMS[name])
    s = _solver(sg, ctx)
    s.set_matrix(rp, ci, v)
    r = np.random.default_rng(1).standard_normal(len(rp) - 1)
    oz, levels, coarse = oracle.amg_apply(rp, ci, v, r)
    assert s.amg_levels() == [n for n, _ in levels]
    for rep in range(2):  # the second apply reuses the sweep marks of the first
        z = np.empty_like(r)
        s.precond_apply(r, z)
        assert bits_equal(z, oz), (name, rep)
    s.close()


def test_amg_single_level_and_1d(sg, ctx, oracle):
    """n <= 32: no coarsening, the dense LU solves the fine system; the
    50-point 1-D Laplacian of tests/unit/solver/test_ssor_preconditioner.cpp."""
    for n in (20, 50):
        rp, ci, va = tridiag(n, -1.0, 2.0, -1.0)
        s = _solver(sg, ctx)
        s.set_matrix(rp, ci, va)
        r = np.linspace(-1.0, 2.0, n)
        z = np.empty(n)
        s.precond_apply(r, z)
        oz, levels, _ = oracle.amg_apply(rp, ci, va, r)
        assert bits_equal(z, oz) and s.amg_levels() == [k for k, _ in levels]
        s.close()


@pytest.mark.parametrize("name", ["box_12x11x10", "cavity_128", "box_32"])
def test_cg_amg_matches_oracle(sg, ctx, oracle, name):
    m, rp, ci, v, rhs, aP, phi = oracle_system(oracle, 0, seed=5, dims=SYSTEMS[name])
    ox, oit, olast = oracle.cg(rp, ci, v, rhs, AMG, 1e-8, 500)
    s = _solver(sg, ctx, maxit=500)
    x = np.zeros(len(rhs))
    it = s.solve(sg.CSRMatrix(rp, ci, v), rhs, x)
    st = s.stats
    s.close()
    assert abs(it - oit) <= 1, (it, oit)
    assert st.converged and st.true_residual < 1e-8
    assert rel(x, ox) <= 1e-10


@pytest.mark.parametrize("kind", [0, 1])
def test_nonsymmetric_krylov_amg(sg, ctx, oracle, kind):
    """GMRES(30) and BiCGSTAB with AMG on a momentum system."""
    from test_gpu_krylov import _momentum_system

    rp, ci, v, b = _momentum_system(oracle, (16, 16, 16), mu=0.002)
    tol = 1e-8
    ox, oit, olast = (oracle.gmres(rp, ci, v, b, AMG, tol, 300, 30) if kind == 0
                      else oracle.bicgstab(rp, ci, v, b, AMG, tol, 300))
    assert oit < 300
    s = _solver(sg, ctx, kind=kind, tol=tol, maxit=300)
    x = np.zeros(len(b))
    it = s.solve(sg.CSRMatrix(rp, ci, v), b, x)
    st = s.stats
    s.close()
    assert abs(it - oit) <= 1, (it, oit)
    assert st.converged
    otrue = np.linalg.norm(b - oracle.spmv(rp, ci, v, ox)) / np.linalg.norm(b)
    assert rel(x, ox) <= 1e4 * max(tol, otrue)


def test_amg_new_values_rebuild_the_hierarchy(sg, ctx, oracle):
    """update_values sets the hierarchy up again (the reference sets its
    preconditioner up on every solve)."""
    m, rp, ci, v, rhs, aP, phi = oracle_system(oracle, 0, seed=9, dims=(12, 11, 10))
    s = _solver(sg, ctx)
    s.set_matrix(rp, ci, v)
    v2 = v * np.random.default_rng(2).uniform(0.5, 2.0, len(v))
    s.update_values(v2)
    r = np.random.default_rng(4).standard_normal(len(rp) - 1)
    z = np.empty_like(r)
    s.precond_apply(r, z)
    assert bits_equal(z, oracle.amg_apply(rp, ci, v2, r)[0])
    s.close()
