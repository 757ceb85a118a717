"""Batched solves: every system of a batch reaches the FP64 true-residual
tolerance and matches the oracle's FP64 CG solution of that system; the
benchmark's own batch of 512 cavity systems against the reference's FP64
CGSolver::solve of each system (tests/golden/batched_512_cg.npz)."""
import os

import numpy as np
import pytest

from helpers import digest, oracle_system

pytestmark = pytest.mark.gpu


def _cfg(sg, tol=1e-8, maxit=5000):
    return sg.LinearSolverConfig(kind=sg.LinearSolverKind.CG, preconditioner=sg.PreconditionerKind.Jacobi,
                                 tolerance=tol, maxIterations=maxit)


def _check(oracle, systems, rhs, x, stats, tol):
    for k, ((rp, ci, va), b) in enumerate(zip(systems, rhs)):
        xs = x[k]
        r = b - oracle.spmv(rp, ci, va, xs)
        true_rel = np.linalg.norm(r) / max(np.linalg.norm(b), 1e-30)
        assert true_rel < tol, (k, true_rel)
        assert stats["converged"][k] == 1
        assert abs(stats["true_residual"][k] - true_rel) <= 1e-3 * true_rel + 1e-15
        xo, _, _ = oracle.cg(rp, ci, va, b, 0, 1e-13, 20000)
        # both solutions satisfy the same system to their tolerances
        assert np.linalg.norm(xs - xo) <= 1e-4 * max(np.linalg.norm(xo), 1e-30)


def test_batched_cavity_systems(sg, ctx, oracle):
    from simall_gb300 import workloads as W

    systems, rhs, sides = W.batched_cavity_systems(count=24, lo=4, hi=40, seed=3, ctx=ctx)
    B = sg.BatchedSolver(_cfg(sg), ctx=ctx)
    rows = B.set_systems(systems)
    b = np.concatenate(rhs)
    x, stats = B.solve(b)
    parts = [x[rows[i]:rows[i + 1]] for i in range(len(systems))]
    _check(oracle, systems, rhs, parts, stats, 1e-8)
    assert B.total.converged == len(systems) and B.total.block_threads in (256, 512, 1024)
    # a second solve reuses the tuned shape and the captured graph
    x2, stats2 = B.solve(b)
    assert np.array_equal(x, x2)


@pytest.mark.parametrize("shape", [(256, 4), (512, 2), (1024, 1)])
def test_batched_mixed_storage_and_shapes(sg, ctx, oracle, shape):
    """Structured (diagonal storage) and RCM-renumbered distorted systems
    (CSR storage) in one batch, with each fixed launch shape."""
    systems, rhs = [], []
    for k, n in enumerate((5, 7, 9)):
        m, rp, ci, v, b, aP, phi = oracle_system(oracle, n, seed=20 + k)
        systems.append((rp, ci, v))
        rhs.append(b)
    from simall_gb300 import workloads as W
    for side in (6, 13, 30):
        rp, ci, v = W.cavity_pressure_matrix(side, ctx)
        systems.append((rp, ci, v))
        rhs.append(W.batched_rhs(side * side, np.random.default_rng(side)))
    B = sg.BatchedSolver(_cfg(sg), ctx=ctx)
    rows = B.set_systems(systems)
    B.launch_shape(*shape)
    x, stats = B.solve(np.concatenate(rhs))
    parts = [x[rows[i]:rows[i + 1]] for i in range(len(systems))]
    _check(oracle, systems, rhs, parts, stats, 1e-8)
    assert (B.total.block_threads, B.total.ctas_per_sm) == shape


def test_batched_device_memory_and_zero_rhs(sg, ctx, oracle):
    torch = pytest.importorskip("torch")
    from simall_gb300 import workloads as W
    systems = [W.cavity_pressure_matrix(s, ctx) for s in (8, 16)]
    B = sg.BatchedSolver(_cfg(sg), ctx=ctx)
    rows = B.set_systems(systems)
    b = np.concatenate([W.batched_rhs(64, np.random.default_rng(1)), np.zeros(256)])
    tb = torch.from_numpy(b).cuda()
    tx = torch.empty_like(tb)
    _, stats = B.solve(tb, tx)
    x = tx.cpu().numpy()
    assert stats["converged"].all() and stats["iterations"][1] == 0 and not np.any(x[rows[1]:])


def test_batched_rejects_bad_system(sg, ctx):
    rp = np.array([0, 2, 4], np.int32)
    ci = np.array([0, 1, 0, 1], np.int32)
    va = np.array([1.0, 2.0, 2.0, -1.0])  # non-positive diagonal
    B = sg.BatchedSolver(_cfg(sg), ctx=ctx)
    with pytest.raises(sg.SimallError) as e:
        B.set_systems([(rp, ci, va)])
    assert e.value.status == 7


def test_benchmark_batch_against_the_reference(sg, ctx):
    """The 512 systems of the benchmark (sides log-uniform in [32, 256], seed
    42): the device assembly gives each system's reference matrix (SHA-256);
    the batched mixed solve brings every system's FP64 true residual, recomputed
    on the host, below 1e-8 and lands within the accuracy that residual allows
    of the reference's solution; the FP64 drop-in solves each system within one
    iteration of the reference's count with x within 1e-10 of the reference's."""
    import scipy.sparse as sps
    from simall_gb300 import workloads as W

    fx = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "batched_512_cg.npz"))
    count, seed = int(fx["count"]), int(fx["seed"])
    systems, rhs, sides = W.batched_cavity_systems(count=count, seed=seed, ctx=ctx)
    assert np.array_equal(sides, fx["sides"])
    assert [digest(v) for _, _, v in systems] == [str(d) for d in fx["values_sha256"]]
    cfg = _cfg(sg, tol=float(fx["tol"]), maxit=50000)

    def summary_err(k, xs):
        n = len(xs)
        w = np.random.default_rng(seed + 13 + k).standard_normal(n)
        xn = float(fx["x_norm"][k])
        smp = xs[::n // fx["x_sample"].shape[1]][:fx["x_sample"].shape[1]]
        return max(abs(np.linalg.norm(xs) - xn) / xn, abs(float(xs @ w) - float(fx["x_dot_w"][k])) / xn / 8.0,
                   np.linalg.norm(smp - fx["x_sample"][k]) / np.linalg.norm(fx["x_sample"][k]))

    B = sg.BatchedSolver(cfg, ctx=ctx)
    rows = B.set_systems(systems)
    x, stats = B.solve(np.concatenate(rhs))
    worst = 0.0
    for k, ((rp, ci, va), b) in enumerate(zip(systems, rhs)):
        xs = x[rows[k]:rows[k + 1]]
        A = sps.csr_matrix((va, ci, rp))
        assert np.linalg.norm(b - A @ xs) / np.linalg.norm(b) < 1e-8, k
        worst = max(worst, summary_err(k, xs))
    assert stats["converged"].all()
    # the reference stops each system at a 1e-8 residual too; pinned Neumann
    # systems with cond up to ~1e6 leave the two solutions up to ~1e-5 apart
    assert worst < 1e-4, worst
    B.close()
    s = sg.GpuCGSolver(cfg, precision=sg.Precision.FP64, ctx=ctx)
    for k, ((rp, ci, va), b) in enumerate(zip(systems, rhs)):
        s.set_matrix(rp, ci, va)
        xs = np.empty_like(b)
        it = s.solve_into(b, xs)
        assert abs(it - int(fx["iters"][k])) <= 1, (k, it, int(fx["iters"][k]))
        assert summary_err(k, xs) <= 1e-10, k
    s.close()


def test_autotuner_cache_across_batch_objects(sg, ctx, tmp_path):
    """The first batch object times the candidate launch shapes and stores the
    winner in the cache file; a second object with the same systems reads it
    instead of timing (autotune_source 2) and solves to the same bits."""
    from simall_gb300 import workloads as W
    from simall_gb300.batch import autotune_cache_lookup

    systems, rhs, sides = W.batched_cavity_systems(count=12, lo=8, hi=48, seed=5, ctx=ctx)
    b = np.concatenate(rhs)
    cache = str(tmp_path / "autotune.json")
    B1 = sg.BatchedSolver(_cfg(sg), ctx=ctx)
    B1.autotune_cache(cache)
    B1.set_systems(systems)
    x1, _ = B1.solve(b)
    assert B1.total.autotune_source == 1
    shape = (B1.total.block_threads, B1.total.ctas_per_sm, B1.total.rows_per_pass, B1.total.cluster_rows,
             B1.total.cluster_ctas, B1.total.clusters)
    doc = open(cache).read()
    assert "batch-fused-v5|" in doc and f'"block_threads": {shape[0]}' in doc
    B2 = sg.BatchedSolver(_cfg(sg), ctx=ctx)
    B2.autotune_cache(cache)
    B2.set_systems(systems)
    x2, _ = B2.solve(b)
    assert B2.total.autotune_source == 2
    assert (B2.total.block_threads, B2.total.ctas_per_sm, B2.total.rows_per_pass, B2.total.cluster_rows,
            B2.total.cluster_ctas, B2.total.clusters) == shape
    assert np.array_equal(x1, x2)
    # a fixed shape is not the autotuner's
    B2.launch_shape(512, 2)
    B2.solve(b)
    assert B2.total.autotune_source == 0 and B2.total.block_threads == 512
    B1.close()
    B2.close()


@pytest.mark.parametrize("ctas,clusters", [(4, 1), (8, 2), (16, 3)])
def test_cluster_route(sg, ctx, oracle, ctas, clusters):
    """The largest systems of a batch on one thread-block cluster each, the
    rest on the one-CTA queue, concurrently: every system reaches the
    tolerance and matches the oracle's solution; the same batch without
    clusters gives solutions equally close to the oracle's."""
    from simall_gb300 import workloads as W

    sides = [120, 96, 70, 33, 20, 9, 64]
    systems = [W.cavity_pressure_matrix(sd, ctx) for sd in sides]
    rng = np.random.default_rng(17)
    rhs = []
    for rp, _, _ in systems:
        r = rng.standard_normal(len(rp) - 1)
        rhs.append(r - r.mean())
    B = sg.BatchedSolver(_cfg(sg, tol=1e-9), ctx=ctx)
    rows = B.set_systems(systems)
    B.cluster_route(4096, ctas, clusters)
    x, stats = B.solve(np.concatenate(rhs))
    assert B.total.cluster_systems == sum(1 for sd in sides if sd * sd >= 4096 and sd * sd <= ctas * 8192)
    assert B.total.cluster_rows == 4096 and B.total.cluster_ctas == ctas and B.total.clusters == clusters
    parts = [x[rows[i]:rows[i + 1]] for i in range(len(systems))]
    _check(oracle, systems, rhs, parts, stats, 1e-9)
    B.close()


def test_step_counts_do_not_depend_on_engine_or_route(sg, ctx):
    """The one-CTA queue and the cluster engine advance the same mixed CG
    with float-float sums: every system takes the same number of steps
    whether it runs on one CTA or on a cluster of 4, 8 or 16 CTAs, and the
    solutions agree to rounding."""
    from simall_gb300 import workloads as W

    sides = [120, 96, 70, 64, 33]
    systems = [W.cavity_pressure_matrix(sd, ctx) for sd in sides]
    rng = np.random.default_rng(23)
    rhs = []
    for rp, _, _ in systems:
        r = rng.standard_normal(len(rp) - 1)
        rhs.append(r - r.mean())
    b = np.concatenate(rhs)
    counts, xs, on_clusters = [], [], []
    for route in [(0, 8, 1), (4096, 4, 1), (4096, 8, 2), (4096, 16, 3)]:
        B = sg.BatchedSolver(_cfg(sg), ctx=ctx)
        B.set_systems(systems)
        B.launch_shape(1024, 1)
        B.cluster_route(*route)
        x, stats = B.solve(b)
        assert B.total.converged == len(sides)
        counts.append(stats["iterations"].copy())
        xs.append(x)
        on_clusters.append(B.total.cluster_systems)
        B.close()
    assert on_clusters[0] == 0 and min(on_clusters[1:]) >= 3
    for c in counts[1:]:
        assert np.array_equal(c, counts[0]), (counts[0], c)
    for x in xs[1:]:
        assert np.linalg.norm(x - xs[0]) <= 1e-10 * np.linalg.norm(xs[0])
