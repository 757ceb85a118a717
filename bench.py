#!/usr/bin/env python3
"""Pressure-correction PCG benchmark on GB300.

Workload (one step = one solve to 1e-8 relative residual):
  256^3 hex box (16,777,216 cells, 7-point CSR, 117,047,296 nnz),
  variable-coefficient Poisson: k_c = exp(N(0,1)) per cell (seed 42),
  harmonic-averaged to faces through aP = 1/k, Dirichlet p' = 0 on x = 0
  (PressureOutlet), walls elsewhere, rhs N(0,1) in FP64.  The matrix is
  assembled on the device by the library's face-loop assembly.
  value  = time of one mixed-precision (FP32 inner, FP64 residual /
           reductions / x) Jacobi-PCG solve, inputs resident in HBM;
  fp64   = time of the plain FP64 Jacobi-PCG solve of the same system;
  e2e    = the mixed solve through the C ABI with host buffers
           (ILinearSolver::solve(A, b, x) semantics: CSR + b copied in,
           preconditioner set up, x copied out).
Every matrix and vector is far larger than the 129 MB L2, so no flush is
needed between steps.

Further legs in the same JSON line (each can be switched off): batched (512
cavity systems in one launch), adjoint (128^3 face-conductance gradient),
poisson3d (128^3 distorted RCM: FP64 Jacobi, ILU(0), mixed), preconditioners
(64^3: every preconditioner and Krylov kind of make_linear_solver),
pressure_step, cavity, simple (SIMPLE outer iterations on the device) and
state (checkpoint, SIMP), each with the oracle's CPU time beside it where
one is meaningful.

`--impl reference` times the reference CG (CGSolver::solve,
src/solver/LinearSolvers.cpp:420-451) on the host: the compiled reference
when oracle/_ref exists, otherwise the oracle's C restatement of it, on a
bounded number of iterations of the same system, scaled to the iteration
count of the full solve.
"""
from __future__ import annotations

import argparse
import csv
import io
import json
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "PCG time to 1e-8 rel-res, mixed vs plain FP64 on 1 GB300; SpMV HBM GB/s"
SEED = 42


def reference_iterations(n: int):
    """CGSolver::solve's Jacobi iteration count on the n^3 workload to 1e-8, as
    the reference itself ran it (tests/golden/varcoef_256_cg.npz, written by
    tests/golden/make_golden.py from the compiled reference); None for sizes
    without such a run.  The reference arm scales its bounded sample by it."""
    try:
        fx = np.load(os.path.join(ROOT, "tests", "golden", "varcoef_256_cg.npz"))
    except OSError:
        return None
    return int(fx["jacobi_iters"]) if int(fx["n"]) == n else None


def host_cores() -> int:
    try:
        return len(os.sched_getaffinity(0))
    except (AttributeError, OSError):
        return os.cpu_count() or 1

# DRAM bytes (read + write) per row of one launch of the fused mixed step, from
# one ncu capture at 200^3 (profiles/mixed_step_varcoef200.md: 255.99 MB read +
# 99.92 MB written for 8,000,000 rows); scaled by the rows of the workload.
NCU_STEP_DRAM_BYTES_PER_ROW = (255.991552e6 + 99.923968e6) / 8.0e6


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--n", type=int, default=256, help="box side (cells per direction)")
    ap.add_argument("--tol", type=float, default=1e-8)
    ap.add_argument("--max-iterations", type=int, default=50000)
    ap.add_argument("--fp64-steps", type=int, default=2)
    ap.add_argument("--e2e-steps", type=int, default=3)
    ap.add_argument("--cpu-seconds", type=float, default=20.0, help="CPU work per baseline sample")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--batched-systems", type=int, default=512,
                    help="systems in the batched leg (0 disables it)")
    ap.add_argument("--adjoint-n", type=int, default=128, help="box side of the differentiation leg (0 disables it)")
    ap.add_argument("--fd-faces", type=int, default=64, help="faces checked by central differences")
    ap.add_argument("--poisson-n", type=int, default=128, help="box side of the Jacobi-vs-ILU0 leg (0 disables it)")
    ap.add_argument("--precond-n", type=int, default=64,
                    help="box side of the preconditioner / Krylov-kind leg (0 disables it)")
    ap.add_argument("--no-cavity", action="store_true", help="skip the 128x128 cavity pressure-step leg")
    ap.add_argument("--library-cg-sample", type=int, default=10,
                    help="iterations of the restated reference GPU path with its host-side Jacobi (0 disables the "
                         "library comparator)")
    ap.add_argument("--simple-iterations", type=int, default=200,
                    help="outer iterations of the device SIMPLE leg (0 disables it)")
    ap.add_argument("--simple-only", action="store_true",
                    help="run only the device SIMPLE leg and print its JSON (profiling runs)")
    ap.add_argument("--state-only", action="store_true",
                    help="run only the checkpoint / SIMP leg and print its JSON")
    ap.add_argument("--no-accuracy", dest="accuracy", action="store_false",
                    help="skip the error check against a 1e-12 FP64 solve")
    ap.add_argument("--check-interval", type=int, default=0,
                    help="solver check_interval: 0 runs each solve as one device-side graph loop, k > 0 polls the "
                         "stop flag from the host every k steps (chunks of captured steps)")
    return ap.parse_args()


from simall_gb300.replicas import max_over_ranks, rank_info, shard_by_cost  # noqa: E402


# ------------------------------------------------------------------ clocks
class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 200 ms."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.proc = None
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.f,
                                         stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
        time.sleep(0.3)

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.3)
        self.proc.terminate()
        try:
            self.proc.wait(5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.f.flush()
        self.f.seek(0)
        rows = [r for r in csv.reader(io.StringIO(self.f.read())) if len(r) >= 9]
        os.unlink(self.f.name)
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            try:
                sm.append(float(r[1]))
                mx = float(r[2])
            except ValueError:
                continue
            for nm, v in zip(names, r[5:9]):
                if v.strip().lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


# ------------------------------------------------------------------ CPU baseline (oracle / compiled reference)
def cpu_cg_sample(rp, ci, v, b, seconds: float, use_ref: bool):
    """Time the reference CG on a bounded number of iterations; returns
    (seconds per iteration, iterations run, kind)."""
    from oracle import oracle as O

    if use_ref and O.RefLib.available():
        R = O.RefLib()
        run = lambda k: R.cg(rp, ci, v, b, 0, 0.0, k)  # noqa: E731
        kind = "reference"
    else:
        run = lambda k: O.cg(rp, ci, v, b, 0, 0.0, k)  # noqa: E731
        kind = "port"
    t = time.perf_counter()
    run(2)
    t2 = (time.perf_counter() - t) / 2.0
    k = int(max(3, min(2000, seconds / max(t2, 1e-6))))
    t = time.perf_counter()
    run(k)
    el = time.perf_counter() - t
    return el / k, k, kind


# ------------------------------------------------------------------ workload
def build_workload(n: int, ctx):
    import simall_gb300 as sg
    from simall_gb300 import workloads as W

    mesh = sg.cartesian(n, n, n)
    aP, phi, rhs = W.varcoef_inputs(mesh, seed=SEED)
    ps = sg.PressureSystem(mesh, W.X0_OUTLET, ctx=ctx)
    ps.assemble(1.0, aP, phi)
    ctx.synchronize()
    return mesh, ps, rhs


def solver_for(sg, ctx, ps, precision, tol, maxit, check_interval=0):
    cfg = sg.LinearSolverConfig(kind=sg.LinearSolverKind.CG, preconditioner=sg.PreconditionerKind.Jacobi,
                                tolerance=tol, maxIterations=maxit)
    s = sg.GpuCGSolver(cfg, precision=precision, ctx=ctx, check_interval=check_interval)
    from simall_gb300._lib import check
    check(s.L.simall_solver_use_pressure_system(s.handle, ps.handle), ctx.handle)
    return s


def library_cg(rp, ci, vals, rhs, tol, maxit, dev, sample_its=10, full_its=None):
    """The reference's own GPU solver path, gpu::CgGpu::solve with Jacobi
    (src/gpu/CgGpu.cpp:181-219; the library calls of src/gpu/GpuKernels.cpp:
    74-190 and 196-281), restated as its call sequence: a CSR SpMV
    (cuSPARSE, through torch's CSR matrix-vector product), blocking dot
    products and norms (cuBLAS ddot / dnrm2 through torch), axpy and
    x + beta p updates.  Two runs:
      as_written -- the Jacobi apply as the reference writes it
        (GpuKernels.cpp:290-330: copy r to z on the device, copy z and the
        diagonal to the host, divide there, copy z back), timed on
        `sample_its` iterations and scaled to `full_its`;
      device_jacobi -- the same library calls with the Jacobi apply as one
        device operation, run to convergence: the library path at its best.
    The stop test is CgGpu's: ||r|| / ||b|| <= tol on the iterated residual."""
    import warnings

    import torch
    n = len(rhs)
    warnings.filterwarnings("ignore", message="Sparse CSR tensor support is in beta state")
    A = torch.sparse_csr_tensor(torch.from_numpy(np.asarray(rp, np.int32)).to(dev),
                                torch.from_numpy(np.asarray(ci, np.int32)).to(dev),
                                torch.from_numpy(np.asarray(vals, np.float64)).to(dev), size=(n, n),
                                check_invariants=False)
    rows = np.repeat(np.arange(n, dtype=np.int64), np.diff(np.asarray(rp, np.int64)))
    dmask = np.asarray(ci, np.int64) == rows
    diag_h = np.zeros(n)
    diag_h[rows[dmask]] = np.asarray(vals)[dmask]
    diag = torch.from_numpy(diag_h).to(dev)
    safe = torch.where(diag != 0, diag, torch.ones_like(diag))
    b = torch.from_numpy(np.asarray(rhs, np.float64)).to(dev)

    def host_jacobi(r):
        z = r.clone()
        hd = diag.cpu().numpy()
        hz = z.cpu().numpy()
        hz /= np.where(hd != 0.0, hd, 1.0)
        z.copy_(torch.from_numpy(hz))
        return z

    def device_jacobi(r):
        return r / safe

    def solve(precond, limit):
        x = torch.zeros_like(b)
        r = b - torch.mv(A, x)
        bref = float(torch.linalg.vector_norm(b)) or 1.0
        rn = float(torch.linalg.vector_norm(r))
        it = 0
        if rn / bref <= tol:
            return x, 0, rn / bref
        z = precond(r)
        p = z.clone()
        rho = float(torch.dot(r, z))
        for it in range(1, limit + 1):
            q = torch.mv(A, p)
            pq = float(torch.dot(p, q))
            if abs(pq) < 1e-300:
                break
            alpha = rho / pq
            x.add_(p, alpha=alpha)
            r.add_(q, alpha=-alpha)
            rn = float(torch.linalg.vector_norm(r))
            if rn / bref <= tol:
                break
            z = precond(r)
            rho_new = float(torch.dot(r, z))
            p.mul_(rho_new / rho).add_(z)
            rho = rho_new
        return x, it, rn / bref

    def timed(fn):
        if dev.type == "cuda":
            torch.cuda.synchronize()
        t = time.perf_counter()
        out = fn()
        if dev.type == "cuda":
            torch.cuda.synchronize()
        return out, time.perf_counter() - t

    solve(device_jacobi, 3)  # warm: cuSPARSE and cuBLAS handles, buffers
    (_, k_host, _), t_host = timed(lambda: solve(host_jacobi, sample_its))
    (x, its, rel), t_dev = timed(lambda: solve(device_jacobi, maxit))
    full = full_its or its
    xr = x.cpu().numpy()
    y = np.add.reduceat(np.asarray(vals) * xr[np.asarray(ci)], np.asarray(rp)[:-1])
    true_res = float(np.linalg.norm(np.asarray(rhs) - y) / (np.linalg.norm(rhs) or 1.0))
    return {"kind": "the reference's gpu::CgGpu call sequence restated: cuSPARSE CSR SpMV and cuBLAS-class "
                    "BLAS-1 through torch, FP64 (a library comparator, not this library's path)",
            "as_written": {"value": round(t_host / max(k_host, 1) * full, 3), "unit": "s",
                           "sample": f"{k_host} iterations with the reference's host-side Jacobi apply "
                                     f"({t_host / max(k_host, 1) * 1e3:.2f} ms/iteration), scaled to {full}"},
            "device_jacobi": {"value": round(t_dev, 4), "unit": "s", "iterations": int(its),
                              "iterated_residual": rel, "true_residual": true_res}}


def time_kernel(s, k, reps=20):
    import ctypes as C
    from simall_gb300._lib import check
    ms = C.c_double()
    by = C.c_double()
    check(s.L.simall_solver_time_kernel(s.handle, k, reps, C.byref(ms), C.byref(by)), s.ctx.handle)
    return ms.value, by.value


def _cpu_batched_solve(args):
    """One batched-leg system solved by the oracle's CGSolver::solve (Jacobi),
    in a worker process; returns (seconds of the solve, iterations)."""
    side, b, tol = args
    from oracle import oracle as O

    m = O.cartesian_mesh(side, side, 1, 1.0, 1.0, 1.0 / side)
    rp, ci = O.build_sparsity(m)
    v, _, _ = O.assemble(m, rp, ci, [], 1.0, np.ones(m.nC), np.zeros(m.nF))
    t = time.perf_counter()
    _, it, _ = O.cg(rp, ci, v, b, 0, tol, 50000)
    return time.perf_counter() - t, it


def cpu_batched_baseline(sides, rhs, tol):
    """The reference's loop of serial CG solves over the batch, timed on the
    host: every system solved once in a pool of worker processes (started
    with spawn); the serial figure is the sum of the per-solve times, the
    parallel one the pool's wall time over all host cores (an upper bound:
    the reference solves the systems one after another)."""
    import multiprocessing as mp

    cores = host_cores()
    t0 = time.perf_counter()
    with mp.get_context("spawn").Pool(cores) as pool:
        res = pool.map(_cpu_batched_solve, [(int(sd), np.asarray(b), tol) for sd, b in zip(sides, rhs)], chunksize=1)
    wall = time.perf_counter() - t0
    serial = float(sum(r[0] for r in res))
    return {"value": round(serial, 3), "unit": "s", "cores": 1, "host_nproc": cores, "kind": "port",
            "iterations": int(sum(r[1] for r in res)),
            "sample": f"the oracle's CGSolver::solve (Jacobi, tol {tol:g}) of every system, one after another "
                      "(sum of the per-solve times)",
            "parallel_upper_bound": {"value": round(wall, 3), "unit": "s", "cores": cores,
                                     "note": "the same solves spread over all host cores; the reference loops "
                                             "over the systems serially"}}


def run_batched(a, ctx, sg, rank=0, world=1, with_cpu=False):
    """Batched leg: `count` cavity pressure systems (sides log-uniform in
    [32, 256], rhs N(0,1) with mean removed, one pinned cell) solved in one
    persistent launch (mixed precision) against a loop of plain FP64
    Jacobi-PCG solves of the same systems with the matrices resident.  With
    N ranks the systems are shared out by size (no exchange between ranks) and
    the reported time is the slowest rank's."""
    import torch
    from simall_gb300 import workloads as W

    count = a.batched_systems
    t0 = time.perf_counter()
    systems, rhs, sides = W.batched_cavity_systems(count=count, seed=SEED, ctx=ctx)
    if world > 1:
        mine = shard_by_cost(np.asarray(sides, np.float64) ** 2, rank, world)
        systems = [systems[i] for i in mine]
        rhs = [rhs[i] for i in mine]
    cfg = sg.LinearSolverConfig(kind=sg.LinearSolverKind.CG, preconditioner=sg.PreconditionerKind.Jacobi,
                                tolerance=a.tol, maxIterations=a.max_iterations)
    B = sg.BatchedSolver(cfg, ctx=ctx)
    rows = B.set_systems(systems)
    b = torch.from_numpy(np.concatenate(rhs)).cuda()
    x = torch.empty_like(b)
    setup = time.perf_counter() - t0
    stream = torch.cuda.ExternalStream(ctx.stream)
    for _ in range(max(1, a.warmup)):
        B.solve(b, x, per_system=False)
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(a.steps):
        _, st = B.solve(b, x)
    e1.record(stream)
    e1.synchronize()
    batch_ms = max_over_ranks(e0.elapsed_time(e1) / a.steps, device=b.device)
    tot = B.total
    # baseline: one FP64 solver per system, matrix resident, solves in a loop
    solvers, bs, xs = [], [], []
    for (rp, ci, va), r in zip(systems, rhs):
        s = sg.GpuCGSolver(cfg, precision=sg.Precision.FP64, ctx=ctx)
        s.set_matrix(rp, ci, va)
        solvers.append(s)
        bs.append(torch.from_numpy(r).cuda())
        xs.append(torch.empty_like(bs[-1]))
    for s, bb, xx in zip(solvers, bs, xs):  # warm (graph capture per solver)
        s.solve_into(bb, xx)
    torch.cuda.synchronize()
    t = time.perf_counter()
    its = 0
    for s, bb, xx in zip(solvers, bs, xs):
        its += s.solve_into(bb, xx)
    torch.cuda.synchronize()
    loop_s = max_over_ranks(time.perf_counter() - t, device=b.device)
    xb = x.cpu().numpy()
    diff = max(float(np.linalg.norm(xb[rows[i]:rows[i + 1]] - xs[i].cpu().numpy()) /
                     max(np.linalg.norm(xs[i].cpu().numpy()), 1e-30)) for i in range(len(systems)))
    for s in solvers:
        s.close()
    cpu = cpu_batched_baseline(sides, rhs, a.tol) if with_cpu else None
    out = {"workload": f"{count} cavity pressure systems, sides log-uniform [32,256] (seed {SEED}), "
                        f"{int(rows[-1])} rows", "value": round(batch_ms / 1e3, 6), "unit": "s",
            "fp64_loop": {"value": round(loop_s, 4), "unit": "s", "iterations": int(its)},
            "speedup_vs_fp64_loop": round(loop_s / (batch_ms / 1e3), 2),
            "converged": int(tot.converged), "systems": int(tot.systems), "max_iterations": int(tot.max_iterations),
            "total_iterations": int(tot.total_iterations), "worst_true_residual": float(tot.worst_true_residual),
            "max_rel_diff_vs_fp64": diff,
            "launch_shape": {"block_threads": int(tot.block_threads), "ctas_per_sm": int(tot.ctas_per_sm),
                             "rows_per_pass": int(tot.rows_per_pass),
                             "cluster_rows": int(tot.cluster_rows), "cluster_ctas": int(tot.cluster_ctas),
                             "clusters": int(tot.clusters), "systems_on_clusters": int(tot.cluster_systems),
                             "source": ["set", "timed", "autotuner cache"][int(tot.autotune_source)]},
            "setup_seconds": round(setup, 2), "ranks": world, "systems_on_rank0": len(systems)}
    # roofline of the fused step: per row and step the packed state is read
    # and written (2 x 16 B), the row sum read (4 B) and the two stored upper
    # diagonals of a 5-point system (2 x 4 B): 44 B x rows x steps of each system
    row_steps = float(sum(int(st["iterations"][i]) * int(rows[i + 1] - rows[i]) for i in range(len(systems))))
    gbs = 44.0 * row_steps / (batch_ms / 1e3) / 1e9
    peak, peak_kind = measured_peaks()
    out["roofline"] = {"bound": "hbm", "bytes_per_row_step": 44, "row_steps": row_steps, "achieved": round(gbs, 1),
                       "peak": peak, "unit": "GB/s", "frac": round(gbs / peak, 4),
                       "peak_source": f"{peak_kind} hbm_gbs",
                       "note": "algorithmic bytes; systems of up to 65,536 rows keep part of their state in L2"}
    if cpu:
        out["cpu_baseline"] = cpu
    return out


def run_adjoint(a, ctx, sg):
    """Differentiation leg: N^3 box, face conductances exp(N(0,0.5)) on
    interior and x=0 faces, Dirichlet values N(0,1) on x=0, cell source
    N(0,1); L = 0.5 ||x - x_t||^2 with x_t the solution for a second seeded
    conductance field.  Timed: forward (assembly + mixed solve) and backward
    (adjoint mixed solve + gradient scatter), both to 1e-10.  Checked: central
    differences (h = 1e-6, FP64 solves to 1e-13) on seeded faces."""
    import torch
    from simall_gb300 import workloads as W

    n = a.adjoint_n
    m = sg.cartesian(n, n, n)
    k, pb, dirichlet, src = W.facek_inputs(m, seed=SEED)
    kt, _, _, _ = W.facek_inputs(m, seed=SEED + 1)
    bcs = [(1, int(sg.BCType.PressureOutlet))] + [(z, int(sg.BCType.NoSlipWall)) for z in range(2, 7)]
    ps = sg.PressureSystem(m, bcs, ctx=ctx)
    mk = lambda tol, prec: sg.GpuCGSolver(sg.LinearSolverConfig(  # noqa: E731
        kind=sg.LinearSolverKind.CG, preconditioner=sg.PreconditionerKind.Jacobi, tolerance=tol,
        maxIterations=a.max_iterations), precision=prec, ctx=ctx)
    smx = mk(1e-10, sg.Precision.MIXED)
    s64 = mk(1e-13, sg.Precision.FP64)
    dev = torch.device("cuda:0")
    tk, tkt, tpb, tsrc = (torch.from_numpy(v).to(dev) for v in (k, kt, pb, src))
    x = torch.empty(m.n_cells, dtype=torch.float64, device=dev)
    xt = torch.empty_like(x)
    lam, dk, dpb = torch.empty_like(x), torch.empty_like(tk), torch.empty_like(tk)
    ps.assemble_face_conductance(1.0, tkt, tpb, tsrc)
    ps.solve(s64, xt)

    def step():
        ps.assemble_face_conductance(1.0, tk, tpb, tsrc)
        ps.solve(smx, x)
        tf = time.perf_counter()
        ps.adjoint(smx, 1.0, tk, tpb, x, x - xt, lam, dk, dpb)
        ctx.synchronize()
        return tf

    for _ in range(max(1, a.warmup)):
        step()
    fw, bw = [], []
    for _ in range(a.steps):
        t0 = time.perf_counter()
        tf = step()
        t1 = time.perf_counter()
        fw.append(tf - t0)
        bw.append(t1 - tf)
    it_fwd = int(smx.stats.iterations)
    # FP64 reference gradient and central differences
    ps.assemble_face_conductance(1.0, k, pb, src)
    x64 = ps.solve(s64)
    xth = xt.cpu().numpy()
    lam64, dk64, dpb64 = ps.adjoint(s64, 1.0, k, pb, x64, x64 - xth)
    g_mx = np.concatenate([dk.cpu().numpy(), dpb.cpu().numpy()])
    g_64 = np.concatenate([dk64, dpb64])
    mixed_vs_fp64 = float(np.linalg.norm(g_mx - g_64) / np.linalg.norm(g_64))

    def solve_x(kk, pp):
        ps.assemble_face_conductance(1.0, kk, pp, src)
        return ps.solve(s64)

    def dloss(xp, xm):
        # L(+) - L(-) = 0.5 (x+ - x-).(x+ + x- - 2 x_t): no cancellation of two ~1e6 losses
        return 0.5 * float(np.dot(xp - xm, xp + xm - 2.0 * xth))

    rng = np.random.default_rng(SEED + 7)
    nd = max(1, a.fd_faces // 8)
    kf = rng.choice(np.flatnonzero(k > 0), size=a.fd_faces - nd, replace=False)
    pf = rng.choice(np.flatnonzero(dirichlet), size=nd, replace=False)
    h = 1e-6
    errs, abs_errs, gmax = [], [], 0.0
    for f in kf:
        kp, km = k.copy(), k.copy()
        kp[f] += h
        km[f] -= h
        fd = dloss(solve_x(kp, pb), solve_x(km, pb)) / (2 * h)
        errs.append(abs(fd - dk64[f]) / max(abs(dk64[f]), 1e-300))
        abs_errs.append(abs(fd - dk64[f]))
        gmax = max(gmax, abs(dk64[f]))
    for f in pf:
        pp, pm = pb.copy(), pb.copy()
        pp[f] += h
        pm[f] -= h
        fd = dloss(solve_x(k, pp), solve_x(k, pm)) / (2 * h)
        errs.append(abs(fd - dpb64[f]) / max(abs(dpb64[f]), 1e-300))
        abs_errs.append(abs(fd - dpb64[f]))
        gmax = max(gmax, abs(dpb64[f]))
    ps.close()
    return {"workload": f"face-conductance Poisson {n}^3, k_f=exp(N(0,0.5)), Dirichlet N(0,1) on x=0, "
                        f"L=0.5|x-x_t|^2", "faces": int(m.n_faces),
            "forward_s": round(float(np.median(fw)), 5), "backward_s": round(float(np.median(bw)), 5),
            "forward_iterations": it_fwd, "tolerance": 1e-10,
            "fd_faces": len(errs), "fd_h": h, "fd_max_rel_err": float(np.max(errs)),
            "fd_median_rel_err": float(np.median(errs)), "fd_max_err_over_max_grad": float(max(abs_errs) / gmax),
            "mixed_vs_fp64_gradient_rel": mixed_vs_fp64}


def run_poisson3d(a, ctx, sg):
    """3-D pressure Poisson: N^3 box, interior nodes shifted by U(-0.2,0.2)h,
    RCM renumbering, aP = 1, interior face flux N(0,1), walls (cell-0 pin);
    FP64 Jacobi-PCG against ILU0-PCG to 1e-8, and the mixed-precision solve
    (after RCM the matrix has no diagonal structure: sliced storage, the whole
    solve in one persistent cooperative launch), with its step kernel timed
    alone against the HBM roofline."""
    import torch
    from simall_gb300 import workloads as W

    n = a.poisson_n
    m, rcm_stats = W.poisson3d_mesh(n, seed=SEED)
    aP, phi = W.poisson3d_inputs(m, seed=SEED)
    ps = sg.PressureSystem(m, W.ALL_WALLS, ctx=ctx)
    ps.assemble(1.0, aP, phi)
    res = {"workload": f"poisson3d {n}^3 distorted +-20%, RCM (bandwidth {rcm_stats[0]} -> {rcm_stats[1]}), "
                       f"walls + cell-0 pin, FP64 PCG to {a.tol:g}", "nnz": int(ps.nnz)}
    stream = torch.cuda.ExternalStream(ctx.stream)
    x = torch.empty(m.n_cells, dtype=torch.float64, device="cuda")
    for name, pc, prec in (("jacobi", sg.PreconditionerKind.Jacobi, sg.Precision.FP64),
                           ("ilu0", sg.PreconditionerKind.ILU, sg.Precision.FP64),
                           ("mixed_jacobi", sg.PreconditionerKind.Jacobi, sg.Precision.MIXED)):
        s = sg.GpuCGSolver(sg.LinearSolverConfig(kind=sg.LinearSolverKind.CG, preconditioner=pc, tolerance=a.tol,
                                                 maxIterations=a.max_iterations), precision=prec, ctx=ctx)
        ps.solve(s, x)  # warm: setup, graph capture
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record(stream)
        ps.solve(s, x)
        e1.record(stream)
        e1.synchronize()
        res[name] = {"value": round(e0.elapsed_time(e1) / 1e3, 5), "unit": "s", "iterations": int(s.stats.iterations),
                     "true_residual": float(s.stats.true_residual), "engine": int(s.stats.engine)}
        if prec == sg.Precision.MIXED:
            # the sliced step kernel alone (CUDA events, back-to-back launches):
            # 6 B per stored entry, 36 B per row (state read + written, e), slice pointers
            ms, by = time_kernel(s, 4)
            peak, peak_kind = measured_peaks()
            gbs = by / ms / 1e6
            st_s = res[name]["value"] / max(1, res[name]["iterations"])
            res[name]["step_kernel"] = {"us": round(ms * 1e3, 2), "algorithmic_bytes": round(by), "gbs": round(gbs, 1),
                                        "frac": round(gbs / peak, 4), "peak": peak,
                                        "peak_source": f"{peak_kind} hbm_gbs"}
            res[name]["per_step_in_solve_us"] = round(st_s * 1e6, 2)
            res[name]["effective_gbs_in_solve"] = round(by / st_s / 1e9, 1)
        s.close()
    ps.close()
    res["speedup_mixed_vs_fp64_jacobi"] = round(res["jacobi"]["value"] / res["mixed_jacobi"]["value"], 3)
    return res


def run_preconditioners(a, ctx, sg, with_cpu):
    """Every preconditioner and Krylov kind of make_linear_solver on one
    system: the N^3 distorted, RCM-renumbered Poisson of the poisson3d leg
    (FP64, tol 1e-8).  setup = set_matrix with the matrix already in device
    memory (pattern analysis, ILU(0) factor, SSOR schedules, the AMG
    hierarchy built on the host), solve = CUDA events around the solve."""
    import torch
    from simall_gb300 import workloads as W

    n = a.precond_n
    m, _ = W.poisson3d_mesh(n, seed=SEED)
    aP, phi = W.poisson3d_inputs(m, seed=SEED)
    ps = sg.PressureSystem(m, W.ALL_WALLS, ctx=ctx)
    ps.assemble(1.0, aP, phi)
    rp_h, ci_h = ps.pattern()
    vals_h, rhs_h = ps.download()
    dev = torch.device("cuda")
    rp, ci = torch.from_numpy(rp_h).to(dev), torch.from_numpy(ci_h).to(dev)
    vals, b = torch.from_numpy(vals_h).to(dev), torch.from_numpy(rhs_h).to(dev)
    x = torch.empty_like(b)
    stream = torch.cuda.ExternalStream(ctx.stream)
    K, P = sg.LinearSolverKind, sg.PreconditionerKind
    cases = [("cg_jacobi", K.CG, P.Jacobi), ("cg_ilu0", K.CG, P.ILU), ("cg_ssor", K.CG, P.SSOR),
             ("cg_amg", K.CG, P.AMG), ("bicgstab_ssor", K.BiCGSTAB, P.SSOR), ("gmres30_ilu0", K.GMRES, P.ILU),
             ("tfqmr_ssor", K.TFQMR, P.SSOR), ("bicgstab_amg", K.BiCGSTAB, P.AMG)]
    res = {"workload": f"poisson3d {n}^3 distorted +-20%, RCM, walls + cell-0 pin, FP64 to {a.tol:g}",
           "rows": int(m.n_cells), "nnz": int(ps.nnz)}
    for name, kind, pc in cases:
        s = sg.make_linear_solver(sg.LinearSolverConfig(kind=kind, preconditioner=pc, tolerance=a.tol,
                                                        maxIterations=2000, restart=30), ctx=ctx)
        s.set_matrix(rp, ci, vals)
        if pc != P.AMG:  # warm: graph capture (an AMG setup drops the graphs: its timed solve recaptures)
            s.solve_into(b, x)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        s.set_matrix(rp, ci, vals)
        s.update_values(vals)  # the preconditioner is set up again, as the reference does per solve
        torch.cuda.synchronize()
        setup = time.perf_counter() - t0
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record(stream)
        s.solve_into(b, x)
        e1.record(stream)
        e1.synchronize()
        r = {"setup_s": round(setup, 4), "solve_s": round(e0.elapsed_time(e1) / 1e3, 5),
             "iterations": int(s.stats.iterations), "true_residual": float(s.stats.true_residual),
             "converged": bool(s.stats.converged)}
        if pc == P.AMG:
            r["amg_levels"] = s.amg_levels()
        res[name] = r
        s.close()
    if with_cpu:
        from oracle import oracle as O

        cpu = {}
        for name, pc in (("cg_jacobi", 0), ("cg_ilu0", 1), ("cg_ssor", 2)):
            t = time.perf_counter()
            _, it, _ = O.cg(rp_h, ci_h, vals_h, rhs_h, pc, a.tol, 2000)
            cpu[name] = {"value": round(time.perf_counter() - t, 3), "unit": "s", "iterations": int(it)}
        res["cpu_baseline"] = {"cores": 1, "host_nproc": host_cores(), "kind": "port", "solves": cpu,
                               "sample": "the oracle's CGSolver::solve (setup included) on 1 host core; AMG is not "
                                         "timed on the CPU: the reference's setup rescans all rows for every C "
                                         "point (O(n^2))"}
    ps.close()
    return res


def run_cavity(a, ctx, sg, with_cpu):
    """2-D lid-driven cavity 128x128 (Re 100, SIMPLE urfP 0.3 / urfU 0.7, 200
    outer iterations): the pressure step of every outer iteration -- aP and
    phi from host memory, device assembly, Jacobi-PCG to 1e-8, p' back to host
    memory.  The systems are the reference SIMPLE loop's first and last ones
    (tests/golden/cavity_simple_128.npz); outer iteration 0 uses the first,
    iterations 1..199 the last (the reference's solves take 737, then 775
    iterations every time)."""
    from simall_gb300 import workloads as W

    c = np.load(os.path.join(ROOT, "tests", "golden", "cavity_simple_128.npz"))
    N, n_outer = int(c["N"]), int(c["n_outer"])
    m = sg.cartesian(N, N, 1, 1.0, 1.0, 1.0 / N)
    ps = sg.PressureSystem(m, W.CAVITY, ctx=ctx)
    aP = [np.ascontiguousarray(c["aP"][k]) for k in range(2)]
    phi = [np.ascontiguousarray(c["phi"][k]) for k in range(2)]
    x = np.empty(m.n_cells)
    res = {"workload": f"cavity {N}x{N} SIMPLE pressure steps (host aP, phi in; device assembly + Jacobi-PCG to "
                       f"1e-8; p' out), {n_outer} outer iterations", "cells": int(m.n_cells), "nnz": int(ps.nnz)}
    for name, prec in (("fp64", sg.Precision.FP64), ("mixed", sg.Precision.MIXED)):
        s = sg.GpuCGSolver(sg.LinearSolverConfig(kind=sg.LinearSolverKind.CG,
                                                 preconditioner=sg.PreconditionerKind.Jacobi, tolerance=1e-8,
                                                 maxIterations=1000), precision=prec, ctx=ctx)
        for k in (0, 1):  # warm: setup, graph capture
            ps.assemble(1.0, aP[k], phi[k])
            ps.solve(s, x)
        ctx.synchronize()
        its, worst = 0, 0.0
        t0 = time.perf_counter()
        for i in range(n_outer):
            k = 0 if i == 0 else 1
            ps.assemble(1.0, aP[k], phi[k])
            ps.solve(s, x)
            its += int(s.stats.iterations)
            worst = max(worst, float(s.stats.true_residual))
        ctx.synchronize()
        res[name] = {"value": round(time.perf_counter() - t0, 4), "unit": "s", "iterations": its,
                     "worst_true_residual": worst}
        s.close()
    ps.close()
    if with_cpu:
        # the reference CG (the oracle's bit-identical restatement) on the same two systems, 1 host core
        from oracle import oracle as O
        om = O.cartesian_mesh(N, N, 1, 1.0, 1.0, 1.0 / N)
        rp, ci = O.build_sparsity(om)
        ts = []
        for k in (0, 1):
            v, rhs, _ = O.assemble(om, rp, ci, [], 1.0, aP[k], phi[k])
            t = time.perf_counter()
            O.cg(rp, ci, v, rhs, 0, 1e-8, 1000)
            ts.append(time.perf_counter() - t)
        res["cpu_baseline"] = {"value": round(ts[0] + (n_outer - 1) * ts[1], 3), "unit": "s", "cores": 1, "host_nproc": host_cores(),
                               "kind": "port", "sample": "one CG solve of each of the two systems on 1 host core, "
                                                         f"scaled to {n_outer} solves (solve only)"}
    return res


def run_pressure_step(a, ctx, sg, with_cpu):
    """The device-resident pressure step on the distorted 128^3 box (RCM):
    compute_face_fluxes -> assembly -> FP64 Jacobi-PCG to 1e-8 ->
    correct_fields, every field in device memory, each stage timed with CUDA
    events; the face loops' algorithmic bytes give their GB/s."""
    import torch
    from simall_gb300 import workloads as W

    n = a.poisson_n
    m, _ = W.poisson3d_mesh(n, seed=SEED)
    ps = sg.PressureSystem(m, W.ALL_WALLS, ctx=ctx)
    ps.setup_field_loops()
    rng = np.random.default_rng(SEED + 9)
    dev = torch.device("cuda")
    U = [torch.from_numpy(rng.standard_normal(m.n_cells)).to(dev) for _ in range(3)]
    aP = torch.from_numpy(rng.uniform(0.5, 2.0, m.n_cells)).to(dev)
    p = torch.zeros(m.n_cells, dtype=torch.float64, device=dev)
    phi = torch.empty(m.n_faces, dtype=torch.float64, device=dev)
    pp = torch.empty_like(p)
    s = sg.GpuCGSolver(sg.LinearSolverConfig(kind=sg.LinearSolverKind.CG, preconditioner=sg.PreconditionerKind.Jacobi,
                                             tolerance=a.tol, maxIterations=a.max_iterations), ctx=ctx)
    stream = torch.cuda.ExternalStream(ctx.stream)
    stages = {"fluxes": lambda: ps.face_fluxes(1.0, U, phi), "assemble": lambda: ps.assemble(1.0, aP, phi),
              "solve": lambda: ps.solve(s, pp), "correct": lambda: ps.correct_fields(1.0, 0.3, aP, pp, p, U, phi)}
    for f in stages.values():  # warm
        f()
    ms = {}
    for name, f in stages.items():
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record(stream)
        f()
        e1.record(stream)
        e1.synchronize()
        ms[name] = e0.elapsed_time(e1)
    nC, nF = m.n_cells, m.n_faces
    nEnt = int(2 * np.count_nonzero(m.neighbor != sg.mesh.BOUNDARY) + np.count_nonzero(m.neighbor == sg.mesh.BOUNDARY))
    by = {"fluxes": 41 * nF + 24 * nC,
          "correct": 4 * nC + 4 * nEnt + 48 * nF + 8 * nC + 48 * nC + 24 * nC + 112 * nC + 40 * nF}
    res = {"workload": f"poisson3d {n}^3 distorted, RCM: fluxes -> assembly -> Jacobi-PCG to {a.tol:g} -> correction, "
                       f"fields in device memory", "cells": nC, "faces": nF,
           "ms": {k: round(v, 3) for k, v in ms.items()}, "iterations": int(s.stats.iterations),
           "gbs": {k: round(by[k] / (ms[k] * 1e6), 1) for k in by}}
    if with_cpu:
        from oracle import oracle as O
        om = O.cartesian_mesh(n, n, n, node_shift=W.interior_node_shift(n, n, n, amp=0.2, seed=SEED))
        O.rcm(om)
        Uh = [u.cpu().numpy() for u in U]
        t = time.perf_counter()
        ph = O.face_fluxes(om, [(z, 1) for z in range(1, 7)], 1.0, Uh)
        t1 = time.perf_counter()
        O.correct_fields(om, 1.0, 0.3, aP.cpu().numpy(), pp.cpu().numpy(), np.zeros(nC), Uh, ph)
        t2 = time.perf_counter()
        res["cpu_baseline"] = {"fluxes_ms": round((t1 - t) * 1e3, 1), "correct_ms": round((t2 - t1) * 1e3, 1),
                               "cores": 1, "host_nproc": host_cores(), "kind": "port"}
    s.close()
    ps.close()
    return res


CAVITY_SIMPLE_BCS = [(z, 1) for z in (1, 2, 3, 5, 6)] + [(4, 2, (1.0, 0.0, 0.0))]


def run_simple(a, ctx, sg, with_cpu):
    """The whole SIMPLE outer iteration on the device (fluxes, momentum
    assembly and three momentum solves, fluxes, pressure-correction assembly
    and solve, correction; U, p, phi resident) on the 128x128 lid-driven
    cavity (Re 100, urfU 0.7, urfP 0.3) from rest, with the reference's
    solver settings (GMRES(30)+ILU(0) momentum to 1e-6, FP64 Jacobi-CG
    pressure to 1e-8) and with GMRES(30)+Jacobi momentum and mixed-precision
    pressure; seconds per outer iteration over `simple_iterations` outer
    iterations from rest (default 200: the cavity configuration as written,
    applications/simall_cavity/main.cpp), against the oracle's restatement of
    SimpleAlgorithm::iterate run for the same iterations on one host core, and
    the fields of both device runs against the oracle's after the last one."""
    from oracle import oracle as O  # the parity check and the CPU baseline only

    N = 128
    n_it = a.simple_iterations
    m = sg.cartesian(N, N, 1, 1.0, 1.0, 1.0 / N)
    configs = {
        "reference_settings": ((0, 1, 1e-6, 200, 30), (2, 0, 1e-8, 1000, 30), sg.Precision.FP64),
        "gb300_settings": ((0, 0, 1e-6, 200, 30), (2, 0, 1e-8, 1000, 30), sg.Precision.MIXED),
    }
    res = {"workload": f"cavity {N}x{N} SIMPLE outer iterations from rest (Re 100), every field in device memory",
           "cells": int(m.n_cells), "iterations_timed": n_it}

    def make(cfg):
        mc, pc, prec = cfg
        mom = sg.make_linear_solver(sg.LinearSolverConfig(sg.LinearSolverKind(mc[0]), sg.PreconditionerKind(mc[1]),
                                                          mc[2], mc[3], mc[4]), ctx=ctx)
        pres = sg.GpuCGSolver(sg.LinearSolverConfig(sg.LinearSolverKind.CG, sg.PreconditionerKind(pc[1]), pc[2],
                                                    pc[3]), precision=prec, ctx=ctx)
        alg = sg.GpuSimpleAlgorithm(m, CAVITY_SIMPLE_BCS, mom, pres, sg.SimpleOptions(mu=0.01), ctx=ctx)
        return alg, mom, pres

    fields = {}
    for name, cfg in configs.items():
        alg, mom, pres = make(cfg)
        for _ in range(2):  # warm: preconditioner analysis, graph capture
            alg.iterate()
        alg.close()
        alg = sg.GpuSimpleAlgorithm(m, CAVITY_SIMPLE_BCS, mom, pres, sg.SimpleOptions(mu=0.01), ctx=ctx)
        ctx.synchronize()
        its = np.zeros(4, np.int64)
        t0 = time.perf_counter()
        for _ in range(n_it):
            r = alg.iterate()
            its += np.array(r.iterations)
        ctx.synchronize()
        sec = (time.perf_counter() - t0) / n_it
        res[name] = {"value": round(sec, 6), "unit": "s per outer iteration", "total_s": round(sec * n_it, 4),
                     "momentum": f"GMRES({cfg[0][4]})+{'ILU(0)' if cfg[0][1] == 1 else 'Jacobi'} to {cfg[0][2]:g}",
                     "pressure": f"{'mixed' if cfg[2] == sg.Precision.MIXED else 'FP64'} Jacobi-CG to {cfg[1][2]:g}",
                     "solve_iterations_per_outer": [round(float(v) / n_it, 1) for v in its]}
        fields[name] = alg.fields()
        alg.close()
        mom.close()
        pres.close()
    # parity: the oracle's SimpleAlgorithm::iterate (reference settings) for the
    # same outer iterations from rest; its time on one host core is the CPU
    # baseline (the whole run, as the cavity configuration is written)
    om = O.cartesian_mesh(N, N, 1, 1.0, 1.0, 1.0 / N)
    so = O.SimpleOracle(om, CAVITY_SIMPLE_BCS, mu=0.01, mom_cfg=configs["reference_settings"][0],
                        p_cfg=configs["reference_settings"][1])
    t = time.perf_counter()
    for _ in range(n_it):
        so.iterate()
    cpu_s = (time.perf_counter() - t) / n_it
    U, p, _ = fields["reference_settings"]
    Um, pm, _ = fields["gb300_settings"]
    res[f"parity_{n_it}_iterations"] = {
        "reference_settings": {"rel_U": float(np.linalg.norm(U - so.U) / np.linalg.norm(so.U)),
                               "rel_p": float(np.linalg.norm(p - so.p) / np.linalg.norm(so.p))},
        "gb300_settings": {"rel_U": float(np.linalg.norm(Um - so.U) / np.linalg.norm(so.U)),
                           "rel_p": float(np.linalg.norm(pm - so.p) / np.linalg.norm(so.p))}}
    if with_cpu:
        res["cpu_baseline"] = {"value": round(cpu_s, 4), "unit": "s per outer iteration", "cores": 1,
                               "host_nproc": host_cores(), "kind": "port", "total_s": round(cpu_s * n_it, 2),
                               "sample": f"the oracle's SimpleAlgorithm::iterate, reference settings, all {n_it} "
                                         "outer iterations from rest on 1 host core"}
    return res


def run_state(a, ctx, sg, with_cpu):
    """The device field registry, io::Checkpoint and SIMP on the 128^3 box
    (RCM): a checkpoint of U (vector) and four scalar fields written from HBM
    to a file and read back (mesh section without nodes), against writing the
    same bytes from host memory; one SIMP design step (filter off and on)
    on the device against the oracle's SimpTopology::step on a 64^3 sample."""
    import tempfile

    from simall_gb300 import workloads as W

    n = a.poisson_n
    m, _ = W.poisson3d_mesh(n, seed=SEED)
    nC = m.n_cells
    reg = sg.DeviceFieldRegistry(ctx)
    rng = np.random.default_rng(SEED + 21)
    reg.upload("U", rng.standard_normal((3, nC)), vector=True)
    for name in ("p", "T", "k", "rho"):
        reg.upload(name, rng.standard_normal(nC))
    mesh = {name: np.zeros(0, dt) for name, dt in sg._lib.CHECKPOINT_MESH_ARRAYS}
    for k in ("owner", "neighbor", "boundary_zone", "volume", "cell_centroid_x", "cell_centroid_y", "cell_centroid_z",
              "cell_face_offsets", "cell_face_indices"):
        mesh[k] = getattr(m, k)
    for k in ("area_x", "area_y", "area_z", "centroid_x", "centroid_y", "centroid_z"):
        mesh[k] = getattr(m, k)
    res = {"workload": f"{n}^3 box: checkpoint of U + 4 scalar fields ({7 * nC * 8 / 1e6:.0f} MB of fields) and the "
                       "mesh arrays; SIMP design steps", "cells": nC}
    empty = {name: np.zeros(0, dt) for name, dt in sg._lib.CHECKPOINT_MESH_ARRAYS}
    with tempfile.TemporaryDirectory() as td:
        out = {}
        for tag, msh in (("fields_only", empty), ("with_mesh", mesh)):
            path = os.path.join(td, tag + ".simallcp")
            sg.checkpoint_write(path, msh, reg, 1, 0.0, 0)  # warm: page cache, pinned staging
            t = time.perf_counter()
            sg.checkpoint_write(path, msh, reg, 2, 0.0, 0)
            tw = time.perf_counter() - t
            size = os.path.getsize(path)
            reg2 = sg.DeviceFieldRegistry(ctx)
            sg.checkpoint_read(path, reg2, with_mesh=True)
            t = time.perf_counter()
            sg.checkpoint_read(path, reg2, with_mesh=True)
            tr = time.perf_counter() - t
            same = bool(np.array_equal(reg2.download("U", vector=True), reg.download("U", vector=True)))
            reg2.close()
            out[tag] = {"bytes": size, "write_s": round(tw, 4), "write_gbs": round(size / tw / 1e9, 2),
                        "read_s": round(tr, 4), "read_gbs": round(size / tr / 1e9, 2), "round_trip_exact": same}
        host = np.concatenate([reg.download("U", vector=True).ravel()] +
                              [reg.download(k) for k in ("p", "T", "k", "rho")])
        t = time.perf_counter()
        host.tofile(os.path.join(td, "host.bin"))
        th = time.perf_counter() - t
        out["host_fields_tofile_gbs"] = round(host.nbytes / th / 1e9, 2)
    res["checkpoint"] = out
    reg.close()
    # SIMP design step at 64^3 on the device and in the oracle
    ns = 64
    ms, _ = W.poisson3d_mesh(ns, seed=SEED)
    ps = sg.PressureSystem(ms, W.ALL_WALLS, ctx=ctx)
    ps.setup_field_loops()
    dC = -np.abs(rng.standard_normal(ms.n_cells)) * 0.1
    simp_res = {"cells": int(ms.n_cells)}
    for tag, radius in (("no_filter", 0.0), ("filter", 1.5 / ns)):
        r3 = sg.DeviceFieldRegistry(ctx)
        simp = sg.GpuSimpTopology(ps, r3, sg.SimpConfig(filterRadius=radius))
        r3.upload("dC_drho", dC)
        simp.step()  # warm
        r3.upload("dC_drho", dC)
        ctx.synchronize()
        t = time.perf_counter()
        simp.step()
        simp_res[tag] = {"value": round(time.perf_counter() - t, 5), "unit": "s per design step"}
        simp.close()
        r3.close()
    ps.close()
    if with_cpu:
        from oracle import oracle as O
        om = O.cartesian_mesh(ns, ns, ns, node_shift=W.interior_node_shift(ns, ns, ns, amp=0.2, seed=SEED))
        O.rcm(om)
        so = O.SimpOracle(om, (3.0, 1e-9, 1.0, 0.0, 0.4, 0.2, 0.5, 1e-3))
        so.dC_drho[:] = dC
        t = time.perf_counter()
        so.step()
        simp_res["cpu_baseline"] = {"value": round(time.perf_counter() - t, 4), "unit": "s per design step",
                                    "cores": 1, "host_nproc": host_cores(), "kind": "port", "sample": "no filter, one step"}
    res["simp"] = simp_res
    return res


def run_ours(a, rank, world, local):
    import torch
    if a.simple_only or a.state_only:
        import simall_gb300 as sg
        sg.build.build()
        sg.load()
        ctx = sg.Context(local)
        leg = ("simple", run_simple) if a.simple_only else ("state", run_state)
        print(json.dumps({leg[0]: leg[1](a, ctx, sg, not a.no_cpu_baseline)}), flush=True)
        return

    import simall_gb300 as sg

    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    ctx = sg.Context(local)
    t0 = time.perf_counter()
    mesh, ps, rhs = build_workload(a.n, ctx)
    setup_s = time.perf_counter() - t0
    dev = torch.device("cuda", local)
    b = torch.from_numpy(rhs).to(dev)
    x = torch.empty_like(b)
    xm = torch.empty_like(b)
    stream = torch.cuda.ExternalStream(ctx.stream)
    s64 = solver_for(sg, ctx, ps, sg.Precision.FP64, a.tol, a.max_iterations, a.check_interval)
    smx = solver_for(sg, ctx, ps, sg.Precision.MIXED, a.tol, a.max_iterations, a.check_interval)

    def barrier():
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()

    def timed(solver, out, steps):
        barrier()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        l0 = ctx.kernel_launches
        e0.record(stream)
        for _ in range(steps):
            solver.solve_into(b, out)
        e1.record(stream)
        e1.synchronize()
        barrier()
        ms = max_over_ranks(e0.elapsed_time(e1) / steps, device=dev)
        return ms, ctx.kernel_launches - l0

    # warm-up: W mixed solves, one FP64 solve
    for _ in range(a.warmup):
        smx.solve_into(b, xm)
    s64.solve_into(b, x)
    clk = ClockSampler(local)
    clk.start()
    mixed_ms, launches = timed(smx, xm, a.steps)
    st_mx = smx.stats
    mx_iters, mx_updates, mx_true = st_mx.iterations, st_mx.reliable_updates, st_mx.true_residual
    mx_engine = int(st_mx.engine)
    fp64_ms, _ = timed(s64, x, a.fp64_steps)
    clocks = clk.stop()
    fp64_iters, fp64_res = s64.stats.iterations, s64.stats.true_residual
    xmn, x64 = xm.double().cpu().numpy(), x.cpu().numpy()
    err_vs_fp64 = float(np.linalg.norm(xmn - x64) / np.linalg.norm(x64))

    # per-matrix setup: new values on an unchanged pattern, which every SIMPLE
    # outer iteration brings (validation, pattern comparison, the Jacobi
    # diagonal and the mixed solver's S A S in FP32 storage), alone and
    # followed by the solve; host clock around synchronous calls
    from simall_gb300._lib import check as lib_check

    def resetup():
        lib_check(smx.L.simall_solver_use_pressure_system(smx.handle, ps.handle), ctx.handle)

    barrier()
    t = time.perf_counter()
    for _ in range(3):
        resetup()
    torch.cuda.synchronize()
    setup_ms = (time.perf_counter() - t) / 3 * 1e3
    barrier()
    t = time.perf_counter()
    for _ in range(a.steps):
        resetup()
        smx.solve_into(b, xm)
    torch.cuda.synchronize()
    with_setup_s = max_over_ranks((time.perf_counter() - t) / a.steps * 1e3, device=dev) / 1e3

    # per-kernel CUDA-event timings (roofline)
    peak, peak_kind = measured_peaks()
    kern = {}
    for name, solver, k in [("mixed_step", smx, 4),
                            ("fp64_spmv", s64, 0), ("fp64_spmv_pap", s64, 1), ("fp64_update", s64, 2),
                            ("fp64_dir", s64, 3)]:
        ms, by = time_kernel(solver, k)
        kern[name] = {"ms": ms, "bytes": by, "gbs": by / ms / 1e6}
    # dominant kernel of the mixed solve: largest time per iteration
    dom = max(("mixed_step",), key=lambda k: kern[k]["ms"])
    traffic = NCU_STEP_DRAM_BYTES_PER_ROW * mesh.n_cells  # natural-order grid: diagonal storage
    rl = {"bound": "hbm", "kernel": dom, "achieved": round(kern[dom]["gbs"], 1), "peak": peak,
          "unit": "GB/s", "frac": round(kern[dom]["gbs"] / peak, 4),
          "traffic": round(traffic) if traffic else None, "algorithmic_bytes": round(kern[dom]["bytes"]),
          "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum, 200^3 capture scaled by rows",
          "peak_source": f"{peak_kind} hbm_gbs"}
    if mx_iters > 0:
        # the same step inside the solve (reliable updates included)
        us = mixed_ms * 1e3 / mx_iters
        gbs = kern[dom]["bytes"] / (us * 1e-3) / 1e6
        rl["in_solve"] = {"us_per_step": round(us, 2), "gbs": round(gbs, 1), "frac": round(gbs / peak, 4)}

    # e2e: C ABI with host buffers (matrix + b in, x out, setup inside); the
    # host arrays are pinned, as the contract's end-to-end step asks
    rp_, ci_ = ps.pattern()
    vals_, _ = ps.download()

    def pinned(arr):
        t = torch.empty(arr.shape, dtype=getattr(torch, str(arr.dtype)), pin_memory=True)
        v = t.numpy()
        v[...] = arr
        return v

    rp, ci, vals = pinned(rp_), pinned(ci_), pinned(vals_)
    rhs = pinned(np.ascontiguousarray(rhs))
    e2e_s, h2d, d2h = None, 0, 0
    if a.e2e_steps > 0:
        e2e_solver = sg.GpuCGSolver(sg.LinearSolverConfig(kind=sg.LinearSolverKind.CG,
                                                          preconditioner=sg.PreconditionerKind.Jacobi,
                                                          tolerance=a.tol, maxIterations=a.max_iterations),
                                    precision=sg.Precision.MIXED, ctx=ctx)
        A = sg.CSRMatrix(rp, ci, vals)
        xh = pinned(np.zeros(len(rhs)))
        e2e_solver.solve(A, rhs, xh)  # warm
        barrier()
        t = time.perf_counter()
        for _ in range(a.e2e_steps):
            e2e_solver.solve(A, rhs, xh)
        e2e_s = round((time.perf_counter() - t) / a.e2e_steps, 6)
        h2d = rp.nbytes + ci.nbytes + vals.nbytes + rhs.nbytes
        d2h = xh.nbytes

    # accuracy: against a tight FP64 solve, and the mixed x's residual recomputed on the host (numpy)
    accuracy = None
    if a.accuracy:
        s_tight = solver_for(sg, ctx, ps, sg.Precision.FP64, 1e-12, a.max_iterations)
        xt = torch.empty_like(b)
        s_tight.solve_into(b, xt)
        xtn = xt.cpu().numpy()

        def err(v):
            return float(np.linalg.norm(v - xtn) / np.linalg.norm(xtn))

        # the loosest tolerance at which the mixed solution is within 1e-9 of
        # the FP64 solve to 1e-12, and both solvers timed there
        at_1e9 = None
        sweep = []
        for tol_k in (1e-10, 3e-11, 1e-11, 3e-12, 1e-12):
            sk = solver_for(sg, ctx, ps, sg.Precision.MIXED, tol_k, a.max_iterations)
            xk = torch.empty_like(b)
            sk.solve_into(b, xk)  # warm: setup and graph capture
            msk, _ = timed(sk, xk, 1)
            ek = err(xk.cpu().numpy())
            sweep.append({"tolerance": tol_k, "mixed_s": round(msk / 1e3, 6), "iterations": int(sk.stats.iterations),
                          "error": ek, "true_residual": float(sk.stats.true_residual)})
            sk.close()
            if ek <= 1e-9:
                s6 = solver_for(sg, ctx, ps, sg.Precision.FP64, tol_k, a.max_iterations)
                x6 = torch.empty_like(b)
                s6.solve_into(b, x6)
                ms6, _ = timed(s6, x6, 1)
                at_1e9 = {"tolerance": tol_k, "mixed": {"value": round(msk / 1e3, 6), "unit": "s",
                                                        "iterations": int(sweep[-1]["iterations"]), "error": ek},
                          "fp64": {"value": round(ms6 / 1e3, 6), "unit": "s", "iterations": int(s6.stats.iterations),
                                   "error": err(x6.cpu().numpy())},
                          "speedup_vs_fp64": round(ms6 / msk, 3)}
                s6.close()
                break
        y = np.add.reduceat(vals * xmn[ci], rp[:-1])
        accuracy = {"reference_solve": f"FP64 Jacobi-PCG to 1e-12 ({int(s_tight.stats.iterations)} it)",
                    "mixed_error": err(xmn), "fp64_error": err(x64),
                    "mixed_host_residual": float(np.linalg.norm(rhs - y) / np.linalg.norm(rhs)),
                    "tolerance_sweep": sweep, "error_1e-9": at_1e9}
        s_tight.close()

    # the reference's own GPU path (cuSPARSE + cuBLAS, its Jacobi on the host) on the same system
    library = None
    if a.library_cg_sample > 0 and rank == 0:
        library = library_cg(rp, ci, vals, rhs, a.tol, a.max_iterations, dev, a.library_cg_sample,
                             int(fp64_iters))
        library["speedup_fp64_vs_device_jacobi"] = round(library["device_jacobi"]["value"] / (fp64_ms / 1e3), 3)
        library["speedup_mixed_vs_device_jacobi"] = round(library["device_jacobi"]["value"] / (mixed_ms / 1e3), 3)
        library["speedup_mixed_vs_as_written"] = round(library["as_written"]["value"] / (mixed_ms / 1e3), 2)

    out = {
        "metric": METRIC, "value": round(mixed_ms / 1e3, 6), "unit": "s", "n_gpus": world, "steps": a.steps,
        "warmup": a.warmup, "ms_per_step": round(mixed_ms, 3), "higher_is_better": False, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32+f64", "data": "synthetic (seeded)",
        "config": {"workload": f"varcoef Poisson {a.n}^3 (k=exp(N(0,1)) harmonic faces, Dirichlet x=0), "
                               f"Jacobi-PCG to {a.tol:g}", "cells": int(mesh.n_cells), "nnz": int(ps.nnz),
                   "seed": SEED, "parallelism": f"replicas x{world}", "l2": "inputs larger than L2 (no flush)",
                   "loop": ({2: "one persistent cooperative launch", 1: "one thread-block cluster"}.get(
                       mx_engine, "device graph loop") if a.check_interval <= 0
                       else f"host poll every {a.check_interval}")},
        "fp64": {"value": round(fp64_ms / 1e3, 6), "unit": "s", "iterations": int(fp64_iters),
                 "true_residual": fp64_res},
        "mixed": {"iterations": int(mx_iters), "reliable_updates": int(mx_updates), "true_residual": mx_true,
                  "rel_diff_vs_fp64": err_vs_fp64},
        "speedup_vs_fp64": round(fp64_ms / mixed_ms, 3),
        "setup_per_matrix": {"ms": round(setup_ms, 3),
                             "what": "new values on the same pattern: validation, pattern check, Jacobi diagonal, "
                                     "S A S in FP32 diagonal storage (paid once per matrix; a SIMPLE outer iteration "
                                     "pays it once per pressure solve)",
                             "mixed_solve_with_setup": {"value": round(with_setup_s, 6), "unit": "s"}},
        "spmv_gbs": {"fp64_csr": round(kern["fp64_spmv"]["gbs"], 1), "fp32_step": round(kern["mixed_step"]["gbs"], 1)},
        "kernels": {k: {"ms": round(v["ms"], 4), "gbs": round(v["gbs"], 1)} for k, v in kern.items()},
        "roofline": rl,
        "e2e": {"value": e2e_s, "unit": "s", "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h)},
        "gpu_launches": int(launches),
        "clocks": clocks,
        "setup_seconds": round(setup_s, 2),
    }
    if accuracy:
        out["accuracy"] = accuracy
    if library:
        out["library_cg"] = library
    if a.batched_systems > 0:
        out["batched"] = run_batched(a, ctx, sg, rank, world, rank == 0 and world == 1 and not a.no_cpu_baseline)
    if a.adjoint_n > 0:
        out["adjoint"] = run_adjoint(a, ctx, sg)
    if a.poisson_n > 0:
        out["poisson3d"] = run_poisson3d(a, ctx, sg)
    if a.precond_n > 0:
        out["preconditioners"] = run_preconditioners(a, ctx, sg, rank == 0 and world == 1 and not a.no_cpu_baseline)
    if a.poisson_n > 0:
        out["pressure_step"] = run_pressure_step(a, ctx, sg, rank == 0 and world == 1 and not a.no_cpu_baseline)
    if not a.no_cavity:
        out["cavity"] = run_cavity(a, ctx, sg, rank == 0 and world == 1 and not a.no_cpu_baseline)
    if a.simple_iterations > 0:
        out["simple"] = run_simple(a, ctx, sg, rank == 0 and world == 1 and not a.no_cpu_baseline)
    if a.poisson_n > 0:
        out["state"] = run_state(a, ctx, sg, rank == 0 and world == 1 and not a.no_cpu_baseline)
    if rank == 0 and world == 1 and not a.no_cpu_baseline:
        per_it, k, kind = cpu_cg_sample(rp, ci, vals, rhs, a.cpu_seconds, use_ref=True)
        ref_iters = reference_iterations(a.n)
        iters = ref_iters or int(fp64_iters)
        out["cpu_baseline"] = {"value": round(per_it * iters, 3), "unit": "s", "cores": 1,
                               "host_nproc": host_cores(), "kind": kind,
                               "sample": f"{k} FP64 Jacobi-CG iterations of this {a.n}^3 system on 1 host core "
                                         f"({per_it * 1e3:.1f} ms/iteration), scaled to the {iters} iterations "
                                         + ("of the reference's own full solve of it" if ref_iters else
                                            "of the device FP64 solve (no reference count at this size)")}
    if rank == 0:
        print(json.dumps(out), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


def run_reference(a, rank, world):
    """The reference CG (CGSolver::solve, Jacobi, 1 core -- it is serial) on the
    host: the compiled reference if present, else the oracle's bit-identical
    restatement.  Each step times a bounded number of iterations of the same
    system; the solve time is that per-iteration time times the reference's own
    iteration count: from its full solve of the 256^3 system
    (tests/golden/varcoef_256_cg.npz), or, for sides up to 64, from a full CG
    run here.  For other sizes no solve time is reported (value null), only the
    per-iteration time."""
    if rank != 0:
        return
    from oracle import oracle as O
    from simall_gb300 import workloads as W

    # input system: the oracle's own mesh, sparsity and assembly
    m = O.cartesian_mesh(a.n, a.n, a.n)
    rng = np.random.default_rng(SEED + 2)
    k = W.portable_exp(rng.standard_normal(m.nC))
    rhs = rng.standard_normal(m.nC)
    rp, ci = O.build_sparsity(m)
    v, _, _ = O.assemble(m, rp, ci, [1], 1.0, 1.0 / k, np.zeros(m.nF))
    del m
    iters = reference_iterations(a.n)
    count_source = "the reference's own full solve of this system" if iters else None
    if iters is None and a.n <= 64:
        if O.RefLib.available():
            _, iters, _, _ = O.RefLib().cg(rp, ci, v, rhs, 0, a.tol, a.max_iterations)
        else:
            _, iters, _ = O.cg(rp, ci, v, rhs, 0, a.tol, a.max_iterations)
        count_source = "a full CG run of this system here"
    per = []
    kind = "port"
    for i in range(a.warmup + a.steps):
        t, kk, kind = cpu_cg_sample(rp, ci, v, rhs, a.cpu_seconds / 2, use_ref=True)
        if i >= a.warmup:
            per.append(t)
    per_it = float(np.mean(per))
    val = round(per_it * iters, 3) if iters else None
    sample = (f"{kk} FP64 Jacobi-CG iterations per step on 1 host core ({per_it * 1e3:.1f} ms/iteration), "
              + (f"scaled to the {iters} iterations of {count_source}" if iters
                 else "no reference iteration count for this size: per-iteration time only"))
    print(json.dumps({"impl": "reference", "metric": METRIC, "value": val, "unit": "s", "n_gpus": world,
                      "steps": a.steps, "warmup": a.warmup,
                      "ms_per_step": round(per_it * iters * 1e3, 1) if iters else None,
                      "ms_per_iteration": round(per_it * 1e3, 3), "reference_iterations": iters,
                      "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
                      "data": "synthetic (seeded)",
                      "config": {"workload": f"varcoef Poisson {a.n}^3, Jacobi-PCG to {a.tol:g}", "seed": SEED},
                      "cpu_baseline": {"value": val, "unit": "s", "cores": 1, "host_nproc": host_cores(),
                                       "kind": kind, "sample": sample},
                      "e2e": {"value": val, "unit": "s", "h2d_bytes_per_step": 0,
                              "d2h_bytes_per_step": 0}}), flush=True)


def main():
    a = parse()
    rank, world, local = rank_info()
    if a.impl == "reference":
        run_reference(a, rank, world)
    else:
        run_ours(a, rank, world, local)


if __name__ == "__main__":
    main()
