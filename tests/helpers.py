"""Shared builders for the parity tests: the same seeded system from the
product (device) and from the oracle (CPU restatement)."""
from __future__ import annotations

import numpy as np


def oracle_system(O, n, seed=7, amp=0.2, renumber=True, pressure_zones=(), aP=None, phi=None, dims=None):
    """Distorted box, optional RCM, assembled by the oracle.
    Returns (mesh, rowPtr, colIdx, values, rhs, aP, phi)."""
    from simall_gb300 import workloads as W

    nx, ny, nz = dims or (n, n, n)
    shift = W.interior_node_shift(nx, ny, nz, amp=amp, seed=seed) if amp else None
    m = O.cartesian_mesh(nx, ny, nz, node_shift=shift)
    if renumber:
        O.rcm(m)
    rng = np.random.default_rng(seed + 100)
    if aP is None:
        aP = rng.uniform(0.5, 2.0, m.nC)
    if phi is None:
        phi = rng.standard_normal(m.nF)
        phi[m.neighbor < 0] = 0.0
    rp, ci = O.build_sparsity(m)
    v, rhs, _ = O.assemble(m, rp, ci, list(pressure_zones), 1.0, aP, phi)
    return m, rp, ci, v, rhs, aP, phi


def product_mesh(sg, n, seed=7, amp=0.2, renumber=True, dims=None):
    from simall_gb300 import workloads as W

    nx, ny, nz = dims or (n, n, n)
    shift = W.interior_node_shift(nx, ny, nz, amp=amp, seed=seed) if amp else None
    m = sg.cartesian(nx, ny, nz, node_shift=shift)
    if renumber:
        sg.rcm(m)
    return m


def rel(a, b):
    nb = np.linalg.norm(b)
    return np.linalg.norm(a - b) / (nb if nb > 0 else 1.0)


def bits_equal(a, b):
    a = np.ascontiguousarray(a, np.float64)
    b = np.ascontiguousarray(b, np.float64)
    return a.shape == b.shape and np.array_equal(a.view(np.uint64), b.view(np.uint64))


def tridiag(n, lo=-1.0, d=4.0, hi=-1.0):
    rp = [0]
    ci = []
    va = []
    for i in range(n):
        if i > 0:
            ci.append(i - 1)
            va.append(lo)
        ci.append(i)
        va.append(d)
        if i + 1 < n:
            ci.append(i + 1)
            va.append(hi)
        rp.append(len(ci))
    return np.array(rp, np.int32), np.array(ci, np.int32), np.array(va, np.float64)


def digest(a) -> str:
    import hashlib

    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def x_summary_error(x, fx, prefix):
    """Largest relative deviation of x from a solution summary stored by
    tests/golden/make_golden.py (_x_summary): the strided sample, ||x||_2 and
    x.w for the seeded w ~ N(0,1).  For x.w the deviation is taken relative to
    ||x||_2: (x - x_ref).w ~ N(0, ||x - x_ref||^2) for an independent w, so it
    stays near ||x - x_ref|| / ||x|| (an eighth of the bound leaves 8 sigma)."""
    stride = int(fx[prefix + "_x_stride"])
    ref = fx[prefix + "_x_sample"]
    e_sample = rel(x[::stride], ref)
    xn = float(fx[prefix + "_x_norm"])
    e_norm = abs(float(np.linalg.norm(x)) - xn) / xn
    w = np.random.default_rng(int(fx[prefix + "_w_seed"])).standard_normal(len(x))
    e_dot = abs(float(x @ w) - float(fx[prefix + "_x_dot_w"])) / xn / 8.0
    return max(e_sample, e_norm, e_dot)


def cggpu_cases(O):
    """gpu::CgGpu cases shared by the oracle-vs-reference, golden and device
    tests: (name, rowPtr, colIdx, values, b, x0, precond, tol, maxIt,
    relativeOrders); precond 0 None, 1 Jacobi, 2 ILU0."""
    m, rp, ci, v, b, _, _ = oracle_system(O, 8, seed=31)
    n = len(b)
    rng = np.random.default_rng(31)
    x0 = rng.standard_normal(n)
    xs, _, _ = O.cg(rp, ci, v, b, 0, 1e-15, 5000)
    # unpreconditioned CG wants a well-conditioned matrix: on the pinned
    # system above (one row scaled by 1e6) rounding alone moves x by 1e-8
    trp0, tci0, tv0 = tridiag(60, -1.0, 3.0, -1.0)
    tb0 = np.random.default_rng(33).standard_normal(60)
    cases = [
        ("jacobi_cold", rp, ci, v, b, np.zeros(n), 1, 1e-8, 1000, 0.0),
        ("jacobi_warm", rp, ci, v, b, x0, 1, 1e-8, 1000, 0.0),
        ("ilu0_warm", rp, ci, v, b, x0, 2, 1e-8, 1000, 0.0),
        ("none_cold", trp0, tci0, tv0, tb0, np.zeros(60), 0, 1e-10, 1000, 0.0),
        ("relative_orders", rp, ci, v, b, x0, 1, 1e-12, 1000, 3.0),
        ("tolerance_first", rp, ci, v, b, np.zeros(n), 2, 1e-3, 1000, 9.0),
        ("x0_exact", rp, ci, v, b, xs, 1, 1e-8, 1000, 0.0),
        ("b_zero_x0_zero", rp, ci, v, np.zeros(n), np.zeros(n), 1, 1e-8, 1000, 0.0),
        ("b_zero_x0_nonzero", rp, ci, v, np.zeros(n), x0, 2, 1e-8, 1000, 0.0),
        ("max_iterations_5", rp, ci, v, b, x0, 1, 1e-8, 5, 0.0),
        ("max_iterations_0", rp, ci, v, b, x0, 1, 1e-8, 0, 0.0),
    ]
    # ILU0 whose factor meets a zero pivot (a_00 = 0, eliminated against by
    # row 1): CgGpu falls back to Jacobi, which divides row 0 by 1
    trp, tci, tv = tridiag(40, -1.0, 4.0, -1.0)
    tv = tv.copy()
    tv[0] = 0.0
    tb = np.random.default_rng(32).standard_normal(40)
    cases.append(("ilu0_zero_pivot_fallback", trp, tci, tv, tb, np.zeros(40), 2, 1e-8, 1000, 0.0))
    # p.q = 0 at the first iteration: an all-zero matrix (diagonal stored)
    zrp, zci, zv = tridiag(16, 0.0, 0.0, 0.0)
    cases.append(("breakdown", zrp, zci, zv, np.ones(16), np.zeros(16), 1, 1e-8, 100, 0.0))
    return cases
