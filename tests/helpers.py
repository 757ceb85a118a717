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
