"""The AMG hierarchy the library builds on the host (csrc/amg_host.cpp: the
reference's Ruge-Stueben setup with the C/F selection on a lazy heap) against
the oracle's literal restatement (its O(n^2) selection rescans, as the
reference's AMGPreconditioner::coarsen does): the same levels and a digest
of every operator, prolongation, restriction and the coarsest LU, bit for
bit.  Host logic only; no GPU is needed."""
import ctypes as C

import numpy as np
import pytest

from helpers import oracle_system, tridiag


@pytest.fixture(scope="module")
def lib():
    import simall_gb300

    simall_gb300.build.build()
    return simall_gb300.load()


def _library_digest(L, rp, ci, v):
    rp = np.ascontiguousarray(rp, np.int32)
    ci = np.ascontiguousarray(ci, np.int32)
    v = np.ascontiguousarray(v, np.float64)
    nlev = C.c_int(0)
    rows = np.zeros(16, np.int32)
    dig = C.c_uint64(0)
    st = L.simall_amg_hierarchy_digest(len(rp) - 1, rp.ctypes.data, ci.ctypes.data, v.ctypes.data, C.byref(nlev),
                                       rows.ctypes.data, 16, C.byref(dig))
    assert st == 0
    return nlev.value, [int(r) for r in rows[:nlev.value]], int(dig.value)


@pytest.mark.parametrize("dims", [(6, 5, 4), (12, 11, 10), (20, 20, 1), (16, 16, 16), (128, 128, 1), (32, 32, 32)])
def test_hierarchy_matches_oracle(lib, oracle, dims):
    m, rp, ci, v, rhs, aP, phi = oracle_system(oracle, 0, seed=3, dims=dims)
    nlev, rows, dig = _library_digest(lib, rp, ci, v)
    onlev, odig = oracle.amg_digest(rp, ci, v)
    _, levels, _ = oracle.amg_apply(rp, ci, v)
    assert (nlev, rows) == (onlev, [n for n, _ in levels])
    assert dig == odig


def test_hierarchy_edge_cases(lib, oracle):
    """A single level (n <= 32), zero diagonals, a non-symmetric matrix."""
    cases = [tridiag(20, -1.0, 2.0, -1.0), tridiag(200, -6.0, 7.0, -1.0)]
    rp, ci, va = tridiag(120, -1.0, 2.5, -1.2)
    va = va.copy()
    for i in (0, 50, 99):
        va[rp[i] + (0 if i == 0 else 1)] = 0.0
    cases.append((rp, ci, va))
    for rp, ci, va in cases:
        nlev, rows, dig = _library_digest(lib, rp, ci, va)
        assert (nlev, dig) == oracle.amg_digest(rp, ci, va)


def test_rejects_bad_arguments(lib):
    nlev = C.c_int(0)
    dig = C.c_uint64(0)
    assert lib.simall_amg_hierarchy_digest(0, None, None, None, C.byref(nlev), None, 0, C.byref(dig)) != 0
