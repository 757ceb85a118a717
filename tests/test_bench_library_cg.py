"""bench.py's library comparator -- the reference's gpu::CgGpu call sequence
(src/gpu/CgGpu.cpp:181-219) through torch's CSR SpMV and BLAS-1 -- on the
CPU against the oracle's restatement of CgGpu::solve with Jacobi."""
import numpy as np
import torch

import bench
from helpers import oracle_system


def test_library_cg_follows_cggpu(oracle):
    _, rp, ci, v, b, _, _ = oracle_system(oracle, 8, seed=31)
    xo, so = oracle.cggpu(rp, ci, v, b, None, 1, 1e-8, 1000)
    out = bench.library_cg(rp, ci, v, b, 1e-8, 1000, torch.device("cpu"), 3, None)
    dj = out["device_jacobi"]
    # same algorithm and stop test; the summation order of the dot products
    # differs (torch against the oracle's loop), so the count may move by one
    assert abs(dj["iterations"] - so["iterations"]) <= 1
    assert dj["iterated_residual"] <= 1e-8
    assert dj["true_residual"] < 1e-7
    assert out["as_written"]["sample"].startswith("3 iterations")
    assert out["as_written"]["value"] > 0.0


def test_library_cg_zero_rhs(oracle):
    _, rp, ci, v, b, _, _ = oracle_system(oracle, 6, seed=3)
    out = bench.library_cg(rp, ci, v, np.zeros_like(b), 1e-8, 100, torch.device("cpu"), 2, None)
    assert out["device_jacobi"]["iterations"] == 0
