"""Object lifetimes across the C ABI: a process that exits with live
contexts, solvers and pressure systems (and PyTorch CUDA state) must exit
cleanly; destroying a context releases its children first."""
import os
import subprocess
import sys

import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

SCRIPT = r"""
import sys
sys.path.insert(0, {root!r})
import numpy as np
import torch
import simall_gb300 as sg
from simall_gb300 import workloads as W
ctx = sg.Context(0)
m = sg.cartesian(6, 6, 6)
ps = sg.PressureSystem(m, W.ALL_WALLS, ctx=ctx)
ps.assemble(1.0, np.ones(m.n_cells), np.zeros(m.n_faces))
s = sg.GpuCGSolver(sg.LinearSolverConfig(kind=sg.LinearSolverKind.CG, preconditioner=sg.PreconditionerKind.Jacobi),
                   ctx=ctx)
x = ps.solve(s)
t = torch.ones(16, device="cuda")
s2 = sg.GpuCGSolver(ctx=sg.default_context())
print("alive", s.stats.iterations)
"""


def test_exit_with_live_objects_is_clean():
    r = subprocess.run([sys.executable, "-c", SCRIPT.format(root=ROOT)], capture_output=True, text=True,
                       timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "alive" in r.stdout


def test_context_close_releases_children(sg):
    ctx = sg.Context(0)
    s = sg.GpuCGSolver(ctx=ctx)
    m = sg.cartesian(3, 3, 3)
    ps = sg.PressureSystem(m, [], ctx=ctx)
    ctx.close()
    assert s.handle is None and ps.handle is None
