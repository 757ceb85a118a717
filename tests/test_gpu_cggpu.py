"""gpu::CgGpu's conventions on the device (SIMALL_SEMANTICS_CGGPU): the
library's FP64 PCG with x0 honoured, the <= / relativeOrders stop test, None
= no preconditioner, the ILU0 -> Jacobi fall-back and the |p.q| < 1e-300 exit,
against the oracle's restatement of CgGpu::set_matrix + solve
(src/gpu/CgGpu.cpp:35-238), which tests/golden/cggpu_cases.npz pins to the
reference bit for bit.  Parity bar: the oracle's iteration count within one
(equal where it is 0), the same converged flag and preconditioner, x within
1e-10.  Also a chain of warm-started solves over the reference SIMPLE loop's
successive pressure systems (a corrector sequence that starts each solve
from the previous solution), and the header-only C++ CgGpu."""
import os
import subprocess

import numpy as np
import pytest

from helpers import cggpu_cases, rel

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLD = os.path.join(ROOT, "tests", "golden")
NAMES = ["jacobi_cold", "jacobi_warm", "ilu0_warm", "none_cold", "relative_orders", "tolerance_first", "x0_exact",
         "b_zero_x0_zero", "b_zero_x0_nonzero", "max_iterations_5", "max_iterations_0", "ilu0_zero_pivot_fallback",
         "breakdown"]


def _device(sg, ctx, rp, ci, v, b, x0, pc, tol, mi, ro):
    cg = sg.CgGpu(sg.GpuSolverConfig(sg.GpuPreconditioner(pc), tol, mi, ro), ctx=ctx)
    cg.set_matrix(np.asarray(rp, np.int32), np.asarray(ci, np.int32), np.asarray(v, np.float64))
    x = np.array(x0, np.float64, copy=True)
    st = cg.solve(np.asarray(b, np.float64), x)
    out = (x, st, int(cg.config().preconditioner), cg.last_residual(), int(cg.stats.status))
    cg.close()
    return out


@pytest.mark.parametrize("name", NAMES)
def test_cggpu_case_matches_oracle(sg, ctx, oracle, name):
    case = {c[0]: c for c in cggpu_cases(oracle)}[name]
    _, rp, ci, v, b, x0, pc, tol, mi, ro = case
    xo, so = oracle.cggpu(rp, ci, v, b, x0, pc, tol, mi, ro)
    x, st, pc_after, last, status = _device(sg, ctx, rp, ci, v, b, x0, pc, tol, mi, ro)
    assert pc_after == so["precond_after"]
    assert st.converged == so["converged"]
    if so["iterations"] == 0:
        assert st.iterations == 0
    else:
        assert abs(st.iterations - so["iterations"]) <= 1, (st.iterations, so["iterations"])
    scale = max(np.linalg.norm(xo), np.linalg.norm(x0), 1e-300)
    assert np.linalg.norm(x - xo) <= 1e-10 * scale
    assert abs(st.initialResidual - so["initial_residual"]) <= 1e-12 * max(so["initial_residual"], 1e-300) + 1e-300
    if name == "breakdown":
        assert status == 9 and st.finalResidual == 0.0 and last == 0.0  # SIMALL_ERR_BREAKDOWN, stats left at 0
    elif so["iterations"] == 0 or not so["converged"]:
        assert st.finalResidual == pytest.approx(so["final_residual"], rel=1e-9, abs=1e-300)
    else:  # converged: the device's residual meets the stop test it ended on
        bref = np.linalg.norm(b) or 1.0
        assert st.finalResidual / bref <= tol or (ro > 0 and st.finalResidual <= st.initialResidual * 10.0 ** -ro)
    assert last == st.finalResidual


def test_cggpu_warm_started_corrector_chain(sg, ctx, oracle):
    """The reference SIMPLE loop's six successive 16x16 cavity pressure
    systems (tests/golden/cavity_simple_16.npz), each solved from the previous
    solve's solution, as PISO/PIMPLE correctors warm-start CgGpu: device and
    oracle run the same chain."""
    c = np.load(os.path.join(GOLD, "cavity_simple_16.npz"))
    rp, ci = c["rowPtr"], c["colIdx"]
    n = len(rp) - 1
    cg = sg.CgGpu(sg.GpuSolverConfig(sg.GpuPreconditioner.Jacobi, 1e-10, 2000, 0.0), ctx=ctx)
    x = np.zeros(n)
    xo = np.zeros(n)
    for k in range(c["values"].shape[0]):
        v, b = c["values"][k], c["rhs"][k]
        cg.set_matrix(rp, ci, v)
        st = cg.solve(b, x)
        xo, so = oracle.cggpu(rp, ci, v, b, xo, 1, 1e-10, 2000, 0.0)
        assert abs(st.iterations - so["iterations"]) <= 1, (k, st.iterations, so["iterations"])
        assert st.converged and so["converged"]
        assert rel(x, xo) <= 1e-10, k
        assert st.initialResidual == pytest.approx(so["initial_residual"], rel=1e-9)
    cg.close()


def test_cggpu_cpp_header(sg, tmp_path):
    lib = sg._lib.lib_path()
    exe = str(tmp_path / "cggpu_main")
    subprocess.run(["g++", "-std=c++20", "-O1", f"-I{ROOT}/include", os.path.join(ROOT, "tests", "cpp", "cggpu_main.cpp"),
                    "-o", exe, lib, f"-Wl,-rpath,{os.path.dirname(lib)}"], check=True)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.count(" ok") == 4


def test_cggpu_rejects_unsupported(sg, ctx):
    from simall_gb300 import _lib
    import ctypes as C

    c = _lib.SolverConfig()
    ctx.L.simall_solver_config_default(C.byref(c))
    c.semantics = 1
    c.precision = 1  # mixed precision has no CgGpu counterpart
    h = C.c_void_p()
    assert ctx.L.simall_solver_create(ctx.handle, C.byref(c), C.byref(h)) == 11  # SIMALL_ERR_UNSUPPORTED
