"""SIMP topology optimisation on the device (SimpTopology,
src/optimization/SimpTopology.cpp:18-227) against the reference's steps
(tests/golden/simp_7x6x5_rcm.npz), and a design loop driven by this
library's adjoint: thermal compliance falls and the volume constraint
holds."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _close(a, b, tol):
    return np.max(np.abs(a - b)) <= tol * max(1.0, np.max(np.abs(b)))


@pytest.mark.parametrize("tag", ["r0", "r3"])
def test_simp_steps_match_reference(sg, ctx, tag):
    from simall_gb300 import workloads as W

    g = np.load(os.path.join(GOLD, "simp_7x6x5_rcm.npz"))
    dims = tuple(int(v) for v in g["dims"])
    m = sg.cartesian(*dims, node_shift=W.interior_node_shift(*dims, amp=0.2, seed=int(g["seed"])))
    sg.rcm(m)
    ps = sg.PressureSystem(m, [(z, 1) for z in range(1, 7)], ctx=ctx)
    ps.setup_field_loops()
    reg = sg.DeviceFieldRegistry(ctx)
    c = g[f"{tag}_cfg"]
    simp = sg.GpuSimpTopology(ps, reg, sg.SimpConfig(*[float(v) for v in c]))
    ch = []
    for k in range(3):
        reg.upload("dC_drho", g["dC"][k])
        ch.append(simp.step())
    # pow() and the filter's CG differ from the host's in the last bits
    assert _close(np.array(ch), g[f"{tag}_change"], 1e-9)
    assert _close(reg.download("rho"), g[f"{tag}_rho"], 1e-9)
    assert _close(reg.download("rhoTilde"), g[f"{tag}_rhoTilde"], 1e-9)
    assert _close(reg.download("K_simp"), g[f"{tag}_K"], 1e-9)
    assert _close(reg.download("dC_drhoTilde"), g[f"{tag}_dCt"], 1e-9)
    simp.close()
    reg.close()
    ps.close()


def test_compliance_design_loop_with_the_adjoint(sg, ctx):
    """Heat conduction on a 32x32 plate (uniform source, T = 0 on the left
    edge): dJ/dK from simall_adjoint_face_conductance, chain rule to the
    density, SIMP steps; compliance decreases and the volume stays at 40%."""
    from simall_gb300.topology import compliance_sensitivity

    N = 32
    m = sg.cartesian(N, N, 1, 1.0, 1.0, 1.0 / N)
    ps = sg.PressureSystem(m, [(1, int(sg.BCType.PressureOutlet))] + [(z, 1) for z in range(2, 7)], ctx=ctx)
    ps.setup_field_loops()
    reg = sg.DeviceFieldRegistry(ctx)
    cfg = sg.SimpConfig(penalty=3.0, K_min=1e-3, K_max=1.0, volumeFraction=0.4, move=0.2)
    simp = sg.GpuSimpTopology(ps, reg, cfg)
    solver = sg.GpuCGSolver(sg.LinearSolverConfig(kind=sg.LinearSolverKind.CG,
                                                  preconditioner=sg.PreconditionerKind.Jacobi, tolerance=1e-10,
                                                  maxIterations=20000), ctx=ctx)
    dirichlet = (m.neighbor == np.iinfo(np.uint64).max) & (m.boundary_zone == 1)
    q = np.full(m.n_cells, 1.0) * m.volume
    Js = []
    for _ in range(8):
        # without the filter, step() takes rhoTilde = rho before it moves rho:
        # the sensitivity belongs to the current rho
        rt = reg.download("rho")
        K = cfg.K_min + (cfg.K_max - cfg.K_min) * rt ** cfg.penalty
        J, dK = compliance_sensitivity(ps, solver, m, K, q, dirichlet)
        Js.append(J)
        reg.upload("dC_drho", dK * cfg.penalty * (cfg.K_max - cfg.K_min) * rt ** (cfg.penalty - 1.0))
        simp.step()
        vol = float(reg.download("rho") @ m.volume)
        assert abs(vol - cfg.volumeFraction * m.volume.sum()) <= 1e-6 * m.volume.sum()
    assert np.count_nonzero(np.diff(Js) > 0) <= 1 and Js[-1] < 0.7 * Js[0], Js
    for o in (simp, solver, reg, ps):
        o.close()
