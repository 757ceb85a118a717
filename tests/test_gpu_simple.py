"""The SIMPLE outer iteration with every field on the device
(simall_simple_*, SimpleAlgorithm::iterate / advance_time_step) against the
reference's own runs from rest (tests/golden/simple_*.npz) and against the
oracle on a larger 3-D channel: U, p, phi and the residuals agree to the
solvers' rounding, every linear solve takes the reference's iteration count
within one."""
import json
import os

import numpy as np
import pytest

from helpers import rel

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _solver(sg, ctx, cfg):
    kind, pc, tol, maxit, restart = cfg
    c = sg.LinearSolverConfig(kind=sg.LinearSolverKind(kind), preconditioner=sg.PreconditionerKind(pc),
                              tolerance=tol, maxIterations=maxit, restart=restart)
    return sg.make_linear_solver(c, ctx=ctx)


def _algorithm(sg, ctx, m, bcs, kw):
    mom = _solver(sg, ctx, kw["mom_cfg"])
    pres = _solver(sg, ctx, kw["p_cfg"])
    opts = sg.SimpleOptions(urfU=kw.get("urfU", 0.7), urfP=kw.get("urfP", 0.3), rho=kw.get("rho", 1.0),
                            mu=kw.get("mu", 1e-3), dt=kw.get("dt", 0.0), bdf2=kw.get("bdf2", False),
                            simplec=kw.get("simplec", False))
    return sg.GpuSimpleAlgorithm(m, bcs, mom, pres, opts, ctx=ctx)


def _run(alg, kw, n_outer, n_inner):
    res, its = [], []
    for _ in range(n_outer):
        r = alg.advance_time_step(n_inner) if kw.get("dt", 0.0) > 0 else alg.iterate()
        res.append(list(r.mom) + [r.cont])
        its.append(r.iterations)
    return np.array(res), np.array(its)


@pytest.mark.parametrize("name", ["simple_cavity_64_gmres_ilu.npz", "simple_channel_8x6x5_simplec.npz",
                                  "simple_cavity_12_bdf2.npz", "simple_periodic_couette_8x6x4.npz"])
def test_simple_runs_against_reference(sg, ctx, name):
    from simall_gb300 import workloads as W

    g = np.load(os.path.join(GOLD, name))
    dims = tuple(int(v) for v in g["dims"])
    amp = float(g["amp"])
    m = sg.cartesian(*dims, node_shift=W.interior_node_shift(*dims, amp=amp, seed=31) if amp else None)
    if bool(g["renumber"]):
        sg.rcm(m)
    bcs = [(int(z), int(t), tuple(v)) for z, t, v in zip(g["bc_zone"], g["bc_type"], g["bc_vec"])]
    kw = json.loads(str(g["options"]))
    alg = _algorithm(sg, ctx, m, bcs, kw)
    res, its = _run(alg, kw, int(g["n_outer"]), int(g["n_inner"]))
    U, p, phi = alg.fields()
    # the last outer call's solve counts (advance_time_step returns its last iterate)
    per_call = g["iters"].reshape(int(g["n_outer"]), -1, 4)[:, -1, :]
    assert np.all(np.abs(its - per_call) <= 1), (its, per_call)
    assert rel(U, g["U"]) <= 1e-8 and rel(p, g["p"]) <= 1e-8 and rel(phi, g["phi"]) <= 1e-8
    # continuity residuals match closely; momentum residuals are solver round-off sized
    assert np.all(np.abs(res[:, 3] - g["res"][:, 3]) <= 1e-8 * np.abs(g["res"][:, 3]))
    alg.close()


def test_simple_channel_against_oracle(sg, ctx, oracle):
    """A 24x20x16 distorted, RCM-renumbered channel (inlet, outlet, walls,
    symmetry), BiCGSTAB + Jacobi momentum and CG + ILU(0) pressure, SIMPLE."""
    from simall_gb300 import workloads as W

    dims = (24, 20, 16)
    bcs = [(1, 4, (1.0, 0.1, 0.0)), (2, 7), (3, 1), (4, 1), (5, 9), (6, 0)]
    kw = dict(mu=0.05, mom_cfg=(1, 0, 1e-9, 300, 30), p_cfg=(2, 1, 1e-9, 2000, 30))
    sh = W.interior_node_shift(*dims, amp=0.2, seed=41)
    m = sg.cartesian(*dims, node_shift=sh)
    sg.rcm(m)
    om = oracle.cartesian_mesh(*dims, node_shift=sh)
    oracle.rcm(om)
    so = oracle.SimpleOracle(om, bcs, **kw)
    alg = _algorithm(sg, ctx, m, bcs, kw)
    for _ in range(4):
        ro, io = so.iterate()
        r = alg.iterate()
        assert np.all(np.abs(np.array(r.iterations) - io) <= 1), (r.iterations, io)
        assert abs(r.cont - ro[3]) <= 1e-8 * ro[3]
    U, p, phi = alg.fields()
    assert rel(U, so.U) <= 1e-8 and rel(p, so.p) <= 1e-8 and rel(phi, so.phi) <= 1e-8
    alg.close()


@pytest.mark.parametrize("name", ["piso_cavity_12.npz", "pimple_channel_8x6x5.npz"])
def test_piso_pimple_against_reference(sg, ctx, name):
    """PisoAlgorithm / PimpleAlgorithm time steps (advance_time_step(1)) on the
    device against the reference's own runs: fields within 1e-8, the
    residuals of every step, and PIMPLE's early-exit index step by step."""
    from simall_gb300 import workloads as W

    g = np.load(os.path.join(GOLD, name))
    dims = tuple(int(v) for v in g["dims"])
    amp = float(g["amp"])
    m = sg.cartesian(*dims, node_shift=W.interior_node_shift(*dims, amp=amp, seed=61) if amp else None)
    if bool(g["renumber"]):
        sg.rcm(m)
    bcs = [(int(z), int(t), tuple(v)) for z, t, v in zip(g["bc_zone"], g["bc_type"], g["bc_vec"])]
    kw = json.loads(str(g["options"]))
    loops = [int(v) for v in g["loops"]]
    if int(g["variant"]) == 1:
        opts = sg.PisoOptions(nCorrectors=loops[1], nNonOrthCorr=loops[2], mu=kw["mu"], dt=kw["dt"])
    else:
        opts = sg.PimpleOptions(nOuterCorrectors=loops[0], nCorrectors=loops[1], nNonOrthCorr=loops[2],
                                momentumPredictor=bool(loops[3]), urfU=kw["urfU"], urfP=kw["urfP"], tolU=kw["tol_u"],
                                tolP=kw["tol_p"], mu=kw["mu"], dt=kw["dt"])
    mom = _solver(sg, ctx, (0, 0, 1e-9, 200, 30))
    pres = _solver(sg, ctx, (2, 0, 1e-9, 1000, 30))
    alg = sg.GpuSimpleAlgorithm(m, bcs, mom, pres, opts, ctx=ctx)
    res, outer = [], []
    for _ in range(int(g["steps"])):
        r = alg.advance_time_step(1)
        res.append(list(r.mom) + [r.cont])
        outer.append(r.outer)
    U, p, phi = alg.fields()
    assert outer == [int(v) for v in g["last_outer"]]
    assert rel(U, g["U"]) <= 1e-8 and rel(p, g["p"]) <= 1e-8 and rel(phi, g["phi"]) <= 1e-8
    res = np.array(res)
    # the last corrector's continuity residual is ~1e-11 here: what is left of
    # the solvers' rounding, so it agrees to 1e-6 relative (1e-16 absolute)
    assert np.all(np.abs(res[:, 3] - g["res"][:, 3]) <= 1e-6 * np.abs(g["res"][:, 3]) + 1e-16)
    alg.close()
