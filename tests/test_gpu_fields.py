"""The face loops around the pressure solve on the device --
compute_face_fluxes, the least-squares gradient, correct_fields -- against
the reference's bytes (tests/golden/field_loops_7x6x5_rcm.npz), with host and
device arrays; and one device-resident pressure step."""
import os

import numpy as np
import pytest

from helpers import bits_equal

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _system(sg, ctx):
    from simall_gb300 import workloads as W

    g = np.load(os.path.join(GOLD, "field_loops_7x6x5_rcm.npz"))
    dims = tuple(int(v) for v in g["dims"])
    m = sg.cartesian(*dims, node_shift=W.interior_node_shift(*dims, amp=0.2, seed=int(g["seed"])))
    sg.rcm(m)
    bcs = [(int(z), int(t)) for z, t in zip(g["bc_zone"], g["bc_type"])]
    ps = sg.PressureSystem(m, bcs, ctx=ctx)
    vel = [(int(z), tuple(v)) for z, t, v in zip(g["bc_zone"], g["bc_type"], g["bc_vec"]) if int(t) in (2, 4)]
    ps.setup_field_loops(vel)
    return g, ps


def test_field_loops_host_arrays(sg, ctx):
    g, ps = _system(sg, ctx)
    phi = ps.face_fluxes(float(g["rho"]), [np.ascontiguousarray(u) for u in g["U"]])
    assert bits_equal(phi, g["phi"])
    assert bits_equal(ps.lsq_gradient(np.ascontiguousarray(g["f"])), g["grad"])
    p = g["p0"].copy()
    U = [np.ascontiguousarray(u).copy() for u in g["U"]]
    ph = g["phi"].copy()
    ps.correct_fields(float(g["rho"]), float(g["urfP"]), np.ascontiguousarray(g["aP"]),
                      np.ascontiguousarray(g["pPrime"]), p, U, ph)
    assert bits_equal(p, g["p1"]) and bits_equal(np.array(U), g["U1"]) and bits_equal(ph, g["phi1"])
    ps.close()


def test_field_loops_device_arrays(sg, ctx):
    torch = pytest.importorskip("torch")
    g, ps = _system(sg, ctx)
    dev = torch.device("cuda:0")
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a).copy()).to(dev)  # noqa: E731
    U = [t(u) for u in g["U"]]
    phi = torch.empty(len(g["phi"]), dtype=torch.float64, device=dev)
    ps.face_fluxes(float(g["rho"]), U, phi)
    ctx.synchronize()
    assert bits_equal(phi.cpu().numpy(), g["phi"])
    p = t(g["p0"])
    ps.correct_fields(float(g["rho"]), float(g["urfP"]), t(g["aP"]), t(g["pPrime"]), p, U, phi)
    ctx.synchronize()
    assert bits_equal(p.cpu().numpy(), g["p1"]) and bits_equal(phi.cpu().numpy(), g["phi1"])
    assert bits_equal(np.array([u.cpu().numpy() for u in U]), g["U1"])
    ps.close()


def test_device_resident_pressure_step(sg, ctx, oracle):
    """fluxes -> assembly -> solve -> correction with every field on the
    device, against the oracle's same step on the host (the solve agrees to
    1e-10; the rest is bit-exact given the solution)."""
    torch = pytest.importorskip("torch")
    from simall_gb300 import workloads as W

    g, ps = _system(sg, ctx)
    dims = tuple(int(v) for v in g["dims"])
    om = oracle.cartesian_mesh(*dims, node_shift=W.interior_node_shift(*dims, amp=0.2, seed=int(g["seed"])))
    oracle.rcm(om)
    bcs = [(int(z), int(t), tuple(v)) for z, t, v in zip(g["bc_zone"], g["bc_type"], g["bc_vec"])]
    dev = torch.device("cuda:0")
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a).copy()).to(dev)  # noqa: E731
    U = [t(u) for u in g["U"]]
    aP, p = t(g["aP"]), t(g["p0"])
    phi = torch.empty(len(g["phi"]), dtype=torch.float64, device=dev)
    pp = torch.empty_like(p)
    s = sg.GpuCGSolver(sg.LinearSolverConfig(kind=sg.LinearSolverKind.CG, preconditioner=sg.PreconditionerKind.Jacobi,
                                             tolerance=1e-12, maxIterations=2000), ctx=ctx)
    ps.face_fluxes(1.2, U, phi)
    ps.assemble(1.2, aP, phi)
    ps.solve(s, pp)
    ps.correct_fields(1.2, 0.3, aP, pp, p, U, phi)
    ctx.synchronize()
    # host oracle step
    ophi = oracle.face_fluxes(om, bcs, 1.2, g["U"])
    orp, oci = oracle.build_sparsity(om)
    ov, orhs, _ = oracle.assemble(om, orp, oci, [2], 1.2, g["aP"], ophi)
    ox, _, _ = oracle.cg(orp, oci, ov, orhs, 0, 1e-12, 2000)
    assert np.linalg.norm(pp.cpu().numpy() - ox) <= 1e-10 * np.linalg.norm(ox)
    # correction given the device's p' is bit-exact
    op, oU, ophi1 = oracle.correct_fields(om, 1.2, 0.3, g["aP"], pp.cpu().numpy(), g["p0"], g["U"], ophi)
    assert bits_equal(p.cpu().numpy(), op) and bits_equal(phi.cpu().numpy(), ophi1)
    assert bits_equal(np.array([u.cpu().numpy() for u in U]), np.array(oU))
    s.close()
    ps.close()
