"""Device assembly vs SimpleAlgorithm::assemble_pressure_correction
(src/solver/SimpleAlgorithm.cpp:358-447) via the oracle: pattern bit-exact,
values and rhs bit-exact (stronger than the 1e-14 relative bar)."""
import numpy as np
import pytest

from helpers import bits_equal, oracle_system, product_mesh

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("dims,renumber,zones", [((8, 8, 8), True, ()), ((9, 6, 5), False, (1,)),
                                                  ((7, 7, 1), False, ()), ((10, 10, 10), True, (1, 4))])
def test_assembly_bit_exact(sg, ctx, oracle, dims, renumber, zones):
    m = product_mesh(sg, None, dims=dims, renumber=renumber, seed=11)
    om, rp, ci, v, rhs, aP, phi = oracle_system(oracle, None, dims=dims, renumber=renumber, seed=11,
                                                pressure_zones=zones)
    bcs = [(z, int(sg.BCType.PressureOutlet)) for z in zones] + [(z, int(sg.BCType.NoSlipWall)) for z in range(1, 7)
                                                                  if z not in zones]
    ps = sg.PressureSystem(m, bcs, ctx=ctx)
    prp, pci = ps.pattern()
    assert np.array_equal(prp, rp) and np.array_equal(pci, ci)
    ps.assemble(1.0, aP, phi)
    pv, prhs = ps.download()
    assert bits_equal(pv, v)
    assert bits_equal(prhs, rhs)
    assert ps.any_dirichlet == bool(zones)


def test_assembly_device_inputs_and_rho(sg, ctx, oracle):
    torch = pytest.importorskip("torch")
    m = product_mesh(sg, 6, seed=3)
    om, rp, ci, v, rhs, aP, phi = oracle_system(oracle, 6, seed=3)
    ov, orhs, _ = oracle.assemble(om, rp, ci, [], 2.5, aP, phi)
    ps = sg.PressureSystem(m, [], ctx=ctx)
    dev = torch.device("cuda:0")
    ps.assemble(2.5, torch.from_numpy(aP).to(dev), torch.from_numpy(phi).to(dev))
    ctx.synchronize()
    pv, prhs = ps.download()
    assert bits_equal(pv, ov) and bits_equal(prhs, orhs)


@pytest.mark.parametrize("on_device", [False, True])
def test_simplec_assembly_bit_exact(sg, ctx, oracle, on_device):
    """SIMPLEC on the device against the reference fixture (SimpleAlgorithm
    with PvCouplingVariant::SIMPLEC, tests/golden/make_golden.py)."""
    import os

    from simall_gb300 import workloads as W

    g = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "simplec_6x5x4_outlet.npz"))
    dims = tuple(int(v) for v in g["dims"])
    m = sg.cartesian(*dims, node_shift=W.interior_node_shift(*dims, amp=0.2, seed=int(g["seed"])))
    bcs = [(1, int(sg.BCType.PressureOutlet))] + [(z, int(sg.BCType.NoSlipWall)) for z in range(2, 7)]
    ps = sg.PressureSystem(m, bcs, ctx=ctx)
    args = (g["aP"], g["mom"], g["phi"])
    if on_device:
        torch = pytest.importorskip("torch")
        args = tuple(torch.from_numpy(np.ascontiguousarray(a)).cuda() for a in args)
    ps.assemble_simplec(float(g["rho"]), *args)
    ctx.synchronize()
    v, rhs = ps.download()
    assert bits_equal(v, g["values"]) and bits_equal(rhs, g["rhs"]) and ps.any_dirichlet
    ps.close()


def test_assembly_then_device_solve(sg, ctx, oracle):
    m = product_mesh(sg, 12, seed=5)
    om, rp, ci, v, rhs, aP, phi = oracle_system(oracle, 12, seed=5)
    ps = sg.PressureSystem(m, [], ctx=ctx)
    ps.assemble(1.0, aP, phi)
    cfg = sg.LinearSolverConfig(kind=sg.LinearSolverKind.CG, preconditioner=sg.PreconditionerKind.Jacobi)
    s = sg.GpuCGSolver(cfg, ctx=ctx)
    x = ps.solve(s)
    xo, ito, lasto = oracle.cg(rp, ci, v, rhs, 0, 1e-8, 1000)
    assert abs(s.stats.iterations - ito) <= 1
    assert np.linalg.norm(x - xo) <= 1e-10 * np.linalg.norm(xo)
    # re-assemble with new aP (values change, pattern and pointers stay)
    aP2 = aP * 1.7
    ps.assemble(1.0, aP2, phi)
    x2 = ps.solve(s)
    ov2, orhs2, _ = oracle.assemble(om, rp, ci, [], 1.0, aP2, phi)
    xo2, ito2, _ = oracle.cg(rp, ci, ov2, orhs2, 0, 1e-8, 1000)
    assert np.linalg.norm(x2 - xo2) <= 1e-10 * np.linalg.norm(xo2)


def test_periodic_distorted_renumbered_box(sg, ctx, oracle):
    """x-periodic distorted, RCM-renumbered box: twins, pattern, values and
    rhs against the oracle (the pairing searches nearest centroids after the
    translation, so distortion and renumbering both reach it)."""
    dims = (6, 5, 4)
    bcs = [(1, int(sg.BCType.Periodic)), (2, int(sg.BCType.Periodic))] + [
        (z, int(sg.BCType.NoSlipWall)) for z in range(3, 7)]
    m = product_mesh(sg, None, dims=dims, renumber=True, seed=21)
    om, _, _, _, _, aP, phi = oracle_system(oracle, None, dims=dims, renumber=True, seed=21)
    ps = sg.PressureSystem(m, bcs, ctx=ctx)
    twin = oracle.periodic_pairs(om, bcs)
    assert np.array_equal(ps.periodic_twins(), twin) and np.count_nonzero(twin >= 0) == 2 * dims[1] * dims[2]
    rp, ci = ps.pattern()
    orp, oci = oracle.build_sparsity(om, twin)
    assert np.array_equal(rp, orp) and np.array_equal(ci, oci)
    ps.assemble(1.0, aP, phi)
    v, rhs = ps.download()
    ov, orhs, _ = oracle.assemble(om, orp, oci, [], 1.0, aP, phi, twin)
    assert bits_equal(v, ov) and bits_equal(rhs, orhs)
    ps.close()
