"""Periodic boundaries on the device: the twin pairing
(SimpleAlgorithm::build_periodic_pairs, src/solver/SimpleAlgorithm.cpp:101-186),
the twin columns of the sparsity (:71-72), the pressure assembly (:411-419),
the face fluxes (:214-219) and the momentum assembly (:275-282), bit for bit
against the reference's bytes (tests/golden/periodic_channel_8x6x5.npz) and
the oracle, including a mesh one cell wide across a periodic pair (each face
is its own cell's twin: the coupling falls on the diagonal)."""
import os

import numpy as np
import pytest

from helpers import bits_equal

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
PERIODIC_BCS = [(1, 11), (2, 11), (3, 1), (4, 2, (1.0, 0.0, 0.0)), (5, 11), (6, 11)]


def _device_system(sg, ctx, dims, seed, amp, renumber, bcs):
    from simall_gb300 import workloads as W

    m = sg.cartesian(*dims, node_shift=W.interior_node_shift(*dims, amp=amp, seed=seed) if amp else None)
    if renumber:
        sg.rcm(m)
    ps = sg.PressureSystem(m, [(b[0], b[1]) for b in bcs], ctx=ctx)
    ps.setup_field_loops([(b[0], b[2]) for b in bcs if b[1] in (2, 4)])
    return m, ps


def test_periodic_channel_against_the_reference(sg, ctx):
    g = np.load(os.path.join(GOLD, "periodic_channel_8x6x5.npz"))
    dims = tuple(int(v) for v in g["dims"])
    m, ps = _device_system(sg, ctx, dims, int(g["seed"]), float(g["amp"]), True, PERIODIC_BCS)
    assert np.array_equal(ps.periodic_twins(), g["twin"])
    rp, ci = ps.pattern()
    assert np.array_equal(rp, g["rowPtr"]) and np.array_equal(ci, g["colIdx"])
    ps.assemble(1.1, g["aP"], g["phi"])
    v, rhs = ps.download()
    assert bits_equal(v, g["values"]) and bits_equal(rhs, g["rhs"])
    flux = ps.face_fluxes(1.2, [np.ascontiguousarray(u) for u in g["U"]])
    assert bits_equal(flux, g["flux"])
    ps.assemble_momentum(1.0, 0.02, 0.7, np.ascontiguousarray(g["U"]), np.ascontiguousarray(g["p"]),
                         np.ascontiguousarray(flux))
    mv, mr, maP = ps.momentum_download()
    assert bits_equal(mv, g["mom_values"]) and bits_equal(mr[0], g["mom_rhs"]) and bits_equal(maP, g["mom_aP"])
    ps.close()


@pytest.mark.parametrize("dims", [(7, 5, 1), (1, 6, 5)])
def test_one_cell_wide_periodic_pair(sg, ctx, oracle, dims):
    """z (or x) one cell wide and periodic: every face of the pair is the twin
    of the opposite face of its own cell, so the twin column is the diagonal;
    device against the oracle (assembly, fluxes, momentum)."""
    bcs = ([(1, 1), (2, 1), (3, 1), (4, 2, (1.0, 0.0, 0.0)), (5, 11), (6, 11)] if dims[2] == 1 else
           [(1, 11), (2, 11), (3, 1), (4, 2, (0.0, 0.0, 1.0)), (5, 1), (6, 1)])
    m, ps = _device_system(sg, ctx, dims, 3, 0.0, False, bcs)
    om = oracle.cartesian_mesh(*dims)
    twin = oracle.periodic_pairs(om, bcs)
    assert np.array_equal(ps.periodic_twins(), twin) and np.count_nonzero(twin >= 0) > 0
    own = om.owner
    assert all(own[twin[f]] == own[f] for f in np.flatnonzero(twin >= 0))
    rp, ci = ps.pattern()
    orp, oci = oracle.build_sparsity(om, twin)
    assert np.array_equal(rp, orp) and np.array_equal(ci, oci)
    rng = np.random.default_rng(8)
    aP = rng.uniform(0.5, 2.0, om.nC)
    phi = rng.standard_normal(om.nF)
    ps.assemble(1.0, aP, phi)
    v, rhs = ps.download()
    ov, orhs, _ = oracle.assemble(om, orp, oci, [], 1.0, aP, phi, twin)
    assert bits_equal(v, ov) and bits_equal(rhs, orhs)
    U = rng.standard_normal((3, om.nC))
    flux = ps.face_fluxes(1.0, [np.ascontiguousarray(u) for u in U])
    assert bits_equal(flux, oracle.face_fluxes(om, bcs, 1.0, U, twin))
    p = rng.standard_normal(om.nC)
    ps.assemble_momentum(1.0, 0.05, 0.7, np.ascontiguousarray(U), p, np.ascontiguousarray(flux))
    mv, mr, maP = ps.momentum_download()
    gp = oracle.lsq_gradient(om, p)
    for comp in range(3):
        ov2, or2, oaP = oracle.assemble_momentum(om, orp, oci, bcs, (1.0, 0.05, 0.7, 0.0), comp, flux, gp[comp],
                                                 U[comp], twin=twin)
        assert bits_equal(mv, ov2) and bits_equal(mr[comp], or2), comp
    ps.close()


def test_face_conductance_rejects_periodic_systems(sg, ctx):
    m, ps = _device_system(sg, ctx, (4, 3, 3), 1, 0.0, False, PERIODIC_BCS)
    k = np.ones(m.n_faces)
    with pytest.raises(sg.SimallError) as e:
        ps.assemble_face_conductance(1.0, k, np.zeros(m.n_faces), np.zeros(m.n_cells))
    assert e.value.status == 11
    ps.close()
