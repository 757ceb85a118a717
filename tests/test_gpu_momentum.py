"""Momentum assembly on the device -- SimpleAlgorithm::assemble_momentum for
the three velocity components in one pass -- against the reference's bytes
(tests/golden/momentum_7x6x5_rcm_bdf2.npz) and against the oracle on steady,
implicit-Euler and BDF2 cases, host and device arrays."""
import os

import numpy as np
import pytest

from helpers import bits_equal

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _system(sg, ctx, dims, seed, renumber, bcs):
    from simall_gb300 import workloads as W

    sh = W.interior_node_shift(*dims, amp=0.2, seed=seed) if dims[2] > 1 else None
    m = sg.cartesian(*dims, node_shift=sh)
    if renumber:
        sg.rcm(m)
    ps = sg.PressureSystem(m, [(b[0], b[1]) for b in bcs], ctx=ctx)
    ps.setup_field_loops([(b[0], b[2]) for b in bcs if b[1] in (2, 4)])
    return ps


def test_momentum_fixture_host_arrays(sg, ctx):
    g = np.load(os.path.join(GOLD, "momentum_7x6x5_rcm_bdf2.npz"))
    bcs = [(int(z), int(t), tuple(v)) for z, t, v in zip(g["bc_zone"], g["bc_type"], g["bc_vec"])]
    ps = _system(sg, ctx, tuple(int(v) for v in g["dims"]), int(g["seed"]), True, bcs)
    rho, mu, urf, dt = (float(v) for v in g["opt"])
    ps.assemble_momentum(rho, mu, urf, np.ascontiguousarray(g["U"]), np.ascontiguousarray(g["p"]),
                         np.ascontiguousarray(g["phi"]), dt, np.ascontiguousarray(g["Un"]),
                         np.ascontiguousarray(g["Unm1"]), bdf2=True)
    v, rhs, aP = ps.momentum_download()
    for comp in range(3):
        assert bits_equal(v, g["values"][comp])
        assert bits_equal(rhs[comp], g["rhs"][comp]), comp
    assert bits_equal(aP, g["aP"])
    ps.close()


MOM_BCS = [(1, 4, (0.7, -0.2, 0.1)), (2, 7, (0, 0, 0)), (3, 1, (0, 0, 0)), (4, 2, (1.0, 0.3, 0.0)),
           (5, 9, (0, 0, 0)), (6, 3, (0, 0, 0))]


@pytest.mark.parametrize("dims,renumber,dt,bdf2", [((6, 5, 4), False, 0.0, False), ((7, 6, 5), True, 0.05, False),
                                                   ((17, 13, 1), False, 0.02, True), ((24, 20, 16), True, 0.1, True)])
def test_momentum_against_oracle_device_arrays(sg, ctx, oracle, dims, renumber, dt, bdf2):
    """Device arrays in and out; the matrix, the three rhs and aP equal the
    oracle's three single-component assemblies bit for bit, including a second
    call with another viscosity (the face diffusion is recomputed)."""
    torch = pytest.importorskip("torch")
    from simall_gb300 import workloads as W

    ps = _system(sg, ctx, dims, 21, renumber, MOM_BCS)
    sh = W.interior_node_shift(*dims, amp=0.2, seed=21) if dims[2] > 1 else None
    om = oracle.cartesian_mesh(*dims, node_shift=sh)
    if renumber:
        oracle.rcm(om)
    rp, ci = oracle.build_sparsity(om)
    rng = np.random.default_rng(22)
    U = rng.standard_normal((3, om.nC))
    p = rng.standard_normal(om.nC)
    Un = rng.standard_normal((3, om.nC))
    Unm1 = rng.standard_normal((3, om.nC))
    phi = oracle.face_fluxes(om, MOM_BCS, 1.1, U)
    phi[::5] = 0.0
    phi[2::9] = -0.0
    gp = oracle.lsq_gradient(om, p)
    dev = torch.device("cuda:0")
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a).copy()).to(dev)  # noqa: E731
    for mu in (0.013, 0.002):
        opt = (1.1, mu, 0.7, dt)
        ps.assemble_momentum(1.1, mu, 0.7, t(U), t(p), t(phi), dt, t(Un), t(Unm1), bdf2=bdf2)
        v, rhs, aP = ps.momentum_download()
        for comp in range(3):
            ov, orhs, oaP = oracle.assemble_momentum(om, rp, ci, MOM_BCS, opt, comp, phi, gp[comp], U[comp],
                                                     Un[comp], Unm1[comp], bdf2=bdf2)
            assert bits_equal(v, ov) and bits_equal(rhs[comp], orhs), (mu, comp)
            assert bits_equal(aP, oaP)
    ps.close()
