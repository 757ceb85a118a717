"""The oracle against the reference's own code, live (oracle/_ref, built from
the reference sources by oracle/build_ref.sh).  Skipped where the compiled
reference is absent."""
import numpy as np
import pytest

from helpers import bits_equal


def _shift(dims, seed, amp):
    from simall_gb300 import workloads as W

    return W.interior_node_shift(*dims, amp=amp, seed=seed) if amp else None


@pytest.mark.parametrize("dims,seed,amp,renumber", [((5, 4, 3), 1, 0.2, False), ((7, 7, 7), 2, 0.2, True),
                                                    ((12, 5, 9), 3, 0.15, True), ((20, 20, 1), 4, 0.0, False)])
def test_mesh_rcm_assembly_cg(oracle, ref, dims, seed, amp, renumber):
    sh = _shift(dims, seed, amp)
    r = ref.cartesian_mesh(*dims, node_shift=sh, do_rcm=renumber)
    m = oracle.cartesian_mesh(*dims, node_shift=sh)
    if renumber:
        _, st = oracle.rcm(m)
        assert st == r["rcm_stats"]
    for k in ("owner", "neighbor", "zone", "cfOff", "cfIdx"):
        assert np.array_equal(getattr(m, k), r[k]), k
    for k in ("ax", "ay", "az", "fcx", "fcy", "fcz", "vol", "ccx", "ccy", "ccz"):
        assert bits_equal(getattr(m, k), r[k]), k
    rng = np.random.default_rng(seed)
    aP = rng.uniform(0.3, 3.0, m.nC)
    phi = rng.standard_normal(m.nF)
    for bcs, pz in (([], []), ([(1, 7), (2, 5)], [1, 2])):
        rp, ci, v, rhs = ref.assemble(r, bcs, 1.3, aP, phi)
        orp, oci = oracle.build_sparsity(m)
        ov, orhs, _ = oracle.assemble(m, orp, oci, pz, 1.3, aP, phi)
        assert np.array_equal(rp, orp) and np.array_equal(ci, oci)
        assert bits_equal(v, ov) and bits_equal(rhs, orhs)
        for pc in (0, 1, 2, 3):
            x, it, last, _ = ref.cg(rp, ci, v, rhs, pc, 1e-9, 3000)
            ox, oit, olast = oracle.cg(rp, ci, v, rhs, pc, 1e-9, 3000)
            assert it == oit and last == olast and bits_equal(x, ox)
        z = np.random.default_rng(seed + 1).standard_normal(m.nC)
        assert bits_equal(ref.precond_apply(2, rp, ci, v, z), oracle.ssor_apply(rp, ci, v, z))
        assert bits_equal(ref.precond_apply(3, rp, ci, v, z), oracle.amg_apply(rp, ci, v, z)[0])
    ref.free_mesh(r)


@pytest.mark.parametrize("dims,renumber,bcs,pz", [((7, 7, 7), True, [], []),
                                                  ((9, 6, 4), False, [(1, 7), (2, 5)], [1, 2])])
def test_simplec_assembly(oracle, ref, dims, renumber, bcs, pz):
    """PvCouplingVariant::SIMPLEC: denominators aP - sum|offdiag(A_mom)|."""
    sh = _shift(dims, 5, 0.2)
    r = ref.cartesian_mesh(*dims, node_shift=sh, do_rcm=renumber)
    m = oracle.cartesian_mesh(*dims, node_shift=sh)
    if renumber:
        oracle.rcm(m)
    rng = np.random.default_rng(5)
    rp, ci = oracle.build_sparsity(m)
    aP = rng.uniform(1.0, 4.0, m.nC)
    mom = rng.standard_normal(len(ci)) * 0.3
    phi = rng.standard_normal(m.nF)
    rrp, rci, rv, rrhs = ref.assemble_simplec(r, bcs, 1.1, aP, mom, phi)
    den = oracle.simplec_denominator(rp, ci, mom, aP)
    ov, orhs, _ = oracle.assemble(m, rp, ci, pz, 1.1, den, phi)
    assert np.array_equal(rrp, rp) and np.array_equal(rci, ci)
    assert bits_equal(rv, ov) and bits_equal(rrhs, orhs)
    ref.free_mesh(r)


@pytest.mark.parametrize("dims,renumber", [((6, 5, 4), False), ((7, 6, 5), True), ((10, 9, 1), False)])
def test_face_loops_around_the_solve(oracle, ref, dims, renumber):
    """compute_face_fluxes, LeastSquaresGradient and correct_fields: the
    oracle reproduces the reference's bytes (distorted mesh, every boundary
    treatment of the flux loop)."""
    sh = _shift(dims, 8, 0.2 if dims[2] > 1 else 0.0)
    r = ref.cartesian_mesh(*dims, node_shift=sh, do_rcm=renumber)
    m = oracle.cartesian_mesh(*dims, node_shift=sh)
    if renumber:
        oracle.rcm(m)
    rng = np.random.default_rng(8)
    U = [rng.standard_normal(m.nC) for _ in range(3)]
    bcs = [(1, 4, (0.7, -0.2, 0.1)), (2, 7), (3, 1), (4, 2, (1.0, 0.0, 0.0)), (5, 9), (6, 3)]
    phi = oracle.face_fluxes(m, bcs, 1.2, U)
    assert bits_equal(phi, ref.face_fluxes(r, bcs, 1.2, U))
    f = rng.standard_normal(m.nC)
    g = oracle.lsq_gradient(m, f)
    assert bits_equal(g, ref.lsq_gradient(r, f))
    aP = rng.uniform(0.5, 2.0, m.nC)
    pp = rng.standard_normal(m.nC) * 1e-2
    p0 = rng.standard_normal(m.nC)
    got = oracle.correct_fields(m, 1.2, 0.3, aP, pp, p0, U, phi)
    want = ref.correct_fields(r, 1.2, 0.3, aP, pp, p0, U, phi)
    assert bits_equal(got[0], want[0]) and bits_equal(got[2], want[2])
    for a, b in zip(got[1], want[1]):
        assert bits_equal(a, b)
    ref.free_mesh(r)


def test_precond_none_maps_to_jacobi(oracle, ref):
    """make_preconditioner's default branch (LinearSolvers.cpp:240-254)."""
    r = ref.cartesian_mesh(4, 4, 4)
    rp, ci, v, rhs = ref.assemble(r, [], 1.0, np.ones(64), np.random.default_rng(0).standard_normal(r["nF"]))
    z = np.random.default_rng(1).standard_normal(64)
    assert bits_equal(ref.precond_apply(4, rp, ci, v, z), ref.precond_apply(0, rp, ci, v, z))
    ref.free_mesh(r)


def test_cavity_trajectory_longer(oracle, ref):
    c = ref.cavity(24, mu=0.01, n_outer=4, n_record=4, precond=1, tol=1e-8, max_it=1000)
    m = oracle.cartesian_mesh(24, 24, 1, 1.0, 1.0, 1.0 / 24)
    rp, ci = oracle.build_sparsity(m)
    for it in range(4):
        v, rhs, _ = oracle.assemble(m, rp, ci, [], 1.0, c["aP"][it], c["phi"][it])
        assert bits_equal(v, c["values"][it]) and bits_equal(rhs, c["rhs"][it])
        x, its, last = oracle.cg(rp, ci, v, rhs, 1, 1e-8, 1000)
        assert its == c["iters"][it] and bits_equal(x, c["x"][it])


def test_discrete_adjoint_2x2_known_answer(ref):
    """tests/unit/longtail/test_longtail_modules.cpp:32-54: A = [[2,1],[0,3]],
    dJ/dQ = (1,1) -> psi = (0.5, 1/6)."""
    rp = np.array([0, 2, 3], np.int32)
    ci = np.array([0, 1, 1], np.int32)
    va = np.array([2.0, 1.0, 3.0])
    psi, grad, its, res, rc = ref.discrete_adjoint(rp, ci, va, np.ones(2), np.zeros(0, np.int64),
                                                   np.zeros(0, np.int64), np.zeros(0, np.int32), np.zeros(0),
                                                   np.zeros(0), np.zeros(0), np.zeros(2))
    assert rc == 0
    assert abs(psi[0] - 0.5) < 1e-6 and abs(psi[1] - 1.0 / 6.0) < 1e-6


# every boundary treatment of assemble_momentum: VelocityInlet, PressureOutlet
# (the "other" branch), NoSlipWall, MovingWall, Symmetry, SlipWall (other), and
# zone 0 of a 2-D mesh's front/back faces without a spec
MOM_BCS = [(1, 4, (0.7, -0.2, 0.1)), (2, 7), (3, 1), (4, 2, (1.0, 0.3, 0.0)), (5, 9), (6, 3)]


@pytest.mark.parametrize("dims,renumber,dt,bdf2", [((6, 5, 4), False, 0.0, False), ((7, 6, 5), True, 0.05, False),
                                                   ((9, 8, 1), False, 0.02, True), ((5, 5, 5), True, 0.1, True)])
def test_momentum_assembly(oracle, ref, dims, renumber, dt, bdf2):
    """assemble_momentum for each component, steady, implicit Euler and BDF2:
    the oracle reproduces the reference's values, rhs and aP_ bytes."""
    sh = _shift(dims, 11, 0.2 if dims[2] > 1 else 0.0)
    r = ref.cartesian_mesh(*dims, node_shift=sh, do_rcm=renumber)
    m = oracle.cartesian_mesh(*dims, node_shift=sh)
    if renumber:
        oracle.rcm(m)
    rp, ci = oracle.build_sparsity(m)
    rng = np.random.default_rng(12)
    U = rng.standard_normal((3, m.nC))
    p = rng.standard_normal(m.nC)
    phi = oracle.face_fluxes(m, MOM_BCS, 1.1, U)
    phi[::7] = 0.0
    phi[3::11] = -0.0
    Un = rng.standard_normal((3, m.nC))
    Unm1 = rng.standard_normal((3, m.nC))
    gp = oracle.lsq_gradient(m, p)
    opt = (1.1, 0.013, 0.7, dt)
    for comp in range(3):
        v, rhs, aP = ref.assemble_momentum(r, MOM_BCS, opt, comp, U, p, phi, Un, Unm1, bdf2=bdf2, time_step=1)
        ov, orhs, oaP = oracle.assemble_momentum(m, rp, ci, MOM_BCS, opt, comp, phi, gp[comp], U[comp], Un[comp],
                                                 Unm1[comp], bdf2=bdf2)
        assert bits_equal(v, ov) and bits_equal(rhs, orhs), comp
        if comp == 0:
            assert bits_equal(aP, oaP)
    ref.free_mesh(r)


def _conv_diff(n, pe=5.0):
    """The non-symmetric 1-D upwind convection-diffusion matrix of
    tests/unit/solver/test_tfqmr_solver.cpp:43-62."""
    rp, ci, v = [0], [], []
    for i in range(n):
        if i > 0:
            ci.append(i - 1)
            v.append(-1.0 - pe)
        ci.append(i)
        v.append(2.0 + pe)
        if i < n - 1:
            ci.append(i + 1)
            v.append(-1.0)
        rp.append(len(ci))
    return np.array(rp, np.int32), np.array(ci, np.int32), np.array(v)


@pytest.mark.parametrize("kind", [0, 1, 3])
@pytest.mark.parametrize("pc", [0, 1, 2, 3])
def test_nonsymmetric_krylov(oracle, ref, kind, pc):
    """GMRES(m), BiCGSTAB and TFQMR with Jacobi, ILU(0), SSOR and AMG: iteration
    count, last residual and x bit-identical to the reference, on the 1-D
    convection-diffusion matrix and on a momentum system (restart short
    enough to cycle)."""
    systems = []
    rp, ci, v = _conv_diff(40)
    systems.append((rp, ci, v, np.ones(40), 1e-8, 500, 30))
    m = oracle.cartesian_mesh(9, 8, 3, node_shift=_shift((9, 8, 3), 4, 0.2))
    rp, ci = oracle.build_sparsity(m)
    rng = np.random.default_rng(5)
    U = rng.standard_normal((3, m.nC))
    phi = oracle.face_fluxes(m, MOM_BCS, 1.0, U)
    gp = oracle.lsq_gradient(m, rng.standard_normal(m.nC))
    mv, mrhs, _ = oracle.assemble_momentum(m, rp, ci, MOM_BCS, (1.0, 0.01, 0.7, 0.0), 0, phi, gp[0], U[0])
    systems.append((rp, ci, mv, mrhs, 1e-10, 200, 5))
    systems.append((rp, ci, mv, mrhs, 1e-12, 7, 3))  # stops on maxIterations mid-cycle
    for rp, ci, v, b, tol, mx, rs in systems:
        x, it, last, _ = ref.krylov(kind, rp, ci, v, b, pc, tol, mx, rs)
        ox, oit, olast = (oracle.gmres(rp, ci, v, b, pc, tol, mx, rs) if kind == 0
                          else oracle.bicgstab(rp, ci, v, b, pc, tol, mx) if kind == 1
                          else oracle.tfqmr(rp, ci, v, b, pc, tol, mx))
        assert (it, last) == (oit, olast) or (np.isnan(last) and np.isnan(olast) and it == oit)
        assert bits_equal(x, ox)


def test_tfqmr_laplacian_jacobi(oracle, ref):
    """tests/unit/solver/test_tfqmr_solver.cpp:67-89's system (30-point 1-D
    Laplacian, b = 1, Jacobi, tol 1e-8): the reference's TfqmrSolver returns
    after 88 iterations with a non-finite x; the oracle returns the same
    count, residual and x bit for bit."""
    from helpers import tridiag

    rp, ci, va = tridiag(30, -1.0, 2.0, -1.0)
    b = np.ones(30)
    x, it, last, _ = ref.krylov(3, rp, ci, va, b, 0, 1e-8, 500)
    ox, oit, olast = oracle.tfqmr(rp, ci, va, b, 0, 1e-8, 500)
    assert it == oit == 88 and last == olast and bits_equal(x, ox)
    assert not np.all(np.isfinite(x))


CAVITY_BCS = [(z, 1) for z in (1, 2, 3, 5, 6)] + [(4, 2, (1.0, 0.0, 0.0))]
CHANNEL_BCS = [(1, 4, (1.0, 0.1, 0.0)), (2, 7), (3, 1), (4, 1), (5, 9), (6, 0)]
# periodic in x (zones 1, 2) and z (5, 6), no-slip floor, lid moving in x
PERIODIC_BCS = [(1, 11), (2, 11), (3, 1), (4, 2, (1.0, 0.0, 0.0)), (5, 11), (6, 11)]

SIMPLE_CASES = {
    # name: (dims, amp, renumber, bcs, kwargs, n_outer, n_inner)
    "cavity_gmres_ilu": ((16, 16, 1), 0.0, False, CAVITY_BCS,
                         dict(mu=0.01, mom_cfg=(0, 1, 1e-6, 200, 30), p_cfg=(2, 0, 1e-8, 1000, 30)), 6, 1),
    "channel_simplec_bicgstab": ((8, 6, 5), 0.2, True, CHANNEL_BCS,
                                 dict(mu=0.1, simplec=True, urfP=0.9, mom_cfg=(1, 0, 1e-8, 200, 30),
                                      p_cfg=(2, 1, 1e-9, 1000, 30)), 5, 1),
    "cavity_bdf2_gmres_jacobi": ((12, 12, 1), 0.0, False, CAVITY_BCS,
                                 dict(mu=0.01, dt=0.01, bdf2=True, mom_cfg=(0, 0, 1e-8, 200, 5),
                                      p_cfg=(2, 0, 1e-9, 1000, 30)), 3, 2),
    "periodic_couette_rcm": ((8, 6, 4), 0.15, True, PERIODIC_BCS,
                             dict(mu=0.05, mom_cfg=(0, 1, 1e-8, 200, 30), p_cfg=(2, 0, 1e-9, 1000, 30)), 6, 1),
}


@pytest.mark.parametrize("case", sorted(SIMPLE_CASES))
def test_simple_outer_iterations(oracle, ref, case):
    """SimpleAlgorithm::iterate / advance_time_step: the oracle's outer
    iterations reproduce the reference's U, p, phi, residuals and every linear
    solve's iteration count, bit for bit."""
    dims, amp, renumber, bcs, kw, n_outer, n_inner = SIMPLE_CASES[case]
    sh = _shift(dims, 31, amp)
    r = ref.cartesian_mesh(*dims, node_shift=sh, do_rcm=renumber)
    m = oracle.cartesian_mesh(*dims, node_shift=sh)
    if renumber:
        oracle.rcm(m)
    want = ref.simple_run(r, bcs, np.zeros((3, m.nC)), np.zeros(m.nC), n_outer, n_inner=n_inner, **kw)
    s = oracle.SimpleOracle(m, bcs, **kw)
    res, its = [], []
    for _ in range(n_outer):
        out = s.advance_time_step(n_inner) if kw.get("dt", 0.0) > 0 else s.iterate()
        res.append(out[0])
    assert np.array_equal(np.array(s.iters), want["iters"])
    assert bits_equal(np.array(res), want["res"])
    assert bits_equal(s.U, want["U"]) and bits_equal(s.p, want["p"]) and bits_equal(s.phi, want["phi"])
    ref.free_mesh(r)


@pytest.mark.parametrize("dims,radius,renumber", [((7, 6, 5), 0.0, False), ((7, 6, 5), 0.3, True),
                                                  ((12, 10, 1), 0.15, False)])
def test_simp_topology_steps(oracle, ref, dims, radius, renumber):
    """SimpTopology::initialize + step (filter, penalised property, OC update
    with bisection): three steps with seeded negative sensitivities, rho,
    rhoTilde, K_simp, dC_drhoTilde and the change bit-identical."""
    sh = _shift(dims, 51, 0.2 if dims[2] > 1 else 0.0)
    r = ref.cartesian_mesh(*dims, node_shift=sh, do_rcm=renumber)
    m = oracle.cartesian_mesh(*dims, node_shift=sh)
    if renumber:
        oracle.rcm(m)
    cfg = (3.0, 1e-9, 1.0, radius, 0.4, 0.2, 0.5, 1e-3)
    rng = np.random.default_rng(52)
    dC = -np.abs(rng.standard_normal((3, m.nC))) * 0.1
    want = ref.simp_run(r, cfg, dC)
    s = oracle.SimpOracle(m, cfg)
    changes = []
    for k in range(3):
        s.dC_drho[:] = dC[k]
        changes.append(s.step())
    assert bits_equal(np.array(changes), want[0])
    for got, w in zip((s.rho, s.rhoTilde, s.K_simp, s.dC_drhoTilde), want[1:]):
        assert bits_equal(got, w)
    ref.free_mesh(r)


PISO_PIMPLE_CASES = {
    # name: (dims, amp, renumber, bcs, variant, loops, extra kwargs, steps)
    "piso_cavity": ((12, 12, 1), 0.0, False, CAVITY_BCS, 1, (1, 2, 1, 1), dict(mu=0.01, dt=0.01), 3),
    "pimple_channel": ((8, 6, 5), 0.2, True, CHANNEL_BCS, 2, (3, 2, 0, 1),
                       dict(mu=0.05, dt=0.02, urfU=0.7, urfP=0.3, tol_u=1e-6, tol_p=0.15), 3),  # exits at 2, 1, 0
    "pimple_as_piso": ((10, 8, 1), 0.0, False, CAVITY_BCS, 2, (1, 2, 0, 1), dict(mu=0.02, dt=0.005), 2),
}


def piso_pimple_oracle(oracle, m, bcs, variant, loops, kw):
    """The oracle configured as PisoAlgorithm / PimpleAlgorithm configure
    SimpleAlgorithm (PisoAlgorithm.hpp:63-74, PimpleAlgorithm.hpp:92-105)."""
    piso_mode = variant == 1 or loops[0] <= 1
    return oracle.SimpleOracle(m, bcs, rho=kw.get("rho", 1.0), mu=kw["mu"], dt=kw["dt"], bdf2=True,
                               urfU=1.0 if piso_mode else kw["urfU"], urfP=1.0 if piso_mode else kw["urfP"],
                               mom_cfg=(0, 0, 1e-9, 200, 30), p_cfg=(2, 0, 1e-9, 1000, 30),
                               n_outer_correctors=1 if variant == 1 else loops[0], n_correctors=loops[1],
                               n_non_orth_corr=loops[2], momentum_predictor=bool(loops[3]),
                               tol_u=kw.get("tol_u", 0.0) if variant == 2 else 0.0,
                               tol_p=kw.get("tol_p", 0.0) if variant == 2 else 0.0)


@pytest.mark.parametrize("case", sorted(PISO_PIMPLE_CASES))
def test_piso_pimple_time_steps(oracle, ref, case):
    """PisoAlgorithm / PimpleAlgorithm::iterate under advance_time_step(1):
    U, p, phi, residuals and PIMPLE's outer-exit index bit-identical."""
    dims, amp, renumber, bcs, variant, loops, kw, steps = PISO_PIMPLE_CASES[case]
    sh = _shift(dims, 61, amp)
    r = ref.cartesian_mesh(*dims, node_shift=sh, do_rcm=renumber)
    m = oracle.cartesian_mesh(*dims, node_shift=sh)
    if renumber:
        oracle.rcm(m)
    want = ref.piso_pimple_run(r, variant, bcs, np.zeros((3, m.nC)), np.zeros(m.nC), steps, loops=loops, **kw)
    s = piso_pimple_oracle(oracle, m, bcs, variant, loops, kw)
    res, last = [], []
    for _ in range(steps):
        res.append(s.advance_time_step(1)[0])
        last.append(s.last_outer if variant == 2 else 0)
    assert bits_equal(np.array(res), want["res"])
    assert list(want["last_outer"]) == last
    assert bits_equal(s.U, want["U"]) and bits_equal(s.p, want["p"]) and bits_equal(s.phi, want["phi"])
    ref.free_mesh(r)


@pytest.mark.parametrize("kind", [0, 1, 3])
def test_krylov_edge_cases(oracle, ref, kind):
    """b = 0, maxIterations = 0 and maxIterations reached after one step:
    the reference's return values and last residuals, for GMRES(m),
    BiCGSTAB and TFQMR."""
    from helpers import tridiag

    rp, ci, va = tridiag(40, -6.0, 7.0, -1.0)
    b = np.linspace(1.0, 2.0, 40)
    for bb, mx in ((np.zeros(40), 100), (b, 0), (b, 1)):
        x, it, last, _ = ref.krylov(kind, rp, ci, va, bb, 0, 1e-12, mx, 3)
        ox, oit, olast = (oracle.gmres(rp, ci, va, bb, 0, 1e-12, mx, 3) if kind == 0
                          else oracle.bicgstab(rp, ci, va, bb, 0, 1e-12, mx) if kind == 1
                          else oracle.tfqmr(rp, ci, va, bb, 0, 1e-12, mx))
        assert (it, last) == (oit, olast), (kind, mx)
        assert bits_equal(x, ox)


def test_cggpu_cases(oracle, ref):
    """gpu::CgGpu (set_matrix + solve, the facade's host path) against the
    oracle's restatement: x and every stat bit for bit, including the ILU0 ->
    Jacobi fall-back, the p.q breakdown, maxIterations 0 and b = 0."""
    from helpers import cggpu_cases

    for name, rp, ci, v, b, x0, pc, tol, mi, ro in cggpu_cases(oracle):
        xr, sr = ref.cggpu(rp, ci, v, b, x0, pc, tol, mi, ro)
        xo, so = oracle.cggpu(rp, ci, v, b, x0, pc, tol, mi, ro)
        assert bits_equal(xr, xo), name
        assert sr == so, (name, sr, so)


def test_periodic_faces(oracle, ref):
    """Periodic pairing, the twin columns, the pressure assembly, the face
    fluxes and the momentum assembly of the oracle against the reference, bit
    for bit, on a distorted channel periodic in x and z and on meshes one cell
    wide across the periodic pair (each face is its own cell's twin)."""
    from simall_gb300 import workloads as W

    for dims, amp, bcs in (((8, 6, 5), 0.2, PERIODIC_BCS),
                           ((7, 5, 1), 0.0, [(1, 1), (2, 1), (3, 1), (4, 2, (1.0, 0.0, 0.0)), (5, 11), (6, 11)]),
                           ((1, 6, 5), 0.0, [(1, 11), (2, 11), (3, 1), (4, 2, (0.0, 0.0, 1.0)), (5, 1), (6, 1)])):
        sh = _shift(dims, 5, amp)
        r = ref.cartesian_mesh(*dims, node_shift=sh)
        m = oracle.cartesian_mesh(*dims, node_shift=sh)
        twin = oracle.periodic_pairs(m, bcs)
        assert np.array_equal(ref.periodic_twins(r, bcs), twin) and np.any(twin >= 0)
        rng = np.random.default_rng(5)
        aP = rng.uniform(0.5, 2.0, m.nC)
        phi = rng.standard_normal(m.nF)
        rp, ci, v, rhs = ref.assemble(r, [(b[0], b[1]) for b in bcs], 1.1, aP, phi)
        orp, oci = oracle.build_sparsity(m, twin)
        ov, orhs, anyD = oracle.assemble(m, orp, oci, [], 1.1, aP, phi, twin)
        assert np.array_equal(rp, orp) and np.array_equal(ci, oci) and not anyD
        assert bits_equal(v, ov) and bits_equal(rhs, orhs)
        U = [rng.standard_normal(m.nC) for _ in range(3)]
        flux = ref.face_fluxes(r, bcs, 1.2, U)
        assert bits_equal(flux, oracle.face_fluxes(m, bcs, 1.2, U, twin))
        p = rng.standard_normal(m.nC)
        g = oracle.lsq_gradient(m, p)
        for comp in range(3):
            vr, rr, aPr = ref.assemble_momentum(r, bcs, (1.0, 0.01, 0.7, 0.0), comp, np.array(U), p, flux)
            vo, ro, aPo = oracle.assemble_momentum(m, orp, oci, bcs, (1.0, 0.01, 0.7, 0.0), comp, flux, g[comp],
                                                   U[comp], twin=twin)
            assert bits_equal(vr, vo) and bits_equal(rr, ro) and (comp > 0 or bits_equal(aPr, aPo))
        ref.free_mesh(r)
