"""Generate the golden fixtures in tests/golden/ from the reference's own code.

Runs only where the reference tree is available (it needs
oracle/_ref/libsimall_ref.so, built by oracle/build_ref.sh from the SimAll
sources).  Every array stored here is an output of the reference's functions
(CartesianMesher + ConnectivityBuilder + compute_geometry,
renumber_cells_cuthill_mckee, SimpleAlgorithm::build_sparsity /
assemble_pressure_correction / assemble_momentum, CGSolver::solve with
Jacobi, ILU0, SSOR and AMG, GMRES(m), BiCGSTAB and TFQMR, the
preconditioners' apply, the SIMPLE cavity loop, SimpleAlgorithm::iterate /
advance_time_step runs, PisoAlgorithm / PimpleAlgorithm time steps,
io::Checkpoint::write, SimpTopology steps,
solve_discrete_adjoint);
inputs are seeded synthetic data.  The fixtures are small (about 2 MB in
all) so that the tests that read them run everywhere, the GPU host included.

Usage:  python tests/golden/make_golden.py            (the small fixtures)
        python tests/golden/make_golden.py NAME.npz   (a benchmark-size one:
        poisson3d_128_cg, varcoef_256_cg, batched_512_cg, adjoint_face_k_24;
        minutes of the reference's serial solvers each)
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402
from simall_gb300 import workloads as W  # noqa: E402

R = O.RefLib()


def mesh_case(name, dims, seed, amp, renumber, bcs, pressure_zones):
    nx, ny, nz = dims
    shift = W.interior_node_shift(nx, ny, nz, amp=amp, seed=seed) if amp else None
    m = R.cartesian_mesh(nx, ny, nz, node_shift=shift, do_rcm=renumber)
    rng = np.random.default_rng(seed + 100)
    aP = rng.uniform(0.5, 2.0, m["nC"])
    phi = rng.standard_normal(m["nF"])
    phi[m["neighbor"] < 0] = 0.0
    rp, ci, v, rhs = R.assemble(m, bcs, 1.0, aP, phi)
    out = {k: m[k] for k in ("owner", "neighbor", "ax", "ay", "az", "fcx", "fcy", "fcz", "zone", "vol", "ccx", "ccy",
                             "ccz", "cfOff", "cfIdx")}
    out.update(dims=np.array(dims), seed=np.array(seed), amp=np.array(amp), renumber=np.array(int(renumber)),
               pressure_zones=np.array(pressure_zones, np.int64), aP=aP, phi=phi, rowPtr=rp, colIdx=ci, values=v,
               rhs=rhs)
    if m["rcm_stats"]:
        out["rcm_stats"] = np.array(m["rcm_stats"])
    for pc, tag in ((0, "jacobi"), (1, "ilu0")):
        x, it, last, _ = R.cg(rp, ci, v, rhs, pc, 1e-8, 2000)
        out[f"cg_{tag}_x"] = x
        out[f"cg_{tag}_iters"] = np.array(it)
        out[f"cg_{tag}_last"] = np.array(last)
        r = np.random.default_rng(seed + 200).standard_normal(len(rhs))
        out[f"apply_{tag}_r"] = r
        out[f"apply_{tag}_z"] = R.precond_apply(pc, rp, ci, v, r)
    xx = np.random.default_rng(seed + 300).standard_normal(len(rhs))
    out["spmv_x"] = xx
    out["spmv_y"] = R.spmv(rp, ci, v, xx)
    R.free_mesh(m)
    np.savez_compressed(os.path.join(HERE, name), **out)


def cavity_case(name, N, n_outer, n_record):
    c = R.cavity(N, mu=0.01, n_outer=n_outer, n_record=n_record, precond=0, tol=1e-8, max_it=1000)
    np.savez_compressed(os.path.join(HERE, name), N=np.array(N), n_outer=np.array(n_outer), rowPtr=c["rowPtr"],
                        colIdx=c["colIdx"], values=c["values"], rhs=c["rhs"], x=c["x"], aP=c["aP"], phi=c["phi"],
                        iters=c["iters"], res=c["res"])


def cavity_case_full_size(name, N, n_outer):
    """The SIMPLE cavity at full size: records the first and the last outer
    iteration's pressure system.  The assembled matrix and rhs are stored as
    SHA-256 digests of their bytes (the test reassembles them from aP and phi);
    aP, phi, the reference's p' and every solve's iteration count and residual
    are stored as arrays."""
    import hashlib

    c = R.cavity(N, mu=0.01, n_outer=n_outer, n_record=1, precond=0, tol=1e-8, max_it=1000, record_stride=n_outer)
    digest = lambda a: hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()  # noqa: E731
    np.savez_compressed(os.path.join(HERE, name), N=np.array(N), n_outer=np.array(n_outer),
                        recorded=np.array([0, n_outer - 1]),
                        pattern_sha256=np.array(digest(c["rowPtr"]) + digest(c["colIdx"])),
                        values_sha256=np.array([digest(v) for v in c["values"]]),
                        rhs_sha256=np.array([digest(v) for v in c["rhs"]]),
                        x=c["x"], aP=c["aP"], phi=c["phi"], iters=c["iters"], res=c["res"],
                        p_solve_seconds=np.array(c["p_solve_seconds"]))


def simplec_case(name):
    """SIMPLEC assembly (PvCouplingVariant::SIMPLEC) on a distorted 6x5x4 box
    with an outlet on zone 1, seeded aP, momentum values and fluxes; some
    cells' off-diagonal sums exceed aP (the 1e-30 clamp)."""
    dims = (6, 5, 4)
    shift = W.interior_node_shift(*dims, amp=0.2, seed=11)
    m = O.cartesian_mesh(*dims, node_shift=shift)
    rp, ci = O.build_sparsity(m)
    rng = np.random.default_rng(11)
    aP = rng.uniform(1.0, 3.0, m.nC)
    mom = rng.standard_normal(len(ci)) * 0.4
    phi = rng.standard_normal(m.nF)
    phi[m.neighbor < 0] = 0.0
    bcs = [(1, 7)] + [(z, 1) for z in range(2, 7)]
    rm = R.cartesian_mesh(*dims, node_shift=shift)
    rrp, rci, rv, rrhs = R.assemble_simplec(rm, bcs, 1.3, aP, mom, phi)
    np.savez_compressed(os.path.join(HERE, name), dims=np.array(dims), seed=np.array(11), aP=aP, mom=mom, phi=phi,
                        rho=np.array(1.3), rowPtr=rrp, colIdx=rci, values=rv, rhs=rrhs)


def field_loops_case(name):
    """compute_face_fluxes, LeastSquaresGradient::evaluate and correct_fields
    of the reference on a distorted, RCM-renumbered 7x6x5 box with every
    boundary treatment of the flux loop."""
    dims = (7, 6, 5)
    shift = W.interior_node_shift(*dims, amp=0.2, seed=13)
    rm = R.cartesian_mesh(*dims, node_shift=shift, do_rcm=True)
    rng = np.random.default_rng(13)
    nC, nF = rm["nC"], rm["nF"]
    U = [rng.standard_normal(nC) for _ in range(3)]
    bcs = [(1, 4, (0.7, -0.2, 0.1)), (2, 7), (3, 1), (4, 2, (1.0, 0.0, 0.0)), (5, 9), (6, 3)]
    phi = R.face_fluxes(rm, bcs, 1.2, U)
    f = rng.standard_normal(nC)
    g = R.lsq_gradient(rm, f)
    aP = rng.uniform(0.5, 2.0, nC)
    pp = rng.standard_normal(nC) * 1e-2
    p0 = rng.standard_normal(nC)
    p1, U1, phi1 = R.correct_fields(rm, 1.2, 0.3, aP, pp, p0, U, phi)
    np.savez_compressed(os.path.join(HERE, name), dims=np.array(dims), seed=np.array(13),
                        bc_zone=np.array([b[0] for b in bcs]), bc_type=np.array([b[1] for b in bcs]),
                        bc_vec=np.array([list(b[2]) if len(b) > 2 else [0.0, 0.0, 0.0] for b in bcs]),
                        rho=np.array(1.2), urfP=np.array(0.3), U=np.array(U), phi=phi, f=f, grad=g, aP=aP,
                        pPrime=pp, p0=p0, p1=p1, U1=np.array(U1), phi1=phi1)


MOM_BCS = [(1, 4, (0.7, -0.2, 0.1)), (2, 7), (3, 1), (4, 2, (1.0, 0.3, 0.0)), (5, 9), (6, 3)]


def momentum_case(name):
    """assemble_momentum of the reference (three components, BDF2 step) on a
    distorted, RCM-renumbered 7x6x5 box with every boundary treatment, and the
    reference's GMRES(5)+ILU(0) and BiCGSTAB+Jacobi solves of the x system."""
    dims = (7, 6, 5)
    shift = W.interior_node_shift(*dims, amp=0.2, seed=17)
    rm = R.cartesian_mesh(*dims, node_shift=shift, do_rcm=True)
    rng = np.random.default_rng(17)
    nC = rm["nC"]
    U = rng.standard_normal((3, nC))
    p = rng.standard_normal(nC)
    Un = rng.standard_normal((3, nC))
    Unm1 = rng.standard_normal((3, nC))
    phi = R.face_fluxes(rm, MOM_BCS, 1.1, U)
    opt = np.array([1.1, 0.013, 0.7, 0.05])
    vals, rhs = [], []
    for comp in range(3):
        v, b, aP = R.assemble_momentum(rm, MOM_BCS, opt, comp, U, p, phi, Un, Unm1, bdf2=True, time_step=1)
        vals.append(v)
        rhs.append(b)
        if comp == 0:
            aP0 = aP
    rp, ci, _, _ = R.assemble(rm, [], 1.0, np.ones(nC), np.zeros(rm["nF"]))
    xg, itg, lg, _ = R.krylov(0, rp, ci, vals[0], rhs[0], 1, 1e-10, 200, 5)
    xb, itb, lb, _ = R.krylov(1, rp, ci, vals[0], rhs[0], 0, 1e-10, 200)
    np.savez_compressed(os.path.join(HERE, name), dims=np.array(dims), seed=np.array(17),
                        bc_zone=np.array([b[0] for b in MOM_BCS]), bc_type=np.array([b[1] for b in MOM_BCS]),
                        bc_vec=np.array([list(b[2]) if len(b) > 2 else [0.0, 0.0, 0.0] for b in MOM_BCS]),
                        opt=opt, U=U, p=p, Un=Un, Unm1=Unm1, phi=phi, rowPtr=rp, colIdx=ci, values=np.array(vals),
                        rhs=np.array(rhs), aP=aP0, x_gmres=xg, it_gmres=np.array(itg), last_gmres=np.array(lg),
                        x_bicgstab=xb, it_bicgstab=np.array(itb), last_bicgstab=np.array(lb))


CAVITY_BCS = [(z, 1) for z in (1, 2, 3, 5, 6)] + [(4, 2, (1.0, 0.0, 0.0))]
CHANNEL_BCS = [(1, 4, (1.0, 0.1, 0.0)), (2, 7), (3, 1), (4, 1), (5, 9), (6, 0)]
# periodic in x (zones 1, 2) and z (5, 6), no-slip floor, lid moving in x
PERIODIC_BCS = [(1, 11), (2, 11), (3, 1), (4, 2, (1.0, 0.0, 0.0)), (5, 11), (6, 11)]
# name: dims, node-shift amplitude (seed 31), RCM, boundary specs, SimpleOptions and solver configs, outer calls, inner
SIMPLE_RUNS = {
    "simple_cavity_64_gmres_ilu.npz": ((64, 64, 1), 0.0, False, CAVITY_BCS,
                                       dict(mu=0.01, mom_cfg=(0, 1, 1e-6, 200, 30), p_cfg=(2, 0, 1e-8, 1000, 30)),
                                       20, 1),
    "simple_channel_8x6x5_simplec.npz": ((8, 6, 5), 0.2, True, CHANNEL_BCS,
                                         dict(mu=0.1, simplec=True, urfP=0.9, mom_cfg=(1, 0, 1e-8, 200, 30),
                                              p_cfg=(2, 1, 1e-9, 1000, 30)), 5, 1),
    "simple_cavity_12_bdf2.npz": ((12, 12, 1), 0.0, False, CAVITY_BCS,
                                  dict(mu=0.01, dt=0.01, bdf2=True, mom_cfg=(0, 0, 1e-8, 200, 5),
                                       p_cfg=(2, 0, 1e-9, 1000, 30)), 3, 2),
    "simple_periodic_couette_8x6x4.npz": ((8, 6, 4), 0.15, True, PERIODIC_BCS,
                                          dict(mu=0.05, mom_cfg=(0, 1, 1e-8, 200, 30), p_cfg=(2, 0, 1e-9, 1000, 30)),
                                          6, 1),
}


def simple_case(name):
    """The reference's SimpleAlgorithm from rest: U, p, phi, the residuals of
    every outer call and every linear solve's iteration count."""
    import json

    dims, amp, renumber, bcs, kw, n_outer, n_inner = SIMPLE_RUNS[name]
    shift = W.interior_node_shift(*dims, amp=amp, seed=31) if amp else None
    rm = R.cartesian_mesh(*dims, node_shift=shift, do_rcm=renumber)
    nC = rm["nC"]
    out = R.simple_run(rm, bcs, np.zeros((3, nC)), np.zeros(nC), n_outer, n_inner=n_inner, **kw)
    np.savez_compressed(os.path.join(HERE, name), dims=np.array(dims), amp=np.array(amp),
                        renumber=np.array(renumber), bc_zone=np.array([b[0] for b in bcs]),
                        bc_type=np.array([b[1] for b in bcs]),
                        bc_vec=np.array([list(b[2]) if len(b) > 2 else [0.0, 0.0, 0.0] for b in bcs]),
                        options=np.array(json.dumps(kw)), n_outer=np.array(n_outer), n_inner=np.array(n_inner),
                        U=out["U"], p=out["p"], phi=out["phi"], res=out["res"], iters=out["iters"])


def checkpoint_case(name):
    """io::Checkpoint::write of the reference: a distorted 4x3x2 box, scalar
    fields "p" and "T" and vector field "U" (inserted in that order), meta
    iteration 17, time 0.125, settings hash 0x123456789abcdef0; the file and,
    beside it, the arrays it holds."""
    dims = (4, 3, 2)
    shift = W.interior_node_shift(*dims, amp=0.2, seed=23)
    rm = R.cartesian_mesh(*dims, node_shift=shift)
    rng = np.random.default_rng(23)
    nC = rm["nC"]
    p, T, U = rng.standard_normal(nC), rng.standard_normal(nC), rng.standard_normal((3, nC))
    path = os.path.join(HERE, name + ".simallcp")
    assert R.checkpoint_write(rm, path, [("p", False, p), ("T", False, T), ("U", True, U)], 17, 0.125,
                              0x123456789ABCDEF0) == 0
    np.savez_compressed(os.path.join(HERE, name + ".npz"), dims=np.array(dims), seed=np.array(23), p=p, T=T, U=U,
                        **{k: rm[k] for k in ("nx", "ny", "nz", "owner", "neighbor", "ax", "ay", "az", "fcx", "fcy",
                                              "fcz", "zone", "fnOff", "fnIdx", "vol", "ccx", "ccy", "ccz", "cfOff",
                                              "cfIdx")})


def simp_case(name):
    """SimpTopology::initialize + three step() calls of the reference on a
    distorted, RCM-renumbered 7x6x5 box, without and with the Helmholtz filter,
    for seeded negative sensitivities."""
    dims = (7, 6, 5)
    shift = W.interior_node_shift(*dims, amp=0.2, seed=51)
    rm = R.cartesian_mesh(*dims, node_shift=shift, do_rcm=True)
    rng = np.random.default_rng(52)
    dC = -np.abs(rng.standard_normal((3, rm["nC"]))) * 0.1
    out = {"dims": np.array(dims), "seed": np.array(51), "dC": dC}
    for tag, radius in (("r0", 0.0), ("r3", 0.3)):
        cfg = np.array([3.0, 1e-9, 1.0, radius, 0.4, 0.2, 0.5, 1e-3])
        ch, rho, rt, K, dct = R.simp_run(rm, cfg, dC)
        out.update({f"{tag}_cfg": cfg, f"{tag}_change": ch, f"{tag}_rho": rho, f"{tag}_rhoTilde": rt,
                    f"{tag}_K": K, f"{tag}_dCt": dct})
    np.savez_compressed(os.path.join(HERE, name), **out)


PISO_PIMPLE_RUNS = {
    # name: dims, node-shift amplitude (seed 61), RCM, specs, variant (1 PISO, 2 PIMPLE), loops, options, steps
    "piso_cavity_12.npz": ((12, 12, 1), 0.0, False, CAVITY_BCS, 1, (1, 2, 1, 1), dict(mu=0.01, dt=0.01), 3),
    "pimple_channel_8x6x5.npz": ((8, 6, 5), 0.2, True, CHANNEL_BCS, 2, (3, 2, 0, 1),
                                 dict(mu=0.05, dt=0.02, urfU=0.7, urfP=0.3, tol_u=1e-6, tol_p=0.15), 3),
}


def piso_pimple_case(name):
    """PisoAlgorithm / PimpleAlgorithm of the reference from rest, BDF2 time
    steps of advance_time_step(1), GMRES(30)+Jacobi momentum and CG+Jacobi
    pressure: U, p, phi, residuals and PIMPLE's outer-exit index per step."""
    import json

    dims, amp, renumber, bcs, variant, loops, kw, steps = PISO_PIMPLE_RUNS[name]
    shift = W.interior_node_shift(*dims, amp=amp, seed=61) if amp else None
    rm = R.cartesian_mesh(*dims, node_shift=shift, do_rcm=renumber)
    nC = rm["nC"]
    out = R.piso_pimple_run(rm, variant, bcs, np.zeros((3, nC)), np.zeros(nC), steps, loops=loops, **kw)
    np.savez_compressed(os.path.join(HERE, name), dims=np.array(dims), amp=np.array(amp),
                        renumber=np.array(renumber), bc_zone=np.array([b[0] for b in bcs]),
                        bc_type=np.array([b[1] for b in bcs]),
                        bc_vec=np.array([list(b[2]) if len(b) > 2 else [0.0, 0.0, 0.0] for b in bcs]),
                        variant=np.array(variant), loops=np.array(loops), options=np.array(json.dumps(kw)),
                        steps=np.array(steps), U=out["U"], p=out["p"], phi=out["phi"], res=out["res"],
                        last_outer=out["last_outer"])


def adjoint_case(name):
    """solve_discrete_adjoint on a small face-conductance Poisson system."""
    nx, ny, nz = 5, 4, 3
    m = O.cartesian_mesh(nx, ny, nz, node_shift=W.interior_node_shift(nx, ny, nz, amp=0.1, seed=9))
    rp, ci = O.build_sparsity(m)
    rng = np.random.default_rng(9)
    dirichlet = ((m.neighbor < 0) & (m.zone == 1)).astype(np.uint8)
    k = np.exp(0.5 * rng.standard_normal(m.nF))
    k[(m.neighbor < 0) & (dirichlet == 0)] = 0.0
    pb = np.where(dirichlet == 1, rng.standard_normal(m.nF), 0.0)
    src = rng.standard_normal(m.nC)
    v, rhs, g = O.assemble_face_k(m, rp, ci, dirichlet, 1.0, k, pb, src)
    x, it, last = O.cg(rp, ci, v, rhs, 0, 1e-14, 5000)
    xt = rng.standard_normal(m.nC)
    dJdQ = x - xt
    psi, grad, its, res, rc = R.discrete_adjoint(rp, ci, v, dJdQ, m.owner, m.neighbor, dirichlet, g, k, pb, x,
                                                 tol=1e-13, max_iter=2000, restart=30)
    np.savez_compressed(os.path.join(HERE, name), dims=np.array([nx, ny, nz]), k=k, pb=pb, src=src,
                        dirichlet=dirichlet, xt=xt, rowPtr=rp, colIdx=ci, values=v, rhs=rhs, g=g, x=x, psi=psi,
                        grad=grad, iters=np.array(its), residual=np.array(res), ok=np.array(rc))


def solvers_case(name):
    """SSOR and AMG (apply, CG), TFQMR, and GMRES/BiCGSTAB with SSOR and AMG
    on a distorted, RCM-renumbered 7x6x5 pressure system and on the 40-point
    upwind convection-diffusion matrix of tests/unit/solver/test_tfqmr_solver.cpp."""
    dims, seed = (7, 6, 5), 71
    m = R.cartesian_mesh(*dims, node_shift=W.interior_node_shift(*dims, amp=0.2, seed=seed), do_rcm=True)
    rng = np.random.default_rng(seed)
    aP = rng.uniform(0.5, 2.0, m["nC"])
    phi = rng.standard_normal(m["nF"])
    phi[m["neighbor"] < 0] = 0.0
    rp, ci, v, rhs = R.assemble(m, [], 1.0, aP, phi)
    R.free_mesh(m)
    out = {"rowPtr": rp, "colIdx": ci, "values": v, "rhs": rhs}
    r = rng.standard_normal(len(rhs))
    out["apply_r"] = r
    for pc, tag in ((2, "ssor"), (3, "amg")):
        out[f"apply_{tag}_z"] = R.precond_apply(pc, rp, ci, v, r)
        x, it, last, _ = R.cg(rp, ci, v, rhs, pc, 1e-10, 500)
        out[f"cg_{tag}_x"], out[f"cg_{tag}_iters"], out[f"cg_{tag}_last"] = x, np.array(it), np.array(last)
    for pc, tag in ((1, "ilu0"), (2, "ssor")):
        x, it, last, _ = R.krylov(3, rp, ci, v, rhs, pc, 1e-8, 300)
        out[f"tfqmr_{tag}_x"], out[f"tfqmr_{tag}_iters"], out[f"tfqmr_{tag}_last"] = x, np.array(it), np.array(last)
    n = 40
    crp, cci, cv = [0], [], []
    for i in range(n):
        for j, a in ((i - 1, -6.0), (i, 7.0), (i + 1, -1.0)):
            if 0 <= j < n:
                cci.append(j)
                cv.append(a)
        crp.append(len(cci))
    crp, cci, cv = np.array(crp, np.int32), np.array(cci, np.int32), np.array(cv)
    cb = np.ones(n)
    out.update(cd_rowPtr=crp, cd_colIdx=cci, cd_values=cv)
    for kind, ktag in ((0, "gmres"), (1, "bicgstab")):
        for pc, tag in ((2, "ssor"), (3, "amg")):
            x, it, last, _ = R.krylov(kind, crp, cci, cv, cb, pc, 1e-8, 500, 30)
            key = f"cd_{ktag}_{tag}"
            out[key + "_x"], out[key + "_iters"], out[key + "_last"] = x, np.array(it), np.array(last)
    np.savez_compressed(os.path.join(HERE, name), **out)


def periodic_case(name):
    """Periodic faces (SimpleAlgorithm.cpp:101-186 pairing, :71-72 sparsity,
    :214-219 fluxes, :275-282 momentum, :411-419 pressure assembly) on a
    distorted, RCM-renumbered 8x6x5 channel periodic in x and z: the
    reference's twin table, CSR, assembled values and rhs, face fluxes and
    x-momentum values / rhs / aP."""
    dims, seed = (8, 6, 5), 41
    shift = W.interior_node_shift(*dims, amp=0.2, seed=seed)
    rm = R.cartesian_mesh(*dims, node_shift=shift, do_rcm=True)
    rng = np.random.default_rng(seed)
    nC, nF = rm["nC"], rm["nF"]
    aP = rng.uniform(0.5, 2.0, nC)
    phi = rng.standard_normal(nF)
    U = rng.standard_normal((3, nC))
    p = rng.standard_normal(nC)
    twin = R.periodic_twins(rm, PERIODIC_BCS)
    rp, ci, v, rhs = R.assemble(rm, [(b[0], b[1]) for b in PERIODIC_BCS], 1.1, aP, phi)
    flux = R.face_fluxes(rm, PERIODIC_BCS, 1.2, U)
    mv, mr, maP = R.assemble_momentum(rm, PERIODIC_BCS, (1.0, 0.02, 0.7, 0.0), 0, U, p, flux)
    np.savez_compressed(os.path.join(HERE, name), dims=np.array(dims), seed=np.array(seed), amp=np.array(0.2),
                        bc_zone=np.array([b[0] for b in PERIODIC_BCS]), bc_type=np.array([b[1] for b in PERIODIC_BCS]),
                        aP=aP, phi=phi, U=U, p=p, twin=twin, rowPtr=rp, colIdx=ci, values=v, rhs=rhs, flux=flux,
                        mom_values=mv, mom_rhs=mr, mom_aP=maP)


def cggpu_case(name):
    """gpu::CgGpu::set_matrix + solve (src/gpu/CgGpu.cpp:35-238, the GPU
    facade's host path) on the cases of tests/helpers.py:cggpu_cases: cold and
    warm starts, every preconditioner, relativeOrders, b = 0, maxIterations 0
    and 5, the ILU0 -> Jacobi fall-back and the p.q breakdown.  Stores each
    case's x and stats."""
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from helpers import cggpu_cases

    out = {}
    for cname, rp, ci, v, b, x0, pc, tol, mi, ro in cggpu_cases(O):
        x, st = R.cggpu(rp, ci, v, b, x0, pc, tol, mi, ro)
        out[cname + "_x"] = x
        out[cname + "_stats"] = np.array([st["iterations"], st["final_residual"], st["initial_residual"],
                                          float(st["converged"]), st["precond_after"], st["last_residual"]])
    np.savez_compressed(os.path.join(HERE, name), **out)


# ---------------------------------------------------------------- benchmark sizes
# The workloads the benchmark times, solved by the reference itself.  Inputs are
# regenerated from their seeds by the tests (simall_gb300.workloads), so only
# digests of the assembled systems and summaries of the solutions are stored:
# the iteration count, last_residual, ||x||_2, sum(x), x.w for a seeded
# w ~ N(0,1) and every `stride`-th entry of x.

def _digest(a):
    import hashlib

    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def _x_summary(x, stride, seed):
    w = np.random.default_rng(seed).standard_normal(len(x))
    return {"x_norm": np.array(np.linalg.norm(x)), "x_sum": np.array(x.sum()), "x_dot_w": np.array(x @ w),
            "x_sample": np.ascontiguousarray(x[::stride]), "x_stride": np.array(stride), "w_seed": np.array(seed)}


def poisson3d_full_case(name, n=128, seed=W.DEFAULT_SEED, tol=1e-8, max_it=50000):
    """The 3-D pressure Poisson of the benchmark: n^3 box, interior nodes shifted
    by U(-0.2,0.2)h, RCM (the reference's renumber_cells_cuthill_mckee), aP = 1,
    interior face fluxes N(0,1), all walls (cell-0 pin); CGSolver::solve with
    Jacobi and with ILU0 to 1e-8."""
    import time

    shift = W.interior_node_shift(n, n, n, seed=seed)
    m = R.cartesian_mesh(n, n, n, node_shift=shift, do_rcm=True)
    rng = np.random.default_rng(seed + 1)  # workloads.poisson3d_inputs
    phi = rng.standard_normal(m["nF"])
    phi[m["neighbor"] < 0] = 0.0
    rp, ci, v, rhs = R.assemble(m, W.ALL_WALLS, 1.0, np.ones(m["nC"]), phi)
    R.free_mesh(m)
    out = {"n": np.array(n), "seed": np.array(seed), "tol": np.array(tol), "nnz": np.array(len(ci)),
           "pattern_sha256": np.array(_digest(rp) + _digest(ci)), "values_sha256": np.array(_digest(v)),
           "rhs_sha256": np.array(_digest(rhs)), "rcm_stats": np.array(m["rcm_stats"])}
    xs = {}
    for pc, tag in ((0, "jacobi"), (1, "ilu0")):
        t = time.perf_counter()
        x, it, last, _ = R.cg(rp, ci, v, rhs, pc, tol, max_it)
        xs[tag] = x
        out[f"{tag}_seconds"] = np.array(time.perf_counter() - t)
        out[f"{tag}_iters"] = np.array(it)
        out[f"{tag}_last"] = np.array(last)
        out.update({f"{tag}_{k}": a for k, a in _x_summary(x, 256, seed + 11).items()})
        print(f"{name}: {tag} {it} iterations, last {last:.3e}, {out[f'{tag}_seconds']:.1f} s", flush=True)
    # the reference's own tight solve: how far each 1e-8 solution is from it
    xt, it, last, _ = R.cg(rp, ci, v, rhs, 1, 1e-13, max_it)
    out.update({f"tight_{k}": a for k, a in _x_summary(xt, 256, seed + 11).items()})
    out["tight_iters"], out["tight_last"] = np.array(it), np.array(last)
    for tag in xs:
        out[f"{tag}_err_vs_tight"] = np.array(np.linalg.norm(xs[tag] - xt) / np.linalg.norm(xt))
    print(f"{name}: tight ILU0 {it} iterations; errors vs tight: "
          + ", ".join(f"{t} {float(out[t + '_err_vs_tight']):.2e}" for t in xs), flush=True)
    np.savez_compressed(os.path.join(HERE, name), **out)


def varcoef_full_case(name, n=256, seed=W.DEFAULT_SEED, tol=1e-8, max_it=50000):
    """The mixed-versus-FP64 workload: n^3 box, aP = 1/k with k = exp(N(0,1))
    per cell (harmonic faces), PressureOutlet on x = 0, walls elsewhere, rhs
    N(0,1); CGSolver::solve with Jacobi to 1e-8 (the FP64 solve the mixed
    precision error is reported against)."""
    import time

    m = R.cartesian_mesh(n, n, n)
    rng = np.random.default_rng(seed + 2)  # workloads.varcoef_inputs
    k = W.portable_exp(rng.standard_normal(m["nC"]))
    b = rng.standard_normal(m["nC"])
    rp, ci, v, rhs = R.assemble(m, W.X0_OUTLET, 1.0, 1.0 / k, np.zeros(m["nF"]))
    R.free_mesh(m)
    del m, rhs
    t = time.perf_counter()
    x, it, last, _ = R.cg(rp, ci, v, b, 0, tol, max_it)
    secs = time.perf_counter() - t
    print(f"{name}: {it} iterations, last {last:.3e}, {secs:.1f} s", flush=True)
    np.savez_compressed(os.path.join(HERE, name), n=np.array(n), seed=np.array(seed), tol=np.array(tol),
                        nnz=np.array(len(ci)), pattern_sha256=np.array(_digest(rp) + _digest(ci)),
                        values_sha256=np.array(_digest(v)), b_sha256=np.array(_digest(b)), jacobi_iters=np.array(it),
                        jacobi_last=np.array(last), jacobi_seconds=np.array(secs),
                        **{f"jacobi_{k}": a for k, a in _x_summary(x, 2048, seed + 12).items()})


def _batched_one(args):
    side, b, tol, max_it = args
    R1 = O.RefLib()
    m = R1.cartesian_mesh(side, side, 1, 1.0, 1.0, 1.0 / side)
    rp, ci, v, _ = R1.assemble(m, W.ALL_WALLS, 1.0, np.ones(m["nC"]), np.zeros(m["nF"]))
    R1.free_mesh(m)
    x, it, last, _ = R1.cg(rp, ci, v, b, 0, tol, max_it)
    return _digest(v), it, last, x


def batched_full_case(name, count=512, seed=W.DEFAULT_SEED, tol=1e-8, max_it=50000, samples=16):
    """The batched workload: `count` cavity pressure systems with sides
    log-uniform in [32, 256] (workloads.batched_cavity_systems: extent
    1 x 1 x 1/side, all walls, aP = 1), rhs N(0,1) with the mean removed and the
    pinned cell zeroed; each solved by its own CGSolver::solve with Jacobi to
    1e-8.  Per system: the values digest, iterations, last_residual, ||x||,
    x.w (w ~ N(0,1) from seed + 13 + system index) and `samples` entries at a
    stride of n // samples."""
    import multiprocessing as mp

    sides = W.batched_sides(count, seed=seed)
    rng = np.random.default_rng(seed + 5)
    rhs = [W.batched_rhs(int(s) * int(s), rng) for s in sides]
    with mp.get_context("spawn").Pool(os.cpu_count()) as pool:
        res = pool.map(_batched_one, [(int(s), b, tol, max_it) for s, b in zip(sides, rhs)], chunksize=1)
    xs = [r[3] for r in res]
    dots = [float(x @ np.random.default_rng(seed + 13 + i).standard_normal(len(x))) for i, x in enumerate(xs)]
    smp = np.stack([x[::len(x) // samples][:samples] for x in xs])
    np.savez_compressed(os.path.join(HERE, name), count=np.array(count), seed=np.array(seed), tol=np.array(tol),
                        sides=sides, values_sha256=np.array([r[0] for r in res]),
                        iters=np.array([r[1] for r in res]), last=np.array([r[2] for r in res]),
                        x_norm=np.array([np.linalg.norm(x) for x in xs]), x_dot_w=np.array(dots), x_sample=smp)
    print(f"{name}: {count} systems, {sum(r[1] for r in res)} iterations in all", flush=True)


def adjoint_full_case(name, n=24, seed=W.DEFAULT_SEED):
    """solve_discrete_adjoint (GMRES(30) on A^T, left Jacobi) on the
    differentiation workload's face-conductance Poisson at n^3 (undistorted
    box, k_f = exp(N(0,0.5)) on interior and x = 0 faces, Dirichlet values
    N(0,1) on x = 0, cell source N(0,1): workloads.facek_inputs), with
    L = 0.5 |x - x_t|^2, x_t the solution for the conductances of seed + 1.
    The assembly is the oracle's face-conductance restatement; the adjoint and
    the gradient contraction are the reference's."""
    m = O.cartesian_mesh(n, n, n)
    rp, ci = O.build_sparsity(m)

    def inputs(s):
        rng = np.random.default_rng(s + 4)  # workloads.facek_inputs on this mesh
        k = W.portable_exp(0.5 * rng.standard_normal(m.nF))
        pb = rng.standard_normal(m.nF)
        dirichlet = (m.neighbor < 0) & (m.zone == 1)
        k[(m.neighbor < 0) & ~dirichlet] = 0.0
        pb[~dirichlet] = 0.0
        return k, pb, dirichlet.astype(np.uint8), rng.standard_normal(m.nC)

    k, pb, dirichlet, src = inputs(seed)
    kt = inputs(seed + 1)[0]
    vt, rhst, _ = O.assemble_face_k(m, rp, ci, dirichlet, 1.0, kt, pb, src)
    xt, _, _ = O.cg(rp, ci, vt, rhst, 0, 1e-14, 20000)
    v, rhs, g = O.assemble_face_k(m, rp, ci, dirichlet, 1.0, k, pb, src)
    x, _, _ = O.cg(rp, ci, v, rhs, 0, 1e-14, 20000)
    psi, grad, its, res, rc = R.discrete_adjoint(rp, ci, v, x - xt, m.owner, m.neighbor, dirichlet, g, k, pb, x,
                                                 tol=1e-12, max_iter=50000, restart=30)
    print(f"{name}: GMRES {its} iterations, residual {res:.3e}, rc {rc}", flush=True)
    np.savez_compressed(os.path.join(HERE, name), n=np.array(n), seed=np.array(seed),
                        k_sha256=np.array(_digest(k)), pb_sha256=np.array(_digest(pb)),
                        src_sha256=np.array(_digest(src)), values_sha256=np.array(_digest(v)),
                        rhs_sha256=np.array(_digest(rhs)), xt=xt, psi=psi, grad=grad, iters=np.array(its),
                        residual=np.array(res), ok=np.array(rc))


FULL_SIZE = {
    "cggpu_cases.npz": cggpu_case,
    "periodic_channel_8x6x5.npz": periodic_case,
    "simple_periodic_couette_8x6x4.npz": simple_case,
    "poisson3d_128_cg.npz": poisson3d_full_case,
    "varcoef_256_cg.npz": varcoef_full_case,
    "batched_512_cg.npz": batched_full_case,
    "adjoint_face_k_24.npz": adjoint_full_case,
}


def main():
    if len(sys.argv) > 1:  # named fixtures only (the benchmark-size ones take minutes)
        for name in sys.argv[1:]:
            FULL_SIZE[name](name)
        return
    mesh_case("box_6x5x4_distorted.npz", (6, 5, 4), 1, 0.2, False, [(z, 1) for z in range(1, 7)], [])
    mesh_case("box_8x8x8_rcm_walls.npz", (8, 8, 8), 7, 0.2, True, [(z, 1) for z in range(1, 7)], [])
    mesh_case("box_9x7x5_rcm_outlet.npz", (9, 7, 5), 3, 0.2, True,
              [(1, 7)] + [(z, 1) for z in range(2, 7)], [1])
    mesh_case("cavity_16x16x1_mesh.npz", (16, 16, 1), 5, 0.0, False, [(z, 1) for z in range(1, 7)], [])
    cavity_case("cavity_simple_16.npz", 16, 6, 6)
    cavity_case_full_size("cavity_simple_128.npz", 128, 200)
    adjoint_case("adjoint_face_k_5x4x3.npz")
    simplec_case("simplec_6x5x4_outlet.npz")
    field_loops_case("field_loops_7x6x5_rcm.npz")
    momentum_case("momentum_7x6x5_rcm_bdf2.npz")
    for name in SIMPLE_RUNS:
        simple_case(name)
    checkpoint_case("checkpoint_4x3x2")
    simp_case("simp_7x6x5_rcm.npz")
    for name in PISO_PIMPLE_RUNS:
        piso_pimple_case(name)
    solvers_case("solvers_7x6x5_rcm.npz")
    cggpu_case("cggpu_cases.npz")
    periodic_case("periodic_channel_8x6x5.npz")
    print("fixtures written to", HERE)


if __name__ == "__main__":
    main()
