"""The hand-written adjoint: face-conductance assembly and gradient scatter
bit-identical to the oracle, gradient equal to the reference's
solve_discrete_adjoint gradient (golden fixture) and to central finite
differences; and a torch.autograd.Function built on the C ABI (tests only)."""
import os

import numpy as np
import pytest

from helpers import bits_equal, digest

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
OUTLET = None


def _bcs(sg):
    return [(1, int(sg.BCType.PressureOutlet))] + [(z, int(sg.BCType.NoSlipWall)) for z in range(2, 7)]


def _cfg(sg, tol):
    return sg.LinearSolverConfig(kind=sg.LinearSolverKind.CG, preconditioner=sg.PreconditionerKind.Jacobi,
                                 tolerance=tol, maxIterations=20000)


def _problem(sg, oracle, dims, seed, amp=0.1):
    from simall_gb300 import workloads as W

    sh = W.interior_node_shift(*dims, amp=amp, seed=seed)
    m = sg.cartesian(*dims, node_shift=sh)
    om = oracle.cartesian_mesh(*dims, node_shift=sh)
    k, pb, dirichlet, src = W.facek_inputs(m, seed=seed)
    return m, om, k, pb, dirichlet, src


def test_face_conductance_assembly_and_gradient_bit_exact(sg, ctx, oracle):
    m, om, k, pb, dirichlet, src = _problem(sg, oracle, (9, 7, 6), 4)
    ps = sg.PressureSystem(m, _bcs(sg), ctx=ctx)
    ps.assemble_face_conductance(1.0, k, pb, src)
    v, rhs = ps.download()
    rp, ci = oracle.build_sparsity(om)
    ov, orhs, g = oracle.assemble_face_k(om, rp, ci, dirichlet, 1.0, k, pb, src)
    assert bits_equal(v, ov) and bits_equal(rhs, orhs)
    rng = np.random.default_rng(0)
    x = rng.standard_normal(m.n_cells)
    lam = rng.standard_normal(m.n_cells)
    dk, dpb = ps.face_conductance_gradient(1.0, k, pb, x, lam)
    odk, odpb = oracle.face_k_gradient(om, dirichlet, g, k, pb, x, lam)
    assert bits_equal(dk, odk) and bits_equal(dpb, odpb)


def test_adjoint_matches_reference_discrete_adjoint_gradient(sg, ctx, oracle):
    """Against adjoint::solve_discrete_adjoint's gradient (GMRES on A^T, 1e-13)."""
    a = np.load(os.path.join(GOLD, "adjoint_face_k_5x4x3.npz"))
    from simall_gb300 import workloads as W
    dims = tuple(int(v) for v in a["dims"])
    m = sg.cartesian(*dims, node_shift=W.interior_node_shift(*dims, amp=0.1, seed=9))
    ps = sg.PressureSystem(m, _bcs(sg), ctx=ctx)
    ps.assemble_face_conductance(1.0, a["k"], a["pb"], a["src"])
    v, rhs = ps.download()
    assert bits_equal(v, a["values"]) and bits_equal(rhs, a["rhs"])
    s = sg.GpuCGSolver(_cfg(sg, 1e-14), ctx=ctx)
    x = ps.solve(s)
    lam, dk, dpb = ps.adjoint(s, 1.0, a["k"], a["pb"], x, x - a["xt"])
    nF = m.n_faces
    ref_dk = a["grad"][:nF]
    ref_dpb = a["grad"][nF:]
    scale = np.abs(ref_dk).max()
    assert np.max(np.abs(dk - ref_dk)) <= 1e-7 * scale
    assert np.max(np.abs(dpb[a["dirichlet"] == 1] - ref_dpb)) <= 1e-7 * np.abs(ref_dpb).max()
    assert np.linalg.norm(lam - a["psi"]) <= 1e-8 * np.linalg.norm(a["psi"])


def test_adjoint_matches_reference_discrete_adjoint_gradient_24(sg, ctx):
    """The differentiation workload's face-conductance system at 24^3 (13,824
    cells, 43,200 faces; k_f = exp(N(0,0.5)), Dirichlet N(0,1) on x = 0, seed
    42) against adjoint::solve_discrete_adjoint run by the reference (GMRES(30)
    on A^T to 1e-12, tests/golden/adjoint_face_k_24.npz)."""
    from simall_gb300 import workloads as W

    a = np.load(os.path.join(GOLD, "adjoint_face_k_24.npz"))
    n, seed = int(a["n"]), int(a["seed"])
    m = sg.cartesian(n, n, n)
    k, pb, dirichlet, src = W.facek_inputs(m, seed=seed)
    assert (digest(k), digest(pb), digest(src)) == (str(a["k_sha256"]), str(a["pb_sha256"]), str(a["src_sha256"]))
    ps = sg.PressureSystem(m, _bcs(sg), ctx=ctx)
    ps.assemble_face_conductance(1.0, k, pb, src)
    v, rhs = ps.download()
    assert digest(v) == str(a["values_sha256"]) and digest(rhs) == str(a["rhs_sha256"])
    s = sg.GpuCGSolver(_cfg(sg, 1e-14), ctx=ctx)
    x = ps.solve(s)
    lam, dk, dpb = ps.adjoint(s, 1.0, k, pb, x, x - a["xt"])
    nF = m.n_faces
    ref_dk, ref_dpb = a["grad"][:nF], a["grad"][nF:]
    assert np.max(np.abs(dk - ref_dk)) <= 1e-7 * np.abs(ref_dk).max()
    assert np.max(np.abs(dpb[dirichlet == 1] - ref_dpb)) <= 1e-7 * np.abs(ref_dpb).max()
    assert np.linalg.norm(lam - a["psi"]) <= 1e-8 * np.linalg.norm(a["psi"])
    s.close()
    ps.close()


def _loss(sg, ps, s, k, pb, src, xt):
    ps.assemble_face_conductance(1.0, k, pb, src)
    x = ps.solve(s)
    return 0.5 * float(np.dot(x - xt, x - xt)), x


def test_adjoint_gradient_matches_central_differences(sg, ctx, oracle):
    m, om, k, pb, dirichlet, src = _problem(sg, oracle, (10, 9, 8), 6)
    from simall_gb300 import workloads as W
    k2, _, _, _ = W.facek_inputs(m, seed=7)
    ps = sg.PressureSystem(m, _bcs(sg), ctx=ctx)
    s = sg.GpuCGSolver(_cfg(sg, 1e-14), ctx=ctx)
    _, xt = _loss(sg, ps, s, k2, pb, src, np.zeros(m.n_cells))
    L0, x = _loss(sg, ps, s, k, pb, src, xt)
    lam, dk, dpb = ps.adjoint(s, 1.0, k, pb, x, x - xt)
    rng = np.random.default_rng(11)
    active = np.flatnonzero(k > 0)
    faces = rng.choice(active, size=24, replace=False)
    dfaces = rng.choice(np.flatnonzero(dirichlet), size=8, replace=False)
    h = 1e-6
    for f in faces:
        kp, km = k.copy(), k.copy()
        kp[f] += h
        km[f] -= h
        fd = (_loss(sg, ps, s, kp, pb, src, xt)[0] - _loss(sg, ps, s, km, pb, src, xt)[0]) / (2 * h)
        assert abs(fd - dk[f]) <= 2e-5 * max(abs(dk[f]), 1e-3 * np.abs(dk).max()), (f, fd, dk[f])
    for f in dfaces:
        pp, pm = pb.copy(), pb.copy()
        pp[f] += h
        pm[f] -= h
        fd = (_loss(sg, ps, s, k, pp, src, xt)[0] - _loss(sg, ps, s, k, pm, src, xt)[0]) / (2 * h)
        assert abs(fd - dpb[f]) <= 2e-5 * max(abs(dpb[f]), 1e-3 * np.abs(dpb).max()), (f, fd, dpb[f])


def test_torch_autograd_wrapper(sg, ctx, oracle):
    """A torch.autograd.Function whose forward assembles and solves on the
    device and whose backward is the hand-written adjoint."""
    torch = pytest.importorskip("torch")
    m, om, k, pb, dirichlet, src = _problem(sg, oracle, (8, 8, 8), 12)
    ps = sg.PressureSystem(m, _bcs(sg), ctx=ctx)
    s = sg.GpuCGSolver(_cfg(sg, 1e-13), ctx=ctx)
    dev = torch.device("cuda:0")
    tsrc = torch.from_numpy(src).to(dev)

    class PressureSolve(torch.autograd.Function):
        @staticmethod
        def forward(fctx, tk, tpb):
            ps.assemble_face_conductance(1.0, tk, tpb, tsrc)
            x = torch.empty(m.n_cells, dtype=torch.float64, device=dev)
            ps.solve(s, x)
            ctx.synchronize()
            fctx.save_for_backward(tk, tpb, x)
            return x

        @staticmethod
        def backward(fctx, gx):
            tk, tpb, x = fctx.saved_tensors
            ps.assemble_face_conductance(1.0, tk, tpb, tsrc)  # operator for the transpose solve
            lam = torch.empty_like(x)
            dk = torch.empty_like(tk)
            dpb = torch.empty_like(tpb)
            ps.adjoint(s, 1.0, tk, tpb, x, gx.contiguous(), lam, dk, dpb)
            ctx.synchronize()
            return dk, dpb

    tk = torch.from_numpy(k).to(dev).requires_grad_(True)
    tpb = torch.from_numpy(pb).to(dev).requires_grad_(True)
    xt = torch.from_numpy(np.random.default_rng(3).standard_normal(m.n_cells)).to(dev)
    x = PressureSolve.apply(tk, tpb)
    loss = 0.5 * ((x - xt) ** 2).sum()
    loss.backward()
    ps.assemble_face_conductance(1.0, k, pb, src)
    xs = ps.solve(s)
    lam, dk, dpb = ps.adjoint(s, 1.0, k, pb, xs, xs - xt.cpu().numpy())
    assert np.allclose(tk.grad.cpu().numpy(), dk, rtol=1e-9, atol=1e-12 * np.abs(dk).max())
    assert np.allclose(tpb.grad.cpu().numpy(), dpb, rtol=1e-9, atol=1e-12 * max(np.abs(dpb).max(), 1e-30))
