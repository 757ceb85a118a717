"""ctypes wrapper over oracle/lib/liboracle.so -- TEST INFRASTRUCTURE.

The C restatement of the SimAll reference algorithms (oracle/simall_oracle.c)
exposed to numpy.  Only tests/, __graft_entry__.smoke() and bench.py's
CPU-baseline leg import this module; the product never does.

`RefLib` wraps oracle/_ref/libsimall_ref.so, the reference's own sources
compiled by oracle/build_ref.sh; it exists only where the reference tree was
present at build time.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from dataclasses import dataclass, field

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "lib", "liboracle.so")
REF_PATH = os.path.join(HERE, "_ref", "libsimall_ref.so")

_P = C.c_void_p
_I64 = C.c_int64
_I32 = C.c_int32
_D = C.c_double


def build_oracle() -> str:
    """Compile liboracle.so (make -C oracle)."""
    subprocess.run(["make", "-s", "-C", HERE], check=True)
    return LIB_PATH


def _ptr(a: np.ndarray | None):
    return None if a is None else a.ctypes.data_as(_P)


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build_oracle()
        L = C.CDLL(LIB_PATH)
        L.orc_cartesian_topology.restype = _I64
        L.orc_cartesian_topology.argtypes = [C.c_int, C.c_int, C.c_int, _D, _D, _D] + [_P] * 9
        L.orc_compute_geometry.restype = None
        L.orc_compute_geometry.argtypes = [_I64, _I64] + [_P] * 18
        L.orc_classify_zones.restype = None
        L.orc_classify_zones.argtypes = [_I64, _P, _P, _P, _P, _D, _D, _D, _P]
        L.orc_rcm.restype = None
        L.orc_rcm.argtypes = [_I64, _I64] + [_P] * 10
        L.orc_build_sparsity.restype = _I64
        L.orc_build_sparsity.argtypes = [_I64, _P, _P, _P, _P, _P, _P, _P]
        L.orc_face_fluxes.restype = None
        L.orc_face_fluxes.argtypes = [_I64] + [_P] * 6 + [_P, _P, C.c_int, _D] + [_P] * 5
        L.orc_lsq_inverse.restype = None
        L.orc_lsq_inverse.argtypes = [_I64, _I64] + [_P] * 9
        L.orc_lsq_gradient.restype = None
        L.orc_lsq_gradient.argtypes = [_I64, _I64] + [_P] * 13
        L.orc_correct_fields.restype = None
        L.orc_correct_fields.argtypes = [_I64, _I64] + [_P] * 12 + [_D, _D] + [_P] * 7
        L.orc_simplec_denominator.restype = None
        L.orc_simplec_denominator.argtypes = [_I64] + [_P] * 5
        L.orc_assemble.restype = C.c_int
        L.orc_assemble.argtypes = [_I64, _I64] + [_P] * 13 + [C.c_int, _D] + [_P] * 7
        L.orc_dot.restype = _D
        L.orc_dot.argtypes = [_I64, _P, _P]
        L.orc_spmv.restype = None
        L.orc_spmv.argtypes = [_I64, _P, _P, _P, _P, _P]
        L.orc_jacobi_setup.restype = None
        L.orc_jacobi_setup.argtypes = [_I64, _P, _P, _P, _P]
        L.orc_ilu0_setup.restype = None
        L.orc_ilu0_setup.argtypes = [_I64, _P, _P, _P, _P, _P]
        L.orc_ilu0_apply.restype = None
        L.orc_ilu0_apply.argtypes = [_I64, _P, _P, _P, _P, _P, _P, _P]
        L.orc_cg.restype = C.c_int
        L.orc_cg.argtypes = [_I64, _P, _P, _P, _P, C.c_int, _D, C.c_int, _P, _P, _P]
        L.orc_assemble_face_k.restype = None
        L.orc_assemble_face_k.argtypes = [_I64, _I64] + [_P] * 12 + [_D] + [_P] * 8
        L.orc_face_k_gradient.restype = None
        L.orc_face_k_gradient.argtypes = [_I64] + [_P] * 10
        L.orc_assemble_momentum.restype = None
        L.orc_assemble_momentum.argtypes = [_I64, _I64] + [_P] * 15 + [C.c_int] + [_P] * 3 + [C.c_int, C.c_int] + \
            [_P] * 8 + [_P]
        L.orc_bicgstab.restype = C.c_int
        L.orc_bicgstab.argtypes = [_I64, _P, _P, _P, _P, C.c_int, _D, C.c_int, _P, _P]
        L.orc_gmres.restype = C.c_int
        L.orc_tfqmr.restype = C.c_int
        L.orc_tfqmr.argtypes = [_I64, _P, _P, _P, _P, C.c_int, _D, C.c_int, _P, _P]
        L.orc_amg_digest.restype = C.c_uint64
        L.orc_amg_digest.argtypes = [_I64, _P, _P, _P, _P]
        L.orc_amg_probe.restype = None
        L.orc_amg_probe.argtypes = [_I64, _P, _P, _P, _P, _P, _P, _P, _P, _P]
        L.orc_ssor_setup.restype = None
        L.orc_ssor_setup.argtypes = [_I64, _P, _P, _P, _P, _P]
        L.orc_ssor_apply.restype = None
        L.orc_ssor_apply.argtypes = [_I64, _P, _P, _P, _P, _P, _D, _P, _P, _P, _P]
        L.orc_gmres.argtypes = [_I64, _P, _P, _P, _P, C.c_int, _D, C.c_int, C.c_int, _P, _P]
        L.orc_simple_iterate.restype = C.c_int
        L.orc_simple_iterate.argtypes = [_I64, _I64] + [_P] * 16 + [C.c_int] + [_P] * 3 + [C.c_int, _P, _D, _P, _D] + \
            [_P] * 11 + [_P]
        L.orc_simp_step.restype = _D
        L.orc_simp_step.argtypes = [_I64, _I64] + [_P] * 17
        L.orc_periodic_pairs.restype = None
        L.orc_periodic_pairs.argtypes = [_I64, _P, _P, _P, _P, _P, C.c_int, _P, _P]
        L.orc_gpu_ilu0_factor.restype = C.c_int
        L.orc_gpu_ilu0_factor.argtypes = [_I64, _P, _P, _P]
        L.orc_cggpu_solve.restype = None
        L.orc_cggpu_solve.argtypes = [C.c_int, _D, C.c_int, _D, _I64] + [_P] * 8
        _lib = L
    return _lib


# ---------------------------------------------------------------- mesh


@dataclass
class Mesh:
    """SoA mesh in the layout of meshing::Mesh (src/meshing/MeshStorage.hpp:37-105);
    neighbor == -1 marks a boundary face."""

    nC: int
    nF: int
    extent: tuple
    nx: np.ndarray
    ny: np.ndarray
    nz: np.ndarray
    fnOff: np.ndarray
    fnIdx: np.ndarray
    owner: np.ndarray
    neighbor: np.ndarray
    cfOff: np.ndarray
    cfIdx: np.ndarray
    ax: np.ndarray = field(default=None)
    ay: np.ndarray = field(default=None)
    az: np.ndarray = field(default=None)
    fcx: np.ndarray = field(default=None)
    fcy: np.ndarray = field(default=None)
    fcz: np.ndarray = field(default=None)
    zone: np.ndarray = field(default=None)
    vol: np.ndarray = field(default=None)
    ccx: np.ndarray = field(default=None)
    ccy: np.ndarray = field(default=None)
    ccz: np.ndarray = field(default=None)


def cartesian_mesh(Nx, Ny, Nz, ex=1.0, ey=1.0, ez=1.0, node_shift=None) -> Mesh:
    """CartesianMesher + ConnectivityBuilder + compute_geometry + zones.

    node_shift: optional (3, nNodes) array added to the node coordinates
    before the geometry is computed (the perturbation of a distorted mesh).
    """
    L = lib()
    nC = Nx * Ny * Nz
    nN = (Nx + 1) * (Ny + 1) * (Nz + 1)
    maxF = 6 * nC
    nx = np.empty(nN)
    ny = np.empty(nN)
    nz = np.empty(nN)
    fnOff = np.empty(maxF + 1, np.int32)
    fnIdx = np.empty(4 * maxF, np.int64)
    owner = np.empty(maxF, np.int64)
    neighbor = np.empty(maxF, np.int64)
    cfOff = np.empty(nC + 1, np.int32)
    cfIdx = np.empty(6 * nC, np.int64)
    nF = L.orc_cartesian_topology(Nx, Ny, Nz, ex, ey, ez, _ptr(nx), _ptr(ny), _ptr(nz), _ptr(fnOff),
                                  _ptr(fnIdx), _ptr(owner), _ptr(neighbor), _ptr(cfOff), _ptr(cfIdx))
    m = Mesh(nC, int(nF), (ex, ey, ez), nx, ny, nz, fnOff[: nF + 1].copy(), fnIdx[: 4 * nF].copy(),
             owner[:nF].copy(), neighbor[:nF].copy(), cfOff, cfIdx)
    if node_shift is not None:
        m.nx = m.nx + node_shift[0]
        m.ny = m.ny + node_shift[1]
        m.nz = m.nz + node_shift[2]
    # Zones are classified on the unperturbed geometry, as CartesianMesher does
    # before any node edit; boundary nodes are never shifted, so the boundary
    # face centroids are the same either way.
    compute_geometry(m)
    m.zone = np.empty(m.nF, np.uint32)
    L.orc_classify_zones(m.nF, _ptr(m.neighbor), _ptr(m.fcx), _ptr(m.fcy), _ptr(m.fcz), ex, ey, ez,
                         _ptr(m.zone))
    return m


def compute_geometry(m: Mesh) -> None:
    L = lib()
    for k in ("ax", "ay", "az", "fcx", "fcy", "fcz"):
        setattr(m, k, np.empty(m.nF))
    for k in ("vol", "ccx", "ccy", "ccz"):
        setattr(m, k, np.empty(m.nC))
    L.orc_compute_geometry(m.nC, m.nF, _ptr(m.nx), _ptr(m.ny), _ptr(m.nz), _ptr(m.fnOff), _ptr(m.fnIdx),
                           _ptr(m.owner), _ptr(m.cfOff), _ptr(m.cfIdx), _ptr(m.ax), _ptr(m.ay), _ptr(m.az),
                           _ptr(m.fcx), _ptr(m.fcy), _ptr(m.fcz), _ptr(m.vol), _ptr(m.ccx), _ptr(m.ccy),
                           _ptr(m.ccz))


def rcm(m: Mesh):
    """In-place reverse Cuthill-McKee; returns (newPos, (bwBefore, bwAfter, permuted))."""
    L = lib()
    newPos = np.empty(m.nC, np.int64)
    stats = np.zeros(3, np.int64)
    L.orc_rcm(m.nC, m.nF, _ptr(m.owner), _ptr(m.neighbor), _ptr(m.vol), _ptr(m.ccx), _ptr(m.ccy),
              _ptr(m.ccz), _ptr(m.cfOff), _ptr(m.cfIdx), _ptr(newPos), _ptr(stats))
    return newPos, tuple(int(s) for s in stats)


PERIODIC = 11  # BCType::Periodic (src/solver/Solver.hpp:105-123)


def periodic_pairs(m: Mesh, bcs):
    """SimpleAlgorithm::build_periodic_pairs (SimpleAlgorithm.cpp:101-186):
    twin[nF] (-1 where none); the periodic zones are those of the Periodic
    specs in bcs, in order."""
    zones = np.array([int(b[0]) for b in bcs if int(b[1]) == PERIODIC] or [0], np.uint32)
    nP = sum(1 for b in bcs if int(b[1]) == PERIODIC)
    twin = np.empty(m.nF, np.int32)
    lib().orc_periodic_pairs(m.nF, _ptr(m.neighbor), _ptr(m.zone), _ptr(m.fcx), _ptr(m.fcy), _ptr(m.fcz), nP,
                             _ptr(zones), _ptr(twin))
    return twin


def _twin(twin):
    return None if twin is None else np.ascontiguousarray(twin, np.int32)


def build_sparsity(m: Mesh, twin=None):
    L = lib()
    rowPtr = np.empty(m.nC + 1, np.int32)
    tw = _twin(twin)
    nnz = L.orc_build_sparsity(m.nC, _ptr(m.owner), _ptr(m.neighbor), _ptr(m.cfOff), _ptr(m.cfIdx),
                               _ptr(rowPtr), None, _ptr(tw))
    colIdx = np.empty(nnz, np.int32)
    L.orc_build_sparsity(m.nC, _ptr(m.owner), _ptr(m.neighbor), _ptr(m.cfOff), _ptr(m.cfIdx), _ptr(rowPtr),
                         _ptr(colIdx), _ptr(tw))
    return rowPtr, colIdx


def _zone_tables(bcs):
    """bcs: list of (zone, BCType ordinal[, (ux, uy, uz)]) -> per-zone type (first
    spec wins, as find_bc) and vector tables."""
    nZ = int(max([7] + [b[0] + 1 for b in bcs]))
    zt = np.full(nZ, -1, np.int32)
    zv = np.zeros(3 * nZ)
    for b in bcs:
        z = int(b[0])
        if zt[z] == -1:
            zt[z] = int(b[1])
            if len(b) > 2:
                zv[3 * z:3 * z + 3] = b[2]
    return nZ, zt, zv


def face_fluxes(m: Mesh, bcs, rho, U, twin=None):
    """compute_face_fluxes (SimpleAlgorithm.cpp:201-237); U = (Ux, Uy, Uz)."""
    nZ, zt, zv = _zone_tables(bcs)
    phi = np.empty(m.nF)
    Ux, Uy, Uz = (np.ascontiguousarray(u, np.float64) for u in U)
    lib().orc_face_fluxes(m.nF, _ptr(m.owner), _ptr(m.neighbor), _ptr(m.ax), _ptr(m.ay), _ptr(m.az), _ptr(m.zone),
                          _ptr(zt), _ptr(zv), nZ, float(rho), _ptr(Ux), _ptr(Uy), _ptr(Uz), _ptr(phi),
                          _ptr(_twin(twin)))
    return phi


def lsq_gradient(m: Mesh, phi):
    """LeastSquaresGradient precompute + evaluate (Gradient.cpp:17-133)."""
    L = lib()
    mInv = np.empty(6 * m.nC)
    L.orc_lsq_inverse(m.nC, m.nF, _ptr(m.owner), _ptr(m.neighbor), _ptr(m.fcx), _ptr(m.fcy), _ptr(m.fcz),
                      _ptr(m.ccx), _ptr(m.ccy), _ptr(m.ccz), _ptr(mInv))
    g = np.empty((3, m.nC))
    L.orc_lsq_gradient(m.nC, m.nF, _ptr(m.owner), _ptr(m.neighbor), _ptr(m.fcx), _ptr(m.fcy), _ptr(m.fcz),
                       _ptr(m.ccx), _ptr(m.ccy), _ptr(m.ccz), _ptr(mInv),
                       _ptr(np.ascontiguousarray(phi, np.float64)), _ptr(g[0]), _ptr(g[1]), _ptr(g[2]))
    return g


def correct_fields(m: Mesh, rho, urfP, aP, pPrime, p, U, phi):
    """correct_fields (SimpleAlgorithm.cpp:450-487); returns (p, (Ux, Uy, Uz), phi), inputs untouched."""
    p = np.array(p, np.float64)
    Ux, Uy, Uz = (np.array(u, np.float64) for u in U)
    phi = np.array(phi, np.float64)
    lib().orc_correct_fields(m.nC, m.nF, _ptr(m.owner), _ptr(m.neighbor), _ptr(m.ax), _ptr(m.ay), _ptr(m.az),
                             _ptr(m.fcx), _ptr(m.fcy), _ptr(m.fcz), _ptr(m.ccx), _ptr(m.ccy), _ptr(m.ccz),
                             _ptr(m.vol), float(rho), float(urfP), _ptr(np.ascontiguousarray(aP, np.float64)),
                             _ptr(np.ascontiguousarray(pPrime, np.float64)), _ptr(p), _ptr(Ux), _ptr(Uy), _ptr(Uz),
                             _ptr(phi))
    return p, (Ux, Uy, Uz), phi


def simplec_denominator(rowPtr, colIdx, mom, aP):
    """SIMPLEC per-cell denominator (SimpleAlgorithm.cpp:380-390)."""
    n = len(rowPtr) - 1
    den = np.empty(n)
    lib().orc_simplec_denominator(n, _ptr(np.ascontiguousarray(rowPtr, np.int32)),
                                  _ptr(np.ascontiguousarray(colIdx, np.int32)),
                                  _ptr(np.ascontiguousarray(mom, np.float64)),
                                  _ptr(np.ascontiguousarray(aP, np.float64)), _ptr(den))
    return den


def assemble(m: Mesh, rowPtr, colIdx, pressure_zones, rho, aP, phi, twin=None):
    """assemble_pressure_correction; pressure_zones = zone ids with a
    PressureOutlet/PressureInlet condition.  Returns (values, rhs, anyDirichlet)."""
    L = lib()
    nZ = int(max([7] + [z + 1 for z in pressure_zones]))
    isP = np.zeros(nZ, np.uint8)
    for z in pressure_zones:
        isP[z] = 1
    values = np.empty(len(colIdx))
    rhs = np.empty(m.nC)
    aP = np.ascontiguousarray(aP, np.float64)
    phi = np.ascontiguousarray(phi, np.float64)
    anyD = L.orc_assemble(m.nC, m.nF, _ptr(m.owner), _ptr(m.neighbor), _ptr(m.ax), _ptr(m.ay), _ptr(m.az),
                          _ptr(m.fcx), _ptr(m.fcy), _ptr(m.fcz), _ptr(m.zone), _ptr(m.ccx), _ptr(m.ccy),
                          _ptr(m.ccz), _ptr(isP), nZ, rho, _ptr(aP), _ptr(phi), _ptr(rowPtr), _ptr(colIdx),
                          _ptr(values), _ptr(rhs), _ptr(_twin(twin)))
    return values, rhs, bool(anyD)


def assemble_face_k(m: Mesh, rowPtr, colIdx, is_dirichlet_face, rho, k, pb, src):
    L = lib()
    values = np.empty(len(colIdx))
    rhs = np.empty(m.nC)
    g = np.empty(m.nF)
    isD = np.ascontiguousarray(is_dirichlet_face, np.uint8)
    k = np.ascontiguousarray(k, np.float64)
    pb = np.ascontiguousarray(pb, np.float64)
    src = np.ascontiguousarray(src, np.float64)
    L.orc_assemble_face_k(m.nC, m.nF, _ptr(m.owner), _ptr(m.neighbor), _ptr(m.ax), _ptr(m.ay), _ptr(m.az),
                          _ptr(m.fcx), _ptr(m.fcy), _ptr(m.fcz), _ptr(m.ccx), _ptr(m.ccy), _ptr(m.ccz),
                          _ptr(isD), rho, _ptr(k), _ptr(pb), _ptr(src), _ptr(rowPtr), _ptr(colIdx),
                          _ptr(values), _ptr(rhs), _ptr(g))
    return values, rhs, g


def face_k_gradient(m: Mesh, is_dirichlet_face, g, k, pb, x, lam):
    L = lib()
    dk = np.empty(m.nF)
    dpb = np.empty(m.nF)
    isD = np.ascontiguousarray(is_dirichlet_face, np.uint8)
    L.orc_face_k_gradient(m.nF, _ptr(m.owner), _ptr(m.neighbor), _ptr(isD), _ptr(g), _ptr(k), _ptr(pb),
                          _ptr(x), _ptr(lam), _ptr(dk), _ptr(dpb))
    return dk, dpb


# ---------------------------------------------------------------- linear algebra


def assemble_momentum(m: Mesh, rowPtr, colIdx, bcs, opt, comp, phi, gp, Ucomp, Un=None, Unm1=None, bdf2=False,
                      twin=None):
    """assemble_momentum (SimpleAlgorithm.cpp:240-355) for component comp;
    bcs as face_fluxes, opt = (rho, mu, urfU, dt), gp = that component of the
    pressure gradient.  Returns (values, rhs, relaxed diagonal)."""
    nZ, zt, zv = _zone_tables(bcs)
    nnz = int(rowPtr[-1])
    values = np.empty(nnz)
    rhs = np.empty(m.nC)
    aP = np.empty(m.nC)
    z = np.zeros(m.nC)
    a = [np.ascontiguousarray(v if v is not None else z, np.float64) for v in (phi, gp, Ucomp, Un, Unm1)]
    lib().orc_assemble_momentum(m.nC, m.nF, _ptr(m.owner), _ptr(m.neighbor), _ptr(m.ax), _ptr(m.ay), _ptr(m.az),
                                _ptr(m.fcx), _ptr(m.fcy), _ptr(m.fcz), _ptr(m.ccx), _ptr(m.ccy), _ptr(m.ccz),
                                _ptr(m.vol), _ptr(m.zone), _ptr(zt), _ptr(zv), nZ,
                                _ptr(np.ascontiguousarray(rowPtr, np.int32)),
                                _ptr(np.ascontiguousarray(colIdx, np.int32)),
                                _ptr(np.ascontiguousarray(opt, np.float64)), int(bool(bdf2)), int(comp),
                                *(_ptr(v) for v in a), _ptr(values), _ptr(rhs), _ptr(aP), _ptr(_twin(twin)))
    return values, rhs, aP


def bicgstab(rowPtr, colIdx, values, b, precond=0, tol=1e-8, max_it=1000):
    """BiCGSTABSolver::solve (LinearSolvers.cpp:363-405); returns (x, iterations, last)."""
    n = len(rowPtr) - 1
    x = np.empty(n)
    last = C.c_double(0)
    it = lib().orc_bicgstab(n, _ptr(np.ascontiguousarray(rowPtr, np.int32)),
                            _ptr(np.ascontiguousarray(colIdx, np.int32)),
                            _ptr(np.ascontiguousarray(values, np.float64)), _ptr(np.ascontiguousarray(b, np.float64)),
                            int(precond), float(tol), int(max_it), _ptr(x), C.byref(last))
    return x, it, last.value


def gmres(rowPtr, colIdx, values, b, precond=1, tol=1e-8, max_it=1000, restart=30):
    """GMRESmSolver::solve (LinearSolvers.cpp:268-343); returns (x, iterations, last)."""
    n = len(rowPtr) - 1
    x = np.empty(n)
    last = C.c_double(0)
    it = lib().orc_gmres(n, _ptr(np.ascontiguousarray(rowPtr, np.int32)), _ptr(np.ascontiguousarray(colIdx, np.int32)),
                         _ptr(np.ascontiguousarray(values, np.float64)), _ptr(np.ascontiguousarray(b, np.float64)),
                         int(precond), float(tol), int(max_it), int(restart), _ptr(x), C.byref(last))
    return x, it, last.value


def tfqmr(rowPtr, colIdx, values, b, precond=0, tol=1e-8, max_it=1000):
    """TfqmrSolver::solve (LinearSolvers.cpp:497-609); returns (x, iterations, last)."""
    n = len(rowPtr) - 1
    x = np.empty(n)
    last = C.c_double(0)
    it = lib().orc_tfqmr(n, _ptr(np.ascontiguousarray(rowPtr, np.int32)), _ptr(np.ascontiguousarray(colIdx, np.int32)),
                         _ptr(np.ascontiguousarray(values, np.float64)), _ptr(np.ascontiguousarray(b, np.float64)),
                         int(precond), float(tol), int(max_it), _ptr(x), C.byref(last))
    return x, it, last.value


def amg_apply(rowPtr, colIdx, values, r=None):
    """AMGPreconditioner setup + apply (src/solver/AMGPreconditioner.cpp)
    with make_preconditioner's defaults.  Returns (z or None, [(rows, nnz) of
    each level], coarsest size)."""
    n = len(rowPtr) - 1
    rp = np.ascontiguousarray(rowPtr, np.int32)
    ci = np.ascontiguousarray(colIdx, np.int32)
    v = np.ascontiguousarray(values, np.float64)
    z = None if r is None else np.empty(n)
    nlev = C.c_int(0)
    cn = C.c_int32(0)
    sizes = np.zeros(10, np.int32)
    nnzs = np.zeros(10, np.int32)
    lib().orc_amg_probe(n, _ptr(rp), _ptr(ci), _ptr(v), _ptr(None if r is None else np.ascontiguousarray(r, np.float64)),
                        _ptr(z), C.byref(nlev), _ptr(sizes), _ptr(nnzs), C.byref(cn))
    return z, [(int(sizes[l]), int(nnzs[l])) for l in range(nlev.value)], int(cn.value)


def amg_digest(rowPtr, colIdx, values):
    """(levels, digest) of the restated AMG hierarchy (orc_amg_digest)."""
    n = len(rowPtr) - 1
    nlev = C.c_int(0)
    d = lib().orc_amg_digest(n, _ptr(np.ascontiguousarray(rowPtr, np.int32)),
                             _ptr(np.ascontiguousarray(colIdx, np.int32)),
                             _ptr(np.ascontiguousarray(values, np.float64)), C.byref(nlev))
    return nlev.value, int(d)


def ssor_apply(rowPtr, colIdx, values, r, omega=1.0):
    """SsorPreconditioner setup + apply (LinearSolvers.cpp:168-231); returns z."""
    n = len(rowPtr) - 1
    rp = np.ascontiguousarray(rowPtr, np.int32)
    ci = np.ascontiguousarray(colIdx, np.int32)
    v = np.ascontiguousarray(values, np.float64)
    diag, inv = np.empty(n), np.empty(n)
    lib().orc_ssor_setup(n, _ptr(rp), _ptr(ci), _ptr(v), _ptr(diag), _ptr(inv))
    z, y, w = np.empty(n), np.empty(n), np.empty(n)
    lib().orc_ssor_apply(n, _ptr(rp), _ptr(ci), _ptr(v), _ptr(diag), _ptr(inv), float(omega),
                         _ptr(np.ascontiguousarray(r, np.float64)), _ptr(z), _ptr(y), _ptr(w))
    return z


class SimpOracle:
    """SimpTopology (src/optimization/SimpTopology.cpp:18-227) restated:
    initialize() fields and step() with the caller's dC_drho."""

    def __init__(self, m: Mesh, cfg):
        self.m = m
        self.cfg = np.ascontiguousarray(cfg, np.float64)
        self.rp, self.ci = build_sparsity(m)
        vf = float(cfg[4])
        self.rho = np.full(m.nC, vf)
        self.rhoTilde = np.full(m.nC, vf)
        self.K_simp = np.full(m.nC, float(cfg[1]))
        self.dC_drho = np.zeros(m.nC)
        self.dC_drhoTilde = np.zeros(m.nC)

    def step(self) -> float:
        m = self.m
        return lib().orc_simp_step(m.nC, m.nF, _ptr(m.owner), _ptr(m.neighbor), _ptr(m.ax), _ptr(m.ay), _ptr(m.az),
                                   _ptr(m.ccx), _ptr(m.ccy), _ptr(m.ccz), _ptr(m.vol), _ptr(self.rp), _ptr(self.ci),
                                   _ptr(self.cfg), _ptr(self.rho), _ptr(self.rhoTilde), _ptr(self.K_simp),
                                   _ptr(self.dC_drho), _ptr(self.dC_drhoTilde))


class SimpleOracle:
    """SimpleAlgorithm::iterate / advance_time_step (SimpleAlgorithm.cpp:522-570)
    restated: the state (U, p, phi, history) lives here, each outer iteration
    runs orc_simple_iterate.  bcs as face_fluxes; pressure zones are those
    with a PressureInlet / PressureOutlet spec; mom_cfg / p_cfg =
    (kind, precond, tol, maxIt, restart)."""

    def __init__(self, m: Mesh, bcs, rho=1.0, mu=1e-3, urfU=0.7, urfP=0.3, dt=0.0, bdf2=False, simplec=False,
                 mom_cfg=(0, 1, 1e-6, 200, 30), p_cfg=(2, 0, 1e-8, 1000, 30), n_outer_correctors=1, n_correctors=1,
                 n_non_orth_corr=0, momentum_predictor=True, tol_u=0.0, tol_p=0.0):
        """SIMPLE by default; PISO: n_correctors >= 1 with urfU = urfP = 1
        (PisoAlgorithm::to_simple_opts); PIMPLE: n_outer_correctors,
        n_correctors, momentum_predictor, tol_u / tol_p."""
        self.m = m
        self.nZ, self.zt, self.zv = _zone_tables(bcs)
        self.isP = np.zeros(self.nZ, np.uint8)
        for b in bcs:
            if int(b[1]) in (5, 7) and self.zt[int(b[0])] == int(b[1]):
                self.isP[int(b[0])] = 1
        # periodic twins (build_sparsity pairs them first, SimpleAlgorithm.cpp:54-56)
        self.twin = periodic_pairs(m, bcs) if any(int(b[1]) == PERIODIC for b in bcs) else None
        self.rp, self.ci = build_sparsity(m, self.twin)
        self.opt = np.array([rho, mu, urfU, urfP, dt], np.float64)
        self.bdf2, self.simplec = bool(bdf2), bool(simplec)
        self.mom_cfg = mom_cfg
        self.p_cfg = p_cfg
        self.U = np.zeros((3, m.nC))
        self.p = np.zeros(m.nC)
        self.phi = np.zeros(m.nF)
        self.aP = np.zeros(m.nC)
        self.pPrime = np.zeros(m.nC)
        self.Un = np.zeros((3, m.nC))
        self.Unm1 = np.zeros((3, m.nC))
        self.time_step = 0
        self.iters = []  # every iterate()'s four solve counts
        self.loops = np.array([n_outer_correctors, n_correctors, n_non_orth_corr, int(bool(momentum_predictor))],
                              np.int32)
        self.tol_up = np.array([tol_u, tol_p], np.float64)
        self.last_outer = 0

    def iterate(self):
        """One outer iteration; returns (res[4] = mom x, y, z, cont, iters[4])."""
        m = self.m
        res = np.zeros(4)
        its = np.zeros(4, np.int32)
        mc = np.array([self.mom_cfg[0], self.mom_cfg[1], self.mom_cfg[3], self.mom_cfg[4]], np.int32)
        pc = np.array([self.p_cfg[0], self.p_cfg[1], self.p_cfg[3], self.p_cfg[4]], np.int32)
        use_bdf2 = self.opt[4] > 0.0 and self.bdf2 and self.time_step >= 1
        flags = (1 if use_bdf2 else 0) | (2 if self.simplec else 0)
        self.last_outer = lib().orc_simple_iterate(m.nC, m.nF, _ptr(m.owner), _ptr(m.neighbor), _ptr(m.ax), _ptr(m.ay), _ptr(m.az),
                                 _ptr(m.fcx), _ptr(m.fcy), _ptr(m.fcz), _ptr(m.ccx), _ptr(m.ccy), _ptr(m.ccz),
                                 _ptr(m.vol), _ptr(m.zone), _ptr(self.zt), _ptr(self.zv), _ptr(self.isP), self.nZ,
                                 _ptr(self.rp), _ptr(self.ci), _ptr(self.opt), flags, _ptr(mc),
                                 float(self.mom_cfg[2]), _ptr(pc), float(self.p_cfg[2]), _ptr(self.loops),
                                 _ptr(self.tol_up), _ptr(self.U), _ptr(self.p),
                                 _ptr(self.Un), _ptr(self.Unm1), _ptr(self.phi), _ptr(self.aP), _ptr(self.pPrime),
                                 _ptr(res), _ptr(its), _ptr(self.twin))
        self.iters.append(its)
        return res, its

    def advance_time_step(self, n_inner=5):
        if self.time_step >= 1:
            self.Unm1[...] = self.Un
        self.Un[...] = self.U
        out = None
        for _ in range(max(1, n_inner)):
            out = self.iterate()
        self.time_step += 1
        return out


def spmv(rowPtr, colIdx, values, x):
    n = len(rowPtr) - 1
    y = np.empty(n)
    x = np.ascontiguousarray(x, np.float64)
    lib().orc_spmv(n, _ptr(rowPtr), _ptr(colIdx), _ptr(values), _ptr(x), _ptr(y))
    return y


def dot(a, b):
    a = np.ascontiguousarray(a, np.float64)
    b = np.ascontiguousarray(b, np.float64)
    return lib().orc_dot(len(a), _ptr(a), _ptr(b))


def jacobi_setup(rowPtr, colIdx, values):
    n = len(rowPtr) - 1
    inv = np.empty(n)
    lib().orc_jacobi_setup(n, _ptr(rowPtr), _ptr(colIdx), _ptr(values), _ptr(inv))
    return inv


def ilu0_setup(rowPtr, colIdx, values):
    n = len(rowPtr) - 1
    lu = np.empty(len(values))
    dp = np.empty(n, np.int32)
    lib().orc_ilu0_setup(n, _ptr(rowPtr), _ptr(colIdx), _ptr(values), _ptr(lu), _ptr(dp))
    return lu, dp


def ilu0_apply(rowPtr, colIdx, lu, diagPtr, r):
    n = len(rowPtr) - 1
    z = np.empty(n)
    y = np.empty(n)
    r = np.ascontiguousarray(r, np.float64)
    lib().orc_ilu0_apply(n, _ptr(rowPtr), _ptr(colIdx), _ptr(lu), _ptr(diagPtr), _ptr(r), _ptr(z), _ptr(y))
    return z


def cg(rowPtr, colIdx, values, b, precond=0, tol=1e-8, max_it=1000, history=False):
    """CGSolver::solve.  Returns (x, iterations, last_residual[, history])."""
    n = len(rowPtr) - 1
    x = np.empty(n)
    last = C.c_double(0.0)
    hist = np.zeros(max_it) if history else None
    b = np.ascontiguousarray(b, np.float64)
    it = lib().orc_cg(n, _ptr(rowPtr), _ptr(colIdx), _ptr(values), _ptr(b), int(precond), float(tol),
                      int(max_it), _ptr(x), C.byref(last), _ptr(hist))
    if history:
        return x, it, last.value, hist[:max(it, 0)]
    return x, it, last.value


def cggpu(rowPtr, colIdx, values, b, x0=None, precond=1, tol=1e-8, max_it=1000, relative_orders=0.0):
    """gpu::CgGpu::set_matrix + solve (host path).  precond: 0 None, 1 Jacobi,
    2 ILU0.  Returns (x, stats) with stats = dict(iterations, final_residual,
    initial_residual, converged, precond_after, last_residual)."""
    return _cggpu_call(lib().orc_cggpu_solve, rowPtr, colIdx, values, b, x0, precond, tol, max_it, relative_orders)


def _cggpu_call(fn, rowPtr, colIdx, values, b, x0, precond, tol, max_it, relative_orders):
    n = len(rowPtr) - 1
    x = np.zeros(n) if x0 is None else np.array(x0, np.float64, copy=True)
    out = np.zeros(4)
    pa = C.c_int(-1)
    last = C.c_double(0.0)
    b = np.ascontiguousarray(b, np.float64)
    fn(int(precond), float(tol), int(max_it), float(relative_orders), n, _ptr(np.ascontiguousarray(rowPtr, np.int32)),
       _ptr(np.ascontiguousarray(colIdx, np.int32)), _ptr(np.ascontiguousarray(values, np.float64)), _ptr(b),
       _ptr(x), _ptr(out), C.byref(pa), C.byref(last))
    return x, {"iterations": int(out[0]), "final_residual": float(out[1]), "initial_residual": float(out[2]),
               "converged": bool(out[3]), "precond_after": int(pa.value), "last_residual": float(last.value)}


# ---------------------------------------------------------------- compiled reference


class RefLib:
    """The reference's own code (oracle/_ref/libsimall_ref.so)."""

    def __init__(self, path: str = REF_PATH):
        L = C.CDLL(path)
        L.ref_mesh_cartesian.restype = _P
        L.ref_mesh_cartesian.argtypes = [C.c_int, C.c_int, C.c_int, _D, _D, _D]
        L.ref_mesh_free.argtypes = [_P]
        L.ref_mesh_sizes.argtypes = [_P, _P]
        L.ref_mesh_get_nodes.argtypes = [_P] * 4
        L.ref_mesh_set_nodes.argtypes = [_P] * 4
        L.ref_mesh_get_faces.argtypes = [_P] * 10
        L.ref_mesh_get_face_nodes.argtypes = [_P] * 3
        L.ref_mesh_get_cells.argtypes = [_P] * 7
        L.ref_mesh_rcm.argtypes = [_P, _P]
        L.ref_sparsity_nnz.restype = _I64
        L.ref_sparsity_nnz.argtypes = [_P, C.c_int, _P, _P]
        L.ref_assemble.restype = C.c_int
        L.ref_assemble.argtypes = [_P, C.c_int, _P, _P, _D] + [_P] * 6
        L.ref_face_fluxes.restype = C.c_int
        L.ref_face_fluxes.argtypes = [_P, C.c_int, _P, _P, _P, _D] + [_P] * 4
        L.ref_lsq_gradient.restype = C.c_int
        L.ref_lsq_gradient.argtypes = [_P] * 5
        L.ref_correct_fields.restype = C.c_int
        L.ref_correct_fields.argtypes = [_P, _D, _D] + [_P] * 7
        L.ref_assemble_simplec.restype = C.c_int
        L.ref_assemble_simplec.argtypes = [_P, C.c_int, _P, _P, _D] + [_P] * 7
        L.ref_cg.restype = C.c_int
        L.ref_cg.argtypes = [C.c_int, _P, _P, _P, _P, C.c_int, _D, C.c_int, _P, _P, _P]
        L.ref_precond_apply.argtypes = [C.c_int, C.c_int] + [_P] * 5
        L.ref_spmv.argtypes = [C.c_int] + [_P] * 5
        L.ref_cavity_run.restype = C.c_int
        L.ref_cavity_run.argtypes = [C.c_int, _D, C.c_int, C.c_int, C.c_int, C.c_int, _D, C.c_int, _P, _P]
        L.ref_cavity_fetch.argtypes = [_P] * 9
        L.ref_plugin_load.restype = _I64
        L.ref_plugin_load.argtypes = [C.c_char_p, C.c_char_p, C.c_int, C.c_char_p, C.c_int, C.POINTER(C.c_int)]
        L.ref_assemble_momentum.restype = C.c_int
        L.ref_assemble_momentum.argtypes = [_P, C.c_int, _P, _P, _P, _P, C.c_int, C.c_int, C.c_int] + [_P] * 8
        L.ref_krylov.restype = C.c_int
        L.ref_krylov.argtypes = [C.c_int, C.c_int, _D, C.c_int, C.c_int, C.c_int] + [_P] * 7
        L.ref_simple_run.restype = C.c_int
        L.ref_simple_run.argtypes = [_P, C.c_int, _P, _P, _P, _P, C.c_int, _P, _D, _P, _D, C.c_int, C.c_int] + \
            [_P] * 5 + [C.c_int, _P, _P]
        L.ref_checkpoint_write.restype = C.c_int
        L.ref_checkpoint_write.argtypes = [_P, C.c_char_p, C.c_int, _P, _P, _P, _P, C.c_int, _D, C.c_uint64]
        L.ref_checkpoint_read.restype = _P
        L.ref_checkpoint_read.argtypes = [C.c_char_p, _P, _P]
        L.ref_checkpoint_field.restype = _I64
        L.ref_checkpoint_field.argtypes = [C.c_char_p, C.c_int, _P]
        L.ref_simp_run.restype = C.c_int
        L.ref_simp_run.argtypes = [_P, _P, C.c_int] + [_P] * 6
        L.ref_piso_pimple_run.restype = C.c_int
        L.ref_piso_pimple_run.argtypes = [_P, C.c_int, C.c_int, _P, _P, _P, _P, _P, C.c_int, _P, _D, _P, _D,
                                          C.c_int] + [_P] * 5
        L.ref_periodic_twins.restype = C.c_int
        L.ref_periodic_twins.argtypes = [_P, C.c_int, _P, _P, _P]
        L.ref_cggpu_solve.restype = C.c_int
        L.ref_cggpu_solve.argtypes = [C.c_int, _D, C.c_int, _D, C.c_int] + [_P] * 8
        L.ref_discrete_adjoint.restype = C.c_int
        L.ref_discrete_adjoint.argtypes = [C.c_int, _P, _P, _P, _P, _D, C.c_int, C.c_int, C.c_int] + [_P] * 11
        self.L = L

    @staticmethod
    def available(path: str = REF_PATH) -> bool:
        return os.path.exists(path)

    # -- mesh
    def cartesian_mesh(self, Nx, Ny, Nz, ex=1.0, ey=1.0, ez=1.0, node_shift=None, do_rcm=False):
        L = self.L
        h = L.ref_mesh_cartesian(Nx, Ny, Nz, ex, ey, ez)
        try:
            s = np.zeros(5, np.int64)
            L.ref_mesh_sizes(h, _ptr(s))
            nC, nF, nN, ncf, nfn = (int(v) for v in s)
            if node_shift is not None:
                nx = np.empty(nN)
                ny = np.empty(nN)
                nz = np.empty(nN)
                L.ref_mesh_get_nodes(h, _ptr(nx), _ptr(ny), _ptr(nz))
                nx = nx + node_shift[0]
                ny = ny + node_shift[1]
                nz = nz + node_shift[2]
                L.ref_mesh_set_nodes(h, _ptr(nx), _ptr(ny), _ptr(nz))
            stats = None
            if do_rcm:
                st = np.zeros(3, np.int64)
                L.ref_mesh_rcm(h, _ptr(st))
                stats = tuple(int(v) for v in st)
            out = self._fetch(h, nC, nF, nN, ncf, nfn)
            out["rcm_stats"] = stats
            out["handle"] = h
            return out
        except Exception:
            L.ref_mesh_free(h)
            raise

    def _fetch(self, h, nC, nF, nN, ncf, nfn):
        L = self.L
        d = {"nC": nC, "nF": nF}
        d["nx"], d["ny"], d["nz"] = np.empty(nN), np.empty(nN), np.empty(nN)
        L.ref_mesh_get_nodes(h, _ptr(d["nx"]), _ptr(d["ny"]), _ptr(d["nz"]))
        own = np.empty(nF, np.uint64)
        nb = np.empty(nF, np.uint64)
        for k in ("ax", "ay", "az", "fcx", "fcy", "fcz"):
            d[k] = np.empty(nF)
        d["zone"] = np.empty(nF, np.uint32)
        L.ref_mesh_get_faces(h, _ptr(own), _ptr(nb), _ptr(d["ax"]), _ptr(d["ay"]), _ptr(d["az"]),
                             _ptr(d["fcx"]), _ptr(d["fcy"]), _ptr(d["fcz"]), _ptr(d["zone"]))
        d["owner"] = own.view(np.int64).copy()
        d["neighbor"] = nb.view(np.int64).copy()
        d["fnOff"] = np.empty(nF + 1, np.int32)
        fn = np.empty(nfn, np.uint64)
        L.ref_mesh_get_face_nodes(h, _ptr(d["fnOff"]), _ptr(fn))
        d["fnIdx"] = fn.view(np.int64).copy()
        for k in ("vol", "ccx", "ccy", "ccz"):
            d[k] = np.empty(nC)
        d["cfOff"] = np.empty(nC + 1, np.int32)
        cf = np.empty(ncf, np.uint64)
        L.ref_mesh_get_cells(h, _ptr(d["vol"]), _ptr(d["ccx"]), _ptr(d["ccy"]), _ptr(d["ccz"]),
                             _ptr(d["cfOff"]), _ptr(cf))
        d["cfIdx"] = cf.view(np.int64).copy()
        return d

    def free_mesh(self, mesh_dict):
        if mesh_dict.get("handle"):
            self.L.ref_mesh_free(mesh_dict["handle"])
            mesh_dict["handle"] = None

    def periodic_twins(self, mesh_dict, bcs):
        """build_periodic_pairs' twin table (-1 where none)."""
        zones = np.array([b[0] for b in bcs] or [0], np.uint32)
        types = np.array([b[1] for b in bcs] or [0], np.int32)
        twin = np.empty(mesh_dict["nF"], np.int32)
        self.L.ref_periodic_twins(mesh_dict["handle"], len(bcs), _ptr(zones), _ptr(types), _ptr(twin))
        return twin

    def assemble(self, mesh_dict, bcs, rho, aP, phi):
        """bcs: list of (zone, BCType ordinal).  Returns rowPtr, colIdx, values, rhs."""
        L = self.L
        h = mesh_dict["handle"]
        nC = mesh_dict["nC"]
        zones = np.array([b[0] for b in bcs] or [0], np.uint32)
        types = np.array([b[1] for b in bcs] or [0], np.int32)
        nnz = L.ref_sparsity_nnz(h, len(bcs), _ptr(zones), _ptr(types))
        rowPtr = np.empty(nC + 1, np.int32)
        colIdx = np.empty(nnz, np.int32)
        values = np.empty(nnz)
        rhs = np.empty(nC)
        aP = np.ascontiguousarray(aP, np.float64)
        phi = np.ascontiguousarray(phi, np.float64)
        L.ref_assemble(h, len(bcs), _ptr(zones), _ptr(types), rho, _ptr(aP), _ptr(phi), _ptr(rowPtr),
                       _ptr(colIdx), _ptr(values), _ptr(rhs))
        return rowPtr, colIdx, values, rhs

    def face_fluxes(self, mesh_dict, bcs, rho, U):
        """bcs: list of (zone, BCType ordinal, (ux, uy, uz))."""
        zones = np.array([b[0] for b in bcs] or [0], np.uint32)
        types = np.array([b[1] for b in bcs] or [0], np.int32)
        vec = np.array([list(b[2]) if len(b) > 2 else [0, 0, 0] for b in bcs] or [[0, 0, 0]], np.float64).ravel()
        Ux, Uy, Uz = (np.ascontiguousarray(u, np.float64) for u in U)
        phi = np.empty(mesh_dict["nF"])
        self.L.ref_face_fluxes(mesh_dict["handle"], len(bcs), _ptr(zones), _ptr(types), _ptr(vec), float(rho),
                               _ptr(Ux), _ptr(Uy), _ptr(Uz), _ptr(phi))
        return phi

    def lsq_gradient(self, mesh_dict, phi):
        g = np.empty((3, mesh_dict["nC"]))
        self.L.ref_lsq_gradient(mesh_dict["handle"], _ptr(np.ascontiguousarray(phi, np.float64)), _ptr(g[0]),
                                _ptr(g[1]), _ptr(g[2]))
        return g

    def correct_fields(self, mesh_dict, rho, urfP, aP, pPrime, p, U, phi):
        p = np.array(p, np.float64)
        Ux, Uy, Uz = (np.array(u, np.float64) for u in U)
        phi = np.array(phi, np.float64)
        self.L.ref_correct_fields(mesh_dict["handle"], float(rho), float(urfP),
                                  _ptr(np.ascontiguousarray(aP, np.float64)),
                                  _ptr(np.ascontiguousarray(pPrime, np.float64)), _ptr(p), _ptr(Ux), _ptr(Uy),
                                  _ptr(Uz), _ptr(phi))
        return p, (Ux, Uy, Uz), phi

    def assemble_simplec(self, mesh_dict, bcs, rho, aP, mom, phi):
        """assemble_pressure_correction with PvCouplingVariant::SIMPLEC, the
        momentum matrix A_mom_ given by its values on the shared pattern."""
        L = self.L
        h = mesh_dict["handle"]
        nC = mesh_dict["nC"]
        zones = np.array([b[0] for b in bcs] or [0], np.uint32)
        types = np.array([b[1] for b in bcs] or [0], np.int32)
        nnz = L.ref_sparsity_nnz(h, len(bcs), _ptr(zones), _ptr(types))
        rowPtr = np.empty(nC + 1, np.int32)
        colIdx = np.empty(nnz, np.int32)
        values = np.empty(nnz)
        rhs = np.empty(nC)
        L.ref_assemble_simplec(h, len(bcs), _ptr(zones), _ptr(types), rho, _ptr(np.ascontiguousarray(aP, np.float64)),
                               _ptr(np.ascontiguousarray(mom, np.float64)), _ptr(np.ascontiguousarray(phi, np.float64)),
                               _ptr(rowPtr), _ptr(colIdx), _ptr(values), _ptr(rhs))
        return rowPtr, colIdx, values, rhs

    def assemble_momentum(self, mesh_dict, bcs, opt, comp, U, p, phi, Un=None, Unm1=None, bdf2=False, time_step=0):
        """SimpleAlgorithm::assemble_momentum(comp); returns (values, rhs, aP_)."""
        L = self.L
        h = mesh_dict["handle"]
        nC = mesh_dict["nC"]
        zones = np.array([b[0] for b in bcs] or [0], np.uint32)
        types = np.array([b[1] for b in bcs] or [0], np.int32)
        nnz = L.ref_sparsity_nnz(h, len(bcs), _ptr(zones), _ptr(types))
        vec = np.array([list(b[2]) if len(b) > 2 else [0, 0, 0] for b in bcs] or [[0, 0, 0]], np.float64).ravel()
        U3 = np.ascontiguousarray(np.asarray(U, np.float64).reshape(3, nC))
        z3 = np.zeros((3, nC))
        Un3 = np.ascontiguousarray(np.asarray(Un, np.float64).reshape(3, nC)) if Un is not None else z3
        Unm13 = np.ascontiguousarray(np.asarray(Unm1, np.float64).reshape(3, nC)) if Unm1 is not None else z3
        values = np.empty(nnz)
        rhs = np.empty(nC)
        aP = np.empty(nC)
        L.ref_assemble_momentum(h, len(bcs), _ptr(zones), _ptr(types), _ptr(vec),
                                _ptr(np.ascontiguousarray(opt, np.float64)), int(bool(bdf2)), int(time_step),
                                int(comp), _ptr(U3), _ptr(np.ascontiguousarray(p, np.float64)),
                                _ptr(np.ascontiguousarray(phi, np.float64)), _ptr(Un3), _ptr(Unm13), _ptr(values),
                                _ptr(rhs), _ptr(aP))
        return values, rhs, aP

    def krylov(self, kind, rowPtr, colIdx, values, b, precond=0, tol=1e-8, max_it=1000, restart=30):
        """make_gmres / make_bicgstab / make_cg by LinearSolverKind ordinal; (x, it, last, seconds)."""
        n = len(rowPtr) - 1
        x = np.empty(n)
        last = C.c_double(0)
        secs = C.c_double(0)
        it = self.L.ref_krylov(int(kind), int(precond), float(tol), int(max_it), int(restart), n,
                               _ptr(np.ascontiguousarray(rowPtr, np.int32)),
                               _ptr(np.ascontiguousarray(colIdx, np.int32)),
                               _ptr(np.ascontiguousarray(values, np.float64)),
                               _ptr(np.ascontiguousarray(b, np.float64)), _ptr(x), C.byref(last), C.byref(secs))
        return x, it, last.value, secs.value

    def simple_run(self, mesh_dict, bcs, U, p, n_outer, rho=1.0, mu=1e-3, urfU=0.7, urfP=0.3, dt=0.0, bdf2=False,
                   simplec=False, mom_cfg=(0, 1, 1e-6, 200, 30), p_cfg=(2, 0, 1e-8, 1000, 30), n_inner=1):
        """The reference's SimpleAlgorithm: n_outer iterate() calls (or
        advance_time_step(n_inner) when dt > 0).  Returns dict U, p, phi, res
        [n_outer, 4], iters [per iterate: mom x, y, z, p], seconds."""
        nC, nF = mesh_dict["nC"], mesh_dict["nF"]
        zones = np.array([b[0] for b in bcs] or [0], np.uint32)
        types = np.array([b[1] for b in bcs] or [0], np.int32)
        vec = np.array([list(b[2]) if len(b) > 2 else [0, 0, 0] for b in bcs] or [[0, 0, 0]], np.float64).ravel()
        U = np.array(U, np.float64).reshape(3, nC).copy()
        p = np.array(p, np.float64).copy()
        phi = np.empty(nF)
        res = np.empty((n_outer, 4))
        cap = 4 * n_outer * max(1, n_inner) + 8
        its = np.empty(cap, np.int32)
        nits = C.c_int(0)
        secs = C.c_double(0)
        opt = np.array([rho, mu, urfU, urfP, dt], np.float64)
        mc = np.array([mom_cfg[0], mom_cfg[1], mom_cfg[3], mom_cfg[4]], np.int32)
        pc = np.array([p_cfg[0], p_cfg[1], p_cfg[3], p_cfg[4]], np.int32)
        flags = (1 if bdf2 else 0) | (2 if simplec else 0)
        self.L.ref_simple_run(mesh_dict["handle"], len(bcs), _ptr(zones), _ptr(types), _ptr(vec), _ptr(opt), flags,
                              _ptr(mc), float(mom_cfg[2]), _ptr(pc), float(p_cfg[2]), int(n_outer), int(n_inner),
                              _ptr(U), _ptr(p), _ptr(phi), _ptr(res), _ptr(its), cap, C.byref(nits), C.byref(secs))
        return {"U": U, "p": p, "phi": phi, "res": res, "iters": its[:nits.value].reshape(-1, 4).copy(),
                "seconds": secs.value}

    def checkpoint_write(self, mesh_dict, path, fields, iteration=0, time=0.0, settings_hash=0):
        """io::Checkpoint::write; fields = [(name, is_vector, array (n,) or (3, n))] in insertion order."""
        arrs = [np.ascontiguousarray(a, np.float64) for _, _, a in fields]
        names = (C.c_char_p * max(1, len(fields)))(*[f[0].encode() for f in fields])
        isv = np.array([int(f[1]) for f in fields] or [0], np.int32)
        sizes = np.array([a.shape[-1] if f[1] else a.size for f, a in zip(fields, arrs)] or [0], np.int64)
        ptrs = (C.c_void_p * max(1, len(fields)))(*[a.ctypes.data for a in arrs])
        return self.L.ref_checkpoint_write(mesh_dict["handle"], path.encode(), len(fields), names, _ptr(isv),
                                           _ptr(sizes), ptrs, int(iteration), float(time), int(settings_hash))

    def checkpoint_read(self, path):
        """io::Checkpoint::read; returns (mesh dict with a handle, meta (iteration, time, hash),
        field getter name, is_vector -> array)."""
        sizes = np.zeros(5, np.int64)
        meta = np.zeros(3)
        h = self.L.ref_checkpoint_read(path.encode(), _ptr(sizes), _ptr(meta))
        if not h:
            return None
        s5 = np.zeros(5, np.int64)
        self.L.ref_mesh_sizes(h, _ptr(s5))
        md = self._fetch(h, *(int(v) for v in s5))
        md["handle"] = h
        md["n_scalars"], md["n_vectors"] = int(sizes[3]), int(sizes[4])

        def field(name, vector=False):
            n = self.L.ref_checkpoint_field(name.encode(), int(vector), None)
            if n < 0:
                return None
            out = np.empty((3, n) if vector else n)
            self.L.ref_checkpoint_field(name.encode(), int(vector), _ptr(out))
            return out

        return md, (int(meta[0]), float(meta[1]), int(meta[2:3].view(np.uint64)[0])), field

    def simp_run(self, mesh_dict, cfg, dC_steps):
        """SimpTopology::initialize + one step() per row of dC_steps (stored in
        "dC_drho" before the step); returns (change[k], rho, rhoTilde, K_simp, dC_drhoTilde)."""
        nC = mesh_dict["nC"]
        dC = np.ascontiguousarray(dC_steps, np.float64).reshape(-1, nC)
        k = dC.shape[0]
        change = np.empty(k)
        out = [np.empty(nC) for _ in range(4)]
        self.L.ref_simp_run(mesh_dict["handle"], _ptr(np.ascontiguousarray(cfg, np.float64)), k, _ptr(dC),
                            _ptr(change), *(_ptr(o) for o in out))
        return (change, *out)

    def piso_pimple_run(self, mesh_dict, variant, bcs, U, p, n_steps, rho=1.0, mu=1e-3, dt=1e-3, urfU=0.7,
                        urfP=0.3, tol_u=0.0, tol_p=0.0, loops=(2, 2, 0, 1), bdf2=True,
                        mom_cfg=(0, 0, 1e-9, 200, 30), p_cfg=(2, 0, 1e-9, 1000, 30)):
        """PisoAlgorithm (variant 1) or PimpleAlgorithm (variant 2):
        n_steps advance_time_step(1) calls; returns dict U, p, phi, res, last_outer."""
        nC, nF = mesh_dict["nC"], mesh_dict["nF"]
        zones = np.array([b[0] for b in bcs] or [0], np.uint32)
        types = np.array([b[1] for b in bcs] or [0], np.int32)
        vec = np.array([list(b[2]) if len(b) > 2 else [0, 0, 0] for b in bcs] or [[0, 0, 0]], np.float64).ravel()
        U = np.array(U, np.float64).reshape(3, nC).copy()
        p = np.array(p, np.float64).copy()
        phi = np.empty(nF)
        res = np.empty((n_steps, 4))
        lo = np.zeros(n_steps, np.int32)
        opt = np.array([rho, mu, dt, urfU, urfP, tol_u, tol_p], np.float64)
        mc = np.array([mom_cfg[0], mom_cfg[1], mom_cfg[3], mom_cfg[4]], np.int32)
        pc = np.array([p_cfg[0], p_cfg[1], p_cfg[3], p_cfg[4]], np.int32)
        self.L.ref_piso_pimple_run(mesh_dict["handle"], int(variant), len(bcs), _ptr(zones), _ptr(types), _ptr(vec),
                                   _ptr(opt), _ptr(np.array(loops, np.int32)), int(bool(bdf2)), _ptr(mc),
                                   float(mom_cfg[2]), _ptr(pc), float(p_cfg[2]), int(n_steps), _ptr(U), _ptr(p),
                                   _ptr(phi), _ptr(res), _ptr(lo))
        return {"U": U, "p": p, "phi": phi, "res": res, "last_outer": lo}

    # -- solvers
    def cg(self, rowPtr, colIdx, values, b, precond=0, tol=1e-8, max_it=1000):
        n = len(rowPtr) - 1
        x = np.empty(n)
        last = C.c_double(0)
        secs = C.c_double(0)
        b = np.ascontiguousarray(b, np.float64)
        it = self.L.ref_cg(n, _ptr(rowPtr), _ptr(colIdx), _ptr(values), _ptr(b), int(precond), float(tol),
                           int(max_it), _ptr(x), C.byref(last), C.byref(secs))
        return x, it, last.value, secs.value

    def cggpu(self, rowPtr, colIdx, values, b, x0=None, precond=1, tol=1e-8, max_it=1000, relative_orders=0.0):
        """gpu::CgGpu (set_matrix + solve) of the reference, host path."""
        return _cggpu_call(self.L.ref_cggpu_solve, rowPtr, colIdx, values, b, x0, precond, tol, max_it,
                           relative_orders)

    def precond_apply(self, kind, rowPtr, colIdx, values, r):
        n = len(rowPtr) - 1
        z = np.empty(n)
        r = np.ascontiguousarray(r, np.float64)
        self.L.ref_precond_apply(int(kind), n, _ptr(rowPtr), _ptr(colIdx), _ptr(values), _ptr(r), _ptr(z))
        return z

    def spmv(self, rowPtr, colIdx, values, x):
        n = len(rowPtr) - 1
        y = np.empty(n)
        x = np.ascontiguousarray(x, np.float64)
        self.L.ref_spmv(n, _ptr(rowPtr), _ptr(colIdx), _ptr(values), _ptr(x), _ptr(y))
        return y

    def cavity(self, N, mu=0.01, n_outer=3, n_record=3, precond=0, tol=1e-8, max_it=1000, record_stride=0):
        """SIMPLE lid-driven cavity; records the first n_record pressure systems
        and, with record_stride > 0, every record_stride-th one."""
        L = self.L
        sizes = np.zeros(5, np.int64)
        secs = C.c_double(0)
        L.ref_cavity_run(N, mu, n_outer, n_record, record_stride, precond, tol, max_it, _ptr(sizes), C.byref(secs))
        nC, nnz, nF, nSolve, nRec = (int(v) for v in sizes)
        out = {
            "rowPtr": np.empty(nC + 1, np.int32), "colIdx": np.empty(nnz, np.int32),
            "values": np.empty((nRec, nnz)), "rhs": np.empty((nRec, nC)), "x": np.empty((nRec, nC)),
            "aP": np.empty((nRec, nC)), "phi": np.empty((nRec, nF)), "iters": np.empty(nSolve, np.int32),
            "res": np.empty(nSolve),
        }
        L.ref_cavity_fetch(*(_ptr(out[k]) for k in ("rowPtr", "colIdx", "values", "rhs", "x", "aP", "phi",
                                                      "iters", "res")))
        out["p_solve_seconds"] = secs.value
        return out

    def plugin_load(self, path: str):
        """core::PluginLoader::load of a plugin library; (cookie, name, version, category)."""
        name = C.create_string_buffer(256)
        ver = C.create_string_buffer(64)
        cat = C.c_int(-1)
        cookie = self.L.ref_plugin_load(path.encode(), name, 256, ver, 64, C.byref(cat))
        return int(cookie), name.value.decode(), ver.value.decode(), cat.value

    def discrete_adjoint(self, rowPtr, colIdx, values, dJdQ, owner, neighbor, is_dirichlet, g, k, pb, x,
                         tol=1e-10, max_iter=500, restart=30):
        n = len(rowPtr) - 1
        nF = len(owner)
        nD = int(np.count_nonzero(is_dirichlet))
        psi = np.empty(n)
        grad = np.empty(nF + nD)
        its = C.c_int64(0)
        res = C.c_double(0)
        arr = [np.ascontiguousarray(a, t) for a, t in ((dJdQ, np.float64), (owner, np.int64),
                                                        (neighbor, np.int64), (is_dirichlet, np.int32),
                                                        (g, np.float64), (k, np.float64), (pb, np.float64),
                                                        (x, np.float64))]
        rc = self.L.ref_discrete_adjoint(n, _ptr(rowPtr), _ptr(colIdx), _ptr(values), _ptr(arr[0]), tol,
                                         max_iter, restart, nF, _ptr(arr[1]), _ptr(arr[2]), _ptr(arr[3]),
                                         _ptr(arr[4]), _ptr(arr[5]), _ptr(arr[6]), _ptr(arr[7]), _ptr(psi),
                                         _ptr(grad), C.byref(its), C.byref(res))
        return psi, grad, int(its.value), res.value, rc
