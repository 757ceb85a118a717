"""Mesh SoA, the device pressure-correction system, and boundary types.

`MeshSoA` holds the reference's mesh layout (src/meshing/MeshStorage.hpp:
37-105): u64 owner/neighbor with UINT64_MAX on boundary faces, FP64 areas and
centroids, u32 zones, and the cell->face CSR.  `cartesian()` builds the
structured box through the library's host generator (bit-identical to
CartesianMesher + ConnectivityBuilder + compute_geometry) and `rcm()` applies
renumber_cells_cuthill_mckee.  `PressureSystem` wraps the device assembly of
SimpleAlgorithm::assemble_pressure_correction.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass
from enum import IntEnum

import numpy as np

from . import _lib
from ._lib import MEM_DEVICE, MEM_HOST, check
from .solver import Context, GpuCGSolver, default_context, ptr_and_mem, register_child

BOUNDARY = np.uint64(0xFFFFFFFFFFFFFFFF)


class BCType(IntEnum):
    """BCType (src/solver/Solver.hpp:105-123)."""

    Wall = 0
    NoSlipWall = 1
    MovingWall = 2
    SlipWall = 3
    VelocityInlet = 4
    PressureInlet = 5
    MassFlowInlet = 6
    PressureOutlet = 7
    OutFlow = 8
    Symmetry = 9
    Axisymmetric = 10
    Periodic = 11


@dataclass
class MeshSoA:
    n_cells: int
    n_faces: int
    owner: np.ndarray
    neighbor: np.ndarray
    area_x: np.ndarray
    area_y: np.ndarray
    area_z: np.ndarray
    centroid_x: np.ndarray
    centroid_y: np.ndarray
    centroid_z: np.ndarray
    boundary_zone: np.ndarray
    volume: np.ndarray
    cell_centroid_x: np.ndarray
    cell_centroid_y: np.ndarray
    cell_centroid_z: np.ndarray
    cell_face_offsets: np.ndarray
    cell_face_indices: np.ndarray

    def interior(self) -> np.ndarray:
        return self.neighbor != BOUNDARY

    def view(self) -> _lib.MeshView:
        v = _lib.MeshView()
        v.n_cells = self.n_cells
        v.n_faces = self.n_faces
        for name in ("owner", "neighbor", "area_x", "area_y", "area_z", "centroid_x", "centroid_y", "centroid_z",
                     "boundary_zone", "cell_centroid_x", "cell_centroid_y", "cell_centroid_z", "cell_face_offsets",
                     "cell_face_indices"):
            setattr(v, name, getattr(self, name).ctypes.data)
        return v


def n_faces_box(nx: int, ny: int, nz: int) -> int:
    return (nx + 1) * ny * nz + nx * (ny + 1) * nz + nx * ny * (nz + 1)


def cartesian(nx: int, ny: int, nz: int, ex: float = 1.0, ey: float = 1.0, ez: float = 1.0,
              node_shift: np.ndarray | None = None) -> MeshSoA:
    L = _lib.load()
    nC = nx * ny * nz
    nF = n_faces_box(nx, ny, nz)
    f64 = lambda k: np.empty(k, np.float64)  # noqa: E731
    m = MeshSoA(nC, nF, np.empty(nF, np.uint64), np.empty(nF, np.uint64), f64(nF), f64(nF), f64(nF), f64(nF),
                f64(nF), f64(nF), np.empty(nF, np.uint32), f64(nC), f64(nC), f64(nC), f64(nC),
                np.empty(nC + 1, np.int32), np.empty(6 * nC, np.uint64))
    if node_shift is not None:
        sh = [np.ascontiguousarray(node_shift[i], np.float64) for i in range(3)]
        shp = [s.ctypes.data for s in sh]
    else:
        shp = [None, None, None]
    st = L.simall_mesh_cartesian(nx, ny, nz, ex, ey, ez, *shp, m.owner.ctypes.data, m.neighbor.ctypes.data,
                                 m.area_x.ctypes.data, m.area_y.ctypes.data, m.area_z.ctypes.data,
                                 m.centroid_x.ctypes.data, m.centroid_y.ctypes.data, m.centroid_z.ctypes.data,
                                 m.boundary_zone.ctypes.data, m.volume.ctypes.data, m.cell_centroid_x.ctypes.data,
                                 m.cell_centroid_y.ctypes.data, m.cell_centroid_z.ctypes.data,
                                 m.cell_face_offsets.ctypes.data, m.cell_face_indices.ctypes.data)
    check(st)
    return m


def rcm(m: MeshSoA):
    """renumber_cells_cuthill_mckee in place; returns (bwBefore, bwAfter, permuted)."""
    L = _lib.load()
    stats = np.zeros(3, np.int64)
    check(L.simall_mesh_rcm(m.n_cells, m.n_faces, m.owner.ctypes.data, m.neighbor.ctypes.data, m.volume.ctypes.data,
                            m.cell_centroid_x.ctypes.data, m.cell_centroid_y.ctypes.data,
                            m.cell_centroid_z.ctypes.data, m.cell_face_offsets.ctypes.data,
                            m.cell_face_indices.ctypes.data, stats.ctypes.data))
    return tuple(int(s) for s in stats)


class PressureSystem:
    """Device pressure-correction system (pattern + assembly + solve)."""

    def __init__(self, mesh: MeshSoA, bcs: list[tuple[int, int]] | None = None, ctx: Context | None = None):
        self.ctx = ctx or default_context()
        self.L = self.ctx.L
        self.mesh = mesh
        bcs = bcs or []
        arr = (_lib.Boundary * max(1, len(bcs)))()
        for i, (z, t) in enumerate(bcs):
            arr[i].zone = int(z)
            arr[i].type = int(t)
        view = mesh.view()
        h = C.c_void_p()
        check(self.L.simall_pressure_system_create(self.ctx.handle, C.byref(view), arr, len(bcs), C.byref(h)),
              self.ctx.handle)
        self.handle = h.value
        register_child(self)
        self.ctx.children.add(self)
        n = C.c_int64()
        nnz = C.c_int64()
        check(self.L.simall_pressure_system_pattern(self.handle, C.byref(n), C.byref(nnz), None, None))
        self.n = n.value
        self.nnz = nnz.value
        self.any_dirichlet = None

    def periodic_twins(self):
        """The twin face of every face (-1 where none): build_periodic_pairs' table."""
        tw = np.empty(self.mesh.n_faces, np.int32)
        check(self.L.simall_pressure_system_periodic_twins(self.handle, tw.ctypes.data))
        return tw

    def pattern(self):
        rp = np.empty(self.n + 1, np.int32)
        ci = np.empty(self.nnz, np.int32)
        check(self.L.simall_pressure_system_pattern(self.handle, None, None, rp.ctypes.data, ci.ctypes.data))
        return rp, ci

    def device_arrays(self):
        """Raw device addresses (rowPtr, colIdx, values, rhs)."""
        a = [C.c_void_p() for _ in range(4)]
        check(self.L.simall_pressure_system_device_arrays(self.handle, *[C.byref(v) for v in a]))
        return tuple(v.value for v in a)

    def assemble(self, rho: float, aP, phi):
        pa, ma = ptr_and_mem(aP)
        pp, mp = ptr_and_mem(phi)
        if ma != mp:
            raise ValueError("aP and phi must live in the same memory")
        anyD = C.c_int()
        check(self.L.simall_assemble_pressure_correction(self.handle, float(rho), pa, pp, ma, C.byref(anyD)),
              self.ctx.handle)
        self.any_dirichlet = bool(anyD.value)

    def assemble_simplec(self, rho: float, aP, mom_values, phi):
        """SIMPLEC variant: denominators max(aP - sum|offdiag(A_mom)|, 1e-30),
        mom_values = the momentum matrix's values on this system's pattern."""
        pa, ma = ptr_and_mem(aP)
        pm, mm = ptr_and_mem(mom_values)
        pp, mp = ptr_and_mem(phi)
        if not (ma == mm == mp):
            raise ValueError("aP, mom_values and phi must live in the same memory")
        anyD = C.c_int()
        check(self.L.simall_assemble_pressure_correction_simplec(self.handle, float(rho), pa, pm, pp, ma,
                                                                 C.byref(anyD)), self.ctx.handle)
        self.any_dirichlet = bool(anyD.value)

    # -- the field loops around the solve ------------------------------------------
    def setup_field_loops(self, velocities=()):
        """velocities: (zone, (ux, uy, uz)) of VelocityInlet / MovingWall zones."""
        arr = (_lib.ZoneVelocity * max(1, len(velocities)))()
        for i, (z, u) in enumerate(velocities):
            arr[i].zone = int(z)
            for k in range(3):
                arr[i].u[k] = float(u[k])
        view = self.mesh.view()
        check(self.L.simall_pressure_system_setup_field_loops(self.handle, C.byref(view), self.mesh.volume.ctypes.data,
                                                              arr, len(velocities)), self.ctx.handle)

    def face_fluxes(self, rho: float, U, phi=None):
        """compute_face_fluxes; U = (Ux, Uy, Uz) numpy or CUDA tensors."""
        ptrs = [ptr_and_mem(u) for u in U]
        if phi is None:
            phi = np.empty(self.mesh.n_faces)
        pp, mp = ptr_and_mem(phi)
        if any(m != mp for _, m in ptrs):
            raise ValueError("U and phi must live in the same memory")
        check(self.L.simall_compute_face_fluxes(self.handle, float(rho), ptrs[0][0], ptrs[1][0], ptrs[2][0], pp, mp),
              self.ctx.handle)
        return phi

    def lsq_gradient(self, f):
        pf, mf = ptr_and_mem(f)
        if mf != _lib.MEM_HOST:
            raise ValueError("lsq_gradient: host arrays only from Python")
        g = np.empty((3, self.mesh.n_cells))
        check(self.L.simall_lsq_gradient(self.handle, pf, g[0].ctypes.data, g[1].ctypes.data, g[2].ctypes.data, mf),
              self.ctx.handle)
        return g

    def correct_fields(self, rho: float, urfP: float, aP, pPrime, p, U, phi):
        """In place on p, U = (Ux, Uy, Uz) and phi (all numpy, or all CUDA tensors)."""
        arrs = [aP, pPrime, p, U[0], U[1], U[2], phi]
        pm = [ptr_and_mem(a) for a in arrs]
        if len({m for _, m in pm}) != 1:
            raise ValueError("all arrays must live in the same memory")
        check(self.L.simall_correct_fields(self.handle, float(rho), float(urfP), *[x for x, _ in pm], pm[0][1]),
              self.ctx.handle)

    # -- momentum --------------------------------------------------------------------
    def assemble_momentum(self, rho: float, mu: float, urfU: float, U, p, phi, dt: float = 0.0, Un=None, Unm1=None,
                          bdf2: bool = False):
        """assemble_momentum for all three components at once (one matrix,
        three right-hand sides).  U, Un, Unm1: (3, n_cells) arrays or CUDA
        tensors; the result stays on the device (momentum_download)."""
        o = _lib.MomentumOptions(float(rho), float(mu), float(urfU), float(dt), int(bool(bdf2)), 0)
        args = [ptr_and_mem(a) for a in (U, p, phi)]
        mem = args[0][1]
        extra = [ptr_and_mem(a)[0] if a is not None else None for a in (Un, Unm1)]
        for a in (Un, Unm1):
            if a is not None and ptr_and_mem(a)[1] != mem:
                raise ValueError("all arrays must live in the same memory")
        if any(m != mem for _, m in args):
            raise ValueError("all arrays must live in the same memory")
        check(self.L.simall_assemble_momentum(self.handle, C.byref(o), *[q for q, _ in args], *extra, mem),
              self.ctx.handle)

    def momentum_download(self):
        """(values[nnz], rhs[3, n_cells], aP[n_cells]) of the last momentum assembly."""
        v = np.empty(self.nnz)
        r = np.empty((3, self.n))
        a = np.empty(self.n)
        check(self.L.simall_momentum_download(self.handle, v.ctypes.data, r.ctypes.data, a.ctypes.data),
              self.ctx.handle)
        return v, r, a

    def momentum_device_arrays(self):
        """Raw device addresses (values, rhs[3][n], aP) of the last momentum assembly."""
        a = [C.c_void_p() for _ in range(3)]
        check(self.L.simall_momentum_device_arrays(self.handle, *[C.byref(v) for v in a]), self.ctx.handle)
        return tuple(v.value for v in a)

    def assemble_face_conductance(self, rho: float, k, pb, src):
        """Face-conductance operator: coef_f = k_f g_f, Dirichlet values pb on
        pressure-boundary faces, rhs from the cell source src."""
        pk, mk = ptr_and_mem(k)
        pp, mp = ptr_and_mem(pb)
        ps_, ms = ptr_and_mem(src)
        if not (mk == mp == ms):
            raise ValueError("k, pb and src must live in the same memory")
        check(self.L.simall_assemble_face_conductance(self.handle, float(rho), pk, pp, ps_, mk), self.ctx.handle)

    def face_conductance_gradient(self, rho: float, k, pb, x, lam, dk=None, dpb=None):
        if dk is None:
            dk = np.empty(self.mesh.n_faces)
            dpb = np.empty(self.mesh.n_faces)
        args = [ptr_and_mem(a) for a in (k, pb, x, lam, dk, dpb)]
        mem = args[0][1]
        if any(m != mem for _, m in args):
            raise ValueError("all arrays must live in the same memory")
        check(self.L.simall_face_conductance_gradient(self.handle, float(rho), *[p for p, _ in args], mem),
              self.ctx.handle)
        return dk, dpb

    def adjoint(self, solver: GpuCGSolver, rho: float, k, pb, x, dLdx, lam=None, dk=None, dpb=None):
        """lambda = A^-T dL/dx (PCG), then dL/dk and dL/dpb per face."""
        if lam is None:
            lam = np.empty(self.n)
            dk = np.empty(self.mesh.n_faces)
            dpb = np.empty(self.mesh.n_faces)
        args = [ptr_and_mem(a) for a in (k, pb, x, dLdx, lam, dk, dpb)]
        mem = args[0][1]
        if any(m != mem for _, m in args):
            raise ValueError("all arrays must live in the same memory")
        check(self.L.simall_adjoint_face_conductance(self.handle, solver.handle, float(rho), *[p for p, _ in args],
                                                     mem, C.byref(solver.stats)), self.ctx.handle)
        return lam, dk, dpb

    def download(self):
        v = np.empty(self.nnz)
        r = np.empty(self.n)
        check(self.L.simall_pressure_system_download(self.handle, v.ctypes.data, r.ctypes.data), self.ctx.handle)
        return v, r

    def solve(self, solver: GpuCGSolver, x=None):
        """Solve the assembled system; x: numpy (default) or a CUDA tensor."""
        if x is None:
            x = np.empty(self.n)
        px, mx = ptr_and_mem(x)
        check(self.L.simall_pressure_system_solve(self.handle, solver.handle, px, mx, C.byref(solver.stats)),
              self.ctx.handle)
        return x

    def close(self):
        if getattr(self, "handle", None) and getattr(self.ctx, "handle", None):
            self.L.simall_pressure_system_destroy(self.handle)
        self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
