"""Python mirror of optimization::SimpTopology (src/optimization/SimpTopology.hpp:36-80)
on the device, and the glue that feeds it a sensitivity from this library's
adjoint (simall_adjoint_face_conductance): thermal compliance of a
face-conductance Poisson problem whose cell conductivity is the SIMP
property."""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _lib
from ._lib import check
from .fields import DeviceFieldRegistry
from .mesh import MeshSoA, PressureSystem
from .solver import register_child


@dataclass
class SimpConfig:
    """SimpConfig (src/optimization/SimpTopology.hpp:36-46), same defaults."""

    penalty: float = 3.0
    K_min: float = 1e-9
    K_max: float = 1.0
    filterRadius: float = 0.0
    volumeFraction: float = 0.4
    move: float = 0.2
    damping: float = 0.5
    rhoMin: float = 1e-3


class GpuSimpTopology:
    """initialize() at construction; step() returns the L1 design change.
    The design fields live in `fields` (a DeviceFieldRegistry)."""

    def __init__(self, system: PressureSystem, fields: DeviceFieldRegistry, cfg: SimpConfig | None = None):
        self.system = system
        self.fields = fields
        self.ctx = system.ctx
        self.L = self.ctx.L
        c = cfg or SimpConfig()
        self.cfg = c
        sc = _lib.SimpConfig(c.penalty, c.K_min, c.K_max, c.filterRadius, c.volumeFraction, c.move, c.damping,
                             c.rhoMin)
        h = C.c_void_p()
        check(self.L.simall_simp_create(system.handle, fields.handle, C.byref(sc), C.byref(h)), self.ctx.handle)
        self.handle = h.value
        register_child(self)
        self.ctx.children.add(self)

    def step(self) -> float:
        ch = C.c_double()
        check(self.L.simall_simp_step(self.handle, C.byref(ch)), self.ctx.handle)
        return ch.value

    def close(self):
        if getattr(self, "handle", None) and getattr(self.ctx, "handle", None):
            self.L.simall_simp_destroy(self.handle)
        self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def face_conductance(mesh: MeshSoA, K: np.ndarray, dirichlet: np.ndarray):
    """Cell conductivity -> face conductance: harmonic mean on interior faces,
    the owner's value on Dirichlet faces, 0 on the other boundary faces; and
    dk_f/dK_owner, dk_f/dK_neighbour for the chain rule."""
    o = mesh.owner.astype(np.int64)
    nb = mesh.neighbor.astype(np.int64)
    inner = mesh.neighbor != np.iinfo(np.uint64).max
    Ko = K[o]
    Kn = np.where(inner, K[np.where(inner, nb, 0)], 0.0)
    s = Ko + Kn
    k = np.where(inner, 2.0 * Ko * Kn / np.where(inner, s, 1.0), np.where(dirichlet, Ko, 0.0))
    dko = np.where(inner, 2.0 * Kn * Kn / np.where(inner, s * s, 1.0), np.where(dirichlet, 1.0, 0.0))
    dkn = np.where(inner, 2.0 * Ko * Ko / np.where(inner, s * s, 1.0), 0.0)
    return k, dko, dkn


def compliance_sensitivity(system: PressureSystem, solver, mesh: MeshSoA, K: np.ndarray, q: np.ndarray,
                           dirichlet: np.ndarray, T_wall: float = 0.0):
    """Thermal compliance J = q . T of -div(K grad T) = q (T = T_wall on the
    Dirichlet faces): the forward solve and the adjoint through the C ABI
    (simall_assemble_face_conductance, simall_pressure_system_solve,
    simall_adjoint_face_conductance), then dJ/dK per cell by the chain rule
    of the harmonic face mean.  Returns (J, dJ/dK)."""
    k, dko, dkn = face_conductance(mesh, K, dirichlet)
    pb = np.where(dirichlet, T_wall, 0.0)
    system.assemble_face_conductance(1.0, k, pb, q)
    T = system.solve(solver)
    J = float(q @ T)
    _, dk, _ = system.adjoint(solver, 1.0, k, pb, T, q)
    o = mesh.owner.astype(np.int64)
    inner = mesh.neighbor != np.iinfo(np.uint64).max
    dK = np.zeros(mesh.n_cells)
    np.add.at(dK, o, dk * dko)
    np.add.at(dK, mesh.neighbor[inner].astype(np.int64), dk[inner] * dkn[inner])
    return J, dK
