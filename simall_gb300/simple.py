"""Python mirror of SimpleAlgorithm (src/solver/SimpleAlgorithm.hpp:60-170),
PisoAlgorithm and PimpleAlgorithm on the device: `GpuSimpleAlgorithm(mesh,
bcs, momentum_solver, pressure_solver, options)` -- options a SimpleOptions,
PisoOptions or PimpleOptions -- with `iterate()` and `advance_time_step(n)`
returning the reference's SimpleResiduals (mom[3], cont).  U, p and phi stay
in device memory between calls; `fields()` copies them out."""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _lib
from ._lib import check
from .mesh import MeshSoA, PressureSystem
from .solver import Context, GpuCGSolver, default_context, ptr_and_mem, register_child


@dataclass
class SimpleOptions:
    """SimpleOptions (src/solver/SimpleAlgorithm.hpp:43-57), same defaults;
    simplec selects PvCouplingVariant::SIMPLEC, bdf2 TemporalScheme::BDF2."""

    urfU: float = 0.7
    urfP: float = 0.3
    rho: float = 1.0
    mu: float = 1.0e-3
    dt: float = 0.0
    bdf2: bool = False
    simplec: bool = False


@dataclass
class PisoOptions:
    """PisoOptions (src/solver/PisoAlgorithm.hpp:33-41), same defaults; PISO
    runs without under-relaxation (PisoAlgorithm::to_simple_opts)."""

    nCorrectors: int = 2
    nNonOrthCorr: int = 0
    rho: float = 1.0
    mu: float = 1.0e-3
    dt: float = 1.0e-3
    bdf2: bool = True


@dataclass
class PimpleOptions:
    """PimpleOptions (src/solver/PimpleAlgorithm.hpp:37-59), same defaults;
    with one outer corrector the under-relaxation is off, as
    PimpleAlgorithm::to_simple_opts does."""

    nOuterCorrectors: int = 2
    nCorrectors: int = 2
    nNonOrthCorr: int = 0
    momentumPredictor: bool = True
    urfU: float = 0.7
    urfP: float = 0.3
    tolU: float = 0.0
    tolP: float = 0.0
    rho: float = 1.0
    mu: float = 1.0e-3
    dt: float = 1.0e-3
    bdf2: bool = True


@dataclass
class SimpleResiduals:
    mom: tuple
    cont: float
    iterations: tuple
    outer: int = 0


class GpuSimpleAlgorithm:
    """bcs: (zone, BCType ordinal[, (ux, uy, uz)]) in the reference's order
    (the first spec of a zone wins, as find_bc)."""

    def __init__(self, mesh: MeshSoA, bcs, momentum: GpuCGSolver, pressure: GpuCGSolver,
                 options: SimpleOptions | None = None, ctx: Context | None = None):
        self.ctx = ctx or default_context()
        self.L = self.ctx.L
        self.mesh = mesh
        self.options = options or SimpleOptions()
        self.system = PressureSystem(mesh, [(int(b[0]), int(b[1])) for b in bcs], ctx=self.ctx)
        vel = [(int(b[0]), tuple(b[2])) for b in bcs if len(b) > 2 and int(b[1]) in (2, 4)]
        self.system.setup_field_loops(vel)
        self.momentum = momentum
        self.pressure = pressure
        o = _lib.SimpleOptions()
        self.L.simall_simple_options_default(C.byref(o))
        opt = self.options
        if isinstance(opt, PisoOptions):
            o.urfU, o.urfP, o.rho, o.mu, o.dt = 1.0, 1.0, float(opt.rho), float(opt.mu), float(opt.dt)
            o.bdf2 = int(bool(opt.bdf2))
            o.n_correctors = int(opt.nCorrectors)
            o.n_non_orth_corr = int(opt.nNonOrthCorr)
        elif isinstance(opt, PimpleOptions):
            piso_mode = opt.nOuterCorrectors <= 1
            o.urfU = 1.0 if piso_mode else float(opt.urfU)
            o.urfP = 1.0 if piso_mode else float(opt.urfP)
            o.rho, o.mu, o.dt = float(opt.rho), float(opt.mu), float(opt.dt)
            o.bdf2 = int(bool(opt.bdf2))
            o.n_outer_correctors = int(opt.nOuterCorrectors)
            o.n_correctors = int(opt.nCorrectors)
            o.n_non_orth_corr = int(opt.nNonOrthCorr)
            o.momentum_predictor = int(bool(opt.momentumPredictor))
            o.tol_u, o.tol_p = float(opt.tolU), float(opt.tolP)
        else:
            o.urfU, o.urfP, o.rho, o.mu, o.dt = (float(v) for v in (opt.urfU, opt.urfP, opt.rho, opt.mu, opt.dt))
            o.bdf2 = int(bool(opt.bdf2))
            o.simplec = int(bool(opt.simplec))
        h = C.c_void_p()
        check(self.L.simall_simple_create(self.system.handle, momentum.handle, pressure.handle, C.byref(o),
                                          C.byref(h)), self.ctx.handle)
        self.handle = h.value
        register_child(self)
        self.ctx.children.add(self)

    def bind_fields(self, registry):
        """Keep U and p in a DeviceFieldRegistry (vector "U", scalar "p")."""
        check(self.L.simall_simple_bind_fields(self.handle, registry.handle), self.ctx.handle)
        self._registry = registry

    def set_fields(self, U=None, p=None):
        """U: (3, n_cells), p: (n_cells,) -- numpy or CUDA tensors."""
        pu, mu_ = ptr_and_mem(U) if U is not None else (None, None)
        pp, mp = ptr_and_mem(p) if p is not None else (None, None)
        mem = mu_ if mu_ is not None else mp
        if mu_ is not None and mp is not None and mu_ != mp:
            raise ValueError("U and p must live in the same memory")
        check(self.L.simall_simple_set_fields(self.handle, pu, pp, mem or 0), self.ctx.handle)

    def fields(self):
        """(U[3, n_cells], p, phi) copied to the host."""
        nC, nF = self.mesh.n_cells, self.mesh.n_faces
        U = np.empty((3, nC))
        p = np.empty(nC)
        phi = np.empty(nF)
        check(self.L.simall_simple_get_fields(self.handle, U.ctypes.data, p.ctypes.data, phi.ctypes.data, 0),
              self.ctx.handle)
        return U, p, phi

    def device_fields(self):
        a = [C.c_void_p() for _ in range(3)]
        check(self.L.simall_simple_device_fields(self.handle, *[C.byref(v) for v in a]), self.ctx.handle)
        return tuple(v.value for v in a)

    @staticmethod
    def _res(r) -> SimpleResiduals:
        return SimpleResiduals(tuple(r.mom), float(r.cont), tuple(r.iterations), int(r.outer))

    def iterate(self) -> SimpleResiduals:
        r = _lib.SimpleResiduals()
        check(self.L.simall_simple_iterate(self.handle, C.byref(r)), self.ctx.handle)
        return self._res(r)

    def advance_time_step(self, n_inner: int = 5) -> SimpleResiduals:
        r = _lib.SimpleResiduals()
        check(self.L.simall_simple_advance_time_step(self.handle, int(n_inner), C.byref(r)), self.ctx.handle)
        return self._res(r)

    def close(self):
        if getattr(self, "handle", None) and getattr(self.ctx, "handle", None):
            self.L.simall_simple_destroy(self.handle)
        self.handle = None
        if getattr(self, "system", None) is not None:
            self.system.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
