"""Seeded synthetic inputs with the shapes of the pressure-path workloads.

All randomness comes from numpy's PCG64 (`np.random.default_rng(seed)`), and
every value derived from it uses correctly rounded IEEE operations only
(`portable_exp` instead of np.exp, whose last bits differ between x86_64 and
aarch64 builds of numpy), so the same seed gives the same inputs bit for bit
on every host -- the reference's fixtures are made on one machine and checked
on another.  These produce input data
only (node shifts, aP, face fluxes, right-hand sides, conductances); the
computation under test stays in the library.

Workloads (sizes as named by the pressure-path benchmark set):
  cavity      2-D lid-driven cavity N x N x 1 (SIMPLE trajectory; the systems
              themselves come from the SIMPLE loop)
  poisson3d   N^3 box, interior nodes shifted by U(-0.2,0.2)*h per
              coordinate, RCM, aP = 1, interior face flux N(0,1), all walls
              (cell-0 pin)
  varcoef     N^3 box, k_c = exp(N(0,1)) per cell -> aP = 1/k_c (harmonic
              face averaging), PressureOutlet (p' = 0) on x = 0, rhs N(0,1)
  batched     many 2-D cavity-type systems, sides log-uniform in [32, 256],
              aP = 1, rhs N(0,1) with its mean removed, cell-0 pin
  facek       N^3 box with face conductances exp(N(0,0.5)) and Dirichlet
              values N(0,1) on x = 0
"""
from __future__ import annotations

import numpy as np

from .mesh import BCType, MeshSoA, cartesian, rcm

DEFAULT_SEED = 42

# Cody-Waite split of ln 2: LN2_HI has 32 significant bits, so k * LN2_HI is
# exact for |k| < 2^20; INV_LN2 = 1/ln 2 rounded.
_LN2_HI = float.fromhex("0x1.62e42feep-1")
_LN2_LO = float.fromhex("0x1.a39ef35793c76p-33")
_INV_LN2 = float.fromhex("0x1.71547652b82fep+0")
# 1/n! for n = 2..13 (Taylor series of e^r - 1 - r on |r| <= ln2/2; the first
# neglected term is below 4e-18)
_INV_FACT = [1.0 / float(np.prod(np.arange(1, n + 1, dtype=np.float64))) for n in range(2, 14)]


def portable_exp(x) -> np.ndarray:
    """e^x from +, -, *, rint and ldexp alone: x = k ln2 + r with |r| <=
    ln2/2 (Cody-Waite), e^r by its Taylor polynomial in Horner form, scaled
    by 2^k.  Within a few ulp of e^x for |x| < 700, and bit-identical on every
    IEEE host (numpy evaluates each operation separately, correctly rounded)."""
    x = np.asarray(x, np.float64)
    k = np.rint(x * _INV_LN2)
    r = (x - k * _LN2_HI) - k * _LN2_LO
    q = np.full_like(r, _INV_FACT[-1])
    for c in reversed(_INV_FACT[:-1]):
        q = q * r + c
    e = 1.0 + (r + r * (r * q))
    return np.ldexp(e, k.astype(np.int64))
ALL_WALLS = [(z, int(BCType.NoSlipWall)) for z in (1, 2, 3, 4, 5, 6)]
X0_OUTLET = [(1, int(BCType.PressureOutlet))] + [(z, int(BCType.NoSlipWall)) for z in (2, 3, 4, 5, 6)]
CAVITY = [(z, int(BCType.NoSlipWall)) for z in (1, 2, 3, 5, 6)] + [(4, int(BCType.MovingWall))]


def interior_node_shift(nx, ny, nz, ex=1.0, ey=1.0, ez=1.0, amp=0.2, seed=DEFAULT_SEED) -> np.ndarray:
    """(3, nNodes) displacement: U(-amp, amp) * h per coordinate on nodes
    strictly inside the box, zero on the boundary."""
    rng = np.random.default_rng(seed)
    px, py, pz = nx + 1, ny + 1, nz + 1
    d = rng.uniform(-amp, amp, size=(3, px * py * pz))
    i = np.arange(px)
    j = np.arange(py)
    k = np.arange(pz)
    inner = ((k[:, None, None] > 0) & (k[:, None, None] < nz) & (j[None, :, None] > 0) & (j[None, :, None] < ny)
             & (i[None, None, :] > 0) & (i[None, None, :] < nx)).ravel()
    d[:, ~inner] = 0.0
    d[0] *= ex / nx
    d[1] *= ey / ny
    d[2] *= ez / nz
    return d


def poisson3d_mesh(n=128, seed=DEFAULT_SEED, amp=0.2, renumber=True) -> tuple[MeshSoA, tuple | None]:
    m = cartesian(n, n, n, 1.0, 1.0, 1.0, node_shift=interior_node_shift(n, n, n, amp=amp, seed=seed))
    stats = rcm(m) if renumber else None
    return m, stats


def poisson3d_inputs(m: MeshSoA, seed=DEFAULT_SEED):
    """aP = 1; phi = N(0,1) on interior faces, 0 on boundary faces."""
    rng = np.random.default_rng(seed + 1)
    phi = rng.standard_normal(m.n_faces)
    phi[~m.interior()] = 0.0
    return np.ones(m.n_cells), phi


def varcoef_mesh(n=256) -> MeshSoA:
    return cartesian(n, n, n, 1.0, 1.0, 1.0)


def varcoef_inputs(m: MeshSoA, seed=DEFAULT_SEED):
    """aP = 1/k with k = exp(N(0,1)) per cell; phi = 0; rhs N(0,1)."""
    rng = np.random.default_rng(seed + 2)
    k = portable_exp(rng.standard_normal(m.n_cells))
    rhs = rng.standard_normal(m.n_cells)
    return 1.0 / k, np.zeros(m.n_faces), rhs


def batched_sides(count=512, lo=32, hi=256, seed=DEFAULT_SEED) -> np.ndarray:
    rng = np.random.default_rng(seed + 3)
    return np.rint(np.exp(rng.uniform(np.log(lo), np.log(hi), size=count))).astype(np.int64)


def batched_rhs(n: int, rng: np.random.Generator) -> np.ndarray:
    b = rng.standard_normal(n)
    b -= b.mean()
    b[0] = 0.0  # the pinned cell
    return b


def facek_inputs(m: MeshSoA, seed=DEFAULT_SEED, sigma=0.5):
    """k_f = exp(N(0, sigma)) on interior and x=0 faces; pb ~ N(0,1) on x=0
    faces; cell source N(0,1)."""
    rng = np.random.default_rng(seed + 4)
    k = portable_exp(sigma * rng.standard_normal(m.n_faces))
    pb = rng.standard_normal(m.n_faces)
    dirichlet = (~m.interior()) & (m.boundary_zone == 1)
    k[(~m.interior()) & ~dirichlet] = 0.0
    pb[~dirichlet] = 0.0
    src = rng.standard_normal(m.n_cells)
    return k, pb, dirichlet.astype(np.uint8), src


def cavity_pressure_matrix(side: int, ctx=None):
    """The pressure-correction matrix of a side x side x 1 lid-driven-cavity
    grid (extent 1 x 1 x 1/side, all walls, aP = 1, rho = 1) assembled by the
    library's device assembly; returns (rowPtr, colIdx, values)."""
    from .mesh import PressureSystem

    m = cartesian(side, side, 1, 1.0, 1.0, 1.0 / side)
    ps = PressureSystem(m, ALL_WALLS, ctx=ctx)
    ps.assemble(1.0, np.ones(m.n_cells), np.zeros(m.n_faces))
    rp, ci = ps.pattern()
    v, _ = ps.download()
    ps.close()
    return rp, ci, v


def batched_cavity_systems(count=512, lo=32, hi=256, seed=DEFAULT_SEED, ctx=None):
    """`count` cavity pressure systems with sides log-uniform in [lo, hi] and
    rhs N(0,1) with the mean removed and the pinned cell zeroed.
    Returns (systems, rhs_list, sides)."""
    sides = batched_sides(count, lo, hi, seed)
    cache = {}
    systems, rhs = [], []
    rng = np.random.default_rng(seed + 5)
    for s in sides:
        s = int(s)
        if s not in cache:
            cache[s] = cavity_pressure_matrix(s, ctx)
        systems.append(cache[s])
        rhs.append(batched_rhs(s * s, rng))
    return systems, rhs, sides
