// Pressure-correction assembly on the device: the GB300 replacement of
// SimpleAlgorithm::build_sparsity + assemble_pressure_correction
// (src/solver/SimpleAlgorithm.cpp:49-98, :358-447), periodic faces included
// (build_periodic_pairs :101-186, the twin column :71-72, the coupling of a
// periodic face with its twin face's owner :411-419).
//
// The reference walks the faces once and scatters each coefficient into four
// CSR slots through a linear column search (find_col/add_at, :23-35).  Here:
//   create()  builds the CSR pattern on the host exactly as build_sparsity
//             does, lists every cell's faces in ascending face id together
//             with the CSR slot of the neighbour column, and precomputes the
//             static face geometry |A|^2 and |d.A| on the device from the
//             mesh SoA (same operation order, no FMA contraction);
//   assemble  k_face_coef  one thread per face: coef_f from aP (gathered);
//             k_cell_rows  one thread per cell: writes its whole CSR row and
//                          rhs entry, summing its faces' contributions in
//                          ascending face id -- the order in which the
//                          reference's face loop adds them -- so values and
//                          rhs are bit-identical to the reference and no
//                          atomics are needed.
#include "device.cuh"
#include "solver.hpp"

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstring>
#include <new>

#include "pressure_system.hpp"

namespace simall {

namespace {


// |A|^2 and |d.A| with the reference's operation order (SimpleAlgorithm.cpp:371-378, :417-420).
__global__ void __launch_bounds__(kBlock) k_face_geometry(int64_t nF, const int32_t *__restrict__ owner,
                                                          const int32_t *__restrict__ neighbor,
                                                          const uint8_t *__restrict__ kind,
                                                          const double *__restrict__ ax, const double *__restrict__ ay,
                                                          const double *__restrict__ az, const double *__restrict__ fx,
                                                          const double *__restrict__ fy, const double *__restrict__ fz,
                                                          const double *__restrict__ cx, const double *__restrict__ cy,
                                                          const double *__restrict__ cz, double *__restrict__ amag2,
                                                          double *__restrict__ ddotA)
{
    for (int64_t f = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; f < nF; f += (int64_t)gridDim.x * blockDim.x) {
        const double Ax = ax[f], Ay = ay[f], Az = az[f];
        amag2[f] = __dadd_rn(__dadd_rn(__dmul_rn(Ax, Ax), __dmul_rn(Ay, Ay)), __dmul_rn(Az, Az));
        const int o = owner[f], n = neighbor[f];
        double dx = 0.0, dy = 0.0, dz = 0.0;
        if (n >= 0) {
            dx = __dsub_rn(cx[n], cx[o]);
            dy = __dsub_rn(cy[n], cy[o]);
            dz = __dsub_rn(cz[n], cz[o]);
        } else if (kind[f] == kPressure || kind[f] == kPeriodic) {
            dx = __dsub_rn(fx[f], cx[o]);
            dy = __dsub_rn(fy[f], cy[o]);
            dz = __dsub_rn(fz[f], cz[o]);
        }
        ddotA[f] = fabs(__dadd_rn(__dadd_rn(__dmul_rn(dx, Ax), __dmul_rn(dy, Ay)), __dmul_rn(dz, Az)));
    }
}

// coef_f = rho |A|^2 / max(aPf |d.A|, 1e-30)   (SimpleAlgorithm.cpp:379-393, :421-428)
__global__ void __launch_bounds__(kBlock) k_face_coef(int64_t nF, double rho, const int32_t *__restrict__ owner,
                                                      const int32_t *__restrict__ neighbor,
                                                      const uint8_t *__restrict__ kind,
                                                      const double *__restrict__ amag2,
                                                      const double *__restrict__ ddotA, const double *__restrict__ aP,
                                                      double *__restrict__ coef)
{
    for (int64_t f = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; f < nF; f += (int64_t)gridDim.x * blockDim.x) {
        const uint8_t k = kind[f];
        double c = 0.0;
        if (k != kOtherBoundary) {
            const int o = owner[f];
            double den;
            if (k == kInterior) {
                const double dOwn = std_max(__ldg(aP + o), 1e-30);
                const double dNbr = std_max(__ldg(aP + neighbor[f]), 1e-30);
                const double aPf = __dmul_rn(0.5, __dadd_rn(dOwn, dNbr));
                den = __dmul_rn(aPf, ddotA[f]);
            } else {
                den = __dmul_rn(std_max(__ldg(aP + o), 1e-30), ddotA[f]);
            }
            c = __ddiv_rn(__dmul_rn(rho, amag2[f]), std_max(den, 1e-30));
        }
        coef[f] = c;
    }
}

// One CSR row and one rhs entry per thread, faces in ascending id.
__global__ void __launch_bounds__(kBlock) k_cell_rows(int64_t nC, const int32_t *__restrict__ rowPtr,
                                                      const int32_t *__restrict__ cfOff,
                                                      const int32_t *__restrict__ cfEnt,
                                                      const int32_t *__restrict__ cfSlot,
                                                      const int32_t *__restrict__ diagSlot,
                                                      const uint8_t *__restrict__ kind,
                                                      const double *__restrict__ coef, const double *__restrict__ phi,
                                                      int anyDirichlet, double *__restrict__ values,
                                                      double *__restrict__ rhs)
{
    for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < nC; c += (int64_t)gridDim.x * blockDim.x) {
        const int r0 = rowPtr[c], r1 = rowPtr[c + 1];
        for (int k = r0; k < r1; ++k)
            values[k] = 0.0;
        const int kd = diagSlot[c];
        double diag = 0.0, b = 0.0;
        for (int e = cfOff[c]; e < cfOff[c + 1]; ++e) {
            const int ent = cfEnt[e];
            const int f = ent & 0x7fffffff;
            const bool isNbr = ent < 0;
            const double cf = __ldg(coef + f);
            const uint8_t k = kind[f];
            if (k != kOtherBoundary)
                diag = __dadd_rn(diag, cf);
            if (k == kInterior || k == kPeriodic) {
                // the other cell's column: the neighbour, or the periodic twin
                // face's owner -- which is this cell itself on a mesh one cell
                // wide across the periodic pair: then the diagonal
                const int slot = cfSlot[e];
                if (slot == kd)
                    diag = __dadd_rn(diag, -cf);
                else if (slot >= 0)
                    values[slot] = __dadd_rn(values[slot], -cf);
            }
            const double ph = __ldg(phi + f);
            b = isNbr ? __dadd_rn(b, ph) : __dsub_rn(b, ph);
        }
        if (!anyDirichlet && c == 0) {
            diag = __dmul_rn(diag, 1.0e6);
            b = 0.0;
        }
        values[kd] = diag;
        rhs[c] = b;
    }
}

// ---------------------------------------------------------------- face-conductance operator
// An extension of the assembly above (the reference cannot express per-face
// conductances or non-zero Dirichlet values): coef_f = k_f * g_f with
// g_f = rho |A|^2 / max(|d.A|, 1e-30) -- the reference face coefficient with
// k_f in place of 1/aP_f -- on interior and pressure-boundary faces; a
// pressure-boundary face also adds coef_f * pb_f to its cell's rhs, which
// starts from the cell source.  No pin.
__device__ __forceinline__ double face_g(double rho, double amag2, double ddotA)
{
    return __ddiv_rn(__dmul_rn(rho, amag2), std_max(ddotA, 1e-30));
}

__global__ void __launch_bounds__(kBlock) k_face_coef_k(int64_t nF, double rho, const uint8_t *__restrict__ kind,
                                                        const double *__restrict__ amag2,
                                                        const double *__restrict__ ddotA, const double *__restrict__ k,
                                                        double *__restrict__ coef)
{
    for (int64_t f = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; f < nF; f += (int64_t)gridDim.x * blockDim.x)
        coef[f] = kind[f] == kOtherBoundary ? 0.0 : __dmul_rn(k[f], face_g(rho, amag2[f], ddotA[f]));
}

__global__ void __launch_bounds__(kBlock) k_cell_rows_k(int64_t nC, const int32_t *__restrict__ rowPtr,
                                                        const int32_t *__restrict__ cfOff,
                                                        const int32_t *__restrict__ cfEnt,
                                                        const int32_t *__restrict__ cfSlot,
                                                        const int32_t *__restrict__ diagSlot,
                                                        const uint8_t *__restrict__ kind,
                                                        const double *__restrict__ coef, const double *__restrict__ pb,
                                                        const double *__restrict__ src, double *__restrict__ values,
                                                        double *__restrict__ rhs)
{
    for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < nC; c += (int64_t)gridDim.x * blockDim.x) {
        const int r0 = rowPtr[c], r1 = rowPtr[c + 1];
        for (int q = r0; q < r1; ++q)
            values[q] = 0.0;
        double diag = 0.0, b = src[c];
        for (int e = cfOff[c]; e < cfOff[c + 1]; ++e) {
            const int f = cfEnt[e] & 0x7fffffff;
            const uint8_t kd = kind[f];
            if (kd == kOtherBoundary)
                continue;
            const double cf = __ldg(coef + f);
            diag = __dadd_rn(diag, cf);
            if (kd == kInterior) {
                const int slot = cfSlot[e];
                if (slot >= 0)
                    values[slot] = __dadd_rn(values[slot], -cf);
            } else {
                b = __dadd_rn(b, __dmul_rn(cf, __ldg(pb + f)));
            }
        }
        values[diagSlot[c]] = diag;
        rhs[c] = b;
    }
}

// dL/dk_f and dL/dpb_f from x and the adjoint lambda = A^-T dL/dx, recomputing
// g_f from the stored geometry (no coefficient is kept from the forward pass):
//   interior f:      dk = -g (lambda_o - lambda_n)(x_o - x_n)
//   pressure face f: dk = -g lambda_o (x_o - pb_f),  dpb = k_f g lambda_o
// This is -(dR/dalpha)^T lambda of solve_discrete_adjoint
// (src/adjoint/DiscreteAdjoint.cpp:170-182) for R = A(k) x - b(k, pb).
__global__ void __launch_bounds__(kBlock) k_face_k_gradient(int64_t nF, double rho, const int32_t *__restrict__ owner,
                                                            const int32_t *__restrict__ neighbor,
                                                            const uint8_t *__restrict__ kind,
                                                            const double *__restrict__ amag2,
                                                            const double *__restrict__ ddotA,
                                                            const double *__restrict__ k, const double *__restrict__ pb,
                                                            const double *__restrict__ x,
                                                            const double *__restrict__ lambda, double *__restrict__ dk,
                                                            double *__restrict__ dpb)
{
    for (int64_t f = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; f < nF; f += (int64_t)gridDim.x * blockDim.x) {
        const uint8_t kd = kind[f];
        double gk = 0.0, gp = 0.0;
        if (kd != kOtherBoundary) {
            const double g = face_g(rho, amag2[f], ddotA[f]);
            const int o = owner[f];
            const double lo = __ldg(lambda + o), xo = __ldg(x + o);
            if (kd == kInterior) {
                const int n = neighbor[f];
                gk = __dmul_rn(__dmul_rn(-g, __dsub_rn(lo, __ldg(lambda + n))), __dsub_rn(xo, __ldg(x + n)));
            } else {
                gk = __dmul_rn(__dmul_rn(-g, lo), __dsub_rn(xo, __ldg(pb + f)));
                gp = __dmul_rn(__dmul_rn(k[f], g), lo);
            }
        }
        dk[f] = gk;
        dpb[f] = gp;
    }
}

}  // namespace

}  // namespace simall

using namespace simall;

namespace simall {
namespace {

// SIMPLEC denominator (SimpleAlgorithm.cpp:380-390, 401-409):
// den_c = max(aP_c - sum_{k != c} |a_mom,ck|, 1e-30), the sum in column order.
__global__ void __launch_bounds__(kBlock) k_simplec_den(int64_t nC, const int32_t *__restrict__ rowPtr,
                                                        const int32_t *__restrict__ colIdx,
                                                        const double *__restrict__ mom, const double *__restrict__ aP,
                                                        double *__restrict__ den)
{
    for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < nC; c += (int64_t)gridDim.x * blockDim.x) {
        double sumOff = 0.0;
        for (int k = rowPtr[c]; k < rowPtr[c + 1]; ++k)
            if (colIdx[k] != c)
                sumOff = __dadd_rn(sumOff, fabs(mom[k]));
        den[c] = std_max(__dsub_rn(aP[c], sumOff), 1e-30);
    }
}

// Periodic pairing, the search: for each face a of zone group A (centroid plus
// the group translation, formed on the host), the face of group B whose
// centroid is nearest, squared distance in the reference's operation order
// (SimpleAlgorithm.cpp:167-176) and the first minimum in B's order.  B is
// streamed through shared memory in tiles.
constexpr int kPairTile = 1024;

__global__ void __launch_bounds__(kBlock) k_periodic_nearest(int nA, const double *__restrict__ ax,
                                                             const double *__restrict__ ay,
                                                             const double *__restrict__ az, int nB,
                                                             const double *__restrict__ bx,
                                                             const double *__restrict__ by,
                                                             const double *__restrict__ bz, int *__restrict__ best)
{
    __shared__ double tx[kPairTile], ty[kPairTile], tz[kPairTile];
    const int a = blockIdx.x * blockDim.x + threadIdx.x;
    const double px = a < nA ? ax[a] : 0.0, py = a < nA ? ay[a] : 0.0, pz = a < nA ? az[a] : 0.0;
    double bestd2 = DBL_MAX;
    int bi = -1;
    for (int t0 = 0; t0 < nB; t0 += kPairTile) {
        const int cnt = min(kPairTile, nB - t0);
        __syncthreads();
        for (int j = threadIdx.x; j < cnt; j += blockDim.x) {
            tx[j] = bx[t0 + j];
            ty[j] = by[t0 + j];
            tz[j] = bz[t0 + j];
        }
        __syncthreads();
        for (int j = 0; j < cnt; ++j) {
            const double dx = __dsub_rn(tx[j], px), dy = __dsub_rn(ty[j], py), dz = __dsub_rn(tz[j], pz);
            const double d2 = __dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz));
            if (d2 < bestd2) {
                bestd2 = d2;
                bi = t0 + j;
            }
        }
    }
    if (a < nA)
        best[a] = bi;
}

// SimpleAlgorithm::build_periodic_pairs (SimpleAlgorithm.cpp:101-186) for the
// Periodic specs of bcs: twin[nF] (-1 where none).  Groups, translations and
// the writes of the result follow the reference on the host, face order kept;
// the O(|A| |B|) nearest-centroid search runs on the device.
int periodic_pairs(simall_context *ctx, const simall_mesh_view *m, const simall_boundary *bcs, int n_bcs,
                   std::vector<int32_t> &twin)
{
    const int64_t nF = m->n_faces;
    twin.assign(static_cast<size_t>(nF), -1);
    std::vector<uint32_t> pz;
    for (int i = 0; i < n_bcs; ++i)
        if (bcs[i].type == SIMALL_BC_PERIODIC)
            pz.push_back(bcs[i].zone);
    if (pz.size() < 2)
        return SIMALL_OK;
    std::vector<std::vector<int32_t>> byZone(pz.size());
    for (int64_t f = 0; f < nF; ++f) {
        if (m->neighbor[f] != ~0ull)
            continue;
        for (size_t i = 0; i < pz.size(); ++i)
            if (pz[i] == m->boundary_zone[f]) {
                byZone[i].push_back(static_cast<int32_t>(f));
                break;
            }
    }
    cudaStream_t st = ctx->stream;
    for (size_t z = 0; z + 1 < pz.size(); z += 2) {
        const auto &A = byZone[z];
        const auto &B = byZone[z + 1];
        if (A.empty() || B.empty())
            continue;
        double Ax = 0, Ay = 0, Az = 0, Bx = 0, By = 0, Bz = 0;
        for (int32_t f : A) {
            Ax += m->centroid_x[f];
            Ay += m->centroid_y[f];
            Az += m->centroid_z[f];
        }
        for (int32_t f : B) {
            Bx += m->centroid_x[f];
            By += m->centroid_y[f];
            Bz += m->centroid_z[f];
        }
        const double invA = 1.0 / static_cast<double>(A.size()), invB = 1.0 / static_cast<double>(B.size());
        const double tx = Bx * invB - Ax * invA, ty = By * invB - Ay * invA, tz = Bz * invB - Az * invA;
        const int nA = static_cast<int>(A.size()), nB = static_cast<int>(B.size());
        std::vector<double> h(static_cast<size_t>(3 * (nA + nB)));
        for (int i = 0; i < nA; ++i) {
            h[i] = m->centroid_x[A[i]] + tx;
            h[nA + i] = m->centroid_y[A[i]] + ty;
            h[2 * nA + i] = m->centroid_z[A[i]] + tz;
        }
        double *hb = h.data() + 3 * nA;
        for (int j = 0; j < nB; ++j) {
            hb[j] = m->centroid_x[B[j]];
            hb[nB + j] = m->centroid_y[B[j]];
            hb[2 * nB + j] = m->centroid_z[B[j]];
        }
        DevBuf<double> d;
        DevBuf<int> best;
        SIMALL_CUDA_TRY(ctx, d.alloc(h.size()));
        SIMALL_CUDA_TRY(ctx, best.alloc(nA));
        SIMALL_CUDA_TRY(ctx, cudaMemcpyAsync(d.p, h.data(), h.size() * sizeof(double), cudaMemcpyHostToDevice, st));
        const double *db = d.p + 3 * nA;
        k_periodic_nearest<<<(nA + kBlock - 1) / kBlock, kBlock, 0, st>>>(nA, d.p, d.p + nA, d.p + 2 * nA, nB, db,
                                                                          db + nB, db + 2 * nB, best.p);
        SIMALL_LAUNCH_CHECK(ctx);
        std::vector<int> hbest(static_cast<size_t>(nA));
        SIMALL_CUDA_TRY(ctx, cudaMemcpyAsync(hbest.data(), best.p, nA * sizeof(int), cudaMemcpyDeviceToHost, st));
        SIMALL_CUDA_TRY(ctx, cudaStreamSynchronize(st));
        for (int i = 0; i < nA; ++i)  // in A's order: a later face choosing the same b rewrites twin[b]
            if (hbest[i] >= 0) {
                twin[A[i]] = B[hbest[i]];
                twin[B[hbest[i]]] = A[i];
            }
    }
    return SIMALL_OK;
}

}  // namespace
}  // namespace simall

extern "C" {

int simall_pressure_system_create(simall_context *ctx, const simall_mesh_view *m, const simall_boundary *bcs,
                                  int n_bcs, simall_pressure_system **out)
{
    if (!ctx || !m || !out || (n_bcs > 0 && !bcs) || n_bcs < 0)
        return SIMALL_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    const int64_t nC = m->n_cells, nF = m->n_faces;
    if (nC <= 0 || nF <= 0 || nC > INT32_MAX - 1 || nF > INT32_MAX - 1)
        return fail(ctx, SIMALL_ERR_INVALID_ARGUMENT, "mesh sizes out of range");
    if (!m->owner || !m->neighbor || !m->area_x || !m->area_y || !m->area_z || !m->centroid_x || !m->centroid_y ||
        !m->centroid_z || !m->boundary_zone || !m->cell_centroid_x || !m->cell_centroid_y || !m->cell_centroid_z ||
        !m->cell_face_offsets || !m->cell_face_indices)
        return fail(ctx, SIMALL_ERR_INVALID_ARGUMENT, "mesh view has a null array");
    SIMALL_CUDA_TRY(ctx, cudaSetDevice(ctx->device));
    const uint64_t kB = ~0ull;
    // ---- validate ids, classify faces
    std::vector<int32_t> own(static_cast<size_t>(nF)), nbr(static_cast<size_t>(nF));
    std::vector<uint8_t> kind(static_cast<size_t>(nF));
    int anyD = 0;
    for (int64_t f = 0; f < nF; ++f) {
        const uint64_t o = m->owner[f], n = m->neighbor[f];
        if (o >= static_cast<uint64_t>(nC) || (n != kB && n >= static_cast<uint64_t>(nC)))
            return fail(ctx, SIMALL_ERR_INDEX_RANGE, "face %lld: owner/neighbor out of range",
                        static_cast<long long>(f));
        own[f] = static_cast<int32_t>(o);
        nbr[f] = n == kB ? -1 : static_cast<int32_t>(n);
    }
    // periodic pairs first: build_sparsity needs the twins (SimpleAlgorithm.cpp:54-56)
    std::vector<int32_t> twin;
    {
        const int pst = periodic_pairs(ctx, m, bcs, n_bcs, twin);
        if (pst)
            return pst;
    }
    for (int64_t f = 0; f < nF; ++f) {
        const uint64_t n = m->neighbor[f];
        if (n != kB) {
            kind[f] = kInterior;
        } else if (twin[f] >= 0) {
            kind[f] = kPeriodic;  // a periodic twin takes precedence over the zone's spec (:214, :279, :411)
        } else {
            // find_bc: first spec of the zone (SimpleAlgorithm.cpp:191-197)
            int type = -1;
            for (int i = 0; i < n_bcs; ++i)
                if (bcs[i].zone == m->boundary_zone[f]) {
                    type = bcs[i].type;
                    break;
                }
            const bool p = (type == SIMALL_BC_PRESSURE_OUTLET || type == SIMALL_BC_PRESSURE_INLET);
            kind[f] = p ? kPressure : kOtherBoundary;
            anyD |= p ? 1 : 0;
        }
    }
    if (m->cell_face_offsets[0] != 0)
        return fail(ctx, SIMALL_ERR_INVALID_ARGUMENT, "cell_face_offsets[0] != 0");
    for (int64_t c = 0; c < nC; ++c)
        if (m->cell_face_offsets[c + 1] < m->cell_face_offsets[c])
            return fail(ctx, SIMALL_ERR_INVALID_ARGUMENT, "cell_face_offsets not monotone at %lld",
                        static_cast<long long>(c));
    const int64_t ncf = m->cell_face_offsets[nC];
    for (int64_t e = 0; e < ncf; ++e)
        if (m->cell_face_indices[e] >= static_cast<uint64_t>(nF))
            return fail(ctx, SIMALL_ERR_INDEX_RANGE, "cell face index out of range");
    auto *ps = new (std::nothrow) simall_pressure_system;
    if (!ps)
        return SIMALL_ERR_OUT_OF_MEMORY;
    ps->ctx = ctx;
    ps->nC = nC;
    ps->nF = nF;
    ps->anyDirichlet = anyD;
    ps->h_bcs.assign(bcs, bcs + n_bcs);
    ps->h_twin = twin;
    ps->periodic = std::any_of(twin.begin(), twin.end(), [](int32_t t) { return t >= 0; });
    // ---- sparsity (build_sparsity :62-82): {c} U other cells of c's faces, sorted, unique
    ps->h_rowPtr.assign(static_cast<size_t>(nC) + 1, 0);
    ps->h_colIdx.reserve(static_cast<size_t>(ncf) + static_cast<size_t>(nC));
    std::vector<int32_t> diagSlot(static_cast<size_t>(nC));
    {
        std::vector<int32_t> nb;
        for (int64_t c = 0; c < nC; ++c) {
            nb.clear();
            nb.push_back(static_cast<int32_t>(c));
            for (int32_t e = m->cell_face_offsets[c]; e < m->cell_face_offsets[c + 1]; ++e) {
                const int32_t f = static_cast<int32_t>(m->cell_face_indices[e]);
                const int32_t oth = (own[f] == c) ? nbr[f] : own[f];
                if (oth >= 0)
                    nb.push_back(oth);
                else if (twin[f] >= 0)
                    nb.push_back(own[twin[f]]);
            }
            std::sort(nb.begin(), nb.end());
            nb.erase(std::unique(nb.begin(), nb.end()), nb.end());
            const int32_t base = static_cast<int32_t>(ps->h_colIdx.size());
            for (size_t t = 0; t < nb.size(); ++t) {
                if (nb[t] == c)
                    diagSlot[c] = base + static_cast<int32_t>(t);
                ps->h_colIdx.push_back(nb[t]);
            }
            ps->h_rowPtr[c + 1] = static_cast<int32_t>(ps->h_colIdx.size());
        }
    }
    // ---- per-cell face entries as the reference face loop (:366-440) sees them:
    // every face touches its owner and, if interior, its neighbour; visiting
    // faces in ascending id lists each cell's faces in that order.  The slot
    // is the CSR position of the other cell in the cell's row, or -1 where
    // add_at would find no column.
    std::vector<int32_t> cfOff(static_cast<size_t>(nC) + 1, 0);
    for (int64_t f = 0; f < nF; ++f) {
        cfOff[own[f] + 1]++;
        if (nbr[f] >= 0)
            cfOff[nbr[f] + 1]++;
    }
    for (int64_t c = 0; c < nC; ++c)
        cfOff[c + 1] += cfOff[c];
    std::vector<int32_t> cfEnt(static_cast<size_t>(cfOff[nC])), cfSlot(static_cast<size_t>(cfOff[nC]));
    {
        std::vector<int32_t> fill(cfOff.begin(), cfOff.end() - 1);
        auto slot_of = [&](int32_t row, int32_t col) -> int32_t {
            const int32_t *b0 = ps->h_colIdx.data() + ps->h_rowPtr[row];
            const int32_t *b1 = ps->h_colIdx.data() + ps->h_rowPtr[row + 1];
            const int32_t *it = std::lower_bound(b0, b1, col);
            return (it != b1 && *it == col) ? static_cast<int32_t>(it - ps->h_colIdx.data()) : -1;
        };
        for (int64_t f = 0; f < nF; ++f) {
            const int32_t o = own[f], n = nbr[f];
            int32_t w = fill[o]++;
            cfEnt[w] = static_cast<int32_t>(f);
            cfSlot[w] = n >= 0 ? slot_of(o, n) : (twin[f] >= 0 ? slot_of(o, own[twin[f]]) : -1);
            if (n >= 0) {
                w = fill[n]++;
                cfEnt[w] = static_cast<int32_t>(static_cast<uint32_t>(f) | 0x80000000u);
                cfSlot[w] = slot_of(n, o);
            }
        }
    }
    ps->nnz = static_cast<int64_t>(ps->h_colIdx.size());
    // ---- upload
    cudaStream_t st = ctx->stream;
    const size_t nEnt = cfEnt.size();
    auto up = [&](void *dst, const void *src, size_t bytes) {
        return cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, st);
    };
    int rc = SIMALL_OK;
#define PS_TRY(call)                                                                                                    \
    do {                                                                                                                \
        cudaError_t e_ = (call);                                                                                        \
        if (e_ != cudaSuccess) {                                                                                        \
            rc = cuda_fail(ctx, e_, #call, __FILE__, __LINE__);                                                         \
            goto fail_out;                                                                                              \
        }                                                                                                               \
    } while (0)
    {
        PS_TRY(ps->rowPtr.alloc(nC + 1));
        PS_TRY(ps->colIdx.alloc(ps->nnz));
        PS_TRY(ps->values.alloc(ps->nnz + 2));
        PS_TRY(ps->rhs.alloc(nC + 2));
        PS_TRY(ps->owner.alloc(nF));
        PS_TRY(ps->neighbor.alloc(nF));
        PS_TRY(ps->amag2.alloc(nF));
        PS_TRY(ps->ddotA.alloc(nF));
        PS_TRY(ps->kind.alloc(nF));
        PS_TRY(ps->coef.alloc(nF));
        PS_TRY(ps->cfOff.alloc(nC + 1));
        PS_TRY(ps->cfEnt.alloc(nEnt ? nEnt : 1));
        PS_TRY(ps->cfSlot.alloc(nEnt ? nEnt : 1));
        PS_TRY(ps->diagSlot.alloc(nC));
        PS_TRY(up(ps->rowPtr.p, ps->h_rowPtr.data(), (nC + 1) * sizeof(int32_t)));
        PS_TRY(up(ps->colIdx.p, ps->h_colIdx.data(), ps->nnz * sizeof(int32_t)));
        PS_TRY(up(ps->owner.p, own.data(), nF * sizeof(int32_t)));
        PS_TRY(up(ps->neighbor.p, nbr.data(), nF * sizeof(int32_t)));
        PS_TRY(up(ps->kind.p, kind.data(), nF));
        PS_TRY(up(ps->cfOff.p, cfOff.data(), (nC + 1) * sizeof(int32_t)));
        if (nEnt) {
            PS_TRY(up(ps->cfEnt.p, cfEnt.data(), nEnt * sizeof(int32_t)));
            PS_TRY(up(ps->cfSlot.p, cfSlot.data(), nEnt * sizeof(int32_t)));
        }
        PS_TRY(up(ps->diagSlot.p, diagSlot.data(), nC * sizeof(int32_t)));
        {
            std::vector<int32_t> partner(nbr);
            for (int64_t f = 0; f < nF; ++f)
                if (partner[f] < 0 && twin[f] >= 0)
                    partner[f] = own[twin[f]];
            PS_TRY(ps->fpartner.alloc(nF));
            PS_TRY(up(ps->fpartner.p, partner.data(), nF * sizeof(int32_t)));
            PS_TRY(cudaStreamSynchronize(st));  // partner dies at scope exit
        }
        // geometry (temporary device copies of the SoA arrays the kernel reads)
        DevBuf<double> g[9];
        const double *src[9] = {m->area_x,     m->area_y,     m->area_z,          m->centroid_x,     m->centroid_y,
                                m->centroid_z, m->cell_centroid_x, m->cell_centroid_y, m->cell_centroid_z};
        for (int i = 0; i < 9; ++i) {
            const int64_t cnt = i < 6 ? nF : nC;
            PS_TRY(g[i].alloc(cnt));
            PS_TRY(up(g[i].p, src[i], cnt * sizeof(double)));
        }
        const int64_t gg = std::min<int64_t>((nF + kBlock - 1) / kBlock, grid_size_streaming(ctx));
        k_face_geometry<<<static_cast<int>(gg), kBlock, 0, st>>>(nF, ps->owner.p, ps->neighbor.p, ps->kind.p, g[0].p,
                                                                 g[1].p, g[2].p, g[3].p, g[4].p, g[5].p, g[6].p, g[7].p,
                                                                 g[8].p, ps->amag2.p, ps->ddotA.p);
        ctx->launches.fetch_add(1, std::memory_order_relaxed);
        PS_TRY(cudaGetLastError());
        PS_TRY(cudaStreamSynchronize(st));  // host vectors and temporaries die at scope exit
    }
#undef PS_TRY
    *out = ps;
    return SIMALL_OK;
fail_out:
    delete ps;
    return rc;
}

int simall_pressure_system_destroy(simall_pressure_system *ps)
{
    if (!ps)
        return SIMALL_ERR_INVALID_ARGUMENT;
    cudaStreamSynchronize(ps->ctx->stream);
    delete ps;
    return SIMALL_OK;
}

int simall_pressure_system_pattern(const simall_pressure_system *ps, int64_t *n, int64_t *nnz, int32_t *rowPtr,
                                   int32_t *colIdx)
{
    if (!ps)
        return SIMALL_ERR_INVALID_ARGUMENT;
    if (n)
        *n = ps->nC;
    if (nnz)
        *nnz = ps->nnz;
    if (rowPtr)
        std::memcpy(rowPtr, ps->h_rowPtr.data(), (ps->nC + 1) * sizeof(int32_t));
    if (colIdx)
        std::memcpy(colIdx, ps->h_colIdx.data(), ps->nnz * sizeof(int32_t));
    return SIMALL_OK;
}

int simall_pressure_system_periodic_twins(const simall_pressure_system *ps, int32_t *twin)
{
    if (!ps || !twin)
        return SIMALL_ERR_INVALID_ARGUMENT;
    std::memcpy(twin, ps->h_twin.data(), ps->nF * sizeof(int32_t));
    return SIMALL_OK;
}

int simall_pressure_system_device_arrays(const simall_pressure_system *ps, const int32_t **rowPtr,
                                         const int32_t **colIdx, double **values, double **rhs)
{
    if (!ps)
        return SIMALL_ERR_INVALID_ARGUMENT;
    if (rowPtr)
        *rowPtr = ps->rowPtr.p;
    if (colIdx)
        *colIdx = ps->colIdx.p;
    if (values)
        *values = ps->values.p;
    if (rhs)
        *rhs = ps->rhs.p;
    return SIMALL_OK;
}

int simall_assemble_pressure_correction_simplec(simall_pressure_system *ps, double rho, const double *aP,
                                                const double *mom_values, const double *phi, int mem,
                                                int *any_dirichlet)
{
    if (!ps || !aP || !mom_values || !phi)
        return SIMALL_ERR_INVALID_ARGUMENT;
    simall_context *ctx = ps->ctx;
    if (mem != SIMALL_MEM_HOST && mem != SIMALL_MEM_DEVICE)
        return fail(ctx, SIMALL_ERR_INVALID_ARGUMENT, "assemble: bad memory kind %d", mem);
    SIMALL_CUDA_TRY(ctx, cudaSetDevice(ctx->device));
    cudaStream_t st = ctx->stream;
    const double *dA = aP, *dM = mom_values, *dPhi = phi;
    DevBuf<double> stageA, stageM, stageP;
    if (mem == SIMALL_MEM_HOST) {
        SIMALL_CUDA_TRY(ctx, stageA.alloc(ps->nC));
        SIMALL_CUDA_TRY(ctx, stageM.alloc(ps->nnz));
        SIMALL_CUDA_TRY(ctx, stageP.alloc(ps->nF));
        SIMALL_CUDA_TRY(ctx, cudaMemcpyAsync(stageA.p, aP, ps->nC * sizeof(double), cudaMemcpyHostToDevice, st));
        SIMALL_CUDA_TRY(ctx, cudaMemcpyAsync(stageM.p, mom_values, ps->nnz * sizeof(double), cudaMemcpyHostToDevice,
                                             st));
        SIMALL_CUDA_TRY(ctx, cudaMemcpyAsync(stageP.p, phi, ps->nF * sizeof(double), cudaMemcpyHostToDevice, st));
        dA = stageA.p;
        dM = stageM.p;
        dPhi = stageP.p;
    }
    SIMALL_CUDA_TRY(ctx, ps->den.alloc(ps->nC));
    const int gc = static_cast<int>(std::min<int64_t>((ps->nC + kBlock - 1) / kBlock, grid_size_streaming(ctx)));
    k_simplec_den<<<gc, kBlock, 0, st>>>(ps->nC, ps->rowPtr.p, ps->colIdx.p, dM, dA, ps->den.p);
    SIMALL_LAUNCH_CHECK(ctx);
    // max(den, 1e-30) is unchanged by the assembly's own max(., 1e-30)
    int r = simall_assemble_pressure_correction(ps, rho, ps->den.p, dPhi, SIMALL_MEM_DEVICE, any_dirichlet);
    if (mem == SIMALL_MEM_HOST)
        SIMALL_CUDA_TRY(ctx, cudaStreamSynchronize(st));  // the staging buffers die at return
    return r;
}

int simall_assemble_pressure_correction(simall_pressure_system *ps, double rho, const double *aP, const double *phi,
                                        int mem, int *any_dirichlet)
{
    if (!ps || !aP || !phi)
        return SIMALL_ERR_INVALID_ARGUMENT;
    simall_context *ctx = ps->ctx;
    if (mem != SIMALL_MEM_HOST && mem != SIMALL_MEM_DEVICE)
        return fail(ctx, SIMALL_ERR_INVALID_ARGUMENT, "assemble: bad memory kind %d", mem);
    SIMALL_CUDA_TRY(ctx, cudaSetDevice(ctx->device));
    cudaStream_t st = ctx->stream;
    const double *dA = aP, *dPhi = phi;
    if (mem == SIMALL_MEM_HOST) {
        SIMALL_CUDA_TRY(ctx, ps->aP.alloc(ps->nC));
        SIMALL_CUDA_TRY(ctx, ps->phi.alloc(ps->nF));
        SIMALL_CUDA_TRY(ctx, cudaMemcpyAsync(ps->aP.p, aP, ps->nC * sizeof(double), cudaMemcpyHostToDevice, st));
        SIMALL_CUDA_TRY(ctx, cudaMemcpyAsync(ps->phi.p, phi, ps->nF * sizeof(double), cudaMemcpyHostToDevice, st));
        dA = ps->aP.p;
        dPhi = ps->phi.p;
    }
    const int gf = static_cast<int>(std::min<int64_t>((ps->nF + kBlock - 1) / kBlock, grid_size_streaming(ctx)));
    const int gc = static_cast<int>(std::min<int64_t>((ps->nC + kBlock - 1) / kBlock, grid_size_streaming(ctx)));
    k_face_coef<<<gf, kBlock, 0, st>>>(ps->nF, rho, ps->owner.p, ps->neighbor.p, ps->kind.p, ps->amag2.p, ps->ddotA.p,
                                       dA, ps->coef.p);
    SIMALL_LAUNCH_CHECK(ctx);
    k_cell_rows<<<gc, kBlock, 0, st>>>(ps->nC, ps->rowPtr.p, ps->cfOff.p, ps->cfEnt.p, ps->cfSlot.p, ps->diagSlot.p,
                                       ps->kind.p, ps->coef.p, dPhi, ps->anyDirichlet, ps->values.p, ps->rhs.p);
    SIMALL_LAUNCH_CHECK(ctx);
    if (mem == SIMALL_MEM_HOST)
        SIMALL_CUDA_TRY(ctx, cudaStreamSynchronize(st));  // staging buffers are reused by the next call
    if (any_dirichlet)
        *any_dirichlet = ps->anyDirichlet;
    return SIMALL_OK;
}

int simall_pressure_system_download(const simall_pressure_system *ps, double *values, double *rhs)
{
    if (!ps)
        return SIMALL_ERR_INVALID_ARGUMENT;
    simall_context *ctx = ps->ctx;
    if (values)
        SIMALL_CUDA_TRY(ctx, cudaMemcpyAsync(values, ps->values.p, ps->nnz * sizeof(double), cudaMemcpyDeviceToHost,
                                             ctx->stream));
    if (rhs)
        SIMALL_CUDA_TRY(ctx,
                        cudaMemcpyAsync(rhs, ps->rhs.p, ps->nC * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    SIMALL_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
    return SIMALL_OK;
}

int simall_solver_use_pressure_system(simall_solver *s, simall_pressure_system *ps)
{
    if (!s || !ps)
        return SIMALL_ERR_INVALID_ARGUMENT;
    // set_matrix recognises an unchanged pattern on the device and keeps its
    // analysis (row-blocks, storage format, ILU0 levels, captured graphs)
    return simall_solver_set_matrix(s, ps->nC, ps->nnz, ps->rowPtr.p, ps->colIdx.p, ps->values.p, SIMALL_MEM_DEVICE);
}

int simall_assemble_face_conductance(simall_pressure_system *ps, double rho, const double *k, const double *pb,
                                     const double *src, int mem)
{
    if (!ps || !k || !pb || !src)
        return SIMALL_ERR_INVALID_ARGUMENT;
    simall_context *ctx = ps->ctx;
    if (mem != SIMALL_MEM_HOST && mem != SIMALL_MEM_DEVICE)
        return fail(ctx, SIMALL_ERR_INVALID_ARGUMENT, "assemble: bad memory kind %d", mem);
    if (ps->periodic)  // the face-conductance extension defines no periodic coupling
        return fail(ctx, SIMALL_ERR_UNSUPPORTED, "face-conductance assembly: the system has periodic faces");
    SIMALL_CUDA_TRY(ctx, cudaSetDevice(ctx->device));
    cudaStream_t st = ctx->stream;
    const double *dk = k, *dpb = pb, *dsrc = src;
    if (mem == SIMALL_MEM_HOST) {
        SIMALL_CUDA_TRY(ctx, ps->kf.alloc(ps->nF));
        SIMALL_CUDA_TRY(ctx, ps->pbf.alloc(ps->nF));
        SIMALL_CUDA_TRY(ctx, ps->aP.alloc(ps->nC));
        SIMALL_CUDA_TRY(ctx, cudaMemcpyAsync(ps->kf.p, k, ps->nF * sizeof(double), cudaMemcpyHostToDevice, st));
        SIMALL_CUDA_TRY(ctx, cudaMemcpyAsync(ps->pbf.p, pb, ps->nF * sizeof(double), cudaMemcpyHostToDevice, st));
        SIMALL_CUDA_TRY(ctx, cudaMemcpyAsync(ps->aP.p, src, ps->nC * sizeof(double), cudaMemcpyHostToDevice, st));
        dk = ps->kf.p;
        dpb = ps->pbf.p;
        dsrc = ps->aP.p;
    }
    const int gf = static_cast<int>(std::min<int64_t>((ps->nF + kBlock - 1) / kBlock, grid_size_streaming(ctx)));
    const int gc = static_cast<int>(std::min<int64_t>((ps->nC + kBlock - 1) / kBlock, grid_size_streaming(ctx)));
    k_face_coef_k<<<gf, kBlock, 0, st>>>(ps->nF, rho, ps->kind.p, ps->amag2.p, ps->ddotA.p, dk, ps->coef.p);
    SIMALL_LAUNCH_CHECK(ctx);
    k_cell_rows_k<<<gc, kBlock, 0, st>>>(ps->nC, ps->rowPtr.p, ps->cfOff.p, ps->cfEnt.p, ps->cfSlot.p, ps->diagSlot.p,
                                         ps->kind.p, ps->coef.p, dpb, dsrc, ps->values.p, ps->rhs.p);
    SIMALL_LAUNCH_CHECK(ctx);
    if (mem == SIMALL_MEM_HOST)
        SIMALL_CUDA_TRY(ctx, cudaStreamSynchronize(st));
    return SIMALL_OK;
}

int simall_face_conductance_gradient(simall_pressure_system *ps, double rho, const double *k, const double *pb,
                                     const double *x, const double *lambda, double *dk, double *dpb, int mem)
{
    if (!ps || !k || !pb || !x || !lambda || !dk || !dpb)
        return SIMALL_ERR_INVALID_ARGUMENT;
    simall_context *ctx = ps->ctx;
    if (mem != SIMALL_MEM_HOST && mem != SIMALL_MEM_DEVICE)
        return fail(ctx, SIMALL_ERR_INVALID_ARGUMENT, "gradient: bad memory kind %d", mem);
    if (ps->periodic)
        return fail(ctx, SIMALL_ERR_UNSUPPORTED, "face-conductance gradient: the system has periodic faces");
    SIMALL_CUDA_TRY(ctx, cudaSetDevice(ctx->device));
    cudaStream_t st = ctx->stream;
    const double *d_k = k, *d_pb = pb, *d_x = x, *d_l = lambda;
    double *d_dk = dk, *d_dpb = dpb;
    DevBuf<double> tk, tpb, tx, tl, tdk, tdpb;
    if (mem == SIMALL_MEM_HOST) {
        SIMALL_CUDA_TRY(ctx, tk.alloc(ps->nF));
        SIMALL_CUDA_TRY(ctx, tpb.alloc(ps->nF));
        SIMALL_CUDA_TRY(ctx, tx.alloc(ps->nC));
        SIMALL_CUDA_TRY(ctx, tl.alloc(ps->nC));
        SIMALL_CUDA_TRY(ctx, tdk.alloc(ps->nF));
        SIMALL_CUDA_TRY(ctx, tdpb.alloc(ps->nF));
        SIMALL_CUDA_TRY(ctx, cudaMemcpyAsync(tk.p, k, ps->nF * sizeof(double), cudaMemcpyHostToDevice, st));
        SIMALL_CUDA_TRY(ctx, cudaMemcpyAsync(tpb.p, pb, ps->nF * sizeof(double), cudaMemcpyHostToDevice, st));
        SIMALL_CUDA_TRY(ctx, cudaMemcpyAsync(tx.p, x, ps->nC * sizeof(double), cudaMemcpyHostToDevice, st));
        SIMALL_CUDA_TRY(ctx, cudaMemcpyAsync(tl.p, lambda, ps->nC * sizeof(double), cudaMemcpyHostToDevice, st));
        d_k = tk.p;
        d_pb = tpb.p;
        d_x = tx.p;
        d_l = tl.p;
        d_dk = tdk.p;
        d_dpb = tdpb.p;
    }
    const int gf = static_cast<int>(std::min<int64_t>((ps->nF + kBlock - 1) / kBlock, grid_size_streaming(ctx)));
    k_face_k_gradient<<<gf, kBlock, 0, st>>>(ps->nF, rho, ps->owner.p, ps->neighbor.p, ps->kind.p, ps->amag2.p,
                                             ps->ddotA.p, d_k, d_pb, d_x, d_l, d_dk, d_dpb);
    SIMALL_LAUNCH_CHECK(ctx);
    if (mem == SIMALL_MEM_HOST) {
        SIMALL_CUDA_TRY(ctx, cudaMemcpyAsync(dk, d_dk, ps->nF * sizeof(double), cudaMemcpyDeviceToHost, st));
        SIMALL_CUDA_TRY(ctx, cudaMemcpyAsync(dpb, d_dpb, ps->nF * sizeof(double), cudaMemcpyDeviceToHost, st));
        SIMALL_CUDA_TRY(ctx, cudaStreamSynchronize(st));
    }
    return SIMALL_OK;
}

int simall_adjoint_face_conductance(simall_pressure_system *ps, simall_solver *s, double rho, const double *k,
                                    const double *pb, const double *x, const double *dLdx, double *lambda,
                                    double *dk, double *dpb, int mem, simall_solver_stats *stats)
{
    if (!ps || !s || !k || !pb || !x || !dLdx || !lambda || !dk || !dpb)
        return SIMALL_ERR_INVALID_ARGUMENT;
    // the assembled operator is symmetric, so A^T lambda = dL/dx is solved
    // with the same PCG on the same device matrix
    int st = simall_solver_use_pressure_system(s, ps);
    if (st)
        return st;
    st = solver_solve_impl(s, dLdx, mem, lambda, mem, stats);
    if (st)
        return st;
    return simall_face_conductance_gradient(ps, rho, k, pb, x, lambda, dk, dpb, mem);
}

int simall_pressure_system_solve(simall_pressure_system *ps, simall_solver *s, double *x, int mem,
                                 simall_solver_stats *stats)
{
    if (!ps || !s || !x)
        return SIMALL_ERR_INVALID_ARGUMENT;
    int st = simall_solver_use_pressure_system(s, ps);
    if (st)
        return st;
    return solver_solve_impl(s, ps->rhs.p, SIMALL_MEM_DEVICE, x, mem, stats);
}

}  // extern "C"
