// The face loops either side of the pressure solve, on the device:
// compute_face_fluxes before the assembly (SimpleAlgorithm.cpp:201-237), and
// correct_fields after the solve (:450-487) with the least-squares gradient it
// calls (Gradient.cpp:17-133).  Each is bit-identical to the reference: every
// product, sum and quotient is rounded where the reference rounds it
// (__dmul_rn/__dadd_rn/... so nothing is contracted into a fused multiply-
// add), and every per-cell sum visits the cell's faces in ascending face id --
// the order of the reference's face loop -- through the per-cell face lists
// the assembly already keeps.  A cell's least-squares contribution from a face
// is the same whether the cell owns the face or neighbours it (the terms are
// even in the vector d), so gathering per cell reproduces the scattered sums.
#include "device.cuh"
#include "pressure_system.hpp"
#include "solver.hpp"

#include <algorithm>
#include <cmath>
#include <new>
#include <vector>

namespace simall {

namespace {

constexpr uint8_t kFaceInterior = 0, kFaceZoneVector = 1, kFaceZero = 2, kFaceOwner = 3;

// Per face: d = C_n - C_o (interior) or F_f - C_o (boundary), w2 = 1/(|d|^2 + 1e-30).
__global__ void __launch_bounds__(kBlock) k_lsq_face(int64_t nF, const int32_t *__restrict__ owner,
                                                     const int32_t *__restrict__ neighbor,
                                                     const double *__restrict__ fx, const double *__restrict__ fy,
                                                     const double *__restrict__ fz, const double *__restrict__ cx,
                                                     const double *__restrict__ cy, const double *__restrict__ cz,
                                                     double *gdx, double *gdy, double *gdz, double *gw2)
{
    for (int64_t f = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; f < nF; f += (int64_t)gridDim.x * blockDim.x) {
        const int o = owner[f], n = neighbor[f];
        double dx, dy, dz;
        if (n >= 0) {
            dx = __dsub_rn(cx[n], cx[o]);
            dy = __dsub_rn(cy[n], cy[o]);
            dz = __dsub_rn(cz[n], cz[o]);
        } else {
            dx = __dsub_rn(fx[f], cx[o]);
            dy = __dsub_rn(fy[f], cy[o]);
            dz = __dsub_rn(fz[f], cz[o]);
        }
        gdx[f] = dx;
        gdy[f] = dy;
        gdz[f] = dz;
        const double s = __dadd_rn(__dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz)), 1e-30);
        gw2[f] = __ddiv_rn(1.0, s);
    }
}

// Per cell: the weighted normal matrix over the cell's faces in ascending id,
// then invert3x3_sym (Gradient.cpp:17-33, 45-88).
__global__ void __launch_bounds__(kBlock) k_lsq_inverse(int64_t nC, const int32_t *__restrict__ cfOff,
                                                        const int32_t *__restrict__ cfEnt,
                                                        const double *__restrict__ gdx, const double *__restrict__ gdy,
                                                        const double *__restrict__ gdz, const double *__restrict__ gw2,
                                                        double *minv)
{
    for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < nC; c += (int64_t)gridDim.x * blockDim.x) {
        double xx = 0.0, xy = 0.0, xz = 0.0, yy = 0.0, yz = 0.0, zz = 0.0;
        for (int e = cfOff[c]; e < cfOff[c + 1]; ++e) {
            const int f = cfEnt[e] & 0x7fffffff;
            const double dx = gdx[f], dy = gdy[f], dz = gdz[f], w2 = gw2[f];
            const double wx = __dmul_rn(w2, dx), wy = __dmul_rn(w2, dy), wz = __dmul_rn(w2, dz);
            xx = __dadd_rn(xx, __dmul_rn(wx, dx));
            xy = __dadd_rn(xy, __dmul_rn(wx, dy));
            xz = __dadd_rn(xz, __dmul_rn(wx, dz));
            yy = __dadd_rn(yy, __dmul_rn(wy, dy));
            yz = __dadd_rn(yz, __dmul_rn(wy, dz));
            zz = __dadd_rn(zz, __dmul_rn(wz, dz));
        }
        const double c0 = __dsub_rn(__dmul_rn(yy, zz), __dmul_rn(yz, yz));
        const double c1 = __dsub_rn(__dmul_rn(xy, zz), __dmul_rn(yz, xz));
        const double c2 = __dsub_rn(__dmul_rn(xy, yz), __dmul_rn(yy, xz));
        const double det = __dadd_rn(__dsub_rn(__dmul_rn(xx, c0), __dmul_rn(xy, c1)), __dmul_rn(xz, c2));
        double out[6];
        if (fabs(det) < 1e-30) {
            for (int k = 0; k < 6; ++k)
                out[k] = 0.0;
        } else {
            const double inv = __ddiv_rn(1.0, det);
            out[0] = __dmul_rn(c0, inv);
            out[1] = __dmul_rn(-c1, inv);
            out[2] = __dmul_rn(c2, inv);
            out[3] = __dmul_rn(__dsub_rn(__dmul_rn(xx, zz), __dmul_rn(xz, xz)), inv);
            out[4] = __dmul_rn(-__dsub_rn(__dmul_rn(xx, yz), __dmul_rn(xy, xz)), inv);
            out[5] = __dmul_rn(__dsub_rn(__dmul_rn(xx, yy), __dmul_rn(xy, xy)), inv);
        }
        for (int k = 0; k < 6; ++k)
            minv[k * nC + c] = out[k];
    }
}

// LeastSquaresGradient::evaluate: per cell, sum over its faces in ascending id
// of w2 d dphi (owner side) or w2 d (-dphi) (neighbour side), dphi = phi_n - phi_o,
// zero on boundary faces; then grad = Minv b.
__global__ void __launch_bounds__(kBlock) k_lsq_gradient(int64_t nC, const int32_t *__restrict__ cfOff,
                                                         const int32_t *__restrict__ cfEnt,
                                                         const int32_t *__restrict__ owner,
                                                         const int32_t *__restrict__ neighbor,
                                                         const double *__restrict__ gdx, const double *__restrict__ gdy,
                                                         const double *__restrict__ gdz, const double *__restrict__ gw2,
                                                         const double *__restrict__ minv, const double *__restrict__ phi,
                                                         double *gx, double *gy, double *gz)
{
    for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < nC; c += (int64_t)gridDim.x * blockDim.x) {
        double bx = 0.0, by = 0.0, bz = 0.0;
        for (int e = cfOff[c]; e < cfOff[c + 1]; ++e) {
            const int ent = cfEnt[e];
            const int f = ent & 0x7fffffff;
            const int n = neighbor[f];
            double dphi = 0.0;
            if (n >= 0) {
                dphi = __dsub_rn(phi[n], phi[owner[f]]);
                if (ent < 0)  // this cell is the face's neighbour
                    dphi = -dphi;
            }
            const double w2 = gw2[f];
            bx = __dadd_rn(bx, __dmul_rn(__dmul_rn(w2, gdx[f]), dphi));
            by = __dadd_rn(by, __dmul_rn(__dmul_rn(w2, gdy[f]), dphi));
            bz = __dadd_rn(bz, __dmul_rn(__dmul_rn(w2, gdz[f]), dphi));
        }
        const double m0 = minv[c], m1 = minv[nC + c], m2 = minv[2 * nC + c];
        const double m3 = minv[3 * nC + c], m4 = minv[4 * nC + c], m5 = minv[5 * nC + c];
        gx[c] = __dadd_rn(__dadd_rn(__dmul_rn(m0, bx), __dmul_rn(m1, by)), __dmul_rn(m2, bz));
        gy[c] = __dadd_rn(__dadd_rn(__dmul_rn(m1, bx), __dmul_rn(m3, by)), __dmul_rn(m4, bz));
        gz[c] = __dadd_rn(__dadd_rn(__dmul_rn(m2, bx), __dmul_rn(m4, by)), __dmul_rn(m5, bz));
    }
}

// compute_face_fluxes: phi_f = rho (u . A) with the face velocity of the kind.
// partner: the neighbour of an interior face, the twin face's owner of a
// periodic one (both kFaceInterior), -1 elsewhere.
__global__ void __launch_bounds__(kBlock) k_face_fluxes(int64_t nF, double rho, const int32_t *__restrict__ owner,
                                                        const int32_t *__restrict__ partner,
                                                        const uint8_t *__restrict__ fkind,
                                                        const int32_t *__restrict__ fvslot,
                                                        const double *__restrict__ zvec, int nslots,
                                                        const double *__restrict__ ax, const double *__restrict__ ay,
                                                        const double *__restrict__ az, const double *__restrict__ Ux,
                                                        const double *__restrict__ Uy, const double *__restrict__ Uz,
                                                        double *phi)
{
    for (int64_t f = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; f < nF; f += (int64_t)gridDim.x * blockDim.x) {
        const int o = owner[f];
        double ux, uy, uz;
        switch (fkind[f]) {
        case kFaceInterior: {
            const int n = partner[f];
            ux = __dmul_rn(0.5, __dadd_rn(Ux[o], Ux[n]));
            uy = __dmul_rn(0.5, __dadd_rn(Uy[o], Uy[n]));
            uz = __dmul_rn(0.5, __dadd_rn(Uz[o], Uz[n]));
            break;
        }
        case kFaceZoneVector: {
            const int sl = fvslot[f];
            ux = zvec[sl];
            uy = zvec[nslots + sl];
            uz = zvec[2 * nslots + sl];
            break;
        }
        case kFaceZero:
            ux = uy = uz = 0.0;
            break;
        default:
            ux = Ux[o];
            uy = Uy[o];
            uz = Uz[o];
        }
        phi[f] = __dmul_rn(rho, __dadd_rn(__dadd_rn(__dmul_rn(ux, ax[f]), __dmul_rn(uy, ay[f])), __dmul_rn(uz, az[f])));
    }
}

// correct_fields, cells: p += urfP p', U -= V / max(aP, 1e-30) grad p'.
__global__ void __launch_bounds__(kBlock) k_correct_cells(int64_t nC, double urfP, const double *__restrict__ vol,
                                                          const double *__restrict__ aP,
                                                          const double *__restrict__ pp, const double *__restrict__ g,
                                                          double *p, double *Ux, double *Uy, double *Uz)
{
    for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < nC; c += (int64_t)gridDim.x * blockDim.x) {
        p[c] = __dadd_rn(p[c], __dmul_rn(urfP, pp[c]));
        const double w = __ddiv_rn(vol[c], std_max(aP[c], 1e-30));
        Ux[c] = __dsub_rn(Ux[c], __dmul_rn(w, g[c]));
        Uy[c] = __dsub_rn(Uy[c], __dmul_rn(w, g[nC + c]));
        Uz[c] = __dsub_rn(Uz[c], __dmul_rn(w, g[2 * nC + c]));
    }
}

// correct_fields, interior faces: phi += rho |A|^2 / max(0.5 (aP_o + aP_n) |d.A|, 1e-30) (p'_o - p'_n).
__global__ void __launch_bounds__(kBlock) k_correct_faces(int64_t nF, double rho, const int32_t *__restrict__ owner,
                                                          const int32_t *__restrict__ neighbor,
                                                          const double *__restrict__ amag2,
                                                          const double *__restrict__ ddotA,
                                                          const double *__restrict__ aP,
                                                          const double *__restrict__ pp, double *phi)
{
    for (int64_t f = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; f < nF; f += (int64_t)gridDim.x * blockDim.x) {
        const int n = neighbor[f];
        if (n < 0)
            continue;
        const int o = owner[f];
        const double aPf = __dmul_rn(0.5, __dadd_rn(aP[o], aP[n]));
        const double coef = __ddiv_rn(__dmul_rn(rho, amag2[f]), std_max(__dmul_rn(aPf, ddotA[f]), 1e-30));
        phi[f] = __dadd_rn(phi[f], __dmul_rn(coef, __dsub_rn(pp[o], pp[n])));
    }
}

int grid_for_ps(simall_context *ctx, int64_t n)
{
    const int64_t g = (n + kBlock - 1) / kBlock;
    const int64_t cap = grid_size_streaming(ctx);
    return static_cast<int>(g < 1 ? 1 : (g < cap ? g : cap));
}

bool bad_mem(int mem) { return mem != SIMALL_MEM_HOST && mem != SIMALL_MEM_DEVICE; }

}  // namespace

int ps_gradient(simall_pressure_system *ps, const double *f, double *g)
{
    simall_context *ctx = ps->ctx;
    const int64_t nC = ps->nC;
    k_lsq_gradient<<<grid_for_ps(ctx, nC), kBlock, 0, ctx->stream>>>(nC, ps->cfOff.p, ps->cfEnt.p, ps->owner.p,
                                                                     ps->neighbor.p, ps->gdx.p, ps->gdy.p, ps->gdz.p,
                                                                     ps->gw2.p, ps->minv.p, f, g, g + nC, g + 2 * nC);
    SIMALL_LAUNCH_CHECK(ctx);
    return SIMALL_OK;
}

}  // namespace simall

using namespace simall;

extern "C" {

int simall_pressure_system_setup_field_loops(simall_pressure_system *ps, const simall_mesh_view *m,
                                             const double *cell_volume, const simall_zone_velocity *velocities,
                                             int n_velocities)
{
    if (!ps || !m || !cell_volume || (n_velocities > 0 && !velocities) || n_velocities < 0)
        return SIMALL_ERR_INVALID_ARGUMENT;
    simall_context *ctx = ps->ctx;
    if (m->n_cells != ps->nC || m->n_faces != ps->nF)
        return fail(ctx, SIMALL_ERR_SIZE_MISMATCH, "field loops: mesh view does not match the system");
    if (!m->area_x || !m->area_y || !m->area_z || !m->centroid_x || !m->centroid_y || !m->centroid_z ||
        !m->boundary_zone || !m->cell_centroid_x || !m->cell_centroid_y || !m->cell_centroid_z)
        return fail(ctx, SIMALL_ERR_INVALID_ARGUMENT, "mesh view has a null array");
    SIMALL_CUDA_TRY(ctx, cudaSetDevice(ctx->device));
    const int64_t nC = ps->nC, nF = ps->nF;
    // face velocity kinds (compute_face_fluxes, SimpleAlgorithm.cpp:208-234):
    // VelocityInlet / MovingWall -> the zone's vector; NoSlipWall / Wall /
    // Symmetry -> zero; any other spec, or none -> the owner's velocity
    std::vector<uint8_t> fk(static_cast<size_t>(nF));
    // momentum boundary kinds (assemble_momentum, SimpleAlgorithm.cpp:278-318)
    std::vector<uint8_t> mk(static_cast<size_t>(nF), kMomInterior);
    std::vector<int32_t> slot(static_cast<size_t>(nF), -1);
    std::vector<double> vx, vy, vz;
    std::vector<std::pair<uint32_t, int32_t>> zoneSlot;  // zone -> slot
    for (int64_t f = 0; f < nF; ++f) {
        if (m->neighbor[f] != ~0ull) {
            fk[f] = kFaceInterior;
            continue;
        }
        if (ps->h_twin[f] >= 0) {  // periodic: averaged with the twin face's owner (:214-219, :275-282)
            fk[f] = kFaceInterior;
            mk[f] = kMomPeriodic;
            continue;
        }
        const uint32_t z = m->boundary_zone[f];
        int type = -1;
        for (const auto &b : ps->h_bcs)
            if (b.zone == z) {
                type = b.type;
                break;
            }
        mk[f] = (type == SIMALL_BC_VELOCITY_INLET || type == SIMALL_BC_MOVING_WALL) ? kMomZoneVector
                : (type == SIMALL_BC_NO_SLIP_WALL || type == SIMALL_BC_WALL)       ? kMomWall
                : (type == SIMALL_BC_SYMMETRY)                                     ? kMomSymmetry
                                                                                   : kMomOther;
        if (type == SIMALL_BC_VELOCITY_INLET || type == SIMALL_BC_MOVING_WALL) {
            fk[f] = kFaceZoneVector;
            int32_t sl = -1;
            for (const auto &zs : zoneSlot)
                if (zs.first == z)
                    sl = zs.second;
            if (sl < 0) {
                double u[3] = {0.0, 0.0, 0.0};
                for (int i = 0; i < n_velocities; ++i)
                    if (velocities[i].zone == z) {
                        u[0] = velocities[i].u[0];
                        u[1] = velocities[i].u[1];
                        u[2] = velocities[i].u[2];
                        break;
                    }
                sl = static_cast<int32_t>(vx.size());
                vx.push_back(u[0]);
                vy.push_back(u[1]);
                vz.push_back(u[2]);
                zoneSlot.emplace_back(z, sl);
            }
            slot[f] = sl;
        } else if (type == SIMALL_BC_NO_SLIP_WALL || type == SIMALL_BC_WALL || type == SIMALL_BC_SYMMETRY) {
            fk[f] = kFaceZero;
        } else {
            fk[f] = kFaceOwner;
        }
    }
    const int nslots = static_cast<int>(vx.size());
    std::vector<double> zv(static_cast<size_t>(3 * std::max(nslots, 1)), 0.0);
    for (int i = 0; i < nslots; ++i) {
        zv[i] = vx[i];
        zv[nslots + i] = vy[i];
        zv[2 * nslots + i] = vz[i];
    }
    cudaStream_t st = ctx->stream;
    auto up = [&](void *dst, const void *src, size_t bytes) {
        return cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, st);
    };
    SIMALL_CUDA_TRY(ctx, ps->ax.alloc(nF));
    SIMALL_CUDA_TRY(ctx, ps->ay.alloc(nF));
    SIMALL_CUDA_TRY(ctx, ps->az.alloc(nF));
    SIMALL_CUDA_TRY(ctx, ps->gdx.alloc(nF));
    SIMALL_CUDA_TRY(ctx, ps->gdy.alloc(nF));
    SIMALL_CUDA_TRY(ctx, ps->gdz.alloc(nF));
    SIMALL_CUDA_TRY(ctx, ps->gw2.alloc(nF));
    SIMALL_CUDA_TRY(ctx, ps->minv.alloc(6 * nC));
    SIMALL_CUDA_TRY(ctx, ps->vol.alloc(nC));
    SIMALL_CUDA_TRY(ctx, ps->fkind.alloc(nF));
    SIMALL_CUDA_TRY(ctx, ps->mkind.alloc(nF));
    SIMALL_CUDA_TRY(ctx, ps->fvslot.alloc(nF));
    SIMALL_CUDA_TRY(ctx, ps->zvec.alloc(zv.size()));
    SIMALL_CUDA_TRY(ctx, ps->grad.alloc(3 * nC));
    SIMALL_CUDA_TRY(ctx, up(ps->ax.p, m->area_x, nF * sizeof(double)));
    SIMALL_CUDA_TRY(ctx, up(ps->ay.p, m->area_y, nF * sizeof(double)));
    SIMALL_CUDA_TRY(ctx, up(ps->az.p, m->area_z, nF * sizeof(double)));
    SIMALL_CUDA_TRY(ctx, up(ps->vol.p, cell_volume, nC * sizeof(double)));
    SIMALL_CUDA_TRY(ctx, up(ps->fkind.p, fk.data(), nF));
    SIMALL_CUDA_TRY(ctx, up(ps->mkind.p, mk.data(), nF));
    ps->momMu = std::nan("");  // the momentum face diffusion is recomputed at the next assembly
    SIMALL_CUDA_TRY(ctx, up(ps->fvslot.p, slot.data(), nF * sizeof(int32_t)));
    SIMALL_CUDA_TRY(ctx, up(ps->zvec.p, zv.data(), zv.size() * sizeof(double)));
    {
        DevBuf<double> g[6];
        const double *src[6] = {m->centroid_x, m->centroid_y, m->centroid_z,
                                m->cell_centroid_x, m->cell_centroid_y, m->cell_centroid_z};
        for (int i = 0; i < 6; ++i) {
            const int64_t cnt = i < 3 ? nF : nC;
            SIMALL_CUDA_TRY(ctx, g[i].alloc(cnt));
            SIMALL_CUDA_TRY(ctx, up(g[i].p, src[i], cnt * sizeof(double)));
        }
        k_lsq_face<<<grid_for_ps(ctx, nF), kBlock, 0, st>>>(nF, ps->owner.p, ps->neighbor.p, g[0].p, g[1].p, g[2].p,
                                                            g[3].p, g[4].p, g[5].p, ps->gdx.p, ps->gdy.p, ps->gdz.p,
                                                            ps->gw2.p);
        SIMALL_LAUNCH_CHECK(ctx);
        k_lsq_inverse<<<grid_for_ps(ctx, nC), kBlock, 0, st>>>(nC, ps->cfOff.p, ps->cfEnt.p, ps->gdx.p, ps->gdy.p,
                                                               ps->gdz.p, ps->gw2.p, ps->minv.p);
        SIMALL_LAUNCH_CHECK(ctx);
        SIMALL_CUDA_TRY(ctx, cudaStreamSynchronize(st));  // host tables and temporaries die here
    }
    ps->nslots = nslots;
    ps->fieldsReady = true;
    return SIMALL_OK;
}

int simall_compute_face_fluxes(simall_pressure_system *ps, double rho, const double *Ux, const double *Uy,
                               const double *Uz, double *phi, int mem)
{
    if (!ps || !Ux || !Uy || !Uz || !phi)
        return SIMALL_ERR_INVALID_ARGUMENT;
    simall_context *ctx = ps->ctx;
    if (bad_mem(mem))
        return fail(ctx, SIMALL_ERR_INVALID_ARGUMENT, "bad memory kind %d", mem);
    if (!ps->fieldsReady)
        return fail(ctx, SIMALL_ERR_INVALID_ARGUMENT, "face fluxes: call simall_pressure_system_setup_field_loops first");
    SIMALL_CUDA_TRY(ctx, cudaSetDevice(ctx->device));
    cudaStream_t st = ctx->stream;
    const int64_t nC = ps->nC, nF = ps->nF;
    const double *u[3] = {Ux, Uy, Uz};
    double *out = phi;
    if (mem == SIMALL_MEM_HOST) {
        SIMALL_CUDA_TRY(ctx, ps->stage.alloc(3 * nC + nF));
        for (int k = 0; k < 3; ++k) {
            SIMALL_CUDA_TRY(ctx, cudaMemcpyAsync(ps->stage.p + k * nC, u[k], nC * sizeof(double),
                                                 cudaMemcpyHostToDevice, st));
            u[k] = ps->stage.p + k * nC;
        }
        out = ps->stage.p + 3 * nC;
    }
    k_face_fluxes<<<grid_for_ps(ctx, nF), kBlock, 0, st>>>(nF, rho, ps->owner.p, ps->fpartner.p, ps->fkind.p,
                                                           ps->fvslot.p, ps->zvec.p, ps->nslots, ps->ax.p, ps->ay.p,
                                                           ps->az.p, u[0], u[1], u[2], out);
    SIMALL_LAUNCH_CHECK(ctx);
    if (mem == SIMALL_MEM_HOST) {
        SIMALL_CUDA_TRY(ctx, cudaMemcpyAsync(phi, out, nF * sizeof(double), cudaMemcpyDeviceToHost, st));
        SIMALL_CUDA_TRY(ctx, cudaStreamSynchronize(st));
    }
    return SIMALL_OK;
}

int simall_lsq_gradient(simall_pressure_system *ps, const double *f, double *gx, double *gy, double *gz, int mem)
{
    if (!ps || !f || !gx || !gy || !gz)
        return SIMALL_ERR_INVALID_ARGUMENT;
    simall_context *ctx = ps->ctx;
    if (bad_mem(mem))
        return fail(ctx, SIMALL_ERR_INVALID_ARGUMENT, "bad memory kind %d", mem);
    if (!ps->fieldsReady)
        return fail(ctx, SIMALL_ERR_INVALID_ARGUMENT, "gradient: call simall_pressure_system_setup_field_loops first");
    SIMALL_CUDA_TRY(ctx, cudaSetDevice(ctx->device));
    cudaStream_t st = ctx->stream;
    const int64_t nC = ps->nC;
    const double *in = f;
    if (mem == SIMALL_MEM_HOST) {
        SIMALL_CUDA_TRY(ctx, ps->stage.alloc(nC));
        SIMALL_CUDA_TRY(ctx, cudaMemcpyAsync(ps->stage.p, f, nC * sizeof(double), cudaMemcpyHostToDevice, st));
        in = ps->stage.p;
    }
    double *g[3] = {gx, gy, gz};
    if (mem == SIMALL_MEM_HOST)
        for (int k = 0; k < 3; ++k)
            g[k] = ps->grad.p + k * nC;
    k_lsq_gradient<<<grid_for_ps(ctx, nC), kBlock, 0, st>>>(nC, ps->cfOff.p, ps->cfEnt.p, ps->owner.p,
                                                            ps->neighbor.p, ps->gdx.p, ps->gdy.p, ps->gdz.p, ps->gw2.p,
                                                            ps->minv.p, in, g[0], g[1], g[2]);
    SIMALL_LAUNCH_CHECK(ctx);
    if (mem == SIMALL_MEM_HOST) {
        double *h[3] = {gx, gy, gz};
        for (int k = 0; k < 3; ++k)
            SIMALL_CUDA_TRY(ctx, cudaMemcpyAsync(h[k], g[k], nC * sizeof(double), cudaMemcpyDeviceToHost, st));
        SIMALL_CUDA_TRY(ctx, cudaStreamSynchronize(st));
    }
    return SIMALL_OK;
}

int simall_correct_fields(simall_pressure_system *ps, double rho, double urfP, const double *aP, const double *pPrime,
                          double *p, double *Ux, double *Uy, double *Uz, double *phi, int mem)
{
    if (!ps || !aP || !pPrime || !p || !Ux || !Uy || !Uz || !phi)
        return SIMALL_ERR_INVALID_ARGUMENT;
    simall_context *ctx = ps->ctx;
    if (bad_mem(mem))
        return fail(ctx, SIMALL_ERR_INVALID_ARGUMENT, "bad memory kind %d", mem);
    if (!ps->fieldsReady)
        return fail(ctx, SIMALL_ERR_INVALID_ARGUMENT, "correction: call simall_pressure_system_setup_field_loops first");
    SIMALL_CUDA_TRY(ctx, cudaSetDevice(ctx->device));
    cudaStream_t st = ctx->stream;
    const int64_t nC = ps->nC, nF = ps->nF;
    // device views of the seven arrays: aP, p', p, Ux, Uy, Uz (cells), phi (faces)
    const double *dA = aP, *dPP = pPrime;
    double *d[5] = {p, Ux, Uy, Uz, phi};
    double *h[5] = {p, Ux, Uy, Uz, phi};
    const int64_t len[5] = {nC, nC, nC, nC, nF};
    if (mem == SIMALL_MEM_HOST) {
        SIMALL_CUDA_TRY(ctx, ps->stage.alloc(6 * nC + nF));
        double *b = ps->stage.p;
        SIMALL_CUDA_TRY(ctx, cudaMemcpyAsync(b, aP, nC * sizeof(double), cudaMemcpyHostToDevice, st));
        SIMALL_CUDA_TRY(ctx, cudaMemcpyAsync(b + nC, pPrime, nC * sizeof(double), cudaMemcpyHostToDevice, st));
        dA = b;
        dPP = b + nC;
        int64_t off = 2 * nC;
        for (int k = 0; k < 5; ++k) {
            SIMALL_CUDA_TRY(ctx, cudaMemcpyAsync(b + off, h[k], len[k] * sizeof(double), cudaMemcpyHostToDevice, st));
            d[k] = b + off;
            off += len[k];
        }
    }
    k_lsq_gradient<<<grid_for_ps(ctx, nC), kBlock, 0, st>>>(nC, ps->cfOff.p, ps->cfEnt.p, ps->owner.p,
                                                            ps->neighbor.p, ps->gdx.p, ps->gdy.p, ps->gdz.p, ps->gw2.p,
                                                            ps->minv.p, dPP, ps->grad.p, ps->grad.p + nC,
                                                            ps->grad.p + 2 * nC);
    SIMALL_LAUNCH_CHECK(ctx);
    k_correct_cells<<<grid_for_ps(ctx, nC), kBlock, 0, st>>>(nC, urfP, ps->vol.p, dA, dPP, ps->grad.p, d[0], d[1],
                                                             d[2], d[3]);
    SIMALL_LAUNCH_CHECK(ctx);
    k_correct_faces<<<grid_for_ps(ctx, nF), kBlock, 0, st>>>(nF, rho, ps->owner.p, ps->neighbor.p, ps->amag2.p,
                                                             ps->ddotA.p, dA, dPP, d[4]);
    SIMALL_LAUNCH_CHECK(ctx);
    if (mem == SIMALL_MEM_HOST) {
        for (int k = 0; k < 5; ++k)
            SIMALL_CUDA_TRY(ctx, cudaMemcpyAsync(h[k], d[k], len[k] * sizeof(double), cudaMemcpyDeviceToHost, st));
        SIMALL_CUDA_TRY(ctx, cudaStreamSynchronize(st));
    }
    return SIMALL_OK;
}

}  // extern "C"
