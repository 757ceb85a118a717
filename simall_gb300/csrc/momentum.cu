// Momentum assembly on the device: the GB300 replacement of
// SimpleAlgorithm::assemble_momentum (src/solver/SimpleAlgorithm.cpp:240-355),
// first-order upwind, periodic faces included.
//
// The reference assembles each velocity component separately, but the matrix
// it builds does not depend on the component (convection, diffusion,
// transient and relaxation terms are the same for U.x, U.y and U.z); only the
// right-hand side does.  Here one pass builds the matrix once and all three
// right-hand sides:
//   k_mom_diffusion  per face, once per viscosity: D_f = mu |A|^2 / max(|d.A|, 1e-30)
//                    with d from owner centroid to neighbour (or face) centroid;
//   k_mom_rows       one thread per cell: zeroes its CSR row, then walks its
//                    faces in ascending id -- the order of the reference's
//                    face loop -- adding the upwind/diffusion coefficients
//                    (ConvO = max(F, 0), ConvN = max(-F, 0)) to its diagonal
//                    and off-diagonal slots and the boundary terms to its
//                    three rhs entries; then the pressure-gradient source,
//                    the transient term and Patankar under-relaxation.
// Every operation is rounded where the reference rounds it, so values, rhs and
// the relaxed diagonal aP are bit-identical to the reference's.
#include "device.cuh"
#include "pressure_system.hpp"
#include "solver.hpp"

#include <algorithm>
#include <cmath>

namespace simall {

namespace {

// D_f (SimpleAlgorithm.cpp:263-272, :282-288): d.A in the reference's order.
__global__ void __launch_bounds__(kBlock) k_mom_diffusion(int64_t nF, double mu, const double *__restrict__ amag2,
                                                          const double *__restrict__ ax, const double *__restrict__ ay,
                                                          const double *__restrict__ az, const double *__restrict__ dx,
                                                          const double *__restrict__ dy, const double *__restrict__ dz,
                                                          double *__restrict__ D)
{
    for (int64_t f = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; f < nF; f += (int64_t)gridDim.x * blockDim.x) {
        const double dA =
            fabs(__dadd_rn(__dadd_rn(__dmul_rn(dx[f], ax[f]), __dmul_rn(dy[f], ay[f])), __dmul_rn(dz[f], az[f])));
        D[f] = __ddiv_rn(__dmul_rn(mu, amag2[f]), std_max(dA, 1e-30));
    }
}

struct MomArgs {
    int64_t nC;
    const int32_t *rowPtr, *cfOff, *cfEnt, *cfSlot, *diagSlot;
    const uint8_t *mkind;
    const int32_t *vslot;
    const double *zvec;
    int nslots;
    const double *phi, *D, *grad, *vol, *U, *Un, *Unm1;
    double rho, dt, urfU;
    int transient, bdf2;
    double *values, *rhs, *aP;
};

__global__ void __launch_bounds__(kBlock) k_mom_rows(const MomArgs a)
{
    const int64_t nC = a.nC;
    for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < nC; c += (int64_t)gridDim.x * blockDim.x) {
        const int r0 = a.rowPtr[c], r1 = a.rowPtr[c + 1];
        for (int k = r0; k < r1; ++k)
            a.values[k] = 0.0;
        const int kd = a.diagSlot[c];
        double diag = 0.0, b0 = 0.0, b1 = 0.0, b2 = 0.0;
        for (int e = a.cfOff[c]; e < a.cfOff[c + 1]; ++e) {
            const int ent = a.cfEnt[e];
            const int f = ent & 0x7fffffff;
            const bool isNbr = ent < 0;
            const double F = __ldg(a.phi + f);
            const double convO = std_max(F, 0.0), convN = std_max(-F, 0.0);
            const double D = __ldg(a.D + f);
            const uint8_t k = a.mkind[f];
            if (k == kMomInterior) {
                // owner row: oo += ConvO + D, on -= ConvN + D; neighbour row: nn += ConvN + D, no -= ConvO + D
                const double self = isNbr ? __dadd_rn(convN, D) : __dadd_rn(convO, D);
                const double other = isNbr ? __dadd_rn(convO, D) : __dadd_rn(convN, D);
                diag = __dadd_rn(diag, self);
                const int slot = a.cfSlot[e];
                if (slot >= 0)
                    a.values[slot] = __dadd_rn(a.values[slot], -other);
            } else if (k == kMomZoneVector || k == kMomWall) {
                diag = __dadd_rn(diag, __dadd_rn(convO, D));
                const double w = __dadd_rn(convN, D);
                double u0 = 0.0, u1 = 0.0, u2 = 0.0;
                if (k == kMomZoneVector) {
                    const int s = a.vslot[f];
                    u0 = a.zvec[s];
                    u1 = a.zvec[a.nslots + s];
                    u2 = a.zvec[2 * a.nslots + s];
                }
                b0 = __dadd_rn(b0, __dmul_rn(w, u0));
                b1 = __dadd_rn(b1, __dmul_rn(w, u1));
                b2 = __dadd_rn(b2, __dmul_rn(w, u2));
            } else if (k == kMomPeriodic) {
                // half an interior face (:275-282): oo += ConvO + D, o,twin -= ConvN + D
                // (the twin face's owner is this cell on a mesh one cell wide
                // across the pair: then the diagonal, in the same order)
                diag = __dadd_rn(diag, __dadd_rn(convO, D));
                const double other = __dadd_rn(convN, D);
                const int slot = a.cfSlot[e];
                if (slot == kd)
                    diag = __dadd_rn(diag, -other);
                else if (slot >= 0)
                    a.values[slot] = __dadd_rn(a.values[slot], -other);
            } else if (k == kMomOther) {
                diag = __dadd_rn(diag, convO);
            }
        }
        // pressure-gradient source (:321-330)
        const double v = a.vol[c];
        b0 = __dsub_rn(b0, __dmul_rn(a.grad[c], v));
        b1 = __dsub_rn(b1, __dmul_rn(a.grad[nC + c], v));
        b2 = __dsub_rn(b2, __dmul_rn(a.grad[2 * nC + c], v));
        double bb[3] = {b0, b1, b2};
        // transient term (:332-352)
        if (a.transient) {
            const double vrdt = __ddiv_rn(__dmul_rn(a.rho, v), a.dt);
            if (a.bdf2) {
                diag = __dadd_rn(diag, __dmul_rn(1.5, vrdt));
#pragma unroll
                for (int q = 0; q < 3; ++q) {
                    const double h = __dsub_rn(__dmul_rn(2.0, a.Un[q * nC + c]), __dmul_rn(0.5, a.Unm1[q * nC + c]));
                    bb[q] = __dadd_rn(bb[q], __dmul_rn(h, vrdt));
                }
            } else {
                diag = __dadd_rn(diag, vrdt);
#pragma unroll
                for (int q = 0; q < 3; ++q)
                    bb[q] = __dadd_rn(bb[q], __dmul_rn(a.Un[q * nC + c], vrdt));
            }
        }
        // Patankar under-relaxation (:355-364)
        const double scaled = __ddiv_rn(diag, a.urfU);
        const double dd = __dsub_rn(scaled, diag);
#pragma unroll
        for (int q = 0; q < 3; ++q)
            a.rhs[q * nC + c] = __dadd_rn(bb[q], __dmul_rn(dd, a.U[q * nC + c]));
        a.values[kd] = scaled;
        a.aP[c] = scaled;
    }
}

int grid_cells(simall_context *ctx, int64_t n)
{
    const int64_t g = (n + kBlock - 1) / kBlock;
    const int64_t cap = grid_size_streaming(ctx);
    return static_cast<int>(g < 1 ? 1 : (g < cap ? g : cap));
}

}  // namespace

}  // namespace simall

using namespace simall;

extern "C" {

int simall_assemble_momentum(simall_pressure_system *ps, const simall_momentum_options *opt, const double *U,
                             const double *p, const double *phi, const double *Un, const double *Unm1, int mem)
{
    if (!ps || !opt || !U || !p || !phi)
        return SIMALL_ERR_INVALID_ARGUMENT;
    simall_context *ctx = ps->ctx;
    if (mem != SIMALL_MEM_HOST && mem != SIMALL_MEM_DEVICE)
        return fail(ctx, SIMALL_ERR_INVALID_ARGUMENT, "momentum: bad memory kind %d", mem);
    if (!ps->fieldsReady)
        return fail(ctx, SIMALL_ERR_INVALID_ARGUMENT, "momentum: call simall_pressure_system_setup_field_loops first");
    const bool transient = opt->dt > 0.0;
    if (transient && (!Un || (opt->bdf2 && !Unm1)))
        return fail(ctx, SIMALL_ERR_INVALID_ARGUMENT, "momentum: dt > 0 needs Un (and Unm1 for BDF2)");
    if (!(opt->urfU != 0.0))
        return fail(ctx, SIMALL_ERR_INVALID_ARGUMENT, "momentum: urfU must be non-zero");
    SIMALL_CUDA_TRY(ctx, cudaSetDevice(ctx->device));
    cudaStream_t st = ctx->stream;
    const int64_t nC = ps->nC, nF = ps->nF;
    const double *dU = U, *dP = p, *dPhi = phi, *dUn = Un, *dUnm1 = Unm1;
    if (mem == SIMALL_MEM_HOST) {
        SIMALL_CUDA_TRY(ctx, ps->stage.alloc(10 * nC + nF));
        double *b = ps->stage.p;
        auto up = [&](double *dst, const double *src, int64_t cnt) {
            return cudaMemcpyAsync(dst, src, cnt * sizeof(double), cudaMemcpyHostToDevice, st);
        };
        SIMALL_CUDA_TRY(ctx, up(b, U, 3 * nC));
        SIMALL_CUDA_TRY(ctx, up(b + 3 * nC, p, nC));
        SIMALL_CUDA_TRY(ctx, up(b + 4 * nC, phi, nF));
        dU = b;
        dP = b + 3 * nC;
        dPhi = b + 4 * nC;
        if (transient) {
            SIMALL_CUDA_TRY(ctx, up(b + 4 * nC + nF, Un, 3 * nC));
            dUn = b + 4 * nC + nF;
            if (opt->bdf2) {
                SIMALL_CUDA_TRY(ctx, up(b + 7 * nC + nF, Unm1, 3 * nC));
                dUnm1 = b + 7 * nC + nF;
            }
        }
    }
    if (!(ps->momMu == opt->mu) || !ps->momD.p) {
        SIMALL_CUDA_TRY(ctx, ps->momD.alloc(nF));
        k_mom_diffusion<<<grid_cells(ctx, nF), kBlock, 0, st>>>(nF, opt->mu, ps->amag2.p, ps->ax.p, ps->ay.p,
                                                                 ps->az.p, ps->gdx.p, ps->gdy.p, ps->gdz.p,
                                                                 ps->momD.p);
        SIMALL_LAUNCH_CHECK(ctx);
        ps->momMu = opt->mu;
    }
    SIMALL_CUDA_TRY(ctx, ps->mvalues.alloc(ps->nnz));
    SIMALL_CUDA_TRY(ctx, ps->mrhs.alloc(3 * nC));
    SIMALL_CUDA_TRY(ctx, ps->maP.alloc(nC));
    int e = ps_gradient(ps, dP, ps->grad.p);
    if (e)
        return e;
    MomArgs a;
    a.nC = nC;
    a.rowPtr = ps->rowPtr.p;
    a.cfOff = ps->cfOff.p;
    a.cfEnt = ps->cfEnt.p;
    a.cfSlot = ps->cfSlot.p;
    a.diagSlot = ps->diagSlot.p;
    a.mkind = ps->mkind.p;
    a.vslot = ps->fvslot.p;
    a.zvec = ps->zvec.p;
    a.nslots = ps->nslots;
    a.phi = dPhi;
    a.D = ps->momD.p;
    a.grad = ps->grad.p;
    a.vol = ps->vol.p;
    a.U = dU;
    a.Un = transient ? dUn : dU;
    a.Unm1 = (transient && opt->bdf2) ? dUnm1 : dU;
    a.rho = opt->rho;
    a.dt = opt->dt;
    a.urfU = opt->urfU;
    a.transient = transient ? 1 : 0;
    a.bdf2 = opt->bdf2 ? 1 : 0;
    a.values = ps->mvalues.p;
    a.rhs = ps->mrhs.p;
    a.aP = ps->maP.p;
    k_mom_rows<<<grid_cells(ctx, nC), kBlock, 0, st>>>(a);
    SIMALL_LAUNCH_CHECK(ctx);
    ps->momReady = true;
    if (mem == SIMALL_MEM_HOST)
        SIMALL_CUDA_TRY(ctx, cudaStreamSynchronize(st));  // the staging buffer is reused by the next call
    return SIMALL_OK;
}

int simall_momentum_device_arrays(const simall_pressure_system *ps, const double **values, const double **rhs,
                                  const double **aP)
{
    if (!ps)
        return SIMALL_ERR_INVALID_ARGUMENT;
    if (!ps->momReady)
        return fail(ps->ctx, SIMALL_ERR_INVALID_ARGUMENT, "no momentum system assembled yet");
    if (values)
        *values = ps->mvalues.p;
    if (rhs)
        *rhs = ps->mrhs.p;
    if (aP)
        *aP = ps->maP.p;
    return SIMALL_OK;
}

int simall_momentum_download(const simall_pressure_system *ps, double *values, double *rhs, double *aP)
{
    if (!ps)
        return SIMALL_ERR_INVALID_ARGUMENT;
    simall_context *ctx = ps->ctx;
    if (!ps->momReady)
        return fail(ctx, SIMALL_ERR_INVALID_ARGUMENT, "no momentum system assembled yet");
    SIMALL_CUDA_TRY(ctx, cudaSetDevice(ctx->device));
    cudaStream_t st = ctx->stream;
    if (values)
        SIMALL_CUDA_TRY(ctx, cudaMemcpyAsync(values, ps->mvalues.p, ps->nnz * sizeof(double), cudaMemcpyDeviceToHost,
                                             st));
    if (rhs)
        SIMALL_CUDA_TRY(ctx, cudaMemcpyAsync(rhs, ps->mrhs.p, 3 * ps->nC * sizeof(double), cudaMemcpyDeviceToHost, st));
    if (aP)
        SIMALL_CUDA_TRY(ctx, cudaMemcpyAsync(aP, ps->maP.p, ps->nC * sizeof(double), cudaMemcpyDeviceToHost, st));
    SIMALL_CUDA_TRY(ctx, cudaStreamSynchronize(st));
    return SIMALL_OK;
}

}  // extern "C"
