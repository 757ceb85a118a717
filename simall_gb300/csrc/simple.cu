// One SIMPLE outer iteration with every field in device memory: the GB300
// replacement of SimpleAlgorithm::iterate and ::advance_time_step
// (src/solver/SimpleAlgorithm.cpp:522-570) and of the PISO and PIMPLE
// iterate() overrides (src/solver/PisoAlgorithm.cpp:27-70,
// PimpleAlgorithm.cpp:48-96: outer correctors, pressure correctors,
// non-orthogonal passes, optional momentum predictor, early exit), no
// periodic faces, no halo exchange (one GPU).
//
//   compute_face_fluxes           simall_compute_face_fluxes
//   assemble_momentum(x, y, z)    simall_assemble_momentum, all three at once:
//                                 the matrix does not depend on the component
//                                 and no component's right-hand side reads
//                                 another component of U, so assembling them
//                                 before the three solves is what the
//                                 reference's interleaved loop computes
//   solve_momentum_component(k)   the momentum solver (any kind), x from 0,
//                                 written into U_k; |A U_k - b| from the
//                                 solver's FP64 true residual
//   compute_face_fluxes           again, from the new U
//   assemble_pressure_correction  SIMPLE (aP) or SIMPLEC (denominator from the
//                                 momentum matrix)
//   solve + correct_fields        the pressure solver, then p, U and phi
// The host only sequences launches; the solvers poll their stop flags.
#include "device.cuh"
#include "pressure_system.hpp"
#include "registry.hpp"
#include "solver.hpp"

#include <cmath>
#include <new>

struct simall_simple {
    simall_context *ctx = nullptr;  // outlives the system and solvers it points to
    simall_pressure_system *ps = nullptr;
    simall_solver *mom = nullptr, *pres = nullptr;
    simall_simple_options o{};
    simall::DevBuf<double> U, p, phi, pPrime, Un, Unm1;
    double *uext = nullptr, *pext = nullptr;  // U and p of a bound field registry
    int timeStep = 0;
    double *Ud() { return uext ? uext : U.p; }
    double *Pd() { return pext ? pext : p.p; }
};

using namespace simall;

namespace {

int copy_in(simall_context *ctx, double *dst, const double *src, int64_t n, int mem)
{
    SIMALL_CUDA_TRY(ctx, cudaMemcpyAsync(dst, src, n * sizeof(double),
                                         mem == SIMALL_MEM_HOST ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice,
                                         ctx->stream));
    return SIMALL_OK;
}

int copy_out(simall_context *ctx, double *dst, const double *src, int64_t n, int mem)
{
    SIMALL_CUDA_TRY(ctx, cudaMemcpyAsync(dst, src, n * sizeof(double),
                                         mem == SIMALL_MEM_HOST ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice,
                                         ctx->stream));
    return SIMALL_OK;
}

}  // namespace

extern "C" {

void simall_simple_options_default(simall_simple_options *o)
{
    if (!o)
        return;
    // SimpleOptions defaults (src/solver/SimpleAlgorithm.hpp:43-57)
    o->urfU = 0.7;
    o->urfP = 0.3;
    o->rho = 1.0;
    o->mu = 1.0e-3;
    o->dt = 0.0;
    o->bdf2 = 0;
    o->simplec = 0;
    o->n_outer_correctors = 1;
    o->n_correctors = 1;
    o->n_non_orth_corr = 0;
    o->momentum_predictor = 1;
    o->tol_u = 0.0;
    o->tol_p = 0.0;
}

int simall_simple_create(simall_pressure_system *ps, simall_solver *momentum, simall_solver *pressure,
                         const simall_simple_options *opt, simall_simple **out)
{
    if (!ps || !momentum || !pressure || !out || momentum == pressure)
        return SIMALL_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    simall_context *ctx = ps->ctx;
    if (!ps->fieldsReady)
        return fail(ctx, SIMALL_ERR_INVALID_ARGUMENT, "SIMPLE: call simall_pressure_system_setup_field_loops first");
    if (momentum->ctx != ctx || pressure->ctx != ctx)
        return fail(ctx, SIMALL_ERR_INVALID_ARGUMENT, "SIMPLE: solvers and system must share one context");
    simall_simple_options o;
    simall_simple_options_default(&o);
    if (opt)
        o = *opt;
    if (!(o.urfU != 0.0) || !(o.rho == o.rho) || !(o.dt >= 0.0))
        return fail(ctx, SIMALL_ERR_INVALID_ARGUMENT, "SIMPLE: urfU must be non-zero and dt >= 0");
    // the clamps of PimpleAlgorithm's constructor (PimpleAlgorithm.cpp:23-29)
    o.n_outer_correctors = o.n_outer_correctors < 1 ? 1 : o.n_outer_correctors;
    o.n_correctors = o.n_correctors < 1 ? 1 : o.n_correctors;
    o.n_non_orth_corr = o.n_non_orth_corr < 0 ? 0 : o.n_non_orth_corr;
    SIMALL_CUDA_TRY(ctx, cudaSetDevice(ctx->device));
    auto *s = new (std::nothrow) simall_simple;
    if (!s)
        return SIMALL_ERR_OUT_OF_MEMORY;
    s->ctx = ctx;
    s->ps = ps;
    s->mom = momentum;
    s->pres = pressure;
    s->o = o;
    const int64_t nC = ps->nC, nF = ps->nF;
    cudaError_t e = cudaSuccess;
    for (auto *b : {&s->U, &s->Un, &s->Unm1})
        if (e == cudaSuccess)
            e = b->alloc(3 * nC);
    for (auto *b : {&s->p, &s->pPrime})
        if (e == cudaSuccess)
            e = b->alloc(nC);
    if (e == cudaSuccess)
        e = s->phi.alloc(nF);
    if (e != cudaSuccess) {
        delete s;
        return cuda_fail(ctx, e, "SIMPLE field allocation", __FILE__, __LINE__);
    }
    cudaStream_t st = ctx->stream;
    SIMALL_CUDA_TRY(ctx, cudaMemsetAsync(s->Ud(), 0, 3 * nC * sizeof(double), st));
    SIMALL_CUDA_TRY(ctx, cudaMemsetAsync(s->Un.p, 0, 3 * nC * sizeof(double), st));
    SIMALL_CUDA_TRY(ctx, cudaMemsetAsync(s->Unm1.p, 0, 3 * nC * sizeof(double), st));
    SIMALL_CUDA_TRY(ctx, cudaMemsetAsync(s->Pd(), 0, nC * sizeof(double), st));
    SIMALL_CUDA_TRY(ctx, cudaMemsetAsync(s->pPrime.p, 0, nC * sizeof(double), st));
    SIMALL_CUDA_TRY(ctx, cudaMemsetAsync(s->phi.p, 0, nF * sizeof(double), st));
    SIMALL_CUDA_TRY(ctx, cudaStreamSynchronize(st));
    *out = s;
    return SIMALL_OK;
}

int simall_simple_destroy(simall_simple *s)
{
    if (!s)
        return SIMALL_ERR_INVALID_ARGUMENT;
    cudaStreamSynchronize(s->ctx->stream);
    delete s;
    return SIMALL_OK;
}

int simall_simple_set_fields(simall_simple *s, const double *U, const double *p, int mem)
{
    if (!s || (mem != SIMALL_MEM_HOST && mem != SIMALL_MEM_DEVICE))
        return SIMALL_ERR_INVALID_ARGUMENT;
    simall_context *ctx = s->ps->ctx;
    SIMALL_CUDA_TRY(ctx, cudaSetDevice(ctx->device));
    const int64_t nC = s->ps->nC;
    if (U) {
        int e = copy_in(ctx, s->Ud(), U, 3 * nC, mem);
        if (e)
            return e;
    }
    if (p) {
        int e = copy_in(ctx, s->Pd(), p, nC, mem);
        if (e)
            return e;
    }
    SIMALL_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
    return SIMALL_OK;
}

int simall_simple_get_fields(simall_simple *s, double *U, double *p, double *phi, int mem)
{
    if (!s || (mem != SIMALL_MEM_HOST && mem != SIMALL_MEM_DEVICE))
        return SIMALL_ERR_INVALID_ARGUMENT;
    simall_context *ctx = s->ps->ctx;
    SIMALL_CUDA_TRY(ctx, cudaSetDevice(ctx->device));
    const int64_t nC = s->ps->nC, nF = s->ps->nF;
    int e = SIMALL_OK;
    if (U && !e)
        e = copy_out(ctx, U, s->Ud(), 3 * nC, mem);
    if (p && !e)
        e = copy_out(ctx, p, s->Pd(), nC, mem);
    if (phi && !e)
        e = copy_out(ctx, phi, s->phi.p, nF, mem);
    if (e)
        return e;
    SIMALL_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
    return SIMALL_OK;
}

int simall_simple_device_fields(simall_simple *s, double **U, double **p, double **phi)
{
    if (!s)
        return SIMALL_ERR_INVALID_ARGUMENT;
    if (U)
        *U = s->Ud();
    if (p)
        *p = s->Pd();
    if (phi)
        *phi = s->phi.p;
    return SIMALL_OK;
}

int simall_simple_bind_fields(simall_simple *s, simall_fields *fields)
{
    if (!s || !fields || fields->ctx != s->ctx)
        return SIMALL_ERR_INVALID_ARGUMENT;
    SIMALL_CUDA_TRY(s->ctx, cudaSetDevice(s->ctx->device));
    int st = SIMALL_OK;
    simall_fields::Field *u = registry_get(fields, "U", s->ps->nC, true, &st);
    if (!u)
        return st;
    simall_fields::Field *p = registry_get(fields, "p", s->ps->nC, false, &st);
    if (!p)
        return st;
    s->uext = u->data.p;
    s->pext = p->data.p;
    return SIMALL_OK;
}

int simall_simple_iterate(simall_simple *s, simall_simple_residuals *res)
{
    if (!s)
        return SIMALL_ERR_INVALID_ARGUMENT;
    simall_pressure_system *ps = s->ps;
    simall_context *ctx = ps->ctx;
    SIMALL_CUDA_TRY(ctx, cudaSetDevice(ctx->device));
    const int64_t nC = ps->nC;
    const simall_simple_options &o = s->o;
    double *U = s->Ud();
    simall_simple_residuals r{};
    int outer = 0;
    for (outer = 0; outer < o.n_outer_correctors; ++outer) {
        int e = simall_compute_face_fluxes(ps, o.rho, U, U + nC, U + 2 * nC, s->phi.p, SIMALL_MEM_DEVICE);
        if (e)
            return e;
        if (o.momentum_predictor) {
            simall_momentum_options mo;
            mo.rho = o.rho;
            mo.mu = o.mu;
            mo.urfU = o.urfU;
            mo.dt = o.dt;
            mo.bdf2 = (o.dt > 0.0 && o.bdf2 && s->timeStep >= 1) ? 1 : 0;  // BDF2 from the second step (:335)
            mo.reserved = 0;
            e = simall_assemble_momentum(ps, &mo, U, s->Pd(), s->phi.p, s->Un.p, s->Unm1.p, SIMALL_MEM_DEVICE);
            if (e)
                return e;
            e = simall_solver_set_matrix(s->mom, nC, ps->nnz, ps->rowPtr.p, ps->colIdx.p, ps->mvalues.p,
                                         SIMALL_MEM_DEVICE);
            if (e)
                return e;
            for (int k = 0; k < 3; ++k) {
                simall_solver_stats st{};
                e = solver_solve_impl(s->mom, ps->mrhs.p + k * nC, SIMALL_MEM_DEVICE, U + k * nC, SIMALL_MEM_DEVICE,
                                      &st);
                if (e)
                    return e;
                r.mom[k] = st.true_residual * st.b_norm;  // |A U_k - b|
                r.iterations[k] = st.iterations;
            }
        } else if (!ps->momReady) {
            return fail(ctx, SIMALL_ERR_INVALID_ARGUMENT, "SIMPLE: no momentum predictor has run to provide aP");
        }
        for (int corr = 0; corr < o.n_correctors; ++corr) {
            e = simall_compute_face_fluxes(ps, o.rho, U, U + nC, U + 2 * nC, s->phi.p, SIMALL_MEM_DEVICE);
            if (e)
                return e;
            for (int no = 0; no <= o.n_non_orth_corr; ++no) {
                e = o.simplec ? simall_assemble_pressure_correction_simplec(ps, o.rho, ps->maP.p, ps->mvalues.p,
                                                                            s->phi.p, SIMALL_MEM_DEVICE, nullptr)
                              : simall_assemble_pressure_correction(ps, o.rho, ps->maP.p, s->phi.p,
                                                                    SIMALL_MEM_DEVICE, nullptr);
                if (e)
                    return e;
                simall_solver_stats st{};
                e = simall_pressure_system_solve(ps, s->pres, s->pPrime.p, SIMALL_MEM_DEVICE, &st);
                if (e)
                    return e;
                r.cont = st.b_norm > 1e-30 ? st.b_norm : 0.0;  // |rhs|; the solver floors its norm at 1e-30
                r.iterations[3] = st.iterations;
                e = simall_correct_fields(ps, o.rho, o.urfP, ps->maP.p, s->pPrime.p, s->Pd(), U, U + nC, U + 2 * nC,
                                          s->phi.p, SIMALL_MEM_DEVICE);
                if (e)
                    return e;
            }
        }
        // PimpleAlgorithm's early exit: every tolerance that is set holds
        bool conv = o.tol_u > 0.0 || o.tol_p > 0.0;
        if (o.tol_u > 0.0) {
            double mm = std::fabs(r.mom[0]);
            mm = (mm < std::fabs(r.mom[1])) ? std::fabs(r.mom[1]) : mm;
            mm = (mm < std::fabs(r.mom[2])) ? std::fabs(r.mom[2]) : mm;
            if (mm > o.tol_u)
                conv = false;
        }
        if (o.tol_p > 0.0 && std::fabs(r.cont) > o.tol_p)
            conv = false;
        if (conv)
            break;
    }
    r.outer = outer < o.n_outer_correctors ? outer : o.n_outer_correctors - 1;
    if (res)
        *res = r;
    return SIMALL_OK;
}

int simall_simple_advance_time_step(simall_simple *s, int n_inner, simall_simple_residuals *res)
{
    if (!s)
        return SIMALL_ERR_INVALID_ARGUMENT;
    simall_context *ctx = s->ps->ctx;
    SIMALL_CUDA_TRY(ctx, cudaSetDevice(ctx->device));
    const size_t bytes = 3 * static_cast<size_t>(s->ps->nC) * sizeof(double);
    // roll the history: U^{n-1} <- U^n (from the second step), U^n <- U
    if (s->timeStep >= 1)
        SIMALL_CUDA_TRY(ctx, cudaMemcpyAsync(s->Unm1.p, s->Un.p, bytes, cudaMemcpyDeviceToDevice, ctx->stream));
    SIMALL_CUDA_TRY(ctx, cudaMemcpyAsync(s->Un.p, s->Ud(), bytes, cudaMemcpyDeviceToDevice, ctx->stream));
    simall_simple_residuals last{};
    for (int k = 0; k < (n_inner > 1 ? n_inner : 1); ++k) {
        int e = simall_simple_iterate(s, &last);
        if (e)
            return e;
    }
    s->timeStep += 1;
    if (res)
        *res = last;
    return SIMALL_OK;
}

}  // extern "C"
