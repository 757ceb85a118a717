// Batched pressure solves: many independent SPD systems of uneven size in one
// persistent launch.
//
// The reference solves each system with its own CGSolver::solve call
// (src/solver/LinearSolvers.cpp:420-451) -- for a batch that is a loop of
// solves, each a few hundred to a few thousand short iterations of tiny
// kernels.  Here one persistent grid (a few CTAs per SM) pulls systems from an
// atomic work queue ordered largest-first and each CTA runs a complete
// mixed-precision Jacobi-PCG on its system: the FP32 CG on S A S (S = D^-1/2)
// with FP64 reliable updates of the same scheme as the single-system mixed
// solver (true residual b - A x in FP64 from the original CSR, stop test on
// it).  A CTA only ever synchronises with itself (__syncthreads), so no CTA
// can wait on another; the iteration limit bounds every loop.
//
// Storage per system: S A S as symmetric diagonal storage when the system is
// numerically symmetric with at most kBatchDiags upper diagonals (every
// structured grid in natural order), otherwise FP32 CSR of its off-diagonal
// part; FP32 work vectors xh, rh, ph, qh; FP64 scale, b and x.  The entries
// of S A S carry 8-bit corrections and every row of the SpMV is summed in
// float-float arithmetic (ffop.cuh): on the pinned cavity systems of a batch
// that keeps the inner iteration count at the FP64 one, where FP32 entries
// and sums cost 15-30% more iterations.  The CTA size
// (threads) and CTAs per SM are picked by a small autotuner that times each
// candidate on the batch itself the first time a batch shape is solved.
#include "device.cuh"
#include "ffop.cuh"
#include "solver.hpp"

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <new>
#include <numeric>
#include <vector>

namespace simall {

constexpr int kBatchDiags = 4;

struct BatchSys {
    int64_t row0;  // first row in the concatenated row arrays
    int64_t rp0;   // first rowPtr entry (row0 + system index)
    int64_t nz0;   // first nonzero
    int64_t u0;    // first element of U (dia) / of the off-diagonal CSR (csr)
    int64_t orp0;  // first off-diagonal rowPtr entry (csr)
    int n;
    int nd;        // stored diagonals; 0 selects the CSR path
    int off[kBatchDiags];
};

struct BatchOut {
    int iterations;
    int updates;
    int status;
    int converged;
    double true_residual;
    double b_norm;
};

}  // namespace simall

struct simall_batch {
    simall_context *ctx = nullptr;
    simall_solver_config cfg{};
    int nsys = 0;
    int64_t rows = 0, nnz = 0;
    std::vector<simall::BatchSys> h_sys;
    std::vector<int> h_order;
    simall::DevBuf<simall::BatchSys> sys;
    simall::DevBuf<int> order, queue;
    simall::DevBuf<int32_t> rowPtr, colIdx, orow, ocol;
    simall::DevBuf<double> values, scale, b, x;
    simall::DevBuf<float> U, oval, xh, rh, ph, qh;
    simall::DevBuf<int8_t> Uc, oc;  // 8-bit corrections of U / oval (ffop.cuh)
    simall::DevBuf<simall::BatchOut> out;
    std::vector<simall::BatchOut> h_out;
    int block = 0, ctas_per_sm = 0;  // autotuned launch shape
    bool ready = false;
    // the solve (queue reset + persistent kernel) captured as a graph for the
    // current shape and b/x pointers
    cudaGraphExec_t gexec = nullptr;
    const double *g_b = nullptr;
    double *g_x = nullptr;
    int g_block = 0, g_ctas = 0;
    ~simall_batch()
    {
        if (gexec)
            cudaGraphExecDestroy(gexec);
    }
    int64_t kernel_launches = 0;
};

namespace simall {

namespace {

// Sum over the CTA: FP32 within each warp, FP64 across warps; every thread
// receives the totals.  red must hold 2*32 doubles.
__device__ __forceinline__ void cta_allreduce2(float a, double b, double *red, double &sa, double &sb)
{
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    a = warp_sum_f(a);
    b = warp_sum(b);
    if (lane == 0) {
        red[wid] = static_cast<double>(a);
        red[32 + wid] = b;
    }
    __syncthreads();
    double ta = 0.0, tb = 0.0;
    for (int w = 0; w < nw; ++w) {  // same order in every thread: identical totals
        ta += red[w];
        tb += red[32 + w];
    }
    __syncthreads();
    sa = ta;
    sb = tb;
}

__device__ __forceinline__ double cta_allreduce_f(float a, double *red)
{
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    a = warp_sum_f(a);
    if (lane == 0)
        red[wid] = static_cast<double>(a);
    __syncthreads();
    double t = 0.0;
    for (int w = 0; w < nw; ++w)
        t += red[w];
    __syncthreads();
    return t;
}

// Rows a thread handles per pass of a loop: it keeps its rows t, t + B,
// t + 2B, ... in the same order, four at a time with all their loads issued
// before the arithmetic, so a CTA alone keeps enough memory requests in
// flight to stream a large system (one CTA per system).
constexpr int kRowsPerPass = 8;

// q = (S A S) p on rows [0, n) of one system: q_i = p_i + sum_j N_ij p_j with
// N (the off-diagonal part of S A S) as FP32 entries plus their 8-bit
// corrections, the row summed in float-float (ffop.cuh); returns this thread's
// p.q part.
__device__ __forceinline__ float batch_spmv(const BatchSys &S, const float *__restrict__ U,
                                            const int8_t *__restrict__ Uc, const int32_t *__restrict__ orow,
                                            const int32_t *__restrict__ ocol, const float *__restrict__ oval,
                                            const int8_t *__restrict__ oc, const float *p, float *q)
{
    float acc = 0.0f;
    const int n = S.n, B = blockDim.x;
    if (S.nd > 0) {
        const float *Us = U + S.u0;
        const int8_t *Ucs = Uc + S.u0;
        for (int i0 = threadIdx.x; i0 < n; i0 += kRowsPerPass * B) {
            float pi[kRowsPerPass];
            FFAcc y[kRowsPerPass];
#pragma unroll
            for (int u = 0; u < kRowsPerPass; ++u) {
                const int i = i0 + u * B;
                pi[u] = i < n ? p[i] : 0.0f;
                y[u] = ff_start(pi[u]);
            }
            for (int d = 0; d < S.nd; ++d) {
                const int off = S.off[d];
                const int64_t dd = static_cast<int64_t>(d) * n;
#pragma unroll
                for (int u = 0; u < kRowsPerPass; ++u) {
                    const int i = i0 + u * B;
                    if (i < n && i + off < n) {
                        const float a = Us[dd + i];
                        ff_add(y[u], a, ff_low(a, Ucs[dd + i]), p[i + off]);
                    }
                    if (i < n && i - off >= 0) {
                        const float a = Us[dd + i - off];
                        ff_add(y[u], a, ff_low(a, Ucs[dd + i - off]), p[i - off]);
                    }
                }
            }
#pragma unroll
            for (int u = 0; u < kRowsPerPass; ++u) {
                const int i = i0 + u * B;
                if (i < n) {
                    const float qi = ff_value(y[u]);
                    q[i] = qi;
                    acc += pi[u] * qi;
                }
            }
        }
    } else {
        const int32_t *rp = orow + S.orp0;
        const int32_t *ci = ocol + S.u0;
        const float *va = oval + S.u0;
        const int8_t *vc = oc + S.u0;
        for (int i = threadIdx.x; i < n; i += B) {
            const float pi = p[i];
            FFAcc y = ff_start(pi);
            for (int k = rp[i]; k < rp[i + 1]; ++k)
                ff_add(y, va[k], ff_low(va[k], vc[k]), p[ci[k]]);
            const float qi = ff_value(y);
            q[i] = qi;
            acc += pi * qi;
        }
    }
    return acc;
}

// One CTA solves one system (mixed precision, reliable updates).
__device__ void batch_solve_one(const BatchSys &S, const int32_t *__restrict__ rowPtr,
                                const int32_t *__restrict__ colIdx, const double *__restrict__ values,
                                const float *__restrict__ U, const int32_t *__restrict__ orow,
                                const int32_t *__restrict__ ocol, const float *__restrict__ oval,
                                const int8_t *__restrict__ Uc, const int8_t *__restrict__ oc,
                                const double *__restrict__ scale_all, const double *__restrict__ b_all,
                                double *x_all, float *xh_all, float *rh_all, float *ph_all, float *qh_all, double tol,
                                double delta, int maxit, BatchOut *out, double *red)
{
    const int n = S.n;
    const double *sc = scale_all + S.row0;
    const double *b = b_all + S.row0;
    double *x = x_all + S.row0;
    float *xh = xh_all + S.row0, *rh = rh_all + S.row0, *ph = ph_all + S.row0, *qh = qh_all + S.row0;
    const int32_t *rp = rowPtr + S.rp0;
    const int32_t *ci = colIdx + S.nz0;
    const double *va = values + S.nz0;

    // init: x = 0, rh = S b, ph = rh, xh = 0
    float a0 = 0.0f;
    double a1 = 0.0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        const double bi = b[i];
        const float r = static_cast<float>(bi * sc[i]);
        x[i] = 0.0;
        rh[i] = r;
        ph[i] = r;
        xh[i] = 0.0f;
        a0 += r * r;
        a1 += bi * bi;
    }
    double rho, bb;
    cta_allreduce2(a0, a1, red, rho, bb);
    const double bn = sqrt(bb);
    const double bnorm = std_max(bn, 1e-30);
    double sigma0 = sqrt(rho), rmax = sigma0, t0 = bn / bnorm, last = t0;
    int it = 0, updates = 0, status = SIMALL_OK;
    bool done = (t0 < tol) || maxit <= 0;
    while (!done) {
        // q = SAS p, alpha
        const double pq = cta_allreduce_f(batch_spmv(S, U, Uc, orow, ocol, oval, oc, ph, qh), red);
        const bool breakdown = !(pq > 0.0);
        const float alpha = breakdown ? 0.0f : static_cast<float>(rho / pq);
        // xh += alpha p, rh -= alpha q (own rows: no barrier needed before)
        float rr_t = 0.0f;
        for (int i0 = threadIdx.x; i0 < n; i0 += kRowsPerPass * blockDim.x) {
            float xv[kRowsPerPass], pv[kRowsPerPass], rv[kRowsPerPass], qv[kRowsPerPass];
#pragma unroll
            for (int u = 0; u < kRowsPerPass; ++u) {
                const int i = i0 + u * blockDim.x;
                xv[u] = i < n ? xh[i] : 0.0f;
                pv[u] = i < n ? ph[i] : 0.0f;
                rv[u] = i < n ? rh[i] : 0.0f;
                qv[u] = i < n ? qh[i] : 0.0f;
            }
#pragma unroll
            for (int u = 0; u < kRowsPerPass; ++u) {
                const int i = i0 + u * blockDim.x;
                if (i < n) {
                    xh[i] = xv[u] + alpha * pv[u];
                    const float r = rv[u] - alpha * qv[u];
                    rh[i] = r;
                    rr_t += r * r;
                }
            }
        }
        const double rr = cta_allreduce_f(rr_t, red);
        ++it;
        const double sigma = sqrt(rr);
        const double est = t0 * sigma / sigma0;
        double beta;
        if (breakdown || sigma < delta * rmax || est < tol || it >= maxit) {
            // reliable update: x += S xh (FP64), r = b - A x, rh = S r
            for (int i = threadIdx.x; i < n; i += blockDim.x) {
                x[i] += sc[i] * static_cast<double>(xh[i]);
                xh[i] = 0.0f;
            }
            __syncthreads();
            float rho_t = 0.0f;
            double r2_t = 0.0;
            for (int i = threadIdx.x; i < n; i += blockDim.x) {
                double s = 0.0;
                for (int k = rp[i]; k < rp[i + 1]; ++k)
                    s = fma(va[k], x[ci[k]], s);
                const double r = b[i] - s;
                const float rf = static_cast<float>(sc[i] * r);
                rh[i] = rf;
                rho_t += rf * rf;
                r2_t += r * r;
            }
            double rho_new, r2;
            cta_allreduce2(rho_t, r2_t, red, rho_new, r2);
            ++updates;
            const double t = sqrt(r2) / bnorm;
            last = t;
            if (t < tol || it >= maxit || breakdown) {
                if (breakdown && !(t < tol))
                    status = SIMALL_ERR_BREAKDOWN;
                done = true;
                break;
            }
            beta = rho_new / rho;
            rho = rho_new;
            sigma0 = sqrt(rho_new);
            t0 = t;
            rmax = sigma0;
        } else {
            beta = rr / rho;
            rho = rr;
            rmax = sigma > rmax ? sigma : rmax;
            last = est;
        }
        const float bf = static_cast<float>(beta);
        for (int i0 = threadIdx.x; i0 < n; i0 += kRowsPerPass * blockDim.x) {
            float rv[kRowsPerPass], pv[kRowsPerPass];
#pragma unroll
            for (int u = 0; u < kRowsPerPass; ++u) {
                const int i = i0 + u * blockDim.x;
                rv[u] = i < n ? rh[i] : 0.0f;
                pv[u] = i < n ? ph[i] : 0.0f;
            }
#pragma unroll
            for (int u = 0; u < kRowsPerPass; ++u) {
                const int i = i0 + u * blockDim.x;
                if (i < n)
                    ph[i] = rv[u] + bf * pv[u];
            }
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        out->iterations = it;
        out->updates = updates;
        out->status = status;
        out->converged = last < tol ? 1 : 0;
        out->true_residual = last;
        out->b_norm = bn;
    }
    __syncthreads();
}

__global__ void __launch_bounds__(1024) k_batch_solve(const BatchSys *__restrict__ sys, const int *__restrict__ order, int nsys, int *queue,
                              const int32_t *__restrict__ rowPtr, const int32_t *__restrict__ colIdx,
                              const double *__restrict__ values, const float *__restrict__ U,
                              const int32_t *__restrict__ orow, const int32_t *__restrict__ ocol,
                              const float *__restrict__ oval, const int8_t *__restrict__ Uc,
                              const int8_t *__restrict__ oc,
                              const double *__restrict__ scale, const double *__restrict__ b, double *x, float *xh,
                              float *rh, float *ph, float *qh, double tol, double delta, int maxit, BatchOut *out)
{
    __shared__ double red[64];
    __shared__ int s_next;
    for (;;) {
        if (threadIdx.x == 0)
            s_next = atomicAdd(queue, 1);
        __syncthreads();
        const int k = s_next;
        __syncthreads();
        if (k >= nsys)
            return;
        const int id = order[k];
        const BatchSys S = sys[id];
        batch_solve_one(S, rowPtr, colIdx, values, U, orow, ocol, oval, Uc, oc, scale, b, x, xh, rh, ph, qh, tol, delta,
                        maxit, out + id, red);
    }
}

}  // namespace

namespace {

int launch_batch(simall_batch *B, int block, int ctas_per_sm, const double *b, double *x)
{
    simall_context *ctx = B->ctx;
    SIMALL_CUDA_TRY(ctx, cudaMemsetAsync(B->queue.p, 0, sizeof(int), ctx->stream));
    const int grid = std::max(1, std::min(B->nsys, ctx->num_sms * ctas_per_sm));
    k_batch_solve<<<grid, block, 0, ctx->stream>>>(B->sys.p, B->order.p, B->nsys, B->queue.p, B->rowPtr.p, B->colIdx.p,
                                                   B->values.p, B->U.p, B->orow.p, B->ocol.p, B->oval.p, B->Uc.p, B->oc.p,
                                                   B->scale.p, b,
                                                   x, B->xh.p, B->rh.p, B->ph.p, B->qh.p, B->cfg.tolerance,
                                                   B->cfg.reliable_delta, B->cfg.max_iterations, B->out.p);
    ctx->launches.fetch_add(1, std::memory_order_relaxed);
    B->kernel_launches += 1;
    SIMALL_CUDA_TRY(ctx, cudaGetLastError());
    return SIMALL_OK;
}

// Times each launch shape on the batch (device b -> scratch x) and keeps the
// fastest.  Candidates: CTA sizes 256/512/1024 threads, 1-4 CTAs per SM.
int autotune(simall_batch *B, const double *b)
{
    simall_context *ctx = B->ctx;
    const int shapes[][2] = {{256, 4}, {256, 2}, {512, 2}, {512, 1}, {1024, 1}};
    cudaEvent_t e0, e1;
    SIMALL_CUDA_TRY(ctx, cudaEventCreate(&e0));
    SIMALL_CUDA_TRY(ctx, cudaEventCreate(&e1));
    float best = 1e30f;
    for (const auto &sh : shapes) {
        SIMALL_CUDA_TRY(ctx, cudaEventRecord(e0, ctx->stream));
        int st = launch_batch(B, sh[0], sh[1], b, B->x.p);
        if (st)
            return st;
        SIMALL_CUDA_TRY(ctx, cudaEventRecord(e1, ctx->stream));
        SIMALL_CUDA_TRY(ctx, cudaEventSynchronize(e1));
        float ms = 0.0f;
        cudaEventElapsedTime(&ms, e0, e1);
        if (ms < best) {
            best = ms;
            B->block = sh[0];
            B->ctas_per_sm = sh[1];
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return SIMALL_OK;
}

}  // namespace

}  // namespace simall

using namespace simall;

extern "C" {

int simall_batch_create(simall_context *ctx, const simall_solver_config *cfg, simall_batch **out)
{
    if (!ctx || !out)
        return SIMALL_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    simall_solver_config c;
    simall_solver_config_default(&c);
    if (cfg)
        c = *cfg;
    if (c.preconditioner == SIMALL_PRECOND_NONE)
        c.preconditioner = SIMALL_PRECOND_JACOBI;
    if (c.preconditioner != SIMALL_PRECOND_JACOBI)
        return fail(ctx, SIMALL_ERR_UNSUPPORTED, "batched solves use the Jacobi preconditioner");
    if (!(c.tolerance >= 0.0) || c.reliable_delta <= 0.0 || c.reliable_delta >= 1.0)
        return fail(ctx, SIMALL_ERR_INVALID_ARGUMENT, "tolerance / reliable_delta out of range");
    auto *B = new (std::nothrow) simall_batch;
    if (!B)
        return SIMALL_ERR_OUT_OF_MEMORY;
    B->ctx = ctx;
    B->cfg = c;
    *out = B;
    return SIMALL_OK;
}

int simall_batch_destroy(simall_batch *B)
{
    if (!B)
        return SIMALL_ERR_INVALID_ARGUMENT;
    cudaStreamSynchronize(B->ctx->stream);
    delete B;
    return SIMALL_OK;
}

int simall_batch_set_systems(simall_batch *B, int n_systems, const int64_t *row_offsets, const int64_t *nnz_offsets,
                             const int32_t *rowPtr, const int32_t *colIdx, const double *values)
{
    if (!B || n_systems <= 0 || !row_offsets || !nnz_offsets || !rowPtr || !colIdx || !values)
        return SIMALL_ERR_INVALID_ARGUMENT;
    simall_context *ctx = B->ctx;
    SIMALL_CUDA_TRY(ctx, cudaSetDevice(ctx->device));
    B->ready = false;
    const int64_t rows = row_offsets[n_systems], nnz = nnz_offsets[n_systems];
    if (row_offsets[0] != 0 || nnz_offsets[0] != 0 || rows <= 0 || nnz <= 0 || rows > INT32_MAX)
        return fail(ctx, SIMALL_ERR_SIZE_MISMATCH, "batch offsets must start at 0 and grow");
    std::vector<BatchSys> sys(static_cast<size_t>(n_systems));
    std::vector<double> scale(static_cast<size_t>(rows));
    std::vector<float> U;
    std::vector<int8_t> Uc, oc;
    std::vector<int32_t> orow, ocol;
    std::vector<float> oval;
    std::vector<int32_t> offs;
    for (int s = 0; s < n_systems; ++s) {
        const int64_t r0 = row_offsets[s], r1 = row_offsets[s + 1];
        const int64_t z0 = nnz_offsets[s], z1 = nnz_offsets[s + 1];
        const int64_t n = r1 - r0;
        if (n <= 0 || z1 < z0)
            return fail(ctx, SIMALL_ERR_SIZE_MISMATCH, "system %d: empty or negative size", s);
        const int32_t *rp = rowPtr + r0 + s;
        const int32_t *ci = colIdx + z0;
        const double *va = values + z0;
        int st = check_csr_host(ctx, n, z1 - z0, rp, ci, va, true);
        if (st)
            return fail(ctx, st, "system %d: %s", s, ctx->last_error.c_str());
        BatchSys &S = sys[s];
        S.row0 = r0;
        S.rp0 = r0 + s;
        S.nz0 = z0;
        S.n = static_cast<int>(n);
        // scale, symmetry, diagonal structure
        offs.clear();
        bool dia = true, sym = true;
        int64_t upper = 0;
        for (int64_t i = 0; i < n; ++i) {
            double d = 0.0;
            for (int k = rp[i]; k < rp[i + 1]; ++k) {
                const int j = ci[k];
                if (j == i)
                    d = va[k];
                if (j <= i)
                    continue;
                ++upper;
                const int32_t off = j - static_cast<int32_t>(i);
                if (std::find(offs.begin(), offs.end(), off) == offs.end()) {
                    if (static_cast<int>(offs.size()) == kBatchDiags)
                        dia = false;
                    else
                        offs.push_back(off);
                }
                // a_ji must equal a_ij
                const int32_t *b0 = ci + rp[j], *b1 = ci + rp[j + 1];
                const int32_t *p = std::lower_bound(b0, b1, static_cast<int32_t>(i));
                if (p == b1 || *p != i || va[rp[j] + (p - b0)] != va[k])
                    sym = false;
            }
            if (!(d > 0.0))
                return fail(ctx, SIMALL_ERR_NOT_POSITIVE, "system %d: non-positive diagonal in row %lld", s,
                            static_cast<long long>(i));
            scale[r0 + i] = 1.0 / std::sqrt(d);
        }
        if (offs.empty() || static_cast<double>(offs.size()) * n > 1.3 * static_cast<double>(upper))
            dia = false;
        dia = dia && sym;
        const double *sc = scale.data() + r0;
        if (dia) {
            std::sort(offs.begin(), offs.end());
            S.nd = static_cast<int>(offs.size());
            for (int d = 0; d < kBatchDiags; ++d)
                S.off[d] = d < S.nd ? offs[d] : 0;
            S.u0 = static_cast<int64_t>(U.size());
            S.orp0 = 0;
            U.resize(U.size() + static_cast<size_t>(S.nd) * n, 0.0f);
            Uc.resize(U.size(), 0);
            float *Us = U.data() + S.u0;
            int8_t *Ucs = Uc.data() + S.u0;
            for (int64_t i = 0; i < n; ++i)
                for (int k = rp[i]; k < rp[i + 1]; ++k) {
                    const int j = ci[k];
                    if (j <= i)
                        continue;
                    const int d = static_cast<int>(std::find(offs.begin(), offs.end(), j - static_cast<int>(i)) -
                                                   offs.begin());
                    const double a = va[k] * sc[i] * sc[j];
                    const int64_t t = static_cast<int64_t>(d) * n + i;
                    Us[t] = static_cast<float>(a);
                    Ucs[t] = ff_correction(a, Us[t]);
                }
        } else {
            S.nd = 0;
            std::fill(S.off, S.off + kBatchDiags, 0);
            S.orp0 = static_cast<int64_t>(orow.size());
            S.u0 = static_cast<int64_t>(ocol.size());
            int32_t cnt = 0;
            orow.push_back(0);
            for (int64_t i = 0; i < n; ++i) {
                for (int k = rp[i]; k < rp[i + 1]; ++k)
                    if (ci[k] != i) {
                        const double a = va[k] * sc[i] * sc[ci[k]];
                        ocol.push_back(ci[k]);
                        oval.push_back(static_cast<float>(a));
                        oc.push_back(ff_correction(a, oval.back()));
                        ++cnt;
                    }
                orow.push_back(cnt);
            }
        }
    }
    // largest systems first: the persistent grid then ends with the short ones
    std::vector<int> order(static_cast<size_t>(n_systems));
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return sys[a].n > sys[b].n; });
    // upload
    cudaStream_t st = ctx->stream;
    SIMALL_CUDA_TRY(ctx, B->sys.alloc(n_systems));
    SIMALL_CUDA_TRY(ctx, B->order.alloc(n_systems));
    SIMALL_CUDA_TRY(ctx, B->queue.alloc(1));
    SIMALL_CUDA_TRY(ctx, B->out.alloc(n_systems));
    SIMALL_CUDA_TRY(ctx, B->rowPtr.alloc(rows + n_systems));
    SIMALL_CUDA_TRY(ctx, B->colIdx.alloc(nnz));
    SIMALL_CUDA_TRY(ctx, B->values.alloc(nnz));
    SIMALL_CUDA_TRY(ctx, B->scale.alloc(rows));
    SIMALL_CUDA_TRY(ctx, B->b.alloc(rows));
    SIMALL_CUDA_TRY(ctx, B->x.alloc(rows));
    SIMALL_CUDA_TRY(ctx, B->xh.alloc(rows));
    SIMALL_CUDA_TRY(ctx, B->rh.alloc(rows));
    SIMALL_CUDA_TRY(ctx, B->ph.alloc(rows));
    SIMALL_CUDA_TRY(ctx, B->qh.alloc(rows));
    SIMALL_CUDA_TRY(ctx, B->U.alloc(std::max<size_t>(U.size(), 1)));
    SIMALL_CUDA_TRY(ctx, B->Uc.alloc(std::max<size_t>(Uc.size(), 1)));
    SIMALL_CUDA_TRY(ctx, B->oc.alloc(std::max<size_t>(oc.size(), 1)));
    SIMALL_CUDA_TRY(ctx, B->orow.alloc(std::max<size_t>(orow.size(), 1)));
    SIMALL_CUDA_TRY(ctx, B->ocol.alloc(std::max<size_t>(ocol.size(), 1)));
    SIMALL_CUDA_TRY(ctx, B->oval.alloc(std::max<size_t>(oval.size(), 1)));
    auto up = [&](void *d, const void *h, size_t bytes) { return cudaMemcpyAsync(d, h, bytes, cudaMemcpyHostToDevice, st); };
    SIMALL_CUDA_TRY(ctx, up(B->sys.p, sys.data(), sys.size() * sizeof(BatchSys)));
    SIMALL_CUDA_TRY(ctx, up(B->order.p, order.data(), order.size() * sizeof(int)));
    SIMALL_CUDA_TRY(ctx, up(B->rowPtr.p, rowPtr, (rows + n_systems) * sizeof(int32_t)));
    SIMALL_CUDA_TRY(ctx, up(B->colIdx.p, colIdx, nnz * sizeof(int32_t)));
    SIMALL_CUDA_TRY(ctx, up(B->values.p, values, nnz * sizeof(double)));
    SIMALL_CUDA_TRY(ctx, up(B->scale.p, scale.data(), scale.size() * sizeof(double)));
    if (!U.empty()) {
        SIMALL_CUDA_TRY(ctx, up(B->U.p, U.data(), U.size() * sizeof(float)));
        SIMALL_CUDA_TRY(ctx, up(B->Uc.p, Uc.data(), Uc.size()));
    }
    if (!orow.empty()) {
        SIMALL_CUDA_TRY(ctx, up(B->orow.p, orow.data(), orow.size() * sizeof(int32_t)));
        if (!ocol.empty()) {
            SIMALL_CUDA_TRY(ctx, up(B->ocol.p, ocol.data(), ocol.size() * sizeof(int32_t)));
            SIMALL_CUDA_TRY(ctx, up(B->oval.p, oval.data(), oval.size() * sizeof(float)));
            SIMALL_CUDA_TRY(ctx, up(B->oc.p, oc.data(), oc.size()));
        }
    }
    SIMALL_CUDA_TRY(ctx, cudaStreamSynchronize(st));  // host staging vectors die here
    B->nsys = n_systems;
    B->rows = rows;
    B->nnz = nnz;
    B->h_sys = std::move(sys);
    B->h_order = std::move(order);
    B->h_out.assign(static_cast<size_t>(n_systems), BatchOut{});
    B->block = 0;  // re-tune for the new batch
    B->ready = true;
    return SIMALL_OK;
}

int simall_batch_solve(simall_batch *B, const double *b, double *x, int mem, simall_batch_system_stats *per_system,
                       simall_batch_stats *total)
{
    if (!B || !b || !x)
        return SIMALL_ERR_INVALID_ARGUMENT;
    simall_context *ctx = B->ctx;
    if (!B->ready)
        return fail(ctx, SIMALL_ERR_INVALID_ARGUMENT, "batch solve before set_systems");
    if (mem != SIMALL_MEM_HOST && mem != SIMALL_MEM_DEVICE)
        return fail(ctx, SIMALL_ERR_INVALID_ARGUMENT, "batch solve: bad memory kind %d", mem);
    SIMALL_CUDA_TRY(ctx, cudaSetDevice(ctx->device));
    const auto t0 = std::chrono::steady_clock::now();
    const size_t bytes = static_cast<size_t>(B->rows) * sizeof(double);
    const double *db = b;
    if (mem == SIMALL_MEM_HOST) {
        for (int64_t i = 0; i < B->rows; ++i)
            if (!std::isfinite(b[i]))
                return fail(ctx, SIMALL_ERR_NON_FINITE, "b contains NaN or Inf");
        SIMALL_CUDA_TRY(ctx, cudaMemcpyAsync(B->b.p, b, bytes, cudaMemcpyHostToDevice, ctx->stream));
        db = B->b.p;
    }
    if (B->block == 0) {
        int st = autotune(B, db);
        if (st)
            return st;
    }
    double *dx = (mem == SIMALL_MEM_HOST) ? B->x.p : x;
    if (!B->gexec || B->g_b != db || B->g_x != dx || B->g_block != B->block || B->g_ctas != B->ctas_per_sm) {
        if (B->gexec) {
            cudaGraphExecDestroy(B->gexec);
            B->gexec = nullptr;
        }
        cudaGraph_t graph = nullptr;
        SIMALL_CUDA_TRY(ctx, cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
        const int st = launch_batch(B, B->block, B->ctas_per_sm, db, dx);
        const cudaError_t e = cudaStreamEndCapture(ctx->stream, &graph);
        if (st)
            return st;
        if (e != cudaSuccess)
            return cuda_fail(ctx, e, "cudaStreamEndCapture", __FILE__, __LINE__);
        const cudaError_t ei = cudaGraphInstantiate(&B->gexec, graph, 0);
        cudaGraphDestroy(graph);
        if (ei != cudaSuccess)
            return cuda_fail(ctx, ei, "cudaGraphInstantiate", __FILE__, __LINE__);
        B->g_b = db;
        B->g_x = dx;
        B->g_block = B->block;
        B->g_ctas = B->ctas_per_sm;
    } else {
        ctx->launches.fetch_add(1, std::memory_order_relaxed);
        B->kernel_launches += 1;
    }
    SIMALL_CUDA_TRY(ctx, cudaGraphLaunch(B->gexec, ctx->stream));
    SIMALL_CUDA_TRY(ctx, cudaMemcpyAsync(B->h_out.data(), B->out.p, B->nsys * sizeof(BatchOut), cudaMemcpyDeviceToHost,
                                         ctx->stream));
    if (mem == SIMALL_MEM_HOST)
        SIMALL_CUDA_TRY(ctx, cudaMemcpyAsync(x, dx, bytes, cudaMemcpyDeviceToHost, ctx->stream));
    SIMALL_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
    int conv = 0, maxit = 0, worst_status = SIMALL_OK;
    int64_t sum_it = 0;
    double worst = 0.0;
    for (int s = 0; s < B->nsys; ++s) {
        const BatchOut &o = B->h_out[s];
        conv += o.converged;
        sum_it += o.iterations;
        maxit = std::max(maxit, o.iterations);
        worst = std::max(worst, o.true_residual);
        if (o.status != SIMALL_OK)
            worst_status = o.status;
        if (per_system) {
            per_system[s].iterations = o.iterations;
            per_system[s].reliable_updates = o.updates;
            per_system[s].converged = o.converged;
            per_system[s].status = o.status;
            per_system[s].true_residual = o.true_residual;
            per_system[s].b_norm = o.b_norm;
        }
    }
    if (total) {
        total->systems = B->nsys;
        total->converged = conv;
        total->max_iterations = maxit;
        total->total_iterations = sum_it;
        total->worst_true_residual = worst;
        total->status = worst_status;
        total->block_threads = B->block;
        total->ctas_per_sm = B->ctas_per_sm;
        total->seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    }
    return SIMALL_OK;
}

int simall_batch_launch_shape(simall_batch *B, int block_threads, int ctas_per_sm)
{
    if (!B || (block_threads != 0 && block_threads != 256 && block_threads != 512 && block_threads != 1024) ||
        ctas_per_sm < 0 || ctas_per_sm > 8)
        return SIMALL_ERR_INVALID_ARGUMENT;
    B->block = block_threads;
    B->ctas_per_sm = block_threads ? ctas_per_sm : 0;
    return SIMALL_OK;
}

}  // extern "C"
