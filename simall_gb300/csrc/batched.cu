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
// part; the row sums e_i = 1 + sum_j (S A S)_ij (FP64 sum, one rounding) of
// the row-sum product; the iteration state packed per row as one float4
// (r, q, p, xh), double-buffered; FP64 scale, b and x.  Each step is the fused
// single-pass step of the sliced engines (sell.cuh) with float-float sums and
// one block reduction; a CTA takes the step specialised for its system's
// number of stored diagonals, so a row's coefficients and neighbours are all
// loaded before its first multiply (the rows of a CTA's system live in L2,
// and a row's time is its load latency).
//
// Systems of at least cluster_rows rows in diagonal storage run instead on
// one thread-block cluster each (cluster.cu, k_cl_mixed_batch: vectors in the
// cluster's shared memory), a fixed number of clusters striding through them
// on reserved SMs while the one-CTA queue runs the rest on the other SMs: one
// SM took 0.12 s for the ~2000 steps of a 65,025-row system before the
// specialised step (about 47 GB/s), a 16-CTA cluster takes ~13 ms.  The
// one-CTA shape (threads,
// CTAs per SM, rows in flight per thread) and the cluster route (row
// threshold, cluster size, clusters) are picked by an autotuner that times
// candidates on the batch itself and keeps its choice in a JSON cache
// (autotune_cache.cpp) keyed by device and batch shape.
#include "device.cuh"
#include "ffsum.cuh"
#include "mixed_state.cuh"
#include "sell.cuh"
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

using BatchOut = ClBatchResult;

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
    simall::DevBuf<float> U, oval, e;
    simall::DevBuf<float4> st[2];  // (r, q, p, xh) per row, by step parity
    simall::DevBuf<simall::BatchOut> out;
    std::vector<simall::BatchOut> h_out;
    int block = 0, ctas_per_sm = 0, rows_per_pass = 0;  // autotuned launch shape
    int cluster_rows = 0, cluster_ctas = 0;  // systems of at least cluster_rows rows: one cluster of cluster_ctas CTAs
    int clusters = 0;                        // clusters resident at a time (they stride through those systems)
    int tune_source = 0;             // 0 set by the caller, 1 timed on this batch, 2 read from the cache
    // the current plan: the systems on clusters, per stored-diagonal count, and the rest
    int plan_rows = -1, plan_ctas = -1;
    int nsmall = 0, ncluster = 0;
    std::vector<simall::ClBatchItem> h_items[5];
    simall::DevBuf<simall::ClBatchItem> items[5];
    int items_logR[5] = {0, 0, 0, 0, 0};
    cudaStream_t side = nullptr;
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
    std::string cache_path;          // autotuner cache (JSON); empty: none
    std::string shape_key;           // the batch's key in that cache
    bool ready = false;
    // the solve (queue reset + persistent kernel) captured as a graph for the
    // current shape and b/x pointers
    cudaGraphExec_t gexec = nullptr;
    const double *g_b = nullptr;
    double *g_x = nullptr;
    int g_block = 0, g_ctas = 0, g_rpp = 0, g_crows = -1, g_cctas = -1, g_clusters = -1;
    ~simall_batch()
    {
        if (gexec)
            cudaGraphExecDestroy(gexec);
        if (ev_fork)
            cudaEventDestroy(ev_fork);
        if (ev_join)
            cudaEventDestroy(ev_join);
        if (side)
            cudaStreamDestroy(side);
    }
    int64_t kernel_launches = 0;
};

namespace simall {

namespace {

// Everything one launch needs.
struct BatchArgs {
    const BatchSys *sys;
    const int *order;
    int nsys;
    int *queue;
    const int32_t *rowPtr, *colIdx;
    const double *values;
    const float *U;  // dia systems: [nd][n] upper diagonals of S A S
    const int32_t *orow, *ocol;
    const float *oval;  // csr systems: off-diagonal part of S A S
    const float *e;     // row sums 1 + sum_j (S A S)_ij, every row
    const double *scale, *b;
    double *x;
    float4 *st[2];  // (r, q, p, xh) per row, by step parity
    double tol, delta;
    int maxit;
    BatchOut *out;
};

// The row-sum product of row i of one system: e_i p_i - sum_j N_ij (p_i -
// p_j), N = S A S - I, with p_j formed again from the neighbour's previous
// state (sell.cuh p_of: the owner's two roundings, the same bits).  ND > 0:
// ND stored diagonals; every coefficient and neighbour is loaded before the
// first multiply (a neighbour outside [0, n) reads the row itself with a
// zero coefficient, which adds nothing), so a row waits for one round of
// loads instead of one per diagonal.  ND == 0: the system's off-diagonal CSR.
template <int ND>
__device__ __forceinline__ float batch_row(const BatchSys &S, const BatchArgs &a, const float4 *in, int i, float pi,
                                           float alpha, float beta)
{
    const int n = S.n;
    float y = __ldg(a.e + S.row0 + i) * pi;
    if constexpr (ND > 0) {
        const float *U = a.U + S.u0;
        float u[2 * ND];
        float4 g[2 * ND];
#pragma unroll
        for (int d = 0; d < ND; ++d) {
            const int off = S.off[d];
            const float *Ud = U + static_cast<int64_t>(d) * n;
            const bool up = i + off < n, dn = i - off >= 0;
            u[2 * d] = up ? __ldg(Ud + i) : 0.0f;
            u[2 * d + 1] = dn ? __ldg(Ud + i - off) : 0.0f;
            g[2 * d] = in[up ? i + off : i];
            g[2 * d + 1] = in[dn ? i - off : i];
        }
#pragma unroll
        for (int t = 0; t < 2 * ND; ++t)
            y = __fmaf_rn(-u[t], pi - p_of(g[t], alpha, beta), y);
    } else {
        const int32_t *rp = a.orow + S.orp0;
        const int32_t *cc = a.ocol + S.u0;
        const float *vv = a.oval + S.u0;
        for (int k = __ldg(rp + i); k < __ldg(rp + i + 1); ++k)
            y = __fmaf_rn(-__ldg(vv + k), pi - p_of(in[__ldg(cc + k)], alpha, beta), y);
    }
    return y;
}

// One CTA solves one system: the fused mixed-precision CG step of the sliced
// engines (sell.cuh: r, p, xh updates and q = (S A S) p in one pass over the
// packed state, four float-float sums, one block reduction per step), the
// reliable updates and stop test of MixedState.  Rows t, t + B, ... of the
// system belong to thread t; RPP of them are in flight at a time.  The
// state of a step is written by the CTA's own threads in the previous step,
// so plain loads after the block barrier see it.
template <int RPP, int ND> __device__ void batch_solve_one(const BatchSys &S, const BatchArgs &a, BatchOut *out)
{
    __shared__ MixedState ms;
    const int n = S.n, B = blockDim.x;
    const double *sc = a.scale + S.row0;
    const double *b = a.b + S.row0;
    double *x = a.x + S.row0;
    float4 *st[2] = {a.st[0] + S.row0, a.st[1] + S.row0};
    const int32_t *rp = a.rowPtr + S.rp0;
    const int32_t *ci = a.colIdx + S.nz0;
    const double *va = a.values + S.nz0;

    // init: x = 0, state[1] = (S b, 0, 0, 0); |S b|^2, |b|^2
    {
        FF f[1] = {ff_zero()};
        double bb[1] = {0.0};
        for (int i = threadIdx.x; i < n; i += B) {
            const double bi = b[i];
            const float r = static_cast<float>(bi * sc[i]);
            x[i] = 0.0;
            st[1][i] = make_float4(r, 0.0f, 0.0f, 0.0f);
            ff_dot_add(f[0], r, r);
            bb[0] += bi * bi;
        }
        ff_block_allsum<1>(f);
        block_sum<1>(bb);  // thread 0
        if (threadIdx.x == 0)
            ms.start(ff_double(f[0]), bb[0], a.tol, a.maxit);
        __syncthreads();
    }
    const int64_t trip_cap = 2 * static_cast<int64_t>(a.maxit > 0 ? a.maxit : 0) + 16;
    const float tolf = static_cast<float>(a.tol), deltaf = static_cast<float>(a.delta);
    for (int64_t trips = 0; !ms.done; ++trips) {
        if (trips > trip_cap) {  // unreachable: every normal step counts and max_iter ends the solve
            __syncthreads();
            if (threadIdx.x == 0)
                ms.stop(SIMALL_ERR_TIMEOUT);
            __syncthreads();
            break;
        }
        const int par = ms.par;
        const float alpha = ms.fresh ? 0.0f : ms.alpha_f, beta = ms.beta_f;
        const float4 *in = st[par];
        float4 *outp = st[1 - par];
        FF acc[4] = {ff_zero(), ff_zero(), ff_zero(), ff_zero()};
        for (int i0 = threadIdx.x; i0 < n; i0 += RPP * B) {
            float4 o[RPP];
#pragma unroll
            for (int u = 0; u < RPP; ++u) {
                const int i = i0 + u * B;
                o[u] = i < n ? in[i] : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            }
#pragma unroll
            for (int u = 0; u < RPP; ++u) {
                const int i = i0 + u * B;
                if (i < n) {
                    const RowStep rs(o[u], alpha, beta);
                    rs.finish(batch_row<ND>(S, a, in, i, rs.p, alpha, beta), outp + i, acc);
                }
            }
        }
        ff_block_finish<4>(acc, [&](const FF (&t)[4]) { ms.finish_step(t, tolf, deltaf, a.maxit); });
        if (!ms.update)
            continue;
        // reliable update: x += S xh with the xh the triggering step wrote
        const int upar = ms.par;
        for (int i = threadIdx.x; i < n; i += B)
            x[i] += sc[i] * static_cast<double>(st[1 - upar][i].w);
        __syncthreads();
        // r = b - A x (FP64, one FMA per entry); the FP32 replacement S r and
        // xh = 0 into the state the FRESH step reads; |r|^2, |S r|^2
        double r2[2] = {0.0, 0.0};
        for (int i = threadIdx.x; i < n; i += B) {
            double y = 0.0;
            for (int k = rp[i]; k < rp[i + 1]; ++k)
                y = __fma_rn(va[k], x[ci[k]], y);
            const double v = b[i] - y;
            const float f = static_cast<float>(sc[i] * v);
            float *e = reinterpret_cast<float *>(st[upar] + i);
            e[0] = f;
            e[3] = 0.0f;
            r2[0] += v * v;
            r2[1] += static_cast<double>(f) * static_cast<double>(f);
        }
        block_sum<2>(r2);  // thread 0
        if (threadIdx.x == 0)
            ms.finish_update(r2, a.tol, a.maxit);
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        out->iterations = ms.iter;
        out->updates = ms.updates;
        out->status = ms.status;
        out->converged = ms.last < a.tol ? 1 : 0;
        out->true_residual = ms.last;
        out->b_norm = ms.b_norm;
    }
    __syncthreads();
}

template <int RPP> __global__ void __launch_bounds__(1024) k_batch_solve(BatchArgs a)
{
    __shared__ int s_next;
    for (;;) {
        if (threadIdx.x == 0)
            s_next = atomicAdd(a.queue, 1);
        __syncthreads();
        const int k = s_next;
        __syncthreads();
        if (k >= a.nsys)
            return;
        const int id = a.order[k];
        const BatchSys S = a.sys[id];
        switch (S.nd) {  // the stored diagonals, fixed at compile time in the step
        case 1: batch_solve_one<RPP, 1>(S, a, a.out + id); break;
        case 2: batch_solve_one<RPP, 2>(S, a, a.out + id); break;
        case 3: batch_solve_one<RPP, 3>(S, a, a.out + id); break;
        case 4: batch_solve_one<RPP, 4>(S, a, a.out + id); break;
        default: batch_solve_one<RPP, 0>(S, a, a.out + id); break;
        }
    }
}

}  // namespace

namespace {

// Which systems go to clusters: diagonal storage, at least `rows` rows and at
// most ctas x 8192, and an iteration limit the cluster engine accepts; the
// others keep the one-CTA queue (largest first).  rows == 0: none.
int plan_batch(simall_batch *B, int rows, int ctas)
{
    simall_context *ctx = B->ctx;
    if (B->plan_rows == rows && B->plan_ctas == ctas)
        return SIMALL_OK;
    std::vector<int> small;
    for (auto &v : B->h_items)
        v.clear();
    for (int id : B->h_order) {
        const BatchSys &S = B->h_sys[id];
        const bool big = rows > 0 && ctas > 0 && S.nd >= 1 && S.n >= rows &&
                         static_cast<int64_t>(S.n) <= static_cast<int64_t>(ctas) * kClBatchMaxRowsPerCta &&
                         B->cfg.max_iterations <= 200000;
        if (!big) {
            small.push_back(id);
            continue;
        }
        ClBatchItem it{};
        it.n = S.n;
        it.row0 = S.row0;
        it.A.U = B->U.p + S.u0;
        it.A.ldU = S.n;
        it.A.nd = S.nd;
        for (int d = 0; d < 8; ++d)
            it.A.off[d] = d < S.nd ? S.off[d] : 0;
        it.A.e = B->e.p + S.row0;
        it.A.scale = B->scale.p + S.row0;
        it.rowPtr = B->rowPtr.p + S.rp0;
        it.colIdx = B->colIdx.p + S.nz0;
        it.val = B->values.p + S.nz0;
        it.out = B->out.p + id;
        B->h_items[S.nd].push_back(it);
    }
    B->ncluster = 0;
    for (int nd = 1; nd <= 4; ++nd) {
        auto &v = B->h_items[nd];
        if (v.empty())
            continue;
        int lr = 8;  // the slice of the launch: the largest system on `ctas` CTAs
        int nmax = 0;
        for (const ClBatchItem &it : v)
            nmax = std::max(nmax, it.n);
        while ((static_cast<int64_t>(ctas) << lr) < nmax)
            ++lr;
        B->items_logR[nd] = lr;
        for (ClBatchItem &it : v)
            it.logR = lr;
        SIMALL_CUDA_TRY(ctx, B->items[nd].alloc(v.size()));
        SIMALL_CUDA_TRY(ctx, cudaMemcpyAsync(B->items[nd].p, v.data(), v.size() * sizeof(ClBatchItem),
                                             cudaMemcpyHostToDevice, ctx->stream));
        B->ncluster += static_cast<int>(v.size());
    }
    B->nsmall = static_cast<int>(small.size());
    if (!small.empty())
        SIMALL_CUDA_TRY(ctx, cudaMemcpyAsync(B->order.p, small.data(), small.size() * sizeof(int),
                                             cudaMemcpyHostToDevice, ctx->stream));
    SIMALL_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));  // the host lists are reused
    B->plan_rows = rows;
    B->plan_ctas = ctas;
    return SIMALL_OK;
}

int launch_batch(simall_batch *B, int block, int ctas_per_sm, int rpp, int reserved_sms, const double *b, double *x)
{
    simall_context *ctx = B->ctx;
    if (B->nsmall == 0)
        return SIMALL_OK;
    SIMALL_CUDA_TRY(ctx, cudaMemsetAsync(B->queue.p, 0, sizeof(int), ctx->stream));
    // the SMs the clusters hold are left to them
    const int sms = std::max(1, ctx->num_sms - reserved_sms);
    const int grid = std::max(1, std::min(B->nsmall, sms * ctas_per_sm));
    BatchArgs a{};
    a.sys = B->sys.p;
    a.order = B->order.p;
    a.nsys = B->nsmall;
    a.queue = B->queue.p;
    a.rowPtr = B->rowPtr.p;
    a.colIdx = B->colIdx.p;
    a.values = B->values.p;
    a.U = B->U.p;
    a.orow = B->orow.p;
    a.ocol = B->ocol.p;
    a.oval = B->oval.p;
    a.e = B->e.p;
    a.scale = B->scale.p;
    a.b = b;
    a.x = x;
    a.st[0] = B->st[0].p;
    a.st[1] = B->st[1].p;
    a.tol = B->cfg.tolerance;
    a.delta = B->cfg.reliable_delta;
    a.maxit = B->cfg.max_iterations;
    a.out = B->out.p;
    if (rpp >= 4)
        k_batch_solve<4><<<grid, block, 0, ctx->stream>>>(a);
    else if (rpp == 2)
        k_batch_solve<2><<<grid, block, 0, ctx->stream>>>(a);
    else
        k_batch_solve<1><<<grid, block, 0, ctx->stream>>>(a);
    ctx->launches.fetch_add(1, std::memory_order_relaxed);
    B->kernel_launches += 1;
    SIMALL_CUDA_TRY(ctx, cudaGetLastError());
    return SIMALL_OK;
}

// The whole batch: the cluster systems on the side stream, `clusters`
// clusters of cctas CTAs striding through them, the rest on the context's
// stream on the other SMs (a one-CTA-queue CTA of 1024 threads fills an SM's
// registers, so the two never share an SM), joined before returning.
// Capturable.
int launch_all(simall_batch *B, int block, int ctas_per_sm, int rpp, int crows, int cctas, int clusters,
               const double *b, double *x)
{
    simall_context *ctx = B->ctx;
    int st = plan_batch(B, crows, cctas);
    if (st)
        return st;
    if (B->ncluster > 0) {
        if (!B->side) {
            SIMALL_CUDA_TRY(ctx, cudaStreamCreateWithFlags(&B->side, cudaStreamNonBlocking));
            SIMALL_CUDA_TRY(ctx, cudaEventCreateWithFlags(&B->ev_fork, cudaEventDisableTiming));
            SIMALL_CUDA_TRY(ctx, cudaEventCreateWithFlags(&B->ev_join, cudaEventDisableTiming));
        }
        SIMALL_CUDA_TRY(ctx, cudaEventRecord(B->ev_fork, ctx->stream));
        SIMALL_CUDA_TRY(ctx, cudaStreamWaitEvent(B->side, B->ev_fork, 0));
        for (int nd = 1; nd <= 4; ++nd) {
            const int cnt = static_cast<int>(B->h_items[nd].size());
            if (cnt == 0)
                continue;
            st = cluster_mixed_batch(ctx, B->side, nd, cctas, B->items_logR[nd], std::max(1, clusters),
                                     B->items[nd].p, cnt, b, x, B->cfg.tolerance, B->cfg.reliable_delta,
                                     B->cfg.max_iterations);
            if (st)
                return st;
            B->kernel_launches += 1;
        }
        SIMALL_CUDA_TRY(ctx, cudaEventRecord(B->ev_join, B->side));
    }
    st = launch_batch(B, block, ctas_per_sm, rpp, B->ncluster > 0 ? std::max(1, clusters) * cctas : 0, b, x);
    if (st)
        return st;
    if (B->ncluster > 0)
        SIMALL_CUDA_TRY(ctx, cudaStreamWaitEvent(ctx->stream, B->ev_join, 0));
    return SIMALL_OK;
}

// Times each launch shape -- threads per CTA, CTAs per SM, rows a thread
// keeps in flight -- on the batch itself (device b -> scratch x) and keeps
// the fastest; the choice is stored in the autotuner cache under the batch's
// key, so the next process with the same batch shape on the same device
// skips the timing.
int autotune(simall_batch *B, const double *b)
{
    simall_context *ctx = B->ctx;
    int cached[6] = {0, 0, 0, 0, 0, 0};
    if (!B->cache_path.empty() &&
        simall_autotune_cache_lookup(B->cache_path.c_str(), B->shape_key.c_str(), cached) == SIMALL_OK &&
        (cached[0] == 256 || cached[0] == 512 || cached[0] == 1024) && cached[1] >= 1 && cached[1] <= 8 &&
        (cached[2] == 1 || cached[2] == 2 || cached[2] == 4) && cached[0] * cached[1] <= 2048 && cached[3] >= 0 &&
        cached[4] >= 0 && cached[4] <= 16 && cached[5] >= 0) {
        B->block = cached[0];
        B->ctas_per_sm = cached[1];
        B->rows_per_pass = cached[2];
        B->cluster_rows = cached[3];
        B->cluster_ctas = cached[4];
        B->clusters = cached[5];
        B->tune_source = 2;
        return SIMALL_OK;
    }
    cudaEvent_t e0, e1;
    SIMALL_CUDA_TRY(ctx, cudaEventCreate(&e0));
    SIMALL_CUDA_TRY(ctx, cudaEventCreate(&e1));
    float best = 1e30f;
    auto trial = [&](int blk, int cps, int rpp, int crows, int cctas, int ncl) -> int {
        SIMALL_CUDA_TRY(ctx, cudaEventRecord(e0, ctx->stream));
        int st = launch_all(B, blk, cps, rpp, crows, cctas, ncl, b, B->x.p);
        if (st == SIMALL_ERR_UNSUPPORTED && crows > 0) {  // this cluster shape does not fit here
            cudaGetLastError();
            return SIMALL_OK;
        }
        if (st)
            return st;
        SIMALL_CUDA_TRY(ctx, cudaEventRecord(e1, ctx->stream));
        SIMALL_CUDA_TRY(ctx, cudaEventSynchronize(e1));
        float ms = 0.0f;
        cudaEventElapsedTime(&ms, e0, e1);
        if (ms < best) {
            best = ms;
            B->block = blk;
            B->ctas_per_sm = cps;
            B->rows_per_pass = rpp;
            B->cluster_rows = crows;
            B->cluster_ctas = cctas;
            B->clusters = ncl;
        }
        return SIMALL_OK;
    };
    // 1: the one-CTA shape with every system on the queue
    const int shapes[][3] = {{1024, 1, 1}, {1024, 1, 2}, {1024, 1, 4}, {512, 2, 1}, {512, 2, 2},
                             {256, 4, 1},  {256, 4, 2},  {512, 1, 2},  {512, 1, 4}};
    for (const auto &sh : shapes) {
        const int st = trial(sh[0], sh[1], sh[2], 0, 0, 0);
        if (st)
            return st;
    }
    // 2: with that shape, the largest systems on clusters (row threshold,
    // cluster size, SMs the clusters hold -- the rest run the one-CTA queue)
    const int blk = B->block, cps = B->ctas_per_sm, rpp = B->rows_per_pass;
    int64_t nmax = 0;
    for (const BatchSys &S : B->h_sys)
        nmax = std::max<int64_t>(nmax, S.nd >= 1 ? S.n : 0);
    // (rows, cluster CTAs, clusters); on the 512-system cavity batch of
    // sides 32-256 the first takes 0.098 s against 0.188 s for the queue alone,
    // and more clusters than these lose: 16-CTA clusters are placed a GPC
    // at a time and wait for one another, and every SM a cluster holds is
    // one the queue, which streams a system at a third of the SM-time a
    // cluster spends on it, does not have
    const int routes[][3] = {{49152, 16, 4}, {49152, 16, 3}, {49152, 16, 5}, {57344, 16, 3}, {49152, 8, 8},
                             {57344, 8, 6},  {40960, 16, 5}, {40960, 16, 4}, {40960, 16, 6}, {32768, 16, 5},
                             {40960, 8, 10}, {40960, 8, 12}, {32768, 8, 12}, {16384, 4, 16}};
    for (const auto &r : routes) {
        if (nmax < r[0] || r[1] * r[2] >= ctx->num_sms)
            continue;
        const int st = trial(blk, cps, rpp, r[0], r[1], r[2]);
        if (st)
            return st;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    B->tune_source = 1;
    if (!B->cache_path.empty()) {
        const int v[6] = {B->block, B->ctas_per_sm, B->rows_per_pass, B->cluster_rows, B->cluster_ctas, B->clusters};
        simall_autotune_cache_store(B->cache_path.c_str(), B->shape_key.c_str(), v, best);  // best effort
    }
    return SIMALL_OK;
}

// The batch's key in the autotuner cache: device, SM count, kernel revision,
// and an FNV-1a hash of every system's rows, nonzeros and storage.
std::string batch_shape_key(simall_batch *B)
{
    cudaDeviceProp prop{};
    cudaGetDeviceProperties(&prop, B->ctx->device);
    uint64_t h = 1469598103934665603ull;
    auto mix = [&](uint64_t v) {
        for (int k = 0; k < 8; ++k) {
            h ^= (v >> (8 * k)) & 0xffu;
            h *= 1099511628211ull;
        }
    };
    for (const BatchSys &S : B->h_sys) {
        mix(static_cast<uint64_t>(S.n));
        mix(static_cast<uint64_t>(S.nd));
    }
    mix(static_cast<uint64_t>(B->nnz));
    std::string name = prop.name;
    for (char &c : name)
        if (c == '"' || c == '\\' || static_cast<unsigned char>(c) < 32)
            c = '_';
    char buf[256];
    snprintf(buf, sizeof buf, "batch-fused-v5|%s|sm%d|n%d|rows%lld|%016llx", name.c_str(), B->ctx->num_sms, B->nsys,
             static_cast<long long>(B->rows), static_cast<unsigned long long>(h));
    return buf;
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
    B->cache_path = default_autotune_cache_path();
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
    std::vector<float> U, e(static_cast<size_t>(rows));
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
        // e_i = 1 + sum_{j != i} a_ij s_i s_j in FP64, rounded once (the row-sum form)
        for (int64_t i = 0; i < n; ++i) {
            double sum = 1.0;
            for (int k = rp[i]; k < rp[i + 1]; ++k)
                if (ci[k] != i)
                    sum += va[k] * sc[i] * sc[ci[k]];
            e[r0 + i] = static_cast<float>(sum);
        }
        if (dia) {
            std::sort(offs.begin(), offs.end());
            S.nd = static_cast<int>(offs.size());
            for (int d = 0; d < kBatchDiags; ++d)
                S.off[d] = d < S.nd ? offs[d] : 0;
            S.u0 = static_cast<int64_t>(U.size());
            S.orp0 = 0;
            U.resize(U.size() + static_cast<size_t>(S.nd) * n, 0.0f);
            float *Us = U.data() + S.u0;
            for (int64_t i = 0; i < n; ++i)
                for (int k = rp[i]; k < rp[i + 1]; ++k) {
                    const int j = ci[k];
                    if (j <= i)
                        continue;
                    const int d = static_cast<int>(std::find(offs.begin(), offs.end(), j - static_cast<int>(i)) -
                                                   offs.begin());
                    Us[static_cast<int64_t>(d) * n + i] = static_cast<float>(va[k] * sc[i] * sc[j]);
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
                        ocol.push_back(ci[k]);
                        oval.push_back(static_cast<float>(va[k] * sc[i] * sc[ci[k]]));
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
    SIMALL_CUDA_TRY(ctx, B->e.alloc(rows));
    SIMALL_CUDA_TRY(ctx, B->st[0].alloc(rows));
    SIMALL_CUDA_TRY(ctx, B->st[1].alloc(rows));
    SIMALL_CUDA_TRY(ctx, B->U.alloc(std::max<size_t>(U.size(), 1)));
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
    SIMALL_CUDA_TRY(ctx, up(B->e.p, e.data(), e.size() * sizeof(float)));
    if (!U.empty())
        SIMALL_CUDA_TRY(ctx, up(B->U.p, U.data(), U.size() * sizeof(float)));
    if (!orow.empty()) {
        SIMALL_CUDA_TRY(ctx, up(B->orow.p, orow.data(), orow.size() * sizeof(int32_t)));
        if (!ocol.empty()) {
            SIMALL_CUDA_TRY(ctx, up(B->ocol.p, ocol.data(), ocol.size() * sizeof(int32_t)));
            SIMALL_CUDA_TRY(ctx, up(B->oval.p, oval.data(), oval.size() * sizeof(float)));
        }
    }
    SIMALL_CUDA_TRY(ctx, cudaStreamSynchronize(st));  // host staging vectors die here
    B->nsys = n_systems;
    B->rows = rows;
    B->nnz = nnz;
    B->h_sys = std::move(sys);
    B->h_order = std::move(order);
    B->h_out.assign(static_cast<size_t>(n_systems), BatchOut{});
    B->block = 0;  // re-tune for the new batch (or read the cache)
    B->cluster_rows = 0;
    B->cluster_ctas = 0;
    B->clusters = 0;
    B->plan_rows = B->plan_ctas = -1;
    B->shape_key = batch_shape_key(B);
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
    // the plan is made outside the capture (it uploads the item lists)
    int pst = plan_batch(B, B->cluster_rows, B->cluster_ctas);
    if (pst)
        return pst;
    if (!B->gexec || B->g_b != db || B->g_x != dx || B->g_block != B->block || B->g_ctas != B->ctas_per_sm ||
        B->g_rpp != B->rows_per_pass || B->g_crows != B->cluster_rows || B->g_cctas != B->cluster_ctas ||
        B->g_clusters != B->clusters) {
        if (B->gexec) {
            cudaGraphExecDestroy(B->gexec);
            B->gexec = nullptr;
        }
        cudaGraph_t graph = nullptr;
        SIMALL_CUDA_TRY(ctx, cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
        const int st =
            launch_all(B, B->block, B->ctas_per_sm, B->rows_per_pass, B->cluster_rows, B->cluster_ctas, B->clusters, db,
                       dx);
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
        B->g_rpp = B->rows_per_pass;
        B->g_crows = B->cluster_rows;
        B->g_cctas = B->cluster_ctas;
        B->g_clusters = B->clusters;
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
        total->rows_per_pass = B->rows_per_pass;
        total->autotune_source = B->tune_source;
        total->cluster_rows = B->cluster_rows;
        total->cluster_ctas = B->cluster_ctas;
        total->cluster_systems = B->ncluster;
        total->clusters = B->clusters;
        total->seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    }
    return SIMALL_OK;
}

int simall_batch_launch_shape(simall_batch *B, int block_threads, int ctas_per_sm)
{
    if (!B || (block_threads != 0 && block_threads != 256 && block_threads != 512 && block_threads != 1024) ||
        ctas_per_sm < 0 || ctas_per_sm > 8)
        return SIMALL_ERR_INVALID_ARGUMENT;
    if (block_threads && block_threads * ctas_per_sm > 2048)
        return SIMALL_ERR_INVALID_ARGUMENT;
    B->block = block_threads;
    B->ctas_per_sm = block_threads ? ctas_per_sm : 0;
    B->rows_per_pass = block_threads ? 2 : 0;
    B->cluster_rows = 0;  // a fixed shape keeps every system on the one-CTA queue
    B->cluster_ctas = 0;
    B->clusters = 0;
    B->tune_source = 0;
    return SIMALL_OK;
}

int simall_batch_cluster_route(simall_batch *B, int cluster_rows, int cluster_ctas, int clusters)
{
    if (!B || cluster_rows < 0 || (cluster_rows > 0 && (cluster_ctas < 1 || cluster_ctas > 16 || clusters < 1)))
        return SIMALL_ERR_INVALID_ARGUMENT;
    if (B->block == 0) {  // a fixed shape for the one-CTA queue as well
        B->block = 1024;
        B->ctas_per_sm = 1;
        B->rows_per_pass = 2;
    }
    B->cluster_rows = cluster_rows;
    B->cluster_ctas = cluster_rows > 0 ? cluster_ctas : 0;
    B->clusters = cluster_rows > 0 ? clusters : 0;
    B->tune_source = 0;
    return SIMALL_OK;
}

int simall_batch_autotune_cache(simall_batch *B, const char *path)
{
    if (!B)
        return SIMALL_ERR_INVALID_ARGUMENT;
    B->cache_path = path ? path : "";
    return SIMALL_OK;
}

}  // extern "C"
