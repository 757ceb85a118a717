// The AMG preconditioner on the device: AMGPreconditioner::apply
// (src/solver/AMGPreconditioner.cpp:379-427), one V-cycle from z = 0 with one
// symmetric Gauss-Seidel sweep before and after the coarse correction and a
// dense LU solve on the coarsest level.  The hierarchy is built on the host
// (amg_host.cpp) once per matrix and kept in device memory.
//
// Gauss-Seidel is sequential by definition: row i reads the new values of
// the rows before it and the old values of the rows after it (forward; the
// other way round backward).  Each sweep here writes a second buffer, so the
// old values stay readable.  Levels of more than 4,096 rows take their rows
// in dependency-level order from a ticket, each row polling (bounded) the new
// values it reads until they land; smaller levels (the dense
// coarse operators) run in one CTA, dependency level after dependency level,
// the new values in shared memory.  Every row does the reference's operations
// in its column order, products and differences rounded separately and the
// division correctly rounded.  Residual, restriction and prolongation are row sums in
// column order.  The whole apply is bit-identical to the reference's.
//
// Per level above the coarsest: forward sweep x -> t (the pre-smoothing starts
// from x = 0, so it reads no x), backward sweep t -> x, r = b - A x into t,
// b_c = R t; on the way back x += P x_c, forward and backward sweeps.
#include "amg.hpp"
#include "device.cuh"
#include "solver.hpp"
#include "sweep.cuh"

#include <memory>
#include <new>

namespace simall {

struct AmgLevelDev {
    int32_t n = 0, nnz = 0;
    const int32_t *rp = nullptr, *ci = nullptr;  // level 0: the solver's own arrays
    const double *v = nullptr;
    DevBuf<int32_t> rpB, ciB;
    DevBuf<double> vB;
    DevBuf<int32_t> Prp, Pci, Rrp, Rci;  // to the next level
    DevBuf<double> Pv, Rv;
    int32_t nc = 0;
    DevBuf<int32_t> fwdOrder, bwdOrder;  // rows in forward / backward dependency-level order
    DevBuf<int32_t> fwdLvl, bwdLvl;      // level boundaries into the orders (single-CTA sweeps)
    int nlevF = 0, nlevB = 0, smallThreads = 0;
    bool small = false;                  // sweeps in one CTA, the new values in shared memory
    DevBuf<unsigned> ctl;  // free-running sweeps: [0] ticket, [2] timeout flag
    DevBuf<double> x, b, t;  // x, b: levels below the fine one; t: every level
};

struct AmgData {
    std::vector<std::unique_ptr<AmgLevelDev>> lv;
    int nlev = 0;
    int32_t coarseN = 0;
    DevBuf<double> lu, y;
};

namespace {

// One Gauss-Seidel sweep over the rows in `order`.  Forward (BWD false): row i
// reads xout_j (this sweep's values, j < i, polled until they land; xout holds
// kPending before) and xin_j (j > i; ZERO: 0) and writes xout_i = (b_i -
// sum_{j != i} a_ij x_j) / a_ii, or keeps xin_i when |a_ii| <= 1e-30.
// Backward: the same with j > i from xout.
template <bool BWD, bool ZERO>
__global__ void __launch_bounds__(kBlock) k_sgs_free(int n, const int32_t *__restrict__ order,
                                                     const int32_t *__restrict__ rp, const int32_t *__restrict__ ci,
                                                     const double *__restrict__ a, const double *__restrict__ b,
                                                     const double *__restrict__ xin, double *xout, unsigned *ctl,
                                                     unsigned backoff)
{
    const int lane = threadIdx.x & 31;
    bool ok = true;
    for (;;) {
        int base = 0;
        if (lane == 0)
            base = static_cast<int>(atomicAdd(ctl, 32u));
        base = __shfl_sync(0xffffffffu, base, 0);
        if (base >= n)
            break;
        const int t = base + lane;
        if (t < n) {
            const int i = __ldg(order + t);
            double s = __ldg(b + i), aii = 0.0;
            const int end = __ldg(rp + i + 1);
            for (int kp = __ldg(rp + i); kp < end; kp += 4) {
                int j[4];
                bool dep[4];
                double av[4];
#pragma unroll
                for (int q = 0; q < 4; ++q) {
                    const bool in = kp + q < end;
                    j[q] = in ? __ldg(ci + kp + q) : i;  // padding reads as the diagonal: no value, no wait
                    av[q] = in ? __ldg(a + kp + q) : 0.0;
                    dep[q] = BWD ? j[q] > i : j[q] < i;
                }
                double v[4];
                ok = wait_values4(xout, j, dep, v, backoff) && ok;
#pragma unroll
                for (int q = 0; q < 4; ++q)
                    if (!dep[q])
                        v[q] = j[q] == i ? 0.0 : ZERO ? 0.0 : __ldg(xin + j[q]);
#pragma unroll
                for (int q = 0; q < 4; ++q) {
                    if (kp + q >= end)
                        break;
                    if (j[q] == i)
                        aii = av[q];
                    else
                        s = __dsub_rn(s, __dmul_rn(av[q], v[q]));
                }
            }
            const double keep = ZERO ? 0.0 : __ldg(xin + i);
            st_value(xout + i, fabs(aii) > 1e-30 ? __ddiv_rn(s, aii) : keep);
        }
    }
    if (!ok)
        atomicOr(ctl + 2, 1u);
}

// Levels of up to this many rows sweep in one CTA (new values in 32 KB of
// shared memory).  At 64^3 the V-cycle took 158 / 138 / 146 / 177 ms with the
// bound at 24,576 / 4,096 / 2,048 / 512 rows: the free-running sweep is the
// faster one on the sparse-ish upper levels, the one-CTA sweep on the dense
// coarse ones.
constexpr int kSgsSmallRows = 4096;
constexpr int kSgsSmallThreads = 1024;

// The same sweep in one CTA for levels of up to kSgsSmallRows rows: the
// dependency levels one after the other with a block barrier between them,
// this sweep's new values in shared memory, one warp per row.  Coarse AMG
// operators are dense enough (hundreds of entries per row) that their
// dependency chains are nearly as long as their row counts, so the time per
// row is what counts: the lanes load a row's entries and form its products
// a_ij x_j (each rounded) together, then every lane runs the reference's
// ordered chain of subtractions over the broadcast products.  The diagonal's
// product enters the chain as +0.0, which leaves every value unchanged, as
// skipping it does.
template <bool BWD, bool ZERO>
__global__ void __launch_bounds__(kSgsSmallThreads) k_sgs_small(int n, int nlev, const int32_t *__restrict__ lvl,
                                                                const int32_t *__restrict__ order,
                                                                const int32_t *__restrict__ rp,
                                                                const int32_t *__restrict__ ci,
                                                                const double *__restrict__ a,
                                                                const double *__restrict__ b,
                                                                const double *__restrict__ xin,
                                                                double *__restrict__ xout)
{
    extern __shared__ double xs[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
    for (int l = 0; l < nlev; ++l) {
        const int t1 = __ldg(lvl + l + 1);
        for (int t = __ldg(lvl + l) + warp; t < t1; t += nwarps) {
            const int i = __ldg(order + t);
            double s = __ldg(b + i), aii = 0.0;
            const int beg = __ldg(rp + i), end = __ldg(rp + i + 1);
            for (int k0 = beg; k0 < end; k0 += 32) {
                const int k = k0 + lane;
                double p = 0.0;
                if (k < end) {
                    const int j = __ldg(ci + k);
                    const double av = __ldg(a + k);
                    if (j == i) {
                        aii = av;  // this lane's; shared below
                    } else {
                        const bool dep = BWD ? j > i : j < i;
                        const double xv = dep ? xs[j] : ZERO ? 0.0 : __ldg(xin + j);
                        p = __dmul_rn(av, xv);
                    }
                }
                const int cnt = end - k0 < 32 ? end - k0 : 32;
                for (int q = 0; q < cnt; ++q)
                    s = __dsub_rn(s, __shfl_sync(0xffffffffu, p, q));
            }
            // the diagonal value from whichever lane held it (at most one entry per column)
            for (int o = 16; o > 0; o >>= 1) {
                const double other = __shfl_xor_sync(0xffffffffu, aii, o);
                aii = aii != 0.0 ? aii : other;
            }
            if (lane == 0) {
                const double keep = ZERO ? 0.0 : __ldg(xin + i);
                xs[i] = fabs(aii) > 1e-30 ? __ddiv_rn(s, aii) : keep;
            }
        }
        __syncthreads();
    }
    for (int i = threadIdx.x; i < n; i += blockDim.x)
        xout[i] = xs[i];
}

// Row sum of a CSR row in column order from 0.0 (CSRMatrix::spmv,
// src/solver/CSRMatrix.hpp:24-35).
__device__ __forceinline__ double row_sum(const int32_t *__restrict__ rp, const int32_t *__restrict__ ci,
                                          const double *__restrict__ a, const double *__restrict__ x, int i)
{
    double s = 0.0;
    const int end = __ldg(rp + i + 1);
    for (int k = __ldg(rp + i); k < end; ++k)
        s = __dadd_rn(s, __dmul_rn(__ldg(a + k), __ldg(x + __ldg(ci + k))));
    return s;
}

// r = b - A x
__global__ void __launch_bounds__(kBlock) k_amg_residual(int n, const int32_t *__restrict__ rp,
                                                         const int32_t *__restrict__ ci, const double *__restrict__ a,
                                                         const double *__restrict__ x, const double *__restrict__ b,
                                                         double *__restrict__ r)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        r[i] = __dsub_rn(__ldg(b + i), row_sum(rp, ci, a, x, i));
}

// y = M x (restriction: the coarse right-hand side)
__global__ void __launch_bounds__(kBlock) k_amg_spmv(int n, const int32_t *__restrict__ rp,
                                                     const int32_t *__restrict__ ci, const double *__restrict__ a,
                                                     const double *__restrict__ x, double *__restrict__ y)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        y[i] = row_sum(rp, ci, a, x, i);
}

// x += P x_c
__global__ void __launch_bounds__(kBlock) k_amg_prolong(int n, const int32_t *__restrict__ rp,
                                                        const int32_t *__restrict__ ci, const double *__restrict__ a,
                                                        const double *__restrict__ xc, double *__restrict__ x)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        x[i] = __dadd_rn(x[i], row_sum(rp, ci, a, xc, i));
}

// The coarsest level: the reference's dense forward and back substitution
// (AMGPreconditioner::direct_solve, :354-377), one warp.  Forward: each row's
// sum takes y_0, y_1, ... in order as they become final, so the lanes advance
// all rows together; backward: each row's sum starts with x_{i+1}, a chain,
// so lane 0 runs it.
__global__ void k_amg_direct(int n, const double *__restrict__ lu, const double *__restrict__ b, double *y,
                             double *x)
{
    const int lane = threadIdx.x;
    for (int i = lane; i < n; i += 32)
        y[i] = b[i];
    __syncwarp();
    for (int j = 0; j < n; ++j) {
        const double yj = y[j];
        for (int i = j + 1 + lane; i < n; i += 32)
            y[i] = __dsub_rn(y[i], __dmul_rn(lu[static_cast<size_t>(i) * n + j], yj));
        __syncwarp();
    }
    if (lane == 0) {
        for (int i = n - 1; i >= 0; --i) {
            double s = y[i];
            const double *row = lu + static_cast<size_t>(i) * n;
            for (int j = i + 1; j < n; ++j)
                s = __dsub_rn(s, __dmul_rn(row[j], x[j]));
            const double d = row[i];
            x[i] = fabs(d) > 1e-30 ? __ddiv_rn(s, d) : 0.0;
        }
    }
}

// Rows ordered by dependency level; lower: row i waits for j < i, else j > i.
// ptr receives the level boundaries; returns the widest level.
int32_t level_order(const AmgCsr &A, bool lower, std::vector<int32_t> &order, std::vector<int32_t> &ptr)
{
    const int32_t n = A.n;
    std::vector<int32_t> lev(n, 0);
    int32_t nlev = 0;
    auto visit = [&](int32_t i) {
        int32_t l = 0;
        for (int32_t k = A.rp[i]; k < A.rp[i + 1]; ++k) {
            const int32_t j = A.ci[k];
            if (lower ? j < i : j > i)
                l = std::max(l, lev[j] + 1);
        }
        lev[i] = l;
        nlev = std::max(nlev, l + 1);
    };
    if (lower)
        for (int32_t i = 0; i < n; ++i)
            visit(i);
    else
        for (int32_t i = n - 1; i >= 0; --i)
            visit(i);
    ptr.assign(static_cast<size_t>(nlev) + 1, 0);
    for (int32_t i = 0; i < n; ++i)
        ++ptr[lev[i] + 1];
    int32_t widest = 0;
    for (int32_t l = 0; l < nlev; ++l) {
        widest = std::max(widest, ptr[l + 1]);
        ptr[l + 1] += ptr[l];
    }
    order.resize(n);
    std::vector<int32_t> fill(ptr.begin(), ptr.end() - 1);
    for (int32_t i = 0; i < n; ++i)
        order[fill[lev[i]]++] = i;
    return widest;
}

template <class T> cudaError_t upload(DevBuf<T> &dst, const std::vector<T> &src, cudaStream_t st)
{
    cudaError_t e = dst.alloc(src.size() ? src.size() : 1);
    if (e == cudaSuccess && !src.empty())
        e = cudaMemcpyAsync(dst.p, src.data(), src.size() * sizeof(T), cudaMemcpyHostToDevice, st);
    return e;
}

int grid_rows(simall_context *ctx, int64_t n)
{
    const int64_t g = (n + kBlock - 1) / kBlock;
    const int64_t cap = static_cast<int64_t>(ctx->num_sms) * 8;
    return static_cast<int>(g < 1 ? 1 : g < cap ? g : cap);
}

int grid_sweep(simall_context *ctx, int64_t n)
{
    // one warp takes 32 rows per ticket; at most 4 CTAs per SM are resident
    // with room to spare, so every row waited for is held by a running warp
    const int64_t g = (n + kBlock - 1) / kBlock;
    const int64_t cap = static_cast<int64_t>(ctx->num_sms) * 4;
    return static_cast<int>(g < 1 ? 1 : g < cap ? g : cap);
}

int sweep(simall_context *ctx, AmgLevelDev &L, bool backward, bool zero, const double *b, const double *xin,
          double *xout)
{
    if (L.small) {
        const size_t smem = static_cast<size_t>(L.n) * sizeof(double);
        const int nl = backward ? L.nlevB : L.nlevF;
        const int32_t *lvl = backward ? L.bwdLvl.p : L.fwdLvl.p, *order = backward ? L.bwdOrder.p : L.fwdOrder.p;
        if (backward)
            k_sgs_small<true, false><<<1, L.smallThreads, smem, ctx->stream>>>(L.n, nl, lvl, order, L.rp, L.ci, L.v,
                                                                                 b, xin, xout);
        else if (zero)
            k_sgs_small<false, true><<<1, L.smallThreads, smem, ctx->stream>>>(L.n, nl, lvl, order, L.rp, L.ci, L.v,
                                                                                 b, xin, xout);
        else
            k_sgs_small<false, false><<<1, L.smallThreads, smem, ctx->stream>>>(L.n, nl, lvl, order, L.rp, L.ci,
                                                                                  L.v, b, xin, xout);
        SIMALL_LAUNCH_CHECK(ctx);
        return SIMALL_OK;
    }
    k_sweep_begin_values<<<grid_rows(ctx, L.n), kBlock, 0, ctx->stream>>>(L.ctl.p, xout, L.n);
    SIMALL_LAUNCH_CHECK(ctx);
    const int g = grid_sweep(ctx, L.n);
    const int32_t *order = backward ? L.bwdOrder.p : L.fwdOrder.p;
    if (backward)
        k_sgs_free<true, false><<<g, kBlock, 0, ctx->stream>>>(L.n, order, L.rp, L.ci, L.v, b, xin, xout, L.ctl.p,
                                                      g_sweep_backoff_ns);
    else if (zero)
        k_sgs_free<false, true><<<g, kBlock, 0, ctx->stream>>>(L.n, order, L.rp, L.ci, L.v, b, xin, xout, L.ctl.p,
                                                      g_sweep_backoff_ns);
    else
        k_sgs_free<false, false><<<g, kBlock, 0, ctx->stream>>>(L.n, order, L.rp, L.ci, L.v, b, xin, xout, L.ctl.p,
                                                      g_sweep_backoff_ns);
    SIMALL_LAUNCH_CHECK(ctx);
    return SIMALL_OK;
}

}  // namespace

int amg_setup(simall_solver *s)
{
    simall_context *ctx = s->ctx;
    int hp = solver_host_pattern(s);
    if (hp)
        return hp;
    if (!s->amg) {
        s->amg = new (std::nothrow) AmgData;
        if (!s->amg)
            return fail(ctx, SIMALL_ERR_OUT_OF_MEMORY, "AMG state");
    }
    AmgData *d = s->amg;
    cudaStream_t st = ctx->stream;
    std::vector<double> vals(static_cast<size_t>(s->nnz));
    SIMALL_CUDA_TRY(ctx, cudaMemcpyAsync(vals.data(), s->values, vals.size() * sizeof(double), cudaMemcpyDeviceToHost,
                                         st));
    SIMALL_CUDA_TRY(ctx, cudaStreamSynchronize(st));
    AmgHierarchy h;
    amg_build_hierarchy(static_cast<int32_t>(s->n), s->h_rowPtr.data(), s->h_colIdx.data(), vals.data(), AmgParams{},
                        h);
    const int nlev = static_cast<int>(h.A.size());
    while (static_cast<int>(d->lv.size()) < nlev) {
        d->lv.emplace_back(new (std::nothrow) AmgLevelDev);
        if (!d->lv.back())
            return fail(ctx, SIMALL_ERR_OUT_OF_MEMORY, "AMG level");
    }
    d->nlev = nlev;
    std::vector<int32_t> ord;
    for (int l = 0; l < nlev; ++l) {
        AmgLevelDev &L = *d->lv[l];
        const AmgCsr &A = h.A[l];
        L.n = A.n;
        L.nnz = A.rp[A.n];
        if (l == 0) {
            L.rp = s->rowPtr;
            L.ci = s->colIdx;
            L.v = s->values;
        } else {
            SIMALL_CUDA_TRY(ctx, upload(L.rpB, A.rp, st));
            SIMALL_CUDA_TRY(ctx, upload(L.ciB, A.ci, st));
            SIMALL_CUDA_TRY(ctx, upload(L.vB, A.v, st));
            L.rp = L.rpB.p;
            L.ci = L.ciB.p;
            L.v = L.vB.p;
            SIMALL_CUDA_TRY(ctx, L.x.alloc(A.n));
            SIMALL_CUDA_TRY(ctx, L.b.alloc(A.n));
        }
        SIMALL_CUDA_TRY(ctx, L.t.alloc(A.n));
        if (l + 1 < nlev) {
            SIMALL_CUDA_TRY(ctx, upload(L.Prp, h.P[l].rp, st));
            SIMALL_CUDA_TRY(ctx, upload(L.Pci, h.P[l].ci, st));
            SIMALL_CUDA_TRY(ctx, upload(L.Pv, h.P[l].v, st));
            SIMALL_CUDA_TRY(ctx, upload(L.Rrp, h.R[l].rp, st));
            SIMALL_CUDA_TRY(ctx, upload(L.Rci, h.R[l].ci, st));
            SIMALL_CUDA_TRY(ctx, upload(L.Rv, h.R[l].v, st));
            L.nc = h.R[l].n;
            // only levels that are smoothed need the sweep schedules
            std::vector<int32_t> ordB, ptrF, ptrB;
            const int32_t wF = level_order(A, true, ord, ptrF);
            const int32_t wB = level_order(A, false, ordB, ptrB);
            SIMALL_CUDA_TRY(ctx, upload(L.fwdOrder, ord, st));
            SIMALL_CUDA_TRY(ctx, upload(L.bwdOrder, ordB, st));
            SIMALL_CUDA_TRY(ctx, upload(L.fwdLvl, ptrF, st));
            SIMALL_CUDA_TRY(ctx, upload(L.bwdLvl, ptrB, st));
            L.nlevF = static_cast<int>(ptrF.size()) - 1;
            L.nlevB = static_cast<int>(ptrB.size()) - 1;
            L.small = A.n <= kSgsSmallRows;
            // one warp per row of the widest level: every warp pays each level's barrier
            const int32_t w = std::max(wF, wB);
            L.smallThreads = std::min(kSgsSmallThreads, std::max(32, 32 * w));
            SIMALL_CUDA_TRY(ctx, cudaStreamSynchronize(st));  // the schedules die at the end of this block
            SIMALL_CUDA_TRY(ctx, L.ctl.alloc(4));
            SIMALL_CUDA_TRY(ctx, cudaMemsetAsync(L.ctl.p, 0, 4 * sizeof(unsigned), st));
        }
        // the host hierarchy dies at return: finish this level's copies first
        SIMALL_CUDA_TRY(ctx, cudaStreamSynchronize(st));
    }
    {
        const int smem = kSgsSmallRows * static_cast<int>(sizeof(double));
        SIMALL_CUDA_TRY(ctx, cudaFuncSetAttribute(k_sgs_small<false, true>,
                                                  cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
        SIMALL_CUDA_TRY(ctx, cudaFuncSetAttribute(k_sgs_small<false, false>,
                                                  cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
        SIMALL_CUDA_TRY(ctx, cudaFuncSetAttribute(k_sgs_small<true, false>,
                                                  cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
    }
    d->coarseN = h.coarseN;
    SIMALL_CUDA_TRY(ctx, upload(d->lu, h.lu, st));
    SIMALL_CUDA_TRY(ctx, d->y.alloc(h.coarseN > 0 ? h.coarseN : 1));
    SIMALL_CUDA_TRY(ctx, cudaStreamSynchronize(st));
    return SIMALL_OK;
}

int amg_apply(simall_solver *s, const double *r, double *z)
{
    simall_context *ctx = s->ctx;
    AmgData *d = s->amg;
    const int L = d->nlev;
    auto xb = [&](int l, const double **b, double **x) {
        *b = l == 0 ? r : d->lv[l]->b.p;
        *x = l == 0 ? z : d->lv[l]->x.p;
    };
    for (int l = 0; l + 1 < L; ++l) {
        AmgLevelDev &Lv = *d->lv[l];
        const double *b;
        double *x;
        xb(l, &b, &x);
        int e = sweep(ctx, Lv, false, true, b, nullptr, Lv.t.p);
        if (e)
            return e;
        e = sweep(ctx, Lv, true, false, b, Lv.t.p, x);
        if (e)
            return e;
        k_amg_residual<<<grid_rows(ctx, Lv.n), kBlock, 0, ctx->stream>>>(Lv.n, Lv.rp, Lv.ci, Lv.v, x, b, Lv.t.p);
        SIMALL_LAUNCH_CHECK(ctx);
        k_amg_spmv<<<grid_rows(ctx, Lv.nc), kBlock, 0, ctx->stream>>>(Lv.nc, Lv.Rrp.p, Lv.Rci.p, Lv.Rv.p, Lv.t.p,
                                                                      d->lv[l + 1]->b.p);
        SIMALL_LAUNCH_CHECK(ctx);
    }
    {
        const double *b;
        double *x;
        xb(L - 1, &b, &x);
        k_amg_direct<<<1, 32, 0, ctx->stream>>>(d->coarseN, d->lu.p, b, d->y.p, x);
        SIMALL_LAUNCH_CHECK(ctx);
    }
    for (int l = L - 2; l >= 0; --l) {
        AmgLevelDev &Lv = *d->lv[l];
        const double *b;
        double *x;
        xb(l, &b, &x);
        k_amg_prolong<<<grid_rows(ctx, Lv.n), kBlock, 0, ctx->stream>>>(Lv.n, Lv.Prp.p, Lv.Pci.p, Lv.Pv.p,
                                                                         d->lv[l + 1]->x.p, x);
        SIMALL_LAUNCH_CHECK(ctx);
        int e = sweep(ctx, Lv, false, false, b, x, Lv.t.p);
        if (e)
            return e;
        e = sweep(ctx, Lv, true, false, b, Lv.t.p, x);
        if (e)
            return e;
    }
    return SIMALL_OK;
}

int amg_apply_launches(const simall_solver *s)
{
    const AmgData *d = s->amg;
    if (!d)
        return 1;
    int k = 1;  // the coarsest level's solve
    for (int l = 0; l + 1 < d->nlev; ++l)
        k += d->lv[l]->small ? 7 : 11;  // 4 sweeps (+ 4 ticket resets), residual, restriction, prolongation
    return k;
}

int amg_check(simall_solver *s)
{
    simall_context *ctx = s->ctx;
    AmgData *d = s->amg;
    for (int l = 0; l + 1 < d->nlev; ++l) {
        unsigned h = 0;
        SIMALL_CUDA_TRY(ctx, cudaMemcpyAsync(&h, d->lv[l]->ctl.p + 2, sizeof(unsigned), cudaMemcpyDeviceToHost,
                                             ctx->stream));
        SIMALL_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
        if (h) {
            SIMALL_CUDA_TRY(ctx, cudaMemsetAsync(d->lv[l]->ctl.p + 2, 0, sizeof(unsigned), ctx->stream));
            return fail(ctx, SIMALL_ERR_CUDA, "AMG smoother: a row wait timed out on level %d", l);
        }
    }
    return SIMALL_OK;
}

int amg_levels(const simall_solver *s, int *nlev, int32_t *rows, int max_levels)
{
    const AmgData *d = s->amg;
    *nlev = d ? d->nlev : 0;
    for (int l = 0; d && l < d->nlev && l < max_levels; ++l)
        rows[l] = d->lv[l]->n;
    return SIMALL_OK;
}

void amg_free(simall_solver *s)
{
    delete s->amg;
    s->amg = nullptr;
}

}  // namespace simall
