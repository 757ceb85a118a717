// Level-scheduled ILU(0) on the device.
//
// ILU0Preconditioner::setup (src/solver/LinearSolvers.cpp:81-122) factors row
// i using only rows k < i of its own lower pattern, each already final, and
// the triangular sweeps of ILU0Preconditioner::apply (:123-151) have the same
// dependency structure.  Grouping rows into dependency levels (row i's level
// is one more than the deepest row it reads) lets every row of a level run in
// parallel while each row keeps the reference's exact sequence of operations:
// products and differences are rounded separately (__dmul_rn/__dsub_rn) and
// in column order, so the factor and both sweeps are bit-identical to the
// reference.  Multicolouring would be faster but changes the factor.
//
// Systems of up to kIluSmallRows rows factor and sweep in one CTA (below).
// Larger ones: the factorisation (once per solve) launches one kernel per
// level, and the sweeps (twice per PCG iteration) run as one kernel each
// without levels
// between launches: warps take 32 consecutive rows of the level order from an
// atomic ticket, and a row waits only for the rows it reads, each of which
// publishes its value and then its "done" mark (release) and is read after the
// mark (acquire).  Rows are handed out in level order, so every row waited for
// was handed to a warp that is already running; the wait is bounded and a
// timeout is reported (it never happens unless a row is never produced).
#include "device.cuh"
#include "solver.hpp"

#include <algorithm>
#include <chrono>
#include <new>

namespace simall {

namespace {

// One level of the IKJ factorisation, one thread per row.
__global__ void __launch_bounds__(kBlock) k_ilu_factor_level(const int32_t *__restrict__ rows, int cnt,
                                                             const int32_t *__restrict__ rowPtr,
                                                             const int32_t *__restrict__ colIdx,
                                                             const int32_t *__restrict__ diagPtr, double *lu)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= cnt)
        return;
    const int i = rows[t];
    const int end = rowPtr[i + 1];
    for (int kp = rowPtr[i]; kp < end; ++kp) {
        const int k = colIdx[kp];
        if (k >= i)
            break;
        const int dk = diagPtr[k];
        if (dk < 0)
            continue;
        const double piv = lu[dk];
        if (piv == 0.0)
            continue;
        const double m = __ddiv_rn(lu[kp], piv);
        lu[kp] = m;
        const int kend = rowPtr[k + 1];
        for (int jp = dk + 1; jp < kend; ++jp) {
            const int j = colIdx[jp];
            for (int qp = kp + 1; qp < end; ++qp) {
                const int c = colIdx[qp];
                if (c == j) {
                    lu[qp] = __dsub_rn(lu[qp], __dmul_rn(m, lu[jp]));
                    break;
                }
                if (c > j)
                    break;
            }
        }
    }
}

// Forward sweep of one level: y_i = r_i - sum_{j<i} l_ij y_j.
__global__ void __launch_bounds__(kBlock) k_ilu_fwd_level(const int32_t *__restrict__ rows, int cnt,
                                                          const int32_t *__restrict__ rowPtr,
                                                          const int32_t *__restrict__ colIdx,
                                                          const double *__restrict__ lu, const double *__restrict__ r,
                                                          double *y)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= cnt)
        return;
    const int i = rows[t];
    double s = r[i];
    for (int kp = rowPtr[i]; kp < rowPtr[i + 1]; ++kp) {
        const int j = colIdx[kp];
        if (j >= i)
            break;
        s = __dsub_rn(s, __dmul_rn(lu[kp], __ldcg(y + j)));
    }
    y[i] = s;
}

// Backward sweep of one level: z_i = (y_i - sum_{j>i} u_ij z_j) / u_ii.
__global__ void __launch_bounds__(kBlock) k_ilu_bwd_level(const int32_t *__restrict__ rows, int cnt,
                                                          const int32_t *__restrict__ rowPtr,
                                                          const int32_t *__restrict__ colIdx,
                                                          const int32_t *__restrict__ diagPtr,
                                                          const double *__restrict__ lu, const double *__restrict__ y,
                                                          double *z)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= cnt)
        return;
    const int i = rows[t];
    double s = y[i];
    const int kd = diagPtr[i];
    for (int kp = kd + 1; kp < rowPtr[i + 1]; ++kp)
        s = __dsub_rn(s, __dmul_rn(lu[kp], __ldcg(z + colIdx[kp])));
    z[i] = (kd >= 0 && lu[kd] != 0.0) ? __ddiv_rn(s, lu[kd]) : s;
}

__device__ __forceinline__ unsigned ld_acquire(const unsigned *p)
{
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ void st_release(unsigned *p, unsigned v)
{
    asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

constexpr unsigned kSweepMaxSpins = 1u << 20;  // ~0.5 s of polling: far beyond any dependency chain

// Wait until row j carries the current sweep's mark; false on timeout.  The
// first polls are immediate (the row is usually done or nearly so); later
// ones back off so that thousands of waiting warps do not flood L2 while the
// rows they wait for are being computed.
__device__ __forceinline__ bool wait_row(const unsigned *done, int j, unsigned sweep)
{
    unsigned ns = 16;
    for (unsigned spins = 0; ld_acquire(done + j) != sweep; ++spins) {
        if (spins >= kSweepMaxSpins)
            return false;
        if (spins >= 4) {
            __nanosleep(ns);
            ns = ns < 256 ? 2 * ns : 256;
        }
    }
    return true;
}

// Next sweep: reset the ticket, advance the sweep number.
__global__ void k_sweep_begin(unsigned *ctl)
{
    ctl[0] = 0u;
    ctl[1] += 1u;
}

// Waits for up to 4 rows at once (their marks polled together), so a row
// with several dependencies costs one memory round trip per poll, not one per
// dependency; false on timeout.
__device__ __forceinline__ bool wait_rows4(const unsigned *done, const int (&j)[4], int cnt, unsigned sweep)
{
    unsigned ns = 16;
    for (unsigned spins = 0;; ++spins) {
        bool all = true;
#pragma unroll
        for (int q = 0; q < 4; ++q)
            if (q < cnt)
                all = (ld_acquire(done + j[q]) == sweep) && all;
        if (all)
            return true;
        if (spins >= kSweepMaxSpins)
            return false;
        if (spins >= 4) {
            __nanosleep(ns);
            ns = ns < 256 ? 2 * ns : 256;
        }
    }
}

// Forward sweep y_i = r_i - sum_{j<i} l_ij y_j over rows in level order.
// Dependencies are taken four at a time: wait for the four marks, load the
// four values, then apply them in column order (the reference's order).
__global__ void __launch_bounds__(kBlock) k_ilu_fwd_free(int n, const int32_t *__restrict__ order,
                                                         const int32_t *__restrict__ rowPtr,
                                                         const int32_t *__restrict__ colIdx,
                                                         const double *__restrict__ lu, const double *__restrict__ r,
                                                         double *y, unsigned *done, unsigned *ctl)
{
    const int lane = threadIdx.x & 31;
    const unsigned sweep = __ldcg(ctl + 1);
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
            double s = __ldg(r + i);
            const int end = __ldg(rowPtr + i + 1);
            for (int kp = __ldg(rowPtr + i); kp < end;) {
                int j[4];
                double a[4];
                int cnt = 0;
#pragma unroll
                for (int q = 0; q < 4; ++q) {
                    const bool in = kp + q < end;
                    const int jj = in ? __ldg(colIdx + kp + q) : i;
                    a[q] = in ? __ldg(lu + kp + q) : 0.0;  // the row's own data: loaded before the wait
                    j[q] = jj < i ? jj : i;
                    cnt += (jj < i && cnt == q) ? 1 : 0;
                }
                if (cnt == 0)
                    break;
                ok = wait_rows4(done, j, cnt, sweep) && ok;
                double v[4];
#pragma unroll
                for (int q = 0; q < 4; ++q)
                    v[q] = q < cnt ? __ldcg(y + j[q]) : 0.0;
#pragma unroll
                for (int q = 0; q < 4; ++q)
                    if (q < cnt)
                        s = __dsub_rn(s, __dmul_rn(a[q], v[q]));
                kp += cnt;
                if (cnt < 4)
                    break;
            }
            __stcg(y + i, s);
            st_release(done + i, sweep);
        }
    }
    if (!ok)
        atomicOr(ctl + 2, 1u);
}

// Backward sweep z_i = (y_i - sum_{j>i} u_ij z_j) / u_ii over rows in level order.
__global__ void __launch_bounds__(kBlock) k_ilu_bwd_free(int n, const int32_t *__restrict__ order,
                                                         const int32_t *__restrict__ rowPtr,
                                                         const int32_t *__restrict__ colIdx,
                                                         const int32_t *__restrict__ diagPtr,
                                                         const double *__restrict__ lu, const double *__restrict__ y,
                                                         double *z, unsigned *done, unsigned *ctl)
{
    const int lane = threadIdx.x & 31;
    const unsigned sweep = __ldcg(ctl + 1);
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
            double s = __ldcg(y + i);
            const int kd = __ldg(diagPtr + i);
            const int end = __ldg(rowPtr + i + 1);
            for (int kp = kd + 1; kp < end;) {
                int j[4];
                double a[4];
                int cnt = 0;
#pragma unroll
                for (int q = 0; q < 4; ++q) {
                    const bool in = kp + q < end;
                    j[q] = in ? __ldg(colIdx + kp + q) : i;
                    a[q] = in ? __ldg(lu + kp + q) : 0.0;
                    cnt += in ? 1 : 0;
                }
                ok = wait_rows4(done, j, cnt, sweep) && ok;
                double v[4];
#pragma unroll
                for (int q = 0; q < 4; ++q)
                    v[q] = q < cnt ? __ldcg(z + j[q]) : 0.0;
#pragma unroll
                for (int q = 0; q < 4; ++q)
                    if (q < cnt)
                        s = __dsub_rn(s, __dmul_rn(a[q], v[q]));
                kp += cnt;
            }
            const double dv = kd >= 0 ? __ldg(lu + kd) : 0.0;
            __stcg(z + i, (kd >= 0 && dv != 0.0) ? __ddiv_rn(s, dv) : s);
            st_release(done + i, sweep);
        }
    }
    if (!ok)
        atomicOr(ctl + 2, 1u);
}

// ---------------------------------------------------------------- one CTA
// For small systems the dependency chain, not the bandwidth, sets the time:
// one kernel launch per level or a mark per row cost microseconds per level,
// while one CTA walking the levels with a block barrier between them pays a
// barrier and an L2 round trip.  The sweep vector lives in shared memory (the
// backward sweep overwrites y with z in place: row i reads y_i and the final
// z_j of rows in earlier backward levels only).  Same per-row operations, so
// the results are bit-identical to the reference's.
constexpr int kIluSmallThreads = 1024;
constexpr int kIluSmallRows = 24576;  // 192 KB of shared memory

__global__ void __launch_bounds__(kIluSmallThreads) k_ilu_factor_small(int nlev, const int32_t *__restrict__ lvl,
                                                                       const int32_t *__restrict__ rows,
                                                                       const int32_t *__restrict__ rowPtr,
                                                                       const int32_t *__restrict__ colIdx,
                                                                       const int32_t *__restrict__ diagPtr, double *lu)
{
    for (int l = 1; l < nlev; ++l) {  // level 0 rows have no lower entries
        const int a = lvl[l], b = lvl[l + 1];
        for (int t = a + threadIdx.x; t < b; t += blockDim.x) {
            const int i = rows[t];
            const int end = rowPtr[i + 1];
            for (int kp = rowPtr[i]; kp < end; ++kp) {
                const int k = colIdx[kp];
                if (k >= i)
                    break;
                const int dk = diagPtr[k];
                if (dk < 0)
                    continue;
                const double piv = lu[dk];
                if (piv == 0.0)
                    continue;
                const double m = __ddiv_rn(lu[kp], piv);
                lu[kp] = m;
                const int kend = rowPtr[k + 1];
                for (int jp = dk + 1; jp < kend; ++jp) {
                    const int j = colIdx[jp];
                    for (int qp = kp + 1; qp < end; ++qp) {
                        const int c = colIdx[qp];
                        if (c == j) {
                            lu[qp] = __dsub_rn(lu[qp], __dmul_rn(m, lu[jp]));
                            break;
                        }
                        if (c > j)
                            break;
                    }
                }
            }
        }
        __syncthreads();
    }
}

__global__ void __launch_bounds__(kIluSmallThreads) k_ilu_sweeps_small(
    int n, int nlevF, const int32_t *__restrict__ lvlF, const int32_t *__restrict__ rowsF, int nlevB,
    const int32_t *__restrict__ lvlB, const int32_t *__restrict__ rowsB, const int32_t *__restrict__ rowPtr,
    const int32_t *__restrict__ colIdx, const int32_t *__restrict__ diagPtr, const double *__restrict__ lu,
    const double *__restrict__ r, double *__restrict__ z)
{
    extern __shared__ double ys[];
    for (int l = 0; l < nlevF; ++l) {
        const int a = __ldg(lvlF + l), b = __ldg(lvlF + l + 1);
        for (int t = a + threadIdx.x; t < b; t += blockDim.x) {
            const int i = __ldg(rowsF + t);
            double s = __ldg(r + i);
            const int end = __ldg(rowPtr + i + 1);
            for (int kp = __ldg(rowPtr + i); kp < end; ++kp) {
                const int j = __ldg(colIdx + kp);
                if (j >= i)
                    break;
                s = __dsub_rn(s, __dmul_rn(__ldg(lu + kp), ys[j]));
            }
            ys[i] = s;
        }
        __syncthreads();
    }
    for (int l = 0; l < nlevB; ++l) {
        const int a = __ldg(lvlB + l), b = __ldg(lvlB + l + 1);
        for (int t = a + threadIdx.x; t < b; t += blockDim.x) {
            const int i = __ldg(rowsB + t);
            double s = ys[i];
            const int kd = __ldg(diagPtr + i);
            const int end = __ldg(rowPtr + i + 1);
            for (int kp = kd + 1; kp < end; ++kp)
                s = __dsub_rn(s, __dmul_rn(__ldg(lu + kp), ys[__ldg(colIdx + kp)]));
            const double dv = kd >= 0 ? __ldg(lu + kd) : 0.0;
            ys[i] = (kd >= 0 && dv != 0.0) ? __ddiv_rn(s, dv) : s;
        }
        __syncthreads();
    }
    for (int i = threadIdx.x; i < n; i += blockDim.x)
        z[i] = ys[i];
}

// One warp waits for a mark that nothing sets: the bounded wait of the sweeps
// running out, observed from the host.
__global__ void k_wait_probe(const unsigned *flag, unsigned *out)
{
    const int j[4] = {0, 0, 0, 0};
    const bool ok = wait_rows4(flag, j, 1, 1u);
    if (threadIdx.x == 0)
        out[0] = ok ? 0u : 1u;
}

__global__ void k_zero_pivot_check(int n, const int32_t *__restrict__ diagPtr, const double *__restrict__ lu, int *flag)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int d = diagPtr[i];
        if (d < 0 || lu[d] == 0.0)
            atomicOr(flag, 1);
    }
}

// Rows grouped by level; `lower` selects the forward (j < i) or backward
// (j > i) dependency structure.
void levels(int64_t n, const int32_t *rowPtr, const int32_t *colIdx, const std::vector<int32_t> &diagPtr, bool lower,
            std::vector<int32_t> &rowsOut, std::vector<int32_t> &levelPtr, int &maxRows)
{
    std::vector<int32_t> lev(static_cast<size_t>(n), 0);
    int nlev = 0;
    if (lower) {
        for (int64_t i = 0; i < n; ++i) {
            int l = 0;
            for (int k = rowPtr[i]; k < rowPtr[i + 1]; ++k) {
                const int j = colIdx[k];
                if (j >= i)
                    break;
                l = std::max(l, lev[j] + 1);
            }
            lev[i] = l;
            nlev = std::max(nlev, l + 1);
        }
    } else {
        for (int64_t i = n - 1; i >= 0; --i) {
            int l = 0;
            const int kd = diagPtr[i];
            // the backward sweep reads columns after the diagonal (or the
            // whole row when the diagonal is missing, as the reference's
            // kd+1 = 0 start does; such rows are rejected before we get here)
            for (int k = kd + 1; k < rowPtr[i + 1]; ++k) {
                const int j = colIdx[k];
                if (j > i)
                    l = std::max(l, lev[j] + 1);
            }
            lev[i] = l;
            nlev = std::max(nlev, l + 1);
        }
    }
    levelPtr.assign(static_cast<size_t>(nlev) + 1, 0);
    for (int64_t i = 0; i < n; ++i)
        levelPtr[lev[i] + 1]++;
    maxRows = 0;
    for (int l = 0; l < nlev; ++l) {
        maxRows = std::max(maxRows, levelPtr[l + 1]);
        levelPtr[l + 1] += levelPtr[l];
    }
    rowsOut.resize(static_cast<size_t>(n));
    std::vector<int32_t> fill(levelPtr.begin(), levelPtr.end() - 1);
    for (int64_t i = 0; i < n; ++i)
        rowsOut[fill[lev[i]]++] = static_cast<int32_t>(i);
}

int analyse(simall_context *ctx, IluData *d, int64_t n, const int32_t *rowPtr, const int32_t *colIdx)
{
    d->h_diagPtr.assign(static_cast<size_t>(n), -1);
    for (int64_t i = 0; i < n; ++i)
        for (int k = rowPtr[i]; k < rowPtr[i + 1]; ++k)
            if (colIdx[k] == i) {
                d->h_diagPtr[i] = k;
                break;
            }
    std::vector<int32_t> fr, br;
    int m1 = 0, m2 = 0;
    levels(n, rowPtr, colIdx, d->h_diagPtr, true, fr, d->fwdLevelPtr, m1);
    levels(n, rowPtr, colIdx, d->h_diagPtr, false, br, d->bwdLevelPtr, m2);
    d->maxLevelRows = std::max(m1, m2);
    SIMALL_CUDA_TRY(ctx, d->diagPtr.alloc(n));
    SIMALL_CUDA_TRY(ctx, d->fwdRows.alloc(n));
    SIMALL_CUDA_TRY(ctx, d->bwdRows.alloc(n));
    SIMALL_CUDA_TRY(ctx, d->y.alloc(n));
    SIMALL_CUDA_TRY(ctx, d->done.alloc(n));
    SIMALL_CUDA_TRY(ctx, d->sweepCtl.alloc(4));
    SIMALL_CUDA_TRY(ctx, cudaMemsetAsync(d->done.p, 0, n * sizeof(unsigned), ctx->stream));
    SIMALL_CUDA_TRY(ctx, cudaMemsetAsync(d->sweepCtl.p, 0, 4 * sizeof(unsigned), ctx->stream));
    SIMALL_CUDA_TRY(ctx, cudaMemcpyAsync(d->diagPtr.p, d->h_diagPtr.data(), n * sizeof(int32_t),
                                         cudaMemcpyHostToDevice, ctx->stream));
    SIMALL_CUDA_TRY(ctx, cudaMemcpyAsync(d->fwdRows.p, fr.data(), n * sizeof(int32_t), cudaMemcpyHostToDevice,
                                         ctx->stream));
    SIMALL_CUDA_TRY(ctx, cudaMemcpyAsync(d->bwdRows.p, br.data(), n * sizeof(int32_t), cudaMemcpyHostToDevice,
                                         ctx->stream));
    SIMALL_CUDA_TRY(ctx, d->fwdLvl.alloc(d->fwdLevelPtr.size()));
    SIMALL_CUDA_TRY(ctx, d->bwdLvl.alloc(d->bwdLevelPtr.size()));
    SIMALL_CUDA_TRY(ctx, cudaMemcpyAsync(d->fwdLvl.p, d->fwdLevelPtr.data(), d->fwdLevelPtr.size() * sizeof(int32_t),
                                         cudaMemcpyHostToDevice, ctx->stream));
    SIMALL_CUDA_TRY(ctx, cudaMemcpyAsync(d->bwdLvl.p, d->bwdLevelPtr.data(), d->bwdLevelPtr.size() * sizeof(int32_t),
                                         cudaMemcpyHostToDevice, ctx->stream));
    d->small = n <= kIluSmallRows;
    if (d->small)
        SIMALL_CUDA_TRY(ctx, cudaFuncSetAttribute(k_ilu_sweeps_small, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                  static_cast<int>(n * sizeof(double))));
    // the copies above read host vectors that die at return
    SIMALL_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
    d->analysed = true;
    return SIMALL_OK;
}

int factor(simall_context *ctx, IluData *d, const int32_t *rowPtr, const int32_t *colIdx)
{
    const int nlev = static_cast<int>(d->fwdLevelPtr.size()) - 1;
    if (d->small) {
        k_ilu_factor_small<<<1, kIluSmallThreads, 0, ctx->stream>>>(nlev, d->fwdLvl.p, d->fwdRows.p, rowPtr, colIdx,
                                                                   d->diagPtr.p, d->lu.p);
        SIMALL_LAUNCH_CHECK(ctx);
        return SIMALL_OK;
    }
    for (int l = 1; l < nlev; ++l) {  // level 0 rows have no lower entries
        const int a = d->fwdLevelPtr[l], cnt = d->fwdLevelPtr[l + 1] - a;
        k_ilu_factor_level<<<(cnt + kBlock - 1) / kBlock, kBlock, 0, ctx->stream>>>(d->fwdRows.p + a, cnt, rowPtr,
                                                                                    colIdx, d->diagPtr.p, d->lu.p);
        SIMALL_LAUNCH_CHECK(ctx);
    }
    return SIMALL_OK;
}

int sweeps(simall_context *ctx, IluData *d, const int32_t *rowPtr, const int32_t *colIdx, const double *lu,
           const double *r, double *z)
{
    const int n = static_cast<int>(d->h_diagPtr.size());
    if (d->small) {
        k_ilu_sweeps_small<<<1, kIluSmallThreads, n * sizeof(double), ctx->stream>>>(
            n, static_cast<int>(d->fwdLevelPtr.size()) - 1, d->fwdLvl.p, d->fwdRows.p,
            static_cast<int>(d->bwdLevelPtr.size()) - 1, d->bwdLvl.p, d->bwdRows.p, rowPtr, colIdx, d->diagPtr.p, lu,
            r, z);
        SIMALL_LAUNCH_CHECK(ctx);
        return SIMALL_OK;
    }
    const int grid = ctx->num_sms * 4;  // 32 warps per SM take rows; more only add waiting warps
    k_sweep_begin<<<1, 1, 0, ctx->stream>>>(d->sweepCtl.p);
    SIMALL_LAUNCH_CHECK(ctx);
    k_ilu_fwd_free<<<grid, kBlock, 0, ctx->stream>>>(n, d->fwdRows.p, rowPtr, colIdx, lu, r, d->y.p, d->done.p,
                                                     d->sweepCtl.p);
    SIMALL_LAUNCH_CHECK(ctx);
    k_sweep_begin<<<1, 1, 0, ctx->stream>>>(d->sweepCtl.p);
    SIMALL_LAUNCH_CHECK(ctx);
    k_ilu_bwd_free<<<grid, kBlock, 0, ctx->stream>>>(n, d->bwdRows.p, rowPtr, colIdx, d->diagPtr.p, lu, d->y.p, z,
                                                     d->done.p, d->sweepCtl.p);
    SIMALL_LAUNCH_CHECK(ctx);
    return SIMALL_OK;
}

}  // namespace

int ilu_setup(simall_solver *s)
{
    simall_context *ctx = s->ctx;
    if (!s->ilu) {
        s->ilu = new (std::nothrow) IluData;
        if (!s->ilu)
            return SIMALL_ERR_OUT_OF_MEMORY;
    }
    IluData *d = s->ilu;
    if (!d->analysed) {
        int hp = solver_host_pattern(s);
        if (hp)
            return hp;
        int st = analyse(ctx, d, s->n, s->h_rowPtr.data(), s->h_colIdx.data());
        if (st)
            return st;
    }
    SIMALL_CUDA_TRY(ctx, d->lu.alloc(s->nnz));
    SIMALL_CUDA_TRY(ctx, cudaMemcpyAsync(d->lu.p, s->values, s->nnz * sizeof(double), cudaMemcpyDeviceToDevice,
                                         ctx->stream));
    return factor(ctx, d, s->rowPtr, s->colIdx);
}

int ilu_apply(simall_solver *s, const double *r, double *z)
{
    return sweeps(s->ctx, s->ilu, s->rowPtr, s->colIdx, s->ilu->lu.p, r, z);
}

// Whether a sweep gave up waiting for a row (a device-side timeout); clears
// the flag.
int ilu_check(simall_context *ctx, IluData *d)
{
    unsigned h = 0;
    SIMALL_CUDA_TRY(ctx, cudaMemcpyAsync(&h, d->sweepCtl.p + 2, sizeof(unsigned), cudaMemcpyDeviceToHost, ctx->stream));
    SIMALL_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
    if (h) {
        SIMALL_CUDA_TRY(ctx, cudaMemsetAsync(d->sweepCtl.p + 2, 0, sizeof(unsigned), ctx->stream));
        return fail(ctx, SIMALL_ERR_CUDA, "ILU(0) sweep: a row wait timed out");
    }
    return SIMALL_OK;
}

int ilu_check(simall_solver *s) { return s->ilu ? ilu_check(s->ctx, s->ilu) : SIMALL_OK; }

int ilu_apply_launches(const simall_solver *s) { return (s->ilu && s->ilu->small) ? 1 : 4; }

void ilu_free(simall_solver *s)
{
    delete s->ilu;
    s->ilu = nullptr;
}

}  // namespace simall

using namespace simall;

// ---------------------------------------------------------------- reference facade (GpuKernels.hpp:89-108)
namespace {
struct FacadeIlu {
    simall_context ctx;
    IluData d;
};

int facade_ctx(simall_context &ctx, void *stream)
{
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess)
        return SIMALL_ERR_NO_DEVICE;
    ctx.device = dev;
    if (cudaDeviceGetAttribute(&ctx.num_sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
        return SIMALL_ERR_CUDA;
    ctx.stream = static_cast<cudaStream_t>(stream);
    return SIMALL_OK;
}

int facade_pattern(simall_context &ctx, size_t n, const int32_t *rowPtr, const int32_t *colIdx,
                   std::vector<int32_t> &hr, std::vector<int32_t> &hc)
{
    hr.resize(n + 1);
    SIMALL_CUDA_TRY(&ctx, cudaMemcpyAsync(hr.data(), rowPtr, (n + 1) * sizeof(int32_t), cudaMemcpyDeviceToHost,
                                          ctx.stream));
    SIMALL_CUDA_TRY(&ctx, cudaStreamSynchronize(ctx.stream));
    hc.resize(static_cast<size_t>(hr[n]));
    SIMALL_CUDA_TRY(&ctx, cudaMemcpyAsync(hc.data(), colIdx, hc.size() * sizeof(int32_t), cudaMemcpyDeviceToHost,
                                          ctx.stream));
    SIMALL_CUDA_TRY(&ctx, cudaStreamSynchronize(ctx.stream));
    return check_csr_host(&ctx, static_cast<int64_t>(n), hr[n], hr.data(), hc.data(), nullptr, false);
}
}  // namespace

extern "C" {

int simall_gpu_ilu0_factor_inplace(size_t n, const int32_t *rowPtr, const int32_t *colIdx, double *values,
                                   void *stream, int *ok)
{
    if (!rowPtr || !colIdx || !values || !ok)
        return SIMALL_ERR_INVALID_ARGUMENT;
    *ok = 0;
    if (n == 0) {
        *ok = 1;
        return SIMALL_OK;
    }
    auto *f = new (std::nothrow) FacadeIlu;
    if (!f)
        return SIMALL_ERR_OUT_OF_MEMORY;
    std::vector<int32_t> hr, hc;
    int st = facade_ctx(f->ctx, stream);
    if (!st)
        st = facade_pattern(f->ctx, n, rowPtr, colIdx, hr, hc);
    if (!st)
        st = analyse(&f->ctx, &f->d, static_cast<int64_t>(n), hr.data(), hc.data());
    if (!st) {
        // factor in place: point lu at the caller's values
        double *saved = f->d.lu.p;
        f->d.lu.p = values;
        st = factor(&f->ctx, &f->d, rowPtr, colIdx);
        f->d.lu.p = saved;
    }
    if (!st) {
        st = f->d.y.alloc(1) == cudaSuccess ? SIMALL_OK : SIMALL_ERR_OUT_OF_MEMORY;
        int *flag = reinterpret_cast<int *>(f->d.y.p);
        if (!st && cudaMemsetAsync(flag, 0, sizeof(int), f->ctx.stream) != cudaSuccess)
            st = SIMALL_ERR_CUDA;
        if (!st) {
            k_zero_pivot_check<<<64, kBlock, 0, f->ctx.stream>>>(static_cast<int>(n), f->d.diagPtr.p, values, flag);
            int h = 1;
            if (cudaMemcpyAsync(&h, flag, sizeof(int), cudaMemcpyDeviceToHost, f->ctx.stream) != cudaSuccess ||
                cudaStreamSynchronize(f->ctx.stream) != cudaSuccess)
                st = SIMALL_ERR_CUDA;
            else
                *ok = h ? 0 : 1;
        }
    }
    delete f;
    return st;
}

int simall_diagnose_bounded_wait(simall_context *ctx, int *timed_out, double *seconds)
{
    if (!ctx || !timed_out)
        return SIMALL_ERR_INVALID_ARGUMENT;
    SIMALL_CUDA_TRY(ctx, cudaSetDevice(ctx->device));
    DevBuf<unsigned> buf;
    SIMALL_CUDA_TRY(ctx, buf.alloc(2));
    SIMALL_CUDA_TRY(ctx, cudaMemsetAsync(buf.p, 0, 2 * sizeof(unsigned), ctx->stream));
    const auto t0 = std::chrono::steady_clock::now();
    k_wait_probe<<<1, 32, 0, ctx->stream>>>(buf.p, buf.p + 1);
    SIMALL_LAUNCH_CHECK(ctx);
    unsigned h = 0;
    SIMALL_CUDA_TRY(ctx, cudaMemcpyAsync(&h, buf.p + 1, sizeof(unsigned), cudaMemcpyDeviceToHost, ctx->stream));
    SIMALL_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
    *timed_out = static_cast<int>(h);
    if (seconds)
        *seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    return SIMALL_OK;
}

int simall_gpu_ilu0_apply(size_t n, const int32_t *rowPtr, const int32_t *colIdx, const double *values,
                          const double *r, double *z, void *stream)
{
    if (!rowPtr || !colIdx || !values || !r || !z)
        return SIMALL_ERR_INVALID_ARGUMENT;
    if (n == 0)
        return SIMALL_OK;
    auto *f = new (std::nothrow) FacadeIlu;
    if (!f)
        return SIMALL_ERR_OUT_OF_MEMORY;
    std::vector<int32_t> hr, hc;
    int st = facade_ctx(f->ctx, stream);
    if (!st)
        st = facade_pattern(f->ctx, n, rowPtr, colIdx, hr, hc);
    if (!st)
        st = analyse(&f->ctx, &f->d, static_cast<int64_t>(n), hr.data(), hc.data());
    if (!st)
        st = sweeps(&f->ctx, &f->d, rowPtr, colIdx, values, r, z);
    if (!st && cudaStreamSynchronize(f->ctx.stream) != cudaSuccess)
        st = SIMALL_ERR_CUDA;
    if (!st)
        st = ilu_check(&f->ctx, &f->d);
    delete f;
    return st;
}

}  // extern "C"
