// Mixed-precision CG in one persistent cooperative launch: sliced storage
// (k_mx_grid_solve, the TMA-staged step of sell.cuh) and symmetric diagonal
// storage (k_mx_grid_dia, the step of dia_step.cuh).
//
// The per-step kernels of mixed.cu run one launch per CG step inside a
// device-side graph loop; between two steps the graph pays a controller
// kernel, a conditional node and the launch latency of the next step, about
// 7 us on GB300 -- a quarter of a step at 128^3.  Here every CTA stays
// resident for the whole solve (cudaLaunchCooperativeKernel guarantees that
// all of them are), and a step ends in one grid barrier:
//   - each CTA reduces its threads' four partial sums in float-float
//     (mixed_state.cuh, ffsum.cuh) and publishes them in slot
//     [epoch & 1][cta] of a double buffer;
//   - thread 0 releases its CTA's writes and adds one to a 64-bit arrival
//     counter, then polls it with acquire loads until all gridDim.x CTAs of
//     this epoch have arrived (bounded: ~4 s by %globaltimer, then the CTA
//     records a timeout and leaves; every other CTA then times out at its
//     next barrier, so the launch always ends);
//   - every CTA reads all partials in the same order and reduces them in the
//     same tree, so all CTAs hold bit-identical totals and take identical
//     decisions (step length, reliable update, stop) without another barrier.
// A CTA can be at most one barrier ahead of any other, so two partial slots
// suffice.  Vectors written in one step are read by other CTAs in the next:
// those loads are plain (coherent) loads, ordered by the barrier's acquire;
// only the matrix goes through the read-only path.
//
// The algorithm is the one of mixed.cu step for step (the fused step of
// sell.cuh or dia_step.cuh, van der Vorst-Ye reliable updates with the same
// trigger, the FP64 true residual r = b - A x from the original CSR, the stop
// test on it), so iteration counts and results agree with the per-step engine
// up to the order of the partial sums.  A reliable update costs two more barriers
// (after the fold x += S xh, and after the true residual with the FP32
// replacement r = S (b - A x) written in the same pass).
#include "device.cuh"
#include "dia_step.cuh"
#include "mixed_state.cuh"
#include "sell.cuh"
#include "solver.hpp"

#include <algorithm>
#include <cmath>

namespace simall {

namespace {

constexpr unsigned long long kGridWaitNs = 4000000000ull;  // one barrier wait gives up after ~4 s

struct GridArgs {
    SellOp A;
    const int32_t *rowPtr;
    const int32_t *colIdx;
    const double *val;
    const double *b;
    const double *sc;
    double *x;
    float4 *st[2];  // (r, q, p, xh) per row, by step parity (sell.cuh)
    double *part;  // [2][gridDim.x][4]
    unsigned long long *ctr;
    int *err;
    SolveScalars *s;
    double tol, delta;
    int max_iter;
};

__device__ __forceinline__ unsigned long long ld_acquire(const unsigned long long *p)
{
    unsigned long long v;
    asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ unsigned long long global_ns()
{
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Grid barrier of epoch `epoch` (1, 2, ...): returns false (in every thread of
// the CTA) when the wait ran out.
__device__ bool grid_barrier(unsigned long long *ctr, unsigned long long epoch, int *err)
{
    __shared__ int ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        atomicAdd(ctr, 1ull);
        const unsigned long long target = epoch * gridDim.x;
        int good = 1;
        if (ld_acquire(ctr) < target) {
            const unsigned long long t0 = global_ns();
            for (unsigned spins = 1; ld_acquire(ctr) < target; ++spins)
                if ((spins & 63u) == 0 && global_ns() - t0 > kGridWaitNs) {
                    good = 0;
                    atomicExch(err, 1);
                    break;
                }
        }
        // the acquire loads order what follows; the block barrier below passes
        // that on to the other threads
        ok = good;
    }
    __syncthreads();
    return ok != 0;
}

// Every grid sum uses slots of kSlot values per CTA in two halves by epoch
// parity, whatever its number of values: a CTA may still read the half of
// the previous sum while a faster one writes the other half, so the halves
// must not overlap for sums of different sizes.
constexpr int kSlot = 4;

// Sum of NV <= kSlot FP64 values over the grid, the same bits in every CTA:
// block tree, one slot per CTA, barrier, then every CTA sums all slots in
// index order and reduces them in the same tree.  Returns false on a barrier
// timeout.
template <int NV>
__device__ bool grid_allsum(double (&v)[NV], double *part, unsigned long long *ctr, unsigned long long &epoch,
                            int *err)
{
    static_assert(NV <= kSlot, "a grid sum holds at most kSlot values per CTA");
    __shared__ double tot[NV];
    block_sum<NV>(v);
    double *slot = part + (epoch & 1ull) * gridDim.x * kSlot;
    if (threadIdx.x == 0) {
#pragma unroll
        for (int k = 0; k < NV; ++k)
            slot[static_cast<int64_t>(blockIdx.x) * kSlot + k] = v[k];
    }
    ++epoch;
    if (!grid_barrier(ctr, epoch, err))
        return false;
    double acc[NV];
#pragma unroll
    for (int k = 0; k < NV; ++k)
        acc[k] = 0.0;
    for (unsigned c = threadIdx.x; c < gridDim.x; c += blockDim.x) {
#pragma unroll
        for (int k = 0; k < NV; ++k)
            acc[k] += __ldcg(slot + static_cast<int64_t>(c) * kSlot + k);
    }
    block_sum<NV>(acc);
    if (threadIdx.x == 0) {
#pragma unroll
        for (int k = 0; k < NV; ++k)
            tot[k] = acc[k];
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < NV; ++k)
        v[k] = tot[k];
    __syncthreads();
    return true;
}

// The end of a step with four block barriers: each warp sums its threads'
// float-float values; a block barrier (which also joins the threads'
// verdicts); warp 0 sums the warps, publishes the CTA's slot, arrives at the
// grid barrier and polls it (lane 0; the other lanes wait at a shuffle); a
// block barrier; every thread then sums its share of the CTA slots (at most a
// few, all loads in flight at once), the warps and warp 0 combine them in a
// fixed order, and lane 0 finishes the step; a last block barrier hands the
// state to the CTA.  Returns false (in every thread) on a timeout or a failed
// verdict.
template <class Finish>
__device__ bool step_allsum(bool ok_thread, FF (&acc)[4], double *part, unsigned long long *ctr,
                            unsigned long long &epoch, int *err, Finish fin)
{
    __shared__ FF ws[4][32];
    __shared__ int s_ok;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const FF w = ff_warp_allsum(acc[k]);
        if (lane == 0)
            ws[k][wid] = w;
    }
    if (!__syncthreads_and(ok_thread)) {
        if (threadIdx.x == 0)
            atomicExch(err, 1);
        return false;
    }
    FF *slot = reinterpret_cast<FF *>(part) + (epoch & 1ull) * gridDim.x * kSlot;
    ++epoch;
    if (wid == 0) {
        FF c[4];
#pragma unroll
        for (int k = 0; k < 4; ++k)
            c[k] = ff_warp_allsum(lane < nw ? ws[k][lane] : ff_zero());
        if (lane == 0) {
            int good = 1;
#pragma unroll
            for (int k = 0; k < 4; ++k)
                slot[static_cast<int64_t>(blockIdx.x) * kSlot + k] = c[k];
            __threadfence();
            atomicAdd(ctr, 1ull);
            const unsigned long long target = epoch * gridDim.x;
            if (ld_acquire(ctr) < target) {
                const unsigned long long t0 = global_ns();
                for (unsigned spins = 1; ld_acquire(ctr) < target; ++spins)
                    if ((spins & 63u) == 0 && global_ns() - t0 > kGridWaitNs) {
                        good = 0;
                        atomicExch(err, 1);
                        break;
                    }
            }
            s_ok = good;
        }
    }
    __syncthreads();
    if (!s_ok)
        return false;
    FF t[4] = {ff_zero(), ff_zero(), ff_zero(), ff_zero()};
    for (unsigned cta = threadIdx.x; cta < gridDim.x; cta += blockDim.x) {
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const float2 v = __ldcg(reinterpret_cast<const float2 *>(slot) + cta * kSlot + k);
            t[k] = ff_add(t[k], FF{v.x, v.y});
        }
    }
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const FF w = ff_warp_allsum(t[k]);
        if (lane == 0)
            ws[k][wid] = w;
    }
    __syncthreads();
    if (wid == 0) {
        FF tot[4];
#pragma unroll
        for (int k = 0; k < 4; ++k)
            tot[k] = ff_warp_allsum(lane < nw ? ws[k][lane] : ff_zero());
        if (lane == 0)
            fin(tot);
    }
    __syncthreads();
    return true;
}

// FP32 per-thread partials: lanes summed in FP32, everything above in FP64.
template <int NV>
__device__ bool grid_allsum_f(const float (&v)[NV], double (&out)[NV], double *part, unsigned long long *ctr,
                              unsigned long long &epoch, int *err)
{
#pragma unroll
    for (int k = 0; k < NV; ++k) {
        float w = v[k];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1)
            w += __shfl_down_sync(0xffffffffu, w, o);
        out[k] = (threadIdx.x & 31) == 0 ? static_cast<double>(w) : 0.0;  // block_sum adds lane 0 of each warp
    }
    return grid_allsum<NV>(out, part, ctr, epoch, err);
}

template <bool WIDE, bool STAGED>
__global__ void __launch_bounds__(kSellThreads, 1) k_mx_grid_solve(GridArgs g)
{
    extern __shared__ __align__(128) unsigned char sell_smem[];
    __shared__ uint64_t bars[2 * kSellStages];
    if (STAGED && threadIdx.x == 0)
        sell_ring_init(bars);
    __syncthreads();
    SellRing<WIDE> R{reinterpret_cast<SellStageBuf<WIDE> *>(sell_smem), bars, 0};
    // this CTA's slices of the staged steps
    const int64_t c0 = blockIdx.x * g.A.nslices / gridDim.x, c1 = (blockIdx.x + 1) * g.A.nslices / gridDim.x;
    const int64_t n = g.A.n;
    const int64_t tid = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
    const int64_t nthr = static_cast<int64_t>(gridDim.x) * blockDim.x;
    const int64_t warp = tid >> 5, nwarps = nthr >> 5;
    unsigned long long epoch = 0;
    bool ok = true;

    // init: x = 0, state[1] = (S b, 0, 0, 0); |S b|^2 (FP32 rows), |b|^2
    double tot[2];
    {
        float a0 = 0.0f;
        double a1 = 0.0;
        for (int64_t i = tid; i < n; i += nthr) {
            const double bi = g.b[i];
            const float r = static_cast<float>(bi * g.sc[i]);
            g.x[i] = 0.0;
            g.st[1][i] = make_float4(r, 0.0f, 0.0f, 0.0f);
            a0 += r * r;
            a1 += bi * bi;
        }
        float f[1] = {a0};
        double d1[1];
        ok = grid_allsum_f<1>(f, d1, g.part, g.ctr, epoch, g.err);
        double d2[1] = {a1};
        ok = ok && grid_allsum<1>(d2, g.part, g.ctr, epoch, g.err);
        tot[0] = d1[0];
        tot[1] = d2[0];
    }
    // The solver state: identical in every CTA (it follows from the identical
    // totals), kept in shared memory and advanced by thread 0 alone after each
    // grid sum; the other threads read the control values after a block barrier.
    __shared__ MixedState st;
    if (threadIdx.x == 0)
        st.start(tot[0], tot[1], g.tol, g.max_iter);
    __syncthreads();
    const int64_t trip_cap = 2 * static_cast<int64_t>(g.max_iter > 0 ? g.max_iter : 0) + 16;
    const float tolf = static_cast<float>(g.tol), deltaf = static_cast<float>(g.delta);
    for (int64_t trips = 0; ok && !st.done; ++trips) {
        if (trips > trip_cap) {  // unreachable: every normal step counts and max_iter ends the solve
            if (threadIdx.x == 0)
                st.stop(SIMALL_ERR_TIMEOUT);
            break;
        }
        // ---- one fused step
        const int par = st.par;
        const float alpha = st.fresh ? 0.0f : st.alpha_f, beta = st.beta_f;
        FF acc[4] = {ff_zero(), ff_zero(), ff_zero(), ff_zero()};
        bool step_ok = true;
        if (STAGED) {
            step_ok = sell_step_staged<WIDE, false>(g.A, c0, c1, g.st[par], g.st[1 - par], alpha, beta, acc, R, true);
        } else {
            for (int64_t sl = warp; sl < g.A.nslices; sl += nwarps)
                sell_slice<WIDE, false>(g.A, sl, g.st[par], g.st[1 - par], alpha, beta, acc);
        }
        if (!(ok = step_allsum(step_ok, acc, g.part, g.ctr, epoch, g.err,
                               [&](const FF (&t)[4]) { st.finish_step(t, tolf, deltaf, g.max_iter); })))
            break;
        if (!st.update)
            continue;
        // ---- reliable update: x += S xh with the xh the triggering step wrote
        {
            const float4 *so = g.st[1 - st.par];
            for (int64_t i = tid; i < n; i += nthr)
                g.x[i] += g.sc[i] * static_cast<double>(so[i].w);
        }
        ++epoch;
        if (!(ok = grid_barrier(g.ctr, epoch, g.err)))
            break;
        // r = b - A x in FP64; the replacement S r (FP32), and xh = 0, into the
        // state the FRESH step reads (its q and p stay); |r|^2 and |S r|^2
        float4 *srep = g.st[st.par];
        double a[2] = {0.0, 0.0};
        for (int64_t i = tid; i < n; i += nthr) {
            // one FMA per entry from 0.0 in column order (the per-step
            // engine's true residual, spmv_rowblocks_fma); A is streamed with
            // the evict-first hint (__ldcs) so the iteration state stays in L2
            const int k1 = __ldcs(g.rowPtr + i + 1);
            double y = 0.0;
            for (int k = __ldcs(g.rowPtr + i); k < k1; ++k)
                y = __fma_rn(__ldcs(g.val + k), g.x[__ldcs(g.colIdx + k)], y);
            const double v = g.b[i] - y;
            const float f = static_cast<float>(g.sc[i] * v);
            float *e = reinterpret_cast<float *>(srep + i);
            e[0] = f;
            e[3] = 0.0f;
            a[0] += v * v;
            a[1] += static_cast<double>(f) * static_cast<double>(f);
        }
        if (!(ok = grid_allsum<2>(a, g.part, g.ctr, epoch, g.err)))
            break;
        if (threadIdx.x == 0)
            st.finish_update(a, g.tol, g.max_iter);
        __syncthreads();
    }
    if (blockIdx.x == 0 && threadIdx.x == 0)
        st.publish(g.s, ok);
}

// ---------------------------------------------------------------- diagonal storage
// The same solve for symmetric diagonal storage: the step of dia_step.cuh
// (coherent vector loads), one CTA of kGridDiaThreads per SM.  The state is
// r, q, p by step parity and one xh, as in the per-step engine: the first
// step (FRESH, parity 1) reads r from r[0] and p_old = 0 from p[1]; after a
// step of parity P asks for a reliable update, x += S xh, the replacement
// S (b - A x) goes to r[1 - P] and a FRESH step of parity P follows.
constexpr int kGridDiaThreads = 512;

struct GridDiaDev {
    int n;
    int64_t ldU;
    DiaOffsets o;
    const float *U, *e;
    float *rv[2], *qv[2], *pv[2], *xh;
    const int32_t *rowPtr;
    const int32_t *colIdx;
    const double *val;
    const double *b;
    const double *sc;
    double *x;
    double *part;
    unsigned long long *ctr;
    int *err;
    SolveScalars *s;
    double tol, delta;
    int max_iter;
};

// The FRESH step (the first one and one after each reliable update) out of
// line, so that its copy of the step does not add to the registers of the
// ordinary step's loop.
template <int ND, bool GRID>
__device__ __noinline__ void grid_dia_fresh(const GridDiaDev &g, const IterVecs &v, float beta, float (&acc)[4])
{
    dia_step<ND, GRID, true, true>(g.n, g.ldU, g.o, g.U, g.e, v, 0.0f, beta, acc);
}

template <int ND, bool GRID>
__global__ void __launch_bounds__(kGridDiaThreads, 1) k_mx_grid_dia(GridDiaDev g)
{
    const int64_t n = g.n;
    const int64_t tid = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
    const int64_t nthr = static_cast<int64_t>(gridDim.x) * blockDim.x;
    unsigned long long epoch = 0;
    bool ok = true;

    // init: x = 0, r[0] = S b, p[1] = 0, xh = 0; |S b|^2 (FP32 rows), |b|^2
    double tot[2];
    {
        float a0 = 0.0f;
        double a1 = 0.0;
        for (int64_t i = tid; i < n; i += nthr) {
            const double bi = g.b[i];
            const float r = static_cast<float>(bi * g.sc[i]);
            g.x[i] = 0.0;
            g.rv[0][i] = r;
            g.pv[1][i] = 0.0f;
            g.xh[i] = 0.0f;
            a0 += r * r;
            a1 += bi * bi;
        }
        float f[1] = {a0};
        double d1[1];
        ok = grid_allsum_f<1>(f, d1, g.part, g.ctr, epoch, g.err);
        double d2[1] = {a1};
        ok = ok && grid_allsum<1>(d2, g.part, g.ctr, epoch, g.err);
        tot[0] = d1[0];
        tot[1] = d2[0];
    }
    __shared__ MixedState st;
    if (threadIdx.x == 0)
        st.start(tot[0], tot[1], g.tol, g.max_iter);
    __syncthreads();
    const int64_t trip_cap = 2 * static_cast<int64_t>(g.max_iter > 0 ? g.max_iter : 0) + 16;
    const float tolf = static_cast<float>(g.tol), deltaf = static_cast<float>(g.delta);
    for (int64_t trips = 0; ok && !st.done; ++trips) {
        if (trips > trip_cap) {  // unreachable: every normal step counts and max_iter ends the solve
            if (threadIdx.x == 0)
                st.stop(SIMALL_ERR_TIMEOUT);
            break;
        }
        // ---- one fused step
        const int par = st.par;
        const float alpha = st.fresh ? 0.0f : st.alpha_f, beta = st.beta_f;
        const IterVecs v{g.rv[par], g.qv[par], g.pv[par], g.rv[1 - par], g.qv[1 - par], g.pv[1 - par], g.xh};
        float acc[4] = {0.0f, 0.0f, 0.0f, 0.0f};
        if (st.fresh)
            grid_dia_fresh<ND, GRID>(g, v, beta, acc);
        else
            dia_step<ND, GRID, false, true>(g.n, g.ldU, g.o, g.U, g.e, v, alpha, beta, acc);
        FF facc[4] = {FF{acc[0], 0.0f}, FF{acc[1], 0.0f}, FF{acc[2], 0.0f}, FF{acc[3], 0.0f}};
        if (!(ok = step_allsum(true, facc, g.part, g.ctr, epoch, g.err,
                               [&](const FF (&t)[4]) { st.finish_step(t, tolf, deltaf, g.max_iter); })))
            break;
        if (!st.update)
            continue;
        // ---- reliable update: x += S xh with the xh the triggering step wrote
        for (int64_t i = tid; i < n; i += nthr) {
            g.x[i] += g.sc[i] * static_cast<double>(g.xh[i]);
            g.xh[i] = 0.0f;
        }
        ++epoch;
        if (!(ok = grid_barrier(g.ctr, epoch, g.err)))
            break;
        // r = b - A x in FP64 (one FMA per entry from 0.0 in column order, as
        // the per-step engine's true residual; A streamed with the evict-first
        // hint); the replacement S r (FP32) into the r the FRESH step reads;
        // |r|^2 and |S r|^2
        float *rrep = g.rv[1 - st.par];
        double a[2] = {0.0, 0.0};
        for (int64_t i = tid; i < n; i += nthr) {
            const int k1 = __ldcs(g.rowPtr + i + 1);
            double y = 0.0;
            for (int k = __ldcs(g.rowPtr + i); k < k1; ++k)
                y = __fma_rn(__ldcs(g.val + k), g.x[__ldcs(g.colIdx + k)], y);
            const double r = g.b[i] - y;
            const float f = static_cast<float>(g.sc[i] * r);
            rrep[i] = f;
            a[0] += r * r;
            a[1] += static_cast<double>(f) * static_cast<double>(f);
        }
        if (!(ok = grid_allsum<2>(a, g.part, g.ctr, epoch, g.err)))
            break;
        if (threadIdx.x == 0)
            st.finish_update(a, g.tol, g.max_iter);
        __syncthreads();
    }
    if (blockIdx.x == 0 && threadIdx.x == 0)
        st.publish(g.s, ok);
}

template <int ND> const void *grid_dia_kernel(bool grid)
{
    return grid ? reinterpret_cast<const void *>(k_mx_grid_dia<ND, true>)
                : reinterpret_cast<const void *>(k_mx_grid_dia<ND, false>);
}

// The cooperative launch of a whole persistent solve and its verdict: 0 when
// the launch is refused (too large for the device, or no cooperative
// launch), else 1 with *status: the launch error, a grid barrier's timeout,
// or whether the solve reached its stop test.  `args` points to the kernel's
// one argument struct; ctr and err are reset first.
int launch_persistent(simall_solver *s, const void *fn, int grid, int threads, size_t smem, void *args,
                      unsigned long long *ctr, int *err, int *status)
{
    simall_context *ctx = s->ctx;
    SIMALL_CUDA_TRY(ctx, cudaMemsetAsync(ctr, 0, sizeof(unsigned long long), ctx->stream));
    SIMALL_CUDA_TRY(ctx, cudaMemsetAsync(err, 0, sizeof(int), ctx->stream));
    void *argv[] = {args};
    cudaError_t e = cudaLaunchCooperativeKernel(fn, dim3(grid), dim3(threads), argv, smem, ctx->stream);
    if (e == cudaErrorCooperativeLaunchTooLarge || e == cudaErrorNotSupported) {
        cudaGetLastError();
        return 0;
    }
    ctx->launches.fetch_add(1, std::memory_order_relaxed);
    if (e != cudaSuccess) {
        *status = cuda_fail(ctx, e, "cudaLaunchCooperativeKernel", __FILE__, __LINE__);
        return 1;
    }
    int timed_out = 0;
    e = cudaMemcpyAsync(&timed_out, err, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream);
    if (e != cudaSuccess) {
        *status = cuda_fail(ctx, e, "cudaMemcpyAsync", __FILE__, __LINE__);
        return 1;
    }
    int st = solver_fetch_scalars(s);  // synchronises the stream
    if (st) {
        *status = st;
        return 1;
    }
    s->engine = 2;
    if (timed_out || s->h_scal->status == SIMALL_ERR_TIMEOUT) {
        *status = fail(ctx, SIMALL_ERR_TIMEOUT, "mixed precision: a grid barrier of the persistent solve timed out");
        return 1;
    }
    *status = s->h_scal->done ? SIMALL_OK : fail(ctx, SIMALL_ERR_CUDA, "persistent solve ended before its stop test");
    return 1;
}

}  // namespace

int grid_mixed_solve(simall_solver *s, const GridMixedArgs &a, int *status)
{
    simall_context *ctx = s->ctx;
    if (s->n <= 0 || s->cfg.check_interval > 0 || s->cfg.engine != SIMALL_ENGINE_AUTO)
        return 0;
    int coop = 0;
    if (cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, ctx->device) != cudaSuccess || !coop)
        return 0;
    const void *fn = a.wide ? (a.staged ? reinterpret_cast<const void *>(k_mx_grid_solve<true, true>)
                                        : reinterpret_cast<const void *>(k_mx_grid_solve<true, false>))
                            : (a.staged ? reinterpret_cast<const void *>(k_mx_grid_solve<false, true>)
                                        : reinterpret_cast<const void *>(k_mx_grid_solve<false, false>));
    const size_t smem = a.staged ? (a.wide ? sell_stage_smem<true>() : sell_stage_smem<false>()) : 0;
    int per_sm = 0;
    if (staged_residency(ctx, fn, kSellThreads, smem, &per_sm) != SIMALL_OK) {
        cudaGetLastError();
        return 0;
    }
    // a stage of slices per CTA at least, never more CTAs than are resident
    const int64_t want = std::max<int64_t>(1, (a.nslices + kSellStageSlices - 1) / kSellStageSlices);
    const int use = g_grid_ctas_per_sm > 0 ? std::min(per_sm, g_grid_ctas_per_sm) : per_sm;
    const int64_t cap = static_cast<int64_t>(ctx->num_sms) * std::min(use, kGridMaxCtasPerSm);
    const int grid = static_cast<int>(std::min(want, cap));
    if (static_cast<size_t>(grid) * 8 > a.partCap)
        return 0;
    GridArgs g{};
    g.A.n = s->n;
    g.A.nslices = a.nslices;
    g.A.sptr = a.sptr;
    g.A.off16 = a.off16;
    g.A.off32 = a.off32;
    g.A.val = a.sval;
    g.A.e = a.e;
    g.A.prefetch = g_sell_prefetch;
    g.rowPtr = s->rowPtr;
    g.colIdx = s->colIdx;
    g.val = s->values;
    g.b = s->b.p;
    g.sc = a.scale;
    g.x = s->x.p;
    g.st[0] = a.st[0];
    g.st[1] = a.st[1];
    g.part = a.part;
    g.ctr = a.ctr;
    g.err = a.err;
    g.s = s->scal.p;
    g.tol = s->cfg.tolerance;
    g.delta = s->cfg.reliable_delta;
    g.max_iter = s->cfg.max_iterations;
    return launch_persistent(s, fn, grid, kSellThreads, smem, &g, a.ctr, a.err, status);
}

int grid_dia_solve(simall_solver *s, const GridDiaArgs &a, int *status)
{
    simall_context *ctx = s->ctx;
    if (s->n <= 0 || s->n > INT32_MAX - 8 || s->cfg.check_interval > 0 || s->cfg.engine != SIMALL_ENGINE_AUTO ||
        a.nd < 1 || a.nd > kGridDiaMaxDiags)
        return 0;
    int coop = 0;
    if (cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, ctx->device) != cudaSuccess || !coop)
        return 0;
    const void *fn = a.nd == 1   ? grid_dia_kernel<1>(a.grid)
                     : a.nd == 2 ? grid_dia_kernel<2>(a.grid)
                     : a.nd == 3 ? grid_dia_kernel<3>(a.grid)
                                 : grid_dia_kernel<4>(a.grid);
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, kGridDiaThreads, 0) != cudaSuccess ||
        per_sm < 1) {
        cudaGetLastError();
        return 0;
    }
    // one CTA per SM, never more than there are quads of rows for
    const int64_t quads = (s->n + 3) / 4;
    const int64_t want = std::max<int64_t>(1, (quads + kGridDiaThreads - 1) / kGridDiaThreads);
    const int grid = static_cast<int>(std::min<int64_t>(want, ctx->num_sms));
    if (static_cast<size_t>(grid) * 2 * kSlot > a.partCap)
        return 0;
    GridDiaDev g{};
    g.n = static_cast<int>(s->n);
    g.ldU = a.ldU;
    for (int d = 0; d < kMaxDiags; ++d)
        g.o.off[d] = d < a.nd ? a.off[d] : 0;
    g.o.nd = a.nd;
    g.U = a.U;
    g.e = a.e;
    for (int k = 0; k < 2; ++k) {
        g.rv[k] = a.rv[k];
        g.qv[k] = a.qv[k];
        g.pv[k] = a.pv[k];
    }
    g.xh = a.xh;
    g.rowPtr = s->rowPtr;
    g.colIdx = s->colIdx;
    g.val = s->values;
    g.b = s->b.p;
    g.sc = a.scale;
    g.x = s->x.p;
    g.part = a.part;
    g.ctr = a.ctr;
    g.err = a.err;
    g.s = s->scal.p;
    g.tol = s->cfg.tolerance;
    g.delta = s->cfg.reliable_delta;
    g.max_iter = s->cfg.max_iterations;
    return launch_persistent(s, fn, grid, kGridDiaThreads, 0, &g, a.ctr, a.err, status);
}

}  // namespace simall
