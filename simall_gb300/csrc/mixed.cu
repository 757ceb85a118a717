// Mixed-precision Jacobi-PCG: FP32 inner iteration, FP64 true residual,
// global reductions and solution.
//
// Jacobi PCG on A is plain CG on the scaled matrix S A S (S = D^-1/2, unit
// diagonal) in the variables y = S^-1 x.  The inner iteration runs that CG in
// FP32 on an FP32 copy of S A S; its correction accumulates in an FP32 vector
// that is folded into the FP64 solution x at "reliable updates" (residual
// replacement, van der Vorst & Ye 2000; Strzodka & Goddeke 2006): whenever the
// iterated residual has dropped by reliable_delta since the last update, or
// its estimate says the stop test may hold, x += S xh in FP64, the true
// residual r = b - A x is recomputed in FP64 with the original CSR, the stop
// test ||r|| / max(||b||,1e-30) < tol is applied to it, and the FP32 residual
// is replaced by S r.  The search direction is kept, so the Krylov process is
// not restarted.  Per-thread partial sums are FP32; every cross-thread and
// cross-CTA reduction is FP64.
//
// Storage of S A S: when A is numerically symmetric and its off-diagonal
// entries lie on at most kMaxDiags distinct diagonals (every structured grid
// in natural order), only the upper diagonals are stored, FP32, one array per
// offset: 4 B per stored diagonal per row and no column indices.  Otherwise
// the off-diagonal entries are kept in sliced storage (sell.cuh: slices of 32
// rows, entry-major, 16-bit column offsets where the bandwidth allows, FP32
// values, 6 B per entry) with the iteration state packed per row (r, q, p,
// xh); its steps stage the streamed operands through shared memory by bulk
// copies.  With the default engine the sliced form runs the whole solve in
// one persistent cooperative launch (mixed_grid.cu); per-step kernels
// otherwise.
//
// Row-sum form of the product (diagonal storage).  With N the off-diagonal part of S A S and
// e_i = 1 + sum_j N_ij (summed in FP64 from A, stored rounded to FP32), the
// inner SpMV evaluates
//     q_i = e_i p_i - sum_j N_ij (p_i - p_j)
// which equals p_i + sum_j N_ij p_j.  For a pressure Laplacian the terms of
// the plain form cancel on smooth directions (q is far smaller than p), and
// rounding N to FP32 then moves the smallest eigenvalues of the inner operator
// by far more than their own size; in the row-sum form the rounding only
// perturbs the positive couplings of a Laplacian whose row sums stay exact to
// one FP32 rounding, and the differences p_i - p_j of a smooth direction are
// small and exact.  On the 128 x 128 cavity's pressure systems (one pinned
// cell) the FP32 inner CG needs 1075 iterations with the plain form and 776
// with this one, against 775 for FP64 CG; it costs one 4-byte stream per row.
#include "device.cuh"
#include "dia_step.cuh"
#include "sell.cuh"
#include "solver.hpp"

#include <algorithm>
#include <climits>
#include <cmath>
#include <new>

namespace simall {

int g_sell_prefetch = 0;
int g_grid_ctas_per_sm = 0;

struct MixedData {
    bool dia = false;
    DiaOffsets offs{};
    DevBuf<float> U;          // [nd][ldU] upper diagonals of S A S (dia)
    int64_t ldU = 0;          // diagonal stride, n rounded up to 4 (16-byte aligned rows)
    // sliced storage (sell.cuh) of every other pattern
    int64_t nslices = 0;
    int64_t sEntries = 0;      // stored entries, padding included (32 per slice per unit of width)
    bool sWide = false;        // int32 column offsets
    int sMaxW = 0;             // widest slice (entries per row); up to kSellStageMaxW the steps are staged
    DevBuf<int32_t> sptr;      // [nslices + 1]
    DevBuf<int16_t> soff16;
    DevBuf<int32_t> soff32;
    DevBuf<int32_t> spos;      // CSR position of each stored entry, -1 for padding
    DevBuf<float> sval;
    // the persistent engine's grid reduction buffers and barrier (mixed_grid.cu)
    DevBuf<double> gpart;
    DevBuf<unsigned long long> gctr;
    DevBuf<int> gerr;
    bool noGrid = false;       // cooperative launch unavailable or refused: per-step kernels
    DevBuf<double> scale;     // s_i = 1/sqrt(a_ii)
    DevBuf<float> e;          // dia: e_i = 1 + sum_j (S A S)_ij, summed in FP64 from A, then rounded
    DevBuf<float> xh;         // FP32 correction, folded into x at reliable updates
    DevBuf<float> rv[2], qv[2], pv[2];  // dia: r, q = (S A S) p, p; double-buffered by step parity
    DevBuf<float4> st[2];               // sliced: (r, q, p, xh) per row, double-buffered (sell.cuh)
    bool patternReady = false;
    bool noDeviceLoop = false;  // conditional graph nodes unavailable
};

namespace {

__device__ __forceinline__ int ld_flag(const int *p) { return __ldcg(p); }

// s_i = 1/sqrt(a_ii); flag if a_ii <= 0.
__global__ void __launch_bounds__(kBlock) k_mx_scale(int64_t n, const int32_t *__restrict__ rowPtr,
                                                     const int32_t *__restrict__ colIdx, const double *__restrict__ val,
                                                     double *__restrict__ sc, int *flag)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        double d = 0.0;
        for (int k = rowPtr[i]; k < rowPtr[i + 1]; ++k)
            if (colIdx[k] == i) {
                d = val[k];
                break;
            }
        if (!(d > 0.0)) {
            atomicOr(flag, 1);
            d = 1.0;
        }
        sc[i] = 1.0 / sqrt(d);
    }
}

// Numerical symmetry: a_ji must exist and equal a_ij bit for bit.
__global__ void __launch_bounds__(kBlock) k_mx_symcheck(int64_t n, const int32_t *__restrict__ rowPtr,
                                                        const int32_t *__restrict__ colIdx,
                                                        const double *__restrict__ val, int *flag)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        for (int k = rowPtr[i]; k < rowPtr[i + 1]; ++k) {
            const int j = colIdx[k];
            if (j <= i)
                continue;
            int lo = rowPtr[j], hi = rowPtr[j + 1] - 1, pos = -1;
            while (lo <= hi) {
                const int mid = (lo + hi) >> 1;
                const int c = colIdx[mid];
                if (c == i) {
                    pos = mid;
                    break;
                }
                if (c < i)
                    lo = mid + 1;
                else
                    hi = mid - 1;
            }
            if (pos < 0 || val[pos] != val[k])
                atomicOr(flag, 2);
        }
    }
}

__global__ void __launch_bounds__(kBlock) k_mx_build_dia(int64_t n, int64_t ldU, const int32_t *__restrict__ rowPtr,
                                                         const int32_t *__restrict__ colIdx,
                                                         const double *__restrict__ val, const double *__restrict__ sc,
                                                         DiaOffsets o, float *__restrict__ U)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        float u[kMaxDiags];
#pragma unroll
        for (int d = 0; d < kMaxDiags; ++d)
            u[d] = 0.0f;
        const double si = sc[i];
        for (int k = rowPtr[i]; k < rowPtr[i + 1]; ++k) {
            const int j = colIdx[k];
            if (j <= i)
                continue;
            const int off = j - static_cast<int>(i);
#pragma unroll
            for (int d = 0; d < kMaxDiags; ++d)
                if (d < o.nd && o.off[d] == off)
                    u[d] = static_cast<float>(val[k] * si * sc[j]);
        }
        for (int d = 0; d < o.nd; ++d)
            U[d * ldU + i] = u[d];
    }
}

// e_i = 1 + sum_{j != i} a_ij s_i s_j in FP64 (column order), rounded once to
// FP32: the row sum of S A S, exact up to that one rounding.
__global__ void __launch_bounds__(kBlock) k_mx_row_defect(int64_t n, const int32_t *__restrict__ rowPtr,
                                                          const int32_t *__restrict__ colIdx,
                                                          const double *__restrict__ val,
                                                          const double *__restrict__ sc, float *__restrict__ e)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const double si = sc[i];
        double sum = 1.0;
        for (int k = rowPtr[i]; k < rowPtr[i + 1]; ++k) {
            const int j = colIdx[k];
            if (j != i)
                sum += val[k] * si * sc[j];
        }
        e[i] = static_cast<float>(sum);
    }
}

// Values of the sliced storage: N_ij = a_ij s_i s_j in FP64 (the product in
// that order), stored rounded to FP32; padding entries 0.  One thread per row.
__global__ void __launch_bounds__(kBlock) k_mx_build_sell(int64_t n, const int32_t *__restrict__ sptr,
                                                          const int32_t *__restrict__ spos,
                                                          const int32_t *__restrict__ colIdx,
                                                          const double *__restrict__ val, const double *__restrict__ sc,
                                                          float *__restrict__ sval)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t sl = i >> 5;
        const int32_t e0 = sptr[sl];
        const int w = (sptr[sl + 1] - e0) >> 5;
        const double si = sc[i];
        for (int k = 0; k < w; ++k) {
            const int64_t e = static_cast<int64_t>(e0) + static_cast<int64_t>(k) * 32 + (i & 31);
            const int pos = spos[e];
            sval[e] = pos >= 0 ? static_cast<float>(val[pos] * si * sc[colIdx[pos]]) : 0.0f;
        }
    }
}

// Thread 0 of the last CTA of an init: the solve's scalars from |S b|^2
// (FP32 rows) and |b|^2.
__device__ void mx_start(SolveScalars *s, double sbb, double bb)
{
    const double bn = sqrt(bb);
    s->bnorm = std_max(bn, 1e-30);
    s->rz = sbb;
    s->sigma0 = sqrt(sbb);
    s->rmax = s->sigma0;
    s->smin = s->sigma0;
    s->stall = 0;
    s->t0 = bn / s->bnorm;
    s->last = s->t0;
    s->rr = bb;
    s->alpha = 0.0;
    s->beta = 0.0;
    s->iter = 0;
    s->updates = 0;
    s->need_update = 2;  // run the first (FRESH) step; not counted as an update
    s->seen = -1;
    s->status = SIMALL_OK;
    s->done = 0;
    s->result = 0;
    if (s->t0 < s->tol) {
        s->done = 1;  // b == 0: x = 0 is exact
    } else if (s->max_iter <= 0) {
        s->done = 1;
        s->result = s->max_iter;
    }
}

// ---------------------------------------------------------------- iteration kernels
// Init: x = 0, r = S b (into r[0]), p_old = 0 (p[1]), xh = 0, beta = 0;
// ||b||.  The first step is a FRESH step of parity 1 (reads r[0] and p[1]).
__global__ void __launch_bounds__(kBlock) k_mx_init(int64_t n, const double *__restrict__ b,
                                                    const double *__restrict__ sc, double *__restrict__ x,
                                                    float *__restrict__ r0, float *__restrict__ p1,
                                                    float *__restrict__ xh, double *partials, SolveScalars *s)
{
    float a0 = 0.0f;
    double a1 = 0.0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const double bi = b[i];
        const float r = static_cast<float>(bi * sc[i]);
        x[i] = 0.0;
        r0[i] = r;
        p1[i] = 0.0f;
        xh[i] = 0.0f;
        a0 += r * r;
        a1 += bi * bi;
    }
    double acc[2] = {static_cast<double>(a0), a1};
    if (grid_sum_last<2>(acc, partials, &s->counter[0]) && threadIdx.x == 0)
        mx_start(s, acc[0], acc[1]);
}

// ---------------------------------------------------------------- the fused iteration
// One kernel per CG step.  With the step length alpha and beta of the
// previous step (device scalars), every row forms
//     r = r_old - alpha q_old,  p = r + beta p_old,  xh += alpha p_old,
// then q = (S A S) p and the sums p.q, q.q, r.r, r.q.  A neighbour's p is
// formed again from its r_old, q_old, p_old with the same two fused
// multiply-adds, so every thread that forms p_j gets the same bits.  The
// vectors are double-buffered (read *_in, write *_out); the host alternates
// the two buffers between launches.
//
// FRESH: the step after a residual replacement (and the first step): r is
// the replaced residual, read from r_out and not rewritten; alpha = 0.

// Thread 0 of the last CTA: alpha = r.r / p.q and beta of the next step,
// beta = |r - alpha q|^2 / r.r with |r - alpha q|^2 = rr - 2 alpha rq + alpha^2 qq.
__device__ __forceinline__ void mx_step(SolveScalars *s, double pq, double qq, double rr, double rq)
{
    s->pAp = pq;
    if (!(pq > 0.0) || !(rr > 0.0)) {
        // not SPD in FP32, or exact breakdown: fold in what we have and stop
        s->status = SIMALL_ERR_BREAKDOWN;
        s->need_update = 1;
        s->alpha = 0.0;
        s->beta = 0.0;
        return;
    }
    const double alpha = rr / pq;
    const double next = rr - 2.0 * alpha * rq + alpha * alpha * qq;
    s->alpha = alpha;
    s->beta = (next > 0.0 ? next : 0.0) / rr;
}

// Thread 0 of the last CTA of a step.
template <bool FRESH>
__device__ __forceinline__ void mx_finish(SolveScalars *s, const double (&t)[4])
{
    const double pq = t[0], qq = t[1], rr = t[2], rq = t[3];
    if (FRESH) {
        // r is the replaced (true) residual; restart the update trigger
        s->rz = rr;
        s->sigma0 = sqrt(rr);
        s->rmax = s->sigma0;
        s->smin = s->sigma0;
        s->stall = 0;
        if (s->need_update == 1)
            s->updates += 1;
        s->need_update = 0;
        mx_step(s, pq, qq, rr, rq);
        return;
    }
    s->iter += 1;
    const double sigma = sqrt(rr);
    const double est = s->t0 * sigma / s->sigma0;
    s->last = est;
    if (sigma < s->smin) {
        s->smin = sigma;
        s->stall = 0;
    } else {
        s->stall += 1;
    }
    if (s->need_update || sigma < s->delta * s->rmax || est < s->tol || s->iter >= s->max_iter ||
        s->stall >= kMixedStallSteps) {
        s->need_update = 1;  // fold, true residual, replacement, then a FRESH step
        return;
    }
    if (sigma > s->rmax)
        s->rmax = sigma;
    s->rz = rr;
    mx_step(s, pq, qq, rr, rq);
}

template <bool FRESH> __device__ __forceinline__ bool mx_skip(const SolveScalars *s)
{
    return ld_flag(&s->done) || (FRESH && !ld_flag(&s->need_update));
}

// Condition handles of the device-side loop: a graph WHILE node over pairs of
// steps, each step followed by this controller and an IF node holding the
// reliable-update kernels.
struct CondHandles {
    cudaGraphConditionalHandle loop;
    cudaGraphConditionalHandle branch;
};

// One thread after each step: run the reliable-update branch when the step
// asked for it; keep looping unless the solve is done.  The loop also ends
// when a step made no progress (the iteration count did not move since the
// previous controller ran -- unreachable, since every step that is not done
// counts) or the count passed max_iter + 4 (also unreachable: the true-
// residual stop test ends the solve at max_iter).  Keeping the device-side
// graph calls out of the step kernel leaves its registers to the step.
__global__ void k_mx_control(SolveScalars *s, CondHandles c)
{
    if (threadIdx.x != 0)
        return;
    const int iter = ld_flag(&s->iter);
    const bool stop = ld_flag(&s->done) || iter - 4 > ld_flag(&s->max_iter) || iter == s->seen;
    s->seen = iter;
    cudaGraphSetConditional(c.branch, (!stop && ld_flag(&s->need_update)) ? 1u : 0u);
    cudaGraphSetConditional(c.loop, stop ? 0u : 1u);
}

// The step of dia_step.cuh as one kernel of the per-step engine: the sums
// finished by the last CTA (mx_finish).
template <int ND, bool GRID, bool FRESH>
__global__ void __launch_bounds__(kBlock, 3) k_mx_iter_dia(int n, int64_t ldU, DiaOffsets o, const float *__restrict__ U,
                                                        const float *__restrict__ e, IterVecs v, double *partials,
                                                        SolveScalars *s)
{
    if (mx_skip<FRESH>(s))
        return;
    const float alpha = FRESH ? 0.0f : static_cast<float>(__ldcg(&s->alpha));
    const float beta = static_cast<float>(__ldcg(&s->beta));
    float acc[4] = {0.0f, 0.0f, 0.0f, 0.0f};  // p.q, q.q, r.r, r.q
    dia_step<ND, GRID, FRESH, false>(n, ldU, o, U, e, v, alpha, beta, acc);
    double t[4];
    if (grid_sum_last_fv<4>(acc, partials, &s->counter[1], t) && threadIdx.x == 0)
        mx_finish<FRESH>(s, t);
}

// Sliced storage (sell.cuh): a warp per slice of 32 rows, grid-stride over
// the slices; the packed state of step parity par is read from `in`, the
// next written to `out`.  FRESH (after a replacement): alpha = 0.
template <bool FRESH, bool WIDE>
__global__ void __launch_bounds__(kBlock) k_mx_iter_sell(SellOp A, const float4 *in, float4 *out, double *partials,
                                                         SolveScalars *s)
{
    if (mx_skip<FRESH>(s))
        return;
    const float alpha = FRESH ? 0.0f : static_cast<float>(__ldcg(&s->alpha));
    const float beta = static_cast<float>(__ldcg(&s->beta));
    FF acc[4] = {ff_zero(), ff_zero(), ff_zero(), ff_zero()};
    const int64_t nw = (static_cast<int64_t>(gridDim.x) * blockDim.x) >> 5;
    for (int64_t sl = (blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x) >> 5; sl < A.nslices; sl += nw)
        sell_slice<WIDE, true>(A, sl, in, out, alpha, beta, acc);
    double t[4];
    if (ff_grid_sum_last<4>(acc, reinterpret_cast<FF *>(partials), &s->counter[1], t) && threadIdx.x == 0)
        mx_finish<FRESH>(s, t);
}

// The same step with the streamed operands staged by bulk copies
// (sell_step_staged); CTA b owns slices [b nslices / grid, (b + 1) nslices /
// grid).  A copy that does not complete in time ends the solve with
// SIMALL_ERR_TIMEOUT.
template <bool FRESH, bool WIDE>
__global__ void __launch_bounds__(kSellThreads) k_mx_iter_sell_staged(SellOp A, const float4 *in, float4 *out,
                                                                      double *partials, SolveScalars *s)
{
    extern __shared__ __align__(128) unsigned char sell_smem[];
    __shared__ uint64_t bars[2 * kSellStages];
    __shared__ int skip;
    if (threadIdx.x == 0)  // one decision per CTA: a timed-out CTA of this launch may raise done meanwhile
        skip = mx_skip<FRESH>(s) ? 1 : 0;
    __syncthreads();
    if (skip)
        return;
    if (threadIdx.x == 0)
        sell_ring_init(bars);
    __syncthreads();
    SellRing<WIDE> R{reinterpret_cast<SellStageBuf<WIDE> *>(sell_smem), bars, 0};
    const float alpha = FRESH ? 0.0f : static_cast<float>(__ldcg(&s->alpha));
    const float beta = static_cast<float>(__ldcg(&s->beta));
    const int64_t c0 = blockIdx.x * A.nslices / gridDim.x, c1 = (blockIdx.x + 1) * A.nslices / gridDim.x;
    FF acc[4] = {ff_zero(), ff_zero(), ff_zero(), ff_zero()};
    const bool ok = __syncthreads_and(sell_step_staged<WIDE, true>(A, c0, c1, in, out, alpha, beta, acc, R, false));
    if (!ok && threadIdx.x == 0) {
        atomicExch(&s->status, SIMALL_ERR_TIMEOUT);
        atomicExch(&s->done, 1);
    }
    double t[4];
    if (ff_grid_sum_last<4>(acc, reinterpret_cast<FF *>(partials), &s->counter[1], t) && threadIdx.x == 0 &&
        !ld_flag(&s->done))
        mx_finish<FRESH>(s, t);
}

// Sliced storage, packed state: init (x = 0, state[1] = (S b, 0, 0, 0): the
// first step, a FRESH one at parity 1, forms p = r), and the update kernels:
// fold x += S xh with the xh the triggering step wrote (state[1 - par]), and
// the replacement r = S (b - A x), xh = 0 written into state[par], which the
// FRESH step reads.
__global__ void __launch_bounds__(kBlock) k_mx_init_packed(int64_t n, const double *__restrict__ b,
                                                           const double *__restrict__ sc, double *__restrict__ x,
                                                           float4 *__restrict__ st1, double *partials, SolveScalars *s)
{
    float a0 = 0.0f;
    double a1 = 0.0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const double bi = b[i];
        const float r = static_cast<float>(bi * sc[i]);
        x[i] = 0.0;
        st1[i] = make_float4(r, 0.0f, 0.0f, 0.0f);
        a0 += r * r;
        a1 += bi * bi;
    }
    double acc[2] = {static_cast<double>(a0), a1};
    if (grid_sum_last<2>(acc, partials, &s->counter[0]) && threadIdx.x == 0)
        mx_start(s, acc[0], acc[1]);
}

__global__ void __launch_bounds__(kBlock) k_mx_fold_packed(int64_t n, const double *__restrict__ sc,
                                                           const float4 *__restrict__ st, double *__restrict__ x,
                                                           const SolveScalars *s)
{
    if (!ld_flag(&s->need_update) || ld_flag(&s->done))
        return;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        x[i] += sc[i] * static_cast<double>(st[i].w);
}

__global__ void __launch_bounds__(kBlock) k_mx_replace_packed(int64_t n, const double *__restrict__ sc,
                                                              const double *__restrict__ r, float4 *__restrict__ st,
                                                              double *partials, SolveScalars *s)
{
    if (!ld_flag(&s->need_update) || ld_flag(&s->done))
        return;
    float acc = 0.0f;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const float v = static_cast<float>(sc[i] * r[i]);
        float *e = reinterpret_cast<float *>(st + i);
        e[0] = v;
        e[3] = 0.0f;
        acc += v * v;
    }
    double rho;
    if (grid_sum_last_f(acc, partials, &s->counter[4], rho) && threadIdx.x == 0)
        s->beta = rho / s->rz;
}

// U1: x += S xh (FP64), xh = 0.
__global__ void __launch_bounds__(kBlock) k_mx_fold(int64_t n, const double *__restrict__ sc, float *__restrict__ xh,
                                                    double *__restrict__ x, const SolveScalars *s)
{
    if (!ld_flag(&s->need_update) || ld_flag(&s->done))
        return;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        x[i] += sc[i] * static_cast<double>(xh[i]);
        xh[i] = 0.0f;
    }
}

// U2: r = b - A x in FP64 (staged CSR SpMV, one FMA per entry); stop test on
// the true residual.
struct ResEpi {
    const double *b;
    double *r;
    double acc;
    __device__ __forceinline__ void operator()(int row, double y)
    {
        const double v = __ldg(b + row) - y;
        r[row] = v;
        acc += v * v;
    }
};

__global__ void __launch_bounds__(kBlock) k_mx_true_residual(const int32_t *__restrict__ rowPtr,
                                                             const int32_t *__restrict__ colIdx,
                                                             const double *__restrict__ val,
                                                             const int32_t *__restrict__ rb, int nRB,
                                                             const double *__restrict__ x, const double *__restrict__ b,
                                                             double *__restrict__ r, double *partials, SolveScalars *s)
{
    if (!ld_flag(&s->need_update) || ld_flag(&s->done))
        return;
    ResEpi epi{b, r, 0.0};
    spmv_rowblocks_fma(rowPtr, colIdx, val, rb, nRB, x, epi);  // one FMA per entry: GB300's FP64 pipe is narrow
    double v[1] = {epi.acc};
    if (grid_sum_last<1>(v, partials, &s->counter[3]) && threadIdx.x == 0) {
        s->rr = v[0];
        const double t = sqrt(v[0]) / s->bnorm;
        s->last = t;
        s->t0 = t;
        if (t < s->tol) {
            s->done = 1;
            s->result = s->iter;
        } else if (s->iter >= s->max_iter || s->status == SIMALL_ERR_BREAKDOWN) {
            s->done = 1;
            s->result = s->iter >= s->max_iter ? s->max_iter : s->iter;
        }
    }
}

// U3: r_out = S r (FP32), beta = |S r|^2 / r.r of the last step; the FRESH
// step that follows forms p = r_out + beta p_in and resets the trigger.
__global__ void __launch_bounds__(kBlock) k_mx_replace(int64_t n, const double *__restrict__ sc,
                                                       const double *__restrict__ r, float *__restrict__ rout,
                                                       double *partials, SolveScalars *s)
{
    if (!ld_flag(&s->need_update) || ld_flag(&s->done))
        return;
    float acc = 0.0f;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const float v = static_cast<float>(sc[i] * r[i]);
        rout[i] = v;
        acc += v * v;
    }
    double rho;
    if (grid_sum_last_f(acc, partials, &s->counter[4], rho) && threadIdx.x == 0)
        s->beta = rho / s->rz;
}

int grid_n(simall_context *ctx, int64_t n)
{
    const int64_t g = (n + kBlock - 1) / kBlock;
    const int64_t cap = grid_size_streaming(ctx);
    return static_cast<int>(g < 1 ? 1 : (g < cap ? g : cap));
}

// Distinct upper-triangle offsets j - i of the pattern (a table of
// kOffTable slots, empty = INT_MIN), the count of upper entries, and an
// overflow flag when there are more than kMaxDiags distinct offsets.
constexpr int kOffTable = 16;

__device__ __forceinline__ bool table_insert(int *tab, int off)
{
    for (int s = 0; s < kOffTable; ++s) {
        const int cur = tab[s];
        if (cur == off)
            return true;
        if (cur == INT_MIN) {
            const int prev = atomicCAS(tab + s, INT_MIN, off);
            if (prev == INT_MIN || prev == off)
                return true;
        }
    }
    return false;
}

__global__ void __launch_bounds__(kBlock) k_mx_offsets(int64_t n, const int32_t *__restrict__ rowPtr,
                                                       const int32_t *__restrict__ colIdx, int *table,
                                                       unsigned long long *upper, int *overflow)
{
    __shared__ int stab[kOffTable];
    __shared__ int sover;
    __shared__ unsigned long long scount;
    if (threadIdx.x < kOffTable)
        stab[threadIdx.x] = INT_MIN;
    if (threadIdx.x == 0) {
        sover = 0;
        scount = 0ull;
    }
    __syncthreads();
    int local[kMaxDiags];
    int nl = 0;
    bool over = false;
    unsigned long long cnt = 0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        for (int k = rowPtr[i]; k < rowPtr[i + 1]; ++k) {
            const int j = colIdx[k];
            if (j <= i)
                continue;
            ++cnt;
            const int off = j - static_cast<int>(i);
            bool seen = false;
            for (int t = 0; t < nl; ++t)
                seen |= (local[t] == off);
            if (!seen) {
                if (nl < kMaxDiags)
                    local[nl++] = off;
                else
                    over = true;
            }
        }
    for (int t = 0; t < nl; ++t)
        if (!table_insert(stab, local[t]))
            over = true;
    if (over)
        atomicOr(&sover, 1);
    atomicAdd(&scount, cnt);
    __syncthreads();
    if (threadIdx.x < kOffTable && stab[threadIdx.x] != INT_MIN)
        if (!table_insert(table, stab[threadIdx.x]))
            atomicOr(overflow, 1);
    if (threadIdx.x == 0) {
        atomicAdd(upper, scount);
        if (sover)
            atomicOr(overflow, 1);
    }
}

// The sliced storage's pattern from a host copy of A's: slice widths, each
// stored entry's CSR position (-1 for padding) and column offset, narrow
// offsets when every |j - i| fits 16 bits.
int build_sell_pattern(simall_solver *s, MixedData *m)
{
    simall_context *ctx = s->ctx;
    const int64_t n = s->n;
    int st = solver_host_pattern(s);
    if (st)
        return st;
    const int32_t *rp = s->h_rowPtr.data(), *ci = s->h_colIdx.data();
    const int64_t ns = (n + 31) / 32;
    std::vector<int32_t> sptr(static_cast<size_t>(ns) + 1, 0);
    int64_t total = 0;
    for (int64_t sl = 0; sl < ns; ++sl) {
        int w = 0;
        for (int64_t i = sl * 32; i < std::min(n, sl * 32 + 32); ++i) {
            int c = 0;
            for (int k = rp[i]; k < rp[i + 1]; ++k)
                c += ci[k] != i ? 1 : 0;
            w = std::max(w, c);
        }
        sptr[sl] = static_cast<int32_t>(total);
        total += 32 * static_cast<int64_t>(w);
        if (total > INT32_MAX)
            return fail(ctx, SIMALL_ERR_UNSUPPORTED, "mixed precision: sliced storage above 2^31 entries");
    }
    sptr[ns] = static_cast<int32_t>(total);
    std::vector<int32_t> pos(static_cast<size_t>(total), -1), off(static_cast<size_t>(total), 0);
    int64_t band = 0;
    for (int64_t i = 0; i < n; ++i) {
        int64_t e = sptr[i >> 5] + (i & 31);
        for (int k = rp[i]; k < rp[i + 1]; ++k)
            if (ci[k] != i) {
                pos[e] = k;
                off[e] = static_cast<int32_t>(ci[k] - i);
                band = std::max<int64_t>(band, std::abs(static_cast<int64_t>(off[e])));
                e += 32;
            }
    }
    m->nslices = ns;
    m->sEntries = total;
    m->sMaxW = 0;
    for (int64_t sl = 0; sl < ns; ++sl)
        m->sMaxW = std::max(m->sMaxW, (sptr[sl + 1] - sptr[sl]) >> 5);
    m->sWide = band > 32767;
    const size_t cap = static_cast<size_t>(std::max<int64_t>(total, 1));
    SIMALL_CUDA_TRY(ctx, m->sptr.alloc(static_cast<size_t>(ns) + 1));
    SIMALL_CUDA_TRY(ctx, m->spos.alloc(cap));
    SIMALL_CUDA_TRY(ctx, m->sval.alloc(cap));
    SIMALL_CUDA_TRY(ctx, cudaMemcpyAsync(m->sptr.p, sptr.data(), sptr.size() * sizeof(int32_t),
                                         cudaMemcpyHostToDevice, ctx->stream));
    std::vector<int16_t> off16;
    if (total > 0) {
        SIMALL_CUDA_TRY(ctx, cudaMemcpyAsync(m->spos.p, pos.data(), pos.size() * sizeof(int32_t),
                                             cudaMemcpyHostToDevice, ctx->stream));
        if (m->sWide) {
            SIMALL_CUDA_TRY(ctx, m->soff32.alloc(cap));
            SIMALL_CUDA_TRY(ctx, cudaMemcpyAsync(m->soff32.p, off.data(), off.size() * sizeof(int32_t),
                                                 cudaMemcpyHostToDevice, ctx->stream));
        } else {
            off16.assign(off.begin(), off.end());
            SIMALL_CUDA_TRY(ctx, m->soff16.alloc(cap));
            SIMALL_CUDA_TRY(ctx, cudaMemcpyAsync(m->soff16.p, off16.data(), off16.size() * sizeof(int16_t),
                                                 cudaMemcpyHostToDevice, ctx->stream));
        }
    }
    SIMALL_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));  // the host arrays die here
    return SIMALL_OK;
}

SellOp sell_op(const simall_solver *s, const MixedData *m)
{
    SellOp A;
    A.n = s->n;
    A.nslices = m->nslices;
    A.sptr = m->sptr.p;
    A.off16 = m->soff16.p;
    A.off32 = m->soff32.p;
    A.val = m->sval.p;
    A.e = m->e.p;
    A.prefetch = g_sell_prefetch;
    return A;
}

// Choose the storage format of S A S from the pattern (diagonal storage only
// if allowed).  The diagonal test runs on the device; the CSR fallback is
// built from a host copy of the pattern.
int analyse_pattern(simall_solver *s, MixedData *m, bool allow_dia)
{
    simall_context *ctx = s->ctx;
    const int64_t n = s->n;
    std::vector<int32_t> offs;
    bool ok = allow_dia;
    if (ok) {
        DevBuf<int> tab;
        DevBuf<unsigned long long> cnt;
        SIMALL_CUDA_TRY(ctx, tab.alloc(kOffTable + 1));
        SIMALL_CUDA_TRY(ctx, cnt.alloc(1));
        std::vector<int> init(kOffTable + 1, INT_MIN);
        init[kOffTable] = 0;
        SIMALL_CUDA_TRY(ctx, cudaMemcpyAsync(tab.p, init.data(), init.size() * sizeof(int), cudaMemcpyHostToDevice,
                                             ctx->stream));
        SIMALL_CUDA_TRY(ctx, cudaMemsetAsync(cnt.p, 0, sizeof(unsigned long long), ctx->stream));
        k_mx_offsets<<<grid_n(ctx, n), kBlock, 0, ctx->stream>>>(n, s->rowPtr, s->colIdx, tab.p, cnt.p,
                                                                 tab.p + kOffTable);
        SIMALL_LAUNCH_CHECK(ctx);
        std::vector<int> h(kOffTable + 1);
        unsigned long long upper = 0;
        SIMALL_CUDA_TRY(ctx, cudaMemcpyAsync(h.data(), tab.p, h.size() * sizeof(int), cudaMemcpyDeviceToHost,
                                             ctx->stream));
        SIMALL_CUDA_TRY(ctx, cudaMemcpyAsync(&upper, cnt.p, sizeof(upper), cudaMemcpyDeviceToHost, ctx->stream));
        SIMALL_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
        for (int t = 0; t < kOffTable; ++t)
            if (h[t] != INT_MIN)
                offs.push_back(h[t]);
        ok = !h[kOffTable] && !offs.empty() && static_cast<int>(offs.size()) <= kMaxDiags &&
             static_cast<double>(offs.size()) * n <= 1.3 * static_cast<double>(upper);
    }
    m->dia = ok;
    if (m->dia) {
        std::sort(offs.begin(), offs.end());
        m->offs.nd = static_cast<int>(offs.size());
        for (int d = 0; d < kMaxDiags; ++d)
            m->offs.off[d] = d < m->offs.nd ? offs[d] : 0;
    } else {
        int st = build_sell_pattern(s, m);
        if (st)
            return st;
    }
    m->patternReady = true;
    return SIMALL_OK;
}

IterVecs iter_vecs(MixedData *m, int par)
{
    IterVecs v;
    v.rin = m->rv[par].p;
    v.qin = m->qv[par].p;
    v.pin = m->pv[par].p;
    v.rout = m->rv[1 - par].p;
    v.qout = m->qv[1 - par].p;
    v.pout = m->pv[1 - par].p;
    v.xh = m->xh.p;
    return v;
}

}  // namespace

// Resident CTAs per SM of a kernel of `threads` threads with `smem` bytes of
// dynamic shared memory (raising its limit first); cached per context and kernel.
int staged_residency(simall_context *ctx, const void *fn, int threads, size_t smem, int *per_sm)
{
    std::lock_guard<std::mutex> lock(ctx->occupancy_mu);
    auto it = ctx->resident_per_sm.find(fn);
    if (it != ctx->resident_per_sm.end()) {
        *per_sm = it->second;
        return SIMALL_OK;
    }
    SIMALL_CUDA_TRY(ctx, cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem)));
    int n = 0;
    SIMALL_CUDA_TRY(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, fn, threads, smem));
    if (n < 1)
        return fail(ctx, SIMALL_ERR_CUDA, "a staged kernel does not fit on an SM");
    ctx->resident_per_sm.emplace(fn, n);
    *per_sm = n;
    return SIMALL_OK;
}

namespace {

template <bool FRESH> int launch_iter_t(simall_context *ctx, simall_solver *s, MixedData *m, int par)
{
    const int64_t n = s->n;
    if (!m->dia) {
        const SellOp A = sell_op(s, m);
        const float4 *in = m->st[par].p;
        float4 *out = m->st[1 - par].p;
        if (m->sMaxW <= kSellStageMaxW) {
            const size_t smem = m->sWide ? sell_stage_smem<true>() : sell_stage_smem<false>();
            const void *fn = m->sWide ? reinterpret_cast<const void *>(k_mx_iter_sell_staged<FRESH, true>)
                                      : reinterpret_cast<const void *>(k_mx_iter_sell_staged<FRESH, false>);
            int per_sm = 0;
            int st = staged_residency(ctx, fn, kSellThreads, smem, &per_sm);
            if (st)
                return st;
            const int64_t stages = (m->nslices + kSellStageSlices - 1) / kSellStageSlices;
            const int grid = static_cast<int>(std::max<int64_t>(
                1, std::min<int64_t>(stages, static_cast<int64_t>(ctx->num_sms) * per_sm)));
            if (m->sWide)
                k_mx_iter_sell_staged<FRESH, true>
                    <<<grid, kSellThreads, smem, ctx->stream>>>(A, in, out, s->partials.p, s->scal.p);
            else
                k_mx_iter_sell_staged<FRESH, false>
                    <<<grid, kSellThreads, smem, ctx->stream>>>(A, in, out, s->partials.p, s->scal.p);
            SIMALL_LAUNCH_CHECK(ctx);
            return SIMALL_OK;
        }
        const void *fn = m->sWide ? reinterpret_cast<const void *>(k_mx_iter_sell<FRESH, true>)
                                  : reinterpret_cast<const void *>(k_mx_iter_sell<FRESH, false>);
        const int grid = resident_grid(ctx, fn, m->nslices * 32);
        if (m->sWide)
            k_mx_iter_sell<FRESH, true><<<grid, kBlock, 0, ctx->stream>>>(A, in, out, s->partials.p, s->scal.p);
        else
            k_mx_iter_sell<FRESH, false><<<grid, kBlock, 0, ctx->stream>>>(A, in, out, s->partials.p, s->scal.p);
        SIMALL_LAUNCH_CHECK(ctx);
        return SIMALL_OK;
    }
    const IterVecs v = iter_vecs(m, par);
    const int64_t quads = (n + 3) / 4;
    const int ni = static_cast<int>(n);
    bool grid = m->offs.nd >= 1 && m->offs.off[0] == 1;
    for (int d = 1; d < m->offs.nd; ++d)
        grid = grid && (m->offs.off[d] & 3) == 0;
    switch (m->offs.nd) {
#define SIMALL_DIA_CASE(ND)                                                                                           \
    case ND:                                                                                                          \
        if (grid) {                                                                                                   \
            const void *fn = reinterpret_cast<const void *>(k_mx_iter_dia<ND, true, FRESH>);                          \
            k_mx_iter_dia<ND, true, FRESH><<<resident_grid(ctx, fn, quads), kBlock, 0, ctx->stream>>>(                \
                ni, m->ldU, m->offs, m->U.p, m->e.p, v, s->partials.p, s->scal.p);                                    \
        } else {                                                                                                      \
            const void *fn = reinterpret_cast<const void *>(k_mx_iter_dia<ND, false, FRESH>);                         \
            k_mx_iter_dia<ND, false, FRESH><<<resident_grid(ctx, fn, quads), kBlock, 0, ctx->stream>>>(               \
                ni, m->ldU, m->offs, m->U.p, m->e.p, v, s->partials.p, s->scal.p);                                    \
        }                                                                                                             \
        break;
        SIMALL_DIA_CASE(1)
        SIMALL_DIA_CASE(2)
        SIMALL_DIA_CASE(3)
        SIMALL_DIA_CASE(4)
        SIMALL_DIA_CASE(5)
        SIMALL_DIA_CASE(6)
        SIMALL_DIA_CASE(7)
        SIMALL_DIA_CASE(8)
#undef SIMALL_DIA_CASE
    default:
        return fail(ctx, SIMALL_ERR_INVALID_ARGUMENT, "dia storage with %d diagonals", m->offs.nd);
    }
    SIMALL_LAUNCH_CHECK(ctx);
    return SIMALL_OK;
}

// One CG step of parity `par` (reads buffers [par], writes [1 - par]).
int launch_iter(simall_context *ctx, simall_solver *s, int par, bool fresh)
{
    return fresh ? launch_iter_t<true>(ctx, s, s->mixed, par) : launch_iter_t<false>(ctx, s, s->mixed, par);
}

}  // namespace

int mixed_setup(simall_solver *s)
{
    simall_context *ctx = s->ctx;
    if (!s->mixed) {
        s->mixed = new (std::nothrow) MixedData;
        if (!s->mixed)
            return SIMALL_ERR_OUT_OF_MEMORY;
    }
    MixedData *m = s->mixed;
    const int64_t n = s->n;
    if (!m->patternReady) {
        int st = analyse_pattern(s, m, true);
        if (st)
            return st;
    }
    SIMALL_CUDA_TRY(ctx, m->scale.alloc(n));
    SIMALL_CUDA_TRY(ctx, s->flag.alloc(1));
    SIMALL_CUDA_TRY(ctx, cudaMemsetAsync(s->flag.p, 0, sizeof(int), ctx->stream));
    const int g = grid_n(ctx, n);
    k_mx_scale<<<g, kBlock, 0, ctx->stream>>>(n, s->rowPtr, s->colIdx, s->values, m->scale.p, s->flag.p);
    SIMALL_LAUNCH_CHECK(ctx);
    if (m->dia) {
        k_mx_symcheck<<<g, kBlock, 0, ctx->stream>>>(n, s->rowPtr, s->colIdx, s->values, s->flag.p);
        SIMALL_LAUNCH_CHECK(ctx);
    }
    int h = 0;
    SIMALL_CUDA_TRY(ctx, cudaMemcpyAsync(&h, s->flag.p, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    SIMALL_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
    if (h & 1)
        return fail(ctx, SIMALL_ERR_NOT_POSITIVE, "mixed precision needs a positive diagonal");
    if (m->dia && (h & 2)) {
        int st = analyse_pattern(s, m, false);  // not numerically symmetric: keep every off-diagonal entry
        if (st)
            return st;
    }
    // the iteration vectors of the storage the solve will use
    if (m->dia) {
        SIMALL_CUDA_TRY(ctx, m->xh.alloc(n + 4));
        for (int k = 0; k < 2; ++k) {
            SIMALL_CUDA_TRY(ctx, m->rv[k].alloc(n + 4));
            SIMALL_CUDA_TRY(ctx, m->qv[k].alloc(n + 4));
            SIMALL_CUDA_TRY(ctx, m->pv[k].alloc(n + 4));
        }
    } else {
        for (int k = 0; k < 2; ++k)
            SIMALL_CUDA_TRY(ctx, m->st[k].alloc(n));
    }
    {
        // diagonal storage: n + 4 (the quad loads); sliced: whole slices, zero past n
        const int64_t ne = m->dia ? n + 4 : m->nslices * 32;
        SIMALL_CUDA_TRY(ctx, m->e.alloc(ne));
        if (!m->dia)
            SIMALL_CUDA_TRY(ctx, cudaMemsetAsync(m->e.p, 0, ne * sizeof(float), ctx->stream));
        k_mx_row_defect<<<g, kBlock, 0, ctx->stream>>>(n, s->rowPtr, s->colIdx, s->values, m->scale.p, m->e.p);
        SIMALL_LAUNCH_CHECK(ctx);
    }
    if (m->dia) {
        m->ldU = (n + 3) & ~static_cast<int64_t>(3);
        SIMALL_CUDA_TRY(ctx, m->U.alloc(static_cast<size_t>(m->offs.nd) * m->ldU));
        SIMALL_CUDA_TRY(ctx, cudaMemsetAsync(m->U.p, 0, static_cast<size_t>(m->offs.nd) * m->ldU * sizeof(float),
                                             ctx->stream));
        k_mx_build_dia<<<g, kBlock, 0, ctx->stream>>>(n, m->ldU, s->rowPtr, s->colIdx, s->values, m->scale.p, m->offs,
                                                      m->U.p);
        SIMALL_LAUNCH_CHECK(ctx);
    } else if (m->sEntries > 0) {
        k_mx_build_sell<<<g, kBlock, 0, ctx->stream>>>(n, m->sptr.p, m->spos.p, s->colIdx, s->values, m->scale.p,
                                                       m->sval.p);
        SIMALL_LAUNCH_CHECK(ctx);
    }
    return SIMALL_OK;
}

namespace {

// The reliable-update kernels after a step of parity `par`: fold, true
// residual, replacement, FRESH step.  Each returns at once unless the step
// raised need_update.
int enqueue_update_branch(simall_solver *s, int par)
{
    simall_context *ctx = s->ctx;
    MixedData *m = s->mixed;
    const int64_t n = s->n;
    const int g = grid_n(ctx, n);
    if (m->dia)
        k_mx_fold<<<g, kBlock, 0, ctx->stream>>>(n, m->scale.p, m->xh.p, s->x.p, s->scal.p);
    else
        k_mx_fold_packed<<<g, kBlock, 0, ctx->stream>>>(n, m->scale.p, m->st[1 - par].p, s->x.p, s->scal.p);
    SIMALL_LAUNCH_CHECK(ctx);
    k_mx_true_residual<<<resident_grid(ctx, reinterpret_cast<const void *>(k_mx_true_residual),
                                       spmv_items(s)),
                         kBlock, 0, ctx->stream>>>(s->rowPtr, s->colIdx, s->values, s->rowBlocks.p, spmv_schedule(s),
                                                   s->x.p, s->b.p, s->r.p, s->partials.p, s->scal.p);
    SIMALL_LAUNCH_CHECK(ctx);
    if (m->dia)
        k_mx_replace<<<g, kBlock, 0, ctx->stream>>>(n, m->scale.p, s->r.p, m->rv[1 - par].p, s->partials.p,
                                                    s->scal.p);
    else
        k_mx_replace_packed<<<g, kBlock, 0, ctx->stream>>>(n, m->scale.p, s->r.p, m->st[par].p, s->partials.p,
                                                           s->scal.p);
    SIMALL_LAUNCH_CHECK(ctx);
    return launch_iter(ctx, s, par, true);
}

// One step of parity `par` followed by its reliable-update kernels.  A
// solve's first step has parity 1 and every captured chunk has an even
// length, so every chunk starts at parity 0.
int enqueue_mixed_iteration(simall_solver *s, int par)
{
    int st = launch_iter(s->ctx, s, par, false);
    return st ? st : enqueue_update_branch(s, par);
}

constexpr int kMixedKernelsPerIteration = 5;
constexpr int kDeviceLoop = 0;  // GraphChunk::len of the device-side loop graph

// The whole iteration as one graph: WHILE(loop) { step(0); control;
// IF(b0) {update branch(0)}; step(1); control; IF(b1) {update branch(1)} }.
// The controllers set the conditions from the device, so a solve is one graph
// launch with no host round trip until it has finished.
int build_device_loop(simall_solver *s, cudaGraphExec_t *out)
{
    simall_context *ctx = s->ctx;
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaGraphCreate(&g, 0);
    if (e != cudaSuccess)
        return cuda_fail(ctx, e, "cudaGraphCreate", __FILE__, __LINE__);
    int st = SIMALL_OK;
    auto check = [&](cudaError_t err, const char *what) {
        if (err != cudaSuccess && st == SIMALL_OK)
            st = cuda_fail(ctx, err, what, __FILE__, __LINE__);
        return st == SIMALL_OK;
    };
    cudaGraphConditionalHandle loop = 0, branch[2] = {0, 0};
    cudaGraph_t body = nullptr, arm[2] = {nullptr, nullptr};
    if (check(cudaGraphConditionalHandleCreate(&loop, g, 1u, cudaGraphCondAssignDefault), "loop handle")) {
        cudaGraphNodeParams wp{};
        wp.type = cudaGraphNodeTypeConditional;
        wp.conditional.handle = loop;
        wp.conditional.type = cudaGraphCondTypeWhile;
        wp.conditional.size = 1;
        cudaGraphNode_t wn;
        if (check(cudaGraphAddNode(&wn, g, nullptr, nullptr, 0, &wp), "while node"))
            body = wp.conditional.phGraph_out[0];
    }
    for (int k = 0; k < 2 && st == SIMALL_OK; ++k)
        check(cudaGraphConditionalHandleCreate(&branch[k], body, 0u, cudaGraphCondAssignDefault), "branch handle");
    // the loop body: two steps, each followed by its IF node
    if (st == SIMALL_OK &&
        check(cudaStreamBeginCaptureToGraph(ctx->stream, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal),
              "capture body")) {
        for (int par = 0; par < 2 && st == SIMALL_OK; ++par) {
            st = launch_iter(ctx, s, par, false);
            if (st)
                break;
            k_mx_control<<<1, 32, 0, ctx->stream>>>(s->scal.p, CondHandles{loop, branch[par]});
            ctx->launches.fetch_add(1, std::memory_order_relaxed);
            if (!check(cudaGetLastError(), "controller launch"))
                break;
            cudaStreamCaptureStatus cs;
            const cudaGraphNode_t *deps = nullptr;
            size_t nd = 0;
            if (!check(cudaStreamGetCaptureInfo(ctx->stream, &cs, nullptr, nullptr, &deps, nullptr, &nd), "capture info"))
                break;
            cudaGraphNodeParams ip{};
            ip.type = cudaGraphNodeTypeConditional;
            ip.conditional.handle = branch[par];
            ip.conditional.type = cudaGraphCondTypeIf;
            ip.conditional.size = 1;
            cudaGraphNode_t in;
            if (!check(cudaGraphAddNode(&in, body, deps, nullptr, nd, &ip), "if node"))
                break;
            arm[par] = ip.conditional.phGraph_out[0];
            check(cudaStreamUpdateCaptureDependencies(ctx->stream, &in, nullptr, 1, cudaStreamSetCaptureDependencies),
                  "capture dependencies");
        }
        cudaGraph_t captured = nullptr;
        e = cudaStreamEndCapture(ctx->stream, &captured);
        check(e, "end body capture");
    }
    // the IF arms: the reliable-update kernels of each parity
    for (int par = 0; par < 2 && st == SIMALL_OK; ++par) {
        if (!check(cudaStreamBeginCaptureToGraph(ctx->stream, arm[par], nullptr, nullptr, 0,
                                                 cudaStreamCaptureModeThreadLocal),
                   "capture arm"))
            break;
        const int bst = enqueue_update_branch(s, par);
        cudaGraph_t captured = nullptr;
        e = cudaStreamEndCapture(ctx->stream, &captured);
        if (bst && st == SIMALL_OK)
            st = bst;
        check(e, "end arm capture");
    }
    if (st == SIMALL_OK)
        check(cudaGraphInstantiate(out, g, 0), "instantiate device loop");
    cudaGraphDestroy(g);
    return st;
}

int run_mixed_chunk(simall_solver *s, int len)
{
    simall_context *ctx = s->ctx;
    for (auto &gc : s->graphs)
        if (gc.len == len) {
            SIMALL_CUDA_TRY(ctx, cudaGraphLaunch(gc.exec, ctx->stream));
            ctx->launches.fetch_add(static_cast<int64_t>(len) * kMixedKernelsPerIteration, std::memory_order_relaxed);
            return SIMALL_OK;
        }
    cudaGraph_t graph = nullptr;
    SIMALL_CUDA_TRY(ctx, cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
    int st = SIMALL_OK;
    for (int i = 0; i < len && st == SIMALL_OK; ++i)
        st = enqueue_mixed_iteration(s, i & 1);
    cudaError_t e = cudaStreamEndCapture(ctx->stream, &graph);
    if (st)
        return st;
    if (e != cudaSuccess)
        return cuda_fail(ctx, e, "cudaStreamEndCapture", __FILE__, __LINE__);
    GraphChunk gc;
    gc.len = len;
    e = cudaGraphInstantiate(&gc.exec, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess)
        return cuda_fail(ctx, e, "cudaGraphInstantiate", __FILE__, __LINE__);
    s->graphs.push_back(gc);
    SIMALL_CUDA_TRY(ctx, cudaGraphLaunch(gc.exec, ctx->stream));
    return SIMALL_OK;
}

}  // namespace

int mixed_solve(simall_solver *s, simall_solver_stats *st)
{
    (void)st;
    simall_context *ctx = s->ctx;
    MixedData *m = s->mixed;
    const int64_t n = s->n;
    double tol = s->cfg.tolerance, delta = s->cfg.reliable_delta;
    int maxit = s->cfg.max_iterations;
    SIMALL_CUDA_TRY(ctx, cudaMemcpyAsync(&s->scal.p->tol, &tol, sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
    SIMALL_CUDA_TRY(ctx,
                    cudaMemcpyAsync(&s->scal.p->delta, &delta, sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
    SIMALL_CUDA_TRY(ctx,
                    cudaMemcpyAsync(&s->scal.p->max_iter, &maxit, sizeof(int), cudaMemcpyHostToDevice, ctx->stream));
    if (!m->dia && !m->noGrid && s->cfg.check_interval <= 0 && s->cfg.engine == SIMALL_ENGINE_AUTO) {
        const size_t cap = static_cast<size_t>(ctx->num_sms) * kGridMaxCtasPerSm * 8;
        if (m->gpart.n < cap)
            SIMALL_CUDA_TRY(ctx, m->gpart.alloc(cap));
        if (!m->gctr.p)
            SIMALL_CUDA_TRY(ctx, m->gctr.alloc(1));
        if (!m->gerr.p)
            SIMALL_CUDA_TRY(ctx, m->gerr.alloc(1));
        GridMixedArgs a{};
        a.nslices = m->nslices;
        a.wide = m->sWide;
        a.staged = m->sMaxW <= kSellStageMaxW;
        a.sptr = m->sptr.p;
        a.off16 = m->soff16.p;
        a.off32 = m->soff32.p;
        a.sval = m->sval.p;
        a.e = m->e.p;
        a.scale = m->scale.p;
        a.st[0] = m->st[0].p;
        a.st[1] = m->st[1].p;
        a.part = m->gpart.p;
        a.partCap = m->gpart.n;
        a.ctr = m->gctr.p;
        a.err = m->gerr.p;
        int gst = SIMALL_OK;
        if (grid_mixed_solve(s, a, &gst))
            return gst;
        m->noGrid = true;  // not available on this device: per-step kernels from now on
    }
    if (m->dia && s->cfg.check_interval <= 0 && s->cfg.engine == SIMALL_ENGINE_AUTO) {
        ClusterMixedArgs a{};
        a.U = m->U.p;
        a.ldU = m->ldU;
        a.nd = m->offs.nd;
        for (int d = 0; d < kMaxDiags && d < 8; ++d)
            a.off[d] = m->offs.off[d];
        a.e = m->e.p;
        a.scale = m->scale.p;
        int cst = SIMALL_OK;
        if (cluster_mixed_solve(s, a, &cst))
            return cst;
    }
    if (m->dia && !m->noGrid && s->cfg.check_interval <= 0 && s->cfg.engine == SIMALL_ENGINE_AUTO &&
        m->offs.nd <= kGridDiaMaxDiags) {
        const size_t cap = static_cast<size_t>(ctx->num_sms) * 8;
        if (m->gpart.n < cap)
            SIMALL_CUDA_TRY(ctx, m->gpart.alloc(cap));
        if (!m->gctr.p)
            SIMALL_CUDA_TRY(ctx, m->gctr.alloc(1));
        if (!m->gerr.p)
            SIMALL_CUDA_TRY(ctx, m->gerr.alloc(1));
        GridDiaArgs a{};
        a.nd = m->offs.nd;
        a.grid = m->offs.nd >= 1 && m->offs.off[0] == 1;
        for (int d = 0; d < m->offs.nd; ++d) {
            a.off[d] = m->offs.off[d];
            if (d >= 1)
                a.grid = a.grid && (m->offs.off[d] & 3) == 0;
        }
        a.ldU = m->ldU;
        a.U = m->U.p;
        a.e = m->e.p;
        a.scale = m->scale.p;
        for (int k = 0; k < 2; ++k) {
            a.rv[k] = m->rv[k].p;
            a.qv[k] = m->qv[k].p;
            a.pv[k] = m->pv[k].p;
        }
        a.xh = m->xh.p;
        a.part = m->gpart.p;
        a.partCap = m->gpart.n;
        a.ctr = m->gctr.p;
        a.err = m->gerr.p;
        int gst = SIMALL_OK;
        if (grid_dia_solve(s, a, &gst))
            return gst;
        m->noGrid = true;  // not available on this device: per-step kernels from now on
    }
    if (m->dia)
        k_mx_init<<<grid_n(ctx, n), kBlock, 0, ctx->stream>>>(n, s->b.p, m->scale.p, s->x.p, m->rv[0].p,
                                                              m->pv[1].p, m->xh.p, s->partials.p, s->scal.p);
    else
        k_mx_init_packed<<<grid_n(ctx, n), kBlock, 0, ctx->stream>>>(n, s->b.p, m->scale.p, s->x.p, m->st[1].p,
                                                                     s->partials.p, s->scal.p);
    SIMALL_LAUNCH_CHECK(ctx);
    int first = launch_iter(ctx, s, 1, true);
    if (first)
        return first;
    if (s->cfg.check_interval <= 0 && !m->noDeviceLoop) {
        cudaGraphExec_t ex = nullptr;
        for (auto &gc : s->graphs)
            if (gc.len == kDeviceLoop)
                ex = gc.exec;
        if (!ex) {
            if (build_device_loop(s, &ex) == SIMALL_OK) {
                GraphChunk gc;
                gc.len = kDeviceLoop;
                gc.exec = ex;
                s->graphs.push_back(gc);
            } else {
                m->noDeviceLoop = true;  // no conditional graph nodes here: poll from the host instead
                ex = nullptr;
                cudaGetLastError();
            }
        }
        if (ex) {
            SIMALL_CUDA_TRY(ctx, cudaGraphLaunch(ex, ctx->stream));
            int e = solver_fetch_scalars(s);
            if (e)
                return e;
            const SolveScalars &h = *s->h_scal;
            ctx->launches.fetch_add(2 * (static_cast<int64_t>(h.iter) + 2) + 4 * (static_cast<int64_t>(h.updates) + 1),
                                    std::memory_order_relaxed);
            if (!h.done)
                return fail(ctx, SIMALL_ERR_CUDA, "device loop ended before the stop test held");
            return SIMALL_OK;
        }
    }
    int done_iters = 0;
    // even chunk lengths keep the direction's double buffer in step
    int chunk = s->cfg.check_interval > 0 ? (s->cfg.check_interval + 1) & ~1 : 16;
    double prev_last = -1.0;
    int prev_iter = 0;
    for (;;) {
        int e = run_mixed_chunk(s, chunk);
        if (e)
            return e;
        done_iters += chunk;
        e = solver_fetch_scalars(s);
        if (e)
            return e;
        if (s->h_scal->done)
            break;
        if (done_iters > 2 * maxit + 64)
            return fail(ctx, SIMALL_ERR_CUDA, "mixed solver did not raise its stop flag");
        if (s->cfg.check_interval <= 0) {
            const double last = s->h_scal->last;
            const int it = s->h_scal->iter;
            int next = 64;
            if (prev_last > 0.0 && last > 0.0 && last < prev_last && it > prev_iter) {
                const double rate = std::log(last / prev_last) / (it - prev_iter);
                const double need = std::log(tol / last) / rate;
                next = need < 4 ? 4 : (need > 64 ? 64 : static_cast<int>(need) + 1);
            }
            prev_last = last;
            prev_iter = it;
            chunk = next;
            // snap to a few captured lengths to bound the number of graphs
            chunk = chunk <= 4 ? 4 : chunk <= 8 ? 8 : chunk <= 16 ? 16 : chunk <= 32 ? 32 : 64;
        }
    }
    return SIMALL_OK;
}

int mixed_enqueue_kernel(simall_solver *s, int k, double *bytes)
{
    simall_context *ctx = s->ctx;
    MixedData *m = s->mixed;
    const double nd = static_cast<double>(s->n);
    if (k != 4)
        return fail(ctx, SIMALL_ERR_INVALID_ARGUMENT, "mixed kernel id %d", k);
    // r, q, p read at parity 0 and written at parity 1, xh read and written
    // (each gathered vector counted once), e, plus the matrix: diagonal
    // storage 4 B per stored diagonal per row; sliced storage 6 B per stored
    // entry (8 B with wide offsets: offset and value) and the slice pointers
    *bytes = m->dia ? (4.0 * m->offs.nd + 36.0) * nd
                    : (m->sWide ? 8.0 : 6.0) * static_cast<double>(m->sEntries) + 36.0 * nd +
                          4.0 * static_cast<double>(m->nslices + 1);
    return launch_iter(ctx, s, 0, false);
}

void mixed_invalidate_pattern(simall_solver *s)
{
    if (s->mixed)
        s->mixed->patternReady = false;
}

void mixed_free(simall_solver *s)
{
    delete s->mixed;
    s->mixed = nullptr;
}

}  // namespace simall
