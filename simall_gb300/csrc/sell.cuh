// Sliced storage of the mixed-precision operator for matrices without diagonal
// structure (RCM-renumbered and unstructured meshes), and the fused CG step
// over one slice, shared by the per-step kernel (mixed.cu) and the persistent
// whole-solve kernel (mixed_grid.cu).
//
// Layout (SELL-32): rows are cut into slices of 32 consecutive rows; slice s
// holds w_s = its longest row's off-diagonal count entries per row, stored
// entry-major: entry k of row 32 s + l sits at sptr[s] + 32 k + l.  A warp
// owns a slice, so every load of the matrix is one contiguous 32-lane access
// (64 B of offsets, 128 B of values, 32 B of corrections).  Per entry:
//   off  column - row: int16 when every |j - i| <= 32767 (an RCM-ordered
//        128^3 box has bandwidth 12,352), else int32;
//   val  N_ij = (S A S)_ij rounded to FP32, S = D^-1/2;
//   cor  the int8 correction of val (ffop.cuh).
// Rows shorter than their slice's width are padded with (off 0, val 0, cor 0),
// which adds 0 to the row.  The diagonal of S A S is 1 and is not stored.
//
// The product is the compensated plain form q_i = p_i + sum_j N_ij p_j in
// float-float arithmetic (ffop.cuh): on pinned Neumann pressure systems it
// keeps the FP32 inner CG at the FP64 iteration count.
#pragma once

#include "bulk.cuh"
#include "ffop.cuh"

#include <cstdint>
#include <type_traits>

namespace simall {

struct SellOp {
    int64_t n = 0;
    int64_t nslices = 0;
    const int32_t *sptr = nullptr;  // [nslices + 1] first entry of each slice (multiples of 32)
    const int16_t *off16 = nullptr; // narrow column offsets
    const int32_t *off32 = nullptr; // wide column offsets
    const float *val = nullptr;
    const int8_t *cor = nullptr;
};

// The iteration state of the sliced engines is packed per row, one float4
// (r, q, p, xh): r the residual, q = (S A S) p, p the direction, xh the FP32
// correction of x; double-buffered by step parity.  A neighbour's p is formed
// again from its r, q and p of the previous step, one 16-byte gather.
//
// Vector loads: through the read-only path in per-step kernels (NC), plain
// coherent loads in the persistent kernel, whose vectors change between the
// grid barriers of one launch.
template <bool NC> __device__ __forceinline__ float4 ld_state(const float4 *p) { return NC ? __ldg(p) : *p; }

// One CG step over slice sl for the lane's row i = 32 sl + lane, reading the
// state of the previous step from `in` and writing this step's to `out`:
//     r = r_old - alpha q_old,  p = r + beta p_old,  xh += alpha p_old,
//     q = (I + N) p,  and the row's shares of p.q, q.q, r.r, r.q.
// The step after a residual replacement has alpha = 0: r is the replaced
// residual already in `in` (fma(-0, q, r) == r), xh is left as it is.  Every
// thread that forms p_j uses the same two roundings, so p_j has the same bits
// wherever it is formed, and no grid-wide barrier separates the update from
// the product.
template <bool WIDE, bool NC>
__device__ __forceinline__ void sell_slice(const SellOp &A, int64_t sl, const float4 *in, float4 *out, float alpha,
                                           float beta, float (&acc)[4])
{
    const int lane = threadIdx.x & 31;
    const int64_t i = sl * 32 + lane;
    const bool live = i < A.n;
    const int32_t e0 = __ldg(A.sptr + sl);
    const int w = (__ldg(A.sptr + sl + 1) - e0) >> 5;
    const float4 o = live ? ld_state<NC>(in + i) : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    const float ri = __fmaf_rn(-alpha, o.y, o.x);
    const float pi = __fmaf_rn(beta, o.z, ri);
    const float xi = __fmaf_rn(alpha, o.z, o.w);
    FFAcc y = ff_start(pi);
    // entries eight at a time: offsets, values and corrections, then the
    // gathers, all issued before the arithmetic (w is uniform over the warp)
    for (int k0 = 0; k0 < w; k0 += 8) {
        int64_t j[8];
        float a[8], al[8];
        float4 g[8];
        bool in_[8];
#pragma unroll
        for (int q = 0; q < 8; ++q) {
            in_[q] = live && k0 + q < w;
            const int64_t e = static_cast<int64_t>(e0) + static_cast<int64_t>(k0 + q) * 32 + lane;
            const int off = in_[q] ? (WIDE ? __ldg(A.off32 + e) : static_cast<int>(__ldg(A.off16 + e))) : 0;
            a[q] = in_[q] ? __ldg(A.val + e) : 0.0f;
            al[q] = in_[q] ? ff_low(a[q], static_cast<int8_t>(__ldg(reinterpret_cast<const signed char *>(A.cor) + e)))
                           : 0.0f;
            j[q] = i + off;
        }
#pragma unroll
        for (int q = 0; q < 8; ++q)
            g[q] = in_[q] ? ld_state<NC>(in + j[q]) : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
#pragma unroll
        for (int q = 0; q < 8; ++q)
            if (in_[q])
                ff_add(y, a[q], al[q], __fmaf_rn(beta, g[q].z, __fmaf_rn(-alpha, g[q].y, g[q].x)));
    }
    if (live) {
        const float yi = ff_value(y);
        out[i] = make_float4(ri, yi, pi, xi);
        acc[0] += pi * yi;
        acc[1] += yi * yi;
        acc[2] += ri * ri;
        acc[3] += ri * yi;
    }
}

// ---------------------------------------------------------------- staged step
// The same step with the streamed operands staged through shared memory by
// bulk copies (TMA).  A CTA owns the contiguous slices [c0, c1) and walks
// them in stages of 8 slices (one per warp).  For a stage, thread 0 issues
// four bulk copies -- the rows' packed state, and the stage's offsets, values
// and corrections, each one contiguous range because slices are stored one
// after the other -- into one slot of a ring of kSellStages buffers, with an
// mbarrier counting the bytes; the copies of the next kSellStages - 1 stages
// are in flight while a stage is computed.  The threads then read their row's
// state and entries from shared memory and only the neighbours' state is
// gathered from global memory (L1/L2).  Slices up to kSellStageMaxW entries
// wide take this path (every hex, tet or prism mesh); wider ones the direct
// sell_slice.
constexpr int kSellStageSlices = 8;  // slices per stage: one per warp of a 256-thread CTA
constexpr int kSellStageMaxW = 8;    // widest slice a stage buffer holds
constexpr int kSellStages = 3;       // ring depth
constexpr int kSellStageEntries = kSellStageSlices * 32 * kSellStageMaxW;

template <bool WIDE> struct SellStageBuf {
    float4 state[kSellStageSlices * 32];
    float val[kSellStageEntries];
    typename std::conditional<WIDE, int32_t, int16_t>::type off[kSellStageEntries];
    int8_t cor[kSellStageEntries];
};

template <bool WIDE> constexpr size_t sell_stage_smem() { return kSellStages * sizeof(SellStageBuf<WIDE>); }

// The ring of one CTA: kSellStages buffers (dynamic shared memory) and their
// mbarriers; q counts the stages this CTA has issued, the same value in every
// thread, so slot and phase parity of every stage follow from it.
template <bool WIDE> struct SellRing {
    SellStageBuf<WIDE> *buf;
    uint64_t *bar;
    uint32_t q;
};

template <bool WIDE>
__device__ __forceinline__ void sell_issue_stage(const SellOp &A, int64_t c0, int64_t c1, int s, const float4 *in,
                                                 SellRing<WIDE> &R, uint32_t gq)
{
    SellStageBuf<WIDE> &B = R.buf[gq % kSellStages];
    uint64_t *bar = R.bar + gq % kSellStages;
    const int64_t sa = c0 + static_cast<int64_t>(s) * kSellStageSlices;
    const int64_t sb = sa + kSellStageSlices < c1 ? sa + kSellStageSlices : c1;
    const int32_t ea = __ldg(A.sptr + sa), eb = __ldg(A.sptr + sb);
    const unsigned ne = static_cast<unsigned>(eb - ea);  // a multiple of 32
    const int64_t r0 = sa * 32, r1 = sb * 32 < A.n ? sb * 32 : A.n;
    const unsigned sbytes = static_cast<unsigned>(r1 - r0) * 16u;
    const unsigned ob = WIDE ? 4u : 2u;
    mbar_arrive_expect_tx(bar, sbytes + ne * (4u + ob + 1u));
    bulk_load(B.state, in + r0, sbytes, bar);
    if (ne) {
        bulk_load(B.val, A.val + ea, ne * 4u, bar);
        if (WIDE)
            bulk_load(B.off, A.off32 + ea, ne * 4u, bar);
        else
            bulk_load(B.off, A.off16 + ea, ne * 2u, bar);
        bulk_load(B.cor, A.cor + ea, ne, bar);
    }
}

// One step over the CTA's slices [c0, c1), staged.  in_written_here: `in` was
// written earlier in the same launch (the persistent kernel), so the copies
// follow a proxy fence.  Returns false -- the same in every thread -- when a
// copy did not complete in time; the copies still in flight are then waited
// for (bounded) before returning.
template <bool WIDE, bool NC>
__device__ bool sell_step_staged(const SellOp &A, int64_t c0, int64_t c1, const float4 *in, float4 *out, float alpha,
                                 float beta, float (&acc)[4], SellRing<WIDE> &R, bool in_written_here)
{
    const int nst = static_cast<int>((c1 - c0 + kSellStageSlices - 1) / kSellStageSlices);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (threadIdx.x == 0) {
        if (in_written_here)
            fence_proxy_async_global();
        fence_proxy_async_shared();
        for (int s = 0; s < kSellStages - 1 && s < nst; ++s)
            sell_issue_stage<WIDE>(A, c0, c1, s, in, R, R.q + s);
    }
    bool ok = true;
    int s = 0;
    for (; s < nst; ++s) {
        if (threadIdx.x == 0 && s + kSellStages - 1 < nst) {
            fence_proxy_async_shared();  // the slot was read (generic proxy) in stage s - 1
            sell_issue_stage<WIDE>(A, c0, c1, s + kSellStages - 1, in, R, R.q + s + kSellStages - 1);
        }
        const uint32_t gq = R.q + s;
        const int64_t sa = c0 + static_cast<int64_t>(s) * kSellStageSlices;
        const int64_t sl = sa + warp;
        const bool has = sl < c1;
        const int32_t ea = __ldg(A.sptr + sa);
        const int32_t e0 = has ? __ldg(A.sptr + sl) : ea;
        const int w = has ? (__ldg(A.sptr + sl + 1) - e0) >> 5 : 0;
        ok = mbar_wait(R.bar + gq % kSellStages, (gq / kSellStages) & 1u) && ok;
        const SellStageBuf<WIDE> &B = R.buf[gq % kSellStages];
        const int64_t i = sl * 32 + lane;
        const bool live = ok && has && i < A.n;
        if (live) {
            const float4 o = B.state[warp * 32 + lane];
            const float ri = __fmaf_rn(-alpha, o.y, o.x);
            const float pi = __fmaf_rn(beta, o.z, ri);
            const float xi = __fmaf_rn(alpha, o.z, o.w);
            FFAcc y = ff_start(pi);
            const int base = e0 - ea + lane;
            int32_t j[kSellStageMaxW];
            float4 g[kSellStageMaxW];
#pragma unroll
            for (int k = 0; k < kSellStageMaxW; ++k)
                j[k] = k < w ? static_cast<int32_t>(i) + static_cast<int32_t>(B.off[base + 32 * k]) : 0;
#pragma unroll
            for (int k = 0; k < kSellStageMaxW; ++k)
                g[k] = k < w ? ld_state<NC>(in + j[k]) : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
#pragma unroll
            for (int k = 0; k < kSellStageMaxW; ++k)
                if (k < w) {
                    const float a = B.val[base + 32 * k];
                    ff_add(y, a, ff_low(a, B.cor[base + 32 * k]),
                           __fmaf_rn(beta, g[k].z, __fmaf_rn(-alpha, g[k].y, g[k].x)));
                }
            const float yi = ff_value(y);
            out[i] = make_float4(ri, yi, pi, xi);
            acc[0] += pi * yi;
            acc[1] += yi * yi;
            acc[2] += ri * ri;
            acc[3] += ri * yi;
        }
        ok = __syncthreads_and(ok) != 0;  // every thread is done with the slot; one verdict for the CTA
        if (!ok)
            break;
    }
    if (!ok) {
        // stages s .. the last issued may still be copying into this CTA's shared memory
        const int issued = nst < s + kSellStages ? nst : s + kSellStages;
        for (int t = s; t < issued; ++t)
            mbar_wait(R.bar + (R.q + t) % kSellStages, ((R.q + t) / kSellStages) & 1u);
    }
    R.q += static_cast<uint32_t>(nst);
    return ok;
}

}  // namespace simall
