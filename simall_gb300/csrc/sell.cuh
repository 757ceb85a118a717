// Sliced storage of the mixed-precision operator for matrices without diagonal
// structure (RCM-renumbered and unstructured meshes), and the fused CG step
// over it, shared by the per-step kernels (mixed.cu) and the persistent
// whole-solve kernel (mixed_grid.cu).
//
// Layout (SELL-32): rows are cut into slices of 32 consecutive rows; slice s
// holds w_s = its longest row's off-diagonal count entries per row, stored
// entry-major: entry k of row 32 s + l sits at sptr[s] + 32 k + l.  A warp
// owns a slice, so every load of the matrix is one contiguous 32-lane access
// (64 B of offsets, 128 B of values).  Per entry:
//   off  column - row: int16 when every |j - i| <= 32767 (an RCM-ordered
//        128^3 box has bandwidth 12,352), else int32;
//   val  N_ij = (S A S)_ij rounded to FP32, S = D^-1/2.
// Rows shorter than their slice's width are padded with (off 0, val 0).  The
// diagonal of S A S is 1 and is not stored.  Per row, e_i = 1 + sum_j N_ij
// (summed in FP64 from A, rounded once), padded with zeros to whole slices.
//
// The product is the row-sum form of mixed.cu: q_i = e_i p_i - sum_j N_ij
// (p_i - p_j), which equals p_i + sum_j N_ij p_j and keeps the FP32 inner CG
// of pinned pressure systems near the FP64 iteration count.
//
// The iteration state is packed per row, one float4 (r, q, p, xh): r the
// residual, q = (S A S) p, p the direction, xh the FP32 correction of x;
// double-buffered by step parity.  A neighbour's p is formed again from its
// r, q and p of the previous step -- one 16-byte gather per entry.
#pragma once

#include "bulk.cuh"
#include "ffsum.cuh"

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
    const float *e = nullptr;       // [nslices * 32] row sums, zero past n
    int prefetch = 0;               // staged steps: stages ahead whose operands are prefetched into L2 (0 = off)
};

// Vector loads: through the read-only path in per-step kernels (NC), plain
// coherent loads in the persistent kernel, whose state changes between the
// grid barriers of one launch.
template <bool NC> __device__ __forceinline__ float4 ld_state(const float4 *p) { return NC ? __ldg(p) : *p; }

// p_j of the current step from a neighbour's state of the previous one; the
// owner forms p_i with the same two roundings, so the bits agree.  After a
// residual replacement alpha = 0 and fma(-0, q, r) == r.
__device__ __forceinline__ float p_of(const float4 &g, float alpha, float beta)
{
    return __fmaf_rn(beta, g.z, __fmaf_rn(-alpha, g.y, g.x));
}

// y - sum_k N_ik (p_i - p_k) over W entries at off[base + 32 k],
// val[base + 32 k] (k < W): the offsets first, then all gathers, then the
// arithmetic in entry order.
template <int W, bool NC, class OffT>
__device__ __forceinline__ float sell_row(const OffT *off, const float *val, int base, int32_t i, float pi, float y,
                                          const float4 *in, float alpha, float beta)
{
    if constexpr (W > 0) {
        int32_t j[W];
        float4 g[W];
#pragma unroll
        for (int k = 0; k < W; ++k)
            j[k] = i + static_cast<int32_t>(off[base + 32 * k]);
#pragma unroll
        for (int k = 0; k < W; ++k)
            g[k] = ld_state<NC>(in + j[k]);
#pragma unroll
        for (int k = 0; k < W; ++k)
            y = __fmaf_rn(-val[base + 32 * k], pi - p_of(g[k], alpha, beta), y);
    }
    return y;
}

// The row-sum product e_i p_i - sum_k N_ik (p_i - p_k), dispatched on the
// slice width (uniform over the warp): widths up to 8 run fully unrolled;
// wider rows in blocks of 8, then one at a time.
template <bool NC, class OffT>
__device__ __forceinline__ float sell_row_any(int w, const OffT *off, const float *val, int base, int32_t i, float pi,
                                              float ei, const float4 *in, float alpha, float beta)
{
    const float y0 = ei * pi;
    switch (w) {
    case 0: return sell_row<0, NC>(off, val, base, i, pi, y0, in, alpha, beta);
    case 1: return sell_row<1, NC>(off, val, base, i, pi, y0, in, alpha, beta);
    case 2: return sell_row<2, NC>(off, val, base, i, pi, y0, in, alpha, beta);
    case 3: return sell_row<3, NC>(off, val, base, i, pi, y0, in, alpha, beta);
    case 4: return sell_row<4, NC>(off, val, base, i, pi, y0, in, alpha, beta);
    case 5: return sell_row<5, NC>(off, val, base, i, pi, y0, in, alpha, beta);
    case 6: return sell_row<6, NC>(off, val, base, i, pi, y0, in, alpha, beta);
    case 7: return sell_row<7, NC>(off, val, base, i, pi, y0, in, alpha, beta);
    case 8: return sell_row<8, NC>(off, val, base, i, pi, y0, in, alpha, beta);
    default: {
        float y = sell_row<8, NC>(off, val, base, i, pi, y0, in, alpha, beta);
        int k = 8;
        for (; k + 8 <= w; k += 8)
            y = sell_row<8, NC>(off, val, base + 32 * k, i, pi, y, in, alpha, beta);
        for (; k < w; ++k)
            y = sell_row<1, NC>(off, val, base + 32 * k, i, pi, y, in, alpha, beta);
        return y;
    }
    }
}

// The step of one row from its previous state o:
//     r = r_old - alpha q_old,  p = r + beta p_old,  xh += alpha p_old,
//     q = (S A S) p,  and the row's shares of p.q, q.q, r.r, r.q, added to
// the thread's float-float sums (ffsum.cuh).
struct RowStep {
    float r, p, xh;
    __device__ __forceinline__ RowStep(const float4 &o, float alpha, float beta)
    {
        r = __fmaf_rn(-alpha, o.y, o.x);
        p = __fmaf_rn(beta, o.z, r);
        xh = __fmaf_rn(alpha, o.z, o.w);
    }
    __device__ __forceinline__ void finish(float q, float4 *out, FF (&acc)[4]) const
    {
        *out = make_float4(r, q, p, xh);
        ff_dot_add(acc[0], p, q);
        ff_dot_add(acc[1], q, q);
        ff_dot_add(acc[2], r, r);
        ff_dot_add(acc[3], r, q);
    }
};

// One step over slice sl (direct loads; any width).
template <bool WIDE, bool NC>
__device__ __forceinline__ void sell_slice(const SellOp &A, int64_t sl, const float4 *in, float4 *out, float alpha,
                                           float beta, FF (&acc)[4])
{
    const int lane = threadIdx.x & 31;
    const int64_t i = sl * 32 + lane;
    const int32_t e0 = __ldg(A.sptr + sl);
    const int w = (__ldg(A.sptr + sl + 1) - e0) >> 5;
    if (i >= A.n)
        return;
    const RowStep rs(ld_state<NC>(in + i), alpha, beta);
    float y;
    if (WIDE)
        y = sell_row_any<NC>(w, A.off32 + e0, A.val + e0, lane, static_cast<int32_t>(i), rs.p, __ldg(A.e + i), in,
                             alpha, beta);
    else
        y = sell_row_any<NC>(w, A.off16 + e0, A.val + e0, lane, static_cast<int32_t>(i), rs.p, __ldg(A.e + i), in,
                             alpha, beta);
    rs.finish(y, out + i, acc);
}

// ---------------------------------------------------------------- staged step
// The same step with the streamed operands staged through shared memory by
// bulk copies (TMA).  A CTA of kSellThreads owns the contiguous slices
// [c0, c1) and walks them in stages of 24 slices: warps 0-23 each compute one
// slice of a stage, warp 24 produces.  For a stage the producer issues four
// bulk copies -- the rows' packed state and row sums, and the stage's offsets
// and values, each one contiguous range because slices are stored one after
// the other -- into one slot of a ring of kSellStages buffers, announced on
// the slot's `full` mbarrier; it refills a slot once all 24 compute warps have
// arrived on its `empty` mbarrier.  A compute warp waits for its slot's copies
// only, reads its rows' state and entries from shared memory and gathers
// only the neighbours' state from global memory (L1/L2), so warps run up to
// kSellStages - 1 stages apart and never wait for one another.  Slices up to
// kSellStageMaxW entries wide take this path (every hex, tet or prism mesh);
// wider ones the direct sell_slice.
constexpr int kSellStageSlices = 24;  // slices per stage: one per compute warp (one 800-thread CTA per SM)
constexpr int kSellThreads = 32 * (kSellStageSlices + 1);  // 8 compute warps + the producer warp
constexpr int kSellStageMaxW = 6;    // widest slice a stage buffer holds (hex meshes: 6); less shared memory, more L1
constexpr int kSellStages = 3;       // ring depth
constexpr int kSellStageEntries = kSellStageSlices * 32 * kSellStageMaxW;

template <bool WIDE> struct SellStageBuf {
    float4 state[kSellStageSlices * 32];
    float e[kSellStageSlices * 32];
    float val[kSellStageEntries];
    typename std::conditional<WIDE, int32_t, int16_t>::type off[kSellStageEntries];
};

template <bool WIDE> constexpr size_t sell_stage_smem() { return kSellStages * sizeof(SellStageBuf<WIDE>); }

// The ring of one CTA: kSellStages buffers (dynamic shared memory), their
// full and empty mbarriers (2 kSellStages, initialised by sell_ring_init);
// q counts the stages this CTA has used, the same value in every thread, so
// the slot and phase parity of every stage follow from it.
template <bool WIDE> struct SellRing {
    SellStageBuf<WIDE> *buf;
    uint64_t *bar;  // [0, kSellStages) full, [kSellStages, 2 kSellStages) empty
    uint32_t q;
};

// Thread 0, once per launch, before a block barrier.
__device__ __forceinline__ void sell_ring_init(uint64_t *bar)
{
    for (int b = 0; b < kSellStages; ++b) {
        mbar_init(bar + b, 1);
        mbar_init(bar + kSellStages + b, kSellStageSlices);
    }
    mbar_fence_init();
}

// L2 prefetch of stage s's four ranges (the same ranges sell_issue_stage copies).
template <bool WIDE>
__device__ __forceinline__ void sell_prefetch_stage(const SellOp &A, int64_t c0, int64_t c1, int s, const float4 *in)
{
    const int64_t sa = c0 + static_cast<int64_t>(s) * kSellStageSlices;
    const int64_t sb = sa + kSellStageSlices < c1 ? sa + kSellStageSlices : c1;
    const int32_t ea = __ldg(A.sptr + sa), eb = __ldg(A.sptr + sb);
    const unsigned ne = static_cast<unsigned>(eb - ea);
    const int64_t r0 = sa * 32, r1 = sb * 32 < A.n ? sb * 32 : A.n;
    bulk_prefetch_l2(in + r0, static_cast<unsigned>(r1 - r0) * 16u);
    bulk_prefetch_l2(A.e + r0, static_cast<unsigned>(sb - sa) * 128u);
    if (ne) {
        bulk_prefetch_l2(A.val + ea, ne * 4u);
        if (WIDE)
            bulk_prefetch_l2(A.off32 + ea, ne * 4u);
        else
            bulk_prefetch_l2(A.off16 + ea, ne * 2u);
    }
}

template <bool WIDE>
__device__ __forceinline__ void sell_issue_stage(const SellOp &A, int64_t c0, int64_t c1, int s, const float4 *in,
                                                 SellStageBuf<WIDE> &B, uint64_t *bar)
{
    const int64_t sa = c0 + static_cast<int64_t>(s) * kSellStageSlices;
    const int64_t sb = sa + kSellStageSlices < c1 ? sa + kSellStageSlices : c1;
    const int32_t ea = __ldg(A.sptr + sa), eb = __ldg(A.sptr + sb);
    const unsigned ne = static_cast<unsigned>(eb - ea);  // a multiple of 32
    const int64_t r0 = sa * 32, r1 = sb * 32 < A.n ? sb * 32 : A.n;
    const unsigned sbytes = static_cast<unsigned>(r1 - r0) * 16u;
    const unsigned ebytes = static_cast<unsigned>(sb - sa) * 128u;  // whole slices: e is padded
    const unsigned ob = WIDE ? 4u : 2u;
    // the matrix streams are read once per step: evict them first, so the
    // state the neighbours gather stays in L2 between steps
    const uint64_t once = l2_evict_first_policy();
    mbar_arrive_expect_tx(bar, sbytes + ebytes + ne * (4u + ob));
    bulk_load(B.state, in + r0, sbytes, bar);
    bulk_load_hint(B.e, A.e + r0, ebytes, bar, once);
    if (ne) {
        bulk_load_hint(B.val, A.val + ea, ne * 4u, bar, once);
        if (WIDE)
            bulk_load_hint(B.off, A.off32 + ea, ne * 4u, bar, once);
        else
            bulk_load_hint(B.off, A.off16 + ea, ne * 2u, bar, once);
    }
}

// One step over the CTA's slices [c0, c1), staged; every thread of the CTA
// calls it.  in_written_here: `in` was written earlier in the same launch (the
// persistent kernel), so the copies follow a proxy fence.  Returns this
// thread's verdict, false when one of its waits ran out (a copy that did not
// land, a slot that was not released; the producer then waits, bounded, for
// the copies still in flight); no block barrier at the end: the caller folds
// the verdicts into the barrier of its reduction (__syncthreads_and).
template <bool WIDE, bool NC>
__device__ bool sell_step_staged(const SellOp &A, int64_t c0, int64_t c1, const float4 *in, float4 *out, float alpha,
                                 float beta, FF (&acc)[4], SellRing<WIDE> &R, bool in_written_here)
{
    const int nst = static_cast<int>((c1 - c0 + kSellStageSlices - 1) / kSellStageSlices);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    uint64_t *full = R.bar, *empty = R.bar + kSellStages;
    bool ok = true;
    if (warp == kSellStageSlices) {
        // producer
        if (lane == 0) {
            if (in_written_here)
                fence_proxy_async_global();
            int s = 0;
            for (; s < nst; ++s) {
                const uint32_t u = R.q + s;
                if (u >= static_cast<uint32_t>(kSellStages) &&
                    !mbar_wait(empty + u % kSellStages, (u / kSellStages - 1) & 1u)) {
                    ok = false;
                    break;
                }
                fence_proxy_async_shared();  // the slot's previous contents were read through the generic proxy
                sell_issue_stage<WIDE>(A, c0, c1, s, in, R.buf[u % kSellStages], full + u % kSellStages);
                if (A.prefetch > 0 && s + A.prefetch < nst)
                    sell_prefetch_stage<WIDE>(A, c0, c1, s + A.prefetch, in);
            }
            if (!ok) {
                // the copies issued and not yet consumed: let them land before the CTA can leave
                for (int t = s - kSellStages < 0 ? 0 : s - kSellStages; t < s; ++t)
                    mbar_wait(full + (R.q + t) % kSellStages, ((R.q + t) / kSellStages) & 1u);
            }
        }
    } else {
        for (int s = 0; s < nst; ++s) {
            const uint32_t u = R.q + s;
            const int64_t sa = c0 + static_cast<int64_t>(s) * kSellStageSlices;
            const int64_t sl = sa + warp;
            const bool has = sl < c1;
            const int32_t ea = __ldg(A.sptr + sa);
            const int32_t e0 = has ? __ldg(A.sptr + sl) : ea;
            const int w = has ? (__ldg(A.sptr + sl + 1) - e0) >> 5 : 0;
            if (!mbar_wait(full + u % kSellStages, (u / kSellStages) & 1u)) {
                ok = false;
                break;
            }
            const SellStageBuf<WIDE> &B = R.buf[u % kSellStages];
            const int64_t i = sl * 32 + lane;
            if (has && i < A.n) {
                const int t = warp * 32 + lane;
                const RowStep rs(B.state[t], alpha, beta);
                const float y = sell_row_any<NC>(w, B.off, B.val, e0 - ea + lane, static_cast<int32_t>(i), rs.p,
                                                 B.e[t], in, alpha, beta);
                rs.finish(y, out + i, acc);
            }
            __syncwarp();
            if (lane == 0)
                mbar_arrive(empty + u % kSellStages);
        }
    }
    R.q += static_cast<uint32_t>(nst);
    return ok;
}

}  // namespace simall
