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

#include "ffop.cuh"

#include <cstdint>

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

// p of a row from its r, q and p of the previous step (FRESH: r already
// replaced, no alpha update).  Every thread that forms p_j uses these two
// roundings, so p_j has the same bits wherever it is formed.
template <bool FRESH>
__device__ __forceinline__ float pdir(float r, float q, float p, float alpha, float beta)
{
    const float rn = FRESH ? r : __fmaf_rn(-alpha, q, r);
    return __fmaf_rn(beta, p, rn);
}

// Vector loads: through the read-only path in per-step kernels (NC), plain
// coherent loads in the persistent kernel, whose vectors change between the
// grid barriers of one launch.
template <bool NC> __device__ __forceinline__ float ldv(const float *p) { return NC ? __ldg(p) : *p; }

// One CG step over slice sl for the lane's row i = 32 sl + lane:
//     r = r_old - alpha q_old,  p = r + beta p_old,  xh += alpha p_old,
//     q = (I + N) p,  and the row's shares of p.q, q.q, r.r, r.q.
// FRESH: r is the replaced residual, read from rout and not rewritten; no xh
// update.  Neighbour p_j is formed again from r_j, q_j, p_j of the previous
// step, so no grid-wide barrier separates the update from the product.
template <bool FRESH, bool WIDE, bool NC>
__device__ __forceinline__ void sell_slice(const SellOp &A, int64_t sl, const float *rs, const float *qs,
                                           const float *ps, float *rout, float *qout, float *pout, float *xh,
                                           float alpha, float beta, float (&acc)[4])
{
    const int lane = threadIdx.x & 31;
    const int64_t i = sl * 32 + lane;
    const bool live = i < A.n;
    const int32_t e0 = __ldg(A.sptr + sl);
    const int w = (__ldg(A.sptr + sl + 1) - e0) >> 5;
    float ri = 0.0f, pi = 0.0f;
    if (live) {
        const float ro = ldv<NC>(rs + i), po = ldv<NC>(ps + i);
        ri = FRESH ? ro : __fmaf_rn(-alpha, ldv<NC>(qs + i), ro);
        pi = __fmaf_rn(beta, po, ri);
        if (!FRESH) {
            rout[i] = ri;
            xh[i] = __fmaf_rn(alpha, po, xh[i]);
        }
        pout[i] = pi;
    }
    FFAcc y = ff_start(pi);
    // entries eight at a time: offsets, values and corrections, then the
    // gathers, all issued before the arithmetic (w is uniform over the warp)
    for (int k0 = 0; k0 < w; k0 += 8) {
        int64_t j[8];
        float a[8], al[8], gr[8], gq[8], gp[8];
        bool in[8];
#pragma unroll
        for (int q = 0; q < 8; ++q) {
            in[q] = live && k0 + q < w;
            const int64_t e = static_cast<int64_t>(e0) + static_cast<int64_t>(k0 + q) * 32 + lane;
            const int off = in[q] ? (WIDE ? __ldg(A.off32 + e) : static_cast<int>(__ldg(A.off16 + e))) : 0;
            a[q] = in[q] ? __ldg(A.val + e) : 0.0f;
            al[q] = in[q] ? ff_low(a[q], static_cast<int8_t>(__ldg(reinterpret_cast<const signed char *>(A.cor) + e)))
                          : 0.0f;
            j[q] = i + off;
        }
#pragma unroll
        for (int q = 0; q < 8; ++q) {
            gr[q] = in[q] ? ldv<NC>(rs + j[q]) : 0.0f;
            gq[q] = (!FRESH && in[q]) ? ldv<NC>(qs + j[q]) : 0.0f;
            gp[q] = in[q] ? ldv<NC>(ps + j[q]) : 0.0f;
        }
#pragma unroll
        for (int q = 0; q < 8; ++q)
            if (in[q])
                ff_add(y, a[q], al[q], pdir<FRESH>(gr[q], gq[q], gp[q], alpha, beta));
    }
    if (live) {
        const float yi = ff_value(y);
        qout[i] = yi;
        acc[0] += pi * yi;
        acc[1] += yi * yi;
        acc[2] += ri * ri;
        acc[3] += ri * yi;
    }
}

}  // namespace simall
