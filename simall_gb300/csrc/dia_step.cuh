// One fused mixed-precision CG step over a system in symmetric diagonal
// storage (the step of k_mx_iter_dia, mixed.cu), shared by the per-step
// kernel and the persistent cooperative solve (mixed_grid.cu).
//
// With the step length alpha and beta of the previous step, every row forms
//     r = r_old - alpha q_old,  p = r + beta p_old,  xh += alpha p_old,
// then q = (S A S) p in the row-sum form and the sums p.q, q.q, r.r, r.q.  A
// neighbour's p is formed again from its r_old, q_old, p_old with the same
// two fused multiply-adds, so every thread that forms p_j gets the same bits.
// The vectors are double-buffered (read *_in, write *_out).  FRESH: the step
// after a residual replacement (and the first step): r is the replaced
// residual, read from r_out and not rewritten; alpha = 0.
//
// COH selects how the iteration vectors are read: through the read-only path
// in the per-step kernels (the vectors do not change during a launch), with
// coherent loads (ld.global.ca) in the persistent solve, where other CTAs
// rewrite them between steps and the grid barrier's acquire orders the reads.
// The matrix (U, e) is read-only in both.
#pragma once

#include <cstdint>

namespace simall {

constexpr int kMaxDiags = 8;

struct DiaOffsets {
    int32_t off[kMaxDiags];
    int nd;
};

struct IterVecs {
    const float *rin, *qin, *pin;  // step k-1
    float *rout, *qout, *pout;     // step k
    float *xh;
};

// Four consecutive floats starting at p; p is 16-byte aligned when `aligned`.
__device__ __forceinline__ float4 ld4(const float *__restrict__ p, bool aligned)
{
    if (aligned)
        return __ldg(reinterpret_cast<const float4 *>(p));
    return make_float4(__ldg(p), __ldg(p + 1), __ldg(p + 2), __ldg(p + 3));
}

__device__ __forceinline__ float4 ldv4(const float *__restrict__ p) { return __ldg(reinterpret_cast<const float4 *>(p)); }

// y -= a (p - pn), componentwise: one off-diagonal of the row-sum form.
__device__ __forceinline__ void dfma4(float (&y)[4], float4 a, float4 p, float4 pn)
{
    y[0] = __fmaf_rn(-a.x, p.x - pn.x, y[0]);
    y[1] = __fmaf_rn(-a.y, p.y - pn.y, y[1]);
    y[2] = __fmaf_rn(-a.z, p.z - pn.z, y[2]);
    y[3] = __fmaf_rn(-a.w, p.w - pn.w, y[3]);
}

template <bool COH> __device__ __forceinline__ float ldvec(const float *p)
{
    if constexpr (COH)
        return __ldca(p);
    else
        return __ldg(p);
}

template <bool COH> __device__ __forceinline__ float4 ldvec4(const float *p)
{
    if constexpr (COH)
        return __ldca(reinterpret_cast<const float4 *>(p));
    else
        return __ldg(reinterpret_cast<const float4 *>(p));
}

template <bool COH> __device__ __forceinline__ float4 ldvec4u(const float *p, bool aligned)
{
    if (aligned)
        return ldvec4<COH>(p);
    return make_float4(ldvec<COH>(p), ldvec<COH>(p + 1), ldvec<COH>(p + 2), ldvec<COH>(p + 3));
}

template <bool FRESH>
__device__ __forceinline__ float pdir(float r, float q, float p, float alpha, float beta)
{
    const float rn = FRESH ? r : __fmaf_rn(-alpha, q, r);
    return __fmaf_rn(beta, p, rn);
}

template <bool FRESH>
__device__ __forceinline__ float4 pdir4(float4 r, float4 q, float4 p, float alpha, float beta)
{
    return make_float4(pdir<FRESH>(r.x, q.x, p.x, alpha, beta), pdir<FRESH>(r.y, q.y, p.y, alpha, beta),
                       pdir<FRESH>(r.z, q.z, p.z, alpha, beta), pdir<FRESH>(r.w, q.w, p.w, alpha, beta));
}

// Diagonal storage: ND upper diagonals at ascending offsets; row i reads
// U_d[i] p_{i+off} and, by symmetry, U_d[i-off] p_{i-off}.  One thread per 4
// consecutive rows, a warp per 128 consecutive rows, grid-stride over the
// quads, 128-bit loads of every 16-byte aligned stream.  Warps that touch the
// first or last maxoff rows take the bounds-checked path.
//
// GRID (offset 1 is the first diagonal and every other offset is a multiple
// of 4, as on any natural-order structured grid with a row length divisible
// by 4): every load of a warp's 128 rows is issued before the first multiply,
// so one memory round trip covers all diagonals; p_{i-1}, p_{i+4} and
// U_0[i-1] come from the neighbouring lanes' registers, the warp's two edge
// lanes load them.  Otherwise each diagonal loads as it goes.  acc receives
// this thread's p.q, q.q, r.r, r.q (FP32).
template <int ND, bool GRID, bool FRESH, bool COH>
__device__ __forceinline__ void dia_step(int n, int64_t ldU, const DiaOffsets &o, const float *__restrict__ U,
                                         const float *__restrict__ e, const IterVecs &v, float alpha, float beta,
                                         float (&acc)[4])
{
    const float *__restrict__ rs = FRESH ? v.rout : v.rin;  // where r (before this step's update) lives
    const float *__restrict__ qs = v.qin;
    const float *__restrict__ ps = v.pin;
    const int nq = (n + 3) >> 2;
    const int maxoff = o.off[ND - 1];
    const int lane = threadIdx.x & 31;
    const int stride = gridDim.x * blockDim.x;
    for (int q0 = blockIdx.x * blockDim.x + threadIdx.x - lane; q0 < nq; q0 += stride) {
        const int qd = q0 + lane;
        const int i = qd << 2;
        const bool fast = qd < nq && i >= maxoff && i + 3 + maxoff < n;
        float4 r4, p4;
        float y[4];
        if (__all_sync(0xffffffffu, fast)) {
            if (GRID) {
                constexpr int NF = ND > 1 ? ND - 1 : 1;
                const float4 ro = ldvec4<COH>(rs + i), po = ldvec4<COH>(ps + i), e4 = ldv4(e + i);
                const float4 qo = FRESH ? make_float4(0.f, 0.f, 0.f, 0.f) : ldvec4<COH>(qs + i);
                const float4 xo = FRESH ? make_float4(0.f, 0.f, 0.f, 0.f) : ldvec4<COH>(v.xh + i);
                float4 u[ND];
#pragma unroll
                for (int d = 0; d < ND; ++d)
                    u[d] = ldv4(U + d * ldU + i);
                float4 rp[NF], qp[NF], pp[NF], rm[NF], qm[NF], pm[NF], um[NF];
#pragma unroll
                for (int d = 1; d < ND; ++d) {
                    const int off = o.off[d];
                    rp[d - 1] = ldvec4<COH>(rs + i + off);
                    pp[d - 1] = ldvec4<COH>(ps + i + off);
                    rm[d - 1] = ldvec4<COH>(rs + i - off);
                    pm[d - 1] = ldvec4<COH>(ps + i - off);
                    if (!FRESH) {
                        qp[d - 1] = ldvec4<COH>(qs + i + off);
                        qm[d - 1] = ldvec4<COH>(qs + i - off);
                    }
                    um[d - 1] = ldv4(U + d * ldU + i - off);
                }
                // lane 0 needs row i-1, lane 31 row i+4 (both inside [0, n) on this path)
                const int ie = lane == 0 ? i - 1 : i + 4;
                const float re = ldvec<COH>(rs + ie), pe0 = ldvec<COH>(ps + ie), ue = __ldg(U + (i - 1));
                const float qe = FRESH ? 0.0f : ldvec<COH>(qs + ie);
                // own rows
                r4 = FRESH ? ro
                           : make_float4(__fmaf_rn(-alpha, qo.x, ro.x), __fmaf_rn(-alpha, qo.y, ro.y),
                                         __fmaf_rn(-alpha, qo.z, ro.z), __fmaf_rn(-alpha, qo.w, ro.w));
                p4 = make_float4(__fmaf_rn(beta, po.x, r4.x), __fmaf_rn(beta, po.y, r4.y),
                                 __fmaf_rn(beta, po.z, r4.z), __fmaf_rn(beta, po.w, r4.w));
                if (!FRESH) {
                    *reinterpret_cast<float4 *>(v.rout + i) = r4;
                    *reinterpret_cast<float4 *>(v.xh + i) =
                        make_float4(__fmaf_rn(alpha, po.x, xo.x), __fmaf_rn(alpha, po.y, xo.y),
                                    __fmaf_rn(alpha, po.z, xo.z), __fmaf_rn(alpha, po.w, xo.w));
                }
                *reinterpret_cast<float4 *>(v.pout + i) = p4;
                y[0] = e4.x * p4.x;
                y[1] = e4.y * p4.y;
                y[2] = e4.z * p4.z;
                y[3] = e4.w * p4.w;
                {
                    const float pe = pdir<FRESH>(re, qe, pe0, alpha, beta);
                    float pn = __shfl_down_sync(0xffffffffu, p4.x, 1);  // p[i+4]
                    float pl = __shfl_up_sync(0xffffffffu, p4.w, 1);    // p[i-1]
                    float ul = __shfl_up_sync(0xffffffffu, u[0].w, 1);  // U_0[i-1]
                    if (lane == 31)
                        pn = pe;
                    if (lane == 0) {
                        pl = pe;
                        ul = ue;
                    }
                    dfma4(y, u[0], p4, make_float4(p4.y, p4.z, p4.w, pn));
                    dfma4(y, make_float4(ul, u[0].x, u[0].y, u[0].z), p4, make_float4(pl, p4.x, p4.y, p4.z));
                }
#pragma unroll
                for (int d = 1; d < ND; ++d) {
                    dfma4(y, u[d], p4, pdir4<FRESH>(rp[d - 1], FRESH ? rp[d - 1] : qp[d - 1], pp[d - 1], alpha, beta));
                    dfma4(y, um[d - 1], p4,
                          pdir4<FRESH>(rm[d - 1], FRESH ? rm[d - 1] : qm[d - 1], pm[d - 1], alpha, beta));
                }
            } else {
                const float4 ro = ldvec4<COH>(rs + i), po = ldvec4<COH>(ps + i);
                const float4 qo = FRESH ? ro : ldvec4<COH>(qs + i);
                r4 = FRESH ? ro
                           : make_float4(__fmaf_rn(-alpha, qo.x, ro.x), __fmaf_rn(-alpha, qo.y, ro.y),
                                         __fmaf_rn(-alpha, qo.z, ro.z), __fmaf_rn(-alpha, qo.w, ro.w));
                p4 = make_float4(__fmaf_rn(beta, po.x, r4.x), __fmaf_rn(beta, po.y, r4.y),
                                 __fmaf_rn(beta, po.z, r4.z), __fmaf_rn(beta, po.w, r4.w));
                if (!FRESH) {
                    const float4 xo = ldvec4<COH>(v.xh + i);
                    *reinterpret_cast<float4 *>(v.rout + i) = r4;
                    *reinterpret_cast<float4 *>(v.xh + i) =
                        make_float4(__fmaf_rn(alpha, po.x, xo.x), __fmaf_rn(alpha, po.y, xo.y),
                                    __fmaf_rn(alpha, po.z, xo.z), __fmaf_rn(alpha, po.w, xo.w));
                }
                *reinterpret_cast<float4 *>(v.pout + i) = p4;
                const float4 e4 = ldv4(e + i);
                y[0] = e4.x * p4.x;
                y[1] = e4.y * p4.y;
                y[2] = e4.z * p4.z;
                y[3] = e4.w * p4.w;
#pragma unroll
                for (int d = 0; d < ND; ++d) {
                    const int off = o.off[d];
                    const float *Ud = U + d * ldU;
                    const bool al = (off & 3) == 0;
                    const float4 rp = ldvec4u<COH>(rs + i + off, al), rm = ldvec4u<COH>(rs + i - off, al);
                    const float4 qp = FRESH ? rp : ldvec4u<COH>(qs + i + off, al), qm = FRESH ? rm : ldvec4u<COH>(qs + i - off, al);
                    dfma4(y, ldv4(Ud + i), p4, pdir4<FRESH>(rp, qp, ldvec4u<COH>(ps + i + off, al), alpha, beta));
                    dfma4(y, ld4(Ud + i - off, al), p4, pdir4<FRESH>(rm, qm, ldvec4u<COH>(ps + i - off, al), alpha, beta));
                }
            }
            *reinterpret_cast<float4 *>(v.qout + i) = make_float4(y[0], y[1], y[2], y[3]);
            acc[0] += p4.x * y[0] + p4.y * y[1] + p4.z * y[2] + p4.w * y[3];
            acc[1] += y[0] * y[0] + y[1] * y[1] + y[2] * y[2] + y[3] * y[3];
            acc[2] += r4.x * r4.x + r4.y * r4.y + r4.z * r4.z + r4.w * r4.w;
            acc[3] += r4.x * y[0] + r4.y * y[1] + r4.z * y[2] + r4.w * y[3];
        } else if (qd < nq) {
            for (int k = 0; k < 4; ++k) {
                const int row = i + k;
                if (row >= n)
                    break;
                const float ro = ldvec<COH>(rs + row), po = ldvec<COH>(ps + row);
                const float rk = FRESH ? ro : __fmaf_rn(-alpha, ldvec<COH>(qs + row), ro);
                const float pk = __fmaf_rn(beta, po, rk);
                if (!FRESH) {
                    v.rout[row] = rk;
                    v.xh[row] = __fmaf_rn(alpha, po, v.xh[row]);
                }
                v.pout[row] = pk;
                float yk = __ldg(e + row) * pk;
#pragma unroll
                for (int d = 0; d < ND; ++d) {
                    const int off = o.off[d];
                    const float *Ud = U + d * ldU;
                    if (row + off < n) {
                        const int j = row + off;
                        const float pj =
                            pdir<FRESH>(ldvec<COH>(rs + j), FRESH ? 0.0f : ldvec<COH>(qs + j), ldvec<COH>(ps + j), alpha, beta);
                        yk = __fmaf_rn(-__ldg(Ud + row), pk - pj, yk);
                    }
                    if (row - off >= 0) {
                        const int j = row - off;
                        const float pj =
                            pdir<FRESH>(ldvec<COH>(rs + j), FRESH ? 0.0f : ldvec<COH>(qs + j), ldvec<COH>(ps + j), alpha, beta);
                        yk = __fmaf_rn(-__ldg(Ud + j), pk - pj, yk);
                    }
                }
                v.qout[row] = yk;
                acc[0] += pk * yk;
                acc[1] += yk * yk;
                acc[2] += rk * rk;
                acc[3] += rk * yk;
            }
        }
    }
}

}  // namespace simall
