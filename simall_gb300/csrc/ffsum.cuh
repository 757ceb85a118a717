// Float-float (hi + lo, ~48-bit) dot products and grid reductions for the FP32
// kernels of the mixed-precision solvers.
//
// The inner CG's coefficients come from four dot products per step (p.q,
// q.q, r.r, r.q).  Summed in FP32 per thread and per warp, their relative
// error (~1e-6) moves the iteration count by 10% on pinned 128^3 pressure
// systems with nothing but the grouping of the partial sums changed.  Double
// precision would fix it, but GB300's FP64 pipe runs at 1/64 of the FP32 rate:
// an FP64 accumulation per row, or an FP64 shuffle tree per warp, costs more
// than the step it finishes.  So the sums stay on the FP32 pipe in float-float
// arithmetic: each product with its exact rounding error (an FMA), each
// addition with its error carried (TwoSum), warp trees and the sums across
// warps and CTAs the same way; only the final totals become FP64.  The order
// is fixed for a fixed grid, so the totals are reproducible run to run.
#pragma once

namespace simall {

struct FF {
    float hi, lo;
};

__device__ __forceinline__ FF ff_zero() { return FF{0.0f, 0.0f}; }

// a + b with the rounding error: s = RN(a + b), e exact (Knuth's TwoSum).
__device__ __forceinline__ void two_sum(float a, float b, float &s, float &e)
{
    s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

// acc += a b (the product's rounding error from an FMA).
__device__ __forceinline__ void ff_dot_add(FF &acc, float a, float b)
{
    const float p = __fmul_rn(a, b);
    const float pe = __fmaf_rn(a, b, -p);
    float s, e;
    two_sum(acc.hi, p, s, e);
    acc.hi = s;
    acc.lo = __fadd_rn(acc.lo, __fadd_rn(e, pe));
}

// a + b, renormalised so that |lo| <= ulp(hi) / 2.
__device__ __forceinline__ FF ff_add(FF a, FF b)
{
    float s, e;
    two_sum(a.hi, b.hi, s, e);
    const float lo = __fadd_rn(e, __fadd_rn(a.lo, b.lo));
    const float hi = __fadd_rn(s, lo);
    return FF{hi, __fsub_rn(lo, __fsub_rn(hi, s))};
}

// x a for a float a, renormalised (the product's error from an FMA).
__device__ __forceinline__ FF ff_mul_f(FF x, float a)
{
    const float p = __fmul_rn(x.hi, a);
    const float e = __fmaf_rn(x.lo, a, __fmaf_rn(x.hi, a, -p));
    const float hi = __fadd_rn(p, e);
    return FF{hi, __fsub_rn(e, __fsub_rn(hi, p))};
}

// |r - alpha q|^2 = rr + alpha (alpha qq - 2 rq) from renormalised totals: it
// cancels, so it is formed in float-float; the result's sign is its high part's.
__device__ __forceinline__ FF ff_next_rr(FF rr, FF qq, FF rq, float alpha)
{
    return ff_add(rr, ff_mul_f(ff_add(ff_mul_f(qq, alpha), FF{-2.0f * rq.hi, -2.0f * rq.lo}), alpha));
}

__device__ __forceinline__ double ff_double(FF a) { return static_cast<double>(a.hi) + static_cast<double>(a.lo); }

// Butterfly over the warp: every lane ends with the same bits (each level adds
// the pair in both lanes, and ff_add(a, b) == ff_add(b, a)).
__device__ __forceinline__ FF ff_warp_allsum(FF v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const FF w{__shfl_xor_sync(0xffffffffu, v.hi, o), __shfl_xor_sync(0xffffffffu, v.lo, o)};
        v = ff_add(v, w);
    }
    return v;
}

// Sum of NV values over the block; the result is in every thread.  Every
// thread must call it.
template <int NV> __device__ __forceinline__ void ff_block_allsum(FF (&v)[NV])
{
    __shared__ FF ws[NV][32];
    __shared__ FF tot[NV];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
#pragma unroll
    for (int k = 0; k < NV; ++k) {
        v[k] = ff_warp_allsum(v[k]);
        if (lane == 0)
            ws[k][wid] = v[k];
    }
    __syncthreads();
    if (wid == 0) {
#pragma unroll
        for (int k = 0; k < NV; ++k) {
            FF t = lane < nw ? ws[k][lane] : ff_zero();
            t = ff_warp_allsum(t);
            if (lane == 0)
                tot[k] = t;
        }
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < NV; ++k)
        v[k] = tot[k];
    __syncthreads();
}

// Sum of NV values over the block, handed to `fin(const FF (&tot)[NV])` in
// thread 0, whose results every thread may read after the return: two block
// barriers (ff_block_allsum followed by a barrier around thread 0's work
// takes four).  Every thread must call it.
template <int NV, class Fin> __device__ __forceinline__ void ff_block_finish(FF (&v)[NV], Fin fin)
{
    __shared__ FF ws[NV][32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
#pragma unroll
    for (int k = 0; k < NV; ++k) {
        v[k] = ff_warp_allsum(v[k]);
        if (lane == 0)
            ws[k][wid] = v[k];
    }
    __syncthreads();
    if (wid == 0) {
        FF t[NV];
#pragma unroll
        for (int k = 0; k < NV; ++k)
            t[k] = ff_warp_allsum(lane < nw ? ws[k][lane] : ff_zero());
        if (lane == 0)
            fin(t);
    }
    __syncthreads();
}

// Sum of the CTA slots part[c * NV + k], c < nslots, in a fixed order; the
// result is in every thread.  Every thread must call it.
template <int NV> __device__ __forceinline__ void ff_sum_slots(const FF *part, unsigned nslots, FF (&out)[NV])
{
#pragma unroll
    for (int k = 0; k < NV; ++k)
        out[k] = ff_zero();
    for (unsigned c = threadIdx.x; c < nslots; c += blockDim.x) {
#pragma unroll
        for (int k = 0; k < NV; ++k) {
            const float2 p = __ldcg(reinterpret_cast<const float2 *>(part) + c * NV + k);
            out[k] = ff_add(out[k], FF{p.x, p.y});
        }
    }
    ff_block_allsum<NV>(out);
}

// Grid-wide sum for per-step kernels: every CTA deposits its block sum in
// part[b * NV + k] and takes a ticket; the last CTA to arrive sums all slots
// in index order, resets the ticket and returns true with the totals (FP64)
// in every one of its threads.
template <int NV>
__device__ __forceinline__ bool ff_grid_sum_last(FF (&v)[NV], FF *part, unsigned *ticket, double (&total)[NV])
{
    __shared__ unsigned s_last;
    ff_block_allsum<NV>(v);
    if (threadIdx.x == 0) {
#pragma unroll
        for (int k = 0; k < NV; ++k)
            part[blockIdx.x * NV + k] = v[k];
        __threadfence();
        const unsigned t = atomicAdd(ticket, 1u);
        s_last = (t == gridDim.x - 1) ? 1u : 0u;
    }
    __syncthreads();
    if (!s_last)
        return false;
    __threadfence();
    FF out[NV];
    ff_sum_slots<NV>(part, gridDim.x, out);
#pragma unroll
    for (int k = 0; k < NV; ++k)
        total[k] = ff_double(out[k]);
    if (threadIdx.x == 0)
        *ticket = 0u;
    return true;
}

}  // namespace simall
