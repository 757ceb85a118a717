// Device helpers: deterministic block/grid reductions and the staged CSR
// row-block SpMV shared by the solver kernels.
#pragma once

#include "internal.hpp"

#include <cuda_runtime.h>

namespace simall {

__device__ __forceinline__ double warp_sum(double v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
        v += __shfl_down_sync(0xffffffffu, v, o);
    return v;  // valid in lane 0
}

__device__ __forceinline__ float warp_sum_f(float v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
        v += __shfl_down_sync(0xffffffffu, v, o);
    return v;  // valid in lane 0
}

// Sum of NV values over the block in a fixed tree; the result is valid in
// thread 0.  Every thread of the block must call it.
template <int NV> __device__ __forceinline__ void block_sum(double (&v)[NV])
{
    __shared__ double red[NV][32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
#pragma unroll
    for (int k = 0; k < NV; ++k)
        v[k] = warp_sum(v[k]);
    if (lane == 0) {
#pragma unroll
        for (int k = 0; k < NV; ++k)
            red[k][wid] = v[k];
    }
    __syncthreads();
    if (wid == 0) {
#pragma unroll
        for (int k = 0; k < NV; ++k)
            v[k] = warp_sum(lane < nw ? red[k][lane] : 0.0);
    }
    __syncthreads();
}

// Grid-wide sum: every block deposits its block sum in partials[k*gridDim.x+b]
// and takes a ticket; the last block to arrive sums the partials in index
// order (fixed for a fixed grid, so the result is reproducible run to run),
// resets the ticket and returns true with the totals in thread 0's v.
template <int NV> __device__ __forceinline__ bool grid_sum_last(double (&v)[NV], double *partials, unsigned *ticket)
{
    __shared__ unsigned s_last;
    block_sum<NV>(v);
    if (threadIdx.x == 0) {
#pragma unroll
        for (int k = 0; k < NV; ++k)
            partials[k * gridDim.x + blockIdx.x] = v[k];
        __threadfence();
        const unsigned t = atomicAdd(ticket, 1u);
        s_last = (t == gridDim.x - 1) ? 1u : 0u;
    }
    __syncthreads();
    if (!s_last)
        return false;
    __threadfence();
    double acc[NV];
#pragma unroll
    for (int k = 0; k < NV; ++k) {
        acc[k] = 0.0;
        for (unsigned b = threadIdx.x; b < gridDim.x; b += blockDim.x)
            acc[k] += __ldcg(&partials[k * gridDim.x + b]);
    }
    block_sum<NV>(acc);
    if (threadIdx.x == 0) {
#pragma unroll
        for (int k = 0; k < NV; ++k)
            v[k] = acc[k];
        *ticket = 0u;
    }
    return true;
}

// grid_sum_last for FP32 per-thread partials: the 32 lanes of a warp are
// summed in FP32 (one warp's worth of a partial sum), every sum above the warp
// -- across warps, CTAs and the grid -- is FP64.  On GB300 a double-precision
// shuffle tree per thread costs more FP64-pipe time than the FP32 streaming
// kernels it would finish.
__device__ __forceinline__ bool grid_sum_last_f(float v, double *partials, unsigned *ticket, double &total)
{
    __shared__ double wsum[32];
    __shared__ unsigned s_last;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
    v = warp_sum_f(v);
    if (lane == 0)
        wsum[wid] = static_cast<double>(v);
    __syncthreads();
    if (threadIdx.x == 0) {
        double b = 0.0;
        for (int w = 0; w < nw; ++w)
            b += wsum[w];
        partials[blockIdx.x] = b;
        __threadfence();
        const unsigned t = atomicAdd(ticket, 1u);
        s_last = (t == gridDim.x - 1) ? 1u : 0u;
    }
    __syncthreads();
    if (!s_last)
        return false;
    __threadfence();
    double acc[1] = {0.0};
    for (unsigned b = threadIdx.x; b < gridDim.x; b += blockDim.x)
        acc[0] += __ldcg(&partials[b]);
    block_sum<1>(acc);
    if (threadIdx.x == 0) {
        total = acc[0];
        *ticket = 0u;
    }
    return true;
}

// grid_sum_last_f for NV values at once (partials[k*gridDim.x + b]); the
// totals land in thread 0's `total`.
template <int NV>
__device__ __forceinline__ bool grid_sum_last_fv(const float (&v)[NV], double *partials, unsigned *ticket,
                                                 double (&total)[NV])
{
    __shared__ double wsum[NV][32];
    __shared__ unsigned s_last;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
#pragma unroll
    for (int k = 0; k < NV; ++k) {
        const float w = warp_sum_f(v[k]);
        if (lane == 0)
            wsum[k][wid] = static_cast<double>(w);
    }
    __syncthreads();
    if (threadIdx.x == 0) {
#pragma unroll
        for (int k = 0; k < NV; ++k) {
            double b = 0.0;
            for (int w = 0; w < nw; ++w)
                b += wsum[k][w];
            partials[k * gridDim.x + blockIdx.x] = b;
        }
        __threadfence();
        const unsigned t = atomicAdd(ticket, 1u);
        s_last = (t == gridDim.x - 1) ? 1u : 0u;
    }
    __syncthreads();
    if (!s_last)
        return false;
    __threadfence();
    double acc[NV];
#pragma unroll
    for (int k = 0; k < NV; ++k) {
        acc[k] = 0.0;
        for (unsigned b = threadIdx.x; b < gridDim.x; b += blockDim.x)
            acc[k] += __ldcg(&partials[k * gridDim.x + b]);
    }
    block_sum<NV>(acc);
    if (threadIdx.x == 0) {
#pragma unroll
        for (int k = 0; k < NV; ++k)
            total[k] = acc[k];
        *ticket = 0u;
    }
    return true;
}

// Row schedule of the SpMV helpers below: nRB >= 0 row-blocks listed in rb
// (staged through shared memory), or nRB < 0 for one thread per row over
// -nRB rows (matrices whose rows are short; see spmv_schedule).
//
// y-rows of A x with one thread per row and no staging: each thread issues
// the column indices and values of up to 8 of its entries, then their
// gathers, before any arithmetic, and no barrier separates loads from
// arithmetic, so resident warps cover one another's latency.  The products
// are rounded and summed from 0.0 in column order, as in spmv_rowblocks.
template <class Epi>
__device__ __forceinline__ void spmv_rows_exact(const int32_t *__restrict__ rowPtr, const int32_t *__restrict__ colIdx,
                                                const double *__restrict__ val, int64_t n,
                                                const double *__restrict__ x, Epi &epi)
{
    for (int64_t row = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; row < n;
         row += (int64_t)gridDim.x * blockDim.x) {
        const int k1 = __ldg(rowPtr + row + 1);
        double s = 0.0;
        for (int k0 = __ldg(rowPtr + row); k0 < k1; k0 += 8) {
            int c[8];
            double a[8], g[8];
#pragma unroll
            for (int q = 0; q < 8; ++q) {
                c[q] = k0 + q < k1 ? __ldg(colIdx + k0 + q) : -1;
                a[q] = k0 + q < k1 ? __ldg(val + k0 + q) : 0.0;
            }
#pragma unroll
            for (int q = 0; q < 8; ++q)
                g[q] = c[q] >= 0 ? __ldg(x + c[q]) : 0.0;
#pragma unroll
            for (int q = 0; q < 8; ++q)
                if (c[q] >= 0)
                    s = __dadd_rn(s, __dmul_rn(a[q], g[q]));
        }
        epi(static_cast<int>(row), s);
    }
}

// The same with one FMA per nonzero, the operations of spmv_rowblocks_fma.
template <class Epi>
__device__ __forceinline__ void spmv_rows_fma(const int32_t *__restrict__ rowPtr, const int32_t *__restrict__ colIdx,
                                              const double *__restrict__ val, int64_t n,
                                              const double *__restrict__ x, Epi &epi)
{
    for (int64_t row = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; row < n;
         row += (int64_t)gridDim.x * blockDim.x) {
        const int k1 = __ldg(rowPtr + row + 1);
        double s = 0.0;
        for (int k0 = __ldg(rowPtr + row); k0 < k1; k0 += 8) {
            int c[8];
            double a[8], g[8];
#pragma unroll
            for (int q = 0; q < 8; ++q) {
                c[q] = k0 + q < k1 ? __ldg(colIdx + k0 + q) : -1;
                a[q] = k0 + q < k1 ? __ldg(val + k0 + q) : 0.0;
            }
#pragma unroll
            for (int q = 0; q < 8; ++q)
                g[q] = c[q] >= 0 ? __ldg(x + c[q]) : 0.0;
#pragma unroll
            for (int q = 0; q < 8; ++q)
                if (c[q] >= 0)
                    s = fma(a[q], g[q], s);
        }
        epi(static_cast<int>(row), s);
    }
}

// y-rows of A x for the row-blocks this CTA owns (blockIdx.x, +gridDim.x, ...).
// Each product a_ij*x_j is rounded once into shared memory and every row is
// summed from 0.0 in column order with separate roundings, the same operation
// sequence as CSRMatrix::spmv (src/solver/CSRMatrix.hpp:24-35), so the result
// is bit-identical to it.  epi(row, y_row) consumes each row.
template <class Epi>
__device__ __forceinline__ void spmv_rowblocks(const int32_t *__restrict__ rowPtr, const int32_t *__restrict__ colIdx,
                                               const double *__restrict__ val, const int32_t *__restrict__ rb,
                                               int nRB, const double *__restrict__ x, Epi &epi)
{
    if (nRB < 0) {
        spmv_rows_exact(rowPtr, colIdx, val, -static_cast<int64_t>(nRB), x, epi);
        return;
    }
    __shared__ double prod[kSpmvNnzCap];
    for (int b = blockIdx.x; b < nRB; b += gridDim.x) {
        const int r0 = __ldg(rb + b), r1 = __ldg(rb + b + 1);
        const int base = __ldg(rowPtr + r0);
        const int cnt = __ldg(rowPtr + r1) - base;
        if (cnt <= kSpmvNnzCap) {
            // every load of this thread's slots is issued before any is used
            constexpr int J = kSpmvNnzCap / kBlock;
            int c[J];
            double a[J], g[J];
#pragma unroll
            for (int j = 0; j < J; ++j) {
                const int k = threadIdx.x + j * kBlock;
                c[j] = k < cnt ? __ldg(colIdx + base + k) : 0;
            }
#pragma unroll
            for (int j = 0; j < J; ++j) {
                const int k = threadIdx.x + j * kBlock;
                a[j] = k < cnt ? __ldg(val + base + k) : 0.0;
                g[j] = k < cnt ? __ldg(x + c[j]) : 0.0;
            }
#pragma unroll
            for (int j = 0; j < J; ++j) {
                const int k = threadIdx.x + j * kBlock;
                if (k < cnt)
                    prod[k] = __dmul_rn(a[j], g[j]);
            }
            __syncthreads();
            for (int row = r0 + threadIdx.x; row < r1; row += blockDim.x) {
                const int k0 = __ldg(rowPtr + row) - base, k1 = __ldg(rowPtr + row + 1) - base;
                double s = 0.0;
                for (int k = k0; k < k1; ++k)
                    s = __dadd_rn(s, prod[k]);
                epi(row, s);
            }
            __syncthreads();
        } else {
            // one row longer than the staging buffer: block-strided sum
            double s[1] = {0.0};
            for (int k = threadIdx.x; k < cnt; k += blockDim.x)
                s[0] += __ldg(val + base + k) * __ldg(x + __ldg(colIdx + base + k));
            block_sum<1>(s);
            if (threadIdx.x == 0)
                epi(r0, s[0]);
            __syncthreads();
        }
    }
}

// Same row-blocks, fused multiply-add form: a_ij and the gathered x_j are
// staged in shared memory, then each row is accumulated with one FMA per
// nonzero.  Half the FP64 instructions of the exact form (GB300's FP64 rate
// is low enough for that to matter); the sum differs from CSRMatrix::spmv
// only in rounding.
template <class Epi>
__device__ __forceinline__ void spmv_rowblocks_fma(const int32_t *__restrict__ rowPtr,
                                                   const int32_t *__restrict__ colIdx,
                                                   const double *__restrict__ val, const int32_t *__restrict__ rb,
                                                   int nRB, const double *__restrict__ x, Epi &epi)
{
    if (nRB < 0) {
        spmv_rows_fma(rowPtr, colIdx, val, -static_cast<int64_t>(nRB), x, epi);
        return;
    }
    __shared__ double sv[kSpmvNnzCap];
    __shared__ double sx[kSpmvNnzCap];
    for (int b = blockIdx.x; b < nRB; b += gridDim.x) {
        const int r0 = __ldg(rb + b), r1 = __ldg(rb + b + 1);
        const int base = __ldg(rowPtr + r0);
        const int cnt = __ldg(rowPtr + r1) - base;
        if (cnt <= kSpmvNnzCap) {
            // stage a_ij and the gathered x_j; all loads issued before use
            constexpr int J = kSpmvNnzCap / kBlock;
            int c[J];
            double a[J], g[J];
#pragma unroll
            for (int j = 0; j < J; ++j) {
                const int k = threadIdx.x + j * kBlock;
                c[j] = k < cnt ? __ldg(colIdx + base + k) : 0;
            }
#pragma unroll
            for (int j = 0; j < J; ++j) {
                const int k = threadIdx.x + j * kBlock;
                a[j] = k < cnt ? __ldg(val + base + k) : 0.0;
                g[j] = k < cnt ? __ldg(x + c[j]) : 0.0;
            }
#pragma unroll
            for (int j = 0; j < J; ++j) {
                const int k = threadIdx.x + j * kBlock;
                if (k < cnt) {
                    sv[k] = a[j];
                    sx[k] = g[j];
                }
            }
            __syncthreads();
            for (int row = r0 + threadIdx.x; row < r1; row += blockDim.x) {
                const int k0 = __ldg(rowPtr + row) - base, k1 = __ldg(rowPtr + row + 1) - base;
                double s = 0.0;
                for (int k = k0; k < k1; ++k)
                    s = fma(sv[k], sx[k], s);
                epi(row, s);
            }
            __syncthreads();
        } else {
            double s[1] = {0.0};
            for (int k = threadIdx.x; k < cnt; k += blockDim.x)
                s[0] = fma(__ldg(val + base + k), __ldg(x + __ldg(colIdx + base + k)), s[0]);
            block_sum<1>(s);
            if (threadIdx.x == 0)
                epi(r0, s[0]);
            __syncthreads();
        }
    }
}

// std::max(a, b) as the reference evaluates it.
__device__ __forceinline__ double std_max(double a, double b) { return (a < b) ? b : a; }

}  // namespace simall
