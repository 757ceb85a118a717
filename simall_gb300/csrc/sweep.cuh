// Waits of the sweeps that run without level barriers (ILU(0)/SSOR in
// ilu0.cu, the AMG smoother in amg.cu): rows are taken in dependency-level
// order from a ticket and wait (bounded) for the rows they read.  ctl[0] is
// the work ticket, ctl[2] the wait-timeout flag.
#pragma once

#include <cuda_runtime.h>

namespace simall {
namespace {

constexpr unsigned kSweepMaxSpins = 1u << 20;  // ~0.5 s of polling: far beyond any dependency chain

// Values published as they land: before a sweep its output vector is
// filled with kPending, a signalling NaN with a fixed payload, each row
// publishes its value with one relaxed store, and a reader polls the values
// it needs until none is pending.  One memory round trip less per dependency
// level than a separate "done" mark followed by the value.  No arithmetic
// produces a signalling NaN, and the solver rejects non-finite right-hand
// sides and matrices; a row value that still equalled kPending (only by
// copying that exact bit pattern in from an input) would make its readers
// run out their bounded wait and report it, not hang.
constexpr unsigned long long kPending = 0x7FF4C0DE5EED5A1EULL;

__device__ __forceinline__ double ld_value(const double *p)
{
    unsigned long long v;
    asm volatile("ld.relaxed.gpu.global.b64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return __longlong_as_double(static_cast<long long>(v));
}

__device__ __forceinline__ void st_value(double *p, double v)
{
    asm volatile("st.relaxed.gpu.global.b64 [%0], %1;" ::"l"(p), "l"(__double_as_longlong(v)) : "memory");
}

__device__ __forceinline__ bool pending(double v)
{
    return static_cast<unsigned long long>(__double_as_longlong(v)) == kPending;
}

// Polls x[j[q]] for the flagged q until none is pending; v receives the
// values, 0 for the others.  Bounded: false after kSweepMaxSpins polls.  The
// first polls are immediate (the rows are usually done or nearly so); later
// ones back off, doubling from 16 ns up to max_ns, so that thousands of
// waiting warps do not flood L2 (max_ns = 0: never sleep).
__device__ __forceinline__ bool wait_values4(const double *x, const int (&j)[4], const bool (&dep)[4],
                                             double (&v)[4], unsigned max_ns = 256)
{
    unsigned ns = 16 < max_ns ? 16 : max_ns;
    for (unsigned spins = 0;; ++spins) {
        bool all = true;
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            v[q] = dep[q] ? ld_value(x + j[q]) : 0.0;
            all = !(dep[q] && pending(v[q])) && all;
        }
        if (all)
            return true;
        if (spins >= kSweepMaxSpins)
            return false;
        if (spins >= 4 && max_ns) {
            __nanosleep(ns);
            ns = 2 * ns < max_ns ? 2 * ns : max_ns;
        }
    }
}

// Next sweep: the output vector to kPending, the ticket to 0.
[[maybe_unused]] __global__ void k_sweep_begin_values(unsigned *ctl, double *out, int n)
{
    const double p = __longlong_as_double(static_cast<long long>(kPending));
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        out[i] = p;
    if (blockIdx.x == 0 && threadIdx.x == 0)
        ctl[0] = 0u;
}

}  // namespace
}  // namespace simall
