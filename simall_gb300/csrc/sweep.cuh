// Waits of the sweeps that run without level barriers (ILU(0)/SSOR in
// ilu0.cu, the AMG smoother in amg.cu): rows are taken in dependency-level
// order from a ticket and wait (bounded) for the rows they read.  ctl[0] is
// the work ticket, ctl[1] a sweep number (row marks), ctl[2] the wait-timeout
// flag.
#pragma once

#include <cuda_runtime.h>

namespace simall {
namespace {

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
[[maybe_unused]] __global__ void k_sweep_begin(unsigned *ctl)
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

// Values published in place of marks: before a sweep its output vector is
// filled with kPending, a signalling NaN (no arithmetic produces one, and the
// solver rejects non-finite input), each row publishes its value with one
// relaxed store, and a reader polls the values it needs until none is pending.
// One memory round trip less per dependency level than mark-then-value.
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

// Polls x[j[q]] for the flagged q until none is pending (bounded, backing off
// as wait_rows4 does); v receives the values, 0 for the others.  False on
// timeout.
__device__ __forceinline__ bool wait_values4(const double *x, const int (&j)[4], const bool (&dep)[4],
                                             double (&v)[4])
{
    unsigned ns = 16;
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
        if (spins >= 4) {
            __nanosleep(ns);
            ns = ns < 256 ? 2 * ns : 256;
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
