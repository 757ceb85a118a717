// Row marks for sweeps that run without level barriers (ILU(0)/SSOR in
// ilu0.cu, the AMG smoother in amg.cu): a row publishes its value, then its
// mark (release); a reader waits for the marks of the rows it reads (acquire,
// bounded) before loading their values.  ctl[0] is the work ticket, ctl[1]
// the sweep number the marks carry, ctl[2] the wait-timeout flag.
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

}  // namespace
}  // namespace simall
