// Small systems on one thread-block cluster.
//
// Below some 10^5 rows a Krylov iteration spread over the whole GPU is bound by
// launch and grid-synchronisation latency, not by bandwidth: on the 128 x 128
// cavity (16,384 rows, 2.7 MB per FP64 iteration) the multi-kernel PCG spends
// ~17 us per iteration.  Here one cluster of up to 16 CTAs (one per SM) runs
// the whole solve in a single launch.  Each CTA owns a contiguous slice of
// rows; the vectors that other CTAs read (the preconditioned residual and the
// double-buffered search direction, and for mixed precision the FP32 residual,
// product and direction) live in the owners' shared memory and are read by the
// other CTAs through distributed shared memory; a CTA's private per-row state
// stays in registers.  Every global sum is one cluster barrier: each CTA
// pushes its partial sums into every CTA's shared memory, and after the
// barrier one warp of every CTA reduces all partials in rank order with the
// same butterfly, so all CTAs hold bit-identical totals and take identical
// decisions without further communication.
//
// 512 threads per CTA (one CTA per SM): 16 warps hide the latency of the
// neighbour loads that 8 could not (a 65,025-row system on 16 CTAs: 8.0 ->
// 6.2 us per step).  The row index of a thread is made opaque to the compiler
// in each step (clmix_rows), so per-row addresses are not hoisted out of the
// solve loop into registers: that hoisting had held up to 255 registers per
// thread with spills, and at 512 threads a thread has 128.  A step's scalar
// work is FP32 (ClMixState): with FP64 state and per-thread conversions of
// alpha and beta, a step cost 1 us more at every size (3.2 against 2.2 us on
// 2,025 rows; 6.2 against 5.2 us on 65,025, both with FP32 sums).  The step's
// sums are float-float (cl_allreduce), at ~0.5 us per step and ~0.2 ns per
// row of a slice more than FP32 sums (2.7 and 6.7 us on those systems), so
// that the step count does not depend on the launch shape.  The only waits are hardware
// cluster barriers, reached the same number of times by every CTA (the trip
// count follows from the identical totals and is bounded by max_iter), so no
// CTA can wait for one that has left.
//
// Two solvers, chosen by the single-system solver when the system fits:
//   FP64 Jacobi PCG (CGSolver::solve, src/solver/LinearSolvers.cpp:420-451):
//     per iteration q = A p with p = z + beta p_old formed on the fly, p.q;
//     x, r, z = D^-1 r, r.r, r.z -- two barriers.
//   Mixed precision (diagonal storage): the fused FP32 step of mixed.cu (row-
//     sum form, beta from |r - alpha q|^2) with FP64 reliable updates -- one
//     barrier per step, three more per reliable update.
#include "bulk.cuh"
#include "device.cuh"
#include "ffsum.cuh"
#include "solver.hpp"

#include <cooperative_groups.h>

#include <algorithm>
#include <cmath>
#include <type_traits>

namespace cg = cooperative_groups;

namespace simall {

constexpr int kClThreads = 512;
constexpr int kClMaxRowsPerCta = 8192;  // mixed: 6 FP32 vectors of a slice in shared memory
constexpr int kClPcg64MaxRowsPerCta = 4096;  // FP64: five FP64 registers per owned row and thread
constexpr int kClMaxIterations = 200000;  // longer limits take the multi-kernel path

namespace {

struct ClShared {
    double inbox[2][16][4];   // every CTA's partial sums, pushed here by their owners; two slots used alternately
    float2 inboxff[2][16][4]; // the same for float-float partials (hi, lo)
    double wsum[4][32];       // per-warp sums (FP64 values)
    FF wsumff[4][32];         // per-warp sums (float-float values)
    double tot[4];            // the cluster totals, broadcast to the CTA
    FF totf[4];               // the same, float-float
    double ctl[8];            // scalars derived from the totals by one thread, broadcast
};

struct NoFinish {
    template <typename... Args> __device__ void operator()(Args...) const {}
};

// Butterfly sums of NV values over groups of 2^LEVELS lanes, level by level
// so the NV dependent chains overlap; every lane of a group ends with the same
// bits (each level adds a pair in both lanes of the pair, and a + b == b + a).
template <int LEVELS, int NV, typename T> __device__ __forceinline__ void butterfly(T (&v)[NV])
{
#pragma unroll
    for (int l = 0; l < LEVELS; ++l) {
        T o[NV];
#pragma unroll
        for (int k = 0; k < NV; ++k)
            o[k] = __shfl_xor_sync(0xffffffffu, v[k], 1 << l);
#pragma unroll
        for (int k = 0; k < NV; ++k)
            v[k] += o[k];
    }
}

constexpr int kClWarps = kClThreads / 32;
constexpr int kClWarpLevels = kClWarps <= 1 ? 0 : kClWarps <= 2 ? 1 : kClWarps <= 4 ? 2 : kClWarps <= 8 ? 3 : kClWarps <= 16 ? 4 : 5;
constexpr int kClMaxCtas = 16;  // cluster sizes up to 16: 4 butterfly levels

// Cluster-wide sum of NV values; every thread of every CTA receives the same
// totals.  Two kinds of partials: float-float (the mixed solver's per-thread
// sums of FP32 products, with each product's and each addition's error
// carried) summed in float-float at every level on the FP32 pipe, and FP64
// (the FP64 solver, and the mixed solver's FP64 residual sums at reliable
// updates) summed in FP64.  With plain FP32 sums the mixed solver's step count
// moved by up to 8% with nothing but the thread count changed (783 against
// 849 steps on a 128^2 cavity system); in float-float it does not depend on
// the grouping.  Each CTA pushes its partials into every CTA's shared memory
// before the barrier (stores through the cluster window, whose latency the
// barrier absorbs; the kernels start with a cluster barrier so that no CTA
// writes into one that has not started), so after it the sum reads only local
// shared memory.  The butterflies run level by level over all NV values, so
// the NV dependent chains overlap, with no more levels than there are warps or
// CTAs.  `fin(tot, ctl)` runs in one thread of each CTA before the broadcast:
// scalar arithmetic done once per CTA instead of once per thread.
template <int NV, typename T, typename Fin = NoFinish>
__device__ __forceinline__ void cl_allreduce(const T (&v)[NV], T (&out)[NV], ClShared &sh, int &slot,
                                             const cg::cluster_group &cl, Fin fin = Fin{})
{
    constexpr bool kFF = std::is_same<T, FF>::value;
    static_assert(kFF || std::is_same<T, double>::value, "float-float or FP64 partials");
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    T w[NV];
#pragma unroll
    for (int k = 0; k < NV; ++k) {
        if constexpr (kFF)
            w[k] = ff_warp_allsum(v[k]);
        else
            w[k] = v[k];
    }
    if constexpr (!kFF)
        butterfly<5>(w);
    if (lane == 0) {
#pragma unroll
        for (int k = 0; k < NV; ++k) {
            if constexpr (kFF)
                sh.wsumff[k][wid] = w[k];
            else
                sh.wsum[k][wid] = w[k];
        }
    }
    __syncthreads();
    const int C = static_cast<int>(cl.num_blocks());
    if (wid == 0) {
        T c[NV];
#pragma unroll
        for (int k = 0; k < NV; ++k) {
            if constexpr (kFF)
                c[k] = lane < kClWarps ? sh.wsumff[k][lane] : ff_zero();
            else
                c[k] = lane < kClWarps ? sh.wsum[k][lane] : 0.0;
        }
        if constexpr (kFF) {
#pragma unroll
            for (int l = 0; l < kClWarpLevels; ++l) {
#pragma unroll
                for (int k = 0; k < NV; ++k)
                    c[k] = ff_add(c[k], FF{__shfl_xor_sync(0xffffffffu, c[k].hi, 1 << l),
                                           __shfl_xor_sync(0xffffffffu, c[k].lo, 1 << l)});
            }
        } else {
            butterfly<kClWarpLevels>(c);
        }
        // Only lanes 0 .. kClWarps-1 hold the CTA's sum after that butterfly:
        // take lane 0's before lane L pushes it to rank L.  (Pushing another
        // lane's value gave the CTAs different totals, different branches,
        // and CTAs that left while others still used their shared memory.)
#pragma unroll
        for (int k = 0; k < NV; ++k) {
            if constexpr (kFF)
                c[k] = FF{__shfl_sync(0xffffffffu, c[k].hi, 0), __shfl_sync(0xffffffffu, c[k].lo, 0)};
            else
                c[k] = __shfl_sync(0xffffffffu, c[k], 0);
        }
        // push this CTA's partials into every CTA's inbox (lane L -> rank L)
        if (lane < C) {
            if constexpr (kFF) {
                float2 *dst = cl.map_shared_rank(&sh.inboxff[slot][cl.block_rank()][0], lane);
#pragma unroll
                for (int k = 0; k < NV; ++k)
                    dst[k] = make_float2(c[k].hi, c[k].lo);
            } else {
                double *dst = cl.map_shared_rank(&sh.inbox[slot][cl.block_rank()][0], lane);
#pragma unroll
                for (int k = 0; k < NV; ++k)
                    dst[k] = c[k];
            }
        }
    }
    cl.sync();
    if (wid == 0) {
        T t[NV];
#pragma unroll
        for (int k = 0; k < NV; ++k) {
            if constexpr (kFF) {
                const float2 e = lane < C ? sh.inboxff[slot][lane][k] : make_float2(0.0f, 0.0f);
                t[k] = FF{e.x, e.y};
            } else {
                t[k] = lane < C ? sh.inbox[slot][lane][k] : 0.0;
            }
        }
        if constexpr (kFF) {
#pragma unroll
            for (int l = 0; l < 4; ++l) {
#pragma unroll
                for (int k = 0; k < NV; ++k)
                    t[k] = ff_add(t[k], FF{__shfl_xor_sync(0xffffffffu, t[k].hi, 1 << l),
                                           __shfl_xor_sync(0xffffffffu, t[k].lo, 1 << l)});
            }
        } else {
            butterfly<4>(t);
        }
        if (lane == 0) {
#pragma unroll
            for (int k = 0; k < NV; ++k) {
                if constexpr (kFF)
                    sh.totf[k] = t[k];
                else
                    sh.tot[k] = t[k];
            }
            if constexpr (kFF)
                fin(sh.totf, sh.ctl);
            else
                fin(sh.tot, sh.ctl);
        }
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < NV; ++k) {
        if constexpr (kFF)
            out[k] = sh.totf[k];
        else
            out[k] = sh.tot[k];
    }
    slot ^= 1;
}

// Value at global row j of a shared-memory array distributed by slices of
// 2^logR rows, read through the cluster window from the owner.
template <typename T>
__device__ __forceinline__ T cl_load(const cg::cluster_group &cl, T *local, int logR, int j)
{
    return *cl.map_shared_rank(local + (j & ((1 << logR) - 1)), static_cast<unsigned>(j >> logR));
}

// ---------------------------------------------------------------- FP64 Jacobi PCG
// CGSolver::solve (src/solver/LinearSolvers.cpp:420-451) with Jacobi: x = 0,
// r = b, z = D^-1 r, p = z; per iteration q = A p, alpha = r.z / p.q,
// x += alpha p, r -= alpha q, stop when ||r|| / max(||b||, 1e-30) < tol,
// z = D^-1 r, beta = r.z' / r.z, p = z + beta p.  The direction is the only
// vector other CTAs read; it is written after the second sum of an iteration
// and read after the next barrier.  Per row an iteration issues 12 FP64
// instructions; alpha, beta and the stop test are computed once per CTA.
enum ClCtl { kAlpha = 0, kBeta = 1, kLast = 2, kStop = 3, kRz = 4 };

template <int RPT>
__global__ void __launch_bounds__(kClThreads, 1)
    k_cl_pcg64(int n, int logR, const int32_t *__restrict__ rowPtr, const int32_t *__restrict__ colIdx,
               const double *__restrict__ val, const double *__restrict__ invD, const double *__restrict__ b,
               double *__restrict__ x, SolveScalars *s)
{
    const cg::cluster_group cl = cg::this_cluster();
    const int rank = static_cast<int>(cl.block_rank());
    cl.sync();  // every CTA of the cluster has started before any shared memory is written remotely
    extern __shared__ __align__(16) double cl_sm[];
    double *ps = cl_sm;  // the direction of the owned rows
    const int R = 1 << logR;
    __shared__ ClShared sh;
    const int row0 = rank * R;
    const int nr = max(0, min(R, n - row0));
    const double tol = s->tol;
    const int max_iter = s->max_iter;

    double xr[RPT], rr[RPT], dr[RPT], qr[RPT];
    double a[2] = {0.0, 0.0};
#pragma unroll
    for (int k = 0; k < RPT; ++k) {
        const int il = threadIdx.x + k * kClThreads;
        xr[k] = rr[k] = dr[k] = qr[k] = 0.0;
        if (il < nr) {
            const int i = row0 + il;
            const double bi = b[i], d = invD[i], z = d * bi;
            rr[k] = bi;
            dr[k] = d;
            ps[il] = z;
            a[0] += bi * z;
            a[1] += bi * bi;
        }
    }
    int slot = 0;
    double t2[2];
    cl_allreduce<2>(a, t2, sh, slot, cl, [](const double *t, double *c) {
        c[kRz] = t[0];
        c[kLast] = sqrt(t[1]) / std_max(sqrt(t[1]), 1e-30);
    });
    double rz = sh.ctl[kRz];
    const double bnorm = std_max(sqrt(t2[1]), 1e-30);
    double last = sh.ctl[kLast];
    int it = 0, result = 0, status = SIMALL_OK;
    bool run = max_iter > 0;
    if (!run)
        result = max_iter;
    while (run) {
        cl.sync();  // every CTA's direction is complete
        double acc[1] = {0.0};
#pragma unroll
        for (int k = 0; k < RPT; ++k) {
            const int il = threadIdx.x + k * kClThreads;
            if (il < nr) {
                const int i = row0 + il;
                double q = 0.0;
                for (int e = __ldg(rowPtr + i); e < __ldg(rowPtr + i + 1); ++e) {
                    const int j = __ldg(colIdx + e);
                    const int jl = j - row0;
                    const double pj = (jl >= 0 && jl < R) ? ps[jl] : cl_load(cl, ps, logR, j);
                    q = fma(__ldg(val + e), pj, q);
                }
                qr[k] = q;
                acc[0] += ps[il] * q;
            }
        }
        double pq[1];
        cl_allreduce<1>(acc, pq, sh, slot, cl, [rz](const double *t, double *c) {
            c[kAlpha] = t[0] == 0.0 ? 0.0 : rz / t[0];
        });
        if (pq[0] == 0.0) {
            last = sqrt(rz) / bnorm;
            result = it;
            status = SIMALL_ERR_BREAKDOWN;
            break;
        }
        const double alpha = sh.ctl[kAlpha];
        double c[2] = {0.0, 0.0};
        double zr[RPT];
#pragma unroll
        for (int k = 0; k < RPT; ++k) {
            const int il = threadIdx.x + k * kClThreads;
            zr[k] = 0.0;
            if (il < nr) {
                xr[k] = fma(alpha, ps[il], xr[k]);
                rr[k] = fma(-alpha, qr[k], rr[k]);
                zr[k] = dr[k] * rr[k];
                c[0] += rr[k] * rr[k];
                c[1] += rr[k] * zr[k];
            }
        }
        double t[2];
        cl_allreduce<2>(c, t, sh, slot, cl, [rz, bnorm, tol, it, max_iter](const double *tt, double *cc) {
            const double l = sqrt(tt[0]) / bnorm;
            cc[kLast] = l;
            cc[kBeta] = tt[1] / rz;
            cc[kStop] = l < tol ? 1.0 : (it + 1 >= max_iter ? 2.0 : 0.0);
        });
        last = sh.ctl[kLast];
        const double stop = sh.ctl[kStop];
        if (stop == 1.0) {
            result = it + 1;
            break;
        }
        const double beta = sh.ctl[kBeta];
        rz = t[1];
        if (stop == 2.0) {
            it = max_iter;
            result = max_iter;
            break;
        }
        ++it;
        // p = z + beta p: read by the other CTAs after the barrier at the top of the loop
#pragma unroll
        for (int k = 0; k < RPT; ++k) {
            const int il = threadIdx.x + k * kClThreads;
            if (il < nr)
                ps[il] = fma(beta, ps[il], zr[k]);
        }
    }
#pragma unroll
    for (int k = 0; k < RPT; ++k) {
        const int il = threadIdx.x + k * kClThreads;
        if (il < nr)
            x[row0 + il] = xr[k];
    }
    if (rank == 0 && threadIdx.x == 0) {
        s->rz = rz;
        s->bnorm = bnorm;
        s->last = last;
        s->iter = it;
        s->result = result;
        s->status = status;
        s->done = 1;
    }
    cl.sync();  // no CTA leaves while another may still read its shared memory
}

}  // namespace

namespace {

// ---------------------------------------------------------------- mixed precision
// The mixed solver of mixed.cu on one cluster: FP32 CG on S A S (diagonal
// storage, row-sum form), one fused step per iteration (r, x, p updates, the
// product and its four sums; beta from |r - alpha q|^2), FP64 reliable updates
// (x += S xh, r = b - A x from the FP64 CSR, stop test on it, r = S r, then a
// FRESH step that forms p from the replaced residual).  r, q and p are
// double-buffered by step parity in the owners' shared memory; xh stays in
// registers; x lives in global memory (written at folds, read by the true
// residual after a barrier).  The scalar state of the iteration is kept by one
// thread per CTA and broadcast after every sum; all CTAs hold identical state.
// A step's scalars are FP32 and its sums float-float: one thread updates them
// while every other warp of the CTA waits, and on GB300's narrow FP64 pipe
// each FP64 operation or conversion there costs tens of cycles.  FP64 is kept
// for the reliable updates: the true residual, the norms of b.
struct ClMixState {
    double last, bnorm, rr64, b_norm;  // true relative residual; |b| (floored), |r|^2, |b|
    FF rz;                             // r.r of the current step (float-float)
    float t0, sigma0, rmax, alpha, beta;
    float smin;  // smallest iterated residual norm since the last update
    int iter, updates, need, done, result, status, stall;
};

// The shared::cluster address of shared address `a` in the CTA of rank `rank`.
__device__ __forceinline__ uint32_t cl_mapa(uint32_t a, unsigned rank)
{
    uint32_t r;
    asm("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(a), "r"(rank));
    return r;
}

// A load through the cluster's shared window (a shared::cta address names
// this CTA's own memory).  Volatile: kept in program order with the cluster
// barriers around the step.
__device__ __forceinline__ float cl_ld(uint32_t a)
{
    float v;
    asm volatile("ld.shared::cluster.f32 %0, [%1];" : "=f"(v) : "r"(a));
    return v;
}

template <bool FRESH>
__device__ __forceinline__ float cl_pdir(float r, float q, float p, float alpha, float beta)
{
    const float rn = FRESH ? r : __fmaf_rn(-alpha, q, r);
    return __fmaf_rn(beta, p, rn);
}

// alpha = rr / pq and beta = |r - alpha q|^2 / rr, divided in FP32 (they are
// used in FP32); the cancelling sum |r - alpha q|^2 = rr + alpha (alpha qq -
// 2 rq) in float-float.  The totals are renormalised float-float values, so
// their signs are those of their high parts.
__device__ __forceinline__ void clmix_step(ClMixState &st, FF pq, FF qq, FF rr, FF rq)
{
    if (!(pq.hi > 0.0f) || !(rr.hi > 0.0f)) {
        st.status = SIMALL_ERR_BREAKDOWN;
        st.need = 1;
        st.alpha = 0.0f;
        st.beta = 0.0f;
        return;
    }
    const float alpha = __fdiv_rn(rr.hi, pq.hi);
    const FF next = ff_next_rr(rr, qq, rq, alpha);
    st.alpha = alpha;
    st.beta = __fdiv_rn(next.hi > 0.0f ? next.hi : 0.0f, rr.hi);
}

// One fused step over the owned rows.  Buffers [par] hold step k-1, [par ^ 1]
// receive step k; FRESH takes r from rv[par ^ 1] (the replaced residual).
// Shared layout: r[0] r[1] q[0] q[1] p[0] p[1], R floats each; R = 2^logR, so
// the owner of row j is j >> logR and its slot j & (R - 1).  When both
// neighbours of a row on a diagonal lie in this CTA's slice (most rows, on
// most diagonals) they are plain shared-memory loads.  Otherwise they are
// read with 32-bit shared::cluster addresses: this CTA's own shared address
// for a row it owns, the owner's mapped address (mapa) for any other; the
// address is selected, not branched on, so the loads issue together.  A
// neighbour outside [0, n) reads the row itself with a zero coefficient.
template <int ND, int RPT, bool FRESH>
__device__ __forceinline__ void clmix_rows(const cg::cluster_group &cl, int n, int logR, int row0, int nr,
                                           const ClusterMixedArgs &A, const int (&off)[ND], float *base, int par,
                                           float alpha, float beta, float (&xh)[RPT], FF (&acc)[4])
{
    const int R = 1 << logR;
    const unsigned me = static_cast<unsigned>(row0 >> logR);  // this CTA's rank
    // the thread's row index, opaque to the compiler: per-row addresses are
    // formed in every step instead of being hoisted out of the solve loop and
    // held in registers across it
    int tx = static_cast<int>(threadIdx.x);
    asm volatile("" : "+r"(tx));
    const float *rs = base + (FRESH ? par ^ 1 : par) * R;
    const float *qs = base + (2 + par) * R;
    const float *ps = base + (4 + par) * R;
    // shared-window addresses: r's, and the distances from r's array to q's and p's
    const uint32_t rs_a = smem_u32(rs);
    const uint32_t qs_d = smem_u32(qs) - rs_a, ps_d = smem_u32(ps) - rs_a;
    float *rout = base + (par ^ 1) * R;
    float *qout = base + (2 + (par ^ 1)) * R;
    float *pout = base + (4 + (par ^ 1)) * R;
#pragma unroll
    for (int k = 0; k < RPT; ++k) {
        const int il = tx + k * kClThreads;
        if (il >= nr)
            continue;
        const int i = row0 + il;
        float u[2 * ND], rj[2 * ND], qj[2 * ND], pj[2 * ND];
#pragma unroll
        for (int d = 0; d < ND; ++d) {
            const int od = off[d];
            const float *Ud = A.U + d * A.ldU;
            if (ND <= 3 && il >= od && il + od < nr) {
                // both neighbours on this diagonal in this CTA's slice (so in
                // [0, n)): plain shared-memory loads, no checks (not with 4
                // diagonals: the two paths then spill at 128 registers)
                u[2 * d] = __ldg(Ud + i);
                u[2 * d + 1] = __ldg(Ud + i - od);
                rj[2 * d] = rs[il + od];
                rj[2 * d + 1] = rs[il - od];
                qj[2 * d] = FRESH ? 0.0f : qs[il + od];
                qj[2 * d + 1] = FRESH ? 0.0f : qs[il - od];
                pj[2 * d] = ps[il + od];
                pj[2 * d + 1] = ps[il - od];
                continue;
            }
#pragma unroll
            for (int side = 0; side < 2; ++side) {
                const int t = 2 * d + side;
                const int j0 = side ? i - od : i + od;
                const bool ok = j0 >= 0 && j0 < n;
                const int j = ok ? j0 : i;
                u[t] = ok ? __ldg(Ud + (side ? j : i)) : 0.0f;
                const unsigned owner = static_cast<unsigned>(j >> logR);
                const int jl = j & (R - 1);
                const uint32_t a = owner == me ? rs_a + 4u * jl : cl_mapa(rs_a + 4u * jl, owner);
                rj[t] = cl_ld(a);
                qj[t] = FRESH ? 0.0f : cl_ld(a + qs_d);
                pj[t] = cl_ld(a + ps_d);
            }
        }
        const float ro = rs[il], po = ps[il], ei = __ldg(A.e + i);
        const float rk = FRESH ? ro : __fmaf_rn(-alpha, qs[il], ro);
        const float pk = __fmaf_rn(beta, po, rk);
        if (!FRESH) {
            rout[il] = rk;
            xh[k] = __fmaf_rn(alpha, po, xh[k]);
        }
        pout[il] = pk;
        float y = ei * pk;
#pragma unroll
        for (int t = 0; t < 2 * ND; ++t)
            y = __fmaf_rn(-u[t], pk - cl_pdir<FRESH>(rj[t], qj[t], pj[t], alpha, beta), y);
        qout[il] = y;
        ff_dot_add(acc[0], pk, y);
        ff_dot_add(acc[1], y, y);
        ff_dot_add(acc[2], rk, rk);
        ff_dot_add(acc[3], rk, y);
    }
}

// The whole mixed solve of one system on the calling cluster; returns the
// final state (identical in every CTA).
template <int ND, int RPT>
__device__ __forceinline__ const ClMixState &cl_mixed_body(const cg::cluster_group &cl, int n, int logR,
                                                           const ClusterMixedArgs &A,
                                                           const int32_t *__restrict__ rowPtr,
                                                           const int32_t *__restrict__ colIdx,
                                                           const double *__restrict__ val,
                                                           const double *__restrict__ b, double *__restrict__ x,
                                                           double tol, double delta, int max_iter)
{
    const int rank = static_cast<int>(cl.block_rank());
    cl.sync();  // every CTA of the cluster has started before any shared memory is written remotely
    extern __shared__ __align__(16) double cl_sm[];
    const int R = 1 << logR;
    float *base = reinterpret_cast<float *>(cl_sm);  // r[0] r[1] q[0] q[1] p[0] p[1]
    int off[ND];
#pragma unroll
    for (int d = 0; d < ND; ++d)
        off[d] = A.off[d];
    __shared__ ClShared sh;
    __shared__ ClMixState st_sh;
    ClMixState &st = st_sh;
    ClMixState *const stp = &st_sh;
    const int row0 = rank * R;
    const int nr = max(0, min(R, n - row0));

    // init: x = 0, r = S b (r[0]), p_old = 0 (p[1]), xh = 0
    float xh[RPT];
    float a0 = 0.0f;
    double a1 = 0.0;
#pragma unroll
    for (int k = 0; k < RPT; ++k) {
        xh[k] = 0.0f;
        const int il = threadIdx.x + k * kClThreads;
        if (il < nr) {
            const int i = row0 + il;
            const double bi = b[i];
            const float r = static_cast<float>(bi * A.scale[i]);
            x[i] = 0.0;
            base[il] = r;          // r[0]
            base[5 * R + il] = 0.0f;  // p[1]
            a0 += r * r;
            a1 += bi * bi;
        }
    }
    int slot = 0;
    {
        const double v[2] = {static_cast<double>(a0), a1};
        double t[2];
        cl_allreduce<2>(v, t, sh, slot, cl, [stp, tol, max_iter](const double *tt, double *) {
            const double bn = sqrt(tt[1]);
            stp->b_norm = bn;
            stp->bnorm = std_max(bn, 1e-30);
            stp->rz = FF{static_cast<float>(tt[0]), 0.0f};
            stp->sigma0 = sqrtf(static_cast<float>(tt[0]));
            stp->rmax = stp->sigma0;
            stp->smin = stp->sigma0;
            stp->stall = 0;
            const double t0 = bn / stp->bnorm;
            stp->t0 = static_cast<float>(t0);
            stp->last = t0;
            stp->rr64 = tt[1];
            stp->alpha = 0.0f;
            stp->beta = 0.0f;
            stp->iter = 0;
            stp->updates = 0;
            stp->need = 2;
            stp->status = SIMALL_OK;
            stp->done = 0;
            stp->result = 0;
            if (t0 < tol) {
                stp->done = 1;
            } else if (max_iter <= 0) {
                stp->done = 1;
                stp->result = max_iter;
            }
        });
    }
    auto fresh_fin = [stp](const FF *t, double *) {
        stp->rz = t[2];
        stp->sigma0 = sqrtf(t[2].hi);
        stp->rmax = stp->sigma0;
        stp->smin = stp->sigma0;
        stp->stall = 0;
        if (stp->need == 1)
            stp->updates += 1;
        stp->need = 0;
        clmix_step(*stp, t[0], t[1], t[2], t[3]);
    };
    const float tolf = static_cast<float>(tol), deltaf = static_cast<float>(delta);
    int par = 1;
    if (!st.done) {
        FF acc[4] = {ff_zero(), ff_zero(), ff_zero(), ff_zero()};
        clmix_rows<ND, RPT, true>(cl, n, logR, row0, nr, A, off, base, par, 0.0f, st.beta, xh, acc);
        FF t[4];
        cl_allreduce<4>(acc, t, sh, slot, cl, fresh_fin);
    }
    par = 0;
    while (!st.done) {
        FF acc[4] = {ff_zero(), ff_zero(), ff_zero(), ff_zero()};
        clmix_rows<ND, RPT, false>(cl, n, logR, row0, nr, A, off, base, par, st.alpha, st.beta, xh, acc);
        FF t[4];
        cl_allreduce<4>(acc, t, sh, slot, cl, [stp, tolf, deltaf, max_iter](const FF *tt, double *) {
            // the trigger and the estimate in FP32 (the stop test itself is the
            // FP64 true residual of the reliable update it triggers)
            stp->iter += 1;
            const float sigma = sqrtf(tt[2].hi);
            const float est = stp->t0 * __fdiv_rn(sigma, stp->sigma0);
            if (sigma < stp->smin) {
                stp->smin = sigma;
                stp->stall = 0;
            } else {
                stp->stall += 1;
            }
            if (stp->need || sigma < deltaf * stp->rmax || est < tolf || stp->iter >= max_iter ||
                stp->stall >= kMixedStallSteps) {
                stp->need = 1;
                return;
            }
            if (sigma > stp->rmax)
                stp->rmax = sigma;
            stp->rz = tt[2];
            clmix_step(*stp, tt[0], tt[1], tt[2], tt[3]);
        });
        if (st.need) {
            // reliable update: x += S xh (FP64), r = b - A x, r = S r into r[par ^ 1]
#pragma unroll
            for (int k = 0; k < RPT; ++k) {
                const int il = threadIdx.x + k * kClThreads;
                if (il < nr) {
                    const int i = row0 + il;
                    x[i] += A.scale[i] * static_cast<double>(xh[k]);
                }
                xh[k] = 0.0f;
            }
            cl.sync();  // x complete in global memory
            double v[2] = {0.0, 0.0};
#pragma unroll
            for (int k = 0; k < RPT; ++k) {
                const int il = threadIdx.x + k * kClThreads;
                if (il < nr) {
                    const int i = row0 + il;
                    double y = 0.0;
                    for (int e = __ldg(rowPtr + i); e < __ldg(rowPtr + i + 1); ++e)
                        y = fma(__ldg(val + e), __ldcg(x + __ldg(colIdx + e)), y);  // other SMs' x: via L2
                    const double r = b[i] - y;
                    const float rf = static_cast<float>(A.scale[i] * r);
                    base[(par ^ 1) * R + il] = rf;
                    v[0] += r * r;
                    v[1] += static_cast<double>(rf) * rf;
                }
            }
            double t2[2];
            cl_allreduce<2>(v, t2, sh, slot, cl, [stp, tol, max_iter](const double *tt, double *) {
                stp->rr64 = tt[0];
                const double tr = sqrt(tt[0]) / stp->bnorm;
                stp->last = tr;
                stp->t0 = static_cast<float>(tr);
                if (tr < tol) {
                    stp->done = 1;
                    stp->result = stp->iter;
                } else if (stp->iter >= max_iter || stp->status == SIMALL_ERR_BREAKDOWN) {
                    stp->done = 1;
                    stp->result = stp->iter >= max_iter ? max_iter : stp->iter;
                } else {
                    stp->beta = static_cast<float>(tt[1] / ff_double(stp->rz));
                }
            });
            if (st.done)
                break;
            FF acc2[4] = {ff_zero(), ff_zero(), ff_zero(), ff_zero()};
            clmix_rows<ND, RPT, true>(cl, n, logR, row0, nr, A, off, base, par, 0.0f, st.beta, xh, acc2);
            FF t4[4];
            cl_allreduce<4>(acc2, t4, sh, slot, cl, fresh_fin);
        }
        par ^= 1;
    }
    cl.sync();  // no CTA leaves while another may still read its shared memory
    return st;
}

template <int ND, int RPT>
__global__ void __launch_bounds__(kClThreads, 1)
    k_cl_mixed(int n, int logR, ClusterMixedArgs A, const int32_t *__restrict__ rowPtr,
               const int32_t *__restrict__ colIdx, const double *__restrict__ val, const double *__restrict__ b,
               double *__restrict__ x, SolveScalars *s)
{
    const cg::cluster_group cl = cg::this_cluster();
    const ClMixState &st =
        cl_mixed_body<ND, RPT>(cl, n, logR, A, rowPtr, colIdx, val, b, x, s->tol, s->delta, s->max_iter);
    if (cl.block_rank() == 0 && threadIdx.x == 0) {
        s->bnorm = st.bnorm;
        s->last = st.last;
        s->rr = st.rr64;
        s->iter = st.iter;
        s->result = st.result;
        s->status = st.status;
        s->updates = st.updates;
        s->done = 1;
    }
}

// Many systems on a fixed set of clusters: cluster c solves items c, c + K,
// c + 2K, ... (K clusters in the grid; the items are ordered largest first),
// so the batch decides how many SMs the clusters hold.  b, x and the results
// are the batch's, at each item's row offset.
template <int ND, int RPT>
__global__ void __launch_bounds__(kClThreads, 1)
    k_cl_mixed_batch(const ClBatchItem *__restrict__ items, int count, const double *__restrict__ b,
                     double *__restrict__ x, double tol, double delta, int max_iter)
{
    const cg::cluster_group cl = cg::this_cluster();
    const int K = static_cast<int>(gridDim.x / cl.num_blocks());
    for (int c = static_cast<int>(blockIdx.x / cl.num_blocks()); c < count; c += K) {
        const ClBatchItem it = items[c];
        const ClMixState &st = cl_mixed_body<ND, RPT>(cl, it.n, it.logR, it.A, it.rowPtr, it.colIdx, it.val,
                                                      b + it.row0, x + it.row0, tol, delta, max_iter);
        if (cl.block_rank() == 0 && threadIdx.x == 0) {
            ClBatchResult &o = *it.out;
            o.iterations = st.iter;
            o.updates = st.updates;
            o.status = st.status;
            o.converged = st.last < tol ? 1 : 0;
            o.true_residual = st.last;
            o.b_norm = st.b_norm;
        }
        cl.sync();  // the state of this item is read before the next item's init overwrites it
    }
}

}  // namespace

namespace {

// Whether `kernel` can run as one cluster of C CTAs with `smem` bytes of
// dynamic shared memory each on this device.
bool cluster_fits(simall_context *ctx, const void *kernel, int C, size_t smem)
{
    if (C > 8 && cudaFuncSetAttribute(kernel, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    if (cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem)) !=
        cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    cudaLaunchConfig_t cfg{};
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = C;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.gridDim = dim3(C);
    cfg.blockDim = dim3(kClThreads);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = ctx->stream;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    int clusters = 0;
    if (cudaOccupancyMaxActiveClusters(&clusters, kernel, &cfg) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return clusters >= 1;
}

template <typename K, typename... Args>
int launch_cluster(simall_context *ctx, K kernel, int C, size_t smem, Args... args)
{
    cudaLaunchConfig_t cfg{};
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = C;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.gridDim = dim3(C);
    cfg.blockDim = dim3(kClThreads);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = ctx->stream;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    SIMALL_CUDA_TRY(ctx, cudaLaunchKernelEx(&cfg, kernel, args...));
    SIMALL_LAUNCH_CHECK(ctx);
    return SIMALL_OK;
}

template <int RPT> int try_pcg64(simall_solver *s, int C, int logR, int *status)
{
    simall_context *ctx = s->ctx;
    const size_t smem = sizeof(double) * (static_cast<size_t>(1) << logR);
    if (!cluster_fits(ctx, reinterpret_cast<const void *>(k_cl_pcg64<RPT>), C, smem))
        return 0;
    const int st = launch_cluster(ctx, k_cl_pcg64<RPT>, C, smem, static_cast<int>(s->n), logR, s->rowPtr, s->colIdx,
                                  s->values, static_cast<const double *>(s->invDiag.p),
                                  static_cast<const double *>(s->b.p), s->x.p, s->scal.p);
    *status = st ? st : solver_fetch_scalars(s);
    s->engine = 1;
    return 1;
}

// As try_mixed_rpt, up to kClPcg64MaxRowsPerCta rows.
template <int RPT> int try_pcg64_rpt(simall_solver *s, int C, int logR, int rpt, int *status)
{
    if (rpt <= RPT)
        return try_pcg64<RPT>(s, C, logR, status);
    if constexpr (2 * RPT * kClThreads <= kClPcg64MaxRowsPerCta)
        return try_pcg64_rpt<2 * RPT>(s, C, logR, rpt, status);
    return 0;
}

template <int ND, int RPT> int try_mixed(simall_solver *s, const ClusterMixedArgs &a, int C, int logR, int *status)
{
    simall_context *ctx = s->ctx;
    const size_t smem = 6 * sizeof(float) * (static_cast<size_t>(1) << logR);
    if (!cluster_fits(ctx, reinterpret_cast<const void *>(k_cl_mixed<ND, RPT>), C, smem))
        return 0;
    const int st = launch_cluster(ctx, k_cl_mixed<ND, RPT>, C, smem, static_cast<int>(s->n), logR, a, s->rowPtr,
                                  s->colIdx, s->values, static_cast<const double *>(s->b.p), s->x.p, s->scal.p);
    *status = st ? st : solver_fetch_scalars(s);
    s->engine = 1;
    return 1;
}

// The smallest RPT (a power of two, from RPT up) with RPT * kClThreads >= the
// slice's rows, instantiated only up to kClMaxRowsPerCta rows.
template <int ND, int RPT>
int try_mixed_rpt(simall_solver *s, const ClusterMixedArgs &a, int C, int logR, int rpt, int *status)
{
    if (rpt <= RPT)
        return try_mixed<ND, RPT>(s, a, C, logR, status);
    if constexpr (2 * RPT * kClThreads <= kClMaxRowsPerCta)
        return try_mixed_rpt<ND, 2 * RPT>(s, a, C, logR, rpt, status);
    return 0;
}

template <int ND> int try_mixed_nd(simall_solver *s, const ClusterMixedArgs &a, int C, int logR, int *status)
{
    // every row of the slice needs a slot: RPT * kClThreads >= 2^logR
    const int rpt = ((1 << logR) + kClThreads - 1) / kClThreads;
    return try_mixed_rpt<ND, 1>(s, a, C, logR, rpt, status);
}

// Slice length (a power of two, at least 256 rows) and cluster size for n rows
// on at most maxC CTAs; false when n does not fit.
bool cluster_shape(int64_t n, int maxC, int *C, int *logR)
{
    int lr = 8;
    while ((static_cast<int64_t>(maxC) << lr) < n)
        ++lr;
    if ((1 << lr) > kClMaxRowsPerCta)
        return false;
    *logR = lr;
    *C = static_cast<int>((n + (1 << lr) - 1) >> lr);
    return *C >= 1 && *C <= maxC;
}

}  // namespace

// Mixed-precision CG on one cluster (diagonal storage, up to 4 diagonals).
// Returns 0 (not taken) or 1 with *status set.
int cluster_mixed_solve(simall_solver *s, const ClusterMixedArgs &a, int *status)
{
    if (s->n <= 0 || s->n > 16 * kClMaxRowsPerCta || s->cfg.max_iterations > kClMaxIterations || a.nd < 1 ||
        a.nd > 4)
        return 0;
    for (int maxC : {16, 8}) {
        int C = 0, logR = 0;
        if (!cluster_shape(s->n, maxC, &C, &logR))
            continue;
        const int taken = a.nd == 1   ? try_mixed_nd<1>(s, a, C, logR, status)
                          : a.nd == 2 ? try_mixed_nd<2>(s, a, C, logR, status)
                          : a.nd == 3 ? try_mixed_nd<3>(s, a, C, logR, status)
                                      : try_mixed_nd<4>(s, a, C, logR, status);
        if (taken)
            return 1;
    }
    return 0;
}

// The large systems of a batch, one cluster of C CTAs each, rows in slices of
// 2^logR (every item: n <= C 2^logR); all items store nd diagonals.
namespace {
template <int ND, int RPT>
int launch_mixed_batch(simall_context *ctx, cudaStream_t stream, int C, int logR, int clusters, const ClBatchItem *items,
                       int count, const double *b, double *x, double tol, double delta, int max_iter)
{
    const size_t smem = 6 * sizeof(float) * (static_cast<size_t>(1) << logR);
    const void *fn = reinterpret_cast<const void *>(k_cl_mixed_batch<ND, RPT>);
    if (!cluster_fits(ctx, fn, C, smem))
        return fail(ctx, SIMALL_ERR_UNSUPPORTED, "a cluster of %d CTAs with %zu bytes each does not fit", C, smem);
    cudaLaunchConfig_t cfg{};
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = C;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.gridDim = dim3(static_cast<unsigned>(C) * static_cast<unsigned>(std::min(count, clusters)));
    cfg.blockDim = dim3(kClThreads);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = stream;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    SIMALL_CUDA_TRY(ctx,
                    cudaLaunchKernelEx(&cfg, k_cl_mixed_batch<ND, RPT>, items, count, b, x, tol, delta, max_iter));
    SIMALL_LAUNCH_CHECK(ctx);
    return SIMALL_OK;
}

// Smallest RPT (from RPT up, powers of two) that covers the slice; logR is
// checked against kClMaxRowsPerCta by the caller.
template <int ND, int RPT>
int launch_mixed_batch_rpt(simall_context *ctx, cudaStream_t stream, int C, int logR, int rpt, int clusters,
                           const ClBatchItem *items, int count, const double *b, double *x, double tol, double delta,
                           int max_iter)
{
    if constexpr (2 * RPT * kClThreads <= kClMaxRowsPerCta) {
        if (rpt > RPT)
            return launch_mixed_batch_rpt<ND, 2 * RPT>(ctx, stream, C, logR, rpt, clusters, items, count, b, x, tol,
                                                       delta, max_iter);
    }
    return launch_mixed_batch<ND, RPT>(ctx, stream, C, logR, clusters, items, count, b, x, tol, delta, max_iter);
}

template <int ND>
int launch_mixed_batch_nd(simall_context *ctx, cudaStream_t stream, int C, int logR, int clusters,
                          const ClBatchItem *items, int count, const double *b, double *x, double tol, double delta,
                          int max_iter)
{
    const int rpt = ((1 << logR) + kClThreads - 1) / kClThreads;
    constexpr int kMinRpt = 4 * 256 / kClThreads > 1 ? 4 * 256 / kClThreads : 1;  // slices of >= 1024 rows
    return launch_mixed_batch_rpt<ND, kMinRpt>(ctx, stream, C, logR, rpt, clusters, items, count, b, x, tol, delta,
                                               max_iter);
}
}  // namespace

int cluster_mixed_batch(simall_context *ctx, cudaStream_t stream, int nd, int C, int logR, int clusters,
                        const ClBatchItem *items, int count, const double *b, double *x, double tol, double delta,
                        int max_iter)
{
    if (count <= 0)
        return SIMALL_OK;
    if (nd < 1 || nd > 4 || C < 1 || C > kClMaxCtas || logR < 8 || (1 << logR) > kClMaxRowsPerCta ||
        max_iter > kClMaxIterations || clusters < 1)
        return fail(ctx, SIMALL_ERR_INVALID_ARGUMENT, "cluster batch: nd %d, C %d, logR %d", nd, C, logR);
    switch (nd) {
    case 1: return launch_mixed_batch_nd<1>(ctx, stream, C, logR, clusters, items, count, b, x, tol, delta, max_iter);
    case 2: return launch_mixed_batch_nd<2>(ctx, stream, C, logR, clusters, items, count, b, x, tol, delta, max_iter);
    case 3: return launch_mixed_batch_nd<3>(ctx, stream, C, logR, clusters, items, count, b, x, tol, delta, max_iter);
    default: return launch_mixed_batch_nd<4>(ctx, stream, C, logR, clusters, items, count, b, x, tol, delta,
                                             max_iter);
    }
}

// FP64 Jacobi PCG on one cluster.  Returns 0 (not taken: the system does not
// fit, or the device cannot run the cluster) or 1 with *status set.
int cluster_fp64_solve(simall_solver *s, int *status)
{
    // one launch runs the whole solve: keep it short even when it does not converge
    if (s->n <= 0 || s->n > 16 * kClPcg64MaxRowsPerCta || s->nnz > INT32_MAX || s->cfg.max_iterations > kClMaxIterations)
        return 0;
    for (int maxC : {16, 8}) {
        int C = 0, logR = 0;
        if (!cluster_shape(s->n, maxC, &C, &logR))
            continue;
        const int rpt = ((1 << logR) + kClThreads - 1) / kClThreads;
        const int taken = try_pcg64_rpt<1>(s, C, logR, rpt, status);
        if (taken)
            return 1;
    }
    return 0;
}

}  // namespace simall
