// Level-scheduled ILU(0) on the device.
//
// ILU0Preconditioner::setup (src/solver/LinearSolvers.cpp:81-122) factors row
// i using only rows k < i of its own lower pattern, each already final, and
// the triangular sweeps of ILU0Preconditioner::apply (:123-151) have the same
// dependency structure.  Grouping rows into dependency levels (row i's level
// is one more than the deepest row it reads) lets every row of a level run in
// parallel while each row keeps the reference's exact sequence of operations:
// products and differences are rounded separately (__dmul_rn/__dsub_rn) and
// in column order, so the factor and both sweeps are bit-identical to the
// reference.  Multicolouring would be faster but changes the factor.
//
// Systems of up to kIluSmallRows rows factor and sweep in one CTA (below).
// Larger ones: the factorisation (once per solve) launches one kernel per
// level, and the sweeps (twice per PCG iteration) run as one kernel each
// without levels
// between launches: warps take 32 consecutive rows of the level order from an
// atomic ticket, and a row waits only for the rows it reads: the output
// vector starts the sweep filled with a pending marker (a signalling NaN),
// each row publishes its value with one relaxed store, and a reader polls the
// values it needs until none is pending.  Rows are handed out in level order,
// so every row waited for was handed to a warp that is already running; the
// wait is bounded and a timeout is reported (it never happens unless a row is
// never produced).
//
// SSOR (SsorPreconditioner, :163-231, with the w = 1 that make_preconditioner
// gives it) has the same dependency structure and runs on the same schedule
// with A's own values: forward y_i = (r_i - sum_{j<i} a_ij y_j) invD_i,
// backward z_i = (a_ii y_i - sum_{j>i} a_ij z_j) invD_i, each product and
// difference rounded as the reference rounds it (w = 1 and 2 - w = 1 scale
// exactly).
#include "device.cuh"
#include "solver.hpp"
#include "sweep.cuh"

#include <algorithm>
#include <chrono>
#include <new>

namespace simall {

int g_sweep_ctas_per_sm = 2;
unsigned g_sweep_backoff_ns = 0;
bool g_sweep_reciprocal = true;

namespace {

// a / b rounded to nearest from rb = RN(1/b) (a correctly rounded reciprocal):
// q = RN(a rb) is within an ulp of a/b, the remainder r = a - b q is exact
// with one FMA, and q + r rb rounded once is RN(a/b) (Markstein's theorem,
// IBM J. Res. Dev. 34(1), 1990; Handbook of Floating-Point Arithmetic,
// 2nd ed., Thm. 5.9).  Three FP64 operations instead of a full division --
// GB300's FP64 pipe is narrow enough that the divisions of the backward sweep
// set its time.  The theorem needs a, b, the quotient and the remainder away
// from overflow and underflow, and a zero numerator keeps its sign only
// through the product; outside that range (or when b has no usable
// reciprocal) the division itself is taken.
// Biased exponent field of x, on the integer pipe (GB300 issues about 1.6 FP64
// operations per clock per SM, so range tests in FP64 would cost as much as
// the division they replace).
__device__ __forceinline__ unsigned biased_exp(double x)
{
    return static_cast<unsigned>(__double2hiint(x) >> 20) & 0x7ffu;
}

__device__ __forceinline__ double div_rn_by_recip(double a, double b, double rb)
{
    const double q = a * rb;
    // |a|, |q|, |rb| in [2^-900, 2^901): biased exponents in [123, 1924]
    const unsigned ea = biased_exp(a) - 123u, eq = biased_exp(q) - 123u, er = biased_exp(rb) - 123u;
    if ((ea | eq | er) <= 1801u && ea <= 1801u && eq <= 1801u && er <= 1801u) {
        const double r = fma(-q, b, a);
        return fma(r, rb, q);
    }
    return __ddiv_rn(a, b);
}


// One level of the IKJ factorisation, one thread per row.
__global__ void __launch_bounds__(kBlock) k_ilu_factor_level(const int32_t *__restrict__ rows, int cnt,
                                                             const int32_t *__restrict__ rowPtr,
                                                             const int32_t *__restrict__ colIdx,
                                                             const int32_t *__restrict__ diagPtr, double *lu)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= cnt)
        return;
    const int i = rows[t];
    const int end = rowPtr[i + 1];
    for (int kp = rowPtr[i]; kp < end; ++kp) {
        const int k = colIdx[kp];
        if (k >= i)
            break;
        const int dk = diagPtr[k];
        if (dk < 0)
            continue;
        const double piv = lu[dk];
        if (piv == 0.0)
            continue;
        const double m = __ddiv_rn(lu[kp], piv);
        lu[kp] = m;
        const int kend = rowPtr[k + 1];
        for (int jp = dk + 1; jp < kend; ++jp) {
            const int j = colIdx[jp];
            for (int qp = kp + 1; qp < end; ++qp) {
                const int c = colIdx[qp];
                if (c == j) {
                    lu[qp] = __dsub_rn(lu[qp], __dmul_rn(m, lu[jp]));
                    break;
                }
                if (c > j)
                    break;
            }
        }
    }
}

// Forward sweep of one level: y_i = r_i - sum_{j<i} l_ij y_j.
__global__ void __launch_bounds__(kBlock) k_ilu_fwd_level(const int32_t *__restrict__ rows, int cnt,
                                                          const int32_t *__restrict__ rowPtr,
                                                          const int32_t *__restrict__ colIdx,
                                                          const double *__restrict__ lu, const double *__restrict__ r,
                                                          double *y)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= cnt)
        return;
    const int i = rows[t];
    double s = r[i];
    for (int kp = rowPtr[i]; kp < rowPtr[i + 1]; ++kp) {
        const int j = colIdx[kp];
        if (j >= i)
            break;
        s = __dsub_rn(s, __dmul_rn(lu[kp], __ldcg(y + j)));
    }
    y[i] = s;
}

// Backward sweep of one level: z_i = (y_i - sum_{j>i} u_ij z_j) / u_ii.
__global__ void __launch_bounds__(kBlock) k_ilu_bwd_level(const int32_t *__restrict__ rows, int cnt,
                                                          const int32_t *__restrict__ rowPtr,
                                                          const int32_t *__restrict__ colIdx,
                                                          const int32_t *__restrict__ diagPtr,
                                                          const double *__restrict__ lu, const double *__restrict__ y,
                                                          double *z)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= cnt)
        return;
    const int i = rows[t];
    double s = y[i];
    const int kd = diagPtr[i];
    for (int kp = kd + 1; kp < rowPtr[i + 1]; ++kp)
        s = __dsub_rn(s, __dmul_rn(lu[kp], __ldcg(z + colIdx[kp])));
    z[i] = (kd >= 0 && lu[kd] != 0.0) ? __ddiv_rn(s, lu[kd]) : s;
}

// Forward sweep y_i = r_i - sum_{j<i} l_ij y_j over rows in level order
// (SSOR: a_ij, and the sum times invD_i).  y holds kPending until a row's value
// lands (k_sweep_begin_values).  Dependencies are taken four at a time: poll
// the four values, then apply them in column order (the reference's order).
template <bool SSOR>
__global__ void __launch_bounds__(kBlock) k_ilu_fwd_free(int n, const int32_t *__restrict__ order,
                                                         const int32_t *__restrict__ rowPtr,
                                                         const int32_t *__restrict__ colIdx,
                                                         const double *__restrict__ lu, const double *__restrict__ r,
                                                         const double *__restrict__ invD, double *y, unsigned *ctl,
                                                         unsigned backoff)
{
    const int lane = threadIdx.x & 31;
    bool ok = true;
    for (;;) {
        int base = 0;
        if (lane == 0)
            base = static_cast<int>(atomicAdd(ctl, 32u));
        base = __shfl_sync(0xffffffffu, base, 0);
        if (base >= n)
            break;
        const int t = base + lane;
        if (t < n) {
            const int i = __ldg(order + t);
            double s = __ldg(r + i);
            const int end = __ldg(rowPtr + i + 1);
            for (int kp = __ldg(rowPtr + i); kp < end;) {
                int j[4];
                bool dep[4];
                double a[4];
                int cnt = 0;
#pragma unroll
                for (int q = 0; q < 4; ++q) {
                    const bool in = kp + q < end;
                    const int jj = in ? __ldg(colIdx + kp + q) : i;
                    a[q] = in ? __ldg(lu + kp + q) : 0.0;  // the row's own data: loaded before the wait
                    j[q] = jj < i ? jj : i;
                    cnt += (jj < i && cnt == q) ? 1 : 0;
                }
                if (cnt == 0)
                    break;
#pragma unroll
                for (int q = 0; q < 4; ++q)
                    dep[q] = q < cnt;
                double v[4];
                ok = wait_values4(y, j, dep, v, backoff) && ok;
#pragma unroll
                for (int q = 0; q < 4; ++q)
                    if (q < cnt)
                        s = __dsub_rn(s, __dmul_rn(a[q], v[q]));
                kp += cnt;
                if (cnt < 4)
                    break;
            }
            if (SSOR)
                s = __dmul_rn(s, __ldg(invD + i));
            st_value(y + i, s);
        }
    }
    if (!ok)
        atomicOr(ctl + 2, 1u);
}

// Backward sweep z_i = (y_i - sum_{j>i} u_ij z_j) / u_ii over rows in level order
// (SSOR: (a_ii y_i - sum_{j>i} a_ij z_j) invD_i); z holds kPending until a
// row's value lands.  The division runs through rdiag = RN(1/u_ii) when given
// (div_rn_by_recip: the same bits as the division, three FP64 operations on
// the chain instead of a full divide), else as a division.
template <bool SSOR>
__global__ void __launch_bounds__(kBlock) k_ilu_bwd_free(int n, const int32_t *__restrict__ order,
                                                         const int32_t *__restrict__ rowPtr,
                                                         const int32_t *__restrict__ colIdx,
                                                         const int32_t *__restrict__ diagPtr,
                                                         const double *__restrict__ lu, const double *__restrict__ y,
                                                         const double *__restrict__ invD,
                                                         const double *__restrict__ rdiag, double *z, unsigned *ctl,
                                                         unsigned backoff)
{
    const int lane = threadIdx.x & 31;
    bool ok = true;
    for (;;) {
        int base = 0;
        if (lane == 0)
            base = static_cast<int>(atomicAdd(ctl, 32u));
        base = __shfl_sync(0xffffffffu, base, 0);
        if (base >= n)
            break;
        const int t = base + lane;
        if (t < n) {
            const int i = __ldg(order + t);
            const int kd = __ldg(diagPtr + i);
            double s = __ldcg(y + i);
            if (SSOR)  // v_i = a_ii y_i (the diagonal is present: the CSR contract)
                s = __dmul_rn(__ldg(lu + kd), s);
            const int end = __ldg(rowPtr + i + 1);
            for (int kp = kd + 1; kp < end;) {
                int j[4];
                bool dep[4];
                double a[4];
                int cnt = 0;
#pragma unroll
                for (int q = 0; q < 4; ++q) {
                    const bool in = kp + q < end;
                    j[q] = in ? __ldg(colIdx + kp + q) : i;
                    a[q] = in ? __ldg(lu + kp + q) : 0.0;
                    dep[q] = in;
                    cnt += in ? 1 : 0;
                }
                double v[4];
                ok = wait_values4(z, j, dep, v, backoff) && ok;
#pragma unroll
                for (int q = 0; q < 4; ++q)
                    if (q < cnt)
                        s = __dsub_rn(s, __dmul_rn(a[q], v[q]));
                kp += cnt;
            }
            if (SSOR) {
                st_value(z + i, __dmul_rn(s, __ldg(invD + i)));
            } else {
                const double dv = kd >= 0 ? __ldg(lu + kd) : 0.0;
                double zi = s;
                if (kd >= 0 && dv != 0.0)
                    zi = rdiag ? div_rn_by_recip(s, dv, __ldg(rdiag + i)) : __ddiv_rn(s, dv);
                st_value(z + i, zi);
            }
        }
    }
    if (!ok)
        atomicOr(ctl + 2, 1u);
}

// ---------------------------------------------------------------- one CTA
// For small systems the dependency chain, not the bandwidth, sets the time:
// one kernel launch per level or a polled value per row cost microseconds per level,
// while one CTA walking the levels with a block barrier between them pays a
// barrier and an L2 round trip.  The sweep vector lives in shared memory (the
// backward sweep overwrites y with z in place: row i reads y_i and the final
// z_j of rows in earlier backward levels only).  Same per-row operations, so
// the results are bit-identical to the reference's.
constexpr int kIluSmallThreads = 1024;
constexpr int kIluSmallRows = 24576;  // 192 KB of shared memory

__global__ void __launch_bounds__(kIluSmallThreads) k_ilu_factor_small(int nlev, const int32_t *__restrict__ lvl,
                                                                       const int32_t *__restrict__ rows,
                                                                       const int32_t *__restrict__ rowPtr,
                                                                       const int32_t *__restrict__ colIdx,
                                                                       const int32_t *__restrict__ diagPtr, double *lu,
                                                                       double *rpiv)
{
    // level 0 rows keep their diagonal: their pivots' reciprocals first
    for (int t = lvl[0] + threadIdx.x; t < lvl[nlev > 0 ? 1 : 0]; t += blockDim.x) {
        const int i = rows[t], di = diagPtr[i];
        rpiv[i] = (di >= 0 && lu[di] != 0.0) ? __drcp_rn(lu[di]) : 0.0;
    }
    __syncthreads();
    for (int l = 1; l < nlev; ++l) {  // level 0 rows have no lower entries
        const int a = lvl[l], b = lvl[l + 1];
        for (int t = a + threadIdx.x; t < b; t += blockDim.x) {
            const int i = rows[t];
            const int end = rowPtr[i + 1];
            for (int kp = rowPtr[i]; kp < end; ++kp) {
                const int k = colIdx[kp];
                if (k >= i)
                    break;
                const int dk = diagPtr[k];
                if (dk < 0)
                    continue;
                const double piv = lu[dk];
                if (piv == 0.0)
                    continue;
                const double m = div_rn_by_recip(lu[kp], piv, rpiv[k]);
                lu[kp] = m;
                const int kend = rowPtr[k + 1];
                for (int jp = dk + 1; jp < kend; ++jp) {
                    const int j = colIdx[jp];
                    for (int qp = kp + 1; qp < end; ++qp) {
                        const int c = colIdx[qp];
                        if (c == j) {
                            lu[qp] = __dsub_rn(lu[qp], __dmul_rn(m, lu[jp]));
                            break;
                        }
                        if (c > j)
                            break;
                    }
                }
            }
            const int di = diagPtr[i];
            rpiv[i] = (di >= 0 && lu[di] != 0.0) ? __drcp_rn(lu[di]) : 0.0;
        }
        __syncthreads();
    }
}

// Asynchronous global -> shared copies (LDGSTS): a thread issues them and goes
// on; cp.async.wait_group retires its own groups in order.
__device__ __forceinline__ void cp_async4(void *smem, const void *gmem)
{
    const unsigned sa = static_cast<unsigned>(__cvta_generic_to_shared(smem));
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(sa), "l"(gmem) : "memory");
}

__device__ __forceinline__ void cp_async8(void *smem, const void *gmem)
{
    const unsigned sa = static_cast<unsigned>(__cvta_generic_to_shared(smem));
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(sa), "l"(gmem) : "memory");
}

__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }

constexpr int kIluStages = 12;        // levels in flight: the copy of level l + 11 overlaps the work of level l
constexpr int kIluSmallMaxLevels = 4096;
constexpr int kIluSmallMaxK = 8;      // entries per row of one triangle
constexpr int kIluSmallSmem = 220 * 1024;

__device__ __forceinline__ void cp_async_wait_pipeline()
{
    asm volatile("cp.async.wait_group %0;" ::"n"(kIluStages - 2) : "memory");
}

// One triangle of the packed level-ordered sweep: rows (row | count << 24),
// their entries' columns and values at a stride of k per row, and (backward)
// the diagonal.
struct PackedSweep {
    const int32_t *row, *col;
    const double *val, *diag, *rdiag;
    int nlev, k;
};

// Shared-memory stage of one level: vals [R k], diag [R], rdiag [R], cols [R k], rows [R].
struct StageView {
    double *val, *diag, *rdiag;
    int32_t *col, *row;
};

__device__ __forceinline__ StageView stage_view(unsigned char *base, int stageBytes, int s, int R, int k)
{
    unsigned char *b = base + static_cast<size_t>(s) * stageBytes;
    StageView v;
    v.val = reinterpret_cast<double *>(b);
    v.diag = v.val + static_cast<size_t>(R) * k;
    v.rdiag = v.diag + R;
    v.col = reinterpret_cast<int32_t *>(v.rdiag + R);
    v.row = v.col + static_cast<size_t>(R) * k;
    return v;
}

__device__ __forceinline__ void issue_level(const PackedSweep &p, const int *lvl, int l, StageView st)
{
    if (l < p.nlev) {
        const int a = lvl[l], cnt = lvl[l + 1] - a, k = p.k;
        for (int q = threadIdx.x; q < cnt; q += blockDim.x) {
            cp_async4(st.row + q, p.row + a + q);
            if (p.diag)
                cp_async8(st.diag + q, p.diag + a + q);
            if (p.rdiag)
                cp_async8(st.rdiag + q, p.rdiag + a + q);
        }
        for (int q = threadIdx.x; q < cnt * k; q += blockDim.x) {
            cp_async4(st.col + q, p.col + static_cast<size_t>(a) * k + q);
            cp_async8(st.val + q, p.val + static_cast<size_t>(a) * k + q);
        }
    }
    cp_async_commit();  // one group per level, empty past the end, so the wait count stays uniform
}

// One triangular sweep in place on ys: forward ys_i -= sum l_ij ys_j, backward
// the same with u_ij and a final division by the diagonal (when non-zero).
// SSOR: forward (ys_i - sum a_ij ys_j) invD_i, backward (a_ii ys_i - sum a_ij
// ys_j) invD_i.
template <bool BACKWARD, bool SSOR>
__device__ __forceinline__ void sweep_levels(const PackedSweep &p, const int *lvl, double *ys, unsigned char *stages,
                                             int stageBytes, int R)
{
    for (int s = 0; s < kIluStages - 1; ++s)
        issue_level(p, lvl, s, stage_view(stages, stageBytes, s, R, p.k));
    for (int l = 0; l < p.nlev; ++l) {
        cp_async_wait_pipeline();  // this thread's copies of level l have landed
        __syncthreads();           // everyone's copies of level l, and level l - 1's results, are visible
        issue_level(p, lvl, l + kIluStages - 1, stage_view(stages, stageBytes, (l + kIluStages - 1) % kIluStages, R, p.k));
        const StageView st = stage_view(stages, stageBytes, l % kIluStages, R, p.k);
        const int cnt = lvl[l + 1] - lvl[l], k = p.k;
        for (int t = threadIdx.x; t < cnt; t += blockDim.x) {
            const int packed = st.row[t];
            const int i = packed & 0xffffff, c = packed >> 24;
            double s = ys[i];
            if (SSOR && BACKWARD)
                s = __dmul_rn(st.diag[t], s);
            for (int q = 0; q < c; ++q)
                s = __dsub_rn(s, __dmul_rn(st.val[t * k + q], ys[st.col[t * k + q]]));
            if (SSOR) {
                s = __dmul_rn(s, st.rdiag[t]);
            } else if (BACKWARD) {
                const double dv = st.diag[t];
                s = dv != 0.0 ? div_rn_by_recip(s, dv, st.rdiag[t]) : s;
            }
            ys[i] = s;
        }
    }
    asm volatile("cp.async.wait_all;" ::: "memory");
    __syncthreads();
}

// z = (LU)^-1 r (or SSOR's M^-1 r) in one CTA: ys = r, forward sweep, backward
// sweep, z = ys.
template <bool SSOR>
__global__ void __launch_bounds__(kIluSmallThreads) k_ilu_sweeps_small(int n, PackedSweep fwd, PackedSweep bwd,
                                                                       const int *__restrict__ lvlF,
                                                                       const int *__restrict__ lvlB, int R,
                                                                       int stageBytes, const double *__restrict__ r,
                                                                       double *__restrict__ z)
{
    extern __shared__ __align__(16) unsigned char smem[];
    int *sl = reinterpret_cast<int *>(smem);                           // level pointers of both sweeps
    int *slF = sl, *slB = sl + fwd.nlev + 1;
    double *ys = reinterpret_cast<double *>(smem + 8 * ((fwd.nlev + bwd.nlev + 3) / 2 + 1));
    unsigned char *stages = reinterpret_cast<unsigned char *>(ys + n) + ((16 - ((8 * n) & 15)) & 15);
    for (int q = threadIdx.x; q <= fwd.nlev; q += blockDim.x)
        slF[q] = lvlF[q];
    for (int q = threadIdx.x; q <= bwd.nlev; q += blockDim.x)
        slB[q] = lvlB[q];
    for (int i = threadIdx.x; i < n; i += blockDim.x)
        ys[i] = r[i];
    __syncthreads();
    sweep_levels<false, SSOR>(fwd, slF, ys, stages, stageBytes, R);
    sweep_levels<true, SSOR>(bwd, slB, ys, stages, stageBytes, R);
    for (int i = threadIdx.x; i < n; i += blockDim.x)
        z[i] = ys[i];
}

// Values of the packed sweeps from the factor: entry e of position t reads
// lu[pos[t k + e]] (pos -1: padding); the backward diagonal is lu[diagPtr[i]]
// (0 when the row has none).  SSOR (frdiag given): lu holds A, rdiag is the
// inverse diagonal invD of the row in each sweep's order.
__global__ void __launch_bounds__(kBlock) k_ilu_pack(int n, int kf, int kb, const int32_t *__restrict__ fpos,
                                                     const int32_t *__restrict__ bpos,
                                                     const int32_t *__restrict__ frow,
                                                     const int32_t *__restrict__ brow,
                                                     const int32_t *__restrict__ diagPtr,
                                                     const double *__restrict__ lu, const double *__restrict__ invD,
                                                     double *__restrict__ fval, double *__restrict__ bval,
                                                     double *__restrict__ bdiag, double *__restrict__ brdiag,
                                                     double *__restrict__ frdiag)
{
    const int stride = gridDim.x * blockDim.x;
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < n * kf; e += stride) {
        const int q = fpos[e];
        fval[e] = q >= 0 ? lu[q] : 0.0;
    }
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < n * kb; e += stride) {
        const int q = bpos[e];
        bval[e] = q >= 0 ? lu[q] : 0.0;
    }
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += stride) {
        const int bi = brow[t] & 0xffffff;
        const int kd = diagPtr[bi];
        const double d = kd >= 0 ? lu[kd] : 0.0;
        bdiag[t] = d;
        if (frdiag) {
            brdiag[t] = invD[bi];
            frdiag[t] = invD[frow[t] & 0xffffff];
        } else {
            brdiag[t] = d != 0.0 ? __drcp_rn(d) : 0.0;
        }
    }
}

// a / b both ways (the division the sweeps take from the reciprocal, and the
// division itself) for the self-check of the reciprocal form.
__global__ void __launch_bounds__(kBlock) k_div_check(int n, const double *__restrict__ a,
                                                     const double *__restrict__ b, double *__restrict__ q1,
                                                     double *__restrict__ q2)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const double bi = b[i];
        q1[i] = div_rn_by_recip(a[i], bi, bi != 0.0 ? __drcp_rn(bi) : 0.0);
        q2[i] = __ddiv_rn(a[i], bi);
    }
}

// One warp waits for a value that nothing publishes (x[0] stays pending): the
// bounded wait of the sweeps running out, observed from the host.
__global__ void k_wait_probe(const double *x, unsigned *out)
{
    const int j[4] = {0, 0, 0, 0};
    const bool dep[4] = {true, false, false, false};
    double v[4];
    const bool ok = wait_values4(x, j, dep, v);
    if (threadIdx.x == 0)
        out[0] = ok ? 0u : 1u;
}

__global__ void k_zero_pivot_check(int n, const int32_t *__restrict__ diagPtr, const double *__restrict__ lu, int *flag)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int d = diagPtr[i];
        if (d < 0 || lu[d] == 0.0)
            atomicOr(flag, 1);
    }
}

// Rows grouped by level; `lower` selects the forward (j < i) or backward
// (j > i) dependency structure.
void levels(int64_t n, const int32_t *rowPtr, const int32_t *colIdx, const std::vector<int32_t> &diagPtr, bool lower,
            std::vector<int32_t> &rowsOut, std::vector<int32_t> &levelPtr, int &maxRows)
{
    std::vector<int32_t> lev(static_cast<size_t>(n), 0);
    int nlev = 0;
    if (lower) {
        for (int64_t i = 0; i < n; ++i) {
            int l = 0;
            for (int k = rowPtr[i]; k < rowPtr[i + 1]; ++k) {
                const int j = colIdx[k];
                if (j >= i)
                    break;
                l = std::max(l, lev[j] + 1);
            }
            lev[i] = l;
            nlev = std::max(nlev, l + 1);
        }
    } else {
        for (int64_t i = n - 1; i >= 0; --i) {
            int l = 0;
            const int kd = diagPtr[i];
            // the backward sweep reads columns after the diagonal (or the
            // whole row when the diagonal is missing, as the reference's
            // kd+1 = 0 start does; such rows are rejected before we get here)
            for (int k = kd + 1; k < rowPtr[i + 1]; ++k) {
                const int j = colIdx[k];
                if (j > i)
                    l = std::max(l, lev[j] + 1);
            }
            lev[i] = l;
            nlev = std::max(nlev, l + 1);
        }
    }
    levelPtr.assign(static_cast<size_t>(nlev) + 1, 0);
    for (int64_t i = 0; i < n; ++i)
        levelPtr[lev[i] + 1]++;
    maxRows = 0;
    for (int l = 0; l < nlev; ++l) {
        maxRows = std::max(maxRows, levelPtr[l + 1]);
        levelPtr[l + 1] += levelPtr[l];
    }
    rowsOut.resize(static_cast<size_t>(n));
    std::vector<int32_t> fill(levelPtr.begin(), levelPtr.end() - 1);
    for (int64_t i = 0; i < n; ++i)
        rowsOut[fill[lev[i]]++] = static_cast<int32_t>(i);
}

int analyse(simall_context *ctx, IluData *d, int64_t n, const int32_t *rowPtr, const int32_t *colIdx)
{
    d->h_diagPtr.assign(static_cast<size_t>(n), -1);
    for (int64_t i = 0; i < n; ++i)
        for (int k = rowPtr[i]; k < rowPtr[i + 1]; ++k)
            if (colIdx[k] == i) {
                d->h_diagPtr[i] = k;
                break;
            }
    std::vector<int32_t> fr, br;
    int m1 = 0, m2 = 0;
    levels(n, rowPtr, colIdx, d->h_diagPtr, true, fr, d->fwdLevelPtr, m1);
    levels(n, rowPtr, colIdx, d->h_diagPtr, false, br, d->bwdLevelPtr, m2);
    d->maxLevelRows = std::max(m1, m2);
    SIMALL_CUDA_TRY(ctx, d->diagPtr.alloc(n));
    SIMALL_CUDA_TRY(ctx, d->fwdRows.alloc(n));
    SIMALL_CUDA_TRY(ctx, d->bwdRows.alloc(n));
    SIMALL_CUDA_TRY(ctx, d->y.alloc(n));
    SIMALL_CUDA_TRY(ctx, d->sweepCtl.alloc(4));
    SIMALL_CUDA_TRY(ctx, cudaMemsetAsync(d->sweepCtl.p, 0, 4 * sizeof(unsigned), ctx->stream));
    SIMALL_CUDA_TRY(ctx, cudaMemcpyAsync(d->diagPtr.p, d->h_diagPtr.data(), n * sizeof(int32_t),
                                         cudaMemcpyHostToDevice, ctx->stream));
    SIMALL_CUDA_TRY(ctx, cudaMemcpyAsync(d->fwdRows.p, fr.data(), n * sizeof(int32_t), cudaMemcpyHostToDevice,
                                         ctx->stream));
    SIMALL_CUDA_TRY(ctx, cudaMemcpyAsync(d->bwdRows.p, br.data(), n * sizeof(int32_t), cudaMemcpyHostToDevice,
                                         ctx->stream));
    SIMALL_CUDA_TRY(ctx, d->fwdLvl.alloc(d->fwdLevelPtr.size()));
    SIMALL_CUDA_TRY(ctx, d->bwdLvl.alloc(d->bwdLevelPtr.size()));
    SIMALL_CUDA_TRY(ctx, cudaMemcpyAsync(d->fwdLvl.p, d->fwdLevelPtr.data(), d->fwdLevelPtr.size() * sizeof(int32_t),
                                         cudaMemcpyHostToDevice, ctx->stream));
    SIMALL_CUDA_TRY(ctx, cudaMemcpyAsync(d->bwdLvl.p, d->bwdLevelPtr.data(), d->bwdLevelPtr.size() * sizeof(int32_t),
                                         cudaMemcpyHostToDevice, ctx->stream));
    // the single-CTA path: rows of each sweep in level order with their entries packed at a fixed stride
    d->small = false;
    const int nlevF = static_cast<int>(d->fwdLevelPtr.size()) - 1, nlevB = static_cast<int>(d->bwdLevelPtr.size()) - 1;
    if (n <= kIluSmallRows && nlevF + nlevB + 2 <= 2 * kIluSmallMaxLevels) {
        int kf = 0, kb = 0;
        for (int64_t i = 0; i < n; ++i) {
            int lo = 0;
            for (int k = rowPtr[i]; k < rowPtr[i + 1] && colIdx[k] < i; ++k)
                ++lo;
            kf = std::max(kf, lo);
            const int kd = d->h_diagPtr[i];
            kb = std::max(kb, rowPtr[i + 1] - (kd + 1));
        }
        kf = std::max(kf, 1);
        kb = std::max(kb, 1);
        const int R = std::max(d->maxLevelRows, 1);
        const int K = std::max(kf, kb);
        const int stageBytes = (R * K * 8 + 2 * R * 8 + R * K * 4 + R * 4 + 15) & ~15;
        const int64_t smemBytes = 8 * ((nlevF + nlevB + 3) / 2 + 1) + ((8 * n + 15) & ~int64_t(15)) +
                                  static_cast<int64_t>(kIluStages) * stageBytes;
        if (K <= kIluSmallMaxK && smemBytes <= kIluSmallSmem) {
            std::vector<int32_t> frow(n), brow(n), fcol(n * kf, 0), fpos(n * kf, -1), bcol(n * kb, 0),
                bpos(n * kb, -1);
            for (int64_t t = 0; t < n; ++t) {
                const int i = fr[t];
                int c = 0;
                for (int k = rowPtr[i]; k < rowPtr[i + 1] && colIdx[k] < i; ++k, ++c) {
                    fcol[t * kf + c] = colIdx[k];
                    fpos[t * kf + c] = k;
                }
                frow[t] = i | (c << 24);
                const int j = br[t];
                const int kd = d->h_diagPtr[j];
                c = 0;
                for (int k = kd + 1; k < rowPtr[j + 1]; ++k, ++c) {
                    bcol[t * kb + c] = colIdx[k];
                    bpos[t * kb + c] = k;
                }
                brow[t] = j | (c << 24);
            }
            auto up = [&](DevBuf<int32_t> &dst, const std::vector<int32_t> &src) -> cudaError_t {
                cudaError_t e = dst.alloc(src.size());
                if (e == cudaSuccess)
                    e = cudaMemcpyAsync(dst.p, src.data(), src.size() * sizeof(int32_t), cudaMemcpyHostToDevice,
                                        ctx->stream);
                return e;
            };
            SIMALL_CUDA_TRY(ctx, up(d->frow, frow));
            SIMALL_CUDA_TRY(ctx, up(d->brow, brow));
            SIMALL_CUDA_TRY(ctx, up(d->fcol, fcol));
            SIMALL_CUDA_TRY(ctx, up(d->fpos, fpos));
            SIMALL_CUDA_TRY(ctx, up(d->bcol, bcol));
            SIMALL_CUDA_TRY(ctx, up(d->bpos, bpos));
            SIMALL_CUDA_TRY(ctx, d->fval.alloc(n * kf));
            SIMALL_CUDA_TRY(ctx, d->bval.alloc(n * kb));
            SIMALL_CUDA_TRY(ctx, d->bdiag.alloc(n));
            SIMALL_CUDA_TRY(ctx, d->brdiag.alloc(n));
            SIMALL_CUDA_TRY(ctx, d->rpiv.alloc(n));
            SIMALL_CUDA_TRY(ctx, d->frdiag.alloc(d->mode == 1 ? n : 1));
            SIMALL_CUDA_TRY(ctx, cudaFuncSetAttribute(k_ilu_sweeps_small<false>,
                                                      cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                      static_cast<int>(smemBytes)));
            SIMALL_CUDA_TRY(ctx, cudaFuncSetAttribute(k_ilu_sweeps_small<true>,
                                                      cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                      static_cast<int>(smemBytes)));
            // the copies above read host vectors that die at return
            SIMALL_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
            d->kf = kf;
            d->kb = kb;
            d->stageRows = R;
            d->stageBytes = stageBytes;
            d->smallSmem = static_cast<int>(smemBytes);
            // one thread per row of the widest level: every warp pays each level's barrier and loop
            // control, so warps beyond the widest level only add work to the chain
            d->smallThreads = std::min(kIluSmallThreads, std::max(64, (R + 31) & ~31));
            d->small = true;
        }
    }
    // the copies above read host vectors that die at return
    SIMALL_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
    d->analysed = true;
    return SIMALL_OK;
}

// The packed single-CTA sweep values from lu (the factor, or A for SSOR).
int pack(simall_context *ctx, IluData *d)
{
    const int n = static_cast<int>(d->h_diagPtr.size());
    const int items = n * std::max(d->kf, d->kb);
    const bool ssor = d->mode == 1;
    k_ilu_pack<<<std::min((items + kBlock - 1) / kBlock, ctx->num_sms * 8), kBlock, 0, ctx->stream>>>(
        n, d->kf, d->kb, d->fpos.p, d->bpos.p, d->frow.p, d->brow.p, d->diagPtr.p, d->lu.p, ssor ? d->invD : nullptr,
        d->fval.p, d->bval.p, d->bdiag.p, d->brdiag.p, ssor ? d->frdiag.p : nullptr);
    SIMALL_LAUNCH_CHECK(ctx);
    return SIMALL_OK;
}

// rdiag_i = RN(1/u_ii), 0 where the diagonal is missing or zero (the sweep
// then keeps s, as the reference does).
__global__ void __launch_bounds__(kBlock) k_ilu_rdiag(int n, const int32_t *__restrict__ diagPtr,
                                                      const double *__restrict__ lu, double *__restrict__ rdiag)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int d = diagPtr[i];
        rdiag[i] = (d >= 0 && lu[d] != 0.0) ? __drcp_rn(lu[d]) : 0.0;
    }
}

int factor(simall_context *ctx, IluData *d, const int32_t *rowPtr, const int32_t *colIdx)
{
    const int nlev = static_cast<int>(d->fwdLevelPtr.size()) - 1;
    if (d->small) {
        k_ilu_factor_small<<<1, d->smallThreads, 0, ctx->stream>>>(nlev, d->fwdLvl.p, d->fwdRows.p, rowPtr, colIdx,
                                                                  d->diagPtr.p, d->lu.p, d->rpiv.p);
        SIMALL_LAUNCH_CHECK(ctx);
        return pack(ctx, d);
    }
    for (int l = 1; l < nlev; ++l) {  // level 0 rows have no lower entries
        const int a = d->fwdLevelPtr[l], cnt = d->fwdLevelPtr[l + 1] - a;
        k_ilu_factor_level<<<(cnt + kBlock - 1) / kBlock, kBlock, 0, ctx->stream>>>(d->fwdRows.p + a, cnt, rowPtr,
                                                                                    colIdx, d->diagPtr.p, d->lu.p);
        SIMALL_LAUNCH_CHECK(ctx);
    }
    const int n = static_cast<int>(d->h_diagPtr.size());
    SIMALL_CUDA_TRY(ctx, d->rdiag.alloc(n));
    k_ilu_rdiag<<<std::min((n + kBlock - 1) / kBlock, ctx->num_sms * 8), kBlock, 0, ctx->stream>>>(n, d->diagPtr.p,
                                                                                                d->lu.p, d->rdiag.p);
    SIMALL_LAUNCH_CHECK(ctx);
    return SIMALL_OK;
}

int sweeps(simall_context *ctx, IluData *d, const int32_t *rowPtr, const int32_t *colIdx, const double *lu,
           const double *r, double *z)
{
    const int n = static_cast<int>(d->h_diagPtr.size());
    const bool ssor = d->mode == 1;
    if (d->small && lu == d->lu.p) {
        PackedSweep f{d->frow.p, d->fcol.p, d->fval.p, nullptr, ssor ? d->frdiag.p : nullptr,
                      static_cast<int>(d->fwdLevelPtr.size()) - 1, d->kf};
        PackedSweep b{d->brow.p, d->bcol.p, d->bval.p, d->bdiag.p, d->brdiag.p,
                      static_cast<int>(d->bwdLevelPtr.size()) - 1, d->kb};
        auto kern = ssor ? k_ilu_sweeps_small<true> : k_ilu_sweeps_small<false>;
        kern<<<1, d->smallThreads, d->smallSmem, ctx->stream>>>(n, f, b, d->fwdLvl.p, d->bwdLvl.p, d->stageRows,
                                                                d->stageBytes, r, z);
        SIMALL_LAUNCH_CHECK(ctx);
        return SIMALL_OK;
    }
    // warps beyond a few levels' rows only add polls: g_sweep_ctas_per_sm (2: 16 warps per SM)
    const int grid = ctx->num_sms * g_sweep_ctas_per_sm;
    const unsigned backoff = g_sweep_backoff_ns;
    const double *rdiag = (g_sweep_reciprocal && !ssor && lu == d->lu.p && d->rdiag.p) ? d->rdiag.p : nullptr;
    const int fill = std::min((n + kBlock - 1) / kBlock, ctx->num_sms * 8);
    k_sweep_begin_values<<<fill < 1 ? 1 : fill, kBlock, 0, ctx->stream>>>(d->sweepCtl.p, d->y.p, n);
    SIMALL_LAUNCH_CHECK(ctx);
    auto fwd = ssor ? k_ilu_fwd_free<true> : k_ilu_fwd_free<false>;
    fwd<<<grid, kBlock, 0, ctx->stream>>>(n, d->fwdRows.p, rowPtr, colIdx, lu, r, d->invD, d->y.p, d->sweepCtl.p,
                                          backoff);
    SIMALL_LAUNCH_CHECK(ctx);
    k_sweep_begin_values<<<fill < 1 ? 1 : fill, kBlock, 0, ctx->stream>>>(d->sweepCtl.p, z, n);
    SIMALL_LAUNCH_CHECK(ctx);
    auto bwd = ssor ? k_ilu_bwd_free<true> : k_ilu_bwd_free<false>;
    bwd<<<grid, kBlock, 0, ctx->stream>>>(n, d->bwdRows.p, rowPtr, colIdx, d->diagPtr.p, lu, d->y.p, d->invD, rdiag,
                                          z, d->sweepCtl.p, backoff);
    SIMALL_LAUNCH_CHECK(ctx);
    return SIMALL_OK;
}

}  // namespace

int ilu_setup(simall_solver *s)
{
    if (s->cfg.preconditioner == SIMALL_PRECOND_AMG)
        return amg_setup(s);
    simall_context *ctx = s->ctx;
    if (!s->ilu) {
        s->ilu = new (std::nothrow) IluData;
        if (!s->ilu)
            return SIMALL_ERR_OUT_OF_MEMORY;
    }
    IluData *d = s->ilu;
    d->mode = s->cfg.preconditioner == SIMALL_PRECOND_SSOR ? 1 : 0;
    d->invD = s->invDiag.p;  // SSOR: set up by the caller for the current values
    if (!d->analysed) {
        int hp = solver_host_pattern(s);
        if (hp)
            return hp;
        int st = analyse(ctx, d, s->n, s->h_rowPtr.data(), s->h_colIdx.data());
        if (st)
            return st;
    }
    SIMALL_CUDA_TRY(ctx, d->lu.alloc(s->nnz));
    SIMALL_CUDA_TRY(ctx, cudaMemcpyAsync(d->lu.p, s->values, s->nnz * sizeof(double), cudaMemcpyDeviceToDevice,
                                         ctx->stream));
    if (d->mode == 1)  // SSOR sweeps A itself
        return d->small ? pack(ctx, d) : SIMALL_OK;
    return factor(ctx, d, s->rowPtr, s->colIdx);
}

int ilu_apply(simall_solver *s, const double *r, double *z)
{
    if (s->amg)
        return amg_apply(s, r, z);
    return sweeps(s->ctx, s->ilu, s->rowPtr, s->colIdx, s->ilu->lu.p, r, z);
}

// Whether a sweep gave up waiting for a row (a device-side timeout); clears
// the flag.
int ilu_check(simall_context *ctx, IluData *d)
{
    unsigned h = 0;
    SIMALL_CUDA_TRY(ctx, cudaMemcpyAsync(&h, d->sweepCtl.p + 2, sizeof(unsigned), cudaMemcpyDeviceToHost, ctx->stream));
    SIMALL_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
    if (h) {
        SIMALL_CUDA_TRY(ctx, cudaMemsetAsync(d->sweepCtl.p + 2, 0, sizeof(unsigned), ctx->stream));
        return fail(ctx, SIMALL_ERR_CUDA, "ILU(0) sweep: a row wait timed out");
    }
    return SIMALL_OK;
}

int ilu_check(simall_solver *s)
{
    if (s->amg)
        return amg_check(s);
    return s->ilu ? ilu_check(s->ctx, s->ilu) : SIMALL_OK;
}

int ilu_apply_launches(const simall_solver *s)
{
    if (s->amg)
        return amg_apply_launches(s);
    return (s->ilu && s->ilu->small) ? 1 : 4;
}

void ilu_free(simall_solver *s)
{
    amg_free(s);
    delete s->ilu;
    s->ilu = nullptr;
}

}  // namespace simall

using namespace simall;

// ---------------------------------------------------------------- reference facade (GpuKernels.hpp:89-108)
namespace {
struct FacadeIlu {
    simall_context ctx;
    IluData d;
};

int facade_ctx(simall_context &ctx, void *stream)
{
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess)
        return SIMALL_ERR_NO_DEVICE;
    ctx.device = dev;
    if (cudaDeviceGetAttribute(&ctx.num_sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
        return SIMALL_ERR_CUDA;
    ctx.stream = static_cast<cudaStream_t>(stream);
    return SIMALL_OK;
}

int facade_pattern(simall_context &ctx, size_t n, const int32_t *rowPtr, const int32_t *colIdx,
                   std::vector<int32_t> &hr, std::vector<int32_t> &hc)
{
    hr.resize(n + 1);
    SIMALL_CUDA_TRY(&ctx, cudaMemcpyAsync(hr.data(), rowPtr, (n + 1) * sizeof(int32_t), cudaMemcpyDeviceToHost,
                                          ctx.stream));
    SIMALL_CUDA_TRY(&ctx, cudaStreamSynchronize(ctx.stream));
    hc.resize(static_cast<size_t>(hr[n]));
    SIMALL_CUDA_TRY(&ctx, cudaMemcpyAsync(hc.data(), colIdx, hc.size() * sizeof(int32_t), cudaMemcpyDeviceToHost,
                                          ctx.stream));
    SIMALL_CUDA_TRY(&ctx, cudaStreamSynchronize(ctx.stream));
    return check_csr_host(&ctx, static_cast<int64_t>(n), hr[n], hr.data(), hc.data(), nullptr, false);
}
}  // namespace

extern "C" {

int simall_gpu_ilu0_factor_inplace(size_t n, const int32_t *rowPtr, const int32_t *colIdx, double *values,
                                   void *stream, int *ok)
{
    if (!rowPtr || !colIdx || !values || !ok)
        return SIMALL_ERR_INVALID_ARGUMENT;
    *ok = 0;
    if (n == 0) {
        *ok = 1;
        return SIMALL_OK;
    }
    auto *f = new (std::nothrow) FacadeIlu;
    if (!f)
        return SIMALL_ERR_OUT_OF_MEMORY;
    std::vector<int32_t> hr, hc;
    int st = facade_ctx(f->ctx, stream);
    if (!st)
        st = facade_pattern(f->ctx, n, rowPtr, colIdx, hr, hc);
    if (!st)
        st = analyse(&f->ctx, &f->d, static_cast<int64_t>(n), hr.data(), hc.data());
    if (!st) {
        // factor in place: point lu at the caller's values
        double *saved = f->d.lu.p;
        f->d.lu.p = values;
        st = factor(&f->ctx, &f->d, rowPtr, colIdx);
        f->d.lu.p = saved;
    }
    if (!st) {
        st = f->d.y.alloc(1) == cudaSuccess ? SIMALL_OK : SIMALL_ERR_OUT_OF_MEMORY;
        int *flag = reinterpret_cast<int *>(f->d.y.p);
        if (!st && cudaMemsetAsync(flag, 0, sizeof(int), f->ctx.stream) != cudaSuccess)
            st = SIMALL_ERR_CUDA;
        if (!st) {
            k_zero_pivot_check<<<64, kBlock, 0, f->ctx.stream>>>(static_cast<int>(n), f->d.diagPtr.p, values, flag);
            int h = 1;
            if (cudaMemcpyAsync(&h, flag, sizeof(int), cudaMemcpyDeviceToHost, f->ctx.stream) != cudaSuccess ||
                cudaStreamSynchronize(f->ctx.stream) != cudaSuccess)
                st = SIMALL_ERR_CUDA;
            else
                *ok = h ? 0 : 1;
        }
    }
    delete f;
    return st;
}

int simall_diagnose_sweep_params(int ctas_per_sm, int backoff_ns, int divide_via_reciprocal)
{
    if (ctas_per_sm < 1 || ctas_per_sm > 8 || backoff_ns < 0 || backoff_ns > 4096)
        return SIMALL_ERR_INVALID_ARGUMENT;
    g_sweep_ctas_per_sm = ctas_per_sm;
    g_sweep_backoff_ns = static_cast<unsigned>(backoff_ns);
    g_sweep_reciprocal = divide_via_reciprocal != 0;
    return SIMALL_OK;
}

int simall_diagnose_mixed_params(int prefetch_stages, int grid_ctas_per_sm)
{
    if (prefetch_stages < 0 || prefetch_stages > 64 || grid_ctas_per_sm < 0 || grid_ctas_per_sm > 8)
        return SIMALL_ERR_INVALID_ARGUMENT;
    g_sell_prefetch = prefetch_stages;
    g_grid_ctas_per_sm = grid_ctas_per_sm;
    return SIMALL_OK;
}

int simall_diagnose_bounded_wait(simall_context *ctx, int *timed_out, double *seconds)
{
    if (!ctx || !timed_out)
        return SIMALL_ERR_INVALID_ARGUMENT;
    SIMALL_CUDA_TRY(ctx, cudaSetDevice(ctx->device));
    DevBuf<unsigned> buf;  // [0] ticket of the fill, [2] unused, [4] the probe's result
    DevBuf<double> val;
    SIMALL_CUDA_TRY(ctx, buf.alloc(5));
    SIMALL_CUDA_TRY(ctx, val.alloc(1));
    SIMALL_CUDA_TRY(ctx, cudaMemsetAsync(buf.p, 0, 5 * sizeof(unsigned), ctx->stream));
    k_sweep_begin_values<<<1, 32, 0, ctx->stream>>>(buf.p, val.p, 1);  // val[0] = pending
    SIMALL_LAUNCH_CHECK(ctx);
    const auto t0 = std::chrono::steady_clock::now();
    k_wait_probe<<<1, 32, 0, ctx->stream>>>(val.p, buf.p + 4);
    SIMALL_LAUNCH_CHECK(ctx);
    unsigned h = 0;
    SIMALL_CUDA_TRY(ctx, cudaMemcpyAsync(&h, buf.p + 4, sizeof(unsigned), cudaMemcpyDeviceToHost, ctx->stream));
    SIMALL_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
    *timed_out = static_cast<int>(h);
    if (seconds)
        *seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    return SIMALL_OK;
}

int simall_diagnose_division(simall_context *ctx, int64_t n, const double *a, const double *b, double *q_recip,
                             double *q_div)
{
    if (!ctx || n < 0 || (n > 0 && (!a || !b || !q_recip || !q_div)) || n > INT32_MAX)
        return SIMALL_ERR_INVALID_ARGUMENT;
    if (n == 0)
        return SIMALL_OK;
    SIMALL_CUDA_TRY(ctx, cudaSetDevice(ctx->device));
    DevBuf<double> buf;
    SIMALL_CUDA_TRY(ctx, buf.alloc(4 * n));
    cudaStream_t st = ctx->stream;
    SIMALL_CUDA_TRY(ctx, cudaMemcpyAsync(buf.p, a, n * sizeof(double), cudaMemcpyHostToDevice, st));
    SIMALL_CUDA_TRY(ctx, cudaMemcpyAsync(buf.p + n, b, n * sizeof(double), cudaMemcpyHostToDevice, st));
    const int grid = static_cast<int>(std::min<int64_t>((n + kBlock - 1) / kBlock, ctx->num_sms * 8));
    k_div_check<<<grid, kBlock, 0, st>>>(static_cast<int>(n), buf.p, buf.p + n, buf.p + 2 * n, buf.p + 3 * n);
    SIMALL_LAUNCH_CHECK(ctx);
    SIMALL_CUDA_TRY(ctx, cudaMemcpyAsync(q_recip, buf.p + 2 * n, n * sizeof(double), cudaMemcpyDeviceToHost, st));
    SIMALL_CUDA_TRY(ctx, cudaMemcpyAsync(q_div, buf.p + 3 * n, n * sizeof(double), cudaMemcpyDeviceToHost, st));
    SIMALL_CUDA_TRY(ctx, cudaStreamSynchronize(st));
    return SIMALL_OK;
}

int simall_gpu_ilu0_apply(size_t n, const int32_t *rowPtr, const int32_t *colIdx, const double *values,
                          const double *r, double *z, void *stream)
{
    if (!rowPtr || !colIdx || !values || !r || !z)
        return SIMALL_ERR_INVALID_ARGUMENT;
    if (n == 0)
        return SIMALL_OK;
    auto *f = new (std::nothrow) FacadeIlu;
    if (!f)
        return SIMALL_ERR_OUT_OF_MEMORY;
    std::vector<int32_t> hr, hc;
    int st = facade_ctx(f->ctx, stream);
    if (!st)
        st = facade_pattern(f->ctx, n, rowPtr, colIdx, hr, hc);
    if (!st)
        st = analyse(&f->ctx, &f->d, static_cast<int64_t>(n), hr.data(), hc.data());
    if (!st)
        st = sweeps(&f->ctx, &f->d, rowPtr, colIdx, values, r, z);
    if (!st && cudaStreamSynchronize(f->ctx.stream) != cudaSuccess)
        st = SIMALL_ERR_CUDA;
    if (!st)
        st = ilu_check(&f->ctx, &f->d);
    delete f;
    return st;
}

}  // extern "C"
