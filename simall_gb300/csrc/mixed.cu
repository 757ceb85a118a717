// Mixed-precision Jacobi-PCG: FP32 inner iteration, FP64 true residual,
// global reductions and solution.
//
// Jacobi PCG on A is plain CG on the scaled matrix S A S (S = D^-1/2, unit
// diagonal) in the variables y = S^-1 x.  The inner iteration runs that CG in
// FP32 on an FP32 copy of S A S; its correction accumulates in an FP32 vector
// that is folded into the FP64 solution x at "reliable updates" (residual
// replacement, van der Vorst & Ye 2000; Strzodka & Goddeke 2006): whenever the
// iterated residual has dropped by reliable_delta since the last update, or
// its estimate says the stop test may hold, x += S xh in FP64, the true
// residual r = b - A x is recomputed in FP64 with the original CSR, the stop
// test ||r|| / max(||b||,1e-30) < tol is applied to it, and the FP32 residual
// is replaced by S r.  The search direction is kept, so the Krylov process is
// not restarted.  Per-thread partial sums are FP32; every cross-thread and
// cross-CTA reduction is FP64.
//
// Storage of S A S: when A is numerically symmetric and its off-diagonal
// entries lie on at most kMaxDiags distinct diagonals (every structured grid
// in natural order), only the upper diagonals are stored, FP32, one array per
// offset: 4 B per stored diagonal per row and no column indices.  Otherwise
// the off-diagonal entries are kept as FP32 CSR.
#include "device.cuh"
#include "solver.hpp"

#include <algorithm>
#include <climits>
#include <cmath>
#include <new>

namespace simall {

constexpr int kMaxDiags = 8;

struct DiaOffsets {
    int32_t off[kMaxDiags];
    int nd;
};

struct MixedData {
    bool dia = false;
    DiaOffsets offs{};
    DevBuf<float> U;          // [nd][ldU] upper diagonals of S A S (dia)
    int64_t ldU = 0;          // diagonal stride, n rounded up to 4 (16-byte aligned rows)
    DevBuf<int32_t> orow;     // off-diagonal CSR rowPtr (csr)
    DevBuf<int32_t> ocol;
    DevBuf<float> oval;
    DevBuf<double> scale;     // s_i = 1/sqrt(a_ii)
    DevBuf<float> xh, rh, ph, ph2, qh;  // ph / ph2: the direction, double-buffered
    int nnzOff = 0;
    bool patternReady = false;
    std::vector<int32_t> h_orow, h_ocol, h_opos;  // csr: host pattern and the source position of each entry
    DevBuf<int32_t> opos;
};

namespace {

__device__ __forceinline__ int ld_flag(const int *p) { return __ldcg(p); }

// s_i = 1/sqrt(a_ii); flag if a_ii <= 0.
__global__ void __launch_bounds__(kBlock) k_mx_scale(int64_t n, const int32_t *__restrict__ rowPtr,
                                                     const int32_t *__restrict__ colIdx, const double *__restrict__ val,
                                                     double *__restrict__ sc, int *flag)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        double d = 0.0;
        for (int k = rowPtr[i]; k < rowPtr[i + 1]; ++k)
            if (colIdx[k] == i) {
                d = val[k];
                break;
            }
        if (!(d > 0.0)) {
            atomicOr(flag, 1);
            d = 1.0;
        }
        sc[i] = 1.0 / sqrt(d);
    }
}

// Numerical symmetry: a_ji must exist and equal a_ij bit for bit.
__global__ void __launch_bounds__(kBlock) k_mx_symcheck(int64_t n, const int32_t *__restrict__ rowPtr,
                                                        const int32_t *__restrict__ colIdx,
                                                        const double *__restrict__ val, int *flag)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        for (int k = rowPtr[i]; k < rowPtr[i + 1]; ++k) {
            const int j = colIdx[k];
            if (j <= i)
                continue;
            int lo = rowPtr[j], hi = rowPtr[j + 1] - 1, pos = -1;
            while (lo <= hi) {
                const int mid = (lo + hi) >> 1;
                const int c = colIdx[mid];
                if (c == i) {
                    pos = mid;
                    break;
                }
                if (c < i)
                    lo = mid + 1;
                else
                    hi = mid - 1;
            }
            if (pos < 0 || val[pos] != val[k])
                atomicOr(flag, 2);
        }
    }
}

__global__ void __launch_bounds__(kBlock) k_mx_build_dia(int64_t n, int64_t ldU, const int32_t *__restrict__ rowPtr,
                                                         const int32_t *__restrict__ colIdx,
                                                         const double *__restrict__ val, const double *__restrict__ sc,
                                                         DiaOffsets o, float *__restrict__ U)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        float u[kMaxDiags];
#pragma unroll
        for (int d = 0; d < kMaxDiags; ++d)
            u[d] = 0.0f;
        const double si = sc[i];
        for (int k = rowPtr[i]; k < rowPtr[i + 1]; ++k) {
            const int j = colIdx[k];
            if (j <= i)
                continue;
            const int off = j - static_cast<int>(i);
#pragma unroll
            for (int d = 0; d < kMaxDiags; ++d)
                if (d < o.nd && o.off[d] == off)
                    u[d] = static_cast<float>(val[k] * si * sc[j]);
        }
        for (int d = 0; d < o.nd; ++d)
            U[d * ldU + i] = u[d];
    }
}

__global__ void __launch_bounds__(kBlock) k_mx_build_csr(int nOff, const int32_t *__restrict__ orowOfEntry,
                                                         const int32_t *__restrict__ ocol,
                                                         const int32_t *__restrict__ opos,
                                                         const double *__restrict__ val, const double *__restrict__ sc,
                                                         float *__restrict__ oval)
{
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < nOff; e += gridDim.x * blockDim.x)
        oval[e] = static_cast<float>(val[opos[e]] * sc[orowOfEntry[e]] * sc[ocol[e]]);
}

// ---------------------------------------------------------------- iteration kernels
// Init: x = 0, rh = S b, ph = 0, beta = 0, xh = 0; rho = rh.rh, ||b||.
__global__ void __launch_bounds__(kBlock) k_mx_init(int64_t n, const double *__restrict__ b,
                                                    const double *__restrict__ sc, double *__restrict__ x,
                                                    float *__restrict__ rh, float *__restrict__ ph,
                                                    float *__restrict__ xh, double *partials, SolveScalars *s)
{
    float a0 = 0.0f;
    double a1 = 0.0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const double bi = b[i];
        const float r = static_cast<float>(bi * sc[i]);
        x[i] = 0.0;
        rh[i] = r;
        ph[i] = 0.0f;  // the first SpMV forms p = r + 0 * p
        xh[i] = 0.0f;
        a0 += r * r;
        a1 += bi * bi;
    }
    double acc[2] = {static_cast<double>(a0), a1};
    if (grid_sum_last<2>(acc, partials, &s->counter[0]) && threadIdx.x == 0) {
        const double bn = sqrt(acc[1]);
        s->bnorm = std_max(bn, 1e-30);
        s->rz = acc[0];
        s->sigma0 = sqrt(acc[0]);
        s->rmax = s->sigma0;
        s->t0 = bn / s->bnorm;
        s->last = s->t0;
        s->rr = acc[1];
        s->beta = 0.0;
        s->iter = 0;
        s->updates = 0;
        s->need_update = 0;
        s->status = SIMALL_OK;
        s->done = 0;
        s->result = 0;
        if (s->t0 < s->tol) {
            s->done = 1;  // b == 0: x = 0 is exact
        } else if (s->max_iter <= 0) {
            s->done = 1;
            s->result = s->max_iter;
        }
    }
}

// alpha from pq (shared by both storage formats).  Thread 0 of the last CTA.
__device__ __forceinline__ void mx_alpha(SolveScalars *s, double pq)
{
    s->pAp = pq;
    if (!(pq > 0.0)) {
        // not SPD in FP32 (or exact breakdown): fold in what we have and stop
        s->status = SIMALL_ERR_BREAKDOWN;
        s->need_update = 1;
        s->alpha = 0.0;
    } else {
        s->alpha = s->rz / pq;
    }
}

// Four consecutive floats starting at p; p is 16-byte aligned when `aligned`.
__device__ __forceinline__ float4 ld4(const float *__restrict__ p, bool aligned)
{
    if (aligned)
        return __ldg(reinterpret_cast<const float4 *>(p));
    return make_float4(__ldg(p), __ldg(p + 1), __ldg(p + 2), __ldg(p + 3));
}

__device__ __forceinline__ void fma4(float (&y)[4], float4 a, float4 b)
{
    y[0] += a.x * b.x;
    y[1] += a.y * b.y;
    y[2] += a.z * b.z;
    y[3] += a.w * b.w;
}

// The direction p = r + beta p_old of the next iteration, formed wherever it
// is needed with one fused multiply-add, so every thread that forms a given
// p_i gets the same bits.
__device__ __forceinline__ float dir(float r, float po, float beta) { return __fmaf_rn(beta, po, r); }
__device__ __forceinline__ float4 dir4(float4 r, float4 po, float beta)
{
    return make_float4(dir(r.x, po.x, beta), dir(r.y, po.y, beta), dir(r.z, po.z, beta), dir(r.w, po.w, beta));
}

// K1 (dia): p = r + beta p_old (written to p_new), q = (S A S) p, p.q.  ND
// upper diagonals at ascending offsets; row i reads U_d[i] p_{i+off} and, by
// symmetry, U_d[i-off] p_{i-off}, each p formed from r and p_old on the fly.
// One thread per 4 consecutive rows, a warp per 128 consecutive rows, 128-bit
// loads of every 16-byte aligned stream.  Warps that touch the first or last
// maxoff rows take the bounds-checked path.
//
// GRID (offset 1 is the first diagonal and every other offset is a multiple
// of 4, as on any natural-order structured grid with a row length divisible
// by 4): every load of a warp's 128 rows is issued before the first
// multiply, so one memory round trip covers all diagonals; p_{i-1}, p_{i+4}
// and U_0[i-1] come from the neighbouring lanes' registers, the warp's two
// edge lanes load them.  Otherwise each diagonal loads as it goes.
template <int ND, bool GRID>
__global__ void __launch_bounds__(kBlock) k_mx_spmv_dia(int n, int64_t ldU, DiaOffsets o, const float *__restrict__ U,
                                                        const float *__restrict__ rh, const float *__restrict__ pold,
                                                        float *__restrict__ pnew, float *__restrict__ qh,
                                                        double *partials, SolveScalars *s)
{
    if (ld_flag(&s->done))
        return;
    const float beta = static_cast<float>(__ldcg(&s->beta));
    float acc = 0.0f;
    const int nq = (n + 3) >> 2;
    const int maxoff = o.off[ND - 1];
    const int lane = threadIdx.x & 31;
    const int stride = gridDim.x * blockDim.x;
    for (int q0 = blockIdx.x * blockDim.x + threadIdx.x - lane; q0 < nq; q0 += stride) {
        const int q = q0 + lane;
        const int i = q << 2;
        const bool fast = q < nq && i >= maxoff && i + 3 + maxoff < n;
        if (GRID && __all_sync(0xffffffffu, fast)) {
            // loads: own rows, every diagonal, the far neighbours, the edge lanes' scalars
            const float4 r4 = __ldg(reinterpret_cast<const float4 *>(rh + i));
            const float4 o4 = __ldg(reinterpret_cast<const float4 *>(pold + i));
            float4 u[ND];
#pragma unroll
            for (int d = 0; d < ND; ++d)
                u[d] = __ldg(reinterpret_cast<const float4 *>(U + d * ldU + i));
            float4 rp[ND > 1 ? ND - 1 : 1], op[ND > 1 ? ND - 1 : 1], rm[ND > 1 ? ND - 1 : 1],
                om[ND > 1 ? ND - 1 : 1], um[ND > 1 ? ND - 1 : 1];
#pragma unroll
            for (int d = 1; d < ND; ++d) {
                const int off = o.off[d];
                rp[d - 1] = __ldg(reinterpret_cast<const float4 *>(rh + i + off));
                op[d - 1] = __ldg(reinterpret_cast<const float4 *>(pold + i + off));
                rm[d - 1] = __ldg(reinterpret_cast<const float4 *>(rh + i - off));
                om[d - 1] = __ldg(reinterpret_cast<const float4 *>(pold + i - off));
                um[d - 1] = __ldg(reinterpret_cast<const float4 *>(U + d * ldU + i - off));
            }
            // lane 0 needs row i-1, lane 31 row i+4 (both inside [0, n) on this path)
            const int ie = lane == 0 ? i - 1 : i + 4;
            const float re = __ldg(rh + ie), oe = __ldg(pold + ie), ue = __ldg(U + (i - 1));
            // compute
            const float4 p4 = dir4(r4, o4, beta);
            *reinterpret_cast<float4 *>(pnew + i) = p4;
            float y[4] = {p4.x, p4.y, p4.z, p4.w};
            {
                const float pe = dir(re, oe, beta);
                float pn = __shfl_down_sync(0xffffffffu, p4.x, 1);  // p[i+4]
                float pp = __shfl_up_sync(0xffffffffu, p4.w, 1);    // p[i-1]
                float up = __shfl_up_sync(0xffffffffu, u[0].w, 1);  // U_0[i-1]
                if (lane == 31)
                    pn = pe;
                if (lane == 0) {
                    pp = pe;
                    up = ue;
                }
                y[0] += u[0].x * p4.y + up * pp;
                y[1] += u[0].y * p4.z + u[0].x * p4.x;
                y[2] += u[0].z * p4.w + u[0].y * p4.y;
                y[3] += u[0].w * pn + u[0].z * p4.z;
            }
#pragma unroll
            for (int d = 1; d < ND; ++d) {
                fma4(y, u[d], dir4(rp[d - 1], op[d - 1], beta));
                fma4(y, um[d - 1], dir4(rm[d - 1], om[d - 1], beta));
            }
            *reinterpret_cast<float4 *>(qh + i) = make_float4(y[0], y[1], y[2], y[3]);
            acc += p4.x * y[0] + p4.y * y[1] + p4.z * y[2] + p4.w * y[3];
        } else if (!GRID && __all_sync(0xffffffffu, fast)) {
            const float4 p4 = dir4(__ldg(reinterpret_cast<const float4 *>(rh + i)),
                                   __ldg(reinterpret_cast<const float4 *>(pold + i)), beta);
            *reinterpret_cast<float4 *>(pnew + i) = p4;
            float y[4] = {p4.x, p4.y, p4.z, p4.w};
#pragma unroll
            for (int d = 0; d < ND; ++d) {
                const int off = o.off[d];
                const float *Ud = U + d * ldU;
                const bool al = (off & 3) == 0;
                fma4(y, __ldg(reinterpret_cast<const float4 *>(Ud + i)),
                     dir4(ld4(rh + i + off, al), ld4(pold + i + off, al), beta));
                fma4(y, ld4(Ud + i - off, al), dir4(ld4(rh + i - off, al), ld4(pold + i - off, al), beta));
            }
            *reinterpret_cast<float4 *>(qh + i) = make_float4(y[0], y[1], y[2], y[3]);
            acc += p4.x * y[0] + p4.y * y[1] + p4.z * y[2] + p4.w * y[3];
        } else if (q < nq) {
            for (int r = 0; r < 4; ++r) {
                const int row = i + r;
                if (row >= n)
                    break;
                const float pr = dir(__ldg(rh + row), __ldg(pold + row), beta);
                pnew[row] = pr;
                float v = pr;
#pragma unroll
                for (int d = 0; d < ND; ++d) {
                    const int off = o.off[d];
                    const float *Ud = U + d * ldU;
                    if (row + off < n)
                        v += __ldg(Ud + row) * dir(__ldg(rh + row + off), __ldg(pold + row + off), beta);
                    if (row - off >= 0)
                        v += __ldg(Ud + row - off) * dir(__ldg(rh + row - off), __ldg(pold + row - off), beta);
                }
                qh[row] = v;
                acc += pr * v;
            }
        }
    }
    double total;
    if (grid_sum_last_f(acc, partials, &s->counter[1], total) && threadIdx.x == 0)
        mx_alpha(s, total);
}

// K1 (csr): p = r + beta p_old, q = p + offdiag(S A S) p, p.q.  Thread per row.
__global__ void __launch_bounds__(kBlock) k_mx_spmv_csr(int64_t n, const int32_t *__restrict__ orow,
                                                        const int32_t *__restrict__ ocol,
                                                        const float *__restrict__ oval, const float *__restrict__ rh,
                                                        const float *__restrict__ pold, float *__restrict__ pnew,
                                                        float *__restrict__ qh, double *partials, SolveScalars *s)
{
    if (ld_flag(&s->done))
        return;
    const float beta = static_cast<float>(__ldcg(&s->beta));
    float acc = 0.0f;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const float pi = dir(__ldg(rh + i), __ldg(pold + i), beta);
        pnew[i] = pi;
        float y = pi;
        for (int k = __ldg(orow + i); k < __ldg(orow + i + 1); ++k) {
            const int j = __ldg(ocol + k);
            y += __ldg(oval + k) * dir(__ldg(rh + j), __ldg(pold + j), beta);
        }
        qh[i] = y;
        acc += pi * y;
    }
    double total;
    if (grid_sum_last_f(acc, partials, &s->counter[1], total) && threadIdx.x == 0)
        mx_alpha(s, total);
}

// K2: xh += alpha ph, rh -= alpha qh, rr = rh.rh; decide on a reliable update.
__global__ void __launch_bounds__(kBlock) k_mx_update(int64_t n, const float *__restrict__ ph,
                                                      const float *__restrict__ qh, float *__restrict__ xh,
                                                      float *__restrict__ rh, double *partials, SolveScalars *s)
{
    if (ld_flag(&s->done))
        return;
    const float alpha = static_cast<float>(__ldcg(&s->alpha));
    float acc = 0.0f;
    const int64_t tid = blockIdx.x * (int64_t)blockDim.x + threadIdx.x, stride = (int64_t)gridDim.x * blockDim.x;
    const int64_t n4 = n >> 2;
    for (int64_t i = tid; i < n4; i += stride) {
        const float4 p = reinterpret_cast<const float4 *>(ph)[i];
        const float4 q = reinterpret_cast<const float4 *>(qh)[i];
        float4 x = reinterpret_cast<float4 *>(xh)[i];
        float4 r = reinterpret_cast<float4 *>(rh)[i];
        x.x += alpha * p.x;
        x.y += alpha * p.y;
        x.z += alpha * p.z;
        x.w += alpha * p.w;
        r.x -= alpha * q.x;
        r.y -= alpha * q.y;
        r.z -= alpha * q.z;
        r.w -= alpha * q.w;
        reinterpret_cast<float4 *>(xh)[i] = x;
        reinterpret_cast<float4 *>(rh)[i] = r;
        acc += r.x * r.x + r.y * r.y + r.z * r.z + r.w * r.w;
    }
    for (int64_t i = 4 * n4 + tid; i < n; i += stride) {
        xh[i] += alpha * ph[i];
        const float r = rh[i] - alpha * qh[i];
        rh[i] = r;
        acc += r * r;
    }
    double rr;
    if (grid_sum_last_f(acc, partials, &s->counter[2], rr) && threadIdx.x == 0) {
        s->iter += 1;
        const double sigma = sqrt(rr);
        const double est = s->t0 * sigma / s->sigma0;
        s->last = est;
        if (s->need_update || sigma < s->delta * s->rmax || est < s->tol || s->iter >= s->max_iter) {
            s->need_update = 1;  // beta is formed after the residual replacement
        } else {
            s->beta = rr / s->rz;
            s->rz = rr;
            if (sigma > s->rmax)
                s->rmax = sigma;
        }
    }
}

// U1: x += S xh (FP64), xh = 0.
__global__ void __launch_bounds__(kBlock) k_mx_fold(int64_t n, const double *__restrict__ sc, float *__restrict__ xh,
                                                    double *__restrict__ x, const SolveScalars *s)
{
    if (!ld_flag(&s->need_update) || ld_flag(&s->done))
        return;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        x[i] += sc[i] * static_cast<double>(xh[i]);
        xh[i] = 0.0f;
    }
}

// U2: r = b - A x in FP64 (staged CSR SpMV); stop test on the true residual.
struct ResEpi {
    const double *b;
    double *r;
    double acc;
    __device__ __forceinline__ void operator()(int row, double y)
    {
        const double v = __ldg(b + row) - y;
        r[row] = v;
        acc += v * v;
    }
};

__global__ void __launch_bounds__(kBlock) k_mx_true_residual(const int32_t *__restrict__ rowPtr,
                                                             const int32_t *__restrict__ colIdx,
                                                             const double *__restrict__ val,
                                                             const int32_t *__restrict__ rb, int nRB,
                                                             const double *__restrict__ x, const double *__restrict__ b,
                                                             double *__restrict__ r, double *partials, SolveScalars *s)
{
    if (!ld_flag(&s->need_update) || ld_flag(&s->done))
        return;
    ResEpi epi{b, r, 0.0};
    spmv_rowblocks(rowPtr, colIdx, val, rb, nRB, x, epi);
    double v[1] = {epi.acc};
    if (grid_sum_last<1>(v, partials, &s->counter[3]) && threadIdx.x == 0) {
        s->rr = v[0];
        const double t = sqrt(v[0]) / s->bnorm;
        s->last = t;
        s->t0 = t;
        if (t < s->tol) {
            s->done = 1;
            s->result = s->iter;
        } else if (s->iter >= s->max_iter || s->status == SIMALL_ERR_BREAKDOWN) {
            s->done = 1;
            s->result = s->iter >= s->max_iter ? s->max_iter : s->iter;
        }
    }
}

// U3: rh = S r (FP32), rho_new = rh.rh; beta = rho_new / rho; reset the trigger.
__global__ void __launch_bounds__(kBlock) k_mx_replace(int64_t n, const double *__restrict__ sc,
                                                       const double *__restrict__ r, float *__restrict__ rh,
                                                       double *partials, SolveScalars *s)
{
    if (!ld_flag(&s->need_update) || ld_flag(&s->done))
        return;
    float acc = 0.0f;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const float v = static_cast<float>(sc[i] * r[i]);
        rh[i] = v;
        acc += v * v;
    }
    double rho;
    if (grid_sum_last_f(acc, partials, &s->counter[4], rho) && threadIdx.x == 0) {
        s->beta = rho / s->rz;
        s->rz = rho;
        s->sigma0 = sqrt(rho);
        s->rmax = s->sigma0;
        s->need_update = 0;
        s->updates += 1;
    }
}

int grid_n(simall_context *ctx, int64_t n)
{
    const int64_t g = (n + kBlock - 1) / kBlock;
    const int64_t cap = grid_size_streaming(ctx);
    return static_cast<int>(g < 1 ? 1 : (g < cap ? g : cap));
}

// Distinct upper-triangle offsets j - i of the pattern (a table of
// kOffTable slots, empty = INT_MIN), the count of upper entries, and an
// overflow flag when there are more than kMaxDiags distinct offsets.
constexpr int kOffTable = 16;

__device__ __forceinline__ bool table_insert(int *tab, int off)
{
    for (int s = 0; s < kOffTable; ++s) {
        const int cur = tab[s];
        if (cur == off)
            return true;
        if (cur == INT_MIN) {
            const int prev = atomicCAS(tab + s, INT_MIN, off);
            if (prev == INT_MIN || prev == off)
                return true;
        }
    }
    return false;
}

__global__ void __launch_bounds__(kBlock) k_mx_offsets(int64_t n, const int32_t *__restrict__ rowPtr,
                                                       const int32_t *__restrict__ colIdx, int *table,
                                                       unsigned long long *upper, int *overflow)
{
    __shared__ int stab[kOffTable];
    __shared__ int sover;
    __shared__ unsigned long long scount;
    if (threadIdx.x < kOffTable)
        stab[threadIdx.x] = INT_MIN;
    if (threadIdx.x == 0) {
        sover = 0;
        scount = 0ull;
    }
    __syncthreads();
    int local[kMaxDiags];
    int nl = 0;
    bool over = false;
    unsigned long long cnt = 0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        for (int k = rowPtr[i]; k < rowPtr[i + 1]; ++k) {
            const int j = colIdx[k];
            if (j <= i)
                continue;
            ++cnt;
            const int off = j - static_cast<int>(i);
            bool seen = false;
            for (int t = 0; t < nl; ++t)
                seen |= (local[t] == off);
            if (!seen) {
                if (nl < kMaxDiags)
                    local[nl++] = off;
                else
                    over = true;
            }
        }
    for (int t = 0; t < nl; ++t)
        if (!table_insert(stab, local[t]))
            over = true;
    if (over)
        atomicOr(&sover, 1);
    atomicAdd(&scount, cnt);
    __syncthreads();
    if (threadIdx.x < kOffTable && stab[threadIdx.x] != INT_MIN)
        if (!table_insert(table, stab[threadIdx.x]))
            atomicOr(overflow, 1);
    if (threadIdx.x == 0) {
        atomicAdd(upper, scount);
        if (sover)
            atomicOr(overflow, 1);
    }
}

// Choose the storage format of S A S from the pattern (diagonal storage only
// if allowed).  The diagonal test runs on the device; the CSR fallback is
// built from a host copy of the pattern.
int analyse_pattern(simall_solver *s, MixedData *m, bool allow_dia)
{
    simall_context *ctx = s->ctx;
    const int64_t n = s->n;
    std::vector<int32_t> offs;
    bool ok = allow_dia;
    if (ok) {
        DevBuf<int> tab;
        DevBuf<unsigned long long> cnt;
        SIMALL_CUDA_TRY(ctx, tab.alloc(kOffTable + 1));
        SIMALL_CUDA_TRY(ctx, cnt.alloc(1));
        std::vector<int> init(kOffTable + 1, INT_MIN);
        init[kOffTable] = 0;
        SIMALL_CUDA_TRY(ctx, cudaMemcpyAsync(tab.p, init.data(), init.size() * sizeof(int), cudaMemcpyHostToDevice,
                                             ctx->stream));
        SIMALL_CUDA_TRY(ctx, cudaMemsetAsync(cnt.p, 0, sizeof(unsigned long long), ctx->stream));
        k_mx_offsets<<<grid_n(ctx, n), kBlock, 0, ctx->stream>>>(n, s->rowPtr, s->colIdx, tab.p, cnt.p,
                                                                 tab.p + kOffTable);
        SIMALL_LAUNCH_CHECK(ctx);
        std::vector<int> h(kOffTable + 1);
        unsigned long long upper = 0;
        SIMALL_CUDA_TRY(ctx, cudaMemcpyAsync(h.data(), tab.p, h.size() * sizeof(int), cudaMemcpyDeviceToHost,
                                             ctx->stream));
        SIMALL_CUDA_TRY(ctx, cudaMemcpyAsync(&upper, cnt.p, sizeof(upper), cudaMemcpyDeviceToHost, ctx->stream));
        SIMALL_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
        for (int t = 0; t < kOffTable; ++t)
            if (h[t] != INT_MIN)
                offs.push_back(h[t]);
        ok = !h[kOffTable] && !offs.empty() && static_cast<int>(offs.size()) <= kMaxDiags &&
             static_cast<double>(offs.size()) * n <= 1.3 * static_cast<double>(upper);
    }
    m->dia = ok;
    if (m->dia) {
        std::sort(offs.begin(), offs.end());
        m->offs.nd = static_cast<int>(offs.size());
        for (int d = 0; d < kMaxDiags; ++d)
            m->offs.off[d] = d < m->offs.nd ? offs[d] : 0;
    } else {
        int st = solver_host_pattern(s);
        if (st)
            return st;
        const int32_t *rp = s->h_rowPtr.data(), *ci = s->h_colIdx.data();
        m->h_orow.assign(static_cast<size_t>(n) + 1, 0);
        m->h_ocol.clear();
        m->h_opos.clear();
        for (int64_t i = 0; i < n; ++i) {
            for (int k = rp[i]; k < rp[i + 1]; ++k)
                if (ci[k] != i) {
                    m->h_ocol.push_back(ci[k]);
                    m->h_opos.push_back(k);
                }
            m->h_orow[i + 1] = static_cast<int32_t>(m->h_ocol.size());
        }
        m->nnzOff = static_cast<int>(m->h_ocol.size());
    }
    m->patternReady = true;
    return SIMALL_OK;
}

int launch_spmv_dia(simall_context *ctx, MixedData *m, int64_t n, const float *pold, float *pnew, double *partials,
                    SolveScalars *sc)
{
    const int64_t quads = (n + 3) / 4;
    const int ni = static_cast<int>(n);
    bool grid = m->offs.nd >= 1 && m->offs.off[0] == 1;
    for (int d = 1; d < m->offs.nd; ++d)
        grid = grid && (m->offs.off[d] & 3) == 0;
    switch (m->offs.nd) {
#define SIMALL_DIA_CASE(ND)                                                                                           \
    case ND:                                                                                                          \
        if (grid) {                                                                                                   \
            const int g = resident_grid(ctx, reinterpret_cast<const void *>(k_mx_spmv_dia<ND, true>), quads);         \
            k_mx_spmv_dia<ND, true><<<g, kBlock, 0, ctx->stream>>>(ni, m->ldU, m->offs, m->U.p, m->rh.p, pold, pnew,  \
                                                                   m->qh.p, partials, sc);                            \
        } else {                                                                                                      \
            const int g = resident_grid(ctx, reinterpret_cast<const void *>(k_mx_spmv_dia<ND, false>), quads);        \
            k_mx_spmv_dia<ND, false><<<g, kBlock, 0, ctx->stream>>>(ni, m->ldU, m->offs, m->U.p, m->rh.p, pold, pnew, \
                                                                    m->qh.p, partials, sc);                           \
        }                                                                                                             \
        break;
        SIMALL_DIA_CASE(1)
        SIMALL_DIA_CASE(2)
        SIMALL_DIA_CASE(3)
        SIMALL_DIA_CASE(4)
        SIMALL_DIA_CASE(5)
        SIMALL_DIA_CASE(6)
        SIMALL_DIA_CASE(7)
        SIMALL_DIA_CASE(8)
#undef SIMALL_DIA_CASE
    default:
        return fail(ctx, SIMALL_ERR_INVALID_ARGUMENT, "dia storage with %d diagonals", m->offs.nd);
    }
    SIMALL_LAUNCH_CHECK(ctx);
    return SIMALL_OK;
}

}  // namespace

int mixed_setup(simall_solver *s)
{
    simall_context *ctx = s->ctx;
    if (!s->mixed) {
        s->mixed = new (std::nothrow) MixedData;
        if (!s->mixed)
            return SIMALL_ERR_OUT_OF_MEMORY;
    }
    MixedData *m = s->mixed;
    const int64_t n = s->n;
    if (!m->patternReady) {
        int st = analyse_pattern(s, m, true);
        if (st)
            return st;
    }
    SIMALL_CUDA_TRY(ctx, m->scale.alloc(n));
    SIMALL_CUDA_TRY(ctx, m->xh.alloc(n + 4));
    SIMALL_CUDA_TRY(ctx, m->rh.alloc(n + 4));
    SIMALL_CUDA_TRY(ctx, m->ph.alloc(n + 4));
    SIMALL_CUDA_TRY(ctx, m->ph2.alloc(n + 4));
    SIMALL_CUDA_TRY(ctx, m->qh.alloc(n + 4));
    SIMALL_CUDA_TRY(ctx, s->flag.alloc(1));
    SIMALL_CUDA_TRY(ctx, cudaMemsetAsync(s->flag.p, 0, sizeof(int), ctx->stream));
    const int g = grid_n(ctx, n);
    k_mx_scale<<<g, kBlock, 0, ctx->stream>>>(n, s->rowPtr, s->colIdx, s->values, m->scale.p, s->flag.p);
    SIMALL_LAUNCH_CHECK(ctx);
    if (m->dia) {
        k_mx_symcheck<<<g, kBlock, 0, ctx->stream>>>(n, s->rowPtr, s->colIdx, s->values, s->flag.p);
        SIMALL_LAUNCH_CHECK(ctx);
    }
    int h = 0;
    SIMALL_CUDA_TRY(ctx, cudaMemcpyAsync(&h, s->flag.p, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    SIMALL_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
    if (h & 1)
        return fail(ctx, SIMALL_ERR_NOT_POSITIVE, "mixed precision needs a positive diagonal");
    if (m->dia && (h & 2)) {
        int st = analyse_pattern(s, m, false);  // not numerically symmetric: keep every off-diagonal entry
        if (st)
            return st;
    }
    if (m->dia) {
        m->ldU = (n + 3) & ~static_cast<int64_t>(3);
        SIMALL_CUDA_TRY(ctx, m->U.alloc(static_cast<size_t>(m->offs.nd) * m->ldU));
        SIMALL_CUDA_TRY(ctx, cudaMemsetAsync(m->U.p, 0, static_cast<size_t>(m->offs.nd) * m->ldU * sizeof(float),
                                             ctx->stream));
        k_mx_build_dia<<<g, kBlock, 0, ctx->stream>>>(n, m->ldU, s->rowPtr, s->colIdx, s->values, m->scale.p, m->offs,
                                                      m->U.p);
        SIMALL_LAUNCH_CHECK(ctx);
    } else {
        const int no = m->nnzOff;
        SIMALL_CUDA_TRY(ctx, m->orow.alloc(n + 1));
        SIMALL_CUDA_TRY(ctx, m->ocol.alloc(no > 0 ? no : 1));
        SIMALL_CUDA_TRY(ctx, m->opos.alloc(no > 0 ? no : 1));
        SIMALL_CUDA_TRY(ctx, m->oval.alloc(no > 0 ? no : 1));
        std::vector<int32_t> rowOf(static_cast<size_t>(no));
        for (int64_t i = 0; i < n; ++i)
            for (int k = m->h_orow[i]; k < m->h_orow[i + 1]; ++k)
                rowOf[k] = static_cast<int32_t>(i);
        DevBuf<int32_t> dRowOf;
        SIMALL_CUDA_TRY(ctx, dRowOf.alloc(no > 0 ? no : 1));
        SIMALL_CUDA_TRY(ctx, cudaMemcpyAsync(m->orow.p, m->h_orow.data(), (n + 1) * sizeof(int32_t),
                                             cudaMemcpyHostToDevice, ctx->stream));
        if (no > 0) {
            SIMALL_CUDA_TRY(ctx, cudaMemcpyAsync(m->ocol.p, m->h_ocol.data(), no * sizeof(int32_t),
                                                 cudaMemcpyHostToDevice, ctx->stream));
            SIMALL_CUDA_TRY(ctx, cudaMemcpyAsync(m->opos.p, m->h_opos.data(), no * sizeof(int32_t),
                                                 cudaMemcpyHostToDevice, ctx->stream));
            SIMALL_CUDA_TRY(ctx, cudaMemcpyAsync(dRowOf.p, rowOf.data(), no * sizeof(int32_t), cudaMemcpyHostToDevice,
                                                 ctx->stream));
            k_mx_build_csr<<<grid_n(ctx, no), kBlock, 0, ctx->stream>>>(no, dRowOf.p, m->ocol.p, m->opos.p, s->values,
                                                                        m->scale.p, m->oval.p);
            SIMALL_LAUNCH_CHECK(ctx);
        }
        SIMALL_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));  // dRowOf and rowOf die here
    }
    return SIMALL_OK;
}

namespace {

// One iteration; `parity` selects which of ph / ph2 holds the previous
// direction.  A solve starts at parity 0 (ph = 0) and the captured chunks have
// even lengths, so every chunk starts at parity 0 too.
int enqueue_mixed_iteration(simall_solver *s, int parity)
{
    simall_context *ctx = s->ctx;
    MixedData *m = s->mixed;
    const int64_t n = s->n;
    const float *pold = parity ? m->ph2.p : m->ph.p;
    float *pnew = parity ? m->ph.p : m->ph2.p;
    if (m->dia) {
        int st = launch_spmv_dia(ctx, m, n, pold, pnew, s->partials.p, s->scal.p);
        if (st)
            return st;
    } else {
        k_mx_spmv_csr<<<resident_grid(ctx, reinterpret_cast<const void *>(k_mx_spmv_csr), n), kBlock, 0,
                        ctx->stream>>>(n, m->orow.p, m->ocol.p, m->oval.p, m->rh.p, pold, pnew, m->qh.p,
                                       s->partials.p, s->scal.p);
        SIMALL_LAUNCH_CHECK(ctx);
    }
    k_mx_update<<<resident_grid(ctx, reinterpret_cast<const void *>(k_mx_update), (n + 3) / 4), kBlock, 0,
                  ctx->stream>>>(n, pnew, m->qh.p, m->xh.p, m->rh.p, s->partials.p, s->scal.p);
    SIMALL_LAUNCH_CHECK(ctx);
    // the reliable-update kernels return at once unless an update is due
    const int g = grid_n(ctx, n);
    k_mx_fold<<<g, kBlock, 0, ctx->stream>>>(n, m->scale.p, m->xh.p, s->x.p, s->scal.p);
    SIMALL_LAUNCH_CHECK(ctx);
    k_mx_true_residual<<<resident_grid(ctx, reinterpret_cast<const void *>(k_mx_true_residual),
                                       static_cast<int64_t>(s->nRowBlocks) * kBlock),
                         kBlock, 0, ctx->stream>>>(s->rowPtr, s->colIdx, s->values, s->rowBlocks.p, s->nRowBlocks,
                                                   s->x.p, s->b.p, s->r.p, s->partials.p, s->scal.p);
    SIMALL_LAUNCH_CHECK(ctx);
    k_mx_replace<<<g, kBlock, 0, ctx->stream>>>(n, m->scale.p, s->r.p, m->rh.p, s->partials.p, s->scal.p);
    SIMALL_LAUNCH_CHECK(ctx);
    return SIMALL_OK;
}

constexpr int kMixedKernelsPerIteration = 5;

int run_mixed_chunk(simall_solver *s, int len)
{
    simall_context *ctx = s->ctx;
    for (auto &gc : s->graphs)
        if (gc.len == len) {
            SIMALL_CUDA_TRY(ctx, cudaGraphLaunch(gc.exec, ctx->stream));
            ctx->launches.fetch_add(static_cast<int64_t>(len) * kMixedKernelsPerIteration, std::memory_order_relaxed);
            return SIMALL_OK;
        }
    cudaGraph_t graph = nullptr;
    SIMALL_CUDA_TRY(ctx, cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
    int st = SIMALL_OK;
    for (int i = 0; i < len && st == SIMALL_OK; ++i)
        st = enqueue_mixed_iteration(s, i & 1);
    cudaError_t e = cudaStreamEndCapture(ctx->stream, &graph);
    if (st)
        return st;
    if (e != cudaSuccess)
        return cuda_fail(ctx, e, "cudaStreamEndCapture", __FILE__, __LINE__);
    GraphChunk gc;
    gc.len = len;
    e = cudaGraphInstantiate(&gc.exec, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess)
        return cuda_fail(ctx, e, "cudaGraphInstantiate", __FILE__, __LINE__);
    s->graphs.push_back(gc);
    SIMALL_CUDA_TRY(ctx, cudaGraphLaunch(gc.exec, ctx->stream));
    return SIMALL_OK;
}

}  // namespace

int mixed_solve(simall_solver *s, simall_solver_stats *st)
{
    (void)st;
    simall_context *ctx = s->ctx;
    MixedData *m = s->mixed;
    const int64_t n = s->n;
    double tol = s->cfg.tolerance, delta = s->cfg.reliable_delta;
    int maxit = s->cfg.max_iterations;
    SIMALL_CUDA_TRY(ctx, cudaMemcpyAsync(&s->scal.p->tol, &tol, sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
    SIMALL_CUDA_TRY(ctx,
                    cudaMemcpyAsync(&s->scal.p->delta, &delta, sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
    SIMALL_CUDA_TRY(ctx,
                    cudaMemcpyAsync(&s->scal.p->max_iter, &maxit, sizeof(int), cudaMemcpyHostToDevice, ctx->stream));
    k_mx_init<<<grid_n(ctx, n), kBlock, 0, ctx->stream>>>(n, s->b.p, m->scale.p, s->x.p, m->rh.p, m->ph.p, m->xh.p,
                                                          s->partials.p, s->scal.p);
    SIMALL_LAUNCH_CHECK(ctx);
    int done_iters = 0;
    // even chunk lengths keep the direction's double buffer in step
    int chunk = s->cfg.check_interval > 0 ? (s->cfg.check_interval + 1) & ~1 : 16;
    double prev_last = -1.0;
    int prev_iter = 0;
    for (;;) {
        int e = run_mixed_chunk(s, chunk);
        if (e)
            return e;
        done_iters += chunk;
        e = solver_fetch_scalars(s);
        if (e)
            return e;
        if (s->h_scal->done)
            break;
        if (done_iters > 2 * maxit + 64)
            return fail(ctx, SIMALL_ERR_CUDA, "mixed solver did not raise its stop flag");
        if (s->cfg.check_interval <= 0) {
            const double last = s->h_scal->last;
            const int it = s->h_scal->iter;
            int next = 64;
            if (prev_last > 0.0 && last > 0.0 && last < prev_last && it > prev_iter) {
                const double rate = std::log(last / prev_last) / (it - prev_iter);
                const double need = std::log(tol / last) / rate;
                next = need < 4 ? 4 : (need > 64 ? 64 : static_cast<int>(need) + 1);
            }
            prev_last = last;
            prev_iter = it;
            chunk = next;
            // snap to a few captured lengths to bound the number of graphs
            chunk = chunk <= 4 ? 4 : chunk <= 8 ? 8 : chunk <= 16 ? 16 : chunk <= 32 ? 32 : 64;
        }
    }
    return SIMALL_OK;
}

int mixed_enqueue_kernel(simall_solver *s, int k, double *bytes)
{
    simall_context *ctx = s->ctx;
    MixedData *m = s->mixed;
    const int64_t n = s->n;
    const double nd = static_cast<double>(n);
    switch (k) {
    case 4:
        if (m->dia) {
            // U once; rh and p_old gathered once; p_new and qh written
            *bytes = (4.0 * m->offs.nd + 16.0) * nd;
            return launch_spmv_dia(ctx, m, n, m->ph.p, m->ph2.p, s->partials.p, s->scal.p);
        } else {
            k_mx_spmv_csr<<<resident_grid(ctx, reinterpret_cast<const void *>(k_mx_spmv_csr), n), kBlock, 0,
                            ctx->stream>>>(n, m->orow.p, m->ocol.p, m->oval.p, m->rh.p, m->ph.p, m->ph2.p, m->qh.p,
                                           s->partials.p, s->scal.p);
            *bytes = 8.0 * m->nnzOff + 20.0 * nd + 4.0;
        }
        break;
    case 5:
        k_mx_update<<<resident_grid(ctx, reinterpret_cast<const void *>(k_mx_update), (n + 3) / 4), kBlock, 0,
                      ctx->stream>>>(n, m->ph2.p, m->qh.p, m->xh.p, m->rh.p, s->partials.p, s->scal.p);
        *bytes = 24.0 * nd;  // p, qh, xh, rh read; xh, rh written
        break;
    default:
        return fail(ctx, SIMALL_ERR_INVALID_ARGUMENT, "mixed kernel id %d", k);
    }
    SIMALL_LAUNCH_CHECK(ctx);
    return SIMALL_OK;
}

void mixed_invalidate_pattern(simall_solver *s)
{
    if (s->mixed)
        s->mixed->patternReady = false;
}

void mixed_free(simall_solver *s)
{
    delete s->mixed;
    s->mixed = nullptr;
}

}  // namespace simall
