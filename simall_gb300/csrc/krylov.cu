// The non-symmetric Krylov solvers on the device, FP64: the GB300 replacement
// of BiCGSTABSolver::solve (src/solver/LinearSolvers.cpp:363-405),
// GMRESmSolver::solve (:268-343) and TfqmrSolver::solve (:497-609), with the
// Jacobi, ILU(0) or SSOR preconditioner.
// Both start from x = 0 and follow the reference's recurrences, stop tests and
// return values step for step; only the order of the FP64 sums inside each dot
// product differs (grid reductions instead of one serial loop).
//
// Every scalar lives on the device (KrylovScalars); the last CTA of each
// reducing kernel does the scalar work the reference does between vector
// operations, and every kernel returns at once when the solve (or, for GMRES,
// the current cycle) has stopped.
//
// BiCGSTAB, one iteration (Jacobi: five kernels; ILU(0) adds two sweeps pairs):
//   K1  p = r + beta (p - omega v)          [y = M p fused for Jacobi]
//   K2  v = A y, rh.v -> alpha
//   K3  s = r - alpha v, |s| -> early stop  [z = M s fused for Jacobi]
//   K4  t = A z, t.s, t.t -> omega
//   K5  x += alpha y + omega z, r = s - omega t, |r|, rh.r -> stop test, beta
// The host replays chunks of iterations captured as CUDA graphs and polls the
// stop flag between chunks.
//
// GMRES(m), left-preconditioned, modified Gram-Schmidt.  Arnoldi step j is
//   (a)   v_j = u / h (the previous step's orthogonalised vector and its norm,
//         scaled on the fly while it is gathered) and w = A v_j; Jacobi also
//         forms z = M w and H_0j = v_0.z in the same kernel;
//   (b_i) z -= H_(i-1)j v_(i-1), H_ij = v_i.z          (i = 1..j)
//   (c)   z -= H_jj v_j, H_(j+1)j = |z|; the last CTA applies the previous
//         Givens rotations to column j, forms the new one, rotates s and runs
//         the stop test.
// Each step is one captured graph; the host polls the cycle's stop flag after
// every step.  A cycle ends with the triangular solve (one CTA) and x += V y.
//
// TFQMR, one iteration (Jacobi: six kernels; ILU(0)/SSOR add two sweep pairs):
//   T1  u2 = u1 - alpha M v
//   T2  Au2 = A u2; both half steps' w -= alpha Au and |w|^2 -> theta, c,
//       tau, eta of each half step, the residual bound and the check flag
//   T3  d = u + coef d, x += eta d (both half steps); r -= alpha (Au1 + Au2);
//       rh.r -> beta (or the rho breakdown test)
//   T4  only when the bound passed: |b - A x| -> stop, or go on as T3 would
//   T5  u1 = M r + beta (u2 + beta u1)
//   T6  Au1 = A u1; v = Au1 + beta (Au2 + beta v); rh.v -> the iteration
//       count, the sigma breakdown test and alpha
#include "device.cuh"
#include "solver.hpp"

#include <cmath>
#include <new>
#include <vector>

namespace simall {

struct KrylovScalars {
    double rho, rhoNew, alpha, omega, beta;  // BiCGSTAB
    double bnorm, last, tol;
    double sc;      // GMRES: 1 / norm of the pending basis vector
    int iter, max_iter, done, result, status;
    int exit_s;     // BiCGSTAB: |s| passed the test, x += alpha y pending
    int stale;      // GMRES: the pending vector's norm was 0 (the basis vector is not replaced)
    int jdone;      // GMRES: Arnoldi steps taken in this cycle
    int cycle_stop;
    int cycles;
    // TFQMR
    double tau, theta, eta, coef[2], etaStep[2];
    int check;  // the residual bound passed: T4 takes the true residual
    unsigned counter[8];
};

struct KrylovData {
    // BiCGSTAB vectors beside the solver's x, r, p, z, b
    DevBuf<double> rh, v, sv, t, y;
    // TFQMR (beside rh, v and the solver's x, r, z, b)
    DevBuf<double> tw, td, tu1, tu2, tAu1, tAu2;
    // GMRES
    int m = 0;
    int64_t ldV = 0;
    DevBuf<double> V, w, zb[2], hs;
    DevBuf<KrylovScalars> ks;
    KrylovScalars *h_ks = nullptr;
    std::vector<GraphChunk> chunks;        // BiCGSTAB / TFQMR iteration chunks
    std::vector<cudaGraphExec_t> steps;    // GMRES step j
    std::vector<int64_t> stepKernels;
    cudaGraphExec_t restart = nullptr, finish = nullptr;
    int64_t restartKernels = 0, finishKernels = 0;
    ~KrylovData()
    {
        if (h_ks)
            cudaFreeHost(h_ks);
    }
};

namespace {

__device__ __forceinline__ int kdone(const KrylovScalars *k) { return __ldcg(&k->done); }

// GMRES small dense state: H[(m+1) x m] row-major, cs[m], sn[m], s[m+1], y[m].
struct HsView {
    double *H, *cs, *sn, *s, *y;
    int m;
    __device__ __forceinline__ double &h(int i, int j) const { return H[i * m + j]; }
};

__host__ __device__ inline HsView hs_view(double *base, int m)
{
    HsView v;
    v.m = m;
    v.H = base;
    v.cs = base + (m + 1) * m;
    v.sn = v.cs + m;
    v.s = v.sn + m;
    v.y = v.s + (m + 1);
    return v;
}

inline size_t hs_size(int m) { return static_cast<size_t>((m + 1) * m + 2 * m + (m + 1) + m); }

// ---------------------------------------------------------------- BiCGSTAB

__global__ void __launch_bounds__(kBlock) k_bi_init(int64_t n, const double *__restrict__ b, double *__restrict__ x,
                                                    double *__restrict__ r, double *__restrict__ rh,
                                                    double *__restrict__ p, double *__restrict__ v, double *partials,
                                                    KrylovScalars *k)
{
    double acc[1] = {0.0};
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const double bi = b[i];
        x[i] = 0.0;
        p[i] = 0.0;
        v[i] = 0.0;
        r[i] = bi;  // b - A 0
        rh[i] = bi;
        acc[0] += bi * bi;
    }
    if (grid_sum_last<1>(acc, partials, &k->counter[0]) && threadIdx.x == 0) {
        const double bb = acc[0];
        k->bnorm = std_max(sqrt(bb), 1e-30);
        k->rhoNew = bb;  // rh.r with rh = r = b
        k->rho = k->alpha = k->omega = 1.0;
        k->iter = 0;
        k->exit_s = 0;
        k->status = SIMALL_OK;
        k->last = 0.0;
        k->done = 0;
        k->result = 0;
        if (k->max_iter <= 0) {
            k->done = 1;
            k->result = k->max_iter;
        } else if (bb == 0.0) {
            k->last = sqrt(bb) / k->bnorm;
            k->done = 1;
        } else {
            k->beta = (k->rhoNew / k->rho) * (k->alpha / k->omega);
        }
    }
}

// K1: p = r + beta (p - omega v); y = invD p when invD is given.
__global__ void __launch_bounds__(kBlock) k_bi_dir(int64_t n, const double *__restrict__ r, double *__restrict__ p,
                                                   const double *__restrict__ v, const double *__restrict__ invD,
                                                   double *__restrict__ y, const KrylovScalars *k)
{
    if (kdone(k))
        return;
    const double beta = __ldcg(&k->beta), omega = __ldcg(&k->omega);
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const double pi = r[i] + beta * (p[i] - omega * v[i]);
        p[i] = pi;
        if (invD)
            y[i] = invD[i] * pi;
    }
}

struct DotEpi {
    double *out;
    const double *a;
    double acc;
    __device__ __forceinline__ void operator()(int row, double val)
    {
        out[row] = val;
        acc += __ldg(a + row) * val;
    }
};

// K2: v = A y, rh.v -> alpha = rhoNew / rh.v
__global__ void __launch_bounds__(kBlock) k_bi_spmv_v(const int32_t *__restrict__ rowPtr,
                                                      const int32_t *__restrict__ colIdx,
                                                      const double *__restrict__ val, const int32_t *__restrict__ rb,
                                                      int nRB, const double *__restrict__ y, double *__restrict__ v,
                                                      const double *__restrict__ rh, double *partials,
                                                      KrylovScalars *k)
{
    if (kdone(k))
        return;
    DotEpi epi{v, rh, 0.0};
    spmv_rowblocks_fma(rowPtr, colIdx, val, rb, nRB, y, epi);
    double acc[1] = {epi.acc};
    if (grid_sum_last<1>(acc, partials, &k->counter[1]) && threadIdx.x == 0)
        k->alpha = k->rhoNew / acc[0];
}

// K3: s = r - alpha v, |s| (early stop); z = invD s when invD is given.
__global__ void __launch_bounds__(kBlock) k_bi_s(int64_t n, const double *__restrict__ r, const double *__restrict__ v,
                                                 const double *__restrict__ invD, double *__restrict__ s,
                                                 double *__restrict__ z, double *partials, KrylovScalars *k)
{
    if (kdone(k))
        return;
    const double alpha = __ldcg(&k->alpha);
    double acc[1] = {0.0};
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const double si = r[i] - alpha * v[i];
        s[i] = si;
        if (invD)
            z[i] = invD[i] * si;
        acc[0] += si * si;
    }
    if (grid_sum_last<1>(acc, partials, &k->counter[2]) && threadIdx.x == 0) {
        const double sn = sqrt(acc[0]);
        if (sn < k->tol * k->bnorm) {
            k->exit_s = 1;
            k->last = sn / k->bnorm;
            k->result = k->iter + 1;
        }
    }
}

struct TsEpi {
    double *t;
    const double *s;
    double ts, tt;
    __device__ __forceinline__ void operator()(int row, double val)
    {
        t[row] = val;
        ts += val * __ldg(s + row);
        tt += val * val;
    }
};

// K4: t = A z, omega = t.s / max(t.t, 1e-30)
__global__ void __launch_bounds__(kBlock) k_bi_spmv_t(const int32_t *__restrict__ rowPtr,
                                                      const int32_t *__restrict__ colIdx,
                                                      const double *__restrict__ val, const int32_t *__restrict__ rb,
                                                      int nRB, const double *__restrict__ z, double *__restrict__ t,
                                                      const double *__restrict__ s, double *partials,
                                                      KrylovScalars *k)
{
    if (kdone(k) || __ldcg(&k->exit_s))
        return;
    TsEpi epi{t, s, 0.0, 0.0};
    spmv_rowblocks_fma(rowPtr, colIdx, val, rb, nRB, z, epi);
    double acc[2] = {epi.ts, epi.tt};
    if (grid_sum_last<2>(acc, partials, &k->counter[3]) && threadIdx.x == 0)
        k->omega = acc[0] / std_max(acc[1], 1e-30);
}

// K5: x += alpha y + omega z, r = s - omega t; |r| and rh.r; stop test, beta.
// After an early stop in K3 only x += alpha y.
__global__ void __launch_bounds__(kBlock) k_bi_update(int64_t n, double *__restrict__ x, const double *__restrict__ y,
                                                      const double *__restrict__ z, double *__restrict__ r,
                                                      const double *__restrict__ s, const double *__restrict__ t,
                                                      const double *__restrict__ rh, double *partials,
                                                      KrylovScalars *k)
{
    if (kdone(k))
        return;
    const double alpha = __ldcg(&k->alpha), omega = __ldcg(&k->omega);
    const int64_t tid = blockIdx.x * (int64_t)blockDim.x + threadIdx.x, stride = (int64_t)gridDim.x * blockDim.x;
    if (__ldcg(&k->exit_s)) {
        for (int64_t i = tid; i < n; i += stride)
            x[i] += alpha * y[i];
        double acc[1] = {0.0};
        if (grid_sum_last<1>(acc, partials, &k->counter[4]) && threadIdx.x == 0)
            k->done = 1;
        return;
    }
    double acc[2] = {0.0, 0.0};
    for (int64_t i = tid; i < n; i += stride) {
        x[i] += alpha * y[i] + omega * z[i];
        const double ri = s[i] - omega * t[i];
        r[i] = ri;
        acc[0] += ri * ri;
        acc[1] += rh[i] * ri;
    }
    if (grid_sum_last<2>(acc, partials, &k->counter[4]) && threadIdx.x == 0) {
        k->rho = k->rhoNew;
        const double last = sqrt(acc[0]) / k->bnorm;
        k->last = last;
        if (last < k->tol) {
            k->result = k->iter + 1;
            k->done = 1;
            return;
        }
        k->iter += 1;
        if (k->iter >= k->max_iter) {
            k->result = k->max_iter;
            k->done = 1;
            return;
        }
        const double rhoNew = acc[1];
        k->rhoNew = rhoNew;
        if (rhoNew == 0.0) {  // the next iteration's breakdown test
            k->result = k->iter;
            k->done = 1;
            return;
        }
        k->beta = (rhoNew / k->rho) * (k->alpha / k->omega);
    }
}

// ---------------------------------------------------------------- TFQMR

// T0: x = 0, d = 0, r = rh = w = b, u1 = invD b (Jacobi); |b| -> tau, bnorm, rho
__global__ void __launch_bounds__(kBlock) k_tf_init(int64_t n, const double *__restrict__ b, double *__restrict__ x,
                                                    double *__restrict__ r, double *__restrict__ rh,
                                                    double *__restrict__ w, double *__restrict__ d,
                                                    const double *__restrict__ invD, double *__restrict__ u1,
                                                    double *partials, KrylovScalars *k)
{
    double acc[1] = {0.0};
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const double bi = b[i];
        x[i] = 0.0;
        d[i] = 0.0;
        r[i] = bi;
        rh[i] = bi;
        w[i] = bi;
        if (invD)
            u1[i] = invD[i] * bi;
        acc[0] += bi * bi;
    }
    if (grid_sum_last<1>(acc, partials, &k->counter[0]) && threadIdx.x == 0) {
        const double tau = sqrt(acc[0]);
        k->tau = tau;
        k->bnorm = std_max(tau, 1e-30);
        k->rho = acc[0];  // rh.r with rh = r = b
        k->theta = k->eta = k->alpha = 0.0;
        k->iter = 0;
        k->check = 0;
        k->status = SIMALL_OK;
        k->done = 0;
        k->result = 0;
        if (tau / k->bnorm < k->tol) {
            k->last = tau / k->bnorm;
            k->done = 1;
        } else if (k->max_iter <= 0) {  // the loop does not run; last_residual is left as it was
            k->done = 1;
            k->result = k->max_iter;
        }
    }
}

// The sigma test and alpha, at the top of an iteration (thread 0 of a last CTA).
__device__ __forceinline__ void tf_top(KrylovScalars *k, double sigma)
{
    if (fabs(sigma) < 1.0e-30) {
        k->last = k->tau / k->bnorm;
        k->result = k->iter;
        k->done = 1;
        return;
    }
    k->alpha = k->rho / sigma;
}

struct TfVEpi {
    double *Au1, *v;
    const double *Au2, *rh;
    double beta, acc;
    bool first;
    __device__ __forceinline__ void operator()(int row, double val)
    {
        Au1[row] = val;
        const double vi = first ? val : val + beta * (Au2[row] + beta * v[row]);
        v[row] = vi;
        acc += __ldg(rh + row) * vi;
    }
};

// T6 (and the start, first = 1): Au1 = A u1, v = Au1 + beta (Au2 + beta v)
// (v = Au1 at the start), sigma = rh.v; the iteration count, maxIterations,
// the sigma test and alpha.
__global__ void __launch_bounds__(kBlock) k_tf_spmv_u1(const int32_t *__restrict__ rowPtr,
                                                       const int32_t *__restrict__ colIdx,
                                                       const double *__restrict__ val, const int32_t *__restrict__ rb,
                                                       int nRB, const double *__restrict__ u1, double *__restrict__ Au1,
                                                       const double *__restrict__ Au2, double *__restrict__ v,
                                                       const double *__restrict__ rh, double *partials,
                                                       KrylovScalars *k, int first)
{
    if (kdone(k))
        return;
    TfVEpi epi{Au1, v, Au2, rh, first ? 0.0 : __ldcg(&k->beta), 0.0, first != 0};
    spmv_rowblocks_fma(rowPtr, colIdx, val, rb, nRB, u1, epi);
    double acc[1] = {epi.acc};
    if (grid_sum_last<1>(acc, partials, &k->counter[4]) && threadIdx.x == 0) {
        if (!first) {
            k->rho = k->rhoNew;
            k->iter += 1;
            if (k->iter >= k->max_iter) {
                k->result = k->max_iter;
                k->done = 1;
                return;
            }
        }
        tf_top(k, acc[0]);
    }
}

// T1: u2 = u1 - alpha z, z = invD v (Jacobi) or the sweeps' M v.
__global__ void __launch_bounds__(kBlock) k_tf_u2(int64_t n, const double *__restrict__ u1,
                                                  const double *__restrict__ v, const double *__restrict__ invD,
                                                  const double *__restrict__ z, double *__restrict__ u2,
                                                  const KrylovScalars *k)
{
    if (kdone(k))
        return;
    const double alpha = __ldcg(&k->alpha);
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const double zi = invD ? invD[i] * v[i] : z[i];
        u2[i] = u1[i] - alpha * zi;
    }
}

struct TfWEpi {
    double *Au2, *w;
    const double *Au1;
    double alpha, ww1, ww2;
    __device__ __forceinline__ void operator()(int row, double val)
    {
        Au2[row] = val;
        const double w1 = w[row] - alpha * Au1[row];
        const double w2 = w1 - alpha * val;
        w[row] = w2;
        ww1 += w1 * w1;
        ww2 += w2 * w2;
    }
};

// One quasi-minimal-residual half step from |w| (thread 0 of a last CTA).
__device__ __forceinline__ void tf_half(KrylovScalars *k, int h, double wnorm, double alpha)
{
    const double theta_new = wnorm / std_max(k->tau, 1.0e-30);
    const double c = 1.0 / sqrt(1.0 + theta_new * theta_new);
    k->coef[h] = k->theta * k->theta * k->eta / std_max(alpha, 1.0e-30);
    k->etaStep[h] = c * c * alpha;
    k->tau = k->tau * theta_new * c;
    k->theta = theta_new;
    k->eta = k->etaStep[h];
}

// T2: Au2 = A u2; w -= alpha Au1 and then alpha Au2, the norm after each; the
// scalars of both half steps and the residual bound.
__global__ void __launch_bounds__(kBlock) k_tf_spmv_u2(const int32_t *__restrict__ rowPtr,
                                                       const int32_t *__restrict__ colIdx,
                                                       const double *__restrict__ val, const int32_t *__restrict__ rb,
                                                       int nRB, const double *__restrict__ u2, double *__restrict__ Au2,
                                                       const double *__restrict__ Au1, double *__restrict__ w,
                                                       double *partials, KrylovScalars *k)
{
    if (kdone(k))
        return;
    const double alpha = __ldcg(&k->alpha);
    TfWEpi epi{Au2, w, Au1, alpha, 0.0, 0.0};
    spmv_rowblocks_fma(rowPtr, colIdx, val, rb, nRB, u2, epi);
    double acc[2] = {epi.ww1, epi.ww2};
    if (grid_sum_last<2>(acc, partials, &k->counter[1]) && threadIdx.x == 0) {
        tf_half(k, 0, sqrt(acc[0]), alpha);
        tf_half(k, 1, sqrt(acc[1]), alpha);
        const double resBound = k->tau * sqrt(2.0 * (k->iter + 1) + 1.0);
        k->last = resBound / k->bnorm;
        k->check = k->last < k->tol ? 1 : 0;
    }
}

// After x and r are updated (and the true residual, when taken, failed): the
// rho test on the previous rho, else beta.
__device__ __forceinline__ void tf_beta(KrylovScalars *k)
{
    if (fabs(k->rho) < 1.0e-30) {
        k->last = k->tau / k->bnorm;
        k->result = k->iter;
        k->done = 1;
        return;
    }
    k->beta = k->rhoNew / k->rho;
}

// T3: d = u1 + coef0 d, x += eta0 d, d = u2 + coef1 d, x += eta1 d;
// r -= alpha (Au1 + Au2), rh.r -> rhoNew (and beta unless the check is due).
__global__ void __launch_bounds__(kBlock) k_tf_update(int64_t n, const double *__restrict__ u1,
                                                      const double *__restrict__ u2, const double *__restrict__ Au1,
                                                      const double *__restrict__ Au2, double *__restrict__ d,
                                                      double *__restrict__ x, double *__restrict__ r,
                                                      const double *__restrict__ rh, double *partials,
                                                      KrylovScalars *k)
{
    if (kdone(k))
        return;
    const double alpha = __ldcg(&k->alpha);
    const double c0 = __ldcg(&k->coef[0]), c1 = __ldcg(&k->coef[1]);
    const double e0 = __ldcg(&k->etaStep[0]), e1 = __ldcg(&k->etaStep[1]);
    double acc[1] = {0.0};
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        double di = u1[i] + c0 * d[i];
        double xi = x[i] + e0 * di;
        di = u2[i] + c1 * di;
        x[i] = xi + e1 * di;
        d[i] = di;
        const double ri = r[i] - alpha * (Au1[i] + Au2[i]);
        r[i] = ri;
        acc[0] += rh[i] * ri;
    }
    if (grid_sum_last<1>(acc, partials, &k->counter[2]) && threadIdx.x == 0) {
        k->rhoNew = acc[0];
        if (!k->check)
            tf_beta(k);
    }
}

struct TfResEpi {
    const double *b;
    double acc;
    __device__ __forceinline__ void operator()(int row, double val)
    {
        const double ri = __ldg(b + row) - val;
        acc += ri * ri;
    }
};

// T4: when the bound passed, |b - A x| / bnorm is the residual: stop below
// the tolerance, else the rho test and beta.
__global__ void __launch_bounds__(kBlock) k_tf_check(const int32_t *__restrict__ rowPtr,
                                                     const int32_t *__restrict__ colIdx,
                                                     const double *__restrict__ val, const int32_t *__restrict__ rb,
                                                     int nRB, const double *__restrict__ x,
                                                     const double *__restrict__ b, double *partials,
                                                     KrylovScalars *k)
{
    if (kdone(k) || !__ldcg(&k->check))
        return;
    TfResEpi epi{b, 0.0};
    spmv_rowblocks_fma(rowPtr, colIdx, val, rb, nRB, x, epi);
    double acc[1] = {epi.acc};
    if (grid_sum_last<1>(acc, partials, &k->counter[3]) && threadIdx.x == 0) {
        k->check = 0;
        k->last = sqrt(acc[0]) / k->bnorm;
        if (k->last < k->tol) {
            k->result = k->iter + 1;
            k->done = 1;
            return;
        }
        tf_beta(k);
    }
}

// T5: u1 = z + beta (u2 + beta u1), z = invD r (Jacobi) or the sweeps' M r.
__global__ void __launch_bounds__(kBlock) k_tf_u1(int64_t n, const double *__restrict__ r,
                                                  const double *__restrict__ invD, const double *__restrict__ z,
                                                  const double *__restrict__ u2, double *__restrict__ u1,
                                                  const KrylovScalars *k)
{
    if (kdone(k))
        return;
    const double beta = __ldcg(&k->beta);
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const double zi = invD ? invD[i] * r[i] : z[i];
        u1[i] = zi + beta * (u2[i] + beta * u1[i]);
    }
}

// ---------------------------------------------------------------- GMRES(m)

__global__ void __launch_bounds__(kBlock) k_gm_init(int64_t n, const double *__restrict__ b, double *__restrict__ x,
                                                    double *partials, KrylovScalars *k)
{
    double acc[1] = {0.0};
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const double bi = b[i];
        x[i] = 0.0;
        acc[0] += bi * bi;
    }
    if (grid_sum_last<1>(acc, partials, &k->counter[0]) && threadIdx.x == 0) {
        k->bnorm = std_max(sqrt(acc[0]), 1e-30);
        k->iter = 0;
        k->cycles = 0;
        k->status = SIMALL_OK;
        k->last = 0.0;
        k->result = 0;
        k->cycle_stop = 1;
        k->done = (k->max_iter <= 0) ? 1 : 0;  // no cycle runs: iterations 0, last 0
    }
}

// Start of a cycle, once |M r|^2 is known (thread 0 of the last CTA).
__device__ void gm_cycle_start(KrylovScalars *k, HsView hv, double zz)
{
    if (k->cycles >= k->max_iter) {  // the reference's outer-loop bound
        k->result = k->iter;
        k->done = 1;
        return;
    }
    const double beta = sqrt(zz);
    if (beta < k->tol * k->bnorm) {
        k->last = beta / k->bnorm;
        k->result = k->iter;
        k->done = 1;
        return;
    }
    if (k->iter >= k->max_iter) {  // no Arnoldi step left; later cycles repeat this test on the same x
        k->result = k->iter;
        k->done = 1;
        return;
    }
    for (int i = 0; i <= hv.m; ++i)
        hv.s[i] = 0.0;
    hv.s[0] = beta;
    k->sc = 1.0 / beta;
    k->stale = 0;
    k->jdone = 0;
    k->cycle_stop = 0;
}

struct ResidEpi {
    const double *b, *invD;
    double *r, *z;
    double acc;
    __device__ __forceinline__ void operator()(int row, double val)
    {
        const double ri = __ldg(b + row) - val;
        r[row] = ri;
        if (invD) {
            const double zi = __ldg(invD + row) * ri;
            z[row] = zi;
            acc += zi * zi;
        }
    }
};

// r = b - A x; Jacobi: z = invD r, |z| -> cycle start.
__global__ void __launch_bounds__(kBlock) k_gm_resid(const int32_t *__restrict__ rowPtr,
                                                     const int32_t *__restrict__ colIdx,
                                                     const double *__restrict__ val, const int32_t *__restrict__ rb,
                                                     int nRB, const double *__restrict__ x,
                                                     const double *__restrict__ b, const double *__restrict__ invD,
                                                     double *__restrict__ r, double *__restrict__ z, double *partials,
                                                     KrylovScalars *k, double *hs, int m)
{
    if (kdone(k))
        return;
    ResidEpi epi{b, invD, r, z, 0.0};
    spmv_rowblocks_fma(rowPtr, colIdx, val, rb, nRB, x, epi);
    if (!invD)
        return;
    double acc[1] = {epi.acc};
    if (grid_sum_last<1>(acc, partials, &k->counter[1]) && threadIdx.x == 0)
        gm_cycle_start(k, hs_view(hs, m), acc[0]);
}

// ILU(0): |z|^2 of z = M r -> cycle start.
__global__ void __launch_bounds__(kBlock) k_gm_norm(int64_t n, const double *__restrict__ z, double *partials,
                                                    KrylovScalars *k, double *hs, int m)
{
    if (kdone(k))
        return;
    double acc[1] = {0.0};
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        acc[0] += z[i] * z[i];
    if (grid_sum_last<1>(acc, partials, &k->counter[1]) && threadIdx.x == 0)
        gm_cycle_start(k, hs_view(hs, m), acc[0]);
}

__device__ __forceinline__ bool gm_skip(const KrylovScalars *k) { return kdone(k) || __ldcg(&k->cycle_stop); }

// Gathers u_c * sc, the pending basis vector (or the stored one when its norm was 0).
struct ScaledX {
    const double *u;
    double sc;
};

struct StepEpi {
    const double *src, *invD, *V0;
    double mul;
    double *Vj, *out;
    bool first;
    double acc;
    __device__ __forceinline__ void operator()(int row, double val)
    {
        const double vj = __ldg(src + row) * mul;
        Vj[row] = vj;
        if (invD) {
            const double zi = __ldg(invD + row) * val;
            out[row] = zi;
            acc += (first ? vj : __ldg(V0 + row)) * zi;
        } else {
            out[row] = val;
        }
    }
};

// (a): v_j = u * sc stored; w = A v_j (gathering u * sc); Jacobi: z = invD w, H_0j = v_0.z.
// The products are formed with the scaled gathered values, so A v_j is exactly
// the SpMV of the stored v_j.
__global__ void __launch_bounds__(kBlock) k_gm_step(const int32_t *__restrict__ rowPtr,
                                                    const int32_t *__restrict__ colIdx,
                                                    const double *__restrict__ val, const int32_t *__restrict__ rb,
                                                    int nRB, const double *__restrict__ u, double *__restrict__ Vj,
                                                    const double *__restrict__ V0, const double *__restrict__ invD,
                                                    double *__restrict__ out, double *partials, KrylovScalars *k,
                                                    double *hs, int m, int j)
{
    if (gm_skip(k))
        return;
    const bool stale = __ldcg(&k->stale) != 0;
    const double mul = stale ? 1.0 : __ldcg(&k->sc);
    const double *src = stale ? Vj : u;
    __shared__ double prod[kSpmvNnzCap];
    StepEpi epi{src, invD, V0, mul, Vj, out, j == 0, 0.0};
    if (nRB < 0) {  // one thread per row (the schedule of spmv_rowblocks)
        const int64_t n = -static_cast<int64_t>(nRB);
        for (int64_t row = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; row < n;
             row += (int64_t)gridDim.x * blockDim.x) {
            const int k1 = __ldg(rowPtr + row + 1);
            double sacc = 0.0;
            for (int q = __ldg(rowPtr + row); q < k1; ++q)
                sacc = __dadd_rn(sacc, __dmul_rn(__ldg(val + q), __dmul_rn(__ldg(src + __ldg(colIdx + q)), mul)));
            epi(static_cast<int>(row), sacc);
        }
    }
    // the staged SpMV with the gathered operand scaled on the fly
    for (int bI = blockIdx.x; bI < nRB; bI += gridDim.x) {
        const int r0 = __ldg(rb + bI), r1 = __ldg(rb + bI + 1);
        const int base = __ldg(rowPtr + r0);
        const int cnt = __ldg(rowPtr + r1) - base;
        if (cnt <= kSpmvNnzCap) {
            for (int q = threadIdx.x; q < cnt; q += blockDim.x)
                prod[q] = __ldg(val + base + q) * (__ldg(src + __ldg(colIdx + base + q)) * mul);
            __syncthreads();
            for (int row = r0 + threadIdx.x; row < r1; row += blockDim.x) {
                const int k0 = __ldg(rowPtr + row) - base, k1 = __ldg(rowPtr + row + 1) - base;
                double sacc = 0.0;
                for (int q = k0; q < k1; ++q)
                    sacc += prod[q];
                epi(row, sacc);
            }
            __syncthreads();
        } else {
            double sacc[1] = {0.0};
            for (int q = threadIdx.x; q < cnt; q += blockDim.x)
                sacc[0] += __ldg(val + base + q) * (__ldg(src + __ldg(colIdx + base + q)) * mul);
            block_sum<1>(sacc);
            if (threadIdx.x == 0)
                epi(r0, sacc[0]);
            __syncthreads();
        }
    }
    if (!invD)
        return;
    double acc[1] = {epi.acc};
    if (grid_sum_last<1>(acc, partials, &k->counter[2]) && threadIdx.x == 0)
        hs_view(hs, m).h(0, j) = acc[0];
}

// ILU(0): H_0j = v_0.z
__global__ void __launch_bounds__(kBlock) k_gm_dot0(int64_t n, const double *__restrict__ V0,
                                                    const double *__restrict__ z, double *partials, KrylovScalars *k,
                                                    double *hs, int m, int j)
{
    if (gm_skip(k))
        return;
    double acc[1] = {0.0};
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        acc[0] += V0[i] * z[i];
    if (grid_sum_last<1>(acc, partials, &k->counter[2]) && threadIdx.x == 0)
        hs_view(hs, m).h(0, j) = acc[0];
}

// (b_i): z -= H_(i-1)j v_(i-1); H_ij = v_i.z
__global__ void __launch_bounds__(kBlock) k_gm_mgs(int64_t n, const double *__restrict__ Vprev,
                                                   const double *__restrict__ Vi, double *__restrict__ z,
                                                   double *partials, KrylovScalars *k, double *hs, int m, int i, int j)
{
    if (gm_skip(k))
        return;
    const HsView hv = hs_view(hs, m);
    const double h = -__ldcg(&hv.h(i - 1, j));
    double acc[1] = {0.0};
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < n; q += (int64_t)gridDim.x * blockDim.x) {
        const double zq = z[q] + h * Vprev[q];
        z[q] = zq;
        acc[0] += Vi[q] * zq;
    }
    if (grid_sum_last<1>(acc, partials, &k->counter[3]) && threadIdx.x == 0)
        hv.h(i, j) = acc[0];
}

// (c): z -= H_jj v_j; H_(j+1)j = |z|; Givens rotations and the stop test.
__global__ void __launch_bounds__(kBlock) k_gm_last(int64_t n, const double *__restrict__ Vj, double *__restrict__ z,
                                                    double *partials, KrylovScalars *k, double *hs, int m, int j)
{
    if (gm_skip(k))
        return;
    const HsView hv = hs_view(hs, m);
    const double h = -__ldcg(&hv.h(j, j));
    double acc[1] = {0.0};
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < n; q += (int64_t)gridDim.x * blockDim.x) {
        const double zq = z[q] + h * Vj[q];
        z[q] = zq;
        acc[0] += zq * zq;
    }
    if (grid_sum_last<1>(acc, partials, &k->counter[4]) && threadIdx.x == 0) {
        const double hn = sqrt(acc[0]);
        hv.h(j + 1, j) = hn;
        k->stale = (hn == 0.0) ? 1 : 0;
        if (hn != 0.0)
            k->sc = 1.0 / hn;
        for (int i = 0; i < j; ++i) {
            const double t = hv.cs[i] * hv.h(i, j) + hv.sn[i] * hv.h(i + 1, j);
            hv.h(i + 1, j) = -hv.sn[i] * hv.h(i, j) + hv.cs[i] * hv.h(i + 1, j);
            hv.h(i, j) = t;
        }
        const double dd = hypot(hv.h(j, j), hv.h(j + 1, j));
        hv.cs[j] = hv.h(j, j) / dd;
        hv.sn[j] = hv.h(j + 1, j) / dd;
        hv.h(j, j) = dd;
        hv.h(j + 1, j) = 0.0;
        const double t = hv.cs[j] * hv.s[j];
        hv.s[j + 1] = -hv.sn[j] * hv.s[j];
        hv.s[j] = t;
        const double last = fabs(hv.s[j + 1]) / k->bnorm;
        k->last = last;
        k->jdone = j + 1;
        if (last < k->tol) {
            k->cycle_stop = 1;  // the converging step is not counted (the reference breaks before ++iter)
            return;
        }
        k->iter += 1;
        if (j + 1 == m || k->iter >= k->max_iter)
            k->cycle_stop = 1;
    }
}

// Back substitution H y = s over the cycle's steps (one thread; at most m^2/2 FMAs).
__global__ void k_gm_backsolve(KrylovScalars *k, double *hs, int m)
{
    if (threadIdx.x != 0 || kdone(k))
        return;
    const HsView hv = hs_view(hs, m);
    const int jd = k->jdone;
    for (int i = jd - 1; i >= 0; --i) {
        double sum = hv.s[i];
        for (int q = i + 1; q < jd; ++q)
            sum -= hv.h(i, q) * hv.y[q];
        hv.y[i] = sum / hv.h(i, i);
    }
}

// x += sum_i y_i v_i (in index order, as the reference's axpy sequence), then
// the cycle's exit test.
__global__ void __launch_bounds__(kBlock) k_gm_update(int64_t n, int64_t ldV, const double *__restrict__ V,
                                                      double *__restrict__ x, double *partials, KrylovScalars *k,
                                                      double *hs, int m)
{
    if (kdone(k))
        return;
    const HsView hv = hs_view(hs, m);
    const int jd = __ldcg(&k->jdone);
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < n; q += (int64_t)gridDim.x * blockDim.x) {
        double xq = x[q];
        for (int i = 0; i < jd; ++i)
            xq += __ldcg(&hv.y[i]) * V[i * ldV + q];
        x[q] = xq;
    }
    double acc[1] = {0.0};
    if (grid_sum_last<1>(acc, partials, &k->counter[5]) && threadIdx.x == 0) {
        k->cycles += 1;
        k->cycle_stop = 1;
        if (k->last < k->tol) {
            k->result = k->iter;
            k->done = 1;
        }
    }
}

// ---------------------------------------------------------------- host side

int grid_n(simall_context *ctx, const void *fn, int64_t n) { return resident_grid(ctx, fn, n); }

#define KLAUNCH(fn, items, ...)                                                                                     \
    do {                                                                                                            \
        fn<<<grid_n(ctx, reinterpret_cast<const void *>(fn), (items)), kBlock, 0, ctx->stream>>>(__VA_ARGS__);      \
        SIMALL_LAUNCH_CHECK(ctx);                                                                                   \
    } while (0)

int alloc_data(simall_solver *s)
{
    simall_context *ctx = s->ctx;
    if (!s->krylov) {
        s->krylov = new (std::nothrow) KrylovData;
        if (!s->krylov)
            return fail(ctx, SIMALL_ERR_OUT_OF_MEMORY, "krylov state");
    }
    KrylovData *d = s->krylov;
    const size_t n = static_cast<size_t>(s->n) + 2;
    if (!d->ks.p) {
        SIMALL_CUDA_TRY(ctx, d->ks.alloc(1));
        SIMALL_CUDA_TRY(ctx, cudaMemsetAsync(d->ks.p, 0, sizeof(KrylovScalars), ctx->stream));
        SIMALL_CUDA_TRY(ctx, cudaMallocHost(reinterpret_cast<void **>(&d->h_ks), sizeof(KrylovScalars)));
    }
    if (s->cfg.kind == SIMALL_SOLVER_BICGSTAB) {
        SIMALL_CUDA_TRY(ctx, d->rh.alloc(n));
        SIMALL_CUDA_TRY(ctx, d->v.alloc(n));
        SIMALL_CUDA_TRY(ctx, d->sv.alloc(n));
        SIMALL_CUDA_TRY(ctx, d->t.alloc(n));
        SIMALL_CUDA_TRY(ctx, d->y.alloc(n));
    } else if (s->cfg.kind == SIMALL_SOLVER_TFQMR) {
        SIMALL_CUDA_TRY(ctx, d->rh.alloc(n));
        SIMALL_CUDA_TRY(ctx, d->v.alloc(n));
        SIMALL_CUDA_TRY(ctx, d->tw.alloc(n));
        SIMALL_CUDA_TRY(ctx, d->td.alloc(n));
        SIMALL_CUDA_TRY(ctx, d->tu1.alloc(n));
        SIMALL_CUDA_TRY(ctx, d->tu2.alloc(n));
        SIMALL_CUDA_TRY(ctx, d->tAu1.alloc(n));
        SIMALL_CUDA_TRY(ctx, d->tAu2.alloc(n));
    } else {
        const int m = s->cfg.restart > 1 ? s->cfg.restart : 1;
        if (m != d->m || d->ldV < static_cast<int64_t>(n)) {
            krylov_drop_graphs(s);
            d->m = m;
            d->ldV = (static_cast<int64_t>(n) + 31) & ~int64_t(31);
            SIMALL_CUDA_TRY(ctx, d->V.alloc(static_cast<size_t>(m + 1) * d->ldV));
            SIMALL_CUDA_TRY(ctx, cudaMemsetAsync(d->V.p, 0, static_cast<size_t>(m + 1) * d->ldV * sizeof(double),
                                                 ctx->stream));
            SIMALL_CUDA_TRY(ctx, d->hs.alloc(hs_size(m)));
            SIMALL_CUDA_TRY(ctx, cudaMemsetAsync(d->hs.p, 0, hs_size(m) * sizeof(double), ctx->stream));
        }
        SIMALL_CUDA_TRY(ctx, d->w.alloc(n));
        SIMALL_CUDA_TRY(ctx, d->zb[0].alloc(n));
        SIMALL_CUDA_TRY(ctx, d->zb[1].alloc(n));
    }
    return SIMALL_OK;
}

// ILU(0) or SSOR: the preconditioner is applied by the triangular sweeps
bool use_ilu(const simall_solver *s) { return sweep_preconditioner(s->cfg.preconditioner); }

int enqueue_bicgstab_iteration(simall_solver *s)
{
    simall_context *ctx = s->ctx;
    KrylovData *d = s->krylov;
    const int64_t n = s->n, rbThreads = spmv_items(s);
    const bool ilu = use_ilu(s);
    const double *invD = ilu ? nullptr : s->invDiag.p;
    KrylovScalars *k = d->ks.p;
    KLAUNCH(k_bi_dir, n, n, s->r.p, s->p.p, d->v.p, invD, d->y.p, k);
    if (ilu) {
        int e = ilu_apply(s, s->p.p, d->y.p);
        if (e)
            return e;
    }
    KLAUNCH(k_bi_spmv_v, rbThreads, s->rowPtr, s->colIdx, s->values, s->rowBlocks.p, spmv_schedule(s), d->y.p, d->v.p,
            d->rh.p, s->partials.p, k);
    KLAUNCH(k_bi_s, n, n, s->r.p, d->v.p, invD, d->sv.p, s->z.p, s->partials.p, k);
    if (ilu) {
        int e = ilu_apply(s, d->sv.p, s->z.p);
        if (e)
            return e;
    }
    KLAUNCH(k_bi_spmv_t, rbThreads, s->rowPtr, s->colIdx, s->values, s->rowBlocks.p, spmv_schedule(s), s->z.p, d->t.p,
            d->sv.p, s->partials.p, k);
    KLAUNCH(k_bi_update, n, n, s->x.p, d->y.p, s->z.p, s->r.p, d->sv.p, d->t.p, d->rh.p, s->partials.p, k);
    return SIMALL_OK;
}

int enqueue_tfqmr_iteration(simall_solver *s);

// Captures what `enqueue` puts on the stream into a graph; *kernels = launches it holds.
template <class F> int capture(simall_solver *s, F &&enqueue, cudaGraphExec_t *out, int64_t *kernels)
{
    simall_context *ctx = s->ctx;
    const int64_t before = ctx->launches.load(std::memory_order_relaxed);
    cudaGraph_t graph = nullptr;
    SIMALL_CUDA_TRY(ctx, cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
    int st = enqueue();
    cudaError_t e = cudaStreamEndCapture(ctx->stream, &graph);
    if (st) {
        if (graph)
            cudaGraphDestroy(graph);
        return st;
    }
    if (e != cudaSuccess)
        return cuda_fail(ctx, e, "cudaStreamEndCapture", __FILE__, __LINE__);
    e = cudaGraphInstantiate(out, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess)
        return cuda_fail(ctx, e, "cudaGraphInstantiate", __FILE__, __LINE__);
    // the captured launches were counted while capturing; replays add them again
    *kernels = ctx->launches.load(std::memory_order_relaxed) - before;
    ctx->launches.fetch_sub(*kernels, std::memory_order_relaxed);
    return SIMALL_OK;
}

int replay(simall_context *ctx, cudaGraphExec_t g, int64_t kernels)
{
    SIMALL_CUDA_TRY(ctx, cudaGraphLaunch(g, ctx->stream));
    ctx->launches.fetch_add(kernels, std::memory_order_relaxed);
    return SIMALL_OK;
}

int fetch(simall_solver *s)
{
    simall_context *ctx = s->ctx;
    KrylovData *d = s->krylov;
    SIMALL_CUDA_TRY(ctx, cudaMemcpyAsync(d->h_ks, d->ks.p, sizeof(KrylovScalars), cudaMemcpyDeviceToHost,
                                         ctx->stream));
    SIMALL_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
    return SIMALL_OK;
}

// BiCGSTAB and TFQMR: the start, then chunks of captured iterations until the
// stop flag is raised.
int chunked_solve(simall_solver *s)
{
    simall_context *ctx = s->ctx;
    KrylovData *d = s->krylov;
    const int64_t n = s->n;
    const bool tfqmr = s->cfg.kind == SIMALL_SOLVER_TFQMR;
    if (tfqmr) {
        const bool ilu = use_ilu(s);
        KLAUNCH(k_tf_init, n, n, s->b.p, s->x.p, s->r.p, d->rh.p, d->tw.p, d->td.p, ilu ? nullptr : s->invDiag.p,
                d->tu1.p, s->partials.p, d->ks.p);
        if (ilu) {
            int e = ilu_apply(s, s->r.p, d->tu1.p);
            if (e)
                return e;
        }
        const int64_t rbThreads = spmv_items(s);
        KLAUNCH(k_tf_spmv_u1, rbThreads, s->rowPtr, s->colIdx, s->values, s->rowBlocks.p, spmv_schedule(s), d->tu1.p,
                d->tAu1.p, d->tAu2.p, d->v.p, d->rh.p, s->partials.p, d->ks.p, 1);
    } else {
        KLAUNCH(k_bi_init, n, n, s->b.p, s->x.p, s->r.p, d->rh.p, s->p.p, d->v.p, s->partials.p, d->ks.p);
    }
    const int perIter = tfqmr ? (use_ilu(s) ? 6 + 2 * ilu_apply_launches(s) : 6)
                              : (use_ilu(s) ? 5 + 2 * ilu_apply_launches(s) : 5);
    int done_iters = 0;
    int chunk = s->cfg.check_interval > 0 ? s->cfg.check_interval : 8;
    for (;;) {
        const int len = chunk <= 4 ? chunk : chunk <= 8 ? 8 : chunk <= 16 ? 16 : chunk <= 32 ? 32 : 64;
        GraphChunk *g = nullptr;
        for (auto &c : d->chunks)
            if (c.len == len)
                g = &c;
        int64_t per = 0;
        if (!g) {
            GraphChunk c;
            c.len = len;
            int e = capture(
                s,
                [&]() {
                    int st = SIMALL_OK;
                    for (int i = 0; i < len && st == SIMALL_OK; ++i)
                        st = tfqmr ? enqueue_tfqmr_iteration(s) : enqueue_bicgstab_iteration(s);
                    return st;
                },
                &c.exec, &per);
            if (e)
                return e;
            d->chunks.push_back(c);
            g = &d->chunks.back();
        } else {
            per = static_cast<int64_t>(len) * perIter;
        }
        int e = replay(ctx, g->exec, per);
        if (e)
            return e;
        done_iters += len;
        e = fetch(s);
        if (e)
            return e;
        if (d->h_ks->done)
            return SIMALL_OK;
        if (done_iters > s->cfg.max_iterations + 64)
            return fail(ctx, SIMALL_ERR_CUDA, "%s did not raise its stop flag", tfqmr ? "TFQMR" : "BiCGSTAB");
        if (s->cfg.check_interval <= 0)
            chunk = chunk < 64 ? chunk * 2 : 64;
    }
}

int enqueue_tfqmr_iteration(simall_solver *s)
{
    simall_context *ctx = s->ctx;
    KrylovData *d = s->krylov;
    const int64_t n = s->n, rbThreads = spmv_items(s);
    const bool ilu = use_ilu(s);
    const double *invD = ilu ? nullptr : s->invDiag.p;
    KrylovScalars *k = d->ks.p;
    if (ilu) {
        int e = ilu_apply(s, d->v.p, s->z.p);
        if (e)
            return e;
    }
    KLAUNCH(k_tf_u2, n, n, d->tu1.p, d->v.p, invD, s->z.p, d->tu2.p, k);
    KLAUNCH(k_tf_spmv_u2, rbThreads, s->rowPtr, s->colIdx, s->values, s->rowBlocks.p, spmv_schedule(s), d->tu2.p,
            d->tAu2.p, d->tAu1.p, d->tw.p, s->partials.p, k);
    KLAUNCH(k_tf_update, n, n, d->tu1.p, d->tu2.p, d->tAu1.p, d->tAu2.p, d->td.p, s->x.p, s->r.p, d->rh.p,
            s->partials.p, k);
    KLAUNCH(k_tf_check, rbThreads, s->rowPtr, s->colIdx, s->values, s->rowBlocks.p, spmv_schedule(s), s->x.p, s->b.p,
            s->partials.p, k);
    if (ilu) {
        int e = ilu_apply(s, s->r.p, s->z.p);
        if (e)
            return e;
    }
    KLAUNCH(k_tf_u1, n, n, s->r.p, invD, s->z.p, d->tu2.p, d->tu1.p, k);
    KLAUNCH(k_tf_spmv_u1, rbThreads, s->rowPtr, s->colIdx, s->values, s->rowBlocks.p, spmv_schedule(s), d->tu1.p,
            d->tAu1.p, d->tAu2.p, d->v.p, d->rh.p, s->partials.p, k, 0);
    return SIMALL_OK;
}

int enqueue_gmres_restart(simall_solver *s)
{
    simall_context *ctx = s->ctx;
    KrylovData *d = s->krylov;
    const int64_t n = s->n, rbThreads = spmv_items(s);
    const bool ilu = use_ilu(s);
    // the restart's M r goes to zb[1], the buffer step 0 reads its pending vector from
    KLAUNCH(k_gm_resid, rbThreads, s->rowPtr, s->colIdx, s->values, s->rowBlocks.p, spmv_schedule(s), s->x.p, s->b.p,
            ilu ? nullptr : s->invDiag.p, s->r.p, d->zb[1].p, s->partials.p, d->ks.p, d->hs.p, d->m);
    if (ilu) {
        int e = ilu_apply(s, s->r.p, d->zb[1].p);
        if (e)
            return e;
        KLAUNCH(k_gm_norm, n, n, d->zb[1].p, s->partials.p, d->ks.p, d->hs.p, d->m);
    }
    return SIMALL_OK;
}

int enqueue_gmres_step(simall_solver *s, int j)
{
    simall_context *ctx = s->ctx;
    KrylovData *d = s->krylov;
    const int64_t n = s->n, rbThreads = spmv_items(s);
    const bool ilu = use_ilu(s);
    const int m = d->m;
    auto Vp = [&](int i) { return d->V.p + static_cast<int64_t>(i) * d->ldV; };
    double *z = d->zb[j & 1].p;
    const double *u = d->zb[(j + 1) & 1].p;  // the previous step's (or the restart's) vector
    KLAUNCH(k_gm_step, rbThreads, s->rowPtr, s->colIdx, s->values, s->rowBlocks.p, spmv_schedule(s), u, Vp(j), Vp(0),
            ilu ? nullptr : s->invDiag.p, ilu ? d->w.p : z, s->partials.p, d->ks.p, d->hs.p, m, j);
    if (ilu) {
        int e = ilu_apply(s, d->w.p, z);
        if (e)
            return e;
        KLAUNCH(k_gm_dot0, n, n, Vp(0), z, s->partials.p, d->ks.p, d->hs.p, m, j);
    }
    for (int i = 1; i <= j; ++i)
        KLAUNCH(k_gm_mgs, n, n, Vp(i - 1), Vp(i), z, s->partials.p, d->ks.p, d->hs.p, m, i, j);
    KLAUNCH(k_gm_last, n, n, Vp(j), z, s->partials.p, d->ks.p, d->hs.p, m, j);
    return SIMALL_OK;
}

int enqueue_gmres_finish(simall_solver *s)
{
    simall_context *ctx = s->ctx;
    KrylovData *d = s->krylov;
    k_gm_backsolve<<<1, 32, 0, ctx->stream>>>(d->ks.p, d->hs.p, d->m);
    SIMALL_LAUNCH_CHECK(ctx);
    KLAUNCH(k_gm_update, s->n, s->n, d->ldV, d->V.p, s->x.p, s->partials.p, d->ks.p, d->hs.p, d->m);
    return SIMALL_OK;
}

int gmres_solve(simall_solver *s)
{
    simall_context *ctx = s->ctx;
    KrylovData *d = s->krylov;
    const int m = d->m;
    if (!d->restart) {
        int e = capture(s, [&]() { return enqueue_gmres_restart(s); }, &d->restart, &d->restartKernels);
        if (e)
            return e;
        e = capture(s, [&]() { return enqueue_gmres_finish(s); }, &d->finish, &d->finishKernels);
        if (e)
            return e;
        d->steps.assign(m, nullptr);
        d->stepKernels.assign(m, 0);
    }
    KLAUNCH(k_gm_init, s->n, s->n, s->b.p, s->x.p, s->partials.p, d->ks.p);
    const int64_t maxCycles = static_cast<int64_t>(s->cfg.max_iterations) + 2;
    for (int64_t cycle = 0; cycle < maxCycles; ++cycle) {
        int e = replay(ctx, d->restart, d->restartKernels);
        if (e)
            return e;
        e = fetch(s);
        if (e)
            return e;
        if (d->h_ks->done)
            return SIMALL_OK;
        for (int j = 0; j < m; ++j) {
            if (!d->steps[j]) {
                e = capture(s, [&]() { return enqueue_gmres_step(s, j); }, &d->steps[j], &d->stepKernels[j]);
                if (e)
                    return e;
            }
            e = replay(ctx, d->steps[j], d->stepKernels[j]);
            if (e)
                return e;
            e = fetch(s);
            if (e)
                return e;
            if (d->h_ks->cycle_stop)
                break;
        }
        e = replay(ctx, d->finish, d->finishKernels);
        if (e)
            return e;
        e = fetch(s);
        if (e)
            return e;
        if (d->h_ks->done)
            return SIMALL_OK;
    }
    return fail(ctx, SIMALL_ERR_CUDA, "GMRES did not raise its stop flag");
}

}  // namespace

void krylov_drop_graphs(simall_solver *s)
{
    KrylovData *d = s->krylov;
    if (!d)
        return;
    for (auto &c : d->chunks)
        if (c.exec)
            cudaGraphExecDestroy(c.exec);
    d->chunks.clear();
    for (auto g : d->steps)
        if (g)
            cudaGraphExecDestroy(g);
    d->steps.clear();
    d->stepKernels.clear();
    if (d->restart)
        cudaGraphExecDestroy(d->restart);
    if (d->finish)
        cudaGraphExecDestroy(d->finish);
    d->restart = d->finish = nullptr;
}

void krylov_free(simall_solver *s)
{
    krylov_drop_graphs(s);
    delete s->krylov;
    s->krylov = nullptr;
}

int krylov_solve(simall_solver *s)
{
    simall_context *ctx = s->ctx;
    int e = alloc_data(s);
    if (e)
        return e;
    KrylovData *d = s->krylov;
    // only the control fields are set from the host; the tickets stay zero
    KrylovScalars init{};
    init.tol = s->cfg.tolerance;
    init.max_iter = s->cfg.max_iterations;
    SIMALL_CUDA_TRY(ctx, cudaMemcpyAsync(&d->ks.p->tol, &init.tol, sizeof(double), cudaMemcpyHostToDevice,
                                         ctx->stream));
    SIMALL_CUDA_TRY(ctx, cudaMemcpyAsync(&d->ks.p->max_iter, &init.max_iter, sizeof(int), cudaMemcpyHostToDevice,
                                         ctx->stream));
    e = (s->cfg.kind == SIMALL_SOLVER_BICGSTAB || s->cfg.kind == SIMALL_SOLVER_TFQMR) ? chunked_solve(s)
                                                                                     : gmres_solve(s);
    if (e)
        return e;
    // publish the outcome where the common solve path reads it
    const KrylovScalars &h = *d->h_ks;
    SolveScalars *o = s->h_scal;
    o->result = h.result;
    o->last = h.last;
    o->status = h.status;
    o->bnorm = h.bnorm;
    o->updates = 0;
    o->done = 1;
    return SIMALL_OK;
}

}  // namespace simall
