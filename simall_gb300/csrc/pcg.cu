// FP64 preconditioned CG on a device CSR matrix: the GB300 replacement of
// CGSolver::solve (src/solver/LinearSolvers.cpp:415-459) and gpu::CgGpu
// (src/gpu/CgGpu.cpp:35-238).
//
// One iteration is three kernels with all scalars kept on the device:
//   K1  Ap = A p (staged row-block SpMV) and p.Ap; the last CTA forms alpha.
//   K2  x += alpha p, r -= alpha Ap, z = M r, ||r||^2 and r.z; the last CTA
//       applies the reference stop test and forms beta.
//   K3  p = z + beta p.
// (ILU0 splits K2 around the level-scheduled triangular solves.)  Every
// kernel returns at once when the device stop flag is set, so the host
// enqueues iterations in chunks (captured as CUDA graphs) and polls the flag
// between chunks instead of after each reduction.
#include "device.cuh"
#include "solver.hpp"

#include <chrono>
#include <cmath>
#include <cstring>
#include <new>

namespace simall {

namespace {

__device__ __forceinline__ int ld_done(const SolveScalars *s) { return __ldcg(&s->done); }

__global__ void __launch_bounds__(kBlock) k_jacobi_setup(int64_t n, const int32_t *__restrict__ rowPtr,
                                                         const int32_t *__restrict__ colIdx,
                                                         const double *__restrict__ val, double *__restrict__ invD)
{
    // JacobiPreconditioner::setup (LinearSolvers.cpp:54-65)
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        double d = 1.0;
        for (int k = rowPtr[i]; k < rowPtr[i + 1]; ++k)
            if (colIdx[k] == i) {
                const double a = val[k];
                d = (a != 0.0) ? 1.0 / a : 1.0;
                break;
            }
        invD[i] = d;
    }
}

__global__ void __launch_bounds__(kBlock) k_check_finite(int64_t n, const double *__restrict__ v, int *flag)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        if (!isfinite(v[i]))
            atomicOr(flag, 1);
}

enum : unsigned {
    kBadRowPtr = 1u,     // rowPtr not monotone or outside [0, nnz]
    kBadRange = 2u,      // a column outside [0, n)
    kUnsorted = 4u,      // columns of a row not strictly ascending
    kNoDiag = 8u,        // a row without its diagonal
    kNonFinite = 16u,    // NaN / Inf value
    kPatternDiff = 32u,  // pattern differs from the solver's current one
    kBlockTooBig = 64u,  // a 256-row block holds more nonzeros than the staging buffer
    kBadEnds = 128u      // rowPtr[0] != 0 or rowPtr[n] != nnz
};

__device__ __forceinline__ void or_flags(unsigned f, unsigned *flags)
{
    f = __reduce_or_sync(0xffffffffu, f);
    if ((threadIdx.x & 31) == 0 && f)
        atomicOr(flags, f);
}

// Full CSR validation on the device.  Every row's bounds are checked before
// its columns are read, so a corrupt rowPtr is reported, not followed.
__global__ void __launch_bounds__(kBlock) k_validate_csr(int64_t n, int64_t nnz, const int32_t *__restrict__ rowPtr,
                                                         const int32_t *__restrict__ colIdx,
                                                         const double *__restrict__ values, unsigned *flags)
{
    unsigned f = 0;
    const int64_t tid = blockIdx.x * (int64_t)blockDim.x + threadIdx.x, stride = (int64_t)gridDim.x * blockDim.x;
    if (tid == 0 && (rowPtr[0] != 0 || rowPtr[n] != nnz))
        f |= kBadEnds;
    for (int64_t i = tid; i < n; i += stride) {
        const int a = rowPtr[i], b = rowPtr[i + 1];
        if (a < 0 || b < a || b > nnz) {
            f |= kBadRowPtr;
            continue;
        }
        bool diag = false;
        int prev = -1;
        for (int k = a; k < b; ++k) {
            const int c = colIdx[k];
            if (c < 0 || c >= n) {
                f |= kBadRange;
            } else {
                if (c <= prev)
                    f |= kUnsorted;
                prev = c;
                diag |= (c == i);
            }
            if (values && !isfinite(values[k]))
                f |= kNonFinite;
        }
        if (!diag)
            f |= kNoDiag;
    }
    or_flags(f, flags);
}

__global__ void __launch_bounds__(kBlock) k_compare_pattern(int64_t n, int64_t nnz, const int32_t *__restrict__ ra,
                                                            const int32_t *__restrict__ ca,
                                                            const int32_t *__restrict__ rb,
                                                            const int32_t *__restrict__ cb, unsigned *flags)
{
    unsigned f = 0;
    const int64_t tid = blockIdx.x * (int64_t)blockDim.x + threadIdx.x, stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t i = tid; i <= n; i += stride)
        f |= (ra[i] != rb[i]) ? kPatternDiff : 0u;
    for (int64_t k = tid; k < nnz; k += stride)
        f |= (ca[k] != cb[k]) ? kPatternDiff : 0u;
    or_flags(f, flags);
}

// Row-blocks of kSpmvRows consecutive rows fit the staging buffer?
__global__ void __launch_bounds__(kBlock) k_rowblock_fit(int64_t n, int64_t nb, const int32_t *__restrict__ rowPtr,
                                                         unsigned *flags)
{
    unsigned f = 0;
    const int64_t tid = blockIdx.x * (int64_t)blockDim.x + threadIdx.x, stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t b = tid; b < nb; b += stride) {
        const int64_t r0 = b * kSpmvRows, r1 = (r0 + kSpmvRows < n) ? r0 + kSpmvRows : n;
        f |= (rowPtr[r1] - rowPtr[r0] > kSpmvNnzCap) ? kBlockTooBig : 0u;
    }
    or_flags(f, flags);
}

__global__ void __launch_bounds__(kBlock) k_rowblock_fill(int64_t n, int64_t nb, int32_t *__restrict__ rb)
{
    for (int64_t b = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; b <= nb; b += (int64_t)gridDim.x * blockDim.x)
        rb[b] = static_cast<int32_t>(b * kSpmvRows < n ? b * kSpmvRows : n);
}

// x = 0, r = b, z = invD r, p = z; rz = r.z, bnorm = max(||b||, 1e-30).
__global__ void __launch_bounds__(kBlock) k_init_jacobi(int64_t n, const double *__restrict__ b,
                                                        const double *__restrict__ invD, double *__restrict__ x,
                                                        double *__restrict__ r, double *__restrict__ p,
                                                        double *partials, SolveScalars *s)
{
    double acc[2] = {0.0, 0.0};
    const int64_t tid = blockIdx.x * (int64_t)blockDim.x + threadIdx.x, stride = (int64_t)gridDim.x * blockDim.x;
    const int64_t n2 = n >> 1;
    for (int64_t i = tid; i < n2; i += stride) {
        const double2 bb = reinterpret_cast<const double2 *>(b)[i];
        const double2 id = reinterpret_cast<const double2 *>(invD)[i];
        const double2 z = make_double2(id.x * bb.x, id.y * bb.y);
        reinterpret_cast<double2 *>(x)[i] = make_double2(0.0, 0.0);
        reinterpret_cast<double2 *>(r)[i] = bb;
        reinterpret_cast<double2 *>(p)[i] = z;
        acc[0] += bb.x * z.x + bb.y * z.y;
        acc[1] += bb.x * bb.x + bb.y * bb.y;
    }
    if ((n & 1) && tid == 0) {
        const int64_t i = n - 1;
        const double bi = b[i], zi = invD[i] * bi;
        x[i] = 0.0;
        r[i] = bi;
        p[i] = zi;
        acc[0] += bi * zi;
        acc[1] += bi * bi;
    }
    if (grid_sum_last<2>(acc, partials, &s->counter[0]) && threadIdx.x == 0) {
        s->rz = acc[0];
        s->bnorm = std_max(sqrt(acc[1]), 1e-30);
        s->iter = 0;
        s->status = SIMALL_OK;
        if (s->max_iter <= 0) {
            s->done = 1;
            s->result = s->max_iter;
        } else {
            s->done = 0;
            s->result = 0;
        }
    }
}

struct PapEpi {
    double *Ap;
    const double *p;
    double acc;
    __device__ __forceinline__ void operator()(int row, double y)
    {
        Ap[row] = y;
        acc += __ldg(p + row) * y;
    }
};

// K1: Ap = A p, pAp = p.Ap, alpha = rz / pAp (CGSolver::solve :431-438).
__global__ void __launch_bounds__(kBlock) k_spmv_pap(const int32_t *__restrict__ rowPtr,
                                                     const int32_t *__restrict__ colIdx,
                                                     const double *__restrict__ val, const int32_t *__restrict__ rb,
                                                     int nRB, const double *__restrict__ p, double *__restrict__ Ap,
                                                     double *partials, SolveScalars *s)
{
    if (ld_done(s))
        return;
    PapEpi epi{Ap, p, 0.0};
    spmv_rowblocks_fma(rowPtr, colIdx, val, rb, nRB, p, epi);
    double v[1] = {epi.acc};
    if (grid_sum_last<1>(v, partials, &s->counter[1]) && threadIdx.x == 0) {
        const double pAp = v[0];
        s->pAp = pAp;
        if (s->cggpu ? fabs(pAp) < 1e-300 : pAp == 0.0) {
            // CGSolver returns the iterations done; CgGpu::solve leaves its
            // stats at zero (src/gpu/CgGpu.cpp:190-194)
            s->last = s->cggpu ? 0.0 : sqrt(s->rz) / s->bnorm;
            s->rnorm = s->cggpu ? 0.0 : s->rnorm;
            s->result = s->cggpu ? 0 : s->iter;
            s->done = 1;
            s->status = SIMALL_ERR_BREAKDOWN;
        } else {
            s->alpha = s->rz / pAp;
        }
    }
}

// K1 for matrices with short rows: the same, one thread per row (spmv_rows_fma).
__global__ void __launch_bounds__(kBlock) k_spmv_pap_rows(const int32_t *__restrict__ rowPtr,
                                                          const int32_t *__restrict__ colIdx,
                                                          const double *__restrict__ val, int64_t n,
                                                          const double *__restrict__ p, double *__restrict__ Ap,
                                                          double *partials, SolveScalars *s)
{
    if (ld_done(s))
        return;
    PapEpi epi{Ap, p, 0.0};
    spmv_rows_fma(rowPtr, colIdx, val, n, p, epi);
    double v[1] = {epi.acc};
    if (grid_sum_last<1>(v, partials, &s->counter[1]) && threadIdx.x == 0) {
        const double pAp = v[0];
        s->pAp = pAp;
        if (s->cggpu ? fabs(pAp) < 1e-300 : pAp == 0.0) {
            // CGSolver returns the iterations done; CgGpu::solve leaves its
            // stats at zero (src/gpu/CgGpu.cpp:190-194)
            s->last = s->cggpu ? 0.0 : sqrt(s->rz) / s->bnorm;
            s->rnorm = s->cggpu ? 0.0 : s->rnorm;
            s->result = s->cggpu ? 0 : s->iter;
            s->done = 1;
            s->status = SIMALL_ERR_BREAKDOWN;
        } else {
            s->alpha = s->rz / pAp;
        }
    }
}

struct StoreEpi {
    double *y;
    __device__ __forceinline__ void operator()(int row, double v) { y[row] = v; }
};

// y = A x alone (the SpMV whose HBM bandwidth is reported).
__global__ void __launch_bounds__(kBlock) k_spmv_plain(const int32_t *__restrict__ rowPtr,
                                                       const int32_t *__restrict__ colIdx,
                                                       const double *__restrict__ val, const int32_t *__restrict__ rb,
                                                       int nRB, const double *__restrict__ x, double *__restrict__ y)
{
    StoreEpi epi{y};
    spmv_rowblocks(rowPtr, colIdx, val, rb, nRB, x, epi);
}

// Stop test and beta (CGSolver::solve :439-449; CgGpu::solve, src/gpu/CgGpu.cpp:
// 199-205, with <= and the relative drop).  Thread 0 of the last CTA.
__device__ __forceinline__ void finish_iteration(SolveScalars *s, double rr, double rzNew, bool have_rz)
{
    s->rr = rr;
    const double rn = sqrt(rr);
    const double last = rn / s->bnorm;
    s->last = last;
    s->rnorm = rn;
    const bool stop = s->cggpu ? (last <= s->tol || (s->drop_tol > 0.0 && rn <= s->drop_tol)) : last < s->tol;
    if (stop) {
        s->result = s->iter + 1;
        s->converged = 1;
        s->done = 1;
        return;
    }
    if (have_rz) {
        s->beta = rzNew / s->rz;
        s->rz = rzNew;
        s->iter += 1;
        if (s->iter >= s->max_iter) {
            s->result = s->max_iter;
            s->done = 1;
        }
    }
}

// K2 (Jacobi): x += alpha p, r -= alpha Ap, z = invD r, ||r||^2, r.z.  z is
// stored so K3 does not spend an FP64 multiply recomputing it (same bytes:
// K3 reads z instead of r and invD).
__global__ void __launch_bounds__(kBlock) k_update_jacobi(int64_t n, const double *__restrict__ p,
                                                          const double *__restrict__ Ap,
                                                          const double *__restrict__ invD, double *__restrict__ x,
                                                          double *__restrict__ r, double *__restrict__ z,
                                                          double *partials, SolveScalars *s)
{
    if (ld_done(s))
        return;
    const double alpha = __ldcg(&s->alpha);
    double acc[2] = {0.0, 0.0};
    const int64_t tid = blockIdx.x * (int64_t)blockDim.x + threadIdx.x, stride = (int64_t)gridDim.x * blockDim.x;
    const int64_t n2 = n >> 1;
    for (int64_t i = tid; i < n2; i += stride) {
        const double2 pp = reinterpret_cast<const double2 *>(p)[i];
        const double2 qq = reinterpret_cast<const double2 *>(Ap)[i];
        const double2 id = reinterpret_cast<const double2 *>(invD)[i];
        double2 xx = reinterpret_cast<double2 *>(x)[i];
        double2 rv = reinterpret_cast<double2 *>(r)[i];
        xx.x += alpha * pp.x;
        xx.y += alpha * pp.y;
        rv.x += -alpha * qq.x;
        rv.y += -alpha * qq.y;
        const double2 zz = make_double2(id.x * rv.x, id.y * rv.y);
        reinterpret_cast<double2 *>(x)[i] = xx;
        reinterpret_cast<double2 *>(r)[i] = rv;
        reinterpret_cast<double2 *>(z)[i] = zz;
        acc[0] += rv.x * rv.x + rv.y * rv.y;
        acc[1] += rv.x * zz.x + rv.y * zz.y;
    }
    if ((n & 1) && tid == 0) {
        const int64_t i = n - 1;
        x[i] += alpha * p[i];
        const double ri = r[i] + -alpha * Ap[i];
        const double zi = invD[i] * ri;
        r[i] = ri;
        z[i] = zi;
        acc[0] += ri * ri;
        acc[1] += ri * zi;
    }
    if (grid_sum_last<2>(acc, partials, &s->counter[2]) && threadIdx.x == 0)
        finish_iteration(s, acc[0], acc[1], true);
}

// K3: p = z + beta p (Jacobi and ILU0 alike).
__global__ void __launch_bounds__(kBlock) k_pupdate(int64_t n, const double *__restrict__ z, double *__restrict__ p,
                                                    const SolveScalars *s)
{
    if (ld_done(s))
        return;
    const double beta = __ldcg(&s->beta);
    const int64_t tid = blockIdx.x * (int64_t)blockDim.x + threadIdx.x, stride = (int64_t)gridDim.x * blockDim.x;
    const int64_t n2 = n >> 1;
    for (int64_t i = tid; i < n2; i += stride) {
        const double2 zz = reinterpret_cast<const double2 *>(z)[i];
        double2 pp = reinterpret_cast<double2 *>(p)[i];
        pp.x = zz.x + beta * pp.x;
        pp.y = zz.y + beta * pp.y;
        reinterpret_cast<double2 *>(p)[i] = pp;
    }
    if ((n & 1) && tid == 0) {
        const int64_t i = n - 1;
        p[i] = z[i] + beta * p[i];
    }
}

// ---------------------------------------------------------------- ILU0 variant kernels
// x = 0, r = b, ||b||^2 -> bnorm (z comes from the triangular solves).
__global__ void __launch_bounds__(kBlock) k_init_plain(int64_t n, const double *__restrict__ b, double *__restrict__ x,
                                                       double *__restrict__ r, double *partials, SolveScalars *s)
{
    double acc[1] = {0.0};
    const int64_t tid = blockIdx.x * (int64_t)blockDim.x + threadIdx.x, stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t i = tid; i < n; i += stride) {
        const double bi = b[i];
        x[i] = 0.0;
        r[i] = bi;
        acc[0] += bi * bi;
    }
    if (grid_sum_last<1>(acc, partials, &s->counter[0]) && threadIdx.x == 0) {
        s->bnorm = std_max(sqrt(acc[0]), 1e-30);
        s->iter = 0;
        s->status = SIMALL_OK;
        if (s->max_iter <= 0) {
            s->done = 1;
            s->result = s->max_iter;
        } else {
            s->done = 0;
            s->result = 0;
        }
    }
}

// p = z, rz = r.z
__global__ void __launch_bounds__(kBlock) k_init_p_rz(int64_t n, const double *__restrict__ r,
                                                      const double *__restrict__ z, double *__restrict__ p,
                                                      double *partials, SolveScalars *s)
{
    double acc[1] = {0.0};
    const int64_t tid = blockIdx.x * (int64_t)blockDim.x + threadIdx.x, stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t i = tid; i < n; i += stride) {
        const double zi = z[i];
        p[i] = zi;
        acc[0] += r[i] * zi;
    }
    if (grid_sum_last<1>(acc, partials, &s->counter[3]) && threadIdx.x == 0)
        s->rz = acc[0];
}

// K2a: x += alpha p, r -= alpha Ap, ||r||^2; stop test.
__global__ void __launch_bounds__(kBlock) k_update_xr(int64_t n, const double *__restrict__ p,
                                                      const double *__restrict__ Ap, double *__restrict__ x,
                                                      double *__restrict__ r, double *partials, SolveScalars *s)
{
    if (ld_done(s))
        return;
    const double alpha = __ldcg(&s->alpha);
    double acc[1] = {0.0};
    const int64_t tid = blockIdx.x * (int64_t)blockDim.x + threadIdx.x, stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t i = tid; i < n; i += stride) {
        x[i] += alpha * p[i];
        const double ri = r[i] + -alpha * Ap[i];
        r[i] = ri;
        acc[0] += ri * ri;
    }
    if (grid_sum_last<1>(acc, partials, &s->counter[2]) && threadIdx.x == 0)
        finish_iteration(s, acc[0], 0.0, false);
}

// K2b: rzNew = r.z; beta; iteration count.
__global__ void __launch_bounds__(kBlock) k_rz_beta(int64_t n, const double *__restrict__ r,
                                                    const double *__restrict__ z, double *partials, SolveScalars *s)
{
    if (ld_done(s))
        return;
    double acc[1] = {0.0};
    const int64_t tid = blockIdx.x * (int64_t)blockDim.x + threadIdx.x, stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t i = tid; i < n; i += stride)
        acc[0] += r[i] * z[i];
    if (grid_sum_last<1>(acc, partials, &s->counter[3]) && threadIdx.x == 0) {
        const double rzNew = acc[0];
        s->beta = rzNew / s->rz;
        s->rz = rzNew;
        s->iter += 1;
        if (s->iter >= s->max_iter) {
            s->result = s->max_iter;
            s->done = 1;
        }
    }
}

// r = b - A x and ||r||^2 (FP64 true residual).
struct ResidualEpi {
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

__global__ void __launch_bounds__(kBlock) k_residual(const int32_t *__restrict__ rowPtr, const int32_t *__restrict__ colIdx,
                                                     const double *__restrict__ val, const int32_t *__restrict__ rb,
                                                     int nRB, const double *__restrict__ x, const double *__restrict__ b,
                                                     double *__restrict__ r, double *partials, unsigned *ticket,
                                                     double *out)
{
    ResidualEpi epi{b, r, 0.0};
    spmv_rowblocks(rowPtr, colIdx, val, rb, nRB, x, epi);
    double v[1] = {epi.acc};
    if (grid_sum_last<1>(v, partials, ticket) && threadIdx.x == 0)
        *out = v[0];
}

// CgGpu semantics before the first iteration (CgGpu::solve, src/gpu/CgGpu.cpp:
// 138-168): r = b - A x0 (the SpMV with the reference's rounding, then -y + b),
// ||b||, ||r_0||; bRef = ||b||, or 1 when b = 0; converged at once when
// ||r_0|| / bRef <= tol (0 iterations); dropTol = ||r_0|| 10^-relativeOrders.
struct InitX0Epi {
    const double *b;
    double *r;
    double rr, bb;
    __device__ __forceinline__ void operator()(int row, double y)
    {
        const double bi = __ldg(b + row);
        const double v = -y + bi;
        r[row] = v;
        rr += v * v;
        bb += bi * bi;
    }
};

__global__ void __launch_bounds__(kBlock) k_init_x0(const int32_t *__restrict__ rowPtr,
                                                    const int32_t *__restrict__ colIdx,
                                                    const double *__restrict__ val, const int32_t *__restrict__ rb,
                                                    int nRB, const double *__restrict__ x,
                                                    const double *__restrict__ b, double *__restrict__ r,
                                                    double *partials, SolveScalars *s)
{
    InitX0Epi epi{b, r, 0.0, 0.0};
    spmv_rowblocks(rowPtr, colIdx, val, rb, nRB, x, epi);
    double v[2] = {epi.rr, epi.bb};
    if (grid_sum_last<2>(v, partials, &s->counter[0]) && threadIdx.x == 0) {
        const double bn = sqrt(v[1]);
        const double rn = sqrt(v[0]);
        s->bnorm = bn > 0.0 ? bn : 1.0;
        s->rr = v[0];
        s->rnorm0 = rn;
        s->rnorm = rn;
        s->last = rn / s->bnorm;
        s->drop_tol = s->drop_factor > 0.0 ? rn * s->drop_factor : 0.0;
        s->iter = 0;
        s->result = 0;
        s->status = SIMALL_OK;
        s->converged = 0;
        if (rn / s->bnorm <= s->tol) {
            s->converged = 1;
            s->done = 1;
        } else if (s->max_iter <= 0) {  // the loop never runs: stats stay zero
            s->rnorm = 0.0;
            s->last = 0.0;
            s->done = 1;
        } else {
            s->done = 0;
        }
    }
}

// z = invD r, p = z, rz = r.z (CgGpu semantics, Jacobi or None: invD = 1).
__global__ void __launch_bounds__(kBlock) k_init_jz(int64_t n, const double *__restrict__ r,
                                                    const double *__restrict__ invD, double *__restrict__ z,
                                                    double *__restrict__ p, double *partials, SolveScalars *s)
{
    double acc[1] = {0.0};
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const double ri = r[i];
        const double zi = invD[i] * ri;
        z[i] = zi;
        p[i] = zi;
        acc[0] += ri * zi;
    }
    if (grid_sum_last<1>(acc, partials, &s->counter[3]) && threadIdx.x == 0)
        s->rz = acc[0];
}

__global__ void __launch_bounds__(kBlock) k_fill(int64_t n, double *__restrict__ v, double value)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        v[i] = value;
}

// gpu::ilu0_factor_inplace's verdict (src/gpu/GpuKernels.cpp:345-401) read off a
// finished ILU(0) factor: a missing diagonal, or a zero U_ii of a row i >= 1,
// or a zero U_00 that a later row eliminates against.  Up to the first such
// pivot the two factorisations perform the same operations, so the verdicts
// agree.
__global__ void __launch_bounds__(kBlock) k_cggpu_pivot_check(int64_t n, const int32_t *__restrict__ rowPtr,
                                                              const int32_t *__restrict__ colIdx,
                                                              const int32_t *__restrict__ diagPtr,
                                                              const double *__restrict__ lu, int *flag)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const int d = diagPtr[i];
        if (d < 0 || (i > 0 && lu[d] == 0.0))
            atomicOr(flag, 1);
        const int d0 = diagPtr[0];
        if (i > 0 && d0 >= 0 && rowPtr[i] < rowPtr[i + 1] && colIdx[rowPtr[i]] == 0 && lu[d0] == 0.0)
            atomicOr(flag, 1);
    }
}

int grid_for(simall_context *ctx, int64_t n)
{
    const int64_t g = (n + kBlock - 1) / kBlock;
    const int64_t cap = grid_size_streaming(ctx);
    return static_cast<int>(g < 1 ? 1 : (g < cap ? g : cap));
}

int spmv_grid(simall_context *ctx, int nRB)
{
    const int cap = grid_size_streaming(ctx);
    return nRB < 1 ? 1 : (nRB < cap ? nRB : cap);
}

int check_device_values(simall_solver *s)
{
    simall_context *ctx = s->ctx;
    SIMALL_CUDA_TRY(ctx, s->flag.alloc(1));
    SIMALL_CUDA_TRY(ctx, cudaMemsetAsync(s->flag.p, 0, sizeof(int), ctx->stream));
    k_check_finite<<<grid_for(ctx, s->nnz), kBlock, 0, ctx->stream>>>(s->nnz, s->values, s->flag.p);
    SIMALL_LAUNCH_CHECK(ctx);
    int h = 0;
    SIMALL_CUDA_TRY(ctx, cudaMemcpyAsync(&h, s->flag.p, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    SIMALL_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
    if (h)
        return fail(ctx, SIMALL_ERR_NON_FINITE, "matrix values contain NaN or Inf");
    return SIMALL_OK;
}

void drop_graphs(simall_solver *s);

// Preconditioner / format setup for the current values.
int setup_values(simall_solver *s)
{
    simall_context *ctx = s->ctx;
    if (s->cfg.precision == SIMALL_PRECISION_MIXED)
        return mixed_setup(s);
    const bool cggpu = s->cfg.semantics == SIMALL_SEMANTICS_CGGPU;
    if (cggpu && s->cfg.preconditioner == SIMALL_PRECOND_ILU0) {
        // CgGpu::set_matrix (src/gpu/CgGpu.cpp:60-83): a factor that fails
        // makes the solver Jacobi for good
        const int st = ilu_setup(s);
        if (st)
            return st;
        SIMALL_CUDA_TRY(ctx, s->flag.alloc(1));
        SIMALL_CUDA_TRY(ctx, cudaMemsetAsync(s->flag.p, 0, sizeof(int), ctx->stream));
        k_cggpu_pivot_check<<<grid_for(ctx, s->n), kBlock, 0, ctx->stream>>>(s->n, s->rowPtr, s->colIdx,
                                                                             s->ilu->diagPtr.p, s->ilu->lu.p,
                                                                             s->flag.p);
        SIMALL_LAUNCH_CHECK(ctx);
        int h = 0;
        SIMALL_CUDA_TRY(ctx, cudaMemcpyAsync(&h, s->flag.p, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
        SIMALL_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
        if (!h)
            return SIMALL_OK;
        s->cfg.preconditioner = SIMALL_PRECOND_JACOBI;
        drop_graphs(s);  // the captured iterations hold the ILU(0) sweeps
    }
    if (cggpu && s->cfg.preconditioner == SIMALL_PRECOND_NONE) {  // z = r
        SIMALL_CUDA_TRY(ctx, s->invDiag.alloc(static_cast<size_t>(s->n)));
        k_fill<<<grid_for(ctx, s->n), kBlock, 0, ctx->stream>>>(s->n, s->invDiag.p, 1.0);
        SIMALL_LAUNCH_CHECK(ctx);
        return SIMALL_OK;
    }
    if (s->cfg.preconditioner == SIMALL_PRECOND_ILU0)
        return ilu_setup(s);
    if (s->cfg.preconditioner == SIMALL_PRECOND_AMG) {
        // a new hierarchy may differ in levels and sizes: the captured
        // iteration graphs hold its buffers and launch shapes
        drop_graphs(s);
        return ilu_setup(s);
    }
    SIMALL_CUDA_TRY(ctx, s->invDiag.alloc(static_cast<size_t>(s->n)));
    k_jacobi_setup<<<grid_for(ctx, s->n), kBlock, 0, ctx->stream>>>(s->n, s->rowPtr, s->colIdx, s->values,
                                                                     s->invDiag.p);
    SIMALL_LAUNCH_CHECK(ctx);
    // SSOR's inverse diagonal is Jacobi's (SsorPreconditioner::setup, LinearSolvers.cpp:168-186)
    if (s->cfg.preconditioner == SIMALL_PRECOND_SSOR)
        return ilu_setup(s);
    return SIMALL_OK;
}

int alloc_vectors(simall_solver *s)
{
    simall_context *ctx = s->ctx;
    const size_t n = static_cast<size_t>(s->n) + 2;  // +2 keeps double2 tails in bounds
    SIMALL_CUDA_TRY(ctx, s->x.alloc(n));
    SIMALL_CUDA_TRY(ctx, s->r.alloc(n));
    SIMALL_CUDA_TRY(ctx, s->p.alloc(n));
    SIMALL_CUDA_TRY(ctx, s->Ap.alloc(n));
    SIMALL_CUDA_TRY(ctx, s->b.alloc(n));
    SIMALL_CUDA_TRY(ctx, s->z.alloc(n));
    SIMALL_CUDA_TRY(ctx, s->partials.alloc(static_cast<size_t>(kMaxReduce) * grid_size_streaming(ctx)));
    if (!s->scal.p) {
        SIMALL_CUDA_TRY(ctx, s->scal.alloc(1));
        SIMALL_CUDA_TRY(ctx, cudaMemsetAsync(s->scal.p, 0, sizeof(SolveScalars), ctx->stream));
    }
    if (!s->h_scal)
        SIMALL_CUDA_TRY(ctx, cudaMallocHost(reinterpret_cast<void **>(&s->h_scal), sizeof(SolveScalars)));
    return SIMALL_OK;
}

void drop_graphs(simall_solver *s)
{
    krylov_drop_graphs(s);
    for (auto &g : s->graphs)
        if (g.exec)
            cudaGraphExecDestroy(g.exec);
    s->graphs.clear();
}

// K1: one thread per row when the rows are short on average (no staging
// barrier), else the staged row-blocks.
int enqueue_spmv_pap(simall_solver *s)
{
    simall_context *ctx = s->ctx;
    if (spmv_direct(s)) {
        k_spmv_pap_rows<<<resident_grid(ctx, reinterpret_cast<const void *>(k_spmv_pap_rows), s->n), kBlock, 0,
                          ctx->stream>>>(s->rowPtr, s->colIdx, s->values, s->n, s->p.p, s->Ap.p, s->partials.p,
                                         s->scal.p);
    } else {
        const int64_t rbThreads = static_cast<int64_t>(s->nRowBlocks) * kBlock;
        k_spmv_pap<<<resident_grid(ctx, reinterpret_cast<const void *>(k_spmv_pap), rbThreads), kBlock, 0,
                     ctx->stream>>>(s->rowPtr, s->colIdx, s->values, s->rowBlocks.p, s->nRowBlocks, s->p.p, s->Ap.p,
                                    s->partials.p, s->scal.p);
    }
    SIMALL_LAUNCH_CHECK(ctx);
    return SIMALL_OK;
}

// Enqueue one FP64 iteration (Jacobi or ILU0).
int enqueue_iteration(simall_solver *s)
{
    simall_context *ctx = s->ctx;
    const int64_t n = s->n;
    int e0 = enqueue_spmv_pap(s);
    if (e0)
        return e0;
    if (sweep_preconditioner(s->cfg.preconditioner)) {
        k_update_xr<<<resident_grid(ctx, reinterpret_cast<const void *>(k_update_xr), n), kBlock, 0, ctx->stream>>>(
            n, s->p.p, s->Ap.p, s->x.p, s->r.p, s->partials.p, s->scal.p);
        SIMALL_LAUNCH_CHECK(ctx);
        int st = ilu_apply(s, s->r.p, s->z.p);
        if (st)
            return st;
        k_rz_beta<<<resident_grid(ctx, reinterpret_cast<const void *>(k_rz_beta), n), kBlock, 0, ctx->stream>>>(
            n, s->r.p, s->z.p, s->partials.p, s->scal.p);
        SIMALL_LAUNCH_CHECK(ctx);
    } else {
        k_update_jacobi<<<resident_grid(ctx, reinterpret_cast<const void *>(k_update_jacobi), n), kBlock, 0,
                          ctx->stream>>>(n, s->p.p, s->Ap.p, s->invDiag.p, s->x.p, s->r.p, s->z.p, s->partials.p,
                                         s->scal.p);
        SIMALL_LAUNCH_CHECK(ctx);
    }
    k_pupdate<<<resident_grid(ctx, reinterpret_cast<const void *>(k_pupdate), n), kBlock, 0, ctx->stream>>>(
        n, s->z.p, s->p.p, s->scal.p);
    SIMALL_LAUNCH_CHECK(ctx);
    return SIMALL_OK;
}

// Kernels one FP64 iteration launches (for the launch counter of graph replays).
int64_t kernels_per_iteration(const simall_solver *s)
{
    if (sweep_preconditioner(s->cfg.preconditioner) && (s->ilu || s->amg))
        return 4 + ilu_apply_launches(s);  // SpMV, x/r update, r.z/beta, direction + the sweeps
    return 3;
}

// A chunk of `len` iterations, captured once into a graph and replayed.
int run_chunk(simall_solver *s, int len)
{
    simall_context *ctx = s->ctx;
    for (auto &g : s->graphs)
        if (g.len == len) {
            SIMALL_CUDA_TRY(ctx, cudaGraphLaunch(g.exec, ctx->stream));
            ctx->launches.fetch_add(static_cast<int64_t>(len) * kernels_per_iteration(s), std::memory_order_relaxed);
            return SIMALL_OK;
        }
    cudaGraph_t graph = nullptr;
    SIMALL_CUDA_TRY(ctx, cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
    int st = SIMALL_OK;
    for (int i = 0; i < len && st == SIMALL_OK; ++i)
        st = enqueue_iteration(s);
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

int fp64_solve(simall_solver *s, simall_solver_stats *st)
{
    simall_context *ctx = s->ctx;
    const int g = grid_for(ctx, s->n);
    SolveScalars init{};
    init.tol = s->cfg.tolerance;
    init.max_iter = s->cfg.max_iterations;
    // only the control fields are set from the host; counters stay zero
    SIMALL_CUDA_TRY(ctx, cudaMemcpyAsync(&s->scal.p->tol, &init.tol, sizeof(double), cudaMemcpyHostToDevice,
                                         ctx->stream));
    SIMALL_CUDA_TRY(ctx, cudaMemcpyAsync(&s->scal.p->max_iter, &init.max_iter, sizeof(int), cudaMemcpyHostToDevice,
                                         ctx->stream));
    const bool cggpu = s->cfg.semantics == SIMALL_SEMANTICS_CGGPU;
    init.cggpu = cggpu ? 1 : 0;
    init.drop_factor = cggpu && s->cfg.relative_orders > 0.0 ? std::pow(10.0, -s->cfg.relative_orders) : 0.0;
    SIMALL_CUDA_TRY(ctx, cudaMemcpyAsync(&s->scal.p->cggpu, &init.cggpu, sizeof(int), cudaMemcpyHostToDevice,
                                         ctx->stream));
    SIMALL_CUDA_TRY(ctx, cudaMemcpyAsync(&s->scal.p->drop_factor, &init.drop_factor, sizeof(double),
                                         cudaMemcpyHostToDevice, ctx->stream));
    if (s->cfg.preconditioner == SIMALL_PRECOND_JACOBI && s->cfg.check_interval <= 0 &&
        s->cfg.engine == SIMALL_ENGINE_AUTO && !cggpu) {
        int cst = SIMALL_OK;
        if (cluster_fp64_solve(s, &cst))
            return cst;
    }
    if (cggpu) {
        // x holds x0 (copied in by the solve call)
        k_init_x0<<<resident_grid(ctx, reinterpret_cast<const void *>(k_init_x0), spmv_items(s)), kBlock, 0,
                    ctx->stream>>>(s->rowPtr, s->colIdx, s->values, s->rowBlocks.p, spmv_schedule(s), s->x.p,
                                   s->b.p, s->r.p, s->partials.p, s->scal.p);
        SIMALL_LAUNCH_CHECK(ctx);
        if (sweep_preconditioner(s->cfg.preconditioner)) {
            int e = ilu_apply(s, s->r.p, s->z.p);
            if (e)
                return e;
            k_init_p_rz<<<g, kBlock, 0, ctx->stream>>>(s->n, s->r.p, s->z.p, s->p.p, s->partials.p, s->scal.p);
        } else {
            k_init_jz<<<g, kBlock, 0, ctx->stream>>>(s->n, s->r.p, s->invDiag.p, s->z.p, s->p.p, s->partials.p,
                                                     s->scal.p);
        }
        SIMALL_LAUNCH_CHECK(ctx);
    } else if (sweep_preconditioner(s->cfg.preconditioner)) {
        k_init_plain<<<g, kBlock, 0, ctx->stream>>>(s->n, s->b.p, s->x.p, s->r.p, s->partials.p, s->scal.p);
        SIMALL_LAUNCH_CHECK(ctx);
        int e = ilu_apply(s, s->r.p, s->z.p);
        if (e)
            return e;
        k_init_p_rz<<<g, kBlock, 0, ctx->stream>>>(s->n, s->r.p, s->z.p, s->p.p, s->partials.p, s->scal.p);
        SIMALL_LAUNCH_CHECK(ctx);
    } else {
        k_init_jacobi<<<g, kBlock, 0, ctx->stream>>>(s->n, s->b.p, s->invDiag.p, s->x.p, s->r.p, s->p.p,
                                                     s->partials.p, s->scal.p);
        SIMALL_LAUNCH_CHECK(ctx);
    }
    int done_iters = 0;
    const int max_chunk = 64;
    int chunk = s->cfg.check_interval > 0 ? s->cfg.check_interval : 16;
    double prev_last = -1.0;
    int prev_iter = 0;
    for (;;) {
        const int remaining = s->cfg.max_iterations - done_iters;
        int len = chunk < remaining ? chunk : remaining;
        if (len < 1)
            len = 1;
        // a few distinct lengths only, so the captured graphs are reused
        if (s->cfg.check_interval <= 0)
            len = len <= 4 ? len : len <= 8 ? 8 : len <= 16 ? 16 : len <= 32 ? 32 : 64;
        int e = run_chunk(s, len);
        if (e)
            return e;
        done_iters += len;
        e = solver_fetch_scalars(s);
        if (e)
            return e;
        if (s->h_scal->done)
            break;
        if (done_iters >= s->cfg.max_iterations + 1)
            return fail(ctx, SIMALL_ERR_CUDA, "solver did not raise its stop flag");
        if (s->cfg.check_interval <= 0) {
            // predict the remaining iterations from the observed decay rate
            const double last = s->h_scal->last;
            const int it = s->h_scal->iter;
            int next = max_chunk;
            if (prev_last > 0.0 && last > 0.0 && last < prev_last && it > prev_iter) {
                const double rate = std::log(last / prev_last) / (it - prev_iter);
                const double need = std::log(s->cfg.tolerance / last) / rate;
                next = need < 4 ? 4 : (need > max_chunk ? max_chunk : static_cast<int>(need) + 1);
            }
            prev_last = last;
            prev_iter = it;
            chunk = next;
        }
    }
    (void)st;
    return SIMALL_OK;
}

}  // namespace

int solver_host_pattern(simall_solver *s)
{
    if (s->h_pattern_valid)
        return SIMALL_OK;
    simall_context *ctx = s->ctx;
    s->h_rowPtr.resize(static_cast<size_t>(s->n) + 1);
    s->h_colIdx.resize(static_cast<size_t>(s->nnz));
    SIMALL_CUDA_TRY(ctx, cudaMemcpyAsync(s->h_rowPtr.data(), s->own_rowPtr.p, (s->n + 1) * sizeof(int32_t),
                                         cudaMemcpyDeviceToHost, ctx->stream));
    SIMALL_CUDA_TRY(ctx, cudaMemcpyAsync(s->h_colIdx.data(), s->own_colIdx.p, s->nnz * sizeof(int32_t),
                                         cudaMemcpyDeviceToHost, ctx->stream));
    SIMALL_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
    s->h_pattern_valid = true;
    return SIMALL_OK;
}

int solver_fetch_scalars(simall_solver *s)
{
    simall_context *ctx = s->ctx;
    SIMALL_CUDA_TRY(ctx, cudaMemcpyAsync(s->h_scal, s->scal.p, sizeof(SolveScalars), cudaMemcpyDeviceToHost,
                                         ctx->stream));
    SIMALL_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
    return SIMALL_OK;
}

int solver_true_residual(simall_solver *s, const double *x, const double *b, double *r, double *rr)
{
    simall_context *ctx = s->ctx;
    k_residual<<<spmv_direct(s) ? grid_for(ctx, s->n) : spmv_grid(ctx, s->nRowBlocks), kBlock, 0, ctx->stream>>>(
        s->rowPtr, s->colIdx, s->values, s->rowBlocks.p, spmv_schedule(s), x, b, r, s->partials.p,
        &s->scal.p->counter[4], reinterpret_cast<double *>(&s->scal.p->rr));
    SIMALL_LAUNCH_CHECK(ctx);
    if (rr) {
        SIMALL_CUDA_TRY(ctx, cudaMemcpyAsync(rr, &s->scal.p->rr, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
        SIMALL_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
    }
    return SIMALL_OK;
}

}  // namespace simall

using namespace simall;

extern "C" {

void simall_solver_config_default(simall_solver_config *cfg)
{
    if (!cfg)
        return;
    cfg->preconditioner = SIMALL_PRECOND_JACOBI;
    cfg->tolerance = 1.0e-8;
    cfg->max_iterations = 1000;
    cfg->precision = SIMALL_PRECISION_FP64;
    cfg->reliable_delta = 0.1;
    cfg->check_interval = 0;
    cfg->engine = SIMALL_ENGINE_AUTO;
    cfg->kind = SIMALL_SOLVER_CG;
    cfg->restart = 30;
    cfg->semantics = SIMALL_SEMANTICS_CGSOLVER;
    cfg->relative_orders = 0.0;
}

int simall_solver_create(simall_context *ctx, const simall_solver_config *cfg, simall_solver **out)
{
    if (!ctx || !out)
        return SIMALL_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    simall_solver_config c;
    simall_solver_config_default(&c);
    if (cfg)
        c = *cfg;
    if (c.semantics != SIMALL_SEMANTICS_CGSOLVER && c.semantics != SIMALL_SEMANTICS_CGGPU)
        return fail(ctx, SIMALL_ERR_INVALID_ARGUMENT, "semantics %d", c.semantics);
    if (c.semantics == SIMALL_SEMANTICS_CGGPU) {
        if (c.kind != SIMALL_SOLVER_CG || c.precision != SIMALL_PRECISION_FP64 ||
            (c.preconditioner != SIMALL_PRECOND_JACOBI && c.preconditioner != SIMALL_PRECOND_ILU0 &&
             c.preconditioner != SIMALL_PRECOND_NONE))
            return fail(ctx, SIMALL_ERR_UNSUPPORTED, "CgGpu semantics: FP64 CG with Jacobi, ILU0 or None");
        if (!(c.relative_orders >= 0.0))
            return fail(ctx, SIMALL_ERR_INVALID_ARGUMENT, "relative_orders must be >= 0");
    } else if (c.preconditioner == SIMALL_PRECOND_NONE) {
        c.preconditioner = SIMALL_PRECOND_JACOBI;  // make_preconditioner (LinearSolvers.cpp:240-254)
    }
    if (c.preconditioner != SIMALL_PRECOND_JACOBI && c.preconditioner != SIMALL_PRECOND_NONE &&
        !sweep_preconditioner(c.preconditioner))
        return fail(ctx, SIMALL_ERR_UNSUPPORTED, "preconditioner %d is not on the pressure path", c.preconditioner);
    if (c.precision != SIMALL_PRECISION_FP64 && c.precision != SIMALL_PRECISION_MIXED)
        return fail(ctx, SIMALL_ERR_INVALID_ARGUMENT, "precision %d", c.precision);
    if (c.precision == SIMALL_PRECISION_MIXED && c.preconditioner != SIMALL_PRECOND_JACOBI)
        return fail(ctx, SIMALL_ERR_UNSUPPORTED, "mixed precision runs with the Jacobi preconditioner");
    if (c.kind != SIMALL_SOLVER_CG && c.kind != SIMALL_SOLVER_GMRES && c.kind != SIMALL_SOLVER_BICGSTAB &&
        c.kind != SIMALL_SOLVER_TFQMR)
        return fail(ctx, SIMALL_ERR_UNSUPPORTED, "solver kind %d is not on this path", c.kind);
    if (c.kind != SIMALL_SOLVER_CG && c.precision != SIMALL_PRECISION_FP64)
        return fail(ctx, SIMALL_ERR_UNSUPPORTED, "GMRES, BiCGSTAB and TFQMR run in FP64");
    if (c.kind == SIMALL_SOLVER_GMRES && c.restart < 1)
        c.restart = 1;  // std::max(1, restart), LinearSolvers.cpp:273
    if (!(c.tolerance >= 0.0) || c.reliable_delta <= 0.0 || c.reliable_delta >= 1.0)
        return fail(ctx, SIMALL_ERR_INVALID_ARGUMENT, "tolerance / reliable_delta out of range");
    auto *s = new (std::nothrow) simall_solver;
    if (!s)
        return SIMALL_ERR_OUT_OF_MEMORY;
    s->ctx = ctx;
    s->cfg = c;
    *out = s;
    return SIMALL_OK;
}

int simall_solver_destroy(simall_solver *s)
{
    if (!s)
        return SIMALL_ERR_INVALID_ARGUMENT;
    cudaStreamSynchronize(s->ctx->stream);
    drop_graphs(s);
    ilu_free(s);
    mixed_free(s);
    krylov_free(s);
    if (s->h_scal)
        cudaFreeHost(s->h_scal);
    delete s;
    return SIMALL_OK;
}

int simall_solver_set_matrix(simall_solver *s, int64_t n, int64_t nnz, const int32_t *rowPtr, const int32_t *colIdx,
                             const double *values, int mem)
{
    if (!s)
        return SIMALL_ERR_INVALID_ARGUMENT;
    simall_context *ctx = s->ctx;
    SIMALL_CUDA_TRY(ctx, cudaSetDevice(ctx->device));
    s->ready = false;
    if (n <= 0 || nnz <= 0 || !rowPtr || !colIdx || !values)
        return fail(ctx, SIMALL_ERR_INVALID_ARGUMENT, "set_matrix: empty matrix or null array");
    if (n > INT32_MAX - 1 || nnz > INT32_MAX)
        return fail(ctx, SIMALL_ERR_INVALID_ARGUMENT, "set_matrix: sizes exceed int32 indexing");
    if (mem != SIMALL_MEM_HOST && mem != SIMALL_MEM_DEVICE)
        return fail(ctx, SIMALL_ERR_INVALID_ARGUMENT, "set_matrix: bad memory kind %d", mem);
    cudaStream_t st = ctx->stream;
    const cudaMemcpyKind kind = mem == SIMALL_MEM_HOST ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice;
    if (mem == SIMALL_MEM_HOST && (rowPtr[0] != 0 || rowPtr[n] != nnz))
        return fail(ctx, SIMALL_ERR_SIZE_MISMATCH, "CSR: rowPtr[0]=%d rowPtr[n]=%d, nnz=%lld", rowPtr[0], rowPtr[n],
                    static_cast<long long>(nnz));
    // the new pattern goes to the staging pair, the values to their home
    SIMALL_CUDA_TRY(ctx, s->new_rowPtr.alloc(n + 1));
    SIMALL_CUDA_TRY(ctx, s->new_colIdx.alloc(nnz));
    SIMALL_CUDA_TRY(ctx, cudaMemcpyAsync(s->new_rowPtr.p, rowPtr, (n + 1) * sizeof(int32_t), kind, st));
    SIMALL_CUDA_TRY(ctx, cudaMemcpyAsync(s->new_colIdx.p, colIdx, nnz * sizeof(int32_t), kind, st));
    const double *vals = values;
    if (mem == SIMALL_MEM_HOST) {
        SIMALL_CUDA_TRY(ctx, s->own_values.alloc(nnz));
        SIMALL_CUDA_TRY(ctx, cudaMemcpyAsync(s->own_values.p, values, nnz * sizeof(double), kind, st));
        vals = s->own_values.p;
    }
    // validation, comparison with the current pattern and the row-block test
    // run on the device; the host reads one flag word
    SIMALL_CUDA_TRY(ctx, s->flag.alloc(1));
    unsigned *flags = reinterpret_cast<unsigned *>(s->flag.p);
    SIMALL_CUDA_TRY(ctx, cudaMemsetAsync(flags, 0, sizeof(unsigned), st));
    const int g = grid_for(ctx, n);
    k_validate_csr<<<g, kBlock, 0, st>>>(n, nnz, s->new_rowPtr.p, s->new_colIdx.p, vals, flags);
    SIMALL_LAUNCH_CHECK(ctx);
    const bool comparable = s->have_pattern && n == s->n && nnz == s->nnz;
    if (comparable) {
        k_compare_pattern<<<grid_for(ctx, nnz), kBlock, 0, st>>>(n, nnz, s->new_rowPtr.p, s->new_colIdx.p,
                                                                 s->own_rowPtr.p, s->own_colIdx.p, flags);
        SIMALL_LAUNCH_CHECK(ctx);
    }
    const int64_t nb = (n + kSpmvRows - 1) / kSpmvRows;
    k_rowblock_fit<<<grid_for(ctx, nb), kBlock, 0, st>>>(n, nb, s->new_rowPtr.p, flags);
    SIMALL_LAUNCH_CHECK(ctx);
    unsigned h = 0;
    SIMALL_CUDA_TRY(ctx, cudaMemcpyAsync(&h, flags, sizeof(unsigned), cudaMemcpyDeviceToHost, st));
    SIMALL_CUDA_TRY(ctx, cudaStreamSynchronize(st));
    if (h & kBadEnds)
        return fail(ctx, SIMALL_ERR_SIZE_MISMATCH, "CSR: rowPtr[0] != 0 or rowPtr[n] != nnz (%lld)",
                    static_cast<long long>(nnz));
    if (h & kBadRowPtr)
        return fail(ctx, SIMALL_ERR_UNSORTED_CSR, "CSR: rowPtr decreases or leaves [0, nnz]");
    if (h & kBadRange)
        return fail(ctx, SIMALL_ERR_INDEX_RANGE, "CSR: a column index is outside [0, n)");
    if (h & kUnsorted)
        return fail(ctx, SIMALL_ERR_UNSORTED_CSR, "CSR: columns of a row are not strictly ascending");
    if (h & kNoDiag)
        return fail(ctx, SIMALL_ERR_MISSING_DIAGONAL, "CSR: a row has no diagonal entry");
    if (h & kNonFinite)
        return fail(ctx, SIMALL_ERR_NON_FINITE, "matrix values contain NaN or Inf");
    const bool pattern_changed = !(comparable && !(h & kPatternDiff));
    if (pattern_changed) {
        std::swap(s->own_rowPtr.p, s->new_rowPtr.p);
        std::swap(s->own_rowPtr.n, s->new_rowPtr.n);
        std::swap(s->own_colIdx.p, s->new_colIdx.p);
        std::swap(s->own_colIdx.n, s->new_colIdx.n);
        s->have_pattern = true;
        s->h_pattern_valid = false;
        drop_graphs(s);
        if (s->ilu)
            s->ilu->analysed = false;
        mixed_invalidate_pattern(s);
        s->n = n;
        s->nnz = nnz;
        s->rowPtr = s->own_rowPtr.p;
        s->colIdx = s->own_colIdx.p;
        if (!(h & kBlockTooBig)) {
            s->nRowBlocks = static_cast<int>(nb);
            SIMALL_CUDA_TRY(ctx, s->rowBlocks.alloc(nb + 1));
            k_rowblock_fill<<<grid_for(ctx, nb + 1), kBlock, 0, st>>>(n, nb, s->rowBlocks.p);
            SIMALL_LAUNCH_CHECK(ctx);
        } else {
            int e = solver_host_pattern(s);
            if (e)
                return e;
            std::vector<int32_t> rb = make_row_blocks(n, s->h_rowPtr.data());
            s->nRowBlocks = static_cast<int>(rb.size()) - 1;
            SIMALL_CUDA_TRY(ctx, s->rowBlocks.alloc(rb.size()));
            SIMALL_CUDA_TRY(ctx, cudaMemcpyAsync(s->rowBlocks.p, rb.data(), rb.size() * sizeof(int32_t),
                                                 cudaMemcpyHostToDevice, st));
            SIMALL_CUDA_TRY(ctx, cudaStreamSynchronize(st));
        }
    }
    if (vals != s->values)
        drop_graphs(s);  // captured graphs embed the values pointer
    s->values = vals;
    s->solved = false;
    int e = alloc_vectors(s);
    if (e)
        return e;
    e = setup_values(s);
    if (e)
        return e;
    SIMALL_CUDA_TRY(ctx, cudaStreamSynchronize(st));
    s->ready = true;
    return SIMALL_OK;
}

int simall_solver_update_values(simall_solver *s, const double *values, int mem)
{
    if (!s || !values)
        return SIMALL_ERR_INVALID_ARGUMENT;
    simall_context *ctx = s->ctx;
    if (!s->ready)
        return fail(ctx, SIMALL_ERR_INVALID_ARGUMENT, "update_values before set_matrix");
    SIMALL_CUDA_TRY(ctx, cudaSetDevice(ctx->device));
    if (mem == SIMALL_MEM_HOST) {
        if (s->values != s->own_values.p) {
            SIMALL_CUDA_TRY(ctx, s->own_values.alloc(s->nnz));
            s->values = s->own_values.p;
            drop_graphs(s);
        }
        SIMALL_CUDA_TRY(ctx, cudaMemcpyAsync(s->own_values.p, values, s->nnz * sizeof(double), cudaMemcpyHostToDevice,
                                             ctx->stream));
        int st = check_device_values(s);
        if (st)
            return st;
    } else {
        if (values != s->values)
            drop_graphs(s);
        s->values = values;
        int st = check_device_values(s);
        if (st)
            return st;
    }
    int st = setup_values(s);
    if (st)
        return st;
    return SIMALL_OK;
}

int simall_solver_solve(simall_solver *s, const double *b, double *x, int mem, simall_solver_stats *stats)
{
    return simall::solver_solve_impl(s, b, mem, x, mem, stats);
}

}  // extern "C"

int simall::solver_solve_impl(simall_solver *s, const double *b, int bmem, double *x, int xmem,
                              simall_solver_stats *stats)
{
    if (!s || !b || !x)
        return SIMALL_ERR_INVALID_ARGUMENT;
    simall_context *ctx = s->ctx;
    if (!s->ready)
        return fail(ctx, SIMALL_ERR_INVALID_ARGUMENT, "solve before set_matrix");
    if ((bmem != SIMALL_MEM_HOST && bmem != SIMALL_MEM_DEVICE) || (xmem != SIMALL_MEM_HOST && xmem != SIMALL_MEM_DEVICE))
        return fail(ctx, SIMALL_ERR_INVALID_ARGUMENT, "solve: bad memory kind");
    SIMALL_CUDA_TRY(ctx, cudaSetDevice(ctx->device));
    const auto t0 = std::chrono::steady_clock::now();
    const size_t bytes = static_cast<size_t>(s->n) * sizeof(double);
    SIMALL_CUDA_TRY(ctx, cudaMemcpyAsync(s->b.p, b, bytes,
                                         bmem == SIMALL_MEM_HOST ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice,
                                         ctx->stream));
    {
        SIMALL_CUDA_TRY(ctx, s->flag.alloc(1));
        SIMALL_CUDA_TRY(ctx, cudaMemsetAsync(s->flag.p, 0, sizeof(int), ctx->stream));
        k_check_finite<<<grid_for(ctx, s->n), kBlock, 0, ctx->stream>>>(s->n, s->b.p, s->flag.p);
        SIMALL_LAUNCH_CHECK(ctx);
        int h = 0;
        SIMALL_CUDA_TRY(ctx, cudaMemcpyAsync(&h, s->flag.p, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
        SIMALL_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
        if (h)
            return fail(ctx, SIMALL_ERR_NON_FINITE, "b contains NaN or Inf");
    }
    if (s->cfg.semantics == SIMALL_SEMANTICS_CGGPU) {
        // x is the initial guess (CgGpu::solve uploads x0, src/gpu/CgGpu.cpp:133-136)
        SIMALL_CUDA_TRY(ctx, cudaMemcpyAsync(s->x.p, x, bytes,
                                             xmem == SIMALL_MEM_HOST ? cudaMemcpyHostToDevice
                                                                     : cudaMemcpyDeviceToDevice,
                                             ctx->stream));
        SIMALL_CUDA_TRY(ctx, cudaMemsetAsync(s->flag.p, 0, sizeof(int), ctx->stream));
        k_check_finite<<<grid_for(ctx, s->n), kBlock, 0, ctx->stream>>>(s->n, s->x.p, s->flag.p);
        SIMALL_LAUNCH_CHECK(ctx);
        int h = 0;
        SIMALL_CUDA_TRY(ctx, cudaMemcpyAsync(&h, s->flag.p, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
        SIMALL_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
        if (h)
            return fail(ctx, SIMALL_ERR_NON_FINITE, "the initial guess x contains NaN or Inf");
    }
    simall_solver_stats local{};
    int st;
    s->engine = 0;
    if (s->cfg.kind != SIMALL_SOLVER_CG)
        st = krylov_solve(s);
    else if (s->cfg.precision == SIMALL_PRECISION_MIXED)
        st = mixed_solve(s, &local);
    else
        st = fp64_solve(s, &local);
    if (!st && sweep_preconditioner(s->cfg.preconditioner))
        st = ilu_check(s);
    if (st)
        return st;
    // FP64 true residual of the returned x (r buffer is free after the loop)
    double rr = 0.0;
    if (s->cfg.precision != SIMALL_PRECISION_MIXED) {
        st = solver_true_residual(s, s->x.p, s->b.p, s->r.p, &rr);
        if (st)
            return st;
    } else {
        rr = s->h_scal->rr;
    }
    if (xmem == SIMALL_MEM_HOST)
        SIMALL_CUDA_TRY(ctx, cudaMemcpyAsync(x, s->x.p, bytes, cudaMemcpyDeviceToHost, ctx->stream));
    else
        SIMALL_CUDA_TRY(ctx, cudaMemcpyAsync(x, s->x.p, bytes, cudaMemcpyDeviceToDevice, ctx->stream));
    SIMALL_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
    const SolveScalars &h = *s->h_scal;
    s->last_residual = h.last;
    s->solved = true;
    if (stats) {
        const bool cggpu = s->cfg.semantics == SIMALL_SEMANTICS_CGGPU;
        stats->iterations = h.result;
        stats->final_residual = h.last;
        stats->converged = cggpu ? h.converged : ((h.last < s->cfg.tolerance) ? 1 : 0);
        stats->status = h.status;
        stats->reliable_updates = h.updates;
        stats->b_norm = h.bnorm;
        stats->true_residual = std::sqrt(rr) / h.bnorm;
        stats->seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        stats->engine = s->engine;
        stats->preconditioner = s->cfg.preconditioner;
        stats->residual_norm = cggpu ? h.rnorm : h.last * h.bnorm;
        stats->initial_residual = cggpu ? h.rnorm0 : h.bnorm;
    }
    return SIMALL_OK;
}

extern "C" {

double simall_solver_last_residual(const simall_solver *s) { return s ? s->last_residual : 0.0; }

int simall_solver_preconditioner(const simall_solver *s, int *preconditioner)
{
    if (!s || !preconditioner)
        return SIMALL_ERR_INVALID_ARGUMENT;
    *preconditioner = s->cfg.preconditioner;
    return SIMALL_OK;
}

int simall_solver_time_kernel(simall_solver *s, int kernel, int reps, double *ms, double *bytes)
{
    if (!s || !ms || reps <= 0)
        return SIMALL_ERR_INVALID_ARGUMENT;
    simall_context *ctx = s->ctx;
    if (!s->ready || !s->solved)
        return fail(ctx, SIMALL_ERR_INVALID_ARGUMENT, "time_kernel needs a matrix and one completed solve");
    const bool mixed = s->cfg.precision == SIMALL_PRECISION_MIXED;
    if ((kernel >= 4 && !mixed) || (kernel >= 1 && kernel <= 3 && (mixed || s->cfg.preconditioner != SIMALL_PRECOND_JACOBI)) ||
        kernel < 0 || kernel > 4)
        return fail(ctx, SIMALL_ERR_INVALID_ARGUMENT, "kernel %d not available for this solver", kernel);
    SIMALL_CUDA_TRY(ctx, cudaSetDevice(ctx->device));
    // keep every kernel doing full work: never converge, never stop
    SolveScalars sc{};
    sc.tol = -1.0;
    sc.max_iter = 0x7fffffff;
    sc.delta = 0.0;
    sc.bnorm = 1.0;
    sc.rz = 1.0;
    sc.sigma0 = 1.0;
    sc.t0 = 1.0;
    sc.rmax = 1.0;
    sc.alpha = 1e-3;
    sc.beta = 0.5;
    // the vectors keep the data of the last solve (p.Ap != 0 keeps K1 running)
    SIMALL_CUDA_TRY(ctx, cudaMemcpyAsync(s->scal.p, &sc, sizeof(sc), cudaMemcpyHostToDevice, ctx->stream));
    const int64_t rbThreads = static_cast<int64_t>(s->nRowBlocks) * kBlock;
    auto rg = [&](const void *fn, int64_t items) { return resident_grid(ctx, fn, items); };
    const double nd = static_cast<double>(s->n), nz = static_cast<double>(s->nnz);
    double b = 0.0;
    auto launch = [&]() -> int {
        switch (kernel) {
        case 0:
            k_spmv_plain<<<rg(reinterpret_cast<const void *>(k_spmv_plain), spmv_items(s)), kBlock, 0,
                           ctx->stream>>>(s->rowPtr, s->colIdx, s->values, s->rowBlocks.p, spmv_schedule(s), s->p.p,
                                          s->Ap.p);
            b = 12.0 * nz + 20.0 * nd + 4.0;
            break;
        case 1: {
            const int e1 = enqueue_spmv_pap(s);
            if (e1)
                return e1;
            b = 12.0 * nz + 20.0 * nd + 4.0;
            break;
        }
        case 2:
            k_update_jacobi<<<rg(reinterpret_cast<const void *>(k_update_jacobi), s->n), kBlock, 0, ctx->stream>>>(
                s->n, s->p.p, s->Ap.p, s->invDiag.p, s->x.p, s->r.p, s->z.p, s->partials.p, s->scal.p);
            b = 64.0 * nd;  // p, Ap, invD, x, r read; x, r, z written
            break;
        case 3:
            k_pupdate<<<rg(reinterpret_cast<const void *>(k_pupdate), s->n), kBlock, 0, ctx->stream>>>(
                s->n, s->z.p, s->p.p, s->scal.p);
            b = 24.0 * nd;  // z, p read; p written
            break;
        default:
            return mixed_enqueue_kernel(s, kernel, &b);
        }
        SIMALL_LAUNCH_CHECK(ctx);
        return SIMALL_OK;
    };
    int st = launch();  // warm-up
    if (st)
        return st;
    cudaEvent_t e0, e1;
    SIMALL_CUDA_TRY(ctx, cudaEventCreate(&e0));
    SIMALL_CUDA_TRY(ctx, cudaEventCreate(&e1));
    SIMALL_CUDA_TRY(ctx, cudaEventRecord(e0, ctx->stream));
    for (int i = 0; i < reps && st == SIMALL_OK; ++i)
        st = launch();
    SIMALL_CUDA_TRY(ctx, cudaEventRecord(e1, ctx->stream));
    SIMALL_CUDA_TRY(ctx, cudaEventSynchronize(e1));
    float total = 0.0f;
    cudaEventElapsedTime(&total, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (st)
        return st;
    *ms = static_cast<double>(total) / reps;
    if (bytes)
        *bytes = b;
    return SIMALL_OK;
}

int simall_solver_solve_csr(simall_solver *s, int64_t n, int64_t nnz, const int32_t *rowPtr, const int32_t *colIdx,
                            const double *values, const double *b, double *x, simall_solver_stats *stats)
{
    int st = simall_solver_set_matrix(s, n, nnz, rowPtr, colIdx, values, SIMALL_MEM_HOST);
    if (st)
        return st;
    return simall_solver_solve(s, b, x, SIMALL_MEM_HOST, stats);
}

}  // extern "C"
