// The reference GPU facade (src/gpu/GpuKernels.hpp:48-87) as hand-written
// kernels, plus the solver's standalone SpMV.  The reference routes these
// through cuBLAS / cuSPARSE (GpuKernels.cpp:76-281) with a descriptor and a
// cudaMalloc per SpMV call and host round trips for Jacobi; here every call
// is one kernel on the caller's stream, and dot / nrm2 reduce on the device
// in a fixed order before the single blocking copy their contract requires.
#include "device.cuh"
#include "solver.hpp"

#include <cmath>
#include <mutex>

namespace simall {

namespace {

__global__ void k_axpy(int64_t n, double a, const double *__restrict__ x, double *__restrict__ y)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        y[i] += a * x[i];
}
__global__ void k_scal(int64_t n, double a, double *__restrict__ x)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        x[i] *= a;
}
__global__ void k_axpby(int64_t n, double a, const double *__restrict__ x, double b, double *__restrict__ y)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        y[i] = a * x[i] + b * y[i];
}
__global__ void k_xpby(int64_t n, const double *__restrict__ x, double b, double *__restrict__ y)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        y[i] = x[i] + b * y[i];
}
__global__ void k_jacobi_apply(int64_t n, const double *__restrict__ d, const double *__restrict__ r,
                               double *__restrict__ z)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        z[i] = r[i] / d[i];
}
// z = invD r, JacobiPreconditioner::apply (src/solver/LinearSolvers.cpp:66-71)
__global__ void k_scale_inv(int64_t n, const double *__restrict__ invD, const double *__restrict__ r,
                            double *__restrict__ z)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        z[i] = __dmul_rn(invD[i], r[i]);
}
__global__ void __launch_bounds__(kBlock) k_dot(int64_t n, const double *__restrict__ x, const double *__restrict__ y,
                                                double *partials, unsigned *ticket, double *out)
{
    double acc[1] = {0.0};
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        acc[0] += x[i] * y[i];
    if (grid_sum_last<1>(acc, partials, ticket) && threadIdx.x == 0)
        *out = acc[0];
}
// Thread-per-row CSR SpMV with the reference's rounding sequence (bit-exact
// with CSRMatrix::spmv); the facade has no precomputed row-blocks.
__global__ void __launch_bounds__(kBlock) k_spmv_rows(int64_t n, const int32_t *__restrict__ rowPtr,
                                                      const int32_t *__restrict__ colIdx,
                                                      const double *__restrict__ val, const double *__restrict__ x,
                                                      double *__restrict__ y)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        double s = 0.0;
        for (int k = rowPtr[i]; k < rowPtr[i + 1]; ++k)
            s = __dadd_rn(s, __dmul_rn(val[k], __ldg(x + colIdx[k])));
        y[i] = s;
    }
}

struct SpmvEpi {
    double *y;
    __device__ __forceinline__ void operator()(int row, double v) { y[row] = v; }
};
__global__ void __launch_bounds__(kBlock) k_spmv_staged(const int32_t *__restrict__ rowPtr,
                                                        const int32_t *__restrict__ colIdx,
                                                        const double *__restrict__ val, const int32_t *__restrict__ rb,
                                                        int nRB, const double *__restrict__ x, double *__restrict__ y)
{
    SpmvEpi epi{y};
    spmv_rowblocks(rowPtr, colIdx, val, rb, nRB, x, epi);
}

constexpr int kFacadeGrid = 1024;

// Process-wide reduction scratch of the facade, one per device.
struct FacadeScratch {
    double *partials = nullptr;  // kFacadeGrid doubles + result
    unsigned *ticket = nullptr;
};
std::mutex g_mu;
FacadeScratch g_scratch[64];

int facade_scratch(FacadeScratch **out)
{
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64)
        return SIMALL_ERR_NO_DEVICE;
    std::lock_guard<std::mutex> lk(g_mu);
    FacadeScratch &s = g_scratch[dev];
    if (!s.partials) {
        if (cudaMalloc(&s.partials, (kFacadeGrid + 1) * sizeof(double)) != cudaSuccess)
            return SIMALL_ERR_OUT_OF_MEMORY;
        if (cudaMalloc(&s.ticket, sizeof(unsigned)) != cudaSuccess ||
            cudaMemset(s.ticket, 0, sizeof(unsigned)) != cudaSuccess)
            return SIMALL_ERR_OUT_OF_MEMORY;
    }
    *out = &s;
    return SIMALL_OK;
}

int grid1(size_t n)
{
    const size_t g = (n + kBlock - 1) / kBlock;
    return static_cast<int>(g < 1 ? 1 : (g > kFacadeGrid ? kFacadeGrid : g));
}

int launched() { return cudaGetLastError() == cudaSuccess ? SIMALL_OK : SIMALL_ERR_CUDA; }

int reduce_dot(const double *x, const double *y, size_t n, void *stream, double *result)
{
    FacadeScratch *sc = nullptr;
    int st = facade_scratch(&sc);
    if (st)
        return st;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    std::lock_guard<std::mutex> lk(g_mu);  // the scratch is shared by all callers on this device
    k_dot<<<grid1(n), kBlock, 0, s>>>(static_cast<int64_t>(n), x, y, sc->partials, sc->ticket,
                                      sc->partials + kFacadeGrid);
    if (launched())
        return SIMALL_ERR_CUDA;
    if (cudaMemcpyAsync(result, sc->partials + kFacadeGrid, sizeof(double), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess)
        return SIMALL_ERR_CUDA;
    return SIMALL_OK;
}

}  // namespace
}  // namespace simall

using namespace simall;

extern "C" {

int simall_gpu_axpy(double alpha, const double *x, double *y, size_t n, void *stream)
{
    if (n == 0)
        return SIMALL_OK;
    if (!x || !y)
        return SIMALL_ERR_INVALID_ARGUMENT;
    k_axpy<<<grid1(n), kBlock, 0, static_cast<cudaStream_t>(stream)>>>(static_cast<int64_t>(n), alpha, x, y);
    return launched();
}

int simall_gpu_scal(double alpha, double *x, size_t n, void *stream)
{
    if (n == 0)
        return SIMALL_OK;
    if (!x)
        return SIMALL_ERR_INVALID_ARGUMENT;
    k_scal<<<grid1(n), kBlock, 0, static_cast<cudaStream_t>(stream)>>>(static_cast<int64_t>(n), alpha, x);
    return launched();
}

int simall_gpu_copy(const double *src, double *dst, size_t n, void *stream)
{
    if (n == 0)
        return SIMALL_OK;
    if (!src || !dst)
        return SIMALL_ERR_INVALID_ARGUMENT;
    return cudaMemcpyAsync(dst, src, n * sizeof(double), cudaMemcpyDeviceToDevice, static_cast<cudaStream_t>(stream)) ==
                   cudaSuccess
               ? SIMALL_OK
               : SIMALL_ERR_CUDA;
}

int simall_gpu_dot(const double *x, const double *y, size_t n, void *stream, double *result)
{
    if (!result || (n && (!x || !y)))
        return SIMALL_ERR_INVALID_ARGUMENT;
    if (n == 0) {
        *result = 0.0;
        return SIMALL_OK;
    }
    return reduce_dot(x, y, n, stream, result);
}

int simall_gpu_nrm2(const double *x, size_t n, void *stream, double *result)
{
    if (!result || (n && !x))
        return SIMALL_ERR_INVALID_ARGUMENT;
    if (n == 0) {
        *result = 0.0;
        return SIMALL_OK;
    }
    double d = 0.0;
    int st = reduce_dot(x, x, n, stream, &d);
    *result = std::sqrt(d);
    return st;
}

int simall_gpu_axpby(double a, const double *x, double b, double *y, size_t n, void *stream)
{
    if (n == 0)
        return SIMALL_OK;
    if (!x || !y)
        return SIMALL_ERR_INVALID_ARGUMENT;
    k_axpby<<<grid1(n), kBlock, 0, static_cast<cudaStream_t>(stream)>>>(static_cast<int64_t>(n), a, x, b, y);
    return launched();
}

int simall_gpu_xpby(const double *x, double beta, double *y, size_t n, void *stream)
{
    if (n == 0)
        return SIMALL_OK;
    if (!x || !y)
        return SIMALL_ERR_INVALID_ARGUMENT;
    k_xpby<<<grid1(n), kBlock, 0, static_cast<cudaStream_t>(stream)>>>(static_cast<int64_t>(n), x, beta, y);
    return launched();
}

int simall_gpu_spmv_csr(size_t n, const int32_t *rowPtr, const int32_t *colIdx, const double *values, const double *x,
                        double *y, void *stream)
{
    if (n == 0)
        return SIMALL_OK;
    if (!rowPtr || !colIdx || !values || !x || !y)
        return SIMALL_ERR_INVALID_ARGUMENT;
    k_spmv_rows<<<grid1(n), kBlock, 0, static_cast<cudaStream_t>(stream)>>>(static_cast<int64_t>(n), rowPtr, colIdx,
                                                                            values, x, y);
    return launched();
}

int simall_gpu_jacobi_apply(const double *diag, const double *r, double *z, size_t n, void *stream)
{
    if (n == 0)
        return SIMALL_OK;
    if (!diag || !r || !z)
        return SIMALL_ERR_INVALID_ARGUMENT;
    k_jacobi_apply<<<grid1(n), kBlock, 0, static_cast<cudaStream_t>(stream)>>>(static_cast<int64_t>(n), diag, r, z);
    return launched();
}

int simall_solver_spmv(simall_solver *s, const double *x, double *y, int mem)
{
    if (!s || !x || !y)
        return SIMALL_ERR_INVALID_ARGUMENT;
    simall_context *ctx = s->ctx;
    if (!s->ready)
        return fail(ctx, SIMALL_ERR_INVALID_ARGUMENT, "spmv before set_matrix");
    const size_t bytes = static_cast<size_t>(s->n) * sizeof(double);
    const double *dx = x;
    double *dy = y;
    if (mem == SIMALL_MEM_HOST) {
        SIMALL_CUDA_TRY(ctx, cudaMemcpyAsync(s->p.p, x, bytes, cudaMemcpyHostToDevice, ctx->stream));
        dx = s->p.p;
        dy = s->Ap.p;
    }
    const int64_t cap = grid_size_streaming(ctx);
    const int64_t units = spmv_direct(s) ? (s->n + kBlock - 1) / kBlock : s->nRowBlocks;
    const int g = static_cast<int>(units < cap ? units : cap);
    k_spmv_staged<<<g < 1 ? 1 : g, kBlock, 0, ctx->stream>>>(s->rowPtr, s->colIdx, s->values, s->rowBlocks.p,
                                                             spmv_schedule(s), dx, dy);
    SIMALL_LAUNCH_CHECK(ctx);
    if (mem == SIMALL_MEM_HOST) {
        SIMALL_CUDA_TRY(ctx, cudaMemcpyAsync(y, dy, bytes, cudaMemcpyDeviceToHost, ctx->stream));
        SIMALL_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
    }
    return SIMALL_OK;
}

int simall_solver_precond_apply(simall_solver *s, const double *r, double *z, int mem)
{
    if (!s || !r || !z)
        return SIMALL_ERR_INVALID_ARGUMENT;
    simall_context *ctx = s->ctx;
    if (!s->ready)
        return fail(ctx, SIMALL_ERR_INVALID_ARGUMENT, "precond_apply before set_matrix");
    if (s->cfg.precision != SIMALL_PRECISION_FP64)
        return fail(ctx, SIMALL_ERR_UNSUPPORTED, "precond_apply: the FP64 preconditioners only");
    SIMALL_CUDA_TRY(ctx, cudaSetDevice(ctx->device));
    const size_t bytes = static_cast<size_t>(s->n) * sizeof(double);
    const double *dr = r;
    double *dz = z;
    if (mem == SIMALL_MEM_HOST) {  // the solve's own vectors are free between solves
        SIMALL_CUDA_TRY(ctx, cudaMemcpyAsync(s->p.p, r, bytes, cudaMemcpyHostToDevice, ctx->stream));
        dr = s->p.p;
        dz = s->Ap.p;
    }
    if (sweep_preconditioner(s->cfg.preconditioner)) {
        int e = ilu_apply(s, dr, dz);
        if (e)
            return e;
    } else {
        k_scale_inv<<<grid1(static_cast<size_t>(s->n)), kBlock, 0, ctx->stream>>>(s->n, s->invDiag.p, dr, dz);
        SIMALL_LAUNCH_CHECK(ctx);
    }
    if (mem == SIMALL_MEM_HOST) {
        SIMALL_CUDA_TRY(ctx, cudaMemcpyAsync(z, dz, bytes, cudaMemcpyDeviceToHost, ctx->stream));
        SIMALL_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
    }
    return sweep_preconditioner(s->cfg.preconditioner) ? ilu_check(s) : SIMALL_OK;
}

int simall_solver_amg_levels(const simall_solver *s, int *nlev, int32_t *rows, int max_levels)
{
    if (!s || !nlev || (max_levels > 0 && !rows))
        return SIMALL_ERR_INVALID_ARGUMENT;
    return amg_levels(s, nlev, rows, max_levels);
}

}  // extern "C"
