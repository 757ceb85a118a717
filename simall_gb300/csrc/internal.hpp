// Internal declarations shared by the translation units of libsimall_gpu.so.
#pragma once

#include "simall_gpu.h"

#include <cuda_runtime.h>

#include <atomic>
#include <cstdarg>
#include <cstdint>
#include <cstdio>
#include <mutex>
#include <string>
#include <unordered_map>
#include <vector>

struct simall_context {
    int device = 0;
    int num_sms = 0;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    std::string last_error;
    std::atomic<int64_t> launches{0};
    std::mutex occupancy_mu;
    std::unordered_map<const void *, int> resident_per_sm;  // kernel -> resident CTAs of kBlock threads per SM
};

namespace simall {

constexpr int kBlock = 256;        // threads per CTA for the streaming kernels
constexpr int kSpmvRows = 256;     // max rows of one SpMV row-block
constexpr int kSpmvNnzCap = 2048;  // max nonzeros staged per row-block (16 KB of FP64 per staged array)
static_assert(kSpmvNnzCap % kBlock == 0, "row-block staging assumes whole slots per thread");
constexpr int kMaxReduce = 4;      // values reduced together by one kernel
// Mixed precision: a reliable update is also due when the iterated residual
// has not reached a new minimum for this many steps.  An FP32 inner CG on a
// hard system (a 160^3 distorted Neumann box: 8405 FP64 iterations) can
// stagnate for thousands of steps above the reliable_delta drop that would
// trigger the update; the replacement restarts its residual from the FP64
// one and progress resumes.  64 steps also fired on the 128^3 box's ordinary
// plateaus (18 updates instead of 10, 9% more steps); 256 does not.
constexpr int kMixedStallSteps = 256;

int fail(simall_context *ctx, int status, const char *fmt, ...);
int cuda_fail(simall_context *ctx, cudaError_t e, const char *what, const char *file, int line);

#define SIMALL_CUDA_TRY(ctx, call)                                                                              \
    do {                                                                                                        \
        cudaError_t e_ = (call);                                                                                \
        if (e_ != cudaSuccess)                                                                                  \
            return ::simall::cuda_fail((ctx), e_, #call, __FILE__, __LINE__);                                   \
    } while (0)

// Checks the launch that was just enqueued and counts it.
#define SIMALL_LAUNCH_CHECK(ctx)                                                                                \
    do {                                                                                                        \
        (ctx)->launches.fetch_add(1, std::memory_order_relaxed);                                                \
        cudaError_t e_ = cudaGetLastError();                                                                    \
        if (e_ != cudaSuccess)                                                                                  \
            return ::simall::cuda_fail((ctx), e_, "kernel launch", __FILE__, __LINE__);                         \
    } while (0)

// Owning device buffer (cudaMalloc / cudaFree).
template <class T> struct DevBuf {
    T *p = nullptr;
    size_t n = 0;
    DevBuf() = default;
    DevBuf(const DevBuf &) = delete;
    DevBuf &operator=(const DevBuf &) = delete;
    ~DevBuf() { release(); }
    void release()
    {
        if (p)
            cudaFree(p);
        p = nullptr;
        n = 0;
    }
    cudaError_t alloc(size_t count)
    {
        if (count <= n && p)
            return cudaSuccess;
        release();
        if (count == 0)
            return cudaSuccess;
        cudaError_t e = cudaMalloc(reinterpret_cast<void **>(&p), count * sizeof(T));
        if (e == cudaSuccess)
            n = count;
        else
            p = nullptr;
        return e;
    }
};

// Device-resident scalars of one Krylov solve; all loop control lives here so
// the host never waits on a reduction inside the iteration.
struct SolveScalars {
    double rz;      // r.z of the current iterate (FP64 path) / rho of the scaled system (mixed)
    double pAp;
    double alpha;
    double beta;
    double rr;      // ||r||^2
    double bnorm;   // max(||b||, 1e-30)
    double last;    // last relative residual
    double tol;
    double sigma0;  // mixed: scaled residual norm at the last reliable update
    double t0;      // mixed: true relative residual at the last reliable update
    double rmax;    // mixed: largest scaled residual norm since the last update
    double delta;   // mixed: reliable-update trigger
    int iter;       // completed iterations
    int max_iter;
    int done;       // loop finished
    int result;     // CGSolver::solve return value
    int status;     // SIMALL_OK / SIMALL_ERR_BREAKDOWN
    int need_update;  // mixed: a reliable update is due
    int updates;      // mixed: reliable updates performed
    int seen;         // mixed device loop: iteration count the last controller saw
    unsigned counter[8];  // last-block tickets, one per kernel kind
    // gpu::CgGpu semantics (SIMALL_SEMANTICS_CGGPU; FP64 CG only)
    int cggpu;          // 1: x0 honoured, stop test <= tol or the relative drop, |p.q| < 1e-300 break
    int converged;      // cggpu: set by the stop test that ended the solve
    double drop_factor; // cggpu: 10^-relativeOrders, 0 when off (set by the host)
    double drop_tol;    // cggpu: ||r_0|| * drop_factor
    double rnorm0;      // cggpu: ||b - A x0||
    double rnorm;       // ||r|| at the last stop test (cggpu: finalResidual)
    // mixed: the smallest iterated residual norm since the last reliable
    // update, and the steps since it was last lowered (stagnation trigger)
    double smin;
    int stall;
};

// CSR row-blocks for the staged SpMV: each block holds <= kSpmvRows rows and
// <= kSpmvNnzCap nonzeros, except a single row longer than the cap.
std::vector<int32_t> make_row_blocks(int64_t n, const int32_t *rowPtr);

// Validates a host CSR (monotone rowPtr, strictly ascending in-range columns,
// finite values unless values is NULL).  need_diag: every row must hold its
// diagonal.
int check_csr_host(simall_context *ctx, int64_t n, int64_t nnz, const int32_t *rowPtr, const int32_t *colIdx,
                   const double *values, bool need_diag);

// CTAs of a full-occupancy streaming grid (8 x 256 threads per SM).
int grid_size_streaming(simall_context *ctx);
// Grid of a grid-stride kernel launched with kBlock threads: exactly one wave
// of resident CTAs (SMs x the kernel's resident CTAs per SM, from its register
// and shared-memory use), or fewer when `items` threads' worth of work is
// smaller.  A second, partial wave would leave most SMs idle at the end of
// every launch.  Never larger than grid_size_streaming.
int resident_grid(simall_context *ctx, const void *kernel, int64_t items);

}  // namespace simall
