// Dot product that allocates no device memory.
//
// simall_gpu_dot reduces through a scratch buffer it cudaMallocs on first use.
// Some callers cannot allow that: code running under a fixed device-memory
// budget that another allocator (a framework's caching pool, a solver that
// reserved everything at start-up) already owns, so a fresh cudaMalloc would
// fail or fragment it; latency-critical loops that cannot afford
// cudaMalloc/cudaFree's implicit device-wide synchronisation; and processes
// that must keep a constant device footprint after initialisation.  This
// variant keeps its reduction scratch in a fixed array of the library
// itself (the CUDA runtime places it when the library's device code is
// loaded, and it stays reserved on every GPU that loaded it until the process
// exits).
//
// The array holds one partial sum per CTA for at most kMaxBlocks CTAs of
// kBlock threads that each handle kPerThread elements, so n is limited to
// SIMALL_DOT_NOALLOC_MAX_N (16,777,216 = 2^24 elements, 128 MiB per operand);
// larger n is rejected with SIMALL_ERR_SIZE_MISMATCH before any device work.
//
// All calls share the one array: two calls whose work overlaps on the GPU
// (different streams, or different host threads) race and return wrong
// results.  The CTA ticket must start at zero and is cleared on the stream
// before every launch; the partials and the result are overwritten each call.
//
// Set-up: the first call on each device, with that device current, looks the
// array's device address up with cudaGetSymbolAddress and caches it.  Make
// that first call before any stream capture on the device.  The cached
// address lives as long as the device's context: after cudaDeviceReset the
// library's module is loaded again and the array may move, so a caller that
// resets a device must not use this function on it afterwards.  A call whose
// device work fails to start drops the device's cached address, so the next
// call looks it up again.
#include "device.cuh"

#include <mutex>

namespace {

constexpr int kMaxBlocks = 4096;
constexpr int kPerThread = 16;
constexpr size_t kMaxN = static_cast<size_t>(kMaxBlocks) * simall::kBlock * kPerThread;
static_assert(kMaxN == SIMALL_DOT_NOALLOC_MAX_N, "the header's limit must match the scratch size");

struct DotScratch {
    double partials[kMaxBlocks];
    double result;
    unsigned ticket;
};

static __device__ __align__(256) DotScratch g_dot_scratch;

// x.y over n elements; CTA b covers a contiguous span of kBlock*kPerThread
// elements, read coalesced; the last CTA writes the sum to sc->result.
__global__ void __launch_bounds__(simall::kBlock) k_dot_noalloc(size_t n, const double *__restrict__ x,
                                                                const double *__restrict__ y, DotScratch *sc)
{
    double acc[1] = {0.0};
    const size_t base = static_cast<size_t>(blockIdx.x) * simall::kBlock * kPerThread + threadIdx.x;
#pragma unroll
    for (int j = 0; j < kPerThread; ++j) {
        const size_t i = base + static_cast<size_t>(j) * simall::kBlock;
        if (i < n)
            acc[0] += __ldg(x + i) * __ldg(y + i);
    }
    if (simall::grid_sum_last<1>(acc, sc->partials, &sc->ticket) && threadIdx.x == 0)
        sc->result = acc[0];
}

constexpr int kMaxDevices = 64;
std::mutex g_setup_mu;
DotScratch *g_scratch_addr[kMaxDevices] = {};

// Device address of g_dot_scratch on the current device (looked up once).
int scratch_address(DotScratch **out, int *device)
{
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices)
        return SIMALL_ERR_NO_DEVICE;
    *device = dev;
    std::lock_guard<std::mutex> lk(g_setup_mu);
    if (!g_scratch_addr[dev]) {
        DotScratch *p = nullptr;
        if (cudaGetSymbolAddress(reinterpret_cast<void **>(&p), g_dot_scratch) != cudaSuccess || !p)
            return SIMALL_ERR_CUDA;
        g_scratch_addr[dev] = p;
    }
    *out = g_scratch_addr[dev];
    return SIMALL_OK;
}

int drop_scratch_address(int dev)
{
    std::lock_guard<std::mutex> lk(g_setup_mu);
    g_scratch_addr[dev] = nullptr;
    return SIMALL_ERR_CUDA;
}

}  // namespace

extern "C" int simall_gpu_dot_noalloc(const double *x, const double *y, size_t n, void *stream, double *result)
{
    if (!result || (n && (!x || !y)))
        return SIMALL_ERR_INVALID_ARGUMENT;
    if (n > kMaxN)
        return SIMALL_ERR_SIZE_MISMATCH;
    if (n == 0) {
        *result = 0.0;
        return SIMALL_OK;
    }
    DotScratch *sc = nullptr;
    int dev = 0;
    const int st = scratch_address(&sc, &dev);
    if (st != SIMALL_OK)
        return st;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    if (cudaMemsetAsync(&sc->ticket, 0, sizeof(unsigned), s) != cudaSuccess)
        return drop_scratch_address(dev);
    const size_t per_block = static_cast<size_t>(simall::kBlock) * kPerThread;
    const int blocks = static_cast<int>((n + per_block - 1) / per_block);
    k_dot_noalloc<<<blocks, simall::kBlock, 0, s>>>(n, x, y, sc);
    if (cudaGetLastError() != cudaSuccess)
        return drop_scratch_address(dev);
    if (cudaMemcpyAsync(result, &sc->result, sizeof(double), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess)
        return SIMALL_ERR_CUDA;
    return SIMALL_OK;
}
