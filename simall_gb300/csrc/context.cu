// Context, status strings, error reporting and host-side CSR checks.
#include "internal.hpp"

#include <cmath>
#include <cstring>
#include <new>

namespace simall {

int fail(simall_context *ctx, int status, const char *fmt, ...)
{
    if (ctx) {
        char buf[512];
        va_list ap;
        va_start(ap, fmt);
        vsnprintf(buf, sizeof(buf), fmt, ap);
        va_end(ap);
        ctx->last_error = buf;
    }
    return status;
}

int cuda_fail(simall_context *ctx, cudaError_t e, const char *what, const char *file, int line)
{
    const int st = (e == cudaErrorMemoryAllocation) ? SIMALL_ERR_OUT_OF_MEMORY
                   : (e == cudaErrorNoDevice || e == cudaErrorInvalidDevice) ? SIMALL_ERR_NO_DEVICE
                                                                                : SIMALL_ERR_CUDA;
    return fail(ctx, st, "%s failed: %s (%s:%d)", what, cudaGetErrorString(e), file, line);
}

std::vector<int32_t> make_row_blocks(int64_t n, const int32_t *rowPtr)
{
    std::vector<int32_t> rb;
    rb.reserve(static_cast<size_t>(n / 128 + 2));
    int64_t r = 0;
    rb.push_back(0);
    while (r < n) {
        int64_t e = r;
        const int64_t base = rowPtr[r];
        while (e < n && e - r < kSpmvRows && rowPtr[e + 1] - base <= kSpmvNnzCap)
            ++e;
        if (e == r)
            e = r + 1;  // a single row longer than the cap
        rb.push_back(static_cast<int32_t>(e));
        r = e;
    }
    return rb;
}

int check_csr_host(simall_context *ctx, int64_t n, int64_t nnz, const int32_t *rowPtr, const int32_t *colIdx,
                   const double *values, bool need_diag)
{
    if (n < 0 || nnz < 0 || !rowPtr || (nnz > 0 && !colIdx))
        return fail(ctx, SIMALL_ERR_INVALID_ARGUMENT, "CSR: null array or negative size");
    if (n > INT32_MAX - 1 || nnz > INT32_MAX)
        return fail(ctx, SIMALL_ERR_INVALID_ARGUMENT, "CSR: sizes exceed int32 indexing");
    if (rowPtr[0] != 0 || rowPtr[n] != nnz)
        return fail(ctx, SIMALL_ERR_SIZE_MISMATCH, "CSR: rowPtr[0]=%d rowPtr[n]=%d, nnz=%lld", rowPtr[0],
                    rowPtr[n], static_cast<long long>(nnz));
    for (int64_t i = 0; i < n; ++i) {
        const int32_t a = rowPtr[i], b = rowPtr[i + 1];
        if (b < a)
            return fail(ctx, SIMALL_ERR_UNSORTED_CSR, "CSR: rowPtr decreases at row %lld", static_cast<long long>(i));
        bool diag = false;
        for (int32_t k = a; k < b; ++k) {
            const int32_t c = colIdx[k];
            if (c < 0 || c >= n)
                return fail(ctx, SIMALL_ERR_INDEX_RANGE, "CSR: column %d out of range in row %lld", c,
                            static_cast<long long>(i));
            if (k > a && c <= colIdx[k - 1])
                return fail(ctx, SIMALL_ERR_UNSORTED_CSR, "CSR: row %lld columns not strictly ascending",
                            static_cast<long long>(i));
            if (c == i)
                diag = true;
            if (values && !std::isfinite(values[k]))
                return fail(ctx, SIMALL_ERR_NON_FINITE, "CSR: non-finite value in row %lld",
                            static_cast<long long>(i));
        }
        if (need_diag && !diag)
            return fail(ctx, SIMALL_ERR_MISSING_DIAGONAL, "CSR: row %lld has no diagonal",
                        static_cast<long long>(i));
    }
    return SIMALL_OK;
}

int grid_size_streaming(simall_context *ctx) { return ctx->num_sms * (2048 / kBlock); }

int resident_grid(simall_context *ctx, const void *kernel, int64_t items)
{
    int per_sm = 0;
    {
        std::lock_guard<std::mutex> lock(ctx->occupancy_mu);
        auto it = ctx->resident_per_sm.find(kernel);
        if (it != ctx->resident_per_sm.end()) {
            per_sm = it->second;
        } else {
            if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, kBlock, 0) != cudaSuccess)
                per_sm = 0;
            if (per_sm < 1 || per_sm > 2048 / kBlock)
                per_sm = per_sm < 1 ? 1 : 2048 / kBlock;
            ctx->resident_per_sm.emplace(kernel, per_sm);
        }
    }
    const int64_t g = (items + kBlock - 1) / kBlock;
    const int64_t cap = static_cast<int64_t>(ctx->num_sms) * per_sm;
    return static_cast<int>(g < 1 ? 1 : (g < cap ? g : cap));
}

}  // namespace simall

extern "C" {

const char *simall_status_string(int s)
{
    switch (s) {
    case SIMALL_OK:
        return "ok";
    case SIMALL_ERR_INVALID_ARGUMENT:
        return "invalid argument";
    case SIMALL_ERR_CUDA:
        return "CUDA runtime error";
    case SIMALL_ERR_OUT_OF_MEMORY:
        return "out of device memory";
    case SIMALL_ERR_UNSORTED_CSR:
        return "CSR rows not sorted / rowPtr not monotone";
    case SIMALL_ERR_MISSING_DIAGONAL:
        return "CSR row without diagonal";
    case SIMALL_ERR_NON_FINITE:
        return "non-finite input";
    case SIMALL_ERR_NOT_POSITIVE:
        return "non-positive diagonal";
    case SIMALL_ERR_SIZE_MISMATCH:
        return "size mismatch";
    case SIMALL_ERR_BREAKDOWN:
        return "CG breakdown (p.Ap == 0)";
    case SIMALL_ERR_TIMEOUT:
        return "bounded device wait expired";
    case SIMALL_ERR_IO:
        return "file could not be opened, written or renamed";
    case SIMALL_ERR_FORMAT:
        return "not a readable checkpoint (magic, version) or truncated";
    case SIMALL_ERR_UNSUPPORTED:
        return "unsupported option";
    case SIMALL_ERR_NO_DEVICE:
        return "no CUDA device";
    case SIMALL_ERR_INDEX_RANGE:
        return "index out of range";
    default:
        return "unknown status";
    }
}

const char *simall_version(void) { return "simall_gb300 0.1.0 sm_103a"; }

int simall_context_create(int device, void *stream, simall_context **out)
{
    if (!out)
        return SIMALL_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0) {
        cudaGetLastError();
        return SIMALL_ERR_NO_DEVICE;
    }
    if (device < 0 || device >= count)
        return SIMALL_ERR_INVALID_ARGUMENT;
    auto *ctx = new (std::nothrow) simall_context;
    if (!ctx)
        return SIMALL_ERR_OUT_OF_MEMORY;
    ctx->device = device;
    cudaError_t e = cudaSetDevice(device);
    if (e == cudaSuccess)
        e = cudaDeviceGetAttribute(&ctx->num_sms, cudaDevAttrMultiProcessorCount, device);
    if (e == cudaSuccess) {
        if (stream) {
            ctx->stream = static_cast<cudaStream_t>(stream);
        } else {
            e = cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking);
            ctx->own_stream = (e == cudaSuccess);
        }
    }
    if (e != cudaSuccess) {
        delete ctx;
        return SIMALL_ERR_CUDA;
    }
    *out = ctx;
    return SIMALL_OK;
}

int simall_context_destroy(simall_context *ctx)
{
    if (!ctx)
        return SIMALL_ERR_INVALID_ARGUMENT;
    if (ctx->own_stream) {
        cudaStreamSynchronize(ctx->stream);
        cudaStreamDestroy(ctx->stream);
    }
    delete ctx;
    return SIMALL_OK;
}

const char *simall_context_last_error(const simall_context *ctx) { return ctx ? ctx->last_error.c_str() : ""; }

int simall_context_synchronize(simall_context *ctx)
{
    if (!ctx)
        return SIMALL_ERR_INVALID_ARGUMENT;
    SIMALL_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
    return SIMALL_OK;
}

void *simall_context_stream(const simall_context *ctx) { return ctx ? static_cast<void *>(ctx->stream) : nullptr; }

int64_t simall_context_kernel_launches(const simall_context *ctx)
{
    return ctx ? ctx->launches.load(std::memory_order_relaxed) : 0;
}

}  // extern "C"
