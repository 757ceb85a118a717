// FieldRegistry in device memory: the GB300 replacement of
// solver::FieldRegistry (src/solver/FieldRegistry.hpp:30-80).  A scalar field
// is one FP64 array of n cells; a vector field one [3][n] array (x, y, z back
// to back, the layout the device SIMPLE iteration uses for U).  scalar() /
// vector() create a zeroed field, or re-create it zeroed when the size
// differs, exactly as the reference's accessors; find_* return nothing when
// the name is absent.
#include "registry.hpp"

#include <algorithm>
#include <cstring>
#include <new>

namespace simall {

simall_fields::Field *registry_find(simall_fields *r, const char *name, bool vector)
{
    for (auto *f : vector ? r->vectors : r->scalars)
        if (f->name == name)
            return f;
    return nullptr;
}

simall_fields::Field *registry_get(simall_fields *r, const char *name, int64_t n, bool vector, int *st)
{
    simall_context *ctx = r->ctx;
    *st = SIMALL_OK;
    simall_fields::Field *f = registry_find(r, name, vector);
    if (!f) {
        f = new (std::nothrow) simall_fields::Field;
        if (!f) {
            *st = SIMALL_ERR_OUT_OF_MEMORY;
            return nullptr;
        }
        f->name = name;
        f->n = -1;
        (vector ? r->vectors : r->scalars).push_back(f);
    }
    if (f->n != n) {
        const int64_t len = (vector ? 3 : 1) * n;
        f->data.release();
        cudaError_t e = f->data.alloc(static_cast<size_t>(len > 0 ? len : 0));
        if (e == cudaSuccess && len > 0)
            e = cudaMemsetAsync(f->data.p, 0, len * sizeof(double), ctx->stream);
        if (e == cudaSuccess)
            e = cudaStreamSynchronize(ctx->stream);
        if (e != cudaSuccess) {
            *st = cuda_fail(ctx, e, "field allocation", __FILE__, __LINE__);
            f->n = -1;
            return nullptr;
        }
        f->n = n;
    }
    return f;
}

}  // namespace simall

using namespace simall;

extern "C" {

int simall_fields_create(simall_context *ctx, simall_fields **out)
{
    if (!ctx || !out)
        return SIMALL_ERR_INVALID_ARGUMENT;
    auto *r = new (std::nothrow) simall_fields;
    if (!r)
        return SIMALL_ERR_OUT_OF_MEMORY;
    r->ctx = ctx;
    *out = r;
    return SIMALL_OK;
}

int simall_fields_destroy(simall_fields *r)
{
    if (!r)
        return SIMALL_ERR_INVALID_ARGUMENT;
    cudaStreamSynchronize(r->ctx->stream);
    delete r;
    return SIMALL_OK;
}

int simall_fields_scalar(simall_fields *r, const char *name, int64_t n, double **data)
{
    if (!r || !name || n < 0)
        return SIMALL_ERR_INVALID_ARGUMENT;
    SIMALL_CUDA_TRY(r->ctx, cudaSetDevice(r->ctx->device));
    int st = SIMALL_OK;
    simall_fields::Field *f = registry_get(r, name, n, false, &st);
    if (!f)
        return st;
    if (data)
        *data = f->data.p;
    return SIMALL_OK;
}

int simall_fields_vector(simall_fields *r, const char *name, int64_t n, double **x, double **y, double **z)
{
    if (!r || !name || n < 0)
        return SIMALL_ERR_INVALID_ARGUMENT;
    SIMALL_CUDA_TRY(r->ctx, cudaSetDevice(r->ctx->device));
    int st = SIMALL_OK;
    simall_fields::Field *f = registry_get(r, name, n, true, &st);
    if (!f)
        return st;
    if (x)
        *x = f->data.p;
    if (y)
        *y = f->data.p ? f->data.p + n : nullptr;
    if (z)
        *z = f->data.p ? f->data.p + 2 * n : nullptr;
    return SIMALL_OK;
}

int simall_fields_find(simall_fields *r, const char *name, int vector, double **data, int64_t *n)
{
    if (!r || !name)
        return SIMALL_ERR_INVALID_ARGUMENT;
    simall_fields::Field *f = registry_find(r, name, vector != 0);
    if (data)
        *data = f ? f->data.p : nullptr;
    if (n)
        *n = f ? f->n : -1;
    return SIMALL_OK;
}

int simall_fields_upload(simall_fields *r, const char *name, int vector, const double *host, int64_t n)
{
    if (!r || !name || n < 0 || (n > 0 && !host))
        return SIMALL_ERR_INVALID_ARGUMENT;
    SIMALL_CUDA_TRY(r->ctx, cudaSetDevice(r->ctx->device));
    int st = SIMALL_OK;
    simall_fields::Field *f = registry_get(r, name, n, vector != 0, &st);
    if (!f)
        return st;
    const int64_t len = (vector ? 3 : 1) * n;
    if (len > 0) {
        SIMALL_CUDA_TRY(r->ctx, cudaMemcpyAsync(f->data.p, host, len * sizeof(double), cudaMemcpyHostToDevice,
                                                r->ctx->stream));
        SIMALL_CUDA_TRY(r->ctx, cudaStreamSynchronize(r->ctx->stream));
    }
    return SIMALL_OK;
}

int simall_fields_download(simall_fields *r, const char *name, int vector, double *host)
{
    if (!r || !name)
        return SIMALL_ERR_INVALID_ARGUMENT;
    simall_fields::Field *f = registry_find(r, name, vector != 0);
    if (!f)
        return fail(r->ctx, SIMALL_ERR_INVALID_ARGUMENT, "no %s field named %s", vector ? "vector" : "scalar", name);
    const int64_t len = (vector ? 3 : 1) * f->n;
    if (len > 0) {
        if (!host)
            return SIMALL_ERR_INVALID_ARGUMENT;
        SIMALL_CUDA_TRY(r->ctx, cudaSetDevice(r->ctx->device));
        SIMALL_CUDA_TRY(r->ctx, cudaMemcpyAsync(host, f->data.p, len * sizeof(double), cudaMemcpyDeviceToHost,
                                                r->ctx->stream));
        SIMALL_CUDA_TRY(r->ctx, cudaStreamSynchronize(r->ctx->stream));
    }
    return SIMALL_OK;
}

int simall_fields_count(const simall_fields *r, int *n_scalars, int *n_vectors)
{
    if (!r)
        return SIMALL_ERR_INVALID_ARGUMENT;
    if (n_scalars)
        *n_scalars = static_cast<int>(r->scalars.size());
    if (n_vectors)
        *n_vectors = static_cast<int>(r->vectors.size());
    return SIMALL_OK;
}

int simall_fields_name(const simall_fields *r, int vector, int index, char *buf, int len, int64_t *n)
{
    if (!r || index < 0)
        return SIMALL_ERR_INVALID_ARGUMENT;
    const auto &list = vector ? r->vectors : r->scalars;
    if (index >= static_cast<int>(list.size()))
        return SIMALL_ERR_INVALID_ARGUMENT;
    const simall_fields::Field *f = list[static_cast<size_t>(index)];
    if (buf && len > 0) {
        const size_t m = std::min(static_cast<size_t>(len - 1), f->name.size());
        std::memcpy(buf, f->name.data(), m);
        buf[m] = '\0';
    }
    if (n)
        *n = f->n;
    return SIMALL_OK;
}

}  // extern "C"
