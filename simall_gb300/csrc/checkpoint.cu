// io::Checkpoint (src/io/Checkpoint.cpp:66-227) for a device-resident field
// registry: the reference's file format, byte for byte, written from and read
// into device memory.
//
// Format (little-endian): header {char magic[8] = "SIMALLCP", u32 version = 1,
// u32 flags, u64 timestamp} (24 bytes); meta {i32 iteration, 4 bytes of
// padding, f64 time, u64 settingsHash} (24 bytes, the reference writes the
// struct as it lies in memory; the padding is written as zeros here); the mesh
// as 20 length-prefixed arrays (u64 count, then the elements) in the order of
// Checkpoint::write; u32 scalar count, u32 vector count; each scalar field as
// {u32 name length, name bytes, u64 n, n doubles}; each vector field as
// {name, x, y, z}, every component length-prefixed.
//
// Field payloads move between HBM and the file through two pinned staging
// buffers: the device-to-host copy of one chunk overlaps the write of the
// previous one (and the read of the next chunk overlaps the host-to-device
// copy of the previous one), so a checkpoint of a large state streams at the
// slower of the file and the copy engine instead of their sum.  Writes go to
// "<path>.tmp" and are renamed over <path> only once complete.
#include "registry.hpp"

#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <new>
#include <string>
#include <vector>

namespace simall {

namespace {

constexpr size_t kChunkBytes = 8u << 20;  // per staging buffer

struct Staging {
    simall_context *ctx;
    void *buf[2] = {nullptr, nullptr};
    cudaEvent_t ev[2] = {nullptr, nullptr};
    explicit Staging(simall_context *c) : ctx(c) {}
    ~Staging()
    {
        for (int i = 0; i < 2; ++i) {
            if (buf[i])
                cudaFreeHost(buf[i]);
            if (ev[i])
                cudaEventDestroy(ev[i]);
        }
    }
    int init()
    {
        for (int i = 0; i < 2; ++i) {
            SIMALL_CUDA_TRY(ctx, cudaMallocHost(&buf[i], kChunkBytes));
            SIMALL_CUDA_TRY(ctx, cudaEventCreateWithFlags(&ev[i], cudaEventDisableTiming));
        }
        return SIMALL_OK;
    }
};

struct File {
    FILE *f = nullptr;
    ~File()
    {
        if (f)
            std::fclose(f);
    }
};

bool put(FILE *f, const void *p, size_t bytes) { return bytes == 0 || std::fwrite(p, 1, bytes, f) == bytes; }
bool get(FILE *f, void *p, size_t bytes) { return bytes == 0 || std::fread(p, 1, bytes, f) == bytes; }

template <class T> bool put_vec(FILE *f, const T *p, int64_t n)
{
    const uint64_t c = static_cast<uint64_t>(n);
    return put(f, &c, 8) && (n == 0 || put(f, p, static_cast<size_t>(n) * sizeof(T)));
}

bool put_name(FILE *f, const std::string &s)
{
    const uint32_t n = static_cast<uint32_t>(s.size());
    return put(f, &n, 4) && put(f, s.data(), n);
}

// u64 n, then n doubles streamed from device memory.
int put_device(simall_context *ctx, Staging &st, FILE *f, const double *d, int64_t n)
{
    const uint64_t c = static_cast<uint64_t>(n);
    if (!put(f, &c, 8))
        return fail(ctx, SIMALL_ERR_IO, "checkpoint: write failed");
    const size_t per = kChunkBytes / sizeof(double);
    const int64_t chunks = (n + static_cast<int64_t>(per) - 1) / static_cast<int64_t>(per);
    auto issue = [&](int64_t k) -> int {
        const int64_t a = k * static_cast<int64_t>(per);
        const int64_t m = (n - a < static_cast<int64_t>(per)) ? n - a : static_cast<int64_t>(per);
        SIMALL_CUDA_TRY(ctx, cudaMemcpyAsync(st.buf[k & 1], d + a, m * sizeof(double), cudaMemcpyDeviceToHost,
                                             ctx->stream));
        SIMALL_CUDA_TRY(ctx, cudaEventRecord(st.ev[k & 1], ctx->stream));
        return SIMALL_OK;
    };
    if (chunks > 0) {
        int e = issue(0);
        if (e)
            return e;
    }
    for (int64_t k = 0; k < chunks; ++k) {
        if (k + 1 < chunks) {
            int e = issue(k + 1);  // the next chunk's copy runs while this one is written
            if (e)
                return e;
        }
        SIMALL_CUDA_TRY(ctx, cudaEventSynchronize(st.ev[k & 1]));
        const int64_t a = k * static_cast<int64_t>(per);
        const int64_t m = (n - a < static_cast<int64_t>(per)) ? n - a : static_cast<int64_t>(per);
        if (!put(f, st.buf[k & 1], static_cast<size_t>(m) * sizeof(double)))
            return fail(ctx, SIMALL_ERR_IO, "checkpoint: write failed");
    }
    return SIMALL_OK;
}

// n doubles from the file streamed into device memory.
int get_device(simall_context *ctx, Staging &st, FILE *f, double *d, int64_t n)
{
    const size_t per = kChunkBytes / sizeof(double);
    const int64_t chunks = (n + static_cast<int64_t>(per) - 1) / static_cast<int64_t>(per);
    bool pending[2] = {false, false};
    for (int64_t k = 0; k < chunks; ++k) {
        const int b = static_cast<int>(k & 1);
        if (pending[b])
            SIMALL_CUDA_TRY(ctx, cudaEventSynchronize(st.ev[b]));  // the buffer's previous copy is done
        const int64_t a = k * static_cast<int64_t>(per);
        const int64_t m = (n - a < static_cast<int64_t>(per)) ? n - a : static_cast<int64_t>(per);
        if (!get(f, st.buf[b], static_cast<size_t>(m) * sizeof(double)))
            return fail(ctx, SIMALL_ERR_FORMAT, "checkpoint: truncated field data");
        SIMALL_CUDA_TRY(ctx, cudaMemcpyAsync(d + a, st.buf[b], m * sizeof(double), cudaMemcpyHostToDevice,
                                             ctx->stream));
        SIMALL_CUDA_TRY(ctx, cudaEventRecord(st.ev[b], ctx->stream));
        pending[b] = true;
    }
    SIMALL_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
    return SIMALL_OK;
}

template <class T> bool get_vec(FILE *f, T *&out, int64_t &n)
{
    uint64_t c = 0;
    if (!get(f, &c, 8) || c > (uint64_t(1) << 40))
        return false;
    n = static_cast<int64_t>(c);
    out = static_cast<T *>(std::malloc(c ? c * sizeof(T) : 1));
    return out && get(f, out, static_cast<size_t>(c) * sizeof(T));
}

bool skip_vec(FILE *f, size_t elem)
{
    uint64_t c = 0;
    if (!get(f, &c, 8) || c > (uint64_t(1) << 40))
        return false;
    return std::fseek(f, static_cast<long>(c * elem), SEEK_CUR) == 0;
}

}  // namespace

}  // namespace simall

using namespace simall;

extern "C" {

int simall_checkpoint_write(const char *path, const simall_checkpoint_mesh *m, simall_fields *fields,
                            const simall_checkpoint_meta *meta)
{
    if (!path || !m || !fields || !meta)
        return SIMALL_ERR_INVALID_ARGUMENT;
    simall_context *ctx = fields->ctx;
    if (m->n_nodes < 0 || m->n_faces < 0 || m->n_cells < 0 || m->n_face_nodes < 0 || m->n_cell_faces < 0)
        return fail(ctx, SIMALL_ERR_INVALID_ARGUMENT, "checkpoint: negative mesh size");
    SIMALL_CUDA_TRY(ctx, cudaSetDevice(ctx->device));
    Staging st(ctx);
    int e = st.init();
    if (e)
        return e;
    const std::string tmp = std::string(path) + ".tmp";
    File file;
    file.f = std::fopen(tmp.c_str(), "wb");
    if (!file.f)
        return fail(ctx, SIMALL_ERR_IO, "checkpoint: cannot open %s", tmp.c_str());
    FILE *f = file.f;
    unsigned char hdr[24] = {'S', 'I', 'M', 'A', 'L', 'L', 'C', 'P'};
    const uint32_t version = 1, flags = 0;
    const uint64_t ts = static_cast<uint64_t>(
        std::chrono::duration_cast<std::chrono::seconds>(std::chrono::system_clock::now().time_since_epoch()).count());
    std::memcpy(hdr + 8, &version, 4);
    std::memcpy(hdr + 12, &flags, 4);
    std::memcpy(hdr + 16, &ts, 8);
    unsigned char mt[24] = {0};
    std::memcpy(mt, &meta->iteration, 4);
    std::memcpy(mt + 8, &meta->time, 8);
    std::memcpy(mt + 16, &meta->settings_hash, 8);
    bool ok = put(f, hdr, 24) && put(f, mt, 24);
    const int64_t nN = m->n_nodes, nF = m->n_faces, nC = m->n_cells;
    ok = ok && put_vec(f, m->node_x, nN) && put_vec(f, m->node_y, nN) && put_vec(f, m->node_z, nN);
    ok = ok && put_vec(f, m->owner, nF) && put_vec(f, m->neighbor, nF);
    ok = ok && put_vec(f, m->area_x, nF) && put_vec(f, m->area_y, nF) && put_vec(f, m->area_z, nF);
    ok = ok && put_vec(f, m->centroid_x, nF) && put_vec(f, m->centroid_y, nF) && put_vec(f, m->centroid_z, nF);
    ok = ok && put_vec(f, m->boundary_zone, nF);
    ok = ok && put_vec(f, m->face_node_offsets, m->face_node_offsets ? nF + 1 : 0) &&
         put_vec(f, m->face_node_indices, m->n_face_nodes);
    ok = ok && put_vec(f, m->volume, nC) && put_vec(f, m->cell_centroid_x, nC) &&
         put_vec(f, m->cell_centroid_y, nC) && put_vec(f, m->cell_centroid_z, nC);
    ok = ok && put_vec(f, m->cell_face_offsets, m->cell_face_offsets ? nC + 1 : 0) &&
         put_vec(f, m->cell_face_indices, m->n_cell_faces);
    const uint32_t ns = static_cast<uint32_t>(fields->scalars.size()), nv = static_cast<uint32_t>(fields->vectors.size());
    ok = ok && put(f, &ns, 4) && put(f, &nv, 4);
    if (!ok)
        return fail(ctx, SIMALL_ERR_IO, "checkpoint: write failed");
    for (auto *fl : fields->scalars) {
        if (!put_name(f, fl->name))
            return fail(ctx, SIMALL_ERR_IO, "checkpoint: write failed");
        e = put_device(ctx, st, f, fl->data.p, fl->n);
        if (e)
            return e;
    }
    for (auto *fl : fields->vectors) {
        if (!put_name(f, fl->name))
            return fail(ctx, SIMALL_ERR_IO, "checkpoint: write failed");
        for (int c = 0; c < 3 && !e; ++c)
            e = put_device(ctx, st, f, fl->data.p ? fl->data.p + c * fl->n : nullptr, fl->n);
        if (e)
            return e;
    }
    if (std::fflush(f) != 0)
        return fail(ctx, SIMALL_ERR_IO, "checkpoint: flush failed");
    std::fclose(file.f);
    file.f = nullptr;
    if (std::rename(tmp.c_str(), path) != 0)
        return fail(ctx, SIMALL_ERR_IO, "checkpoint: rename to %s failed", path);
    return SIMALL_OK;
}

void simall_checkpoint_mesh_free(simall_checkpoint_mesh *m)
{
    if (!m)
        return;
    const void *arrays[] = {m->node_x,   m->node_y,     m->node_z,     m->owner,
                            m->neighbor, m->area_x,     m->area_y,     m->area_z,
                            m->centroid_x, m->centroid_y, m->centroid_z, m->boundary_zone,
                            m->face_node_offsets, m->face_node_indices, m->volume, m->cell_centroid_x,
                            m->cell_centroid_y, m->cell_centroid_z, m->cell_face_offsets, m->cell_face_indices};
    for (const void *p : arrays)
        std::free(const_cast<void *>(p));
    std::memset(m, 0, sizeof(*m));
}

int simall_checkpoint_read(const char *path, simall_fields *fields, simall_checkpoint_meta *meta,
                           simall_checkpoint_mesh *mesh_out)
{
    if (!path || !fields)
        return SIMALL_ERR_INVALID_ARGUMENT;
    simall_context *ctx = fields->ctx;
    SIMALL_CUDA_TRY(ctx, cudaSetDevice(ctx->device));
    File file;
    file.f = std::fopen(path, "rb");
    if (!file.f)
        return fail(ctx, SIMALL_ERR_IO, "checkpoint: cannot open %s", path);
    FILE *f = file.f;
    unsigned char hdr[24], mt[24];
    if (!get(f, hdr, 24) || std::memcmp(hdr, "SIMALLCP", 8) != 0)
        return fail(ctx, SIMALL_ERR_FORMAT, "checkpoint: bad magic");
    uint32_t version = 0;
    std::memcpy(&version, hdr + 8, 4);
    if (version > 1)
        return fail(ctx, SIMALL_ERR_FORMAT, "checkpoint: version %u not supported", version);
    if (!get(f, mt, 24))
        return fail(ctx, SIMALL_ERR_FORMAT, "checkpoint: truncated");
    simall_checkpoint_meta md{};
    std::memcpy(&md.iteration, mt, 4);
    std::memcpy(&md.time, mt + 8, 8);
    std::memcpy(&md.settings_hash, mt + 16, 8);
    // the mesh section: read into caller-owned arrays, or skipped
    bool ok = true;
    if (mesh_out) {
        simall_checkpoint_mesh m{};
        int64_t c[20] = {0};
        double *nx = nullptr, *ny = nullptr, *nz = nullptr, *ax = nullptr, *ay = nullptr, *az = nullptr;
        double *fx = nullptr, *fy = nullptr, *fz = nullptr, *vol = nullptr, *cx = nullptr, *cy = nullptr, *cz = nullptr;
        uint64_t *own = nullptr, *nb = nullptr, *fni = nullptr, *cfi = nullptr;
        uint32_t *zone = nullptr;
        int32_t *fno = nullptr, *cfo = nullptr;
        ok = get_vec(f, nx, c[0]) && get_vec(f, ny, c[1]) && get_vec(f, nz, c[2]) && get_vec(f, own, c[3]) &&
             get_vec(f, nb, c[4]) && get_vec(f, ax, c[5]) && get_vec(f, ay, c[6]) && get_vec(f, az, c[7]) &&
             get_vec(f, fx, c[8]) && get_vec(f, fy, c[9]) && get_vec(f, fz, c[10]) && get_vec(f, zone, c[11]) &&
             get_vec(f, fno, c[12]) && get_vec(f, fni, c[13]) && get_vec(f, vol, c[14]) && get_vec(f, cx, c[15]) &&
             get_vec(f, cy, c[16]) && get_vec(f, cz, c[17]) && get_vec(f, cfo, c[18]) && get_vec(f, cfi, c[19]);
        m.node_x = nx;
        m.node_y = ny;
        m.node_z = nz;
        m.owner = own;
        m.neighbor = nb;
        m.area_x = ax;
        m.area_y = ay;
        m.area_z = az;
        m.centroid_x = fx;
        m.centroid_y = fy;
        m.centroid_z = fz;
        m.boundary_zone = zone;
        m.face_node_offsets = fno;
        m.face_node_indices = fni;
        m.volume = vol;
        m.cell_centroid_x = cx;
        m.cell_centroid_y = cy;
        m.cell_centroid_z = cz;
        m.cell_face_offsets = cfo;
        m.cell_face_indices = cfi;
        m.n_nodes = c[0];
        m.n_faces = c[3];
        m.n_cells = c[14];
        m.n_face_nodes = c[13];
        m.n_cell_faces = c[19];
        if (!ok) {
            simall_checkpoint_mesh_free(&m);
            return fail(ctx, SIMALL_ERR_FORMAT, "checkpoint: truncated mesh section");
        }
        *mesh_out = m;
    } else {
        const size_t elem[20] = {8, 8, 8, 8, 8, 8, 8, 8, 8, 8, 8, 4, 4, 8, 8, 8, 8, 8, 4, 8};
        for (int i = 0; i < 20 && ok; ++i)
            ok = skip_vec(f, elem[i]);
        if (!ok)
            return fail(ctx, SIMALL_ERR_FORMAT, "checkpoint: truncated mesh section");
    }
    auto fail_mesh = [&](int status, const char *what) {
        if (mesh_out)
            simall_checkpoint_mesh_free(mesh_out);
        return fail(ctx, status, "checkpoint: %s", what);
    };
    uint32_t ns = 0, nv = 0;
    if (!get(f, &ns, 4) || !get(f, &nv, 4))
        return fail_mesh(SIMALL_ERR_FORMAT, "truncated field section");
    Staging st(ctx);
    int e = st.init();
    if (e)
        return e;
    for (uint32_t i = 0; i < ns + nv; ++i) {
        const bool vec = i >= ns;
        uint32_t len = 0;
        if (!get(f, &len, 4) || len > (1u << 20))
            return fail_mesh(SIMALL_ERR_FORMAT, "bad field name");
        std::string name(len, '\0');
        if (!get(f, name.data(), len))
            return fail_mesh(SIMALL_ERR_FORMAT, "truncated field name");
        uint64_t n = 0;
        if (!get(f, &n, 8) || n > (uint64_t(1) << 40))
            return fail_mesh(SIMALL_ERR_FORMAT, "bad field size");
        int gst = SIMALL_OK;
        simall_fields::Field *fl = registry_get(fields, name.c_str(), static_cast<int64_t>(n), vec, &gst);
        if (!fl) {
            if (mesh_out)
                simall_checkpoint_mesh_free(mesh_out);
            return gst;
        }
        e = get_device(ctx, st, f, fl->data.p, static_cast<int64_t>(n));
        for (int c = 1; vec && c < 3 && !e; ++c) {
            uint64_t nc = 0;
            if (!get(f, &nc, 8) || nc != n)
                return fail_mesh(SIMALL_ERR_FORMAT, "vector components of different sizes");
            e = get_device(ctx, st, f, fl->data.p + c * n, static_cast<int64_t>(n));
        }
        if (e) {
            if (mesh_out)
                simall_checkpoint_mesh_free(mesh_out);
            return e;
        }
    }
    if (meta)
        *meta = md;
    return SIMALL_OK;
}

}  // extern "C"
