// SIMP topology optimisation on the device: the GB300 replacement of
// optimization::SimpTopology (src/optimization/SimpTopology.cpp:18-227), with
// its fields in a device field registry.
//
//   filter      the Helmholtz system -r^2 lap(rt) + rt = rho assembled per
//               cell on the mesh's CSR pattern (volume on the diagonal, r^2
//               |A| / |d| per interior face, faces in ascending id as the
//               reference's face loop adds them) and solved by this library's
//               CG + Jacobi (tol 1e-9, 400 iterations, as the reference's
//               filter solver); rhoTilde = clamp(x, 0, 1)
//   property    K_simp = K_min + (K_max - K_min) rhoTilde^p
//   sensitivity dC_drho through the filter (radius > 0: the reference
//               overwrites rho with dC_drho and filters it) or copied
//   OC update   bisection on the volume multiplier: each halving is one
//               kernel that writes every cell's candidate density and sums
//               the volume, its last CTA moving the bracket; later halvings
//               return at once when the bracket has closed, so the last
//               candidate written is the one the reference keeps
// Every field stays in HBM; the host reads one scalar (the change) per step.
#include "device.cuh"
#include "pressure_system.hpp"
#include "registry.hpp"
#include "solver.hpp"

#include <new>

struct simall_simp {
    simall_context *ctx = nullptr;
    simall_pressure_system *ps = nullptr;
    simall_fields *fields = nullptr;
    simall_simp_config cfg{};
    simall_solver *filter = nullptr;
    simall::DevBuf<double> coef, values, b, x, rhoNew, partials, scal;
    double *h_scal = nullptr;  // pinned: [0] change
};

namespace simall {

namespace {

// OC bisection state: l1, l2, Vtarget, Vtot, change; ints: halvings, done
struct OcState {
    double l1, l2, vtarget, vtot, change;
    int halvings, done;
    unsigned counter[4];
};

__global__ void __launch_bounds__(kBlock) k_helm_face(int64_t nF, double r2, const int32_t *__restrict__ neighbor,
                                                      const double *__restrict__ amag2,
                                                      const double *__restrict__ dx, const double *__restrict__ dy,
                                                      const double *__restrict__ dz, double *__restrict__ coef)
{
    for (int64_t f = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; f < nF; f += (int64_t)gridDim.x * blockDim.x) {
        double c = 0.0;  // boundary, or a degenerate face: no coupling (adding 0 leaves every slot unchanged)
        if (neighbor[f] >= 0) {
            const double a = sqrt(amag2[f]);
            const double d = sqrt(
                __dadd_rn(__dadd_rn(__dmul_rn(dx[f], dx[f]), __dmul_rn(dy[f], dy[f])), __dmul_rn(dz[f], dz[f])));
            if (!(d <= 0) && !(a <= 0))
                c = __ddiv_rn(__dmul_rn(r2, a), d);
        }
        coef[f] = c;
    }
}

__global__ void __launch_bounds__(kBlock) k_helm_rows(int64_t nC, const int32_t *__restrict__ rowPtr,
                                                      const int32_t *__restrict__ cfOff,
                                                      const int32_t *__restrict__ cfEnt,
                                                      const int32_t *__restrict__ cfSlot,
                                                      const int32_t *__restrict__ diagSlot,
                                                      const int32_t *__restrict__ neighbor,
                                                      const double *__restrict__ coef, const double *__restrict__ vol,
                                                      double *__restrict__ values)
{
    for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < nC; c += (int64_t)gridDim.x * blockDim.x) {
        for (int k = rowPtr[c]; k < rowPtr[c + 1]; ++k)
            values[k] = 0.0;
        double diag = vol[c];
        for (int e = cfOff[c]; e < cfOff[c + 1]; ++e) {
            const int f = cfEnt[e] & 0x7fffffff;
            if (neighbor[f] < 0)
                continue;
            const double cf = __ldg(coef + f);
            diag = __dadd_rn(diag, cf);
            const int slot = cfSlot[e];
            if (slot >= 0)
                values[slot] = __dadd_rn(values[slot], -cf);
        }
        values[diagSlot[c]] = diag;
    }
}

__global__ void __launch_bounds__(kBlock) k_mul(int64_t n, const double *__restrict__ a, const double *__restrict__ b,
                                                double *__restrict__ out)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        out[i] = __dmul_rn(a[i], b[i]);
}

// std::clamp(x, 0, 1) as min(max(x, 0), 1)
__global__ void __launch_bounds__(kBlock) k_clamp01(int64_t n, const double *__restrict__ x, double *__restrict__ out)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const double v = x[i];
        const double m = v < 0.0 ? 0.0 : v;
        out[i] = 1.0 < m ? 1.0 : m;
    }
}

__global__ void __launch_bounds__(kBlock) k_copy(int64_t n, const double *__restrict__ a, double *__restrict__ out)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        out[i] = a[i];
}

__global__ void __launch_bounds__(kBlock) k_ksimp(int64_t n, double kmin, double dk, double p,
                                                  const double *__restrict__ rt, double *__restrict__ k)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        k[i] = __dadd_rn(kmin, __dmul_rn(dk, pow(rt[i], p)));
}

__global__ void __launch_bounds__(kBlock) k_oc_init(int64_t n, const double *__restrict__ vol, double vf,
                                                    double *partials, OcState *s)
{
    double acc[1] = {0.0};
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        acc[0] += vol[i];
    if (grid_sum_last<1>(acc, partials, &s->counter[0]) && threadIdx.x == 0) {
        s->vtot = acc[0];
        s->vtarget = __dmul_rn(vf, acc[0]);
        s->l1 = 0.0;
        s->l2 = 1e9;
        s->halvings = 0;
        s->done = 0;
    }
}

// One halving: candidates for lmid = (l1 + l2) / 2 and their volume.
__global__ void __launch_bounds__(kBlock) k_oc_step(int64_t n, double damping, double move, double rhoMin,
                                                    const double *__restrict__ dCt, const double *__restrict__ rho,
                                                    const double *__restrict__ vol, double *__restrict__ rhoNew,
                                                    double *partials, OcState *s)
{
    if (__ldcg(&s->done))
        return;
    const double l1 = __ldcg(&s->l1), l2 = __ldcg(&s->l2);
    const double lmid = __dmul_rn(0.5, __dadd_rn(l1, l2));
    const double den = std_max(1e-12, lmid);
    double acc[1] = {0.0};
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const double sv = __ddiv_rn(-dCt[i], den);
        const double bf = pow(std_max(0.0, sv), damping);
        const double old = rho[i];
        const double lo = std_max(rhoMin, __dsub_rn(old, move));
        const double om = __dadd_rn(old, move);
        const double hi = om < 1.0 ? om : 1.0;
        const double t = __dmul_rn(old, bf);
        const double mx = t < lo ? lo : t;
        const double v = hi < mx ? hi : mx;
        rhoNew[i] = v;
        acc[0] += v * vol[i];
    }
    if (grid_sum_last<1>(acc, partials, &s->counter[1]) && threadIdx.x == 0) {
        if (acc[0] > s->vtarget)
            s->l1 = lmid;
        else
            s->l2 = lmid;
        s->halvings += 1;
        const double a = s->l1, b = s->l2;
        if (s->halvings >= 64 || !((b - a) > 1e-9 * (a + b + 1e-30)))
            s->done = 1;
    }
}

// change = sum |rhoNew - rho| / n; rho = rhoNew
__global__ void __launch_bounds__(kBlock) k_oc_finish(int64_t n, const double *__restrict__ rhoNew,
                                                      double *__restrict__ rho, double *partials, OcState *s)
{
    double acc[1] = {0.0};
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        acc[0] += fabs(rhoNew[i] - rho[i]);
        rho[i] = rhoNew[i];
    }
    if (grid_sum_last<1>(acc, partials, &s->counter[2]) && threadIdx.x == 0)
        s->change = acc[0] / static_cast<double>(n);
}

int grid_cells(simall_context *ctx, int64_t n)
{
    const int64_t g = (n + kBlock - 1) / kBlock;
    const int64_t cap = grid_size_streaming(ctx);
    return static_cast<int>(g < 1 ? 1 : (g < cap ? g : cap));
}

}  // namespace

}  // namespace simall

using namespace simall;

namespace {

simall_fields::Field *field(simall_simp *s, const char *name, int *st)
{
    return registry_get(s->fields, name, s->ps->nC, false, st);
}

// rhoTilde = filter(rho): SimpTopology::apply_helmholtz_filter.
int helmholtz(simall_simp *s, const double *rho, double *rhoT)
{
    simall_context *ctx = s->ctx;
    simall_pressure_system *ps = s->ps;
    const int64_t nC = ps->nC;
    const int g = grid_cells(ctx, nC);
    if (s->cfg.filter_radius <= 0.0) {
        k_copy<<<g, kBlock, 0, ctx->stream>>>(nC, rho, rhoT);
        SIMALL_LAUNCH_CHECK(ctx);
        return SIMALL_OK;
    }
    k_mul<<<g, kBlock, 0, ctx->stream>>>(nC, rho, ps->vol.p, s->b.p);
    SIMALL_LAUNCH_CHECK(ctx);
    simall_solver_stats st{};
    int e = solver_solve_impl(s->filter, s->b.p, SIMALL_MEM_DEVICE, s->x.p, SIMALL_MEM_DEVICE, &st);
    if (e)
        return e;
    k_clamp01<<<g, kBlock, 0, ctx->stream>>>(nC, s->x.p, rhoT);
    SIMALL_LAUNCH_CHECK(ctx);
    return SIMALL_OK;
}

}  // namespace

extern "C" {

void simall_simp_config_default(simall_simp_config *c)
{
    if (!c)
        return;
    // SimpConfig defaults (src/optimization/SimpTopology.hpp:36-46)
    c->penalty = 3.0;
    c->K_min = 1e-9;
    c->K_max = 1.0;
    c->filter_radius = 0.0;
    c->volume_fraction = 0.4;
    c->move = 0.2;
    c->damping = 0.5;
    c->rho_min = 1e-3;
}

int simall_simp_create(simall_pressure_system *ps, simall_fields *fields, const simall_simp_config *cfg,
                       simall_simp **out)
{
    if (!ps || !fields || !out || fields->ctx != ps->ctx)
        return SIMALL_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    simall_context *ctx = ps->ctx;
    if (!ps->fieldsReady)
        return fail(ctx, SIMALL_ERR_INVALID_ARGUMENT, "SIMP: call simall_pressure_system_setup_field_loops first");
    SIMALL_CUDA_TRY(ctx, cudaSetDevice(ctx->device));
    auto *s = new (std::nothrow) simall_simp;
    if (!s)
        return SIMALL_ERR_OUT_OF_MEMORY;
    s->ctx = ctx;
    s->ps = ps;
    s->fields = fields;
    simall_simp_config_default(&s->cfg);
    if (cfg)
        s->cfg = *cfg;
    const int64_t nC = ps->nC, nF = ps->nF;
    auto bail = [&](int st) {
        if (s->filter)
            simall_solver_destroy(s->filter);
        if (s->h_scal)
            cudaFreeHost(s->h_scal);
        delete s;
        return st;
    };
    cudaError_t ce = cudaSuccess;
    for (auto *b : {&s->b, &s->x, &s->rhoNew})
        if (ce == cudaSuccess)
            ce = b->alloc(nC);
    if (ce == cudaSuccess)
        ce = s->partials.alloc(static_cast<size_t>(grid_size_streaming(ctx)) * kMaxReduce);
    if (ce == cudaSuccess)
        ce = s->scal.alloc((sizeof(OcState) + 7) / 8);
    if (ce == cudaSuccess)
        ce = cudaMemsetAsync(s->scal.p, 0, sizeof(OcState), ctx->stream);
    if (ce == cudaSuccess)
        ce = cudaMallocHost(reinterpret_cast<void **>(&s->h_scal), sizeof(double));
    if (ce != cudaSuccess)
        return bail(cuda_fail(ctx, ce, "SIMP allocation", __FILE__, __LINE__));
    // SimpTopology::initialize: rho = rhoTilde = volumeFraction, K_simp = K_min, sensitivities 0
    const char *names[5] = {"rho", "rhoTilde", "K_simp", "dC_drho", "dC_drhoTilde"};
    const double init[5] = {s->cfg.volume_fraction, s->cfg.volume_fraction, s->cfg.K_min, 0.0, 0.0};
    std::vector<double> h(static_cast<size_t>(nC));
    for (int i = 0; i < 5; ++i) {
        int st = SIMALL_OK;
        simall_fields::Field *f = registry_get(fields, names[i], nC, false, &st);
        if (!f)
            return bail(st);
        std::fill(h.begin(), h.end(), init[i]);
        ce = cudaMemcpy(f->data.p, h.data(), nC * sizeof(double), cudaMemcpyHostToDevice);
        if (ce != cudaSuccess)
            return bail(cuda_fail(ctx, ce, "SIMP initial fields", __FILE__, __LINE__));
    }
    if (s->cfg.filter_radius > 0.0) {
        // the filter matrix is geometric: assembled once on the mesh's pattern
        if ((ce = s->coef.alloc(nF)) != cudaSuccess || (ce = s->values.alloc(ps->nnz)) != cudaSuccess)
            return bail(cuda_fail(ctx, ce, "SIMP filter allocation", __FILE__, __LINE__));
        const double r2 = s->cfg.filter_radius * s->cfg.filter_radius;
        k_helm_face<<<grid_cells(ctx, nF), kBlock, 0, ctx->stream>>>(nF, r2, ps->neighbor.p, ps->amag2.p, ps->gdx.p,
                                                                      ps->gdy.p, ps->gdz.p, s->coef.p);
        ctx->launches.fetch_add(1, std::memory_order_relaxed);
        k_helm_rows<<<grid_cells(ctx, nC), kBlock, 0, ctx->stream>>>(nC, ps->rowPtr.p, ps->cfOff.p, ps->cfEnt.p,
                                                                      ps->cfSlot.p, ps->diagSlot.p, ps->neighbor.p,
                                                                      s->coef.p, ps->vol.p, s->values.p);
        ctx->launches.fetch_add(1, std::memory_order_relaxed);
        if ((ce = cudaGetLastError()) != cudaSuccess)
            return bail(cuda_fail(ctx, ce, "SIMP filter assembly", __FILE__, __LINE__));
        simall_solver_config fc;
        simall_solver_config_default(&fc);  // CG, Jacobi, FP64
        fc.tolerance = 1e-9;
        fc.max_iterations = 400;
        int st = simall_solver_create(ctx, &fc, &s->filter);
        if (!st)
            st = simall_solver_set_matrix(s->filter, nC, ps->nnz, ps->rowPtr.p, ps->colIdx.p, s->values.p,
                                          SIMALL_MEM_DEVICE);
        if (st)
            return bail(st);
    }
    SIMALL_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
    *out = s;
    return SIMALL_OK;
}

int simall_simp_destroy(simall_simp *s)
{
    if (!s)
        return SIMALL_ERR_INVALID_ARGUMENT;
    cudaStreamSynchronize(s->ctx->stream);
    if (s->filter)
        simall_solver_destroy(s->filter);
    if (s->h_scal)
        cudaFreeHost(s->h_scal);
    delete s;
    return SIMALL_OK;
}

int simall_simp_step(simall_simp *s, double *change)
{
    if (!s)
        return SIMALL_ERR_INVALID_ARGUMENT;
    simall_context *ctx = s->ctx;
    SIMALL_CUDA_TRY(ctx, cudaSetDevice(ctx->device));
    const int64_t nC = s->ps->nC;
    int st = SIMALL_OK;
    simall_fields::Field *rho = field(s, "rho", &st), *rt = rho ? field(s, "rhoTilde", &st) : nullptr,
                         *ks = rt ? field(s, "K_simp", &st) : nullptr, *dc = ks ? field(s, "dC_drho", &st) : nullptr,
                         *dct = dc ? field(s, "dC_drhoTilde", &st) : nullptr;
    if (!dct)
        return st ? st : SIMALL_ERR_INVALID_ARGUMENT;
    const simall_simp_config &c = s->cfg;
    const int g = grid_cells(ctx, nC);
    int e = helmholtz(s, rho->data.p, rt->data.p);
    if (e)
        return e;
    k_ksimp<<<g, kBlock, 0, ctx->stream>>>(nC, c.K_min, c.K_max - c.K_min, c.penalty, rt->data.p, ks->data.p);
    SIMALL_LAUNCH_CHECK(ctx);
    if (c.filter_radius > 0.0) {
        // as the reference: rho takes the sensitivity, which is filtered into rhoTilde and copied to dC_drhoTilde
        k_copy<<<g, kBlock, 0, ctx->stream>>>(nC, dc->data.p, rho->data.p);
        SIMALL_LAUNCH_CHECK(ctx);
        e = helmholtz(s, rho->data.p, rt->data.p);
        if (e)
            return e;
        k_copy<<<g, kBlock, 0, ctx->stream>>>(nC, rt->data.p, dct->data.p);
        SIMALL_LAUNCH_CHECK(ctx);
    } else {
        k_copy<<<g, kBlock, 0, ctx->stream>>>(nC, dc->data.p, dct->data.p);
        SIMALL_LAUNCH_CHECK(ctx);
    }
    OcState *os = reinterpret_cast<OcState *>(s->scal.p);
    k_oc_init<<<g, kBlock, 0, ctx->stream>>>(nC, s->ps->vol.p, c.volume_fraction, s->partials.p, os);
    SIMALL_LAUNCH_CHECK(ctx);
    for (int it = 0; it < 64; ++it) {
        k_oc_step<<<g, kBlock, 0, ctx->stream>>>(nC, c.damping, c.move, c.rho_min, dct->data.p, rho->data.p,
                                                 s->ps->vol.p, s->rhoNew.p, s->partials.p, os);
        SIMALL_LAUNCH_CHECK(ctx);
    }
    k_oc_finish<<<g, kBlock, 0, ctx->stream>>>(nC, s->rhoNew.p, rho->data.p, s->partials.p, os);
    SIMALL_LAUNCH_CHECK(ctx);
    SIMALL_CUDA_TRY(ctx, cudaMemcpyAsync(s->h_scal, &os->change, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    SIMALL_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
    if (change)
        *change = s->h_scal[0];
    return SIMALL_OK;
}

}  // extern "C"
