// The solver object behind simall_solver_* (shared by pcg.cu, ilu0.cu, mixed.cu).
#pragma once

#include "internal.hpp"

namespace simall {

// Level-scheduled ILU(0) data (ilu0.cu).
struct IluData {
    DevBuf<double> lu;          // factored values on A's pattern
    DevBuf<int32_t> diagPtr;    // position of the diagonal in each row (-1 if missing)
    DevBuf<int32_t> fwdRows;    // rows grouped by forward level
    DevBuf<int32_t> bwdRows;    // rows grouped by backward level
    DevBuf<double> y;           // forward-sweep scratch
    DevBuf<unsigned> sweepCtl;  // sweeps: [0] work ticket, [2] wait-timeout flag
    std::vector<int32_t> fwdLevelPtr, bwdLevelPtr;  // level boundaries into fwdRows / bwdRows (host)
    DevBuf<int32_t> fwdLvl, bwdLvl;                 // the same on the device (single-CTA path)
    std::vector<int32_t> h_diagPtr;
    int maxLevelRows = 0;
    bool analysed = false;
    // small systems: factor and sweeps in one CTA (ilu0.cu); the sweeps' rows in
    // level order, each with its triangle's entries packed at a fixed stride
    bool small = false;
    int kf = 0, kb = 0, stageRows = 0, stageBytes = 0, smallSmem = 0, smallThreads = 0;
    DevBuf<int32_t> frow, brow, fcol, bcol, fpos, bpos;
    DevBuf<double> fval, bval, bdiag, brdiag;  // refreshed from lu after every factorisation
    DevBuf<double> rpiv;                        // reciprocals of the pivots (factor)
    DevBuf<double> rdiag;                       // larger systems: RN(1/u_ii) of the factor, for the backward sweep
    // SSOR (w = 1) runs on the same level schedule: no factor, lu holds A's
    // values, the sweeps scale by the inverse diagonal invD (the Jacobi one)
    int mode = 0;                  // 0 ILU(0), 1 SSOR
    const double *invD = nullptr;  // SSOR: 1/a_ii (1.0 where a_ii == 0)
    DevBuf<double> frdiag;         // SSOR, single-CTA path: invD in forward level order
};

struct MixedData;  // mixed.cu
struct AmgData;    // amg.cu
struct KrylovData;  // krylov.cu

// Chunk of solver iterations captured as a CUDA graph.
struct GraphChunk {
    cudaGraphExec_t exec = nullptr;
    int len = 0;
};

}  // namespace simall

struct simall_solver {
    simall_context *ctx = nullptr;
    simall_solver_config cfg{};
    int64_t n = 0, nnz = 0;
    const int32_t *rowPtr = nullptr;
    const int32_t *colIdx = nullptr;
    const double *values = nullptr;
    // the current pattern (always a private device copy) and the staging pair
    // a new pattern is uploaded into before it is compared with the current one
    simall::DevBuf<int32_t> own_rowPtr, own_colIdx, new_rowPtr, new_colIdx;
    simall::DevBuf<double> own_values;
    std::vector<int32_t> h_rowPtr, h_colIdx;  // host copy of the pattern, filled on demand
    bool h_pattern_valid = false;
    bool have_pattern = false;
    simall::DevBuf<int32_t> rowBlocks;
    int nRowBlocks = 0;
    simall::DevBuf<double> invDiag, x, r, p, Ap, z, b;
    simall::DevBuf<double> partials;
    simall::DevBuf<simall::SolveScalars> scal;
    simall::SolveScalars *h_scal = nullptr;  // pinned mirror
    simall::DevBuf<int> flag;               // device check results
    double last_residual = 0.0;
    bool ready = false;
    bool solved = false;  // a solve completed on the current matrix
    int engine = 0;       // of the last solve: 0 kernels per step, 1 one cluster, 2 one persistent grid
    simall::IluData *ilu = nullptr;
    simall::AmgData *amg = nullptr;
    simall::MixedData *mixed = nullptr;
    simall::KrylovData *krylov = nullptr;
    std::vector<simall::GraphChunk> graphs;  // captured iteration chunks
};

namespace simall {

// Row schedule passed as nRB to the SpMV helpers of device.cuh: matrices
// whose rows are short on average (at most 16 nonzeros) run one thread per
// row without staging (-n), others the staged row-blocks.  spmv_items: the
// threads the schedule wants, for sizing the grid.
inline bool spmv_direct(const simall_solver *s) { return s->nnz <= 16 * s->n; }
inline int spmv_schedule(const simall_solver *s)
{
    return spmv_direct(s) ? -static_cast<int>(s->n) : s->nRowBlocks;
}
inline int64_t spmv_items(const simall_solver *s)
{
    return spmv_direct(s) ? s->n : static_cast<int64_t>(s->nRowBlocks) * kBlock;
}

// The preconditioners applied by kernels of their own (ILU(0) and SSOR
// sweeps, the AMG V-cycle) rather than fused into the Krylov updates as
// Jacobi is.  ilu_setup / ilu_apply / ilu_check / ilu_apply_launches serve
// all three (AMG through amg_*).
inline bool sweep_preconditioner(int pc)
{
    return pc == SIMALL_PRECOND_ILU0 || pc == SIMALL_PRECOND_SSOR || pc == SIMALL_PRECOND_AMG;
}
// Launch shape and polling back-off of the free-running triangular sweeps
// (ILU(0), SSOR, the AMG smoother's large levels): CTAs per SM of the sweep
// grid and the longest sleep between polls (ns; 0 = spin).  Process-wide;
// simall_diagnose_sweep_params changes them for latency measurements.
extern int g_sweep_ctas_per_sm;
extern unsigned g_sweep_backoff_ns;
extern bool g_sweep_reciprocal;  // ILU(0) backward sweep: divide through RN(1/u_ii) (same bits)
int ilu_setup(simall_solver *s);  // ILU(0) factor, SSOR's sweep data or the AMG hierarchy (cfg.preconditioner)
int ilu_check(simall_solver *s);  // a sweep wait timed out -> error
int ilu_apply(simall_solver *s, const double *r, double *z);
int ilu_apply_launches(const simall_solver *s);  // kernels one ilu_apply enqueues
void ilu_free(simall_solver *s);

// AMG (amg.cu): hierarchy built on the host for the current values, V-cycle on the device.
int amg_setup(simall_solver *s);
int amg_apply(simall_solver *s, const double *r, double *z);
int amg_check(simall_solver *s);
int amg_apply_launches(const simall_solver *s);
int amg_levels(const simall_solver *s, int *nlev, int32_t *rows, int max_levels);
void amg_free(simall_solver *s);

int mixed_setup(simall_solver *s);
void mixed_invalidate_pattern(simall_solver *s);
int mixed_solve(simall_solver *s, simall_solver_stats *st);
// Enqueue one launch of mixed kernel k (4..6) and its algorithmic bytes.
int mixed_enqueue_kernel(simall_solver *s, int k, double *bytes);
void mixed_free(simall_solver *s);

// simall_solver_solve with separate memory kinds for b and x.
int solver_solve_impl(simall_solver *s, const double *b, int bmem, double *x, int xmem, simall_solver_stats *stats);
// Whole-solve FP64 Jacobi PCG on one thread-block cluster for systems that fit
// (cluster.cu); 0 = not taken, 1 = taken with *status set.
int cluster_fp64_solve(simall_solver *s, int *status);
// The mixed solver's FP32 operator in diagonal storage (mixed.cu), for the
// whole-solve mixed-precision CG on one cluster.
struct ClusterMixedArgs {
    const float *U;        // [nd][ldU] upper diagonals of S A S
    int64_t ldU;
    int nd;
    int off[8];            // ascending offsets
    const float *e;        // 1 + row sums of S A S (row-sum form)
    const double *scale;   // S = D^-1/2
};
int cluster_mixed_solve(simall_solver *s, const ClusterMixedArgs &a, int *status);

// Batched solves (batched.cu): the per-system result, and the large systems
// of a batch solved one per thread-block cluster (cluster.cu).
struct ClBatchResult {
    int iterations;
    int updates;
    int status;
    int converged;
    double true_residual;
    double b_norm;
};
struct ClBatchItem {
    int n;      // rows
    int logR;   // slice length 2^logR of this launch
    int64_t row0;  // first row in the batch's b and x
    ClusterMixedArgs A;  // the system's S A S (diagonal storage), e and scale
    const int32_t *rowPtr;  // the system's FP64 CSR (local indices)
    const int32_t *colIdx;
    const double *val;
    ClBatchResult *out;
};
constexpr int kClBatchMaxRowsPerCta = 8192;
// `clusters` clusters of C CTAs stride through the `count` items (largest first).
int cluster_mixed_batch(simall_context *ctx, cudaStream_t stream, int nd, int C, int logR, int clusters,
                        const ClBatchItem *items, int count, const double *b, double *x, double tol, double delta,
                        int max_iter);

// The mixed solver's sliced operator (mixed.cu) and work vectors for the
// whole-solve persistent cooperative kernel (mixed_grid.cu); 0 = not taken
// (check_interval > 0, engine KERNELS, no cooperative launch), 1 = taken with
// *status set.  part holds partCap doubles (8 per CTA), ctr and err one word.
// the persistent mixed solve: one CTA of 800 threads (24-slice stages) per SM
// measured fastest at 128^3 (30.2 us per step, against 31.9 us with three
// 288-thread CTAs and 34.3 us with two 544-thread ones)
constexpr int kGridMaxCtasPerSm = 1;
// Mixed precision in sliced storage: stages ahead whose operands the staged
// steps prefetch into L2 (0 = none), and CTAs per SM of the persistent solve
// (0 = as many as fit).  Process-wide; simall_diagnose_mixed_params sets them.
extern int g_sell_prefetch;
extern int g_grid_ctas_per_sm;
// Resident CTAs per SM of a kernel of `threads` threads with `smem` bytes of
// dynamic shared memory (its limit raised first); cached per context and kernel.
int staged_residency(simall_context *ctx, const void *fn, int threads, size_t smem, int *per_sm);
struct GridMixedArgs {
    int64_t nslices;
    bool wide;
    bool staged;  // every slice at most kSellStageMaxW wide: TMA-staged steps
    const int32_t *sptr;
    const int16_t *off16;
    const int32_t *off32;
    const float *sval;
    const float *e;  // row sums, whole slices
    const double *scale;
    float4 *st[2];  // (r, q, p, xh) per row, by step parity (sell.cuh)
    double *part;
    size_t partCap;
    unsigned long long *ctr;
    int *err;
};
int grid_mixed_solve(simall_solver *s, const GridMixedArgs &a, int *status);

// The same persistent solve for symmetric diagonal storage (up to
// kGridDiaMaxDiags upper diagonals), the state in separate r, q, p vectors
// by step parity and one xh.  Returns 0 (not taken) or 1 with *status set.
constexpr int kGridDiaMaxDiags = 4;
struct GridDiaArgs {
    int nd;
    bool grid;  // offset 1 first, every other offset a multiple of 4
    int32_t off[8];
    int64_t ldU;
    const float *U;  // [nd][ldU] upper diagonals of S A S
    const float *e;  // row sums
    const double *scale;
    float *rv[2], *qv[2], *pv[2];
    float *xh;
    double *part;
    size_t partCap;
    unsigned long long *ctr;
    int *err;
};
int grid_dia_solve(simall_solver *s, const GridDiaArgs &a, int *status);

// GMRES(m) / BiCGSTAB (krylov.cu): solve from x = 0 into s->x; fills the
// result fields of s->h_scal.
int krylov_solve(simall_solver *s);
void krylov_drop_graphs(simall_solver *s);
void krylov_free(simall_solver *s);

// The autotuner cache's default path (autotune_cache.cpp).
std::string default_autotune_cache_path();

// Host copy of the current pattern (ILU0 level analysis, CSR fallbacks).
int solver_host_pattern(simall_solver *s);

// Shared by the FP64 and mixed paths.
int solver_true_residual(simall_solver *s, const double *x, const double *b, double *r, double *rr);
int solver_fetch_scalars(simall_solver *s);

}  // namespace simall
