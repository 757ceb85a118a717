/*
 * simall_gpu.h -- C ABI of the GB300 (sm_103a) pressure-correction library.
 *
 * One shared library, libsimall_gpu.so, replaces SimAll's pressure-correction
 * hot path: the face-loop assembly of the pressure-correction Laplacian into
 * the solver's CSR matrix and the preconditioned CG solve on it.  Every entry
 * point is extern "C", takes plain pointers and sizes, returns an int status
 * (SIMALL_OK == 0) and never lets an exception cross the boundary.  Each
 * declaration names the reference interface it replaces (file:line inside the
 * SimAll source tree).
 *
 * Memory: arguments tagged `mem` are host pointers when mem ==
 * SIMALL_MEM_HOST (the call copies them host<->device on the context stream
 * and returns after the result is back on the host) and device pointers when
 * mem == SIMALL_MEM_DEVICE (no copies; the call returns once the result is
 * final in device memory).  Device pointers must be 16-byte aligned.
 *
 * Threading: an object is used by one host thread at a time (as
 * solver::ILinearSolver, src/solver/Solver.hpp:92-100).  All GPU work of a
 * context is ordered on its stream.
 */
#ifndef SIMALL_GPU_H
#define SIMALL_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ------------------------------------------------------------------ status */
enum simall_status {
    SIMALL_OK = 0,
    SIMALL_ERR_INVALID_ARGUMENT = 1, /* null pointer, negative size, bad enum */
    SIMALL_ERR_CUDA = 2,             /* a CUDA runtime call failed; see last_error */
    SIMALL_ERR_OUT_OF_MEMORY = 3,
    SIMALL_ERR_UNSORTED_CSR = 4,     /* a CSR row is not strictly ascending / rowPtr not monotone */
    SIMALL_ERR_MISSING_DIAGONAL = 5, /* a row has no diagonal entry where the method needs one */
    SIMALL_ERR_NON_FINITE = 6,       /* NaN or Inf in an input array */
    SIMALL_ERR_NOT_POSITIVE = 7,     /* non-positive diagonal (mixed precision needs D > 0) */
    SIMALL_ERR_SIZE_MISMATCH = 8,
    SIMALL_ERR_BREAKDOWN = 9,        /* p.Ap == 0 (the reference returns early the same way) */
    SIMALL_ERR_TIMEOUT = 10,         /* a bounded device-side wait ran out */
    SIMALL_ERR_UNSUPPORTED = 11,
    SIMALL_ERR_NO_DEVICE = 12,
    SIMALL_ERR_INDEX_RANGE = 13,     /* a column / cell / face index outside [0, n) */
    SIMALL_ERR_IO = 14,              /* a file could not be opened, written or renamed */
    SIMALL_ERR_FORMAT = 15           /* not a checkpoint this library reads (magic, version) or truncated */
};

enum simall_memory { SIMALL_MEM_HOST = 0, SIMALL_MEM_DEVICE = 1 };

/* PreconditionerKind ordinals (src/solver/Solver.hpp:75-82).  SSOR is
 * SsorPreconditioner with make_preconditioner's w = 1
 * (src/solver/LinearSolvers.cpp:163-231, :247-248); AMG is AMGPreconditioner
 * with its default parameters (src/solver/AMGPreconditioner.cpp; hierarchy
 * built on the host for each new matrix, V-cycle on the device); both FP64
 * only.  None maps to Jacobi, as make_preconditioner's default branch does
 * (:240-254). */
enum simall_preconditioner {
    SIMALL_PRECOND_JACOBI = 0,
    SIMALL_PRECOND_ILU0 = 1,
    SIMALL_PRECOND_SSOR = 2,
    SIMALL_PRECOND_AMG = 3,
    SIMALL_PRECOND_NONE = 4
};

enum simall_precision {
    SIMALL_PRECISION_FP64 = 0, /* the reference CG, FP64 throughout */
    SIMALL_PRECISION_MIXED = 1 /* FP32 inner CG, FP64 true residual, reductions and x (Jacobi only) */
};

/* BCType ordinals (src/solver/Solver.hpp:105-123) used by the assembly. */
enum simall_bc_type {
    SIMALL_BC_WALL = 0,
    SIMALL_BC_NO_SLIP_WALL = 1,
    SIMALL_BC_MOVING_WALL = 2,
    SIMALL_BC_SLIP_WALL = 3,
    SIMALL_BC_VELOCITY_INLET = 4,
    SIMALL_BC_PRESSURE_INLET = 5,
    SIMALL_BC_MASS_FLOW_INLET = 6,
    SIMALL_BC_PRESSURE_OUTLET = 7,
    SIMALL_BC_OUTFLOW = 8,
    SIMALL_BC_SYMMETRY = 9,
    SIMALL_BC_AXISYMMETRIC = 10,
    SIMALL_BC_PERIODIC = 11
};

const char *simall_status_string(int status);
/* Library version string, e.g. "simall_gb300 0.1.0 sm_103a". */
const char *simall_version(void);

/* ------------------------------------------------------------------ context */
/* Replaces gpu::CudaContext (src/gpu/CudaContext.cpp:83-258): a device, a
 * stream and the library's device-resident scratch.  stream == NULL creates a
 * private non-blocking stream; otherwise the caller's cudaStream_t is used. */
typedef struct simall_context simall_context;
int simall_context_create(int device, void *stream, simall_context **out);
int simall_context_destroy(simall_context *ctx);
/* Message of the last failure on this context ("" if none). */
const char *simall_context_last_error(const simall_context *ctx);
int simall_context_synchronize(simall_context *ctx);
/* The cudaStream_t the context orders its work on. */
void *simall_context_stream(const simall_context *ctx);
/* Number of kernels this library launched on the context so far. */
int64_t simall_context_kernel_launches(const simall_context *ctx);

/* ------------------------------------------------------------------ Krylov solver */
/* Replaces solver::ILinearSolver / CGSolver (src/solver/Solver.hpp:92-100,
 * src/solver/LinearSolvers.cpp:415-459) and gpu::CgGpu
 * (src/gpu/CgGpu.hpp:87-124); with `kind` also GMRESmSolver, BiCGSTABSolver
 * and TfqmrSolver (make_linear_solver, src/solver/Solver.cpp:25-39). */
typedef struct simall_solver_config {
    int preconditioner;    /* simall_preconditioner; default Jacobi */
    double tolerance;      /* stop when ||r||/max(||b||,1e-30) < tolerance; default 1e-8 */
    int max_iterations;    /* default 1000 (LinearSolverConfig, Solver.hpp:83-90) */
    int precision;         /* simall_precision; default FP64 */
    double reliable_delta; /* mixed: iterated-residual drop that triggers an FP64 update; default 0.1 */
    int check_interval;    /* iterations between host polls of the device stop flag; 0 = automatic */
    int engine;            /* simall_engine: how the iteration runs; default SIMALL_ENGINE_AUTO */
    int kind;              /* simall_solver_kind; default SIMALL_SOLVER_CG */
    int restart;           /* GMRES(m): basis size m (LinearSolverConfig::restart); default 30 */
    int semantics;         /* simall_semantics; default SIMALL_SEMANTICS_CGSOLVER */
    double relative_orders; /* SIMALL_SEMANTICS_CGGPU: also stop once ||r|| <= ||r_0|| 10^-relative_orders
                               (GpuSolverConfig::relativeOrders, src/gpu/CgGpu.hpp:61-63); 0 = off */
} simall_solver_config;

/* Which reference solver's conventions a CG solve follows.
 * SIMALL_SEMANTICS_CGSOLVER: solver::CGSolver::solve (src/solver/LinearSolvers.cpp:
 *   420-451): x starts from 0; stop when ||r||/max(||b||,1e-30) < tolerance;
 *   None preconditioner means Jacobi (make_preconditioner); pAp == 0 ends the
 *   loop returning the iterations done.
 * SIMALL_SEMANTICS_CGGPU: gpu::CgGpu::solve (src/gpu/CgGpu.cpp:118-238): x is the
 *   initial guess (r = b - A x0) and the solution; stop when ||r||/bRef <=
 *   tolerance (bRef = ||b||, or 1 when b = 0) or, with relative_orders > 0,
 *   ||r|| <= ||r_0|| 10^-relative_orders, whichever comes first, also before the
 *   first iteration (then iterations = 0); None means no preconditioner (z = r);
 *   an ILU0 factor that meets a missing diagonal or a zero pivot
 *   (gpu::ilu0_factor_inplace, src/gpu/GpuKernels.cpp:345-401) makes the solver
 *   Jacobi from then on, as CgGpu::set_matrix does (CgGpu.cpp:64-82; reported in
 *   simall_solver_stats.preconditioner); |p.q| < 1e-300 ends the loop with
 *   iterations = 0, residual_norm = 0, converged = 0 and status
 *   SIMALL_ERR_BREAKDOWN, the values CgGpu::solve leaves (CgGpu.cpp:190-194).
 *   FP64 CG only, with Jacobi, ILU0 or None.  Jacobi applies r * (1/d) where
 *   CgGpu divides r / d: the two differ by at most one rounding per entry. */
enum simall_semantics { SIMALL_SEMANTICS_CGSOLVER = 0, SIMALL_SEMANTICS_CGGPU = 1 };

/* LinearSolverKind ordinals (src/solver/Solver.hpp:67-73).  CG is the pressure
 * path (FP64 or mixed precision); GMRES(m), BiCGSTAB and TFQMR (FP64, Jacobi,
 * ILU(0) or SSOR) follow GMRESmSolver::solve, BiCGSTABSolver::solve and
 * TfqmrSolver::solve (src/solver/LinearSolvers.cpp:268-343, :363-405,
 * :497-609), including their breakdown exits and return values. */
enum simall_solver_kind {
    SIMALL_SOLVER_GMRES = 0,
    SIMALL_SOLVER_BICGSTAB = 1,
    SIMALL_SOLVER_CG = 2,
    SIMALL_SOLVER_TFQMR = 3
};

/* SIMALL_ENGINE_AUTO: systems of up to 131,072 rows (Jacobi FP64, or mixed
 * precision in diagonal storage) run the whole solve on one thread-block
 * cluster; larger mixed-precision solves run the whole solve in one
 * persistent cooperative launch over all SMs, in sliced storage (any pattern
 * without diagonal structure, e.g. RCM-renumbered meshes) or in diagonal
 * storage with up to four upper diagonals (natural-order structured grids);
 * the rest, and any solver with check_interval > 0, launch kernels per
 * iteration (mixed precision: one device-side graph loop).
 * SIMALL_ENGINE_KERNELS: always the per-iteration kernels. */
enum simall_engine { SIMALL_ENGINE_AUTO = 0, SIMALL_ENGINE_KERNELS = 1 };

typedef struct simall_solver_stats {
    int iterations;          /* as CGSolver::solve returns: it+1 at convergence, maxIterations otherwise */
    int converged;           /* 1 when final_residual < tolerance */
    int status;              /* SIMALL_OK or SIMALL_ERR_BREAKDOWN */
    int reliable_updates;    /* mixed precision: FP64 residual replacements performed */
    double final_residual;   /* ||r||/max(||b||,1e-30) at exit (last_residual()) */
    double true_residual;    /* ||b - A x||/max(||b||,1e-30) recomputed in FP64 from the returned x */
    double b_norm;           /* ||b||_2 */
    double seconds;          /* wall time of the solve call */
    int engine;              /* what ran the iteration: 0 kernels per step (device graph loop or host-polled
                                chunks), 1 one thread-block cluster for the whole solve, 2 one persistent
                                cooperative launch for the whole solve */
    int preconditioner;      /* the preconditioner the solve used (CgGpu semantics: Jacobi after an ILU0
                                fall-back) */
    double residual_norm;    /* ||r||_2 of the iterated residual at exit (GpuSolverStats::finalResidual) */
    double initial_residual; /* CgGpu semantics: ||b - A x0||_2 (GpuSolverStats::initialResidual); else ||b||_2 */
} simall_solver_stats;

typedef struct simall_solver simall_solver;
void simall_solver_config_default(simall_solver_config *cfg);
int simall_solver_create(simall_context *ctx, const simall_solver_config *cfg, simall_solver **out);
int simall_solver_destroy(simall_solver *s);
/* CSR with int32 rowPtr[n+1], colIdx[nnz] (columns strictly ascending per row,
 * diagonal present) and FP64 values[nnz] (src/solver/CSRMatrix.hpp:16-22).
 * Copies host arrays to the device (mem == HOST) or references the caller's
 * device arrays (mem == DEVICE; they must stay alive and unchanged until the
 * next set_matrix or destroy).  Runs the preconditioner setup on the device. */
int simall_solver_set_matrix(simall_solver *s, int64_t n, int64_t nnz, const int32_t *rowPtr,
                             const int32_t *colIdx, const double *values, int mem);
/* Re-reads the values of the current pattern (same n, nnz, rowPtr, colIdx) and
 * redoes the preconditioner setup, as CGSolver::solve does on every call. */
int simall_solver_update_values(simall_solver *s, const double *values, int mem);
/* Solves A x = b from x = 0 (CGSolver semantics: the incoming x is ignored). */
int simall_solver_solve(simall_solver *s, const double *b, double *x, int mem, simall_solver_stats *stats);
/* y = A x with the solver's current FP64 matrix (the staged SpMV kernel the
 * solve uses; bit-identical to CSRMatrix::spmv, src/solver/CSRMatrix.hpp:24-35). */
int simall_solver_spmv(simall_solver *s, const double *x, double *y, int mem);
/* z = M^-1 r with the solver's FP64 preconditioner, as set up for its current
 * matrix: IPreconditioner::apply (src/solver/LinearSolvers.hpp:33-34) of
 * JacobiPreconditioner, ILU0Preconditioner, SsorPreconditioner
 * (src/solver/LinearSolvers.cpp:66-71, :127-151, :188-231) or
 * AMGPreconditioner (src/solver/AMGPreconditioner.cpp:418-427),
 * bit-identical to them.  r and z must not alias. */
int simall_solver_precond_apply(simall_solver *s, const double *r, double *z, int mem);
/* The AMG hierarchy built for the current matrix (preconditioner AMG): the
 * number of levels and the rows of each (up to max_levels of them).  *nlev is
 * 0 for the other preconditioners. */
int simall_solver_amg_levels(const simall_solver *s, int *nlev, int32_t *rows, int max_levels);
/* Diagnostic, host only (no device is touched): the AMG hierarchy this
 * library builds for A (host CSR arrays), with make_preconditioner's
 * parameters: the number of levels, the rows of each (up to max_levels), and
 * a 64-bit FNV-1a digest over the words of every level's operator, every
 * prolongation and restriction (rowPtr, colIdx, value bits) and the coarsest
 * level's dense LU.  It has no counterpart in the reference, whose
 * AMGPreconditioner keeps its levels private; it lets a test compare the
 * hierarchy with an independent restatement without a GPU. */
int simall_amg_hierarchy_digest(int64_t n, const int32_t *rowPtr, const int32_t *colIdx, const double *values,
                                int *nlev, int32_t *rows, int max_levels, uint64_t *digest);
/* Times `reps` back-to-back launches of one kernel of the solve on the
 * current matrix, bracketed by CUDA events on the context stream; *ms
 * receives the average duration of one launch and *bytes the algorithmic
 * bytes one launch moves (each array counted once per use, ideal reuse of
 * gathered vectors).  kernel: 0 FP64 CSR SpMV, 1 FP64 SpMV + p.Ap,
 * 2 FP64 Jacobi update (x, r, z, norms), 3 FP64 direction update,
 * 4 mixed FP32 step (r, x, p updates + SpMV + the step's four sums).
 * Kernel 4 needs precision MIXED.  The solver's iteration state is left
 * undefined; the next solve starts from scratch. */
int simall_solver_time_kernel(simall_solver *s, int kernel, int reps, double *ms, double *bytes);
/* ILinearSolver::last_residual(). */
double simall_solver_last_residual(const simall_solver *s);
/* The preconditioner the solver holds now: the configured one, or Jacobi after
 * a CgGpu-semantics ILU0 factor failed (GpuSolverConfig::preconditioner as
 * CgGpu::config() reports it after set_matrix, src/gpu/CgGpu.cpp:64-82). */
int simall_solver_preconditioner(const simall_solver *s, int *preconditioner);
/* ILinearSolver::solve(A, b, x) in one call: set_matrix + solve on host arrays. */
int simall_solver_solve_csr(simall_solver *s, int64_t n, int64_t nnz, const int32_t *rowPtr,
                            const int32_t *colIdx, const double *values, const double *b, double *x,
                            simall_solver_stats *stats);

/* ------------------------------------------------------------------ pressure-correction system */
/* The reference mesh SoA (src/meshing/MeshStorage.hpp:37-105); owner/neighbor
 * and cell_face_indices are u64 ids, neighbor == UINT64_MAX on boundary faces
 * (kBoundaryCell). */
typedef struct simall_mesh_view {
    int64_t n_cells;
    int64_t n_faces;
    const uint64_t *owner;
    const uint64_t *neighbor;
    const double *area_x, *area_y, *area_z;
    const double *centroid_x, *centroid_y, *centroid_z; /* face centroids */
    const uint32_t *boundary_zone;                      /* 0 = interior */
    const double *cell_centroid_x, *cell_centroid_y, *cell_centroid_z;
    const int32_t *cell_face_offsets; /* [n_cells+1] */
    const uint64_t *cell_face_indices;
} simall_mesh_view;

typedef struct simall_boundary {
    uint32_t zone;
    int type; /* simall_bc_type */
} simall_boundary;

/* Replaces SimpleAlgorithm::build_sparsity + assemble_pressure_correction
 * (src/solver/SimpleAlgorithm.cpp:49-98, :358-447).  create() pairs the
 * periodic faces as build_periodic_pairs does (:101-186: the zones of the
 * Periodic specs, in spec order, paired two by two; each face of the first
 * zone of a pair takes the face of the second whose centroid is nearest to
 * its own plus the mean translation between the zones), builds the CSR pattern
 * (bit-exact with build_sparsity, twin columns included), uploads the mesh
 * and precomputes per-face |A|^2 and |d.A| on the device.  A periodic face
 * couples its owner with its twin face's owner in the pressure assembly, the
 * face fluxes and the momentum assembly; it is not a Dirichlet anchor.  The
 * face-conductance extension below rejects systems with periodic faces. */
typedef struct simall_pressure_system simall_pressure_system;
int simall_pressure_system_create(simall_context *ctx, const simall_mesh_view *mesh, const simall_boundary *bcs,
                                  int n_bcs, simall_pressure_system **out);
int simall_pressure_system_destroy(simall_pressure_system *ps);
/* Sizes, and (when the arrays are non-NULL) host copies of the pattern. */
int simall_pressure_system_pattern(const simall_pressure_system *ps, int64_t *n, int64_t *nnz, int32_t *rowPtr,
                                   int32_t *colIdx);
/* The periodic twin of every face (-1 where none), twin[n_faces]: the table
 * SimpleAlgorithm::build_periodic_pairs builds. */
int simall_pressure_system_periodic_twins(const simall_pressure_system *ps, int32_t *twin);
/* Device pointers of the system's CSR (rowPtr, colIdx, values) and rhs. */
int simall_pressure_system_device_arrays(const simall_pressure_system *ps, const int32_t **rowPtr,
                                         const int32_t **colIdx, double **values, double **rhs);
/* assemble_pressure_correction: values and rhs from aP[n_cells] and
 * phi[n_faces] (mem says where aP/phi live).  any_dirichlet (optional)
 * receives 1 when a pressure boundary anchors the system (no cell-0 pin). */
int simall_assemble_pressure_correction(simall_pressure_system *ps, double rho, const double *aP,
                                        const double *phi, int mem, int *any_dirichlet);
/* The same for SIMPLEC (PvCouplingVariant::SIMPLEC): the denominator of every
 * cell is max(aP_c - sum_{k != c} |a_mom,ck|, 1e-30) instead of max(aP_c, 1e-30)
 * (SimpleAlgorithm.cpp:380-390, 401-409), with mom_values the momentum matrix
 * A_mom_ on the pressure system's pattern (build_sparsity gives A_mom_ and A_p_
 * one pattern; nnz values in its order). */
int simall_assemble_pressure_correction_simplec(simall_pressure_system *ps, double rho, const double *aP,
                                                const double *mom_values, const double *phi, int mem,
                                                int *any_dirichlet);
/* Host copies of the assembled values[nnz] and rhs[n]. */
int simall_pressure_system_download(const simall_pressure_system *ps, double *values, double *rhs);
/* Points the solver at the system's device CSR (no copy) and runs the
 * preconditioner setup. */
int simall_solver_use_pressure_system(simall_solver *s, simall_pressure_system *ps);
/* Solves the assembled system for p' (x = 0 start) into x (mem). */
int simall_pressure_system_solve(simall_pressure_system *ps, simall_solver *s, double *x, int mem,
                                 simall_solver_stats *stats);

/* ------------------------------------------------------------------ the field loops around the solve */
/* The face loops either side of the pressure solve of SimpleAlgorithm, on the
 * device and bit-identical to the reference: compute_face_fluxes
 * (SimpleAlgorithm.cpp:201-237; a periodic face averages its owner's velocity
 * with its twin face's owner's, :214-219), the least-squares
 * gradient (LeastSquaresGradient, Gradient.cpp:17-133) and correct_fields
 * (SimpleAlgorithm.cpp:450-487).  A GpuSimpleAlgorithm::iterate() override that
 * keeps U, p, aP, phi and p' in device memory runs the whole pressure step
 * without a host round trip: fluxes -> assemble -> solve -> correct. */
typedef struct simall_zone_velocity {
    uint32_t zone;
    double u[3]; /* BoundarySpec::vectorValue of a VelocityInlet / MovingWall zone */
} simall_zone_velocity;
/* Once per system: face areas, cell volumes (Mesh cells().volume) and the
 * least-squares geometry (the inverse normal matrix of every cell, as the
 * gradient's precompute) go to the device.  The boundary kinds of the flux
 * loop come from the specs given to simall_pressure_system_create; zones of
 * VelocityInlet / MovingWall specs take their vector from `velocities` (zero
 * when absent). */
int simall_pressure_system_setup_field_loops(simall_pressure_system *ps, const simall_mesh_view *m,
                                             const double *cell_volume, const simall_zone_velocity *velocities,
                                             int n_velocities);
/* phi[n_faces] = rho (u_f . A_f) from the cell velocities. */
int simall_compute_face_fluxes(simall_pressure_system *ps, double rho, const double *Ux, const double *Uy,
                               const double *Uz, double *phi, int mem);
/* (gx, gy, gz)[n_cells] = least-squares gradient of f[n_cells]. */
int simall_lsq_gradient(simall_pressure_system *ps, const double *f, double *gx, double *gy, double *gz, int mem);
/* p += urfP p'; U -= V / max(aP, 1e-30) grad p'; on interior faces
 * phi += rho |A|^2 / max(0.5 (aP_o + aP_n) |d.A|, 1e-30) (p'_o - p'_n).
 * p, U and phi are updated in place. */
int simall_correct_fields(simall_pressure_system *ps, double rho, double urfP, const double *aP, const double *pPrime,
                          double *p, double *Ux, double *Uy, double *Uz, double *phi, int mem);

/* ------------------------------------------------------------------ momentum assembly */
/* Replaces SimpleAlgorithm::assemble_momentum (src/solver/SimpleAlgorithm.cpp:240-355),
 * first-order upwind (a periodic face couples its owner with its twin face's
 * owner as half an interior face, :275-282).  The reference assembles one velocity
 * component per call, but its matrix does not depend on the component; one call
 * here builds that matrix once on the system's pattern (the pattern the
 * pressure system shares with the momentum matrix, build_sparsity) and the
 * three right-hand sides, bit-identical to the reference's three assemblies.
 * Needs simall_pressure_system_setup_field_loops (geometry, boundary kinds and
 * zone vectors, the least-squares gradient of p). */
typedef struct simall_momentum_options {
    double rho;  /* SimpleOptions::rho */
    double mu;   /* SimpleOptions::mu */
    double urfU; /* SimpleOptions::urfU (Patankar under-relaxation) */
    double dt;   /* SimpleOptions::dt; > 0 adds the transient term */
    int bdf2;    /* 1: BDF2 (TemporalScheme::BDF2 once timeStep >= 1), 0: implicit Euler */
    int reserved;
} simall_momentum_options;
/* U, Un, Unm1: [3][n_cells] (x, y, z components back to back); p[n_cells];
 * phi[n_faces].  Un is read when dt > 0, Unm1 when dt > 0 and bdf2.  The
 * result stays on the device (simall_momentum_device_arrays / _download). */
int simall_assemble_momentum(simall_pressure_system *ps, const simall_momentum_options *opt, const double *U,
                             const double *p, const double *phi, const double *Un, const double *Unm1, int mem);
/* Device arrays of the last momentum assembly: values[nnz] on the system's
 * pattern, rhs[3][n_cells], aP[n_cells] (the relaxed diagonal, SimpleAlgorithm::aP_). */
int simall_momentum_device_arrays(const simall_pressure_system *ps, const double **values, const double **rhs,
                                  const double **aP);
int simall_momentum_download(const simall_pressure_system *ps, double *values, double *rhs, double *aP);

/* ------------------------------------------------------------------ SIMPLE outer iteration */
/* Replaces SimpleAlgorithm::iterate / advance_time_step
 * (src/solver/SimpleAlgorithm.cpp:522-570) with U, p, phi, aP and p' in device
 * memory: fluxes -> momentum assembly and three momentum solves -> fluxes ->
 * pressure-correction assembly (SIMPLE or SIMPLEC) -> pressure solve ->
 * correct_fields.  The pressure system (with its field loops set up) holds
 * the mesh; the two solvers are any simall_solver of this context (the
 * reference takes the momentum and pressure ILinearSolver the same way). */
typedef struct simall_simple_options {
    double urfU, urfP, rho, mu; /* SimpleOptions (src/solver/SimpleAlgorithm.hpp:43-57) */
    double dt;                  /* > 0: transient (advance_time_step) */
    int bdf2;                   /* TemporalScheme::BDF2 (else implicit Euler) */
    int simplec;                /* PvCouplingVariant::SIMPLEC (else SIMPLE) */
    /* PisoAlgorithm / PimpleAlgorithm (src/solver/PisoAlgorithm.cpp:27-70,
     * PimpleAlgorithm.cpp:48-96): the defaults 1, 1, 0, 1, 0, 0 are SIMPLE;
     * PISO is n_correctors >= 1 with urfU = urfP = 1. */
    int n_outer_correctors;     /* outer correctors per iterate() */
    int n_correctors;           /* pressure correctors per outer corrector */
    int n_non_orth_corr;        /* extra pressure passes per corrector */
    int momentum_predictor;     /* 0: no momentum solve (needs a previous one's aP) */
    double tol_u, tol_p;        /* outer-loop early exit when every set tolerance holds (0 disables) */
} simall_simple_options;
typedef struct simall_simple_residuals {
    double mom[3];     /* |A U_k - b| of each momentum solve (SimpleResiduals::mom) */
    double cont;       /* |rhs| of the last pressure-correction system (SimpleResiduals::cont) */
    int iterations[4]; /* the last momentum x, y, z and pressure solves' counts */
    int outer;         /* index of the last outer corrector run (PimpleAlgorithm::last_outer_iters) */
    int reserved;
} simall_simple_residuals;
typedef struct simall_simple simall_simple;
typedef struct simall_fields simall_fields; /* the field registry, below */
void simall_simple_options_default(simall_simple_options *o);
/* U and p start at zero. */
int simall_simple_create(simall_pressure_system *ps, simall_solver *momentum, simall_solver *pressure,
                         const simall_simple_options *opt, simall_simple **out);
int simall_simple_destroy(simall_simple *s);
/* U [3][n_cells], p [n_cells]; either may be NULL. */
int simall_simple_set_fields(simall_simple *s, const double *U, const double *p, int mem);
int simall_simple_get_fields(simall_simple *s, double *U, double *p, double *phi, int mem);
/* The device arrays the iteration updates in place (valid until destroy). */
int simall_simple_device_fields(simall_simple *s, double **U, double **p, double **phi);
/* Keep U and p in a field registry: the iteration then reads and updates the
 * registry's vector "U" and scalar "p" (created zeroed with n_cells entries
 * when absent or of another size; they must keep that size while bound), so a
 * checkpoint of the registry captures the SIMPLE state and a registry read
 * back from one resumes it. */
int simall_simple_bind_fields(simall_simple *s, simall_fields *fields);
int simall_simple_iterate(simall_simple *s, simall_simple_residuals *res);
/* U^{n-1} <- U^n (from the second step on), U^n <- U, then n_inner iterations. */
int simall_simple_advance_time_step(simall_simple *s, int n_inner, simall_simple_residuals *res);

/* ------------------------------------------------------------------ differentiation */
/* Face-conductance Poisson operator (an extension: the reference expresses
 * neither per-face conductances nor non-zero Dirichlet values).  With
 * g_f = rho |A_f|^2 / max(|d.A_f|, 1e-30) -- the face coefficient of
 * SimpleAlgorithm.cpp:391-393 with k_f in place of 1/aP_f -- interior faces add
 * k_f g_f to (o,o),(n,n) and -k_f g_f to (o,n),(n,o); faces in a
 * PressureOutlet/PressureInlet zone are Dirichlet faces: they add k_f g_f to
 * (o,o) and k_f g_f pb_f to rhs_o; rhs starts from src[n_cells].  k and pb
 * are per face ([n_faces]; pb is read on Dirichlet faces only).  No pin. */
int simall_assemble_face_conductance(simall_pressure_system *ps, double rho, const double *k, const double *pb,
                                     const double *src, int mem);
/* Gradient of a loss L(x) with respect to every face conductance and every
 * Dirichlet value, given the solution x and the adjoint lambda = A^-T dL/dx:
 *   interior f: dk_f = -g_f (lambda_o - lambda_n)(x_o - x_n)
 *   Dirichlet f: dk_f = -g_f lambda_o (x_o - pb_f), dpb_f = k_f g_f lambda_o
 * (dk = dpb = 0 on other faces).  g_f is recomputed from the geometry, not
 * stored by the forward pass.  Equals -(dR/dalpha)^T psi of
 * adjoint::solve_discrete_adjoint (src/adjoint/DiscreteAdjoint.cpp:150-185)
 * for R(x; k, pb) = A(k) x - b(k, pb). */
int simall_face_conductance_gradient(simall_pressure_system *ps, double rho, const double *k, const double *pb,
                                     const double *x, const double *lambda, double *dk, double *dpb, int mem);
/* The backward pass in one call: lambda = A^-T dLdx with solver s on the
 * system's current (face-conductance) matrix -- A is symmetric, so this is the
 * PCG of simall_solver -- then the gradient above. */
int simall_adjoint_face_conductance(simall_pressure_system *ps, simall_solver *s, double rho, const double *k,
                                    const double *pb, const double *x, const double *dLdx, double *lambda,
                                    double *dk, double *dpb, int mem, simall_solver_stats *stats);

/* ------------------------------------------------------------------ field registry */
/* Replaces solver::FieldRegistry (src/solver/FieldRegistry.hpp:30-80) with the
 * fields in device memory: a scalar field is one FP64 array of n entries, a
 * vector field one [3][n] array (x, y, z back to back).  scalar() / vector()
 * return the field, creating it zeroed -- or re-creating it zeroed when its
 * size differs from n -- as the reference's accessors do; the arrays stay
 * valid until the field is re-created or the registry destroyed.  Fields are
 * kept in insertion order. */
int simall_fields_create(simall_context *ctx, simall_fields **out);
int simall_fields_destroy(simall_fields *f);
int simall_fields_scalar(simall_fields *f, const char *name, int64_t n, double **data);
int simall_fields_vector(simall_fields *f, const char *name, int64_t n, double **x, double **y, double **z);
/* find_scalar / find_vector (vector != 0): *data = NULL and *n = -1 when absent. */
int simall_fields_find(simall_fields *f, const char *name, int vector, double **data, int64_t *n);
int simall_fields_count(const simall_fields *f, int *n_scalars, int *n_vectors);
/* Name (NUL-terminated, truncated to len - 1) and size of the index-th field. */
int simall_fields_name(const simall_fields *f, int vector, int index, char *buf, int len, int64_t *n);
/* Host copies: upload creates / re-sizes the field (vector: host holds [3][n]). */
int simall_fields_upload(simall_fields *f, const char *name, int vector, const double *host, int64_t n);
int simall_fields_download(simall_fields *f, const char *name, int vector, double *host);

/* ------------------------------------------------------------------ checkpoint */
/* Replaces io::Checkpoint (src/io/Checkpoint.hpp:26-58, Checkpoint.cpp:66-227):
 * the same binary format byte for byte (header "SIMALLCP" v1 with a
 * timestamp, meta, the mesh SoA, then every scalar and vector field of the
 * registry), written from and read into device memory through pinned,
 * double-buffered staging; writes go to "<path>.tmp" and are renamed over
 * <path> when complete.  CheckpointMeta's layout (int, padding, double,
 * uint64) is kept. */
typedef struct simall_checkpoint_meta {
    int32_t iteration;
    double time;
    uint64_t settings_hash;
} simall_checkpoint_meta;
/* The mesh SoA of meshing::Mesh (src/meshing/MeshStorage.hpp:37-72): host
 * arrays; offsets have n + 1 entries (NULL writes an empty array). */
typedef struct simall_checkpoint_mesh {
    int64_t n_nodes, n_faces, n_cells, n_face_nodes, n_cell_faces;
    const double *node_x, *node_y, *node_z;
    const uint64_t *owner, *neighbor;
    const double *area_x, *area_y, *area_z;
    const double *centroid_x, *centroid_y, *centroid_z;
    const uint32_t *boundary_zone;
    const int32_t *face_node_offsets;
    const uint64_t *face_node_indices;
    const double *volume, *cell_centroid_x, *cell_centroid_y, *cell_centroid_z;
    const int32_t *cell_face_offsets;
    const uint64_t *cell_face_indices;
} simall_checkpoint_mesh;
int simall_checkpoint_write(const char *path, const simall_checkpoint_mesh *mesh, simall_fields *fields,
                            const simall_checkpoint_meta *meta);
/* Reads every field into `fields` (scalar()/vector() semantics), *meta if not
 * NULL, and the mesh into library-allocated host arrays when mesh_out is not
 * NULL (release them with simall_checkpoint_mesh_free). */
int simall_checkpoint_read(const char *path, simall_fields *fields, simall_checkpoint_meta *meta,
                           simall_checkpoint_mesh *mesh_out);
void simall_checkpoint_mesh_free(simall_checkpoint_mesh *mesh);

/* ------------------------------------------------------------------ SIMP topology optimisation */
/* Replaces optimization::SimpTopology (src/optimization/SimpTopology.hpp:48-80,
 * .cpp:18-227) with its fields in a device registry: create() is initialize()
 * (fields "rho", "rhoTilde", "K_simp", "dC_drho", "dC_drhoTilde" of
 * n_cells entries, set to volumeFraction, volumeFraction, K_min, 0, 0); each
 * step() filters rho (Helmholtz, CG + Jacobi on the device), forms
 * K_simp = K_min + (K_max - K_min) rhoTilde^p, takes the caller's "dC_drho"
 * through the filter, and runs the optimality-criteria update with bisection
 * on the volume multiplier; *change = sum |delta rho| / n.  The sensitivity
 * typically comes from simall_adjoint_face_conductance. */
typedef struct simall_simp_config {
    double penalty;         /* SimpConfig::penalty (p) */
    double K_min, K_max;
    double filter_radius;   /* 0 disables the Helmholtz filter */
    double volume_fraction;
    double move;            /* OC move limit */
    double damping;         /* OC damping exponent */
    double rho_min;
} simall_simp_config;
typedef struct simall_simp simall_simp;
void simall_simp_config_default(simall_simp_config *cfg);
int simall_simp_create(simall_pressure_system *ps, simall_fields *fields, const simall_simp_config *cfg,
                       simall_simp **out);
int simall_simp_step(simall_simp *s, double *change);
int simall_simp_destroy(simall_simp *s);

/* ------------------------------------------------------------------ diagnostics */
/* Failure detection without a GPU fault (no reference counterpart): runs one
 * warp that waits, with the same bounded wait as the ILU(0) sweeps, for a mark
 * that nothing sets.  *timed_out = 1 when the wait ran out and the kernel
 * returned on its own (the expected result), *seconds = the wall time of the
 * call (the bound is about a second).  The context stays usable. */
int simall_diagnose_bounded_wait(simall_context *ctx, int *timed_out, double *seconds);
/* Latency measurements of the free-running triangular sweeps (ILU(0), SSOR,
 * the AMG smoother's large levels; no reference counterpart): sets, for the
 * whole process, the CTAs per SM of their grid (1..8; default 2), the longest
 * sleep between two polls of a value not yet published (0..4096 ns, 0 = spin;
 * default 0) and whether the ILU(0) backward sweep divides through the
 * correctly rounded reciprocal of the pivot (1, default) or by a division (0).
 * Results do not depend on any of them.  Solvers capture their iteration
 * graphs at their first solve: set these before creating the solver. */
int simall_diagnose_sweep_params(int ctas_per_sm, int backoff_ns, int divide_via_reciprocal);
/* Launch parameters of the mixed-precision solve in sliced storage, for the
 * whole process: how many stages ahead the staged step prefetches its
 * operands into L2 (0..64; default 0 = none), and the CTAs per SM of the
 * persistent whole-solve launch (0..8; default 0 = as many as fit).  Results
 * do not depend on the first; the second regroups the FP32 partial sums.  Set
 * them before creating the solver. */
int simall_diagnose_mixed_params(int prefetch_stages, int grid_ctas_per_sm);
/* The small-system ILU(0) path divides through a correctly rounded reciprocal
 * (one product and two FMAs, Markstein's correction).  For each i, q_recip[i]
 * is that quotient a[i] / b[i] and q_div[i] the device's correctly rounded
 * division; the two must be bit-identical (host arrays, n entries). */
int simall_diagnose_division(simall_context *ctx, int64_t n, const double *a, const double *b, double *q_recip,
                             double *q_div);

/* ------------------------------------------------------------------ batched solves */
/* Many independent SPD systems of uneven size (e.g. one pressure-correction
 * system per cavity, block or time level) solved in one persistent launch:
 * the work loop a caller would write around CGSolver::solve
 * (src/solver/LinearSolvers.cpp:420-451), with the mixed-precision Jacobi-PCG
 * of simall_solver (FP32 inner iteration, FP64 true residual, reductions and
 * x) run by one CTA per system.  Systems are given concatenated: system s owns
 * rows [row_offsets[s], row_offsets[s+1]) and nonzeros [nnz_offsets[s],
 * nnz_offsets[s+1]); its rowPtr (local, starting at 0, n_s+1 entries) starts at
 * rowPtr[row_offsets[s] + s]; colIdx are local.  b and x are concatenated
 * by rows. */
typedef struct simall_batch simall_batch;
typedef struct simall_batch_system_stats {
    int iterations;
    int reliable_updates;
    int converged;
    int status;
    double true_residual; /* ||b - A x|| / max(||b||, 1e-30) of the returned x, FP64 */
    double b_norm;
} simall_batch_system_stats;
typedef struct simall_batch_stats {
    int systems;
    int converged;
    int max_iterations;
    int status;               /* SIMALL_OK, or the status of a system that did not converge */
    int64_t total_iterations;
    double worst_true_residual;
    int block_threads;        /* launch shape in use (autotuned unless set) */
    int ctas_per_sm;
    double seconds;
    int rows_per_pass;        /* rows each thread keeps in flight */
    int autotune_source;      /* 0 set by simall_batch_launch_shape, 1 timed on this batch, 2 autotuner cache */
    int cluster_rows;         /* systems of at least this many rows (diagonal storage) ran on one
                                 thread-block cluster each; 0: none */
    int cluster_ctas;         /* CTAs per such cluster */
    int cluster_systems;      /* systems that ran on clusters */
    int clusters;             /* clusters resident at a time (cluster_ctas x clusters SMs held) */
} simall_batch_stats;
/* cfg: tolerance, max_iterations, reliable_delta as for simall_solver (Jacobi). */
int simall_batch_create(simall_context *ctx, const simall_solver_config *cfg, simall_batch **out);
int simall_batch_destroy(simall_batch *b);
/* Host arrays; validated, scaled and stored on the device. */
int simall_batch_set_systems(simall_batch *b, int n_systems, const int64_t *row_offsets, const int64_t *nnz_offsets,
                             const int32_t *rowPtr, const int32_t *colIdx, const double *values);
/* Solves every system from x = 0.  per_system (optional) has n_systems entries. */
int simall_batch_solve(simall_batch *b, const double *rhs, double *x, int mem, simall_batch_system_stats *per_system,
                       simall_batch_stats *total);
/* Fixes the launch shape (256/512/1024 threads per CTA, 1-8 CTAs per SM, at
 * most 2048 threads per SM; 2 rows in flight per thread; every system on the
 * one-CTA queue); block_threads == 0 re-enables the autotuner, which at the
 * next solve reads the autotuner cache or times candidates on the batch and
 * keeps the fastest: first the one-CTA shape (threads per CTA, CTAs per SM,
 * rows in flight per thread), then with it which systems run on a
 * thread-block cluster each instead (a row threshold and the cluster size;
 * systems in diagonal storage, concurrently with the one-CTA queue). */
int simall_batch_launch_shape(simall_batch *b, int block_threads, int ctas_per_sm);
/* Fixes which systems run on a thread-block cluster each: systems in diagonal
 * storage of at least cluster_rows rows (and at most cluster_ctas x 8192) on
 * `clusters` clusters of cluster_ctas CTAs (1-16) that take them largest
 * first, on clusters x cluster_ctas SMs; the one-CTA queue runs the rest on
 * the other SMs at the same time.  cluster_rows == 0: none.  Keeps the
 * one-CTA shape (1024 threads, 1 CTA per SM, 2 rows in flight unless set). */
int simall_batch_cluster_route(simall_batch *b, int cluster_rows, int cluster_ctas, int clusters);
/* The autotuner cache file of this batch object (JSON; path NULL or "": no
 * cache).  The default is SIMALL_AUTOTUNE_CACHE when set ("off": none), else
 * $XDG_CACHE_HOME/simall_gb300/autotune.json, else
 * $HOME/.cache/simall_gb300/autotune.json.  Entries are keyed by device name,
 * SM count, kernel revision and a hash of the batch's system sizes. */
int simall_batch_autotune_cache(simall_batch *b, const char *path);
/* The cache itself (host only): values = {block_threads, ctas_per_sm,
 * rows_per_pass, cluster_rows, cluster_ctas, clusters}.  lookup returns SIMALL_OK when the key is present,
 * SIMALL_ERR_IO when it is not (or the file cannot be read); store replaces or
 * appends the key and rewrites the file through a rename. */
int simall_autotune_cache_lookup(const char *path, const char *key, int *values);
int simall_autotune_cache_store(const char *path, const char *key, const int *values, double ms);

/* ------------------------------------------------------------------ reference GPU facade */
/* One-for-one replacements of src/gpu/GpuKernels.hpp:48-108 on device
 * pointers (stream == NULL: the legacy default stream).  dot and nrm2 block
 * the host, as documented there. */
int simall_gpu_axpy(double alpha, const double *x, double *y, size_t n, void *stream);
int simall_gpu_scal(double alpha, double *x, size_t n, void *stream);
int simall_gpu_copy(const double *src, double *dst, size_t n, void *stream);
int simall_gpu_dot(const double *x, const double *y, size_t n, void *stream, double *result);
int simall_gpu_nrm2(const double *x, size_t n, void *stream, double *result);
int simall_gpu_axpby(double a, const double *x, double b, double *y, size_t n, void *stream);
int simall_gpu_xpby(const double *x, double beta, double *y, size_t n, void *stream);
int simall_gpu_spmv_csr(size_t n, const int32_t *rowPtr, const int32_t *colIdx, const double *values,
                        const double *x, double *y, void *stream);
/* Dot product that allocates no device memory.  It has no counterpart in the
 * reference: it exists for callers that must not call cudaMalloc -- code whose
 * device memory is already fully owned by another allocator, loops that cannot
 * take cudaMalloc's implicit synchronisation, processes that keep a fixed
 * device footprint after start-up.  Its reduction scratch is a fixed array
 * inside this library (reserved on every GPU that loads the library, until the
 * process exits), which limits n to SIMALL_DOT_NOALLOC_MAX_N; larger n returns
 * SIMALL_ERR_SIZE_MISMATCH.  The first call on each device looks the array's
 * address up (cudaGetSymbolAddress); make it before any stream capture.  The
 * address is cached for the life of the device's context: do not use this
 * function on a device after calling cudaDeviceReset on it.  All calls share
 * the array, so calls that overlap on the GPU race.  Blocks the host like
 * simall_gpu_dot. */
#define SIMALL_DOT_NOALLOC_MAX_N 16777216
int simall_gpu_dot_noalloc(const double *x, const double *y, size_t n, void *stream, double *result);
/* z[i] = r[i] / diag[i]  (GpuKernels.hpp:87) */
int simall_gpu_jacobi_apply(const double *diag, const double *r, double *z, size_t n, void *stream);
/* In-place ILU(0) of device CSR values (GpuKernels.hpp:89-97); *ok = 0 on a
 * zero pivot.  Level-scheduled on the device; the factor equals
 * ILU0Preconditioner::setup's bit for bit. */
int simall_gpu_ilu0_factor_inplace(size_t n, const int32_t *rowPtr, const int32_t *colIdx, double *values,
                                   void *stream, int *ok);
/* z = U^-1 L^-1 r with the factor above (GpuKernels.hpp:99-108). */
int simall_gpu_ilu0_apply(size_t n, const int32_t *rowPtr, const int32_t *colIdx, const double *values,
                          const double *r, double *z, void *stream);

/* ------------------------------------------------------------------ host preprocessing */
/* Structured n_x*n_y*n_z hex box [0,e_x]x[0,e_y]x[0,e_z] as an unstructured
 * SoA mesh, identical to CartesianMesher::generate + ConnectivityBuilder::build
 * + Mesh::compute_geometry (src/meshing/CartesianMesher.cpp:13-101,
 * Connectivity.cpp:45-115, MeshStorage.cpp:21-97), with an optional
 * per-node displacement (dx,dy,dz may be NULL) applied before the geometry.
 * Sizes: n_cells = nx*ny*nz, n_faces = (nx+1)ny nz + nx(ny+1)nz + nx ny(nz+1),
 * cell_face_indices 6*n_cells.  All output arrays are caller-allocated. */
int simall_mesh_cartesian(int nx, int ny, int nz, double ex, double ey, double ez, const double *dx,
                          const double *dy, const double *dz, uint64_t *owner, uint64_t *neighbor,
                          double *area_x, double *area_y, double *area_z, double *centroid_x,
                          double *centroid_y, double *centroid_z, uint32_t *boundary_zone, double *volume,
                          double *cell_centroid_x, double *cell_centroid_y, double *cell_centroid_z,
                          int32_t *cell_face_offsets, uint64_t *cell_face_indices);
/* Reverse Cuthill-McKee in place, as renumber_cells_cuthill_mckee
 * (src/meshing/MeshOps.cpp:547-676).  stats (optional, 3 entries) receives
 * bandwidth before, after and cells permuted. */
int simall_mesh_rcm(int64_t n_cells, int64_t n_faces, uint64_t *owner, uint64_t *neighbor, double *volume,
                    double *cell_centroid_x, double *cell_centroid_y, double *cell_centroid_z,
                    int32_t *cell_face_offsets, uint64_t *cell_face_indices, int64_t *stats);

#ifdef __cplusplus
}
#endif

#endif /* SIMALL_GPU_H */
