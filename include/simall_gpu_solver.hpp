// simall_gpu_solver.hpp -- header-only drop-in for SimAll's pressure solver.
//
// GpuPcgSolver implements simall::solver::ILinearSolver
// (src/solver/Solver.hpp:92-100) on top of the C ABI in simall_gpu.h, with
// CGSolver's semantics (src/solver/LinearSolvers.cpp:420-451): every solve()
// sets the preconditioner up again, overwrites x starting from zero, and
// returns the iteration count (maxIterations when the tolerance was not
// reached); last_residual() is ||r|| / max(||b||, 1e-30).  Like the reference
// solvers it never throws from solve(): a C-ABI failure returns
// maxIterations with last_residual() = +inf and status() != SIMALL_OK.
//
// Use it wherever SimAll takes an ILinearSolver&, e.g.
//   simall::gpu_gb300::GpuPcgSolver pSolver(cfg);           // cfg.kind == CG
//   simall::solver::SimpleAlgorithm simple(mesh, fields, bcs, momentumSolver, pSolver, opts);
//
// Include with SimAll's src/ directory on the include path; link
// libsimall_gpu.so.
#pragma once

#include "simall_gpu.h"

#include "solver/CSRMatrix.hpp"
#include "solver/Solver.hpp"

#include <limits>
#include <stdexcept>
#include <string>

namespace simall::gpu_gb300 {

class GpuPcgSolver final : public solver::ILinearSolver {
public:
    // precision: SIMALL_PRECISION_FP64 (the reference CG) or
    // SIMALL_PRECISION_MIXED (FP32 inner iteration, FP64 true residual and x).
    explicit GpuPcgSolver(const solver::LinearSolverConfig &cfg, int precision = SIMALL_PRECISION_FP64,
                          int device = 0, void *stream = nullptr)
        : maxIt_(cfg.maxIterations)
    {
        if (simall_context_create(device, stream, &ctx_) != SIMALL_OK)
            throw std::runtime_error("simall_gpu: no usable CUDA device");
        simall_solver_config c;
        simall_solver_config_default(&c);
        c.preconditioner = static_cast<int>(cfg.preconditioner);
        c.tolerance = cfg.tolerance;
        c.max_iterations = cfg.maxIterations;
        c.precision = precision;
        c.kind = static_cast<int>(cfg.kind);  // CG, GMRES(restart), BiCGSTAB or TFQMR, as make_linear_solver
        c.restart = cfg.restart;
        const int st = simall_solver_create(ctx_, &c, &s_);
        if (st != SIMALL_OK) {
            const std::string msg = simall_context_last_error(ctx_);
            simall_context_destroy(ctx_);
            throw std::runtime_error("simall_gpu: " + std::string(simall_status_string(st)) + ": " + msg);
        }
    }

    ~GpuPcgSolver() override
    {
        simall_solver_destroy(s_);
        simall_context_destroy(ctx_);
    }

    GpuPcgSolver(const GpuPcgSolver &) = delete;
    GpuPcgSolver &operator=(const GpuPcgSolver &) = delete;

    int solve(const solver::CSRMatrix &A, const util::aligned_vector<double> &b,
              util::aligned_vector<double> &x) override
    {
        const auto n = static_cast<int64_t>(A.rows());
        x.assign(static_cast<std::size_t>(n), 0.0);
        status_ = simall_solver_solve_csr(s_, n, static_cast<int64_t>(A.colIdx.size()), A.rowPtr.data(),
                                          A.colIdx.data(), A.values.data(), b.data(), x.data(), &stats_);
        if (status_ != SIMALL_OK) {
            stats_ = simall_solver_stats{};
            stats_.final_residual = std::numeric_limits<double>::infinity();
            return maxIt_;
        }
        return stats_.iterations;
    }

    double last_residual() const override
    {
        return status_ == SIMALL_OK ? stats_.final_residual : std::numeric_limits<double>::infinity();
    }

    // Beyond ILinearSolver: the last call's status and statistics.
    int status() const { return status_; }
    const simall_solver_stats &stats() const { return stats_; }
    const char *last_error() const { return simall_context_last_error(ctx_); }

private:
    simall_context *ctx_ = nullptr;
    simall_solver *s_ = nullptr;
    simall_solver_stats stats_{};
    int status_ = SIMALL_OK;
    int maxIt_ = 1000;
};

// The same adapter for any LinearSolverKind the device provides.
using GpuLinearSolver = GpuPcgSolver;

}  // namespace simall::gpu_gb300
