// simall_cggpu.hpp -- header-only drop-in for SimAll's gpu::CgGpu.
//
// CgGpu here has the interface of simall::gpu::CgGpu (src/gpu/CgGpu.hpp:49-124):
// a GpuSolverConfig (preconditioner None / Jacobi / ILU0, tolerance,
// maxIterations, relativeOrders), set_matrix(HostCsrView) that copies the
// matrix and builds the preconditioner (an ILU0 factor that meets a zero pivot
// turns the solver into Jacobi for good, as CgGpu::set_matrix does), and
// solve(b, x) with x as the initial guess and the solution, returning
// GpuSolverStats (iterations, finalResidual = ||r||_2, initialResidual,
// converged, timeSeconds).  The iteration runs on the device through the C ABI
// of simall_gpu.h (SIMALL_SEMANTICS_CGGPU): every vector stays in device
// memory and the loop never synchronises with the host per iteration, where
// the reference pays a host round trip per BLAS call.
//
// Differences a caller can see: Jacobi multiplies by the reciprocal diagonal
// where the reference divides (at most one rounding apart per entry); dot
// products are summed in a tree, not serially.  Iteration counts match the
// reference's to within one and solutions to 1e-10 (tests/test_gpu_cggpu.py).
// A C-ABI failure throws std::runtime_error from set_matrix; solve() returns
// zeroed stats (converged = false) and sets status().
//
// Switch a caller by replacing simall::gpu:: with simall::gpu_gb300:: for
// CgGpu, GpuSolverConfig, GpuPreconditioner, GpuSolverStats and HostCsrView,
// and link libsimall_gpu.so.
#pragma once

#include "simall_gpu.h"

#include <cstddef>
#include <stdexcept>
#include <string>
#include <vector>

namespace simall::gpu_gb300 {

enum class GpuPreconditioner { None, Jacobi, ILU0 };

struct GpuSolverConfig {
    GpuPreconditioner preconditioner = GpuPreconditioner::Jacobi;
    double tolerance = 1.0e-8;  ///< ||r|| / ||b||
    int maxIterations = 1000;
    double relativeOrders = 0.0;  ///< > 0: also stop when ||r|| drops by this many orders (first trigger wins)
};

struct GpuSolverStats {
    int iterations = 0;
    double finalResidual = 0.0;  ///< ||r||_2
    double initialResidual = 0.0;
    bool converged = false;
    double timeSeconds = 0.0;
};

struct HostCsrView {
    std::size_t n = 0;
    std::size_t nnz = 0;
    const int *rowPtr = nullptr;
    const int *colIdx = nullptr;
    const double *values = nullptr;
};

class CgGpu {
public:
    explicit CgGpu(GpuSolverConfig cfg = {}, int device = 0, void *stream = nullptr) : cfg_(cfg)
    {
        if (simall_context_create(device, stream, &ctx_) != SIMALL_OK)
            throw std::runtime_error("simall_gpu: no usable CUDA device");
        make();
    }

    ~CgGpu()
    {
        simall_solver_destroy(s_);
        simall_context_destroy(ctx_);
    }

    CgGpu(const CgGpu &) = delete;
    CgGpu &operator=(const CgGpu &) = delete;

    /// Copies A to the device and builds the preconditioner; call whenever A changes.
    void set_matrix(const HostCsrView &A)
    {
        if (dirty_)
            make();
        n_ = A.n;
        status_ = simall_solver_set_matrix(s_, static_cast<int64_t>(A.n), static_cast<int64_t>(A.nnz), A.rowPtr,
                                           A.colIdx, A.values, SIMALL_MEM_HOST);
        if (status_ != SIMALL_OK)
            throw std::runtime_error("simall_gpu: set_matrix: " + std::string(simall_context_last_error(ctx_)));
        int pc = SIMALL_PRECOND_JACOBI;
        simall_solver_preconditioner(s_, &pc);
        cfg_.preconditioner = pc == SIMALL_PRECOND_ILU0   ? GpuPreconditioner::ILU0
                              : pc == SIMALL_PRECOND_NONE ? GpuPreconditioner::None
                                                          : GpuPreconditioner::Jacobi;
    }

    /// Solve A x = b; x is both the initial guess (in) and the solution (out).
    GpuSolverStats solve(const std::vector<double> &b, std::vector<double> &x)
    {
        GpuSolverStats st{};
        if (n_ == 0 || b.size() != n_ || x.size() != n_)
            return st;  // CgGpu::solve logs and returns zeroed stats on a size mismatch
        simall_solver_stats c{};
        status_ = simall_solver_solve(s_, b.data(), x.data(), SIMALL_MEM_HOST, &c);
        if (status_ != SIMALL_OK)
            return st;
        st.iterations = c.iterations;
        st.finalResidual = c.residual_norm;
        st.initialResidual = c.initial_residual;
        st.converged = c.converged != 0;
        st.timeSeconds = c.seconds;
        lastResidual_ = c.residual_norm;
        return st;
    }

    const GpuSolverConfig &config() const noexcept { return cfg_; }
    /// Takes effect at the next set_matrix (the preconditioner is built there).
    void set_config(GpuSolverConfig c) noexcept
    {
        cfg_ = c;
        dirty_ = true;
    }
    double last_residual() const noexcept { return lastResidual_; }

    // Beyond gpu::CgGpu: the last call's C-ABI status and error text.
    int status() const { return status_; }
    const char *last_error() const { return simall_context_last_error(ctx_); }

private:
    void make()
    {
        if (s_) {
            simall_solver_destroy(s_);
            s_ = nullptr;
        }
        simall_solver_config c;
        simall_solver_config_default(&c);
        c.preconditioner = cfg_.preconditioner == GpuPreconditioner::None     ? SIMALL_PRECOND_NONE
                           : cfg_.preconditioner == GpuPreconditioner::ILU0   ? SIMALL_PRECOND_ILU0
                                                                              : SIMALL_PRECOND_JACOBI;
        c.tolerance = cfg_.tolerance;
        c.max_iterations = cfg_.maxIterations;
        c.semantics = SIMALL_SEMANTICS_CGGPU;
        c.relative_orders = cfg_.relativeOrders;
        status_ = simall_solver_create(ctx_, &c, &s_);
        if (status_ != SIMALL_OK)
            throw std::runtime_error("simall_gpu: " + std::string(simall_status_string(status_)) + ": " +
                                     simall_context_last_error(ctx_));
        dirty_ = false;
        n_ = 0;
    }

    GpuSolverConfig cfg_;
    simall_context *ctx_ = nullptr;
    simall_solver *s_ = nullptr;
    std::size_t n_ = 0;
    double lastResidual_ = 0.0;
    int status_ = SIMALL_OK;
    bool dirty_ = false;
};

}  // namespace simall::gpu_gb300
