// GpuPcgSolver through the ILinearSolver interface: the 1-D Laplacian of
// tests/unit/solver/test_ssor_preconditioner.cpp:65-88 (n = 50, b = 1,
// tol 1e-10), with Jacobi, ILU0 and mixed precision; exits non-zero on a
// failure.
#include "simall_gpu_solver.hpp"

#include <cmath>
#include <cstdio>
#include <memory>

using namespace simall;

int main()
{
    const int n = 50;
    solver::CSRMatrix A;
    A.rowPtr.push_back(0);
    for (int i = 0; i < n; ++i) {
        if (i > 0) {
            A.colIdx.push_back(i - 1);
            A.values.push_back(-1.0);
        }
        A.colIdx.push_back(i);
        A.values.push_back(2.0);
        if (i + 1 < n) {
            A.colIdx.push_back(i + 1);
            A.values.push_back(-1.0);
        }
        A.rowPtr.push_back(static_cast<int>(A.colIdx.size()));
    }
    util::aligned_vector<double> b(n, 1.0), x;
    int failures = 0;
    struct Case {
        solver::PreconditionerKind pc;
        int precision;
        const char *name;
    } cases[] = {{solver::PreconditionerKind::Jacobi, SIMALL_PRECISION_FP64, "jacobi"},
                 {solver::PreconditionerKind::ILU, SIMALL_PRECISION_FP64, "ilu0"},
                 {solver::PreconditionerKind::Jacobi, SIMALL_PRECISION_MIXED, "mixed"}};
    for (const Case &c : cases) {
        solver::LinearSolverConfig cfg;
        cfg.kind = solver::LinearSolverKind::CG;
        cfg.preconditioner = c.pc;
        cfg.maxIterations = 200;
        cfg.tolerance = 1.0e-10;
        std::unique_ptr<solver::ILinearSolver> s = std::make_unique<gpu_gb300::GpuPcgSolver>(cfg, c.precision);
        const int it = s->solve(A, b, x);
        double r2 = 0.0;
        for (int i = 0; i < n; ++i) {
            double s2 = 0.0;
            for (int k = A.rowPtr[i]; k < A.rowPtr[i + 1]; ++k)
                s2 += A.values[k] * x[A.colIdx[k]];
            r2 += (s2 - b[i]) * (s2 - b[i]);
        }
        const bool ok = it > 0 && it < 200 && std::sqrt(r2) < 1.0e-7 && s->last_residual() < 1.0e-10;
        std::printf("%s: it=%d |b-Ax|=%.3e last_residual=%.3e %s\n", c.name, it, std::sqrt(r2), s->last_residual(),
                    ok ? "ok" : "FAIL");
        failures += ok ? 0 : 1;
    }
    return failures;
}
