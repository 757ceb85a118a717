// simall::gpu_gb300::CgGpu through gpu::CgGpu's interface: the 1-D Laplacian
// (n = 50, b = 1) cold and warm started with Jacobi and ILU0, relativeOrders,
// and an ILU0 factor with a zero pivot that falls back to Jacobi; exits
// non-zero on a failure.
#include "simall_cggpu.hpp"

#include <cmath>
#include <cstdio>
#include <vector>

using namespace simall::gpu_gb300;

namespace {

struct Csr {
    std::vector<int> rp{0}, ci;
    std::vector<double> va;
    HostCsrView view() const
    {
        HostCsrView v;
        v.n = rp.size() - 1;
        v.nnz = ci.size();
        v.rowPtr = rp.data();
        v.colIdx = ci.data();
        v.values = va.data();
        return v;
    }
};

Csr laplacian(int n, double d0)
{
    Csr A;
    for (int i = 0; i < n; ++i) {
        if (i > 0) {
            A.ci.push_back(i - 1);
            A.va.push_back(-1.0);
        }
        A.ci.push_back(i);
        A.va.push_back(i == 0 ? d0 : 2.0);
        if (i + 1 < n) {
            A.ci.push_back(i + 1);
            A.va.push_back(-1.0);
        }
        A.rp.push_back(static_cast<int>(A.ci.size()));
    }
    return A;
}

double residual(const Csr &A, const std::vector<double> &b, const std::vector<double> &x)
{
    double s = 0.0;
    for (size_t i = 0; i + 1 < A.rp.size(); ++i) {
        double y = 0.0;
        for (int k = A.rp[i]; k < A.rp[i + 1]; ++k)
            y += A.va[k] * x[A.ci[k]];
        s += (b[i] - y) * (b[i] - y);
    }
    return std::sqrt(s);
}

}  // namespace

int main()
{
    const int n = 50;
    const Csr A = laplacian(n, 2.0);
    std::vector<double> b(n, 1.0);
    int failures = 0;
    auto check = [&](bool ok, const char *what) {
        std::printf("%s %s\n", what, ok ? "ok" : "FAILED");
        failures += ok ? 0 : 1;
    };
    for (GpuPreconditioner pc : {GpuPreconditioner::Jacobi, GpuPreconditioner::ILU0}) {
        GpuSolverConfig cfg;
        cfg.preconditioner = pc;
        cfg.tolerance = 1e-10;
        CgGpu cg(cfg);
        cg.set_matrix(A.view());
        std::vector<double> x(n, 0.0);
        const GpuSolverStats cold = cg.solve(b, x);
        const double r = residual(A, b, x);
        // warm start from the solution: converged before the first iteration
        const GpuSolverStats warm = cg.solve(b, x);
        check(cold.converged && r <= 1e-10 * std::sqrt(double(n)) && warm.converged && warm.iterations == 0 &&
                  warm.initialResidual <= 1e-10 * std::sqrt(double(n)) && cg.last_residual() == warm.finalResidual,
              pc == GpuPreconditioner::Jacobi ? "jacobi cold + warm" : "ilu0 cold + warm");
    }
    {
        GpuSolverConfig cfg;
        cfg.tolerance = 1e-14;
        cfg.relativeOrders = 2.0;
        CgGpu cg(cfg);
        cg.set_matrix(A.view());
        std::vector<double> x(n, 0.0);
        const GpuSolverStats st = cg.solve(b, x);
        check(st.converged && st.finalResidual <= 1e-2 * st.initialResidual, "relativeOrders");
    }
    {
        const Csr Z = laplacian(n, 0.0);  // a_00 = 0: the ILU0 factor meets a zero pivot
        GpuSolverConfig cfg;
        cfg.preconditioner = GpuPreconditioner::ILU0;
        CgGpu cg(cfg);
        cg.set_matrix(Z.view());
        check(cg.config().preconditioner == GpuPreconditioner::Jacobi, "ilu0 -> jacobi fall-back");
    }
    return failures;
}
