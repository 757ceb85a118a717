// Test stand-in for the linear-solver part of simall/solver/Solver.hpp: the
// enums, LinearSolverConfig and the ILinearSolver interface the adapter
// implements, with the same names, ordinals and defaults.
#pragma once
#include "solver/CSRMatrix.hpp"
namespace simall::solver {
enum class LinearSolverKind { GMRES, BiCGSTAB, CG, TFQMR };
enum class PreconditionerKind { Jacobi, ILU, SSOR, AMG, None };
struct LinearSolverConfig {
    LinearSolverKind kind = LinearSolverKind::GMRES;
    PreconditionerKind preconditioner = PreconditionerKind::ILU;
    double tolerance = 1.0e-8;
    int maxIterations = 1000;
    int restart = 30;
};
class ILinearSolver {
public:
    virtual ~ILinearSolver() = default;
    virtual int solve(const CSRMatrix &A, const util::aligned_vector<double> &b, util::aligned_vector<double> &x) = 0;
    virtual double last_residual() const = 0;
};
}  // namespace simall::solver
