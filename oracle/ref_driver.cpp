// Test infrastructure only: a C-callable driver over the SimAll reference
// sources, compiled together with them by oracle/build_ref.sh into
// oracle/_ref/libsimall_ref.so.  Nothing in the product links or loads it;
// the tests and the golden-fixture script use it to pin the C restatement in
// oracle/simall_oracle.c against the reference's own code.
//
// Every entry point calls the reference's public (or subclass-visible) API:
//   meshing::CartesianMesher::generate      src/meshing/CartesianMesher.cpp:13
//   meshing::Mesh::compute_geometry         src/meshing/MeshStorage.cpp:21
//   meshing::ops::renumber_cells_cuthill_mckee  src/meshing/MeshOps.cpp:547
//   SimpleAlgorithm::build_sparsity         src/solver/SimpleAlgorithm.cpp:49
//   SimpleAlgorithm::assemble_pressure_correction  src/solver/SimpleAlgorithm.cpp:358
//   SimpleAlgorithm::iterate                src/solver/SimpleAlgorithm.cpp:522
//   PisoAlgorithm::iterate, PimpleAlgorithm::iterate  src/solver/PisoAlgorithm.cpp:27, PimpleAlgorithm.cpp:48
//   make_cg / make_gmres / make_preconditioner     src/solver/LinearSolvers.cpp:240,462
//   adjoint::solve_discrete_adjoint         src/adjoint/DiscreteAdjoint.cpp:150
//   core::PluginLoader::load / PluginRegistry  src/core/PluginLoader.cpp:68, PluginRegistry.cpp:23
//   io::Checkpoint::write / read            src/io/Checkpoint.cpp:66, :145
//   optimization::SimpTopology              src/optimization/SimpTopology.cpp:18, :132
#include "adjoint/DiscreteAdjoint.hpp"
#include "core/PluginLoader.hpp"
#include "core/PluginRegistry.hpp"
#include "gpu/CgGpu.hpp"
#include "io/Checkpoint.hpp"
#include "optimization/SimpTopology.hpp"
#include "meshing/CartesianMesher.hpp"
#include "meshing/MeshOps.hpp"
#include "meshing/MeshStorage.hpp"
#include "solver/FieldRegistry.hpp"
#include "solver/Gradient.hpp"
#include "solver/LinearSolvers.hpp"
#include "solver/PimpleAlgorithm.hpp"
#include "solver/PisoAlgorithm.hpp"
#include "solver/SimpleAlgorithm.hpp"

#include <algorithm>
#include <chrono>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <memory>
#include <vector>

namespace S = simall::solver;
namespace M = simall::meshing;
using Vec = simall::util::aligned_vector<double>;

namespace
{

struct RefMesh
{
    M::Mesh mesh;
};

// Exposes the protected assembly hooks of SimpleAlgorithm so the driver can
// feed aP_ / phiFlux_ directly and read A_p_ / rhs_ back.
class AssemblyProbe : public S::SimpleAlgorithm
{
public:
    using S::SimpleAlgorithm::SimpleAlgorithm;
    void sparsity() { build_sparsity(); }
    const std::vector<int>& twins() const { return periodicTwin_; }
    void assemble(const double* aP, const double* phi)
    {
        build_sparsity();
        const std::size_t nC = mesh_.cells().size(), nF = mesh_.faces().size();
        aP_.assign(aP, aP + nC);
        phiFlux_.assign(phi, phi + nF);
        assemble_pressure_correction();
    }
    // SIMPLEC: the momentum matrix's values on the shared pattern
    void assemble_simplec(const double* aP, const double* mom, const double* phi)
    {
        build_sparsity();
        const std::size_t nC = mesh_.cells().size(), nF = mesh_.faces().size();
        aP_.assign(aP, aP + nC);
        phiFlux_.assign(phi, phi + nF);
        A_mom_.values.assign(mom, mom + A_mom_.colIdx.size());
        assemble_pressure_correction();
    }
    // compute_face_fluxes with the given cell velocities (after build_sparsity,
    // as iterate() runs it first: it also pairs the periodic faces)
    void fluxes(const double* Ux, const double* Uy, const double* Uz)
    {
        build_sparsity();
        const std::size_t nC = mesh_.cells().size();
        auto& U = F_.vector("U", nC);
        U.x.assign(Ux, Ux + nC);
        U.y.assign(Uy, Uy + nC);
        U.z.assign(Uz, Uz + nC);
        compute_face_fluxes();
    }
    // correct_fields on the given state; the fields are read back by the caller
    void correct(const double* aP, const double* pPrime, const double* p, const double* Ux, const double* Uy,
                 const double* Uz, const double* phi)
    {
        const std::size_t nC = mesh_.cells().size(), nF = mesh_.faces().size();
        auto& U = F_.vector("U", nC);
        auto& pp = F_.scalar("p", nC);
        U.x.assign(Ux, Ux + nC);
        U.y.assign(Uy, Uy + nC);
        U.z.assign(Uz, Uz + nC);
        pp.assign(p, p + nC);
        aP_.assign(aP, aP + nC);
        pPrime_.assign(pPrime, pPrime + nC);
        phiFlux_.assign(phi, phi + nF);
        correct_fields();
    }
    // assemble_momentum(comp) on the given state; opt = {rho, mu, urfU, dt}
    void momentum(const double* opt, int bdf2, int timeStep, int comp, const double* Ux, const double* Uy,
                  const double* Uz, const double* p, const double* phi, const double* Un, const double* Unm1)
    {
        build_sparsity();
        const std::size_t nC = mesh_.cells().size(), nF = mesh_.faces().size();
        auto& U = F_.vector("U", nC);
        U.x.assign(Ux, Ux + nC);
        U.y.assign(Uy, Uy + nC);
        U.z.assign(Uz, Uz + nC);
        F_.scalar("p", nC).assign(p, p + nC);
        phiFlux_.assign(phi, phi + nF);
        aP_.assign(nC, 0.0);
        opt_.rho = opt[0];
        opt_.mu = opt[1];
        opt_.urfU = opt[2];
        opt_.dt = opt[3];
        opt_.timeScheme = bdf2 ? S::TemporalScheme::BDF2 : S::TemporalScheme::ImplicitEuler;
        timeStep_ = timeStep;
        Ux_n_.assign(Un, Un + nC);
        Uy_n_.assign(Un + nC, Un + 2 * nC);
        Uz_n_.assign(Un + 2 * nC, Un + 3 * nC);
        Ux_nm1_.assign(Unm1, Unm1 + nC);
        Uy_nm1_.assign(Unm1 + nC, Unm1 + 2 * nC);
        Uz_nm1_.assign(Unm1 + 2 * nC, Unm1 + 3 * nC);
        assemble_momentum(comp);
    }
    const S::CSRMatrix& Amom() const { return A_mom_; }
    S::FieldRegistry& fields() { return F_; }
    const S::CSRMatrix& Ap() const { return A_p_; }
    const Vec& rhs() const { return rhs_; }
    const Vec& aP() const { return aP_; }
    const Vec& phi() const { return phiFlux_; }
};

std::vector<S::BoundarySpec> make_bcs(int nbc, const std::uint32_t* zones, const int* types)
{
    std::vector<S::BoundarySpec> b;
    for (int i = 0; i < nbc; ++i)
        b.push_back(S::BoundarySpec{zones[i], static_cast<S::BCType>(types[i]), 0.0, {0, 0, 0}, ""});
    return b;
}

S::CSRMatrix make_csr(int n, const int* rowPtr, const int* colIdx, const double* values)
{
    S::CSRMatrix A;
    A.rowPtr.assign(rowPtr, rowPtr + n + 1);
    const int nnz = rowPtr[n];
    A.colIdx.assign(colIdx, colIdx + nnz);
    A.values.assign(values, values + nnz);
    return A;
}

// Pressure solver that records each system it is handed (A_p_, rhs_) and the
// assembly inputs (aP_, phiFlux_) visible at that moment, then solves it with
// the reference CG.
class RecordingSolver final : public S::ILinearSolver
{
public:
    RecordingSolver(S::LinearSolverConfig c) : inner_(S::make_cg(c)) {}
    int solve(const S::CSRMatrix& A, const Vec& b, Vec& x) override
    {
        const int idx = static_cast<int>(iters.size());
        const bool rec = idx < nRecord || (recordStride > 0 && (idx + 1) % recordStride == 0);
        if (rec) {
            if (rowPtr.empty()) {
                rowPtr.assign(A.rowPtr.begin(), A.rowPtr.end());
                colIdx.assign(A.colIdx.begin(), A.colIdx.end());
            }
            values.insert(values.end(), A.values.begin(), A.values.end());
            rhs.insert(rhs.end(), b.begin(), b.end());
            if (probe) {
                aP.insert(aP.end(), probe->aP().begin(), probe->aP().end());
                phi.insert(phi.end(), probe->phi().begin(), probe->phi().end());
            }
        }
        const auto t0 = std::chrono::steady_clock::now();
        const int it = inner_->solve(A, b, x);
        seconds += std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        if (rec) {
            xs.insert(xs.end(), x.begin(), x.end());
            ++nRecorded;
        }
        iters.push_back(it);
        res.push_back(inner_->last_residual());
        return it;
    }
    double last_residual() const override { return inner_->last_residual(); }

    int nRecord = 0;       // record the first nRecord solves
    int recordStride = 0;  // and, when > 0, every recordStride-th solve
    int nRecorded = 0;
    const AssemblyProbe* probe = nullptr;
    std::vector<int> rowPtr, colIdx, iters;
    std::vector<double> values, rhs, xs, aP, phi, res;
    double seconds = 0.0;

private:
    std::unique_ptr<S::ILinearSolver> inner_;
};

RecordingSolver* g_last_cavity = nullptr;

} // namespace

extern "C" {

// ------------------------------------------------------------------ mesh
void* ref_mesh_cartesian(int nx, int ny, int nz, double ex, double ey, double ez)
{
    auto* m = new RefMesh;
    M::CartesianGridSpec gs{{0, 0, 0}, {ex, ey, ez}, nx, ny, nz};
    M::CartesianMesher(gs).generate(m->mesh);
    return m;
}

void ref_mesh_free(void* h) { delete static_cast<RefMesh*>(h); }

void ref_mesh_sizes(void* h, std::int64_t* out)
{
    auto& m = static_cast<RefMesh*>(h)->mesh;
    out[0] = static_cast<std::int64_t>(m.cells().size());
    out[1] = static_cast<std::int64_t>(m.faces().size());
    out[2] = static_cast<std::int64_t>(m.nodes().size());
    out[3] = static_cast<std::int64_t>(m.cells().faceIndices.size());
    out[4] = static_cast<std::int64_t>(m.faces().nodeIndices.size());
}

void ref_mesh_get_nodes(void* h, double* x, double* y, double* z)
{
    auto& N = static_cast<RefMesh*>(h)->mesh.nodes();
    std::copy(N.x.begin(), N.x.end(), x);
    std::copy(N.y.begin(), N.y.end(), y);
    std::copy(N.z.begin(), N.z.end(), z);
}

// Overwrite node coordinates and recompute face/cell geometry.
void ref_mesh_set_nodes(void* h, const double* x, const double* y, const double* z)
{
    auto& m = static_cast<RefMesh*>(h)->mesh;
    auto& N = m.nodes();
    const std::size_t nN = N.size();
    std::copy(x, x + nN, N.x.begin());
    std::copy(y, y + nN, N.y.begin());
    std::copy(z, z + nN, N.z.begin());
    m.compute_geometry();
}

void ref_mesh_get_faces(void* h, std::uint64_t* owner, std::uint64_t* neighbor, double* ax, double* ay,
                        double* az, double* cx, double* cy, double* cz, std::uint32_t* zone)
{
    auto& F = static_cast<RefMesh*>(h)->mesh.faces();
    std::copy(F.owner.begin(), F.owner.end(), owner);
    std::copy(F.neighbor.begin(), F.neighbor.end(), neighbor);
    std::copy(F.areaX.begin(), F.areaX.end(), ax);
    std::copy(F.areaY.begin(), F.areaY.end(), ay);
    std::copy(F.areaZ.begin(), F.areaZ.end(), az);
    std::copy(F.centroidX.begin(), F.centroidX.end(), cx);
    std::copy(F.centroidY.begin(), F.centroidY.end(), cy);
    std::copy(F.centroidZ.begin(), F.centroidZ.end(), cz);
    std::copy(F.boundaryZone.begin(), F.boundaryZone.end(), zone);
}

void ref_mesh_get_face_nodes(void* h, std::int32_t* nodeOffsets, std::uint64_t* nodeIndices)
{
    auto& F = static_cast<RefMesh*>(h)->mesh.faces();
    std::copy(F.nodeOffsets.begin(), F.nodeOffsets.end(), nodeOffsets);
    std::copy(F.nodeIndices.begin(), F.nodeIndices.end(), nodeIndices);
}

void ref_mesh_get_cells(void* h, double* vol, double* cx, double* cy, double* cz,
                        std::int32_t* faceOffsets, std::uint64_t* faceIndices)
{
    auto& C = static_cast<RefMesh*>(h)->mesh.cells();
    std::copy(C.volume.begin(), C.volume.end(), vol);
    std::copy(C.centroidX.begin(), C.centroidX.end(), cx);
    std::copy(C.centroidY.begin(), C.centroidY.end(), cy);
    std::copy(C.centroidZ.begin(), C.centroidZ.end(), cz);
    std::copy(C.faceOffsets.begin(), C.faceOffsets.end(), faceOffsets);
    std::copy(C.faceIndices.begin(), C.faceIndices.end(), faceIndices);
}

void ref_mesh_rcm(void* h, std::int64_t* out)
{
    auto st = M::ops::renumber_cells_cuthill_mckee(static_cast<RefMesh*>(h)->mesh);
    out[0] = static_cast<std::int64_t>(st.bandwidthBefore);
    out[1] = static_cast<std::int64_t>(st.bandwidthAfter);
    out[2] = static_cast<std::int64_t>(st.cellsPermuted);
}

// ------------------------------------------------------------------ assembly
std::int64_t ref_sparsity_nnz(void* h, int nbc, const std::uint32_t* bcZones, const int* bcTypes)
{
    auto& m = static_cast<RefMesh*>(h)->mesh;
    S::FieldRegistry f;
    auto bcs = make_bcs(nbc, bcZones, bcTypes);  // periodic specs add twin columns
    S::LinearSolverConfig c;
    auto s1 = S::make_cg(c), s2 = S::make_cg(c);
    AssemblyProbe p(m, f, bcs, *s1, *s2, S::SimpleOptions{});
    p.sparsity();
    return static_cast<std::int64_t>(p.Ap().colIdx.size());
}

int ref_assemble(void* h, int nbc, const std::uint32_t* bcZones, const int* bcTypes, double rho,
                 const double* aP, const double* phi, std::int32_t* rowPtr, std::int32_t* colIdx,
                 double* values, double* rhs)
{
    auto& m = static_cast<RefMesh*>(h)->mesh;
    S::FieldRegistry f;
    auto bcs = make_bcs(nbc, bcZones, bcTypes);
    S::LinearSolverConfig c;
    auto s1 = S::make_cg(c), s2 = S::make_cg(c);
    S::SimpleOptions o;
    o.rho = rho;
    AssemblyProbe p(m, f, bcs, *s1, *s2, o);
    p.assemble(aP, phi);
    const auto& A = p.Ap();
    std::copy(A.rowPtr.begin(), A.rowPtr.end(), rowPtr);
    std::copy(A.colIdx.begin(), A.colIdx.end(), colIdx);
    std::copy(A.values.begin(), A.values.end(), values);
    std::copy(p.rhs().begin(), p.rhs().end(), rhs);
    return 0;
}

// SimpleAlgorithm::build_periodic_pairs (SimpleAlgorithm.cpp:101-186) through
// build_sparsity: twin[nF], -1 where a face has no periodic partner.
int ref_periodic_twins(void* h, int nbc, const std::uint32_t* bcZones, const int* bcTypes, std::int32_t* twin)
{
    auto& m = static_cast<RefMesh*>(h)->mesh;
    S::FieldRegistry f;
    auto bcs = make_bcs(nbc, bcZones, bcTypes);
    S::LinearSolverConfig c;
    auto s1 = S::make_cg(c), s2 = S::make_cg(c);
    AssemblyProbe p(m, f, bcs, *s1, *s2, S::SimpleOptions{});
    p.sparsity();
    const auto& t = p.twins();
    const std::size_t nF = m.faces().size();
    for (std::size_t i = 0; i < nF; ++i)
        twin[i] = t.empty() ? -1 : t[i];
    return 0;
}

std::vector<S::BoundarySpec> make_bcs_vec(int nbc, const std::uint32_t* zones, const int* types, const double* vec)
{
    std::vector<S::BoundarySpec> b;
    for (int i = 0; i < nbc; ++i) {
        S::BoundarySpec s{zones[i], static_cast<S::BCType>(types[i]), 0.0, {0, 0, 0}, ""};
        if (vec) {
            s.vectorValue[0] = vec[3 * i];
            s.vectorValue[1] = vec[3 * i + 1];
            s.vectorValue[2] = vec[3 * i + 2];
        }
        b.push_back(s);
    }
    return b;
}

// SimpleAlgorithm::compute_face_fluxes (SimpleAlgorithm.cpp:201-237).
int ref_face_fluxes(void* h, int nbc, const std::uint32_t* bcZones, const int* bcTypes, const double* bcVec,
                    double rho, const double* Ux, const double* Uy, const double* Uz, double* phi)
{
    auto& m = static_cast<RefMesh*>(h)->mesh;
    S::FieldRegistry f;
    auto bcs = make_bcs_vec(nbc, bcZones, bcTypes, bcVec);
    S::LinearSolverConfig c;
    auto s1 = S::make_cg(c), s2 = S::make_cg(c);
    S::SimpleOptions o;
    o.rho = rho;
    AssemblyProbe p(m, f, bcs, *s1, *s2, o);
    p.fluxes(Ux, Uy, Uz);
    std::copy(p.phi().begin(), p.phi().end(), phi);
    return 0;
}

// LeastSquaresGradient::evaluate (Gradient.cpp:91-133).
int ref_lsq_gradient(void* h, const double* phi, double* gx, double* gy, double* gz)
{
    auto& m = static_cast<RefMesh*>(h)->mesh;
    const std::size_t nC = m.cells().size();
    S::LeastSquaresGradient G(m);
    S::ScalarField f(phi, phi + nC);
    S::VectorField g;
    G.evaluate(f, g);
    std::copy(g.x.begin(), g.x.end(), gx);
    std::copy(g.y.begin(), g.y.end(), gy);
    std::copy(g.z.begin(), g.z.end(), gz);
    return 0;
}

// SimpleAlgorithm::correct_fields (SimpleAlgorithm.cpp:450-487); p, U and phi in/out.
int ref_correct_fields(void* h, double rho, double urfP, const double* aP, const double* pPrime, double* p, double* Ux,
                       double* Uy, double* Uz, double* phi)
{
    auto& m = static_cast<RefMesh*>(h)->mesh;
    const std::size_t nC = m.cells().size();
    S::FieldRegistry f;
    std::vector<S::BoundarySpec> bcs;
    S::LinearSolverConfig c;
    auto s1 = S::make_cg(c), s2 = S::make_cg(c);
    S::SimpleOptions o;
    o.rho = rho;
    o.urfP = urfP;
    AssemblyProbe pr(m, f, bcs, *s1, *s2, o);
    pr.correct(aP, pPrime, p, Ux, Uy, Uz, phi);
    auto& U = *pr.fields().find_vector("U");
    auto& pp = *pr.fields().find_scalar("p");
    std::copy(pp.begin(), pp.end(), p);
    std::copy(U.x.begin(), U.x.end(), Ux);
    std::copy(U.y.begin(), U.y.end(), Uy);
    std::copy(U.z.begin(), U.z.end(), Uz);
    std::copy(pr.phi().begin(), pr.phi().end(), phi);
    (void)nC;
    return 0;
}

int ref_assemble_simplec(void* h, int nbc, const std::uint32_t* bcZones, const int* bcTypes, double rho,
                         const double* aP, const double* mom, const double* phi, std::int32_t* rowPtr,
                         std::int32_t* colIdx, double* values, double* rhs)
{
    auto& m = static_cast<RefMesh*>(h)->mesh;
    S::FieldRegistry f;
    auto bcs = make_bcs(nbc, bcZones, bcTypes);
    S::LinearSolverConfig c;
    auto s1 = S::make_cg(c), s2 = S::make_cg(c);
    S::SimpleOptions o;
    o.rho = rho;
    o.algorithm = S::PvCouplingVariant::SIMPLEC;
    AssemblyProbe p(m, f, bcs, *s1, *s2, o);
    p.assemble_simplec(aP, mom, phi);
    const auto& A = p.Ap();
    std::copy(A.rowPtr.begin(), A.rowPtr.end(), rowPtr);
    std::copy(A.colIdx.begin(), A.colIdx.end(), colIdx);
    std::copy(A.values.begin(), A.values.end(), values);
    std::copy(p.rhs().begin(), p.rhs().end(), rhs);
    return 0;
}

// SimpleAlgorithm::assemble_momentum (SimpleAlgorithm.cpp:240-355), one
// component.  U, Un, Unm1 are [3][nC]; opt = {rho, mu, urfU, dt}; bdf2 selects
// TemporalScheme::BDF2 (else ImplicitEuler); aP receives aP_ (written by the
// reference for component 0 only, zeros otherwise).
int ref_assemble_momentum(void* h, int nbc, const std::uint32_t* bcZones, const int* bcTypes, const double* bcVec,
                          const double* opt, int bdf2, int timeStep, int comp, const double* U, const double* p,
                          const double* phi, const double* Un, const double* Unm1, double* values, double* rhs,
                          double* aP)
{
    auto& m = static_cast<RefMesh*>(h)->mesh;
    const std::size_t nC = m.cells().size();
    S::FieldRegistry f;
    auto bcs = make_bcs_vec(nbc, bcZones, bcTypes, bcVec);
    S::LinearSolverConfig c;
    auto s1 = S::make_cg(c), s2 = S::make_cg(c);
    AssemblyProbe pr(m, f, bcs, *s1, *s2, S::SimpleOptions{});
    pr.momentum(opt, bdf2, timeStep, comp, U, U + nC, U + 2 * nC, p, phi, Un, Unm1);
    const auto& A = pr.Amom();
    std::copy(A.values.begin(), A.values.end(), values);
    std::copy(pr.rhs().begin(), pr.rhs().end(), rhs);
    std::copy(pr.aP().begin(), pr.aP().end(), aP);
    return 0;
}

// ------------------------------------------------------------------ solvers
// make_gmres / make_bicgstab / make_cg / make_tfqmr (LinearSolvers.cpp:462-473,
// 616-619), as make_linear_solver dispatches them (Solver.cpp:25-39): kind is
// the LinearSolverKind ordinal (0 GMRES, 1 BiCGSTAB, 2 CG, 3 TFQMR).  Returns the
// iteration count; x from 0.
int ref_krylov(int kind, int precond, double tol, int maxit, int restart, int n, const int* rowPtr,
               const int* colIdx, const double* values, const double* b, double* x, double* lastRes,
               double* seconds)
{
    auto A = make_csr(n, rowPtr, colIdx, values);
    S::LinearSolverConfig c;
    c.kind = static_cast<S::LinearSolverKind>(kind);
    c.preconditioner = static_cast<S::PreconditionerKind>(precond);
    c.tolerance = tol;
    c.maxIterations = maxit;
    c.restart = restart;
    std::unique_ptr<S::ILinearSolver> sol = kind == 1   ? S::make_bicgstab(c)
                                            : kind == 2 ? S::make_cg(c)
                                            : kind == 3 ? S::make_tfqmr(c)
                                                        : S::make_gmres(c);
    Vec bb(b, b + n), xx(n, 0.0);
    const auto t0 = std::chrono::steady_clock::now();
    const int it = sol->solve(A, bb, xx);
    if (seconds)
        *seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    std::copy(xx.begin(), xx.end(), x);
    *lastRes = sol->last_residual();
    return it;
}

// CGSolver::solve (LinearSolvers.cpp:420) with the given preconditioner
// (PreconditionerKind ordinal).  Returns the iteration count.
int ref_cg(int n, const int* rowPtr, const int* colIdx, const double* values, const double* b,
           int precond, double tol, int maxit, double* x, double* lastRes, double* seconds)
{
    auto A = make_csr(n, rowPtr, colIdx, values);
    S::LinearSolverConfig c;
    c.kind = S::LinearSolverKind::CG;
    c.preconditioner = static_cast<S::PreconditionerKind>(precond);
    c.tolerance = tol;
    c.maxIterations = maxit;
    auto cg = S::make_cg(c);
    Vec bb(b, b + n), xx(n, 0.0);
    const auto t0 = std::chrono::steady_clock::now();
    const int it = cg->solve(A, bb, xx);
    if (seconds)
        *seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    std::copy(xx.begin(), xx.end(), x);
    *lastRes = cg->last_residual();
    return it;
}

// IPreconditioner::setup + apply for one r.
void ref_precond_apply(int kind, int n, const int* rowPtr, const int* colIdx, const double* values,
                       const double* r, double* z)
{
    auto A = make_csr(n, rowPtr, colIdx, values);
    auto M = S::make_preconditioner(static_cast<S::PreconditionerKind>(kind));
    M->setup(A);
    Vec rr(r, r + n), zz;
    M->apply(rr, zz);
    std::copy(zz.begin(), zz.end(), z);
}

void ref_spmv(int n, const int* rowPtr, const int* colIdx, const double* values, const double* x,
              double* y)
{
    auto A = make_csr(n, rowPtr, colIdx, values);
    Vec xx(x, x + n), yy;
    A.spmv(xx, yy);
    std::copy(yy.begin(), yy.end(), y);
}

// ------------------------------------------------------------------ SIMPLE runs
// An ILinearSolver that records the iteration count of every solve.
class CountingSolver final : public S::ILinearSolver
{
public:
    explicit CountingSolver(std::unique_ptr<S::ILinearSolver> s) : inner_(std::move(s)) {}
    int solve(const S::CSRMatrix& A, const Vec& b, Vec& x) override
    {
        const int it = inner_->solve(A, b, x);
        iters.push_back(it);
        return it;
    }
    double last_residual() const override { return inner_->last_residual(); }
    std::vector<int> iters;

private:
    std::unique_ptr<S::ILinearSolver> inner_;
};

std::unique_ptr<S::ILinearSolver> make_kind(const int* cfg, double tol)
{
    S::LinearSolverConfig c;
    c.kind = static_cast<S::LinearSolverKind>(cfg[0]);
    c.preconditioner = static_cast<S::PreconditionerKind>(cfg[1]);
    c.maxIterations = cfg[2];
    c.restart = cfg[3];
    c.tolerance = tol;
    return cfg[0] == 1   ? S::make_bicgstab(c)
           : cfg[0] == 2 ? S::make_cg(c)
           : cfg[0] == 3 ? S::make_tfqmr(c)
                         : S::make_gmres(c);
}

// SimpleAlgorithm on the given mesh from U (in [3][nC]) and p: nOuter calls of
// iterate() (dt == 0) or of advance_time_step(nInner) (dt > 0).  opt = {rho,
// mu, urfU, urfP, dt}; flags bit 0 TemporalScheme::BDF2 (else ImplicitEuler),
// bit 1 PvCouplingVariant::SIMPLEC.  momCfg / pCfg = {kind, precond, maxIt,
// restart}.  Out: U, p, phi after the run; res[nOuter][4] the residuals each
// call returned; iters[...] every linear solve's count in call order (size
// returned in *nIters, at most maxIters written).
int ref_simple_run(void* h, int nbc, const std::uint32_t* bcZones, const int* bcTypes, const double* bcVec,
                   const double* opt, int flags, const int* momCfg, double momTol, const int* pCfg, double pTol,
                   int nOuter, int nInner, double* U, double* p, double* phi, double* res, int* iters, int maxIters,
                   int* nIters, double* seconds)
{
    auto& m = static_cast<RefMesh*>(h)->mesh;
    const std::size_t nC = m.cells().size();
    S::FieldRegistry f;
    auto& Uf = f.vector("U", nC);
    Uf.x.assign(U, U + nC);
    Uf.y.assign(U + nC, U + 2 * nC);
    Uf.z.assign(U + 2 * nC, U + 3 * nC);
    f.scalar("p", nC).assign(p, p + nC);
    auto bcs = make_bcs_vec(nbc, bcZones, bcTypes, bcVec);
    CountingSolver mom(make_kind(momCfg, momTol)), pres(make_kind(pCfg, pTol));
    S::SimpleOptions o;
    o.rho = opt[0];
    o.mu = opt[1];
    o.urfU = opt[2];
    o.urfP = opt[3];
    o.dt = opt[4];
    o.timeScheme = (flags & 1) ? S::TemporalScheme::BDF2 : S::TemporalScheme::ImplicitEuler;
    o.algorithm = (flags & 2) ? S::PvCouplingVariant::SIMPLEC : S::PvCouplingVariant::SIMPLE;
    AssemblyProbe simple(m, f, bcs, mom, pres, o);
    const auto t0 = std::chrono::steady_clock::now();
    for (int i = 0; i < nOuter; ++i) {
        const S::SimpleResiduals r = o.dt > 0.0 ? simple.advance_time_step(nInner) : simple.iterate();
        res[4 * i] = r.mom[0];
        res[4 * i + 1] = r.mom[1];
        res[4 * i + 2] = r.mom[2];
        res[4 * i + 3] = r.cont;
    }
    if (seconds)
        *seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    auto& Uo = *f.find_vector("U");
    std::copy(Uo.x.begin(), Uo.x.end(), U);
    std::copy(Uo.y.begin(), Uo.y.end(), U + nC);
    std::copy(Uo.z.begin(), Uo.z.end(), U + 2 * nC);
    const auto& pp = *f.find_scalar("p");
    std::copy(pp.begin(), pp.end(), p);
    std::copy(simple.phi().begin(), simple.phi().end(), phi);
    // interleave: mom x, y, z then p for every iterate()
    std::vector<int> all;
    for (std::size_t k = 0; k < pres.iters.size(); ++k) {
        for (int c = 0; c < 3; ++c)
            all.push_back(3 * k + c < mom.iters.size() ? mom.iters[3 * k + c] : -1);
        all.push_back(pres.iters[k]);
    }
    *nIters = static_cast<int>(all.size());
    for (int i = 0; i < static_cast<int>(all.size()) && i < maxIters; ++i)
        iters[i] = all[i];
    return 0;
}

// PisoAlgorithm / PimpleAlgorithm with the face fluxes readable.
class PisoProbe : public S::PisoAlgorithm
{
public:
    using S::PisoAlgorithm::PisoAlgorithm;
    const Vec& phi() const { return phiFlux_; }
};
class PimpleProbe : public S::PimpleAlgorithm
{
public:
    using S::PimpleAlgorithm::PimpleAlgorithm;
    const Vec& phi() const { return phiFlux_; }
};

// PisoAlgorithm (variant 1) or PimpleAlgorithm (variant 2) on the given mesh
// from U, p: nSteps calls of advance_time_step(1).  opt = {rho, mu, dt, urfU,
// urfP, tolU, tolP}; loops = {nOuterCorrectors, nCorrectors, nNonOrthCorr,
// momentumPredictor}; flags bit 0 BDF2 (else ImplicitEuler).  Out as
// ref_simple_run, plus lastOuter[k] (PIMPLE's last_outer_iters after step k).
int ref_piso_pimple_run(void* h, int variant, int nbc, const std::uint32_t* bcZones, const int* bcTypes,
                        const double* bcVec, const double* opt, const int* loops, int flags, const int* momCfg,
                        double momTol, const int* pCfg, double pTol, int nSteps, double* U, double* p, double* phi,
                        double* res, int* lastOuter)
{
    auto& m = static_cast<RefMesh*>(h)->mesh;
    const std::size_t nC = m.cells().size();
    S::FieldRegistry f;
    auto& Uf = f.vector("U", nC);
    Uf.x.assign(U, U + nC);
    Uf.y.assign(U + nC, U + 2 * nC);
    Uf.z.assign(U + 2 * nC, U + 3 * nC);
    f.scalar("p", nC).assign(p, p + nC);
    auto bcs = make_bcs_vec(nbc, bcZones, bcTypes, bcVec);
    auto mom = make_kind(momCfg, momTol);
    auto pres = make_kind(pCfg, pTol);
    const auto scheme = (flags & 1) ? S::TemporalScheme::BDF2 : S::TemporalScheme::ImplicitEuler;
    std::unique_ptr<S::SimpleAlgorithm> alg;
    const Vec* phiRef = nullptr;
    PimpleProbe* pimple = nullptr;
    if (variant == 1) {
        S::PisoOptions o;
        o.nCorrectors = loops[1];
        o.nNonOrthCorr = loops[2];
        o.rho = opt[0];
        o.mu = opt[1];
        o.dt = opt[2];
        o.timeScheme = scheme;
        auto* a = new PisoProbe(m, f, bcs, *mom, *pres, o);
        phiRef = &a->phi();
        alg.reset(a);
    } else {
        S::PimpleOptions o;
        o.nOuterCorrectors = loops[0];
        o.nCorrectors = loops[1];
        o.nNonOrthCorr = loops[2];
        o.momentumPredictor = loops[3] != 0;
        o.urfU = opt[3];
        o.urfP = opt[4];
        o.tolU = opt[5];
        o.tolP = opt[6];
        o.rho = opt[0];
        o.mu = opt[1];
        o.dt = opt[2];
        o.timeScheme = scheme;
        pimple = new PimpleProbe(m, f, bcs, *mom, *pres, o);
        phiRef = &pimple->phi();
        alg.reset(pimple);
    }
    for (int k = 0; k < nSteps; ++k) {
        const S::SimpleResiduals r = alg->advance_time_step(1);
        res[4 * k] = r.mom[0];
        res[4 * k + 1] = r.mom[1];
        res[4 * k + 2] = r.mom[2];
        res[4 * k + 3] = r.cont;
        lastOuter[k] = pimple ? pimple->last_outer_iters() : 0;
    }
    auto& Uo = *f.find_vector("U");
    std::copy(Uo.x.begin(), Uo.x.end(), U);
    std::copy(Uo.y.begin(), Uo.y.end(), U + nC);
    std::copy(Uo.z.begin(), Uo.z.end(), U + 2 * nC);
    const auto& pp = *f.find_scalar("p");
    std::copy(pp.begin(), pp.end(), p);
    std::copy(phiRef->begin(), phiRef->end(), phi);
    return 0;
}

// ------------------------------------------------------------------ checkpoint
// io::Checkpoint::write of the given mesh and fields: nf fields in the given
// insertion order, isVector[i] selects vector (data [3][n]) or scalar (data [n]).
int ref_checkpoint_write(void* h, const char* path, int nf, const char* const* names, const int* isVector,
                         const std::int64_t* sizes, const double* const* data, int iteration, double time,
                         std::uint64_t hash)
{
    auto& m = static_cast<RefMesh*>(h)->mesh;
    S::FieldRegistry f;
    for (int i = 0; i < nf; ++i) {
        const std::size_t n = static_cast<std::size_t>(sizes[i]);
        if (isVector[i]) {
            auto& v = f.vector(names[i], n);
            std::copy(data[i], data[i] + n, v.x.begin());
            std::copy(data[i] + n, data[i] + 2 * n, v.y.begin());
            std::copy(data[i] + 2 * n, data[i] + 3 * n, v.z.begin());
        } else {
            auto& s = f.scalar(names[i], n);
            std::copy(data[i], data[i] + n, s.begin());
        }
    }
    simall::io::CheckpointMeta meta{};
    meta.iteration = iteration;
    meta.time = time;
    meta.settingsHash = hash;
    return simall::io::Checkpoint::write(path, m, f, meta) ? 0 : 1;
}

// io::Checkpoint::read: returns a mesh handle (cells, faces, nodes in sizes[0..2])
// and keeps the fields for ref_checkpoint_field; meta[0] = iteration, [1] = time,
// [2] = settings hash bits.
S::FieldRegistry* g_ckpt_fields = nullptr;
void* ref_checkpoint_read(const char* path, std::int64_t* sizes, double* meta)
{
    auto* rm = new RefMesh;
    delete g_ckpt_fields;
    g_ckpt_fields = new S::FieldRegistry;
    simall::io::CheckpointMeta md{};
    if (!simall::io::Checkpoint::read(path, rm->mesh, *g_ckpt_fields, md)) {
        delete rm;
        return nullptr;
    }
    sizes[0] = static_cast<std::int64_t>(rm->mesh.cells().size());
    sizes[1] = static_cast<std::int64_t>(rm->mesh.faces().size());
    sizes[2] = static_cast<std::int64_t>(rm->mesh.nodes().size());
    sizes[3] = static_cast<std::int64_t>(g_ckpt_fields->scalars().size());
    sizes[4] = static_cast<std::int64_t>(g_ckpt_fields->vectors().size());
    meta[0] = md.iteration;
    meta[1] = md.time;
    std::memcpy(&meta[2], &md.settingsHash, 8);
    return rm;
}

// A field of the last ref_checkpoint_read: returns its size (-1 if absent);
// out receives n (scalar) or 3n (vector) values when not null.
std::int64_t ref_checkpoint_field(const char* name, int isVector, double* out)
{
    if (!g_ckpt_fields)
        return -1;
    if (isVector) {
        auto* v = g_ckpt_fields->find_vector(name);
        if (!v)
            return -1;
        const std::size_t n = v->size();
        if (out) {
            std::copy(v->x.begin(), v->x.end(), out);
            std::copy(v->y.begin(), v->y.end(), out + n);
            std::copy(v->z.begin(), v->z.end(), out + 2 * n);
        }
        return static_cast<std::int64_t>(n);
    }
    auto* s = g_ckpt_fields->find_scalar(name);
    if (!s)
        return -1;
    if (out)
        std::copy(s->begin(), s->end(), out);
    return static_cast<std::int64_t>(s->size());
}

// ------------------------------------------------------------------ SIMP
// SimpTopology::initialize + nSteps step() calls on the given mesh; before
// step k the caller's sensitivity dC[k] (nC values) is stored in "dC_drho".
// cfg = {penalty, K_min, K_max, filterRadius, volumeFraction, move, damping,
// rhoMin}.  Out: change[k], and the final rho, rhoTilde, K_simp,
// dC_drhoTilde.
int ref_simp_run(void* h, const double* cfg, int nSteps, const double* dC, double* change, double* rho,
                 double* rhoT, double* kSimp, double* dCt)
{
    auto& m = static_cast<RefMesh*>(h)->mesh;
    const std::size_t nC = m.cells().size();
    S::FieldRegistry f;
    simall::optimization::SimpConfig c;
    c.penalty = cfg[0];
    c.K_min = cfg[1];
    c.K_max = cfg[2];
    c.filterRadius = cfg[3];
    c.volumeFraction = cfg[4];
    c.move = cfg[5];
    c.damping = cfg[6];
    c.rhoMin = cfg[7];
    simall::optimization::SimpTopology simp;
    simp.initialize(m, f, c);
    for (int k = 0; k < nSteps; ++k) {
        auto& d = *f.find_scalar("dC_drho");
        std::copy(dC + k * nC, dC + (k + 1) * nC, d.begin());
        change[k] = simp.step(m, f);
    }
    auto cp = [&](const char* name, double* out) {
        const auto& v = *f.find_scalar(name);
        std::copy(v.begin(), v.end(), out);
    };
    cp("rho", rho);
    cp("rhoTilde", rhoT);
    cp("K_simp", kSimp);
    cp("dC_drhoTilde", dCt);
    return 0;
}

// ------------------------------------------------------------------ cavity SIMPLE
// Runs nOuter SIMPLE iterations of the lid-driven cavity on an N x N x 1 grid
// (extent 1 x 1 x 1/N; zones 1,2,3,5,6 NoSlipWall, zone 4 MovingWall (1,0,0))
// with momentum GMRES(30)+ILU (tol 1e-6, 200 it) and pressure CG with the
// given preconditioner.  The first nRecord pressure systems are recorded;
// fetch them with ref_cavity_fetch.
int ref_cavity_run(int N, double mu, int nOuter, int nRecord, int recordStride, int precond, double tol, int maxit,
                   std::int64_t* sizes, double* pSolveSeconds)
{
    M::Mesh mesh;
    M::CartesianGridSpec gs{{0, 0, 0}, {1.0, 1.0, 1.0 / N}, N, N, 1};
    M::CartesianMesher(gs).generate(mesh);
    const std::size_t nC = mesh.cells().size();
    S::FieldRegistry fields;
    fields.scalar("p", nC);
    fields.vector("U", nC);
    std::vector<S::BoundarySpec> bcs;
    for (std::uint32_t z : {1u, 2u, 3u, 5u, 6u})
        bcs.push_back(S::BoundarySpec{z, S::BCType::NoSlipWall, 0.0, {0, 0, 0}, ""});
    bcs.push_back(S::BoundarySpec{4u, S::BCType::MovingWall, 0.0, {1.0, 0, 0}, ""});

    S::LinearSolverConfig mc;
    mc.kind = S::LinearSolverKind::GMRES;
    mc.preconditioner = S::PreconditionerKind::ILU;
    mc.tolerance = 1e-6;
    mc.maxIterations = 200;
    mc.restart = 30;
    auto mom = S::make_gmres(mc);
    S::LinearSolverConfig pc;
    pc.kind = S::LinearSolverKind::CG;
    pc.preconditioner = static_cast<S::PreconditionerKind>(precond);
    pc.tolerance = tol;
    pc.maxIterations = maxit;
    delete g_last_cavity;
    g_last_cavity = new RecordingSolver(pc);
    g_last_cavity->nRecord = nRecord;
    g_last_cavity->recordStride = recordStride;
    S::SimpleOptions o;
    o.urfU = 0.7;
    o.urfP = 0.3;
    o.rho = 1.0;
    o.mu = mu;
    AssemblyProbe simple(mesh, fields, bcs, *mom, *g_last_cavity, o);
    g_last_cavity->probe = &simple;
    for (int i = 0; i < nOuter; ++i)
        simple.iterate();
    g_last_cavity->probe = nullptr;
    sizes[0] = static_cast<std::int64_t>(nC);
    sizes[1] = static_cast<std::int64_t>(g_last_cavity->colIdx.size());
    sizes[2] = static_cast<std::int64_t>(mesh.faces().size());
    sizes[3] = static_cast<std::int64_t>(g_last_cavity->iters.size());
    sizes[4] = static_cast<std::int64_t>(g_last_cavity->nRecorded);
    if (pSolveSeconds)
        *pSolveSeconds = g_last_cavity->seconds;
    return 0;
}

void ref_cavity_fetch(std::int32_t* rowPtr, std::int32_t* colIdx, double* values, double* rhs, double* x,
                      double* aP, double* phi, std::int32_t* iters, double* res)
{
    auto* r = g_last_cavity;
    std::copy(r->rowPtr.begin(), r->rowPtr.end(), rowPtr);
    std::copy(r->colIdx.begin(), r->colIdx.end(), colIdx);
    std::copy(r->values.begin(), r->values.end(), values);
    std::copy(r->rhs.begin(), r->rhs.end(), rhs);
    std::copy(r->xs.begin(), r->xs.end(), x);
    std::copy(r->aP.begin(), r->aP.end(), aP);
    std::copy(r->phi.begin(), r->phi.end(), phi);
    std::copy(r->iters.begin(), r->iters.end(), iters);
    std::copy(r->res.begin(), r->res.end(), res);
}

// ------------------------------------------------------------------ adjoint
// solve_discrete_adjoint on the given CSR (size_t CSR copy) with a
// dRdAlphaTransposeTimes callback for per-face conductances k_f and
// Dirichlet values p_b of the face-conductance Poisson problem:
//   interior face f (o,n):  (dR/dk_f)^T psi = g_f (psi_o - psi_n)(x_o - x_n)
//   Dirichlet face f (o):   (dR/dk_f)^T psi = g_f psi_o (x_o - pb_f)
//   and for its value pb_f: (dR/dpb_f)^T psi = -k_f g_f psi_o
// Design variables: [k_0..k_{nF-1}, pb over the Dirichlet faces in face order].
int ref_discrete_adjoint(int n, const int* rowPtr, const int* colIdx, const double* values,
                         const double* dJdQ, double tol, int maxIter, int restart, int nF,
                         const std::int64_t* owner, const std::int64_t* neighbor, const int* isDirichlet,
                         const double* g, const double* k, const double* pb, const double* x,
                         double* psiOut, double* gradOut, std::int64_t* itersOut, double* resOut)
{
    simall::adjoint::CsrMatrix A;
    A.n = static_cast<std::size_t>(n);
    A.rowPtr.assign(rowPtr, rowPtr + n + 1);
    A.colIdx.assign(colIdx, colIdx + rowPtr[n]);
    A.values.assign(values, values + rowPtr[n]);
    simall::adjoint::DiscreteAdjointInputs in;
    in.A = &A;
    in.dJdQ.assign(dJdQ, dJdQ + n);
    int nD = 0;
    for (int f = 0; f < nF; ++f)
        nD += isDirichlet[f] ? 1 : 0;
    const std::size_t nDV = static_cast<std::size_t>(nF + nD);
    simall::adjoint::DiscreteAdjointOptions opt;
    opt.tol = tol;
    opt.maxIter = static_cast<std::size_t>(maxIter);
    opt.restart = static_cast<std::size_t>(restart);
    // solve_discrete_adjoint calls the callback without handing it psi, so
    // psi is taken from a first run without the callback; the second run is
    // deterministic and reproduces the same psi before calling back.
    auto r1 = simall::adjoint::solve_discrete_adjoint(in, nDV, opt);
    const std::vector<double> psi = r1.psi;
    in.dRdAlphaTransposeTimes = [&](std::vector<double>& out) {
        int d = 0;
        for (int f = 0; f < nF; ++f) {
            const std::int64_t o = owner[f], nb = neighbor[f];
            if (nb >= 0) {
                out[f] = g[f] * (psi[o] - psi[nb]) * (x[o] - x[nb]);
            } else if (isDirichlet[f]) {
                out[f] = g[f] * psi[o] * (x[o] - pb[f]);
                out[nF + d] = -k[f] * g[f] * psi[o];
                ++d;
            } else {
                out[f] = 0.0;
            }
        }
    };
    auto r2 = simall::adjoint::solve_discrete_adjoint(in, nDV, opt);
    std::copy(r2.psi.begin(), r2.psi.end(), psiOut);
    std::copy(r2.gradient.begin(), r2.gradient.end(), gradOut);
    *itersOut = static_cast<std::int64_t>(r2.iterations);
    *resOut = r2.residual;
    return r2.ok ? 0 : 1;
}

// ------------------------------------------------------------------ gpu::CgGpu
// gpu::CgGpu (src/gpu/CgGpu.hpp:49-124, CgGpu.cpp:35-238) on the facade's host
// path: set_matrix (Jacobi diagonal; ILU0 factor with the fall-back to Jacobi
// on a zero pivot), then solve with x as the initial guess.  precond: 0 None,
// 1 Jacobi, 2 ILU0 (GpuPreconditioner order).  out[0..3]: iterations,
// finalResidual, initialResidual, converged; *precondAfter: the preconditioner
// the solver holds afterwards (ILU0 -> Jacobi on a failed factor).
int ref_cggpu_solve(int precond, double tol, int maxIt, double relativeOrders, int n, const int* rowPtr,
                    const int* colIdx, const double* values, const double* b, double* x, double* out,
                    int* precondAfter, double* lastResidual)
{
    simall::gpu::GpuSolverConfig cfg;
    cfg.preconditioner = static_cast<simall::gpu::GpuPreconditioner>(precond);
    cfg.tolerance = tol;
    cfg.maxIterations = maxIt;
    cfg.relativeOrders = relativeOrders;
    simall::gpu::CgGpu solver(cfg);
    simall::gpu::HostCsrView A;
    A.n = static_cast<std::size_t>(n);
    A.nnz = static_cast<std::size_t>(rowPtr[n]);
    A.rowPtr = rowPtr;
    A.colIdx = colIdx;
    A.values = values;
    solver.set_matrix(A);
    std::vector<double> bv(b, b + n), xv(x, x + n);
    const auto st = solver.solve(bv, xv);
    std::copy(xv.begin(), xv.end(), x);
    out[0] = st.iterations;
    out[1] = st.finalResidual;
    out[2] = st.initialResidual;
    out[3] = st.converged ? 1.0 : 0.0;
    *precondAfter = static_cast<int>(solver.config().preconditioner);
    *lastResidual = solver.last_residual();
    return 0;
}

// ------------------------------------------------------------------ plugin ABI
// Loads a plugin library with the reference's PluginLoader (dlopen, ABI
// check, CreatePlugin, on_load, PluginRegistry::register_auto).  Returns the
// loader cookie (0 on failure); name/version/category describe what the
// registry now holds for it (category -1 if it is in no bucket).
std::int64_t ref_plugin_load(const char *path, char *name, int nameLen, char *version, int versionLen,
                             int *category)
{
    static simall::core::PluginLoader loader;  // keeps the plugin loaded
    const std::size_t cookie = loader.load(path);
    *category = -1;
    if (!cookie)
        return 0;
    auto &reg = simall::core::PluginRegistry::instance();
    for (int c = 0; c < static_cast<int>(simall::plugins::PluginCategory::_Count); ++c)
        for (auto *p : reg.by_category(static_cast<simall::plugins::PluginCategory>(c))) {
            const std::string nm = p->name(), vs = p->version();
            std::snprintf(name, static_cast<std::size_t>(nameLen), "%s", nm.c_str());
            std::snprintf(version, static_cast<std::size_t>(versionLen), "%s", vs.c_str());
            *category = c;
        }
    return static_cast<std::int64_t>(cookie);
}

} // extern "C"
