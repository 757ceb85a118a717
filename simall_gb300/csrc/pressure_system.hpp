// The device pressure-correction system (assemble.cu) and the field loops
// around its solve (fields.cu): mesh-derived arrays on the device.
#pragma once

#include "internal.hpp"

#include <vector>

struct simall_pressure_system {
    simall_context *ctx = nullptr;
    int64_t nC = 0, nF = 0, nnz = 0;
    std::vector<int32_t> h_rowPtr, h_colIdx;
    simall::DevBuf<int32_t> rowPtr, colIdx;
    simall::DevBuf<double> values, rhs;
    // faces
    simall::DevBuf<int32_t> owner, neighbor;  // neighbor -1 on boundary faces
    simall::DevBuf<double> amag2, ddotA;
    simall::DevBuf<uint8_t> kind;  // 0 interior, 1 pressure boundary, 2 other boundary, 3 periodic
    // periodic faces (SimpleAlgorithm::build_periodic_pairs): the twin face of
    // each boundary face (-1: none), and per face the cell a flux averages
    // with (the neighbour, the twin face's owner, or -1)
    std::vector<int32_t> h_twin;
    simall::DevBuf<int32_t> fpartner;
    bool periodic = false;
    simall::DevBuf<double> coef;
    // cells: faces in ascending id; entry = face id | (cell is the neighbour) << 31;
    // slot = CSR position of the other cell in the row (-1: none)
    simall::DevBuf<int32_t> cfOff, cfEnt, cfSlot, diagSlot;
    int anyDirichlet = 0;
    simall::DevBuf<double> aP, phi;  // staging for host inputs
    simall::DevBuf<double> den;      // SIMPLEC denominators
    simall::DevBuf<double> kf, pbf;  // staging for face-conductance inputs
    // boundary specs given at creation (zone, BCType ordinal), in order: find_bc takes the first
    std::vector<simall_boundary> h_bcs;
    // field loops (simall_pressure_system_setup_field_loops)
    bool fieldsReady = false;
    simall::DevBuf<double> ax, ay, az;          // face areas
    simall::DevBuf<double> gdx, gdy, gdz, gw2;  // least-squares vectors d (cell to neighbour or face), 1/(|d|^2+1e-30)
    simall::DevBuf<double> minv;                // [6][nC] inverse normal matrices (xx xy xz yy yz zz)
    simall::DevBuf<double> vol;                 // cell volumes
    simall::DevBuf<uint8_t> fkind;              // face velocity: 0 interior, 1 zone vector, 2 zero, 3 owner's
    simall::DevBuf<int32_t> fvslot;             // zone-vector slot of the fkind 1 faces
    simall::DevBuf<double> zvec;                // [3][slots] zone velocity vectors
    int nslots = 0;
    simall::DevBuf<double> grad;                // [3][nC] scratch gradient
    simall::DevBuf<double> stage;               // staging for host field arrays
    // momentum assembly (momentum.cu)
    simall::DevBuf<uint8_t> mkind;              // face: kMom* below
    simall::DevBuf<double> momD;                // mu |A|^2 / max(|d.A|, 1e-30) per face, for mu == momMu
    double momMu = 0.0;                         // NaN until the first assembly
    simall::DevBuf<double> mvalues, mrhs, maP;  // values[nnz] (shared pattern), rhs[3][nC], relaxed diagonal
    bool momReady = false;
};

namespace simall {
// Momentum face kinds: interior; VelocityInlet / MovingWall (the zone's vector);
// NoSlipWall / Wall (zero); Symmetry (no contribution); any other boundary
// (upwind outflow).
constexpr uint8_t kMomInterior = 0, kMomZoneVector = 1, kMomWall = 2, kMomSymmetry = 3, kMomOther = 4,
                  kMomPeriodic = 5;
// Pressure-system face kinds (assemble.cu).
constexpr uint8_t kInterior = 0, kPressure = 1, kOtherBoundary = 2, kPeriodic = 3;
// Least-squares gradient of f (device, n_cells) into g[3][n_cells] (fields.cu).
int ps_gradient(simall_pressure_system *ps, const double *f, double *g);
}  // namespace simall

