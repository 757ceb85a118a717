// The AMG preconditioner's hierarchy (amg_host.cpp builds it on the host,
// amg.cu holds it on the device and runs the V-cycle).
#pragma once

#include <cstdint>
#include <vector>

namespace simall {

struct AmgCsr {
    int32_t n = 0;
    std::vector<int32_t> rp, ci;
    std::vector<double> v;
};

// AMGPreconditioner::setup (src/solver/AMGPreconditioner.cpp:249-323) with
// make_preconditioner's parameters (AMGPreconditioner.hpp:39-43).
struct AmgParams {
    double theta = 0.25;
    int maxLevels = 10;
    int preSweeps = 1, postSweeps = 1;
    int coarseThreshold = 32;
};

struct AmgHierarchy {
    // A[0] is the input operator; P[l], R[l] connect level l to l + 1
    std::vector<AmgCsr> A, P, R;
    int32_t coarseN = 0;
    std::vector<double> lu;  // dense [coarseN][coarseN] factor of the coarsest A
};

// Builds the hierarchy of A = (rp, ci, v) (n rows).  Bit-identical to the
// reference's setup: the same strong couplings, C/F split, interpolation
// weights, Galerkin products (accumulation order included) and dense LU.
void amg_build_hierarchy(int32_t n, const int32_t *rp, const int32_t *ci, const double *v, const AmgParams &prm,
                         AmgHierarchy &h);

}  // namespace simall
