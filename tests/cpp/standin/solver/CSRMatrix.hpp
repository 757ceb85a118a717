// Test stand-in for simall::solver::CSRMatrix (same member names and types).
#pragma once
#include "utilities/AlignedAllocator.hpp"
#include <cstddef>
namespace simall::solver {
struct CSRMatrix {
    util::aligned_vector<int> rowPtr;
    util::aligned_vector<int> colIdx;
    util::aligned_vector<double> values;
    std::size_t rows() const noexcept { return rowPtr.empty() ? 0 : rowPtr.size() - 1; }
};
}  // namespace simall::solver
