// Test stand-in for SimAll's util::aligned_vector, so that the header-only
// adapter (include/simall_gpu_solver.hpp) can be compiled and run where the
// SimAll tree is not available.  Only the names the adapter uses.
#pragma once
#include <vector>
namespace simall::util {
template <class T> using aligned_vector = std::vector<T>;
}
