// The device-resident field registry (registry.cu) shared by the checkpoint
// reader/writer (checkpoint.cu) and the SIMPLE iteration (simple.cu).
#pragma once

#include "internal.hpp"

#include <string>
#include <vector>

struct simall_fields {
    struct Field {
        std::string name;
        int64_t n = 0;
        simall::DevBuf<double> data;  // scalar: [n]; vector: [3][n] (x, y, z back to back)
    };
    simall_context *ctx = nullptr;
    // insertion order: a checkpoint written from a registry that was read from
    // a checkpoint keeps the file's field order
    std::vector<Field *> scalars, vectors;
    ~simall_fields()
    {
        for (auto *f : scalars)
            delete f;
        for (auto *f : vectors)
            delete f;
    }
};

namespace simall {
// FieldRegistry::scalar / vector: the field, created or re-created zeroed when
// its size differs from n.  nullptr on allocation failure (status in *st).
simall_fields::Field *registry_get(simall_fields *r, const char *name, int64_t n, bool vector, int *st);
simall_fields::Field *registry_find(simall_fields *r, const char *name, bool vector);
}  // namespace simall
