// lie_tables.hpp -- host construction of the Hall basis and of the sparse
// tensor <-> Lie conversion matrices (internal header).
#pragma once

#include <cstdint>
#include <vector>

namespace rpp_gb {

struct HallTables {
    int32_t width = 0;
    int32_t depth = 0;
    std::vector<int64_t> degree_begin;  // depth + 2
    std::vector<int64_t> pairs;         // 2 * true_size: (left, right) per key
    int64_t true_size() const { return degree_begin.empty() ? 0 : degree_begin.back(); }
};

struct CscMatrix {
    int64_t outer_dim = 0;
    int64_t inner_dim = 0;
    std::vector<int64_t> offsets;
    std::vector<int64_t> indices;
    std::vector<double> values;
};

HallTables build_hall_basis(int32_t width, int32_t depth);
// which = 0: tensor -> Lie (t2l), which = 1: Lie -> tensor (l2t).
CscMatrix build_conversion_matrix(const HallTables& hall, int which);

}  // namespace rpp_gb
