// copy_if (stream compaction) with a predicate from a fixed grammar.
#pragma once

#include <cstddef>
#include <cstdint>
#include <string>

#include "runtime.hpp"

namespace gbc {

// One comparison: lhs cmp constant, lhs one of x, (x % m), (x & m). The
// arithmetic follows OpenCL C's usual conversions of the element type and
// the literals' types (int, unsigned int, long, unsigned long, float, double).
struct pred_clause {
    int lhs = 0;       // 0: x, 1: x % m, 2: x & m
    int cmp = 0;       // 0: <, 1: <=, 2: >, 3: >=, 4: ==, 5: !=
    int ctype = 0;     // common type: 0 int32, 1 uint32, 2 int64, 3 uint64, 4 float, 5 double
    int64_t m_i = 0, c_i = 0;
    double m_f = 0, c_f = 0;
};

struct predicate {
    int count = 0;     // clauses (1..4)
    int join = 0;      // 0: all (&&), 1: any (||)
    pred_clause c[4];
};

//! Parses "x > 0", "(x % 3u) == 0u", "x >= 10 && x < 20", ... for elements of
//! type t; throws unsupported_error for anything outside the grammar.
predicate parse_predicate(const std::string& text, elem t);

//! Stable compaction of the elements satisfying p; returns the count (blocks).
std::size_t copy_if(device_context& ctx, const void* in, void* out, std::size_t n, elem t, const predicate& p);

}  // namespace gbc
