// copy_if (stream compaction) with a predicate compiled from an OpenCL C
// expression over x (the subset transform compiles, see expr.hpp).
#pragma once

#include <cstddef>
#include <cstdint>

#include "expr.hpp"
#include "runtime.hpp"

namespace gbc {

//! Stable compaction of the elements of in (type t) for which the predicate
//! program (xp::compile_predicate) gives 1; returns the count. Blocks.
std::size_t copy_if(device_context& ctx, const void* in, void* out, std::size_t n, elem t, const xp::program& p);

}  // namespace gbc
