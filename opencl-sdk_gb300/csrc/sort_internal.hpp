// Layouts shared by the radix-sort kernels and the host code that allocates
// their control blocks and the context's look-back ring.
#pragma once

#include <cstddef>
#include <cstdint>
#include <string>

namespace gbc {
namespace onesweep {

constexpr int RADIX = 256;  // 8-bit digits

// The look-back status ring holds RING_TILES tiles x 256 digits of 64-bit
// status words (16 MiB): far more tiles than can be resident at once (152 SMs
// x a few CTAs), so a slot is never reused while a successor may still read
// it. Every tile of every pass takes the next sequence number of the context,
// and a word is valid only if its tag matches that sequence number, so the
// ring never needs clearing between sorts.
constexpr int RING_TILES = 8192;
constexpr std::size_t RING_BYTES = (std::size_t)RING_TILES * RADIX * sizeof(uint64_t);

//! Which digit positions are sorted, in order, and where each bin starts.
struct PassPlan {
    uint32_t num_active;
    uint32_t shift[8];
    uint32_t pad[7];
    uint32_t bin_start[8][RADIX];
};

//! Per-call control block (zeroed before each sort).
struct SortControl {
    uint32_t hist[8][RADIX];
    uint32_t tile_ctr[8];
    uint32_t done;
    uint32_t pad[7];
    PassPlan plan;
};

}  // namespace onesweep

int sort_variant_count(int key_bytes, bool has_values);
//! The variant used when the tuning table has no entry for the workload.
int sort_default_variant(int key_bytes, bool has_values, std::size_t n);
std::string sort_tuning_key(int key_bytes, bool has_values, std::size_t n);

}  // namespace gbc
