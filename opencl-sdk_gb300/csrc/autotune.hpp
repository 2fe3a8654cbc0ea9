// Autotuner: times the compiled launch shapes of a sort family on the
// caller's data and stores the fastest in the context's tuning table under
// the workload's key (element type, size class and, for the segmented sort,
// the class of the average segment length).
#pragma once

#include <string>
#include <vector>

#include "runtime.hpp"

namespace gbc {

struct autotune_result {
    std::string key;          // tuning-table key the choice was stored under
    int best = -1;            // chosen variant (plain sort) or CTA capacity (segmented)
    double best_ms = 0;       // its mean time per call
    std::vector<int> candidates;
    std::vector<double> ms;   // mean time per call of every candidate
    double persistent_ms = 0;  // segmented: the fastest one-launch form's time
};

//! Plain radix sort: every compiled digit-pass variant (tile shape, CTAs per
//! SM, look-back window, staging); keys_in must differ from keys_out. The
//! default (the variant used without a table entry) is kept unless another
//! variant is more than 2% faster on the caller's keys.
autotune_result autotune_sort(device_context& ctx, const void* keys_in, void* keys_out, int key_bytes, int key_kind,
                              const uint32_t* vals_in, uint32_t* vals_out, std::size_t n, int repetitions);

//! Segmented sort, in four stages on the caller's batch: the capacity of the
//! one-CTA size class (segments up to that length are sorted in one CTA's
//! shared memory, longer ones by the batched onesweep), the MSD route's
//! bucket capacity, the one-CTA sorts' thread count (256 or 512), and the
//! launch form (the launch sequence or one persistent launch); each is
//! stored under its own key. keys_in must differ from keys_out.
autotune_result autotune_segmented_sort(device_context& ctx, const void* keys_in, void* keys_out, int key_bytes,
                                        int key_kind, const uint32_t* vals_in, uint32_t* vals_out, std::size_t n,
                                        const uint32_t* offsets, std::size_t num_segments, int repetitions);

}  // namespace gbc
