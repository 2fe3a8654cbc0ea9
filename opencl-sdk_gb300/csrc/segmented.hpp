// Batched (segmented) sort and scan: entry points and tunables.
#pragma once

#include <cstddef>
#include <cstdint>

#include "runtime.hpp"

namespace gbc {

//! Launch-shape choices of the segmented sort (picked by the autotuner).
struct seg_options {
    int cta_cap = 0;  // largest segment a single CTA sorts in shared memory (0: the type's maximum)
    // device, one byte per segment or null: nonzero marks a segment already in
    // order (every key equal), left untouched; only for in-place calls
    const uint8_t* skip = nullptr;
    // MSD route: a large segment whose highest varying digit splits it into
    // buckets of at most msd_cap keys takes one pass on that digit, then the
    // shared-memory sorts finish the buckets; 0: every large segment takes
    // all digit passes; -1: the default (the tuning table's entry, else off)
    int msd_cap = -1;
    // 0: a launch per phase, the small/medium and large paths on two
    // streams; 1: the whole batch in one persistent (cooperative) launch with
    // grid barriers between its phases; 2..7: the same with (persistent - 1)
    // eighths of its CTAs sorting the small and medium segments while the
    // others take the large ones; -1: the tuning table's entry, else 0
    int persistent = -1;
    // threads of each one-CTA segment sort: 256, or 512 (where the shared
    // memory of the CTA's capacity fits, else 256), which doubles the warps
    // in flight. 0: the tuning table's entry for this workload (the
    // segmented key with ":threads", stored by the autotuner), else its
    // "segsort:cta_threads" entry, else 256.
    // 512 pays for segments near the capacity (the learned sort's buckets:
    // 2.50 -> 1.92 ms at 2^28 keys) and costs for batches of mostly short
    // ones (200,000 lognormal segments of median 256: 24.7 -> 25.7 ms).
    int cta_threads = 0;
};

//! Sorts every segment [offsets[i], offsets[i+1]) independently and stably.
//! offsets has num_segments + 1 monotone entries (device memory); keys_in ==
//! keys_out sorts in place. Asynchronous; graph-capturable once the pool is
//! warm (every temporary then comes from the cache).
void segmented_sort(device_context& ctx, const void* keys_in, void* keys_out, int key_bytes, int key_kind,
                    const uint32_t* vals_in, uint32_t* vals_out, std::size_t n, const uint32_t* offsets,
                    std::size_t num_segments, bool descending, const seg_options& opt);

//! Scan restarted at every segment start (offsets as for segmented_sort;
//! position 0 always starts a segment). Exclusive: a segment's first output
//! is the identity.
void segmented_scan(device_context& ctx, const void* in, void* out, std::size_t n, elem t, op_kind op,
                    const void* identity, bool exclusive, const uint32_t* offsets, std::size_t num_segments);

std::string segsort_tuning_key(int key_bytes, bool has_values, std::size_t n, std::size_t num_segments);
//! The tuning-table key of the batch's launch form (seg_options::persistent).
std::string segsort_batch_tuning_key(int key_bytes, bool has_values, std::size_t n, std::size_t num_segments);
//! The tuning-table key of the one-CTA sorts' thread count (256 or 512; one
//! entry for every segmented sort of the context).
std::string segsort_cta_threads_tuning_key();
//! The tuning-table key of the one-CTA sorts' thread count for one workload
//! class (the segmented key with ":threads").
std::string segsort_threads_tuning_key(int key_bytes, bool has_values, std::size_t n, std::size_t num_segments);
//! The tuning-table key of the MSD route's bucket capacity (0: off).
std::string segsort_msd_tuning_key(int key_bytes, bool has_values, std::size_t n, std::size_t num_segments);

//! Largest segment the segmented sort finishes in one CTA's shared memory.
uint32_t segsort_cta_cap(int key_bytes, bool has_values);

}  // namespace gbc
