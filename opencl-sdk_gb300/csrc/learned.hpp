// Learned-CDF sort: options, statistics and entry points.
#pragma once

#include <cstddef>
#include <cstdint>

#include "runtime.hpp"

namespace gbc {
namespace learned {
constexpr int H = 32;                      // hidden width: 1 -> H -> H -> 1
constexpr int NPARAM = 4 * H + H * H + 1;  // v1, b1, v2, b2, v3, b3 (weights are exp(v))
}  // namespace learned

struct learned_options {
    int sample = 0;     // sampled keys (0: 2^20)
    int points = 0;     // training points taken from the sorted sample (0: 8192)
    int buckets = 0;    // partition buckets (0: from n, up to what shared memory holds)
    int steps = -1;     // Adam steps (-1: none; the data-driven initial network is used as fitted)
    float lr = 0.f;     // Adam learning rate (0: 0.01)
    bool use_model = true;  // false: equal-width buckets over the sampled key range (no network)
    const float* params_in = nullptr;       // host: start from these parameters instead of the data-driven init
    float* params_out = nullptr;            // host: receives the fitted parameters
    const uint32_t* splitters_in = nullptr; // host: replaces the compiled splitters (buckets - 1 values)
    int refine = -1;    // second level: 1/refine of the buckets split the root buckets the sample predicts
                        // oversized, at sample quantiles (-1: 3; 0: off)
};

struct learned_stats {
    uint32_t buckets = 0;
    uint32_t nonempty_buckets = 0;
    uint32_t largest_bucket = 0;
    uint32_t oversized_buckets = 0;  // larger than one CTA's shared-memory sort
    uint32_t oversized_keys = 0;
    uint32_t constant_keys = 0;      // keys in oversized buckets that hold one key value
    uint32_t estimated_oversized_keys = 0;  // predicted from the sample before the partition
    uint32_t violation = 0;          // bucket order was not monotone
    uint32_t fallback = 0;           // the plain radix sort produced the output
    float first_loss = 0.f, last_loss = 0.f;
    uint32_t refined_splitters = 0;  // splitters the second level added
};

//! Out-of-place sort of 32-bit keys (kind 0 unsigned, 1 signed, 2 float) by a
//! learned CDF partition; output identical to radix_sort's. Synchronises
//! twice: after the splitters (a model that would leave more than half of the
//! keys in oversized buckets sends the input to the plain radix sort) and at
//! the end (statistics, boundary check).
void learned_sort(device_context& ctx, const void* keys_in, void* keys_out, int key_kind, std::size_t n,
                  const learned_options& opt, learned_stats* stats_host);

//! The same for key-value pairs, stable: 32-bit keys (kind 0, 1, 2) or 64-bit
//! keys (kind 0 unsigned, 1 signed) with 32-bit values; output identical to
//! radix_sort's. 64-bit keys are bucketed through a monotone 32-bit
//! projection fitted to the sample's range; the partition keeps the input
//! order inside every bucket (the bucket numbers are sorted stably with the
//! keys' indices, and keys and values gathered in that order), and the
//! buckets are finished by the stable segmented sort.
void learned_sort_pairs(device_context& ctx, const void* keys_in, void* keys_out, int key_bytes, int key_kind,
                        const uint32_t* vals_in, uint32_t* vals_out, std::size_t n, const learned_options& opt,
                        learned_stats* stats_host);

//! One forward/backward pass of the network over m points on the GPU:
//! gradient of the mean squared error with respect to the raw parameters.
//! Points are keys in the order-preserving 32-bit domain; the network's first
//! layer sees (key - centre[j]) * inv_span.
void mlp_gradients(device_context& ctx, const float* params_host, const uint32_t* centres_host, float inv_span,
                   const uint32_t* keys_host, const float* ys_host, std::size_t m, float* grad_host,
                   float* loss_host);

}  // namespace gbc
