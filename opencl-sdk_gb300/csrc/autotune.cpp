// Autotuner (see autotune.hpp). Candidates run back to back on the context's
// stream; each is warmed up once, then timed over `repetitions` calls with
// CUDA events on that stream.
#include "autotune.hpp"

#include <algorithm>
#include <stdexcept>
#include <vector>

#include "segmented.hpp"
#include "sort_internal.hpp"

namespace gbc {
namespace {

class event_pair {
public:
    event_pair()
    {
        check_cuda(cudaEventCreate(&a_), "cudaEventCreate");
        check_cuda(cudaEventCreate(&b_), "cudaEventCreate");
    }
    ~event_pair()
    {
        cudaEventDestroy(a_);
        cudaEventDestroy(b_);
    }
    template <typename F> double time(device_context& ctx, int reps, F&& f)
    {
        f();  // warm-up (first-use allocations, kernel attributes)
        check_cuda(cudaEventRecord(a_, ctx.stream), "cudaEventRecord");
        for (int i = 0; i < reps; ++i) f();
        check_cuda(cudaEventRecord(b_, ctx.stream), "cudaEventRecord");
        check_cuda(cudaEventSynchronize(b_), "cudaEventSynchronize");
        float ms = 0.f;
        check_cuda(cudaEventElapsedTime(&ms, a_, b_), "cudaEventElapsedTime");
        const int err = ctx.take_device_error();
        if (err != 0) throw device_error("autotune: a candidate reported a device error", err);
        return (double)ms / reps;
    }

private:
    cudaEvent_t a_ = nullptr, b_ = nullptr;
};

void check_args(const void* in, const void* out, int reps)
{
    if (in == nullptr || out == nullptr) throw std::invalid_argument("autotune: null keys");
    if (in == out) throw std::invalid_argument("autotune: keys_in and keys_out must differ");
    if (reps < 1 || reps > 1000) throw std::invalid_argument("autotune: repetitions must be in [1, 1000]");
}

// The fastest candidate; with margin > 0, candidate keep (the built-in
// default) unless the fastest beats it by more than that fraction.
void pick(autotune_result& r, device_context& ctx, double margin = 0.0, std::size_t keep = 0)
{
    const auto it = std::min_element(r.ms.begin(), r.ms.end());
    r.best = r.candidates[it - r.ms.begin()];
    r.best_ms = *it;
    if (margin > 0.0 && keep < r.ms.size() && *it >= r.ms[keep] * (1.0 - margin)) {
        r.best = r.candidates[keep];
        r.best_ms = r.ms[keep];
    }
    launch_shape s;
    s.variant = r.best;
    ctx.tuning.store(r.key, s);
}

}  // namespace

autotune_result autotune_sort(device_context& ctx, const void* keys_in, void* keys_out, int key_bytes, int key_kind,
                              const uint32_t* vals_in, uint32_t* vals_out, std::size_t n, int repetitions)
{
    check_args(keys_in, keys_out, repetitions);
    if (key_bytes != 4 && key_bytes != 8) throw std::invalid_argument("autotune: keys must be 32 or 64 bits");
    ctx.activate();
    const bool kv = vals_in != nullptr;
    autotune_result r;
    r.key = sort_tuning_key(key_bytes, kv, n);
    launch_shape before;
    const bool had = ctx.tuning.lookup(r.key, before);
    event_pair ev;
    try {
        for (int v = 0; v < sort_variant_count(key_bytes, kv); ++v) {
            launch_shape s;
            s.variant = v;
            ctx.tuning.store(r.key, s);
            r.candidates.push_back(v);
            r.ms.push_back(ev.time(ctx, repetitions, [&] {
                radix_sort(ctx, keys_in, keys_out, key_bytes, key_kind, vals_in, vals_out, n, false);
            }));
        }
    } catch (...) {
        if (had) ctx.tuning.store(r.key, before);
        throw;
    }
    // The entry serves every key distribution of this size class, and the
    // caller's keys are one of them. The defaults hold up on skewed keys
    // (half-warp count arrays one bank apart); PAD 0 is 0.5-1.3% faster on
    // uniform 2^28 keys but 25-28% slower when the keys are the AND of 4
    // uniform words. So a variant replaces the default only when it is more
    // than 2% faster on the caller's keys.
    pick(r, ctx, 0.02, (std::size_t)sort_default_variant(key_bytes, kv, n));
    return r;
}

autotune_result autotune_segmented_sort(device_context& ctx, const void* keys_in, void* keys_out, int key_bytes,
                                        int key_kind, const uint32_t* vals_in, uint32_t* vals_out, std::size_t n,
                                        const uint32_t* offsets, std::size_t num_segments, int repetitions)
{
    check_args(keys_in, keys_out, repetitions);
    if (key_bytes != 4 && key_bytes != 8) throw std::invalid_argument("autotune: keys must be 32 or 64 bits");
    ctx.activate();
    const bool kv = vals_in != nullptr;
    autotune_result r;
    r.key = segsort_tuning_key(key_bytes, kv, n, num_segments);
    // The one-CTA class's capacity: from a quarter of the shared-memory
    // maximum up to the maximum, in steps of 1024 keys.
    const int cap = (int)segsort_cta_cap(key_bytes, kv);
    for (int c = std::max(1024, cap / 4 / 1024 * 1024); c < cap; c += std::max(1024, cap / 4 / 1024 * 1024))
        r.candidates.push_back(c);
    r.candidates.push_back(cap);
    event_pair ev;
    for (int c : r.candidates) {
        seg_options o;
        o.cta_cap = c;
        o.msd_cap = 0;
        o.persistent = 0;
        o.cta_threads = 256;
        r.ms.push_back(ev.time(ctx, repetitions, [&] {
            segmented_sort(ctx, keys_in, keys_out, key_bytes, key_kind, vals_in, vals_out, n, offsets, num_segments,
                           false, o);
        }));
    }
    pick(r, ctx);
    // Then, with that capacity, the MSD route's bucket capacity (0: off),
    // stored under its own key.
    autotune_result m;
    m.key = segsort_msd_tuning_key(key_bytes, kv, n, num_segments);
    m.candidates.push_back(0);
    for (int c = 2048; c < cap; c += 1024) m.candidates.push_back(c);
    m.candidates.push_back(cap);
    for (int c : m.candidates) {
        seg_options o;
        o.cta_cap = r.best;
        o.msd_cap = c;
        o.persistent = 0;
        o.cta_threads = 256;
        m.ms.push_back(ev.time(ctx, repetitions, [&] {
            segmented_sort(ctx, keys_in, keys_out, key_bytes, key_kind, vals_in, vals_out, n, offsets, num_segments,
                           false, o);
        }));
    }
    pick(m, ctx);
    // Then the one-CTA sorts' thread count at those capacities: 256, or 512
    // (twice the warps per CTA; it pays for segments near the capacity and
    // costs for batches of mostly short ones), stored under its own key.
    autotune_result t;
    t.key = segsort_threads_tuning_key(key_bytes, kv, n, num_segments);
    for (int threads : {256, 512}) {
        seg_options o;
        o.cta_cap = r.best;
        o.msd_cap = m.best;
        o.persistent = 0;
        o.cta_threads = threads;
        t.candidates.push_back(threads);
        t.ms.push_back(ev.time(ctx, repetitions, [&] {
            segmented_sort(ctx, keys_in, keys_out, key_bytes, key_kind, vals_in, vals_out, n, offsets, num_segments,
                           false, o);
        }));
    }
    pick(t, ctx);
    // Last, the launch form: the launch sequence at that capacity against the
    // one persistent launch (every CTA on both paths, or 1/8 .. 3/8 of them
    // on the small and medium segments), at capacities whose shared memory
    // leaves two CTAs per SM; the winner's capacity replaces the first pick.
    struct form {
        int persistent, cap;
    };
    std::vector<form> forms{{0, r.best}};
    std::vector<double> times{std::min({r.best_ms, m.best_ms, t.best_ms})};
    for (int mode = 1; mode <= 4; ++mode)
        for (int c : {1024, 2048}) forms.push_back({mode, std::min(c, cap)});
    for (std::size_t f = 1; f < forms.size(); ++f) {
        seg_options o;
        o.cta_cap = forms[f].cap;
        o.msd_cap = m.best;
        o.persistent = forms[f].persistent;
        o.cta_threads = 256;  // the persistent kernel's CTAs have 256 threads
        times.push_back(ev.time(ctx, repetitions, [&] {
            segmented_sort(ctx, keys_in, keys_out, key_bytes, key_kind, vals_in, vals_out, n, offsets, num_segments,
                           false, o);
        }));
    }
    const std::size_t best = std::min_element(times.begin(), times.end()) - times.begin();
    launch_shape sh;
    sh.variant = forms[best].persistent;
    ctx.tuning.store(segsort_batch_tuning_key(key_bytes, kv, n, num_segments), sh);
    sh.variant = forms[best].cap;
    ctx.tuning.store(r.key, sh);
    r.best = forms[best].cap;
    r.best_ms = times[best];
    r.persistent_ms = *std::min_element(times.begin() + 1, times.end());
    return r;
}

}  // namespace gbc
