// reduce_by_key over sorted keys, fused with a histogram of the low 16 key
// bits: one single-pass decoupled look-back kernel.
//
// No reference counterpart (the reference has no reduce_by_key and no 64-bit
// keys; the pipeline sort -> reduce_by_key -> histogram is the benchmark's).
// For runs of equal keys (keys sorted, or grouped) it writes, in run order,
// the run's key, the sum of its uint32 values as uint64, and the run length;
// the histogram bin (key & 0xFFFF) of every key gets +1, added once per run as
// the run length.
//
// Each element contributes a state (h, s, c, p): h = it starts a run, s = the
// sum since the latest run start, c = the number of run starts, p = the
// position of the latest start. States combine in sequence order:
//   A (+) B = (A.h | B.h, B.h ? B.s : A.s + B.s, A.c + B.c, B.h ? B.p : A.p),
// which is associative; tiles publish their aggregate and inclusive states and
// look back like the scan. The tile holding a run's last element knows the
// run's index (c - 1), sum, start and hence length, and writes the run.
#include <cstring>
#include <string>
#include <type_traits>

#include "device_common.cuh"
#include "runtime.hpp"
#include "sort_internal.hpp"

namespace gbc {
namespace {

using dev::FULL_MASK;
constexpr int ITEMS = 16;
constexpr int LB_PER_LANE = 4;  // look-back window: 32 x 4 tiles per round trip
constexpr uint64_t FLAG_AGG = 1, FLAG_PRE = 2;
constexpr uint64_t TAG_MASK = (1ull << 29) - 1;
constexpr uint64_t HEAD_BIT = 1ull << 61;
constexpr uint64_t SLOTS = onesweep::RING_BYTES / 64;  // 8 words per tile

struct State {
    uint32_t h;  // 0/1
    uint64_t s;
    uint32_t c;
    uint32_t p;
};

__device__ __forceinline__ State combine(const State& a, const State& b)
{
    State r;
    r.h = a.h | b.h;
    r.s = b.h ? b.s : a.s + b.s;
    r.c = a.c + b.c;
    r.p = b.h ? b.p : a.p;
    return r;
}

__device__ __forceinline__ State shfl_up(const State& x, int d)
{
    State y;
    y.h = __shfl_up_sync(FULL_MASK, x.h, d);
    y.s = __shfl_up_sync(FULL_MASK, x.s, d);
    y.c = __shfl_up_sync(FULL_MASK, x.c, d);
    y.p = __shfl_up_sync(FULL_MASK, x.p, d);
    return y;
}
__device__ __forceinline__ State shfl(const State& x, int src)
{
    State y;
    y.h = __shfl_sync(FULL_MASK, x.h, src);
    y.s = __shfl_sync(FULL_MASK, x.s, src);
    y.c = __shfl_sync(FULL_MASK, x.c, src);
    y.p = __shfl_sync(FULL_MASK, x.p, src);
    return y;
}

__device__ __forceinline__ State warp_incl(State x)
{
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const State y = shfl_up(x, o);
        if (lane >= o) x = combine(y, x);
    }
    return x;
}

__device__ void publish(uint64_t* ring, uint64_t seq, uint64_t flag, const State& v)
{
    uint64_t* s = ring + (seq & (SLOTS - 1)) * 8;
    const int o = flag == FLAG_PRE ? 2 : 0;
    dev::st_relaxed(&s[o], v.s);
    dev::st_relaxed(&s[o + 1], (uint64_t)v.c | ((uint64_t)v.p << 32));
    dev::st_release(&s[4], (flag << 62) | (v.h ? HEAD_BIT : 0) | ((seq & TAG_MASK) << 32));
}

__device__ bool read(const uint64_t* ring, uint64_t seq, uint64_t& flag, State& v)
{
    const uint64_t* s = ring + (seq & (SLOTS - 1)) * 8;
    const uint64_t w = dev::ld_acquire(&s[4]);
    flag = w >> 62;
    if (flag == 0 || ((w >> 32) & TAG_MASK) != (seq & TAG_MASK)) return false;
    const int o = flag == FLAG_PRE ? 2 : 0;
    v.h = (w & HEAD_BIT) ? 1u : 0u;
    v.s = dev::ld_relaxed(&s[o]);
    const uint64_t cp = dev::ld_relaxed(&s[o + 1]);
    v.c = (uint32_t)cp;
    v.p = (uint32_t)(cp >> 32);
    return true;
}

template <typename K> struct RbkArgs {
    const K* keys;
    const uint32_t* vals;
    uint32_t n;
    K* keys_out;
    unsigned long long* sums_out;
    uint32_t* counts_out;   // may be null
    uint32_t* hist;         // 65536 bins or null
    uint32_t* num_runs;     // device, written by the last tile
    uint32_t num_tiles;
    uint64_t* ring;
    uint64_t seq0;
    uint32_t* tile_ctr;
    int* err;
};

// THREADS: 256, 128 or 64 per CTA. Every CTA's warps wait at a barrier while
// its first warp looks back, so smaller CTAs (more of them per SM, each with
// its own look-back in flight) keep more warps busy; registers cap any shape
// at 16 warps per SM.
template <typename K, int THREADS> __global__ void __launch_bounds__(THREADS) k_reduce_by_key(RbkArgs<K> a)
{
    constexpr int TILE = THREADS * ITEMS;
    __shared__ State s_warp[THREADS / 32];
    __shared__ State s_prefix;
    __shared__ uint32_t s_tile;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const bool aligned = ((reinterpret_cast<uintptr_t>(a.keys) | reinterpret_cast<uintptr_t>(a.vals)) & 15) == 0;

    for (;;) {
        // The tile index is taken only when the CTA can start on it; the
        // tile a grid further on is prefetched into L2 (cf. the scan).
        if (tid == 0) {
            s_tile = atomicAdd(a.tile_ctr, 1u);
            const uint64_t ahead = (uint64_t)s_tile + gridDim.x;
            if (aligned && (ahead + 1) * TILE <= a.n) {
                dev::prefetch_l2(a.keys + ahead * TILE, TILE * sizeof(K));
                dev::prefetch_l2(a.vals + ahead * TILE, TILE * 4);
            }
        }
        __syncthreads();
        const uint32_t t = s_tile;
        if (t >= a.num_tiles) break;
        const uint32_t first = t * TILE + tid * ITEMS;  // blocked: this thread's items in order

        K key[ITEMS];
        uint32_t val[ITEMS];
        uint32_t head = 0, valid_mask = 0;
        if (aligned && first + ITEMS <= a.n) {
            // 128-bit loads of the thread's consecutive items
            const uint4* kp = reinterpret_cast<const uint4*>(a.keys + first);
#pragma unroll
            for (int j = 0; j < ITEMS * (int)sizeof(K) / 16; ++j) {
                const uint4 w = kp[j];
                memcpy(reinterpret_cast<unsigned char*>(key) + 16 * j, &w, 16);
            }
            const uint4* vp = reinterpret_cast<const uint4*>(a.vals + first);
#pragma unroll
            for (int j = 0; j < ITEMS / 4; ++j) {
                const uint4 w = vp[j];
                memcpy(&val[4 * j], &w, 16);
            }
            valid_mask = (ITEMS == 32) ? 0xFFFFFFFFu : ((1u << ITEMS) - 1);
        } else {
#pragma unroll
            for (int i = 0; i < ITEMS; ++i) {
                const uint32_t idx = first + i;
                if (idx < a.n) {
                    key[i] = a.keys[idx];
                    val[i] = a.vals[idx];
                    valid_mask |= 1u << i;
                } else {
                    key[i] = 0;
                    val[i] = 0;
                }
            }
        }
        const K before = (first > 0 && first - 1 < a.n) ? a.keys[first - 1] : K(0);
#pragma unroll
        for (int i = 0; i < ITEMS; ++i) {
            const uint32_t idx = first + i;
            const K prev = i == 0 ? before : key[i - 1];
            if (((valid_mask >> i) & 1) && (idx == 0 || key[i] != prev)) head |= 1u << i;
        }
        // thread state
        State st{0, 0, 0, 0};
#pragma unroll
        for (int i = 0; i < ITEMS; ++i) {
            if (!((valid_mask >> i) & 1)) continue;
            if ((head >> i) & 1) {
                st.h = 1;
                st.s = val[i];
                st.c += 1;
                st.p = first + i;
            } else {
                st.s += val[i];
            }
        }
        const State incl = warp_incl(st);
        if (lane == 31) s_warp[warp] = incl;
        __syncthreads();

        if (warp == 0) {
            // scan of the warp totals
            State w = lane < THREADS / 32 ? s_warp[lane] : State{0, 0, 0, 0};
            const State wi = warp_incl(w);
            const State wx = shfl_up(wi, 1);
            if (lane < THREADS / 32) s_warp[lane] = lane == 0 ? State{0, 0, 0, 0} : wx;
            const State agg = shfl(wi, THREADS / 32 - 1);
            const uint64_t my_seq = a.seq0 + t;
            if (lane == 0) publish(a.ring, my_seq, t == 0 ? FLAG_PRE : FLAG_AGG, agg);
            State excl{0, 0, 0, 0};
            if (t > 0) {
                // Look back over windows of 32 x LB_PER_LANE tiles (lane l
                // inspects LB_PER_LANE consecutive ones); the nearest tile with
                // an inclusive state ends the walk.
                bool have = false, gave_up = false;
                int64_t w_end = t;
                for (;;) {
                    uint64_t flag[LB_PER_LANE];
                    State v[LB_PER_LANE];
#pragma unroll
                    for (int q = 0; q < LB_PER_LANE; ++q) {
                        const int64_t k = w_end - 32 * LB_PER_LANE + lane * LB_PER_LANE + q;
                        flag[q] = FLAG_PRE;  // before tile 0: the empty state
                        v[q] = State{0, 0, 0, 0};
                        if (k >= 0 && !read(a.ring, a.seq0 + (uint64_t)k, flag[q], v[q])) {
                            const unsigned long long start = dev::globaltimer();
                            for (uint32_t spin = 1;; ++spin) {
                                if (read(a.ring, a.seq0 + (uint64_t)k, flag[q], v[q])) break;
                                if ((spin & 255) == 0 && dev::globaltimer() - start > dev::SPIN_LIMIT_NS) {
                                    gave_up = true;
                                    flag[q] = FLAG_PRE;
                                    v[q] = State{0, 0, 0, 0};
                                    break;
                                }
                                if (spin > 32) __nanosleep(64);
                            }
                        }
                    }
                    int hi = -1;
#pragma unroll
                    for (int q = 0; q < LB_PER_LANE; ++q)
                        if (flag[q] == FLAG_PRE) hi = q;
                    const uint32_t pre = __ballot_sync(FULL_MASK, hi >= 0);
                    const int L = pre ? 31 - __clz(pre) : -1;
                    State contrib{0, 0, 0, 0};
                    if (lane >= L) {
                        const int q0 = lane == L ? hi : 0;
#pragma unroll
                        for (int q = 0; q < LB_PER_LANE; ++q)
                            if (q >= q0) contrib = combine(contrib, v[q]);
                    }
                    const State ws = shfl(warp_incl(contrib), 31);
                    excl = have ? combine(ws, excl) : ws;
                    have = true;
                    if (pre) break;
                    w_end -= 32 * LB_PER_LANE;
                }
                if (__any_sync(FULL_MASK, gave_up) && lane == 0) dev::raise_error(a.err, dev::ERR_LOOKBACK_TIMEOUT);
                if (lane == 0) publish(a.ring, my_seq, FLAG_PRE, combine(excl, agg));
            }
            if (lane == 0) {
                s_prefix = excl;
                if (t == a.num_tiles - 1 && a.num_runs != nullptr) *a.num_runs = combine(excl, agg).c;
            }
        }
        __syncthreads();

        // Walk this thread's items with the running state; close runs.
        State run = combine(s_prefix, s_warp[warp]);
        const State lx = shfl_up(incl, 1);
        if (lane > 0) run = combine(run, lx);
        const K after = (first + ITEMS < a.n) ? a.keys[first + ITEMS] : K(0);
#pragma unroll
        for (int i = 0; i < ITEMS; ++i) {
            if (!((valid_mask >> i) & 1)) continue;
            const uint32_t idx = first + i;
            if ((head >> i) & 1) {
                run.h = 1;
                run.s = val[i];
                run.c += 1;
                run.p = idx;
            } else {
                run.s += val[i];
            }
            const K next = i + 1 < ITEMS ? key[i + 1] : after;
            const bool last = idx + 1 == a.n || ((i + 1 < ITEMS) ? ((valid_mask >> (i + 1)) & 1) == 0 || next != key[i]
                                                                   : next != key[i]);
            if (last && run.c > 0) {
                const uint32_t r = run.c - 1;
                const uint32_t len = idx - run.p + 1;
                a.keys_out[r] = key[i];
                a.sums_out[r] = run.s;
                if (a.counts_out) a.counts_out[r] = len;
                if (a.hist) atomicAdd(&a.hist[(uint32_t)key[i] & 0xFFFFu], len);
            }
        }
        __syncthreads();
    }
}

}  // namespace

void reduce_by_key(device_context& ctx, const void* keys, int key_bytes, const uint32_t* vals, std::size_t n,
                   void* keys_out, unsigned long long* sums_out, uint32_t* counts_out, uint32_t* hist,
                   uint32_t* num_runs_device)
{
    if (key_bytes != 4 && key_bytes != 8) throw std::invalid_argument("reduce_by_key: keys must be 32 or 64 bits");
    check_size(n);
    ctx.activate();
    if (hist != nullptr) check_cuda(cudaMemsetAsync(hist, 0, 65536 * 4, ctx.stream), "cudaMemsetAsync");
    if (n == 0) {
        if (num_runs_device) check_cuda(cudaMemsetAsync(num_runs_device, 0, 4, ctx.stream), "cudaMemsetAsync");
        return;
    }
    if (keys == nullptr || vals == nullptr || keys_out == nullptr || sums_out == nullptr)
        throw std::invalid_argument("reduce_by_key: null argument");
    // CTA size from the tuning table (variant 0: 256 threads, 1: 128, 2: 64)
    launch_shape shape;
    const std::string key = std::string("reduce_by_key:") + (key_bytes == 4 ? "u32" : "u64");
    const int threads = ctx.tuning.lookup(key, shape) ? (shape.variant == 1 ? 128 : shape.variant == 2 ? 64 : 256)
                                                      : 128;
    const uint32_t num_tiles = (uint32_t)((n + (std::size_t)threads * ITEMS - 1) / ((std::size_t)threads * ITEMS));
    unsigned char* ctl = ctx.d_small + 512;
    check_cuda(cudaMemsetAsync(ctl, 0, 64, ctx.stream), "cudaMemsetAsync");
    auto launch = [&](auto tag, auto threads_tag) {
        using K = decltype(tag);
        constexpr int THREADS = decltype(threads_tag)::value;
        RbkArgs<K> a;
        a.keys = static_cast<const K*>(keys);
        a.vals = vals;
        a.n = (uint32_t)n;
        a.keys_out = static_cast<K*>(keys_out);
        a.sums_out = sums_out;
        a.counts_out = counts_out;
        a.hist = hist;
        a.num_runs = num_runs_device;
        a.num_tiles = num_tiles;
        a.ring = ctx.lookback_ring;
        a.seq0 = ctx.reserve_seq(num_tiles);
        a.tile_ctr = reinterpret_cast<uint32_t*>(ctl);
        a.err = ctx.d_error;
        int per_sm = 0;
        check_cuda(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, &k_reduce_by_key<K, THREADS>, THREADS, 0),
                   "cudaOccupancyMaxActiveBlocksPerMultiprocessor");
        const int grid = (int)std::min<std::size_t>(num_tiles, (std::size_t)ctx.sm_count * std::max(per_sm, 1));
        kernel_timer kt(ctx, "reduce_by_key.lookback");
        k_reduce_by_key<K, THREADS><<<grid, THREADS, 0, ctx.stream>>>(a);
        check_cuda(cudaGetLastError(), "reduce_by_key launch");
    };
    auto by_threads = [&](auto tag) {
        if (threads == 64) launch(tag, std::integral_constant<int, 64>{});
        else if (threads == 128) launch(tag, std::integral_constant<int, 128>{});
        else launch(tag, std::integral_constant<int, 256>{});
    };
    if (key_bytes == 4) by_threads(uint32_t{});
    else by_threads(uint64_t{});
}

}  // namespace gbc
