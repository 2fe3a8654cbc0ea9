// Onesweep LSD radix sort for sm_103a: 8-bit digits, one upfront pass that
// builds every digit histogram, then one kernel per digit that ranks a tile of
// keys by peer-mask words in shared memory (or warp votes) and finds the
// tile's global offsets by a decoupled look-back over per-(tile, digit) status
// words.
//
// Reference path replaced: detail::radix_sort (lib/src/Compute/
// Algorithm.cpp:453-527) with its kernels clc_radix_histogram (153-171) and
// clc_radix_scatter (173-212). The reference makes 8 passes of 4 bits, each a
// histogram launch, a recursive scan of the digit-major count table and a
// scatter whose in-tile rank comes from a work-group scan of packed counters.
// This file makes ceil(bits/8) passes; the counts of all digits come from one
// read of the keys, and the per-tile prefix is resolved on the fly, so each
// pass reads and writes the keys once.
//
// Semantics kept from the reference:
//   * stable: equal keys keep their input order (digits are ranked in input
//     order within a tile; tiles are ordered by their look-back sequence);
//   * the key bijection of Algorithm.cpp:459-469 (int: flip sign bit; float:
//     negative -> ~k, else k | sign; descending -> complement) is applied to
//     compute digits only, the stored keys are untouched;
//   * keys and values end up in the caller's buffers.
// Added: 64-bit keys, an out-of-place form, and skipping of digit positions
// on which all keys agree (decided on the device, so the launch sequence is
// fixed and graph-capturable).
#include <algorithm>
#include <cstring>
#include <string>

#include "device_common.cuh"
#include "runtime.hpp"
#include "sort_internal.hpp"

namespace gbc {
namespace onesweep {

using dev::FULL_MASK;

// Status word of one (tile, digit): [63:62] flag, [61:32] sequence tag,
// [31:0] count. FLAG_AGG: the tile's own count; FLAG_PRE: the inclusive count
// of this digit over all tiles up to and including this one.
constexpr uint64_t FLAG_AGG = 1, FLAG_PRE = 2;
constexpr uint64_t TAG_MASK = (1ull << 30) - 1;

__device__ __forceinline__ uint64_t pack_status(uint64_t flag, uint64_t seq, uint32_t v)
{
    return (flag << 62) | ((seq & TAG_MASK) << 32) | v;
}

template <typename K> struct Traits;
template <> struct Traits<uint32_t> {
    static constexpr int PASSES = 4;
};
template <> struct Traits<uint64_t> {
    static constexpr int PASSES = 8;
};

template <typename K> struct SortArgs {
    const K* in_keys;
    K* out_keys;
    K* alt_keys;
    const uint32_t* in_vals;
    uint32_t* out_vals;
    uint32_t* alt_vals;
    uint32_t n;
    int in_place;
    dev::KeyXform<K> xf;
    SortControl* ctl;
    uint64_t* ring;
    uint64_t seq0;
    uint32_t num_tiles;
    int* err;
    // tile-offset form: per tile and digit, the tile's count, then its first
    // output position; per chunk of tiles and digit, the same for the chunk
    uint32_t* tile_off;
    uint32_t* chunk_off;
    uint32_t chunks;
    uint32_t tiles_per_chunk;
};

// ---------------------------------------------------------------------------
// K1: upfront histogram of every digit position, plus the pass plan.
// ---------------------------------------------------------------------------
template <typename K, int THREADS, int NSUB>
__global__ void __launch_bounds__(THREADS) k_upfront(SortArgs<K> a)
{
    constexpr int P = Traits<K>::PASSES;
    constexpr int PER_VEC = 16 / sizeof(K);
    extern __shared__ __align__(16) uint32_t sh_hist[];  // NSUB x P x 256
    __shared__ uint32_t s_scratch[8];
    __shared__ uint32_t s_trivial[8];
    __shared__ int s_last;

    for (int i = threadIdx.x; i < NSUB * P * RADIX; i += THREADS) sh_hist[i] = 0;
    __syncthreads();
    uint32_t* my = sh_hist + ((threadIdx.x >> 5) % NSUB) * (P * RADIX);

    const size_t n = a.n;
    const K* keys = a.in_keys;
    const size_t gtid = (size_t)blockIdx.x * THREADS + threadIdx.x;
    const size_t stride = (size_t)gridDim.x * THREADS;
    auto count = [&](K k) {
        const K t = a.xf(k);
#pragma unroll
        for (int p = 0; p < P; ++p)
            atomicAdd(&my[p * RADIX + (uint32_t)((t >> (8 * p)) & 0xFF)], 1u);
    };
    size_t head = 0;
    if ((reinterpret_cast<uintptr_t>(keys) & 15) == 0) {
        const size_t nv = n / PER_VEC;
        const uint4* kv = reinterpret_cast<const uint4*>(keys);
        size_t v = gtid;
        // four 128-bit loads in flight per thread before they are counted
        for (; v + 3 * stride < nv; v += 4 * stride) {
            uint4 w[4];
#pragma unroll
            for (int q = 0; q < 4; ++q) w[q] = dev::ld_stream(kv + v + q * stride);
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                K ks[PER_VEC];
                memcpy(ks, &w[q], 16);
#pragma unroll
                for (int j = 0; j < PER_VEC; ++j) count(ks[j]);
            }
        }
        for (; v < nv; v += stride) {
            const uint4 w = dev::ld_stream(kv + v);
            K ks[PER_VEC];
            memcpy(ks, &w, 16);
#pragma unroll
            for (int j = 0; j < PER_VEC; ++j) count(ks[j]);
        }
        head = nv * PER_VEC;
    }
    for (size_t i = head + gtid; i < n; i += stride) count(keys[i]);
    __syncthreads();

    uint32_t* g_hist = &a.ctl->hist[0][0];
    for (int i = threadIdx.x; i < P * RADIX; i += THREADS) {
        uint32_t s = 0;
#pragma unroll
        for (int b = 0; b < NSUB; ++b) s += sh_hist[b * P * RADIX + i];
        if (s != 0) atomicAdd(&g_hist[i], s);
    }
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) s_last = atomicAdd(&a.ctl->done, 1u) == gridDim.x - 1;
    __syncthreads();
    if (!s_last) return;
    __threadfence();

    // The last CTA turns the counts into the pass plan: skip every digit
    // position on which all keys agree; exclusive bin starts for the rest.
    if (threadIdx.x < 8) s_trivial[threadIdx.x] = 0;
    __syncthreads();
    for (int p = 0; p < P; ++p)
        if (threadIdx.x < RADIX && dev::ld_relaxed(&g_hist[p * RADIX + threadIdx.x]) == (uint32_t)n)
            s_trivial[p] = 1;
    __syncthreads();
    int slot = 0;
    for (int p = 0; p < P; ++p) {
        if (s_trivial[p]) continue;
        const uint32_t c =
            threadIdx.x < RADIX ? dev::ld_relaxed(&g_hist[p * RADIX + threadIdx.x]) : 0u;
        const uint32_t ex = dev::bins_exclusive_sum(c, s_scratch);
        if (threadIdx.x < RADIX) a.ctl->plan.bin_start[slot][threadIdx.x] = ex;
        if (threadIdx.x == 0) a.ctl->plan.shift[slot] = 8 * p;
        ++slot;
    }
    if (threadIdx.x == 0) a.ctl->plan.num_active = slot;
}

// When the pass count does not land the result in the right buffer: copy the
// input once (out-of-place with nothing to sort, or in-place with an odd
// number of active passes, which then start from the scratch buffer).
template <typename K> __global__ void k_precopy(SortArgs<K> a)
{
    const uint32_t act = a.ctl->plan.num_active;
    const K* s;
    K* d;
    const uint32_t* sv;
    uint32_t* dv;
    if (act == 0 && !a.in_place) {
        s = a.in_keys, d = a.out_keys, sv = a.in_vals, dv = a.out_vals;
    } else if (a.in_place && (act & 1)) {
        s = a.in_keys, d = a.alt_keys, sv = a.in_vals, dv = a.alt_vals;
    } else {
        return;
    }
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    const size_t gtid = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    auto copy = [&](const void* src, void* dst, size_t bytes) {
        // 128-bit copies when both sides are aligned, then the tail
        size_t head = 0;
        if (((reinterpret_cast<uintptr_t>(src) | reinterpret_cast<uintptr_t>(dst)) & 15) == 0) {
            const uint4* s4 = static_cast<const uint4*>(src);
            uint4* d4 = static_cast<uint4*>(dst);
            const size_t nv = bytes / 16;
            for (size_t v = gtid; v < nv; v += stride) d4[v] = dev::ld_stream(s4 + v);
            head = nv * 16;
        }
        const unsigned char* sb = static_cast<const unsigned char*>(src);
        unsigned char* db = static_cast<unsigned char*>(dst);
        for (size_t i = head + gtid; i < bytes; i += stride) db[i] = sb[i];
    };
    copy(s, d, (size_t)a.n * sizeof(K));
    if (sv != nullptr) copy(sv, dv, (size_t)a.n * 4);
}

// ---------------------------------------------------------------------------
// K2: one digit pass (persistent CTAs, tiles handed out in order by an atomic
// counter so every look-back waits only on CTAs that are already running).
// ---------------------------------------------------------------------------
template <typename K, bool HAS_V, int THREADS, int ITEMS, bool MATCH>
__device__ __forceinline__ void pass_body(const SortArgs<K>& a, int slot)
{
    constexpr int WARPS = THREADS / 32;
    constexpr int TILE = THREADS * ITEMS;
    static_assert(THREADS >= RADIX, "one thread per bin");
    static_assert(TILE < (1 << 24), "rank and digit share a word");

    const uint32_t act = a.ctl->plan.num_active;
    if (slot >= (int)act) return;
    const uint32_t shift = a.ctl->plan.shift[slot];

    // Buffer roles for this slot (see k_precopy): the last active pass always
    // writes the caller's output.
    const bool dst_out = ((act - 1 - slot) & 1) == 0;
    K* dst_k = dst_out ? a.out_keys : a.alt_keys;
    uint32_t* dst_v = dst_out ? a.out_vals : a.alt_vals;
    const K* src_k;
    const uint32_t* src_v;
    if (slot == 0) {
        const bool from_alt = a.in_place && (act & 1);
        src_k = from_alt ? a.alt_keys : a.in_keys;
        src_v = from_alt ? a.alt_vals : a.in_vals;
    } else {
        const bool prev_out = ((act - slot) & 1) == 0;
        src_k = prev_out ? a.out_keys : a.alt_keys;
        src_v = prev_out ? a.out_vals : a.alt_vals;
    }

    extern __shared__ __align__(16) unsigned char smem[];
    uint32_t* warp_hist = reinterpret_cast<uint32_t*>(smem);  // WARPS x 256
    K* s_keys = reinterpret_cast<K*>(warp_hist + WARPS * RADIX);
    uint32_t* s_vals = reinterpret_cast<uint32_t*>(s_keys + TILE);
    __shared__ uint32_t s_bin_start[RADIX], s_bin_off[RADIX], s_local[RADIX];
    __shared__ uint32_t s_scratch[8];
    __shared__ uint32_t s_tile;
    __shared__ int s_abort;  // a look-back wait gave up: skip the scatter

    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    if (tid < RADIX) s_bin_start[tid] = a.ctl->plan.bin_start[slot][tid];
    if (tid == 0) s_abort = 0;
    const uint64_t seq0 = a.seq0 + (uint64_t)slot * a.num_tiles;
    uint32_t* ctr = &a.ctl->tile_ctr[slot];
    const uint32_t n = a.n;

    for (;;) {
        if (tid == 0) s_tile = atomicAdd(ctr, 1u);
        for (int i = tid; i < WARPS * RADIX; i += THREADS) warp_hist[i] = 0;
        __syncthreads();
        const uint32_t t = s_tile;
        if (t >= a.num_tiles) break;
        const uint32_t tile_base = t * TILE;
        const uint32_t valid = min((uint32_t)TILE, n - tile_base);

        // Load: warp w owns keys [w*32*ITEMS, (w+1)*32*ITEMS) of the tile,
        // row i of the warp is 32 consecutive keys (one 128-byte line for
        // 32-bit keys). Past the end, the digit is 255 so padding ranks last.
        const uint32_t wbase = tile_base + warp * 32 * ITEMS + lane;
        K key[ITEMS];
        uint32_t rd[ITEMS];  // (rank << 8) | digit
#pragma unroll
        for (int i = 0; i < ITEMS; ++i) {
            const uint32_t idx = wbase + i * 32;
            if (idx < n) {
                key[i] = src_k[idx];
                rd[i] = (uint32_t)(a.xf(key[i]) >> shift) & 0xFFu;
            } else {
                key[i] = 0;
                rd[i] = 0xFFu;
            }
        }

        // Rank within the warp, row by row (= input order): peers are the
        // lanes holding the same digit; the highest peer bumps the warp's
        // count for that digit.
        uint32_t* wh = warp_hist + warp * RADIX;
#pragma unroll
        for (int i = 0; i < ITEMS; ++i) {
            const uint32_t d = rd[i];
            uint32_t peers;
            if (MATCH) {
                peers = __match_any_sync(FULL_MASK, d);
            } else {
                peers = FULL_MASK;
#pragma unroll
                for (int b = 0; b < 8; ++b) {
                    const uint32_t bit = (d >> b) & 1u;
                    const uint32_t vote = __ballot_sync(FULL_MASK, bit);
                    peers &= bit ? vote : ~vote;
                }
            }
            const int leader = 31 - __clz(peers);
            uint32_t before = 0;
            if (lane == leader) {
                before = wh[d];
                wh[d] = before + __popc(peers);
            }
            before = __shfl_sync(FULL_MASK, before, leader);
            rd[i] = ((before + __popc(peers & dev::lanemask_lt())) << 8) | d;
            __syncwarp();
        }
        __syncthreads();

        // Per-digit tile counts; warp_hist becomes the exclusive prefix over
        // warps.
        uint32_t count = 0;
        if (tid < RADIX) {
#pragma unroll
            for (int w = 0; w < WARPS; ++w) {
                const uint32_t c = warp_hist[w * RADIX + tid];
                warp_hist[w * RADIX + tid] = count;
                count += c;
            }
        }
        uint32_t agg = count;
        if (tid == RADIX - 1) agg -= (uint32_t)TILE - valid;  // padding sits in bin 255
        uint64_t* my_status = a.ring + ((seq0 + t) & (RING_TILES - 1)) * RADIX;
        if (tid < RADIX)
            dev::st_relaxed(&my_status[tid],
                            pack_status(t == 0 ? FLAG_PRE : FLAG_AGG, seq0 + t, agg));

        const uint32_t local = dev::bins_exclusive_sum(count, s_scratch);
        if (tid < RADIX) s_local[tid] = local;
        __syncthreads();

        // Local sort of the tile into shared memory.
#pragma unroll
        for (int i = 0; i < ITEMS; ++i) {
            const uint32_t d = rd[i] & 0xFFu;
            const uint32_t pos = s_local[d] + warp_hist[warp * RADIX + d] + (rd[i] >> 8);
            s_keys[pos] = key[i];
            rd[i] = pos;
        }
        if (HAS_V) {
#pragma unroll
            for (int i = 0; i < ITEMS; ++i) {
                const uint32_t idx = wbase + i * 32;
                s_vals[rd[i]] = idx < n ? src_v[idx] : 0u;
            }
        }

        // Decoupled look-back: one thread per digit walks back over the
        // preceding tiles until it meets an inclusive prefix.
        if (tid < RADIX) {
            uint32_t excl = 0;
            if (t > 0) {
                uint64_t k = t - 1;
                for (;;) {
                    const uint64_t seq = seq0 + k;
                    const uint64_t* p = a.ring + (seq & (RING_TILES - 1)) * RADIX + tid;
                    const uint64_t want = seq & TAG_MASK;
                    uint64_t w = dev::ld_relaxed(p);
                    bool gave_up = false;
                    if ((w >> 62) == 0 || ((w >> 32) & TAG_MASK) != want) {
                        const unsigned long long start = dev::globaltimer();
                        for (uint32_t spin = 1;; ++spin) {
                            w = dev::ld_relaxed(p);
                            if ((w >> 62) != 0 && ((w >> 32) & TAG_MASK) == want) break;
                            if ((spin & 255) == 0 && dev::globaltimer() - start > dev::SPIN_LIMIT_NS) {
                                gave_up = true;
                                break;
                            }
                            if (spin > 32) __nanosleep(64);
                        }
                    }
                    if (gave_up) {
                        dev::raise_error(a.err, dev::ERR_LOOKBACK_TIMEOUT);
                        s_abort = 1;
                        break;
                    }
                    excl += (uint32_t)w;
                    if ((w >> 62) == FLAG_PRE || k == 0) break;
                    --k;
                }
                dev::st_relaxed(&my_status[tid], pack_status(FLAG_PRE, seq0 + t, excl + agg));
            }
            s_bin_off[tid] = s_bin_start[tid] + excl - s_local[tid];
        }
        __syncthreads();

        // Write the locally sorted tile: consecutive threads write
        // consecutive addresses within each digit's run. After a timed-out
        // wait the offsets are unknown: nothing is written (the error is
        // reported) and every write is bounds-checked regardless.
        const uint32_t limit = s_abort ? 0u : valid;
        for (uint32_t j = tid; j < limit; j += THREADS) {
            const K kk = s_keys[j];
            const uint32_t d = (uint32_t)(a.xf(kk) >> shift) & 0xFFu;
            const uint32_t o = s_bin_off[d] + j;
            if (o < n) {
                dst_k[o] = kk;
                if (HAS_V) dst_v[o] = s_vals[j];
            }
        }
        __syncthreads();
    }
}

// The digit pass with the compiler's default register budget, and with a
// minimum number of resident CTAs per SM (which caps registers).
template <typename K, bool HAS_V, int THREADS, int ITEMS, bool MATCH>
__global__ void __launch_bounds__(THREADS) k_pass(SortArgs<K> a, int slot)
{
    pass_body<K, HAS_V, THREADS, ITEMS, MATCH>(a, slot);
}
template <typename K, bool HAS_V, int THREADS, int ITEMS, bool MATCH, int MINB>
__global__ void __launch_bounds__(THREADS, MINB) k_pass_mb(SortArgs<K> a, int slot)
{
    pass_body<K, HAS_V, THREADS, ITEMS, MATCH>(a, slot);
}

// ---------------------------------------------------------------------------
// Tile-offset form of the digit pass: every tile's output offsets are
// computed before the pass (reduce, then scan), so the pass reads them
// instead of looking back over its predecessors. Before each pass:
//   k_tile_hist     each CTA counts the digits of every tile of a quarter of
//                   a chunk (contiguous tiles) and adds them to the chunk's
//                   totals;
//   k_chunk_scan    the chunks' totals become their first output positions;
//   k_tile_offsets  each chunk turns its tiles' counts into their first
//                   output positions, in place.
// The pass itself still takes its tiles in input order from the atomic
// counter, so each digit's output is written in one advancing window. (With
// each CTA sorting one chunk of tiles in order instead, 2^28 pairs took
// 7.2 ms against 6.05: every (chunk, digit) is its own write stream.)
// ---------------------------------------------------------------------------
template <typename K>
__device__ __forceinline__ const K* pass_src_keys(const SortArgs<K>& a, int slot, uint32_t act)
{
    if (slot == 0) return (a.in_place && (act & 1)) ? a.alt_keys : a.in_keys;
    return ((act - slot) & 1) == 0 ? a.out_keys : a.alt_keys;
}

constexpr int TH_THREADS = 256;  // = RADIX: thread d owns digit d's counts
constexpr int TH_SPLIT = 4;      // k_tile_hist CTAs per chunk

template <typename K, bool IDENT, int TILE>
__global__ void __launch_bounds__(TH_THREADS) k_tile_hist(SortArgs<K> a, int slot)
{
    constexpr int WARPS = TH_THREADS / 32;
    constexpr int VEC = 16 / (int)sizeof(K);
    constexpr int NV = (TILE / VEC + TH_THREADS - 1) / TH_THREADS;  // 16-byte loads per thread per tile
    static_assert(TH_THREADS == RADIX && TILE % VEC == 0, "one thread per digit; whole vectors per tile");
    __shared__ uint32_t h[WARPS][RADIX];  // per warp
    const uint32_t act = a.ctl->plan.num_active;
    if (slot >= (int)act) return;
    const uint32_t shift = a.ctl->plan.shift[slot];
    const K* src = pass_src_keys(a, slot, act);
    const int tid = threadIdx.x, warp = tid >> 5;
    for (int w = 0; w < WARPS; ++w) h[w][tid] = 0;
    __syncthreads();
    uint32_t* my = h[warp];
    auto count = [&](K k) { atomicAdd(&my[(uint32_t)((IDENT ? k : a.xf(k)) >> shift) & 0xFFu], 1u); };
    const bool aligned = (reinterpret_cast<uintptr_t>(src) & 15) == 0;
    const uint32_t chunk = blockIdx.x / TH_SPLIT, part = blockIdx.x % TH_SPLIT;
    const uint32_t per = (a.tiles_per_chunk + TH_SPLIT - 1) / TH_SPLIT;
    const uint32_t cend = min((chunk + 1) * a.tiles_per_chunk, a.num_tiles);
    const uint32_t t0 = min(chunk * a.tiles_per_chunk + part * per, cend), t1 = min(t0 + per, cend);
    uint32_t total = 0;
    for (uint32_t t = t0; t < t1; ++t) {
        const uint64_t b = (uint64_t)t * TILE;
        if (aligned && b + TILE <= a.n) {
            const uint4* v4 = reinterpret_cast<const uint4*>(src + b);
            uint4 w[NV];
#pragma unroll
            for (int j = 0; j < NV; ++j)
                if (j * TH_THREADS + tid < TILE / VEC) w[j] = dev::ld_stream(v4 + j * TH_THREADS + tid);
#pragma unroll
            for (int j = 0; j < NV; ++j)
                if (j * TH_THREADS + tid < TILE / VEC) {
                    K ks[VEC];
                    memcpy(ks, &w[j], 16);
#pragma unroll
                    for (int q = 0; q < VEC; ++q) count(ks[q]);
                }
        } else {
            const uint64_t e = min(b + TILE, (uint64_t)a.n);
            for (uint64_t i = b + tid; i < e; i += TH_THREADS) count(src[i]);
        }
        __syncthreads();
        uint32_t c = 0;
#pragma unroll
        for (int w = 0; w < WARPS; ++w) {
            c += h[w][tid];
            h[w][tid] = 0;
        }
        a.tile_off[(size_t)t * RADIX + tid] = c;
        total += c;
        __syncthreads();
    }
    if (total != 0) atomicAdd(&a.chunk_off[(size_t)chunk * RADIX + tid], total);
}

// The chunks' counts of each digit become their first output positions
// (the digit's start plus the counts of every earlier chunk), in place. One
// CTA per digit; thread i scans a contiguous run of chunks (one chunk each up
// to 1,024 chunks). (One warp per digit, 32 digits per CTA, took 23.5 us per
// pass at 2^28 keys: 8 CTAs, each lane ten dependent strided loads.)
template <typename K> __global__ void __launch_bounds__(1024) k_chunk_scan(SortArgs<K> a, int slot)
{
    const uint32_t act = a.ctl->plan.num_active;
    if (slot >= (int)act) return;
    __shared__ uint32_t s_warp[32];
    const int d = blockIdx.x, tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    uint32_t* col = a.chunk_off + d;
    const uint32_t per = (a.chunks + 1023) / 1024;
    const uint32_t c0 = min(tid * per, a.chunks), c1 = min(c0 + per, a.chunks);
    uint32_t sum = 0;
    for (uint32_t c = c0; c < c1; ++c) sum += col[(size_t)c * RADIX];
    auto plus = [](uint32_t x, uint32_t y) { return x + y; };
    const uint32_t incl = dev::warp_inclusive_scan(sum, plus);
    if (lane == 31) s_warp[warp] = incl;
    __syncthreads();
    if (warp == 0) {
        const uint32_t w = s_warp[lane];
        s_warp[lane] = dev::warp_inclusive_scan(w, plus) - w;
    }
    __syncthreads();
    uint32_t run = a.ctl->plan.bin_start[slot][d] + s_warp[warp] + incl - sum;
    for (uint32_t c = c0; c < c1; ++c) {
        const uint32_t v = col[(size_t)c * RADIX];
        col[(size_t)c * RADIX] = run;
        run += v;
    }
}

// Each chunk's tiles: counts become first output positions, in place. Four
// threads per digit, each a contiguous quarter of the chunk's tiles: the
// quarters' sums, then each quarter's tiles from its base (8 tiles' counts
// in flight). The chunk's totals are cleared for the next pass's
// k_tile_hist. (One thread per digit walking all the chunk's tiles took
// 43 us per pass at 2^28 keys, 72 tiles per chunk.)
constexpr int TO_QUARTERS = 4;
template <typename K> __global__ void __launch_bounds__(TO_QUARTERS * RADIX) k_tile_offsets(SortArgs<K> a, int slot)
{
    constexpr int B = 8;
    const uint32_t act = a.ctl->plan.num_active;
    if (slot >= (int)act) return;
    __shared__ uint32_t s_quarter[TO_QUARTERS][RADIX];
    const int d = threadIdx.x & (RADIX - 1), q = threadIdx.x / RADIX;
    const uint32_t t0 = blockIdx.x * a.tiles_per_chunk, t1 = min(t0 + a.tiles_per_chunk, a.num_tiles);
    const uint32_t per = (t1 - t0 + TO_QUARTERS - 1) / TO_QUARTERS;
    const uint32_t q0 = min(t0 + q * per, t1), q1 = min(q0 + per, t1);
    uint32_t* col = a.tile_off + d;
    uint32_t sum = 0;
    for (uint32_t t = q0; t < q1; t += B) {
        uint32_t v[B];
#pragma unroll
        for (int j = 0; j < B; ++j) v[j] = t + j < q1 ? col[(size_t)(t + j) * RADIX] : 0u;
#pragma unroll
        for (int j = 0; j < B; ++j) sum += v[j];
    }
    s_quarter[q][d] = sum;
    uint32_t* chunk_row = a.chunk_off + (size_t)blockIdx.x * RADIX;
    uint32_t run = chunk_row[d];
    __syncthreads();  // the quarters' sums are in, and every thread has read the chunk's first positions
    for (int j = 0; j < q; ++j) run += s_quarter[j][d];
    if (q == 0) chunk_row[d] = 0;
    for (uint32_t t = q0; t < q1; t += B) {
        uint32_t v[B];
#pragma unroll
        for (int j = 0; j < B; ++j) v[j] = t + j < q1 ? col[(size_t)(t + j) * RADIX] : 0u;
#pragma unroll
        for (int j = 0; j < B; ++j)
            if (t + j < q1) {
                col[(size_t)(t + j) * RADIX] = run;
                run += v[j];
            }
    }
}

// ---------------------------------------------------------------------------
// K2, second form. The first form executes about 4.3 warp instructions per
// key and keeps the ALU pipe ~64% busy while DRAM runs at ~15%: it is bound
// by instruction issue (8 ballots per row of keys) and by its look-back,
// which walks back one tile per round trip. Here:
//   * rows are ranked by shared-memory peer masks: each lane ORs its bit into
//     its digit's mask word and reads the word back (its peers); the lowest
//     peer bumps the warp's count and clears the word (keeping the rows of a
//     group in separate mask arrays to overlap their round trips measured no
//     faster, and packing mask and count into one 64-bit word slower);
//   * each warp's place offset per digit already includes the digit's start
//     in the tile, so placing a key costs one shared-memory lookup;
//   * the look-back reads LBW predecessors' status words per round trip:
//     tiles start a few tens of nanoseconds apart, so the nearest inclusive
//     prefix is typically several tiles back. (Handing the whole look-back to
//     one warp, 8 digits per lane with 16-byte status loads, made the sort
//     twice as slow, and so did taking the next tile's index early: a tile
//     taken before the CTA can work on it publishes its counts late);
//   * IDENT: the key transform is the identity (unsigned ascending keys);
//   * HALF: rows of 16 keys, one per half-warp, ranked in one 32-bit word per
//     half-warp and digit that holds the count (high 16 bits) and the row's
//     peer mask (low 16 bits): an OR, one read and the lowest peer's store
//     of the new count (which also clears the mask), three shared-memory
//     instructions per 32 keys instead of five. Each half-warp takes a
//     contiguous run of the tile, so ranks stay in input order.
// ---------------------------------------------------------------------------
template <typename K, bool HAS_V, int THREADS, int ITEMS, bool IDENT, int LBW, bool STAGED, bool PREFETCH, int BR,
          bool HALF, int PAD, bool PACK = false, bool TOFF = false>
__device__ __forceinline__ void pass2_body(const SortArgs<K>& a, int slot)
{
    // TOFF: the tile's output offsets come from tile_off (computed before the
    // pass) instead of a look-back.
    // PACK (32-bit keys with values): the locally sorted tile holds each key
    // and its value side by side, placed with one 64-bit store instead of
    // two 32-bit ones (2^28 pairs: 6.25 -> 6.07 ms with PAD 1, 6.07 -> 6.04
    // with PAD 0; keys the AND of 4 words: 6.75 -> 6.52 ms).
    static_assert(!PACK || (HAS_V && sizeof(K) == 4), "packed tiles hold 32-bit key-value pairs");
    constexpr int WARPS = THREADS / 32;
    constexpr int TILE = THREADS * ITEMS;
    constexpr int GROUPS = HALF ? 2 * WARPS : WARPS;  // ranking groups: warps or half-warps
    constexpr int GW = HALF ? 16 : 32;                // keys per row of a group
    // PAD > 0: a half-warp's words sit PAD banks from its partner's, so equal
    // digits in the two halves of a row do not meet in one bank (skewed keys:
    // 2^28 pairs whose keys are the AND of 4 uniform words, 7.9 ms with PAD 0,
    // 6.8 ms with PAD 1). Uniform keys measure fastest with PAD 0 (6.07 ms
    // against 6.27 for any PAD tried: 1, 8, 16), so both are compiled. (The
    // same choice made per pass on the device from the upfront histogram, a
    // stride known only at run time, was slower for both: 6.52 and 7.06 ms.)
    static_assert(PAD >= 0 && PAD <= 16, "the shared-memory size allows 16 words of padding per group");
    constexpr int GSTRIDE = HALF ? RADIX + PAD : RADIX;
    constexpr int TILE_AT = HALF ? GROUPS * GSTRIDE : 2 * WARPS * RADIX;  // words
    static_assert(THREADS >= RADIX, "one thread per bin");
    static_assert(TILE < (1 << 24), "rank and digit share a word");
    static_assert(!HALF || (BR == 0 && GW * ITEMS < (1 << 16)), "half-warp counts are 16-bit");

    const uint32_t act = a.ctl->plan.num_active;
    if (slot >= (int)act) return;
    const uint32_t shift = a.ctl->plan.shift[slot];
    const bool dst_out = ((act - 1 - slot) & 1) == 0;
    K* dst_k = dst_out ? a.out_keys : a.alt_keys;
    uint32_t* dst_v = dst_out ? a.out_vals : a.alt_vals;
    const K* src_k;
    const uint32_t* src_v;
    if (slot == 0) {
        const bool from_alt = a.in_place && (act & 1);
        src_k = from_alt ? a.alt_keys : a.in_keys;
        src_v = from_alt ? a.alt_vals : a.in_vals;
    } else {
        const bool prev_out = ((act - slot) & 1) == 0;
        src_k = prev_out ? a.out_keys : a.alt_keys;
        src_v = prev_out ? a.out_vals : a.alt_vals;
    }

    extern __shared__ __align__(16) unsigned char smem[];
    // Per group and digit: the running count (then the place offset) and the
    // current row's peer mask: two words per warp, or one word per half-warp.
    uint32_t* warp_hist = reinterpret_cast<uint32_t*>(smem);  // GROUPS x GSTRIDE
    uint32_t* warp_mask = warp_hist + WARPS * RADIX;          // WARPS x 256 (not HALF)
    // One tile of keys (+ values); STAGED: two, the next tile's bulk copy
    // landing in one while the current tile is worked on in the other.
    unsigned char* tiles = reinterpret_cast<unsigned char*>(warp_hist + TILE_AT);
    constexpr uint32_t KEY_BYTES = TILE * sizeof(K), VAL_BYTES = HAS_V ? TILE * 4 : 0;
    constexpr uint32_t STAGE_BYTES = KEY_BYTES + VAL_BYTES;
    __shared__ uint32_t s_bin_start[RADIX], s_bin_off[RADIX], s_local[RADIX];
    __shared__ uint32_t s_scratch[8];
    __shared__ int s_abort;
    __shared__ uint32_t s_stage_tile[2];
    __shared__ int s_inflight[2];
    __shared__ __align__(8) uint64_t s_bar[2];

    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int grp = HALF ? 2 * warp + (lane >> 4) : warp;  // ranking group
    const int gl = HALF ? lane & 15 : lane;                // lane within the group
    const uint32_t lt_mask = dev::lanemask_lt();
    auto digit = [&](K k) -> uint32_t { return (uint32_t)((IDENT ? k : a.xf(k)) >> shift) & 0xFFu; };
    if (!HALF)
        for (int i = tid; i < WARPS * RADIX; i += THREADS) warp_mask[i] = 0;
    if (tid < RADIX) s_bin_start[tid] = a.ctl->plan.bin_start[slot][tid];
    const uint64_t seq0 = a.seq0 + (uint64_t)slot * a.num_tiles;
    uint32_t* ctr = &a.ctl->tile_ctr[slot];
    auto take = [&]() -> uint32_t { return atomicAdd(ctr, 1u); };  // thread 0: the next tile
    const uint32_t n = a.n;
    // Bulk copies need 16-byte aligned sources; a partial last tile is loaded
    // by plain loads.
    const bool aligned_src =
        ((reinterpret_cast<uintptr_t>(src_k) | (HAS_V ? reinterpret_cast<uintptr_t>(src_v) : 0)) & 15) == 0;
    const bool aligned = STAGED && aligned_src;
    auto bulk_ok = [&](uint32_t tt) { return aligned && tt < a.num_tiles && (uint64_t)(tt + 1) * TILE <= n; };
    auto issue = [&](int st, uint32_t tt) {  // one thread
        s_stage_tile[st] = tt;
        if (!STAGED || s_abort || !bulk_ok(tt)) return;
        unsigned char* dst = tiles + st * STAGE_BYTES;
        dev::fence_proxy_async();
        dev::mbar_arrive_expect_tx(&s_bar[st], STAGE_BYTES);
        dev::bulk_g2s(dst, src_k + (size_t)tt * TILE, KEY_BYTES, &s_bar[st]);
        if (HAS_V) dev::bulk_g2s(dst + KEY_BYTES, src_v + (size_t)tt * TILE, VAL_BYTES, &s_bar[st]);
        s_inflight[st] = 1;
    };
    if (tid == 0) {
        s_abort = 0;
        s_inflight[0] = s_inflight[1] = 0;
        if (STAGED) {
            dev::mbar_init(&s_bar[0], 1);
            dev::mbar_init(&s_bar[1], 1);
            dev::fence_mbar_init();
        }
        issue(0, take());
    }
    int st = 0;
    uint32_t parity = 0;  // bit s: phase parity of stage s's barrier

    for (;;) {
        if (STAGED && tid == 0) issue(st ^ 1, take());  // the next tile's copy
        if (PREFETCH && tid == 0) {
            // The tile a grid further on, which some CTA takes about one
            // tile-time from now, is prefetched into L2.
            const uint64_t ahead = (uint64_t)s_stage_tile[STAGED ? st ^ 1 : 0] + gridDim.x;
            if (ahead < a.num_tiles && (ahead + 1) * TILE <= n && aligned_src) {
                dev::prefetch_l2(src_k + ahead * TILE, TILE * sizeof(K));
                if (HAS_V) dev::prefetch_l2(src_v + ahead * TILE, TILE * 4);
            }
        }
        for (int i = tid; i < GROUPS * GSTRIDE; i += THREADS) warp_hist[i] = 0;
        __syncthreads();
        const uint32_t t = s_stage_tile[st];
        if (t >= a.num_tiles) break;
        const uint32_t tile_base = t * TILE;
        const uint32_t valid = min((uint32_t)TILE, n - tile_base);
        // TOFF: digit tid's first output position for this tile, used after ranking
        const uint32_t toff = TOFF && tid < RADIX ? a.tile_off[(size_t)t * RADIX + tid] : 0u;
        K* s_keys = reinterpret_cast<K*>(tiles + (STAGED ? st : 0) * STAGE_BYTES);
        uint32_t* s_vals = reinterpret_cast<uint32_t*>(tiles + (STAGED ? st : 0) * STAGE_BYTES + KEY_BYTES);
        const bool staged = s_inflight[st] != 0;
        if (staged) {
            if (!dev::mbar_wait_bounded(&s_bar[st], (parity >> st) & 1u)) {
                dev::raise_error(a.err, dev::ERR_LOOKBACK_TIMEOUT);
                s_abort = 1;
            }
            parity ^= 1u << st;
        }

        // Load: row i of group g is keys tile_base + g*GW*ITEMS + GW*i + gl
        // (groups in input order). Past the end the digit is 255, so padding
        // ranks last.
        const uint32_t wbase = tile_base + grp * GW * ITEMS + gl;
        K key[ITEMS];
        uint32_t rd[ITEMS];
        uint32_t val[HAS_V ? ITEMS : 1];
        if (staged) {
            const uint32_t lb = grp * GW * ITEMS + gl;
#pragma unroll
            for (int i = 0; i < ITEMS; ++i) key[i] = s_keys[lb + i * GW];
            if (HAS_V) {
#pragma unroll
                for (int i = 0; i < ITEMS; ++i) val[i] = s_vals[lb + i * GW];
            }
#pragma unroll
            for (int i = 0; i < ITEMS; ++i) rd[i] = digit(key[i]);
        } else if (valid == (uint32_t)TILE) {
#pragma unroll
            for (int i = 0; i < ITEMS; ++i) key[i] = src_k[wbase + i * GW];
            if (HAS_V) {
#pragma unroll
                for (int i = 0; i < ITEMS; ++i) val[i] = src_v[wbase + i * GW];
            }
#pragma unroll
            for (int i = 0; i < ITEMS; ++i) rd[i] = digit(key[i]);
        } else {
#pragma unroll
            for (int i = 0; i < ITEMS; ++i) {
                const uint32_t idx = wbase + i * GW;
                const bool in = idx < n;
                key[i] = in ? src_k[idx] : K(0);
                if (HAS_V) val[i] = in ? src_v[idx] : 0u;
                rd[i] = in ? digit(key[i]) : 0xFFu;
            }
        }

        // Rank within the warp, row by row (= input order): every lane ORs its
        // bit into its digit's mask word and reads the word back (its peers)
        // and the warp's count of the digit in earlier rows; the lowest peer
        // stores the new count and clears the mask.
        uint32_t* wh = warp_hist + grp * GSTRIDE;
        uint32_t* wm = warp_mask + warp * RADIX;
        if (HALF) {
            const uint32_t hbit = 1u << gl, hlt = hbit - 1u;
#pragma unroll
            for (int i = 0; i < ITEMS; ++i) {
                const uint32_t d = rd[i];
                atomicOr(&wh[d], hbit);
                __syncwarp();
                const uint32_t x = wh[d];
                __syncwarp();
                const uint32_t peers = x & 0xFFFFu, before = x >> 16;
                if ((peers & hlt) == 0) wh[d] = (before + __popc(peers)) << 16;
                __syncwarp();
                rd[i] = ((before + __popc(peers & hlt)) << 8) | d;
            }
        }
#pragma unroll
        for (int i = 0; i < (HALF ? 0 : ITEMS); ++i) {
            const uint32_t d = rd[i];
            // BR of every 4 rows find their peers with 8 ballots (ALU pipe)
            // instead of the mask word (shared-memory pipe)
            const bool by_ballot = (i & 3) < BR;
            uint32_t peers;
            if (by_ballot) {
                peers = FULL_MASK;
#pragma unroll
                for (int b = 0; b < 8; ++b) {
                    const uint32_t bit = (d >> b) & 1u;
                    const uint32_t vote = __ballot_sync(FULL_MASK, bit);
                    peers &= bit ? vote : ~vote;
                }
            } else {
                atomicOr(&wm[d], 1u << lane);
                __syncwarp();
                peers = wm[d];
            }
            const uint32_t before = wh[d];
            __syncwarp();
            const uint32_t lower = peers & lt_mask;
            if (lower == 0) {
                wh[d] = before + __popc(peers);
                if (!by_ballot) wm[d] = 0;
            }
            __syncwarp();
            rd[i] = ((before + __popc(lower)) << 8) | d;
        }
        __syncthreads();

        // Per-digit tile counts; warp_hist becomes each warp's place offsets
        // (exclusive over warps, plus the digit's start within the tile).
        uint32_t count = 0;
        if (tid < RADIX) {
#pragma unroll
            for (int w = 0; w < GROUPS; ++w) {
                const uint32_t c = HALF ? warp_hist[w * GSTRIDE + tid] >> 16 : warp_hist[w * GSTRIDE + tid];
                warp_hist[w * GSTRIDE + tid] = count;
                count += c;
            }
        }
        uint32_t agg = count;
        if (tid == RADIX - 1) agg -= (uint32_t)TILE - valid;  // padding sits in bin 255
        uint64_t* my_status = a.ring + ((seq0 + t) & (RING_TILES - 1)) * RADIX;
        if (!TOFF && tid < RADIX)
            dev::st_relaxed(&my_status[tid], pack_status(t == 0 ? FLAG_PRE : FLAG_AGG, seq0 + t, agg));
        const uint32_t local = dev::bins_exclusive_sum(count, s_scratch);
        if (tid < RADIX) {
            s_local[tid] = local;
#pragma unroll
            for (int w = 0; w < GROUPS; ++w) warp_hist[w * GSTRIDE + tid] += local;
        }
        __syncthreads();

        // Local sort of the tile into shared memory.
#pragma unroll
        for (int i = 0; i < ITEMS; ++i) {
            const uint32_t pos = warp_hist[grp * GSTRIDE + (rd[i] & 0xFFu)] + (rd[i] >> 8);
            if constexpr (PACK) {
                reinterpret_cast<uint2*>(s_keys)[pos] = make_uint2((uint32_t)key[i], val[i]);
            } else {
                s_keys[pos] = key[i];
                if (HAS_V) s_vals[pos] = val[i];
            }
        }

        // The tile's offsets: read (TOFF) or from a decoupled look-back, one
        // thread per digit, LBW status words per round trip.
        if (TOFF) {
            if (tid < RADIX) s_bin_off[tid] = toff - s_local[tid];
        } else if (tid < RADIX) {
            uint32_t excl = 0;
            if (t > 0) {
                int64_t k = (int64_t)t - 1;
                bool done = false;
                while (!done) {
                    uint64_t w[LBW];
#pragma unroll
                    for (int j = 0; j < LBW; ++j)
                        if (k - j >= 0)
                            w[j] = dev::ld_relaxed(a.ring + ((seq0 + (uint64_t)(k - j)) & (RING_TILES - 1)) * RADIX +
                                                   tid);
#pragma unroll
                    for (int j = 0; j < LBW; ++j) {
                        if (done || k - j < 0) break;
                        const uint64_t seq = seq0 + (uint64_t)(k - j);
                        const uint64_t want = seq & TAG_MASK;
                        uint64_t x = w[j];
                        if ((x >> 62) == 0 || ((x >> 32) & TAG_MASK) != want) {
                            const uint64_t* p = a.ring + (seq & (RING_TILES - 1)) * RADIX + tid;
                            const unsigned long long start = dev::globaltimer();
                            for (uint32_t spin = 1;; ++spin) {
                                x = dev::ld_relaxed(p);
                                if ((x >> 62) != 0 && ((x >> 32) & TAG_MASK) == want) break;
                                if ((spin & 63) == 0 && dev::globaltimer() - start > dev::SPIN_LIMIT_NS) {
                                    dev::raise_error(a.err, dev::ERR_LOOKBACK_TIMEOUT);
                                    s_abort = 1;
                                    x = FLAG_PRE << 62;  // stop walking
                                    break;
                                }
                                __nanosleep(spin < 16 ? 32 : 128);
                            }
                        }
                        excl += (uint32_t)x;
                        if ((x >> 62) == FLAG_PRE) done = true;
                    }
                    k -= LBW;
                    if (k < 0) done = true;
                }
                dev::st_relaxed(&my_status[tid], pack_status(FLAG_PRE, seq0 + t, excl + agg));
            }
            s_bin_off[tid] = s_bin_start[tid] + excl - s_local[tid];
        }
        __syncthreads();

        // Write the locally sorted tile (runs of equal digits go to
        // consecutive addresses); unstaged, the next tile's index is fetched
        // meanwhile. After a timed-out wait the offsets are unknown: nothing
        // is written.
        if (!STAGED && tid == 0) s_stage_tile[0] = take();
        const uint32_t limit = s_abort ? 0u : valid;
        if (limit == (uint32_t)TILE) {
            uint32_t o[ITEMS];
            if constexpr (PACK) {
#pragma unroll
                for (int i = 0; i < ITEMS; ++i) {
                    const uint2 kv = reinterpret_cast<const uint2*>(s_keys)[tid + i * THREADS];
                    key[i] = (K)kv.x;
                    val[i] = kv.y;
                }
            } else {
#pragma unroll
                for (int i = 0; i < ITEMS; ++i) key[i] = s_keys[tid + i * THREADS];
                if (HAS_V) {
#pragma unroll
                    for (int i = 0; i < ITEMS; ++i) val[i] = s_vals[tid + i * THREADS];
                }
            }
#pragma unroll
            for (int i = 0; i < ITEMS; ++i) o[i] = s_bin_off[digit(key[i])] + tid + i * THREADS;
#pragma unroll
            for (int i = 0; i < ITEMS; ++i) {
                if (o[i] < n) {
                    dst_k[o[i]] = key[i];
                    if (HAS_V) dst_v[o[i]] = val[i];
                }
            }
        } else {
            for (uint32_t j = tid; j < limit; j += THREADS) {
                const K kk = PACK ? (K)reinterpret_cast<const uint2*>(s_keys)[j].x : s_keys[j];
                const uint32_t o = s_bin_off[digit(kk)] + j;
                if (o < n) {
                    dst_k[o] = kk;
                    if (HAS_V) dst_v[o] = PACK ? reinterpret_cast<const uint2*>(s_keys)[j].y : s_vals[j];
                }
            }
        }
        if (tid == 0) s_inflight[st] = 0;
        __syncthreads();
        if (STAGED) st ^= 1;
    }
    // A copy whose wait gave up may still be landing: let it finish (bounded)
    // before the CTA's shared memory is released.
    if (STAGED && tid == 0) {
        for (int q = 0; q < 2; ++q)
            if (s_inflight[q]) dev::mbar_wait_bounded(&s_bar[q], (parity >> q) & 1u);
    }
}

template <typename K, bool HAS_V, int THREADS, int ITEMS, bool IDENT, int MINB, int LBW, bool STAGED, bool PF, int BR,
          bool HALF, int PAD, bool PACK = false, bool TOFF = false>
__global__ void __launch_bounds__(THREADS, MINB) k_pass2(SortArgs<K> a, int slot)
{
    pass2_body<K, HAS_V, THREADS, ITEMS, IDENT, LBW, STAGED, PF, BR, HALF, PAD, PACK, TOFF>(a, slot);
}

// ---------------------------------------------------------------------------
// Host side
// ---------------------------------------------------------------------------
template <typename K> struct PassVariant {
    int threads, items;
    bool second;                             // second form (k_pass2)
    bool staged;                             // second form: next tile bulk-copied into a second stage
    void (*kernel)(SortArgs<K>, int);        // any key transform
    void (*kernel_ident)(SortArgs<K>, int);  // identity transform (unsigned ascending)
    // tile-offset form (second form): the per-tile digit counts pass run
    // before each digit pass (null otherwise)
    void (*hist)(SortArgs<K>, int) = nullptr;
    void (*hist_ident)(SortArgs<K>, int) = nullptr;
};

template <typename K, bool HAS_V> struct Variants;

// Variant 0 is the default when the tuning table has no entry; the order
// below puts the fastest measured shape first (keys only and key-value
// differ).
#define GBC_P1(K, HV, T, I, M) PassVariant<K>{T, I, false, false, &k_pass<K, HV, T, I, M>, &k_pass<K, HV, T, I, M>}
#define GBC_P1B(K, HV, T, I, B) \
    PassVariant<K>{T, I, false, false, &k_pass_mb<K, HV, T, I, false, B>, &k_pass_mb<K, HV, T, I, false, B>}
#define GBC_P2(K, HV, T, I, B, W, S, PF) GBC_P2XP(K, HV, T, I, B, W, S, PF, 0, false, 0)
#define GBC_P2R(K, HV, T, I, B, W, S, PF, BR) GBC_P2XP(K, HV, T, I, B, W, S, PF, BR, false, 0)
#define GBC_P2H(K, HV, T, I, B, W, S, PF, PD) GBC_P2XP(K, HV, T, I, B, W, S, PF, 0, true, PD)
#define GBC_P2XP(K, HV, T, I, B, W, S, PF, BR, HF, PD) GBC_P2XPK(K, HV, T, I, B, W, S, PF, BR, HF, PD, false)
#define GBC_P2XPK(K, HV, T, I, B, W, S, PF, BR, HF, PD, PK)                                                  \
    PassVariant<K>{T, I, true, S, &k_pass2<K, HV, T, I, false, B, W, S, PF, BR, HF, PD, PK>,              \
                   &k_pass2<K, HV, T, I, true, B, W, S, PF, BR, HF, PD, PK>}
#define GBC_P2T(K, HV, T, I, B, PF, HF, PD, PK)                                                           \
    PassVariant<K>{T, I, true, false, &k_pass2<K, HV, T, I, false, B, 4, false, PF, 0, HF, PD, PK, true>, \
                   &k_pass2<K, HV, T, I, true, B, 4, false, PF, 0, HF, PD, PK, true>,                      \
                   &k_tile_hist<K, false, T * I>, &k_tile_hist<K, true, T * I>}
template <bool HV> struct Variants<uint32_t, HV> {
    static constexpr int count = 13;
    // The tile-offset form (PAD 1), the default for keys without values from
    // 2^27 keys when the tuning table has no entry (2^28 uniform: 4.77 ms
    // against 5.04; 2^27: 2.45 against 2.53; smaller sizes and key-value
    // sorts are faster with the look-back).
    static constexpr int TILE_OFFSETS = 11;
    static PassVariant<uint32_t> get(int i)
    {
        static const PassVariant<uint32_t> v[count] = {
            // half-warp ranking, PAD 1 / PAD 0; key-value: the sorted tile as packed pairs
            GBC_P2XPK(uint32_t, HV, 256, 24, 2, 4, false, true, 0, true, 1, HV),
            GBC_P2XPK(uint32_t, HV, 256, 24, 2, 4, false, true, 0, true, 0, HV),
            GBC_P2H(uint32_t, HV, 256, 24, 2, 4, true, true, 1),
            HV ? GBC_P2(uint32_t, HV, 256, 24, 2, 4, false, true) : GBC_P2(uint32_t, HV, 256, 24, 2, 4, true, true),
            HV ? GBC_P2R(uint32_t, HV, 256, 24, 2, 4, false, true, 1) : GBC_P2R(uint32_t, HV, 256, 24, 2, 4, true, true, 1),
            HV ? GBC_P2R(uint32_t, HV, 256, 24, 2, 4, false, true, 2) : GBC_P2R(uint32_t, HV, 256, 24, 2, 4, true, true, 2),
            HV ? GBC_P2(uint32_t, HV, 256, 24, 2, 4, true, true) : GBC_P2(uint32_t, HV, 256, 24, 2, 4, false, true),
            GBC_P2(uint32_t, HV, 512, 12, 2, 4, false, true),
            GBC_P2(uint32_t, HV, 384, 16, 2, 4, false, true),
            GBC_P1(uint32_t, HV, 256, 16, false),
            GBC_P1B(uint32_t, HV, 256, 16, 3),
            GBC_P2T(uint32_t, HV, 256, 24, 2, true, true, 1, HV),
            GBC_P2T(uint32_t, HV, 256, 24, 2, true, true, 0, HV),
        };
        return v[std::min(std::max(i, 0), count - 1)];
    }
};
template <bool HV> struct Variants<uint64_t, HV> {
    static constexpr int count = 9;
    static PassVariant<uint64_t> get(int i)
    {
        static const PassVariant<uint64_t> v[count] = {
            HV ? GBC_P2H(uint64_t, HV, 256, 20, 2, 4, false, true, 1) : GBC_P2H(uint64_t, HV, 256, 24, 2, 4, false, true, 1),
            HV ? GBC_P2H(uint64_t, HV, 256, 20, 2, 4, false, true, 0) : GBC_P2H(uint64_t, HV, 256, 24, 2, 4, false, true, 0),
            HV ? GBC_P2(uint64_t, HV, 256, 20, 2, 4, false, true) : GBC_P2(uint64_t, HV, 256, 24, 2, 4, false, true),
            HV ? GBC_P2(uint64_t, HV, 256, 24, 2, 4, false, true) : GBC_P2(uint64_t, HV, 256, 20, 2, 4, false, true),
            GBC_P2(uint64_t, HV, 256, 16, 2, 4, false, true),
            GBC_P2(uint64_t, HV, 256, 12, 2, 4, false, true),
            GBC_P2(uint64_t, HV, 256, 16, 2, 1, false, true),
            GBC_P1(uint64_t, HV, 256, 12, false),
            GBC_P1(uint64_t, HV, 256, 12, true),
        };
        return v[std::min(std::max(i, 0), count - 1)];
    }
};
#undef GBC_P1
#undef GBC_P1B
#undef GBC_P2
#undef GBC_P2R
#undef GBC_P2H
#undef GBC_P2XP
#undef GBC_P2XPK
#undef GBC_P2T

template <typename K> std::size_t pass_smem(const PassVariant<K>& pv, bool has_v)
{
    const std::size_t tile = (std::size_t)pv.threads * pv.items;
    const std::size_t one = tile * sizeof(K) + (has_v ? tile * 4 : 0);  // a tile of keys (+ values)
    // counts and peer masks (+ 32 words of bank offset for half-warp ranking), or counts
    const std::size_t per_warp = pv.second ? RADIX * 8 + 128 : RADIX * 4;
    return (std::size_t)(pv.threads / 32) * per_warp + one * (pv.staged ? 2 : 1);
}

struct KernelInfo {
    int blocks_per_sm = 0;
};

template <typename F>
static int prepare_kernel(F* kernel, int threads, std::size_t smem, std::map<std::pair<int, const void*>, int>& cache,
                          std::mutex& m)
{
    // attributes and occupancy are per device
    int dev = 0;
    check_cuda(cudaGetDevice(&dev), "cudaGetDevice");
    const std::pair<int, const void*> key(dev, (const void*)kernel);
    std::lock_guard<std::mutex> lock(m);
    auto it = cache.find(key);
    if (it != cache.end()) return it->second;
    // always: static shared memory adds to the dynamic amount against the 48 KiB default
    if (smem > 0)
        check_cuda(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        (int)smem),
                   "cudaFuncSetAttribute");
    // These kernels use no L1-cached global data worth keeping: give the
    // unified L1/shared storage to shared memory so more CTAs fit per SM.
    check_cuda(cudaFuncSetAttribute(kernel, cudaFuncAttributePreferredSharedMemoryCarveout,
                                    (int)cudaSharedmemCarveoutMaxShared),
               "cudaFuncSetAttribute");
    int blocks = 0;
    check_cuda(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, kernel, threads, smem),
               "cudaOccupancyMaxActiveBlocksPerMultiprocessor");
    cache[key] = std::max(blocks, 1);
    return std::max(blocks, 1);
}

static std::map<std::pair<int, const void*>, int> g_occupancy;  // (device, kernel)
static std::mutex g_occupancy_mutex;

template <typename K, bool HAS_V>
static void run_sort(device_context& ctx, const K* in_k, K* out_k, const uint32_t* in_v,
                     uint32_t* out_v, std::size_t n, dev::KeyXform<K> xf, int variant)
{
    constexpr int P = Traits<K>::PASSES;
    PassVariant<K> pv = Variants<K, HAS_V>::get(variant);
    if (pass_smem<K>(pv, HAS_V) + 8192 > ctx.smem_optin) pv = Variants<K, HAS_V>::get(0);
    const uint32_t tile = (uint32_t)(pv.threads * pv.items);
    const uint32_t num_tiles = (uint32_t)((n + tile - 1) / tile);
    const bool in_place = (const void*)in_k == (const void*)out_k;

    temp_buffer alt_k(ctx.resource, n * sizeof(K));
    temp_buffer alt_v(ctx.resource, HAS_V ? n * sizeof(uint32_t) : 0);
    temp_buffer ctl(ctx.resource, sizeof(SortControl));
    check_cuda(cudaMemsetAsync(ctl.get(), 0, sizeof(SortControl), ctx.stream), "cudaMemsetAsync");

    SortArgs<K> a;
    a.in_keys = in_k;
    a.out_keys = out_k;
    a.alt_keys = alt_k.as<K>();
    a.in_vals = HAS_V ? in_v : nullptr;
    a.out_vals = HAS_V ? out_v : nullptr;
    a.alt_vals = HAS_V ? alt_v.as<uint32_t>() : nullptr;
    a.n = (uint32_t)n;
    a.in_place = in_place ? 1 : 0;
    a.xf = xf;
    a.ctl = ctl.as<SortControl>();
    a.ring = ctx.lookback_ring;
    a.seq0 = ctx.reserve_seq((uint64_t)P * num_tiles);
    a.num_tiles = num_tiles;
    a.err = ctx.d_error;
    a.tile_off = nullptr;
    a.chunk_off = nullptr;
    a.chunks = 0;
    a.tiles_per_chunk = 0;

    // K1
    constexpr int HT = 256, NSUB = 2;
    const std::size_t hsmem = (std::size_t)NSUB * P * RADIX * 4;
    const int hblocks = prepare_kernel(k_upfront<K, HT, NSUB>, HT, hsmem, g_occupancy, g_occupancy_mutex);
    const std::size_t hwork = (n + HT * 16 - 1) / (HT * 16);
    const int hgrid = (int)std::max<std::size_t>(1, std::min<std::size_t>(hwork, (std::size_t)ctx.sm_count * hblocks));
    {
        kernel_timer kt(ctx, "sort.upfront_histogram");
        k_upfront<K, HT, NSUB><<<hgrid, HT, hsmem, ctx.stream>>>(a);
        check_cuda(cudaGetLastError(), "radix sort histogram launch");
    }

    const int cgrid = (int)std::max<std::size_t>(1, std::min<std::size_t>((n + 255) / 256, (std::size_t)ctx.sm_count * 8));
    {
        kernel_timer kt(ctx, "sort.precopy");
        k_precopy<K><<<cgrid, 256, 0, ctx.stream>>>(a);
        check_cuda(cudaGetLastError(), "radix sort copy launch");
    }

    // K2 x P
    const std::size_t psmem = pass_smem<K>(pv, HAS_V);
    const bool ident = xf.a == 0 && xf.b == 0;
    auto* pk = ident ? pv.kernel_ident : pv.kernel;
    const int pblocks = prepare_kernel(pk, pv.threads, psmem, g_occupancy, g_occupancy_mutex);
    const int pgrid = (int)std::min<std::size_t>(num_tiles, (std::size_t)ctx.sm_count * pblocks);
    if (pv.hist == nullptr) {
        for (int s = 0; s < P; ++s) {
            kernel_timer kt(ctx, "sort.digit_pass");
            pk<<<pgrid, pv.threads, psmem, ctx.stream>>>(a, s);
            check_cuda(cudaGetLastError(), "radix sort pass launch");
        }
        return;
    }
    // Tile offsets: chunks of contiguous tiles, 2 per SM (fewer when the
    // tiles do not fill them), each counted by TH_SPLIT CTAs.
    const uint32_t want_chunks = (uint32_t)std::min<std::size_t>(num_tiles, (std::size_t)ctx.sm_count * 2);
    a.tiles_per_chunk = (num_tiles + want_chunks - 1) / want_chunks;
    a.chunks = (num_tiles + a.tiles_per_chunk - 1) / a.tiles_per_chunk;
    temp_buffer tile_off(ctx.resource, (std::size_t)num_tiles * RADIX * sizeof(uint32_t));
    temp_buffer chunk_off(ctx.resource, (std::size_t)a.chunks * RADIX * sizeof(uint32_t));
    a.tile_off = tile_off.as<uint32_t>();
    a.chunk_off = chunk_off.as<uint32_t>();
    check_cuda(cudaMemsetAsync(a.chunk_off, 0, (std::size_t)a.chunks * RADIX * sizeof(uint32_t), ctx.stream),
               "cudaMemsetAsync");
    auto* hk = ident ? pv.hist_ident : pv.hist;
    for (int s = 0; s < P; ++s) {
        {
            kernel_timer kt(ctx, "sort.tile_histogram");
            hk<<<a.chunks * TH_SPLIT, TH_THREADS, 0, ctx.stream>>>(a, s);
            check_cuda(cudaGetLastError(), "radix sort tile histogram launch");
        }
        {
            kernel_timer kt(ctx, "sort.tile_offsets");
            k_chunk_scan<K><<<RADIX, 1024, 0, ctx.stream>>>(a, s);
            check_cuda(cudaGetLastError(), "radix sort chunk scan launch");
            k_tile_offsets<K><<<a.chunks, TO_QUARTERS * RADIX, 0, ctx.stream>>>(a, s);
            check_cuda(cudaGetLastError(), "radix sort tile offsets launch");
        }
        {
            kernel_timer kt(ctx, "sort.digit_pass");
            pk<<<pgrid, pv.threads, psmem, ctx.stream>>>(a, s);
            check_cuda(cudaGetLastError(), "radix sort pass launch");
        }
    }
}

}  // namespace onesweep

int sort_variant_count(int key_bytes, bool has_values)
{
    using namespace onesweep;
    if (key_bytes == 4) return has_values ? Variants<uint32_t, true>::count : Variants<uint32_t, false>::count;
    return has_values ? Variants<uint64_t, true>::count : Variants<uint64_t, false>::count;
}

int sort_default_variant(int key_bytes, bool has_values, std::size_t n)
{
    using namespace onesweep;
    return key_bytes == 4 && !has_values && n >= (std::size_t(1) << 27) ? Variants<uint32_t, false>::TILE_OFFSETS : 0;
}

std::string sort_tuning_key(int key_bytes, bool has_values, std::size_t n)
{
    return std::string("sort:") + (key_bytes == 4 ? "u32" : "u64") + (has_values ? "kv" : "k") +
           ":" + tuning_table::size_class(n);
}

void radix_sort(device_context& ctx, const void* keys_in, void* keys_out, int key_bytes,
                int key_kind, const uint32_t* vals_in, uint32_t* vals_out, std::size_t n,
                bool descending)
{
    using namespace onesweep;
    if (key_bytes != 4 && key_bytes != 8)
        throw std::invalid_argument("sort: keys must be 32 or 64 bits");
    if (key_kind < 0 || key_kind > 2) throw std::invalid_argument("sort: unknown key kind");
    if (keys_in == nullptr || keys_out == nullptr) {
        if (n == 0) return;
        throw std::invalid_argument("sort: null keys");
    }
    if ((vals_in == nullptr) != (vals_out == nullptr))
        throw std::invalid_argument("sort: values need both an input and an output");
    ctx.activate();
    if (n <= 1) {
        if (n == 1 && keys_in != keys_out) {
            check_cuda(cudaMemcpyAsync(keys_out, keys_in, key_bytes, cudaMemcpyDeviceToDevice, ctx.stream),
                       "cudaMemcpyAsync");
            if (vals_in != nullptr && vals_in != vals_out)
                check_cuda(cudaMemcpyAsync(vals_out, vals_in, 4, cudaMemcpyDeviceToDevice, ctx.stream),
                           "cudaMemcpyAsync");
        }
        return;
    }
    check_size(n);
    const bool kv = vals_in != nullptr;
    launch_shape shape;
    if (!ctx.tuning.lookup(sort_tuning_key(key_bytes, kv, n), shape)) shape.variant = sort_default_variant(key_bytes, kv, n);
    if (key_bytes == 4) {
        const auto xf = dev::make_xform<uint32_t>(key_kind, descending);
        const auto* in = static_cast<const uint32_t*>(keys_in);
        auto* out = static_cast<uint32_t*>(keys_out);
        if (kv) run_sort<uint32_t, true>(ctx, in, out, vals_in, vals_out, n, xf, shape.variant);
        else run_sort<uint32_t, false>(ctx, in, out, nullptr, nullptr, n, xf, shape.variant);
    } else {
        const auto xf = dev::make_xform<uint64_t>(key_kind, descending);
        const auto* in = static_cast<const uint64_t*>(keys_in);
        auto* out = static_cast<uint64_t*>(keys_out);
        if (kv) run_sort<uint64_t, true>(ctx, in, out, vals_in, vals_out, n, xf, shape.variant);
        else run_sort<uint64_t, false>(ctx, in, out, nullptr, nullptr, n, xf, shape.variant);
    }
}

}  // namespace gbc
