// Batched segmented sort: every segment [offsets[i], offsets[i+1]) of a key
// (+ value) array is sorted independently and stably, for many segments of
// uneven length in one call whose launch sequence is fixed (every decision is
// made on the device, so the call can be captured in a CUDA graph).
//
// No reference counterpart: the reference sorts one array per call
// (detail::radix_sort, lib/src/Compute/Algorithm.cpp:453-527); sorting a batch
// there means one call per array. The semantics per segment are the same as
// that sort's: stable, the order-preserving key bijection of Algorithm.cpp:
// 459-469, optional 32-bit values moved alongside.
//
// Size classes (decided by k_seg_classify):
//   * tiny/small (<= WARP_CAP): one warp per segment, stable LSD radix sort in
//     warp-private shared memory over the digit positions that vary inside the
//     segment only;
//   * medium (<= cta_cap): one CTA per segment, the same LSD in CTA shared
//     memory;
//   * large: a batched onesweep: the tiles of all large segments form one
//     sequence, per-segment digit histograms come from one read of the keys,
//     and the decoupled look-back of each digit pass stops at the first tile
//     of its segment.
// The small/medium path and the large path are independent and run on two
// streams that fork from and join back to the context's stream.
#include <algorithm>
#include <cstring>
#include <string>

#include "device_common.cuh"
#include "runtime.hpp"
#include "segmented.hpp"
#include "sort_internal.hpp"

namespace gbc {
namespace seg {

using dev::FULL_MASK;
using onesweep::RADIX;
using onesweep::RING_TILES;

constexpr uint64_t FLAG_AGG = 1, FLAG_PRE = 2;
constexpr uint64_t TAG_MASK = (1ull << 30) - 1;
constexpr int WARP_CAP = 256;  // keys a warp sorts on its own
constexpr int SMALL_THREADS = 256;
constexpr int SMALL_WARPS = SMALL_THREADS / 32;

template <typename K> struct Traits;
template <> struct Traits<uint32_t> {
    static constexpr int PASSES = 4;
    static constexpr int CTA_CAP = 8192;
};
template <> struct Traits<uint64_t> {
    static constexpr int PASSES = 8;
    static constexpr int CTA_CAP = 6144;
};

__device__ __forceinline__ uint64_t pack_status(uint64_t flag, uint64_t seq, uint32_t v)
{
    return (flag << 62) | ((seq & TAG_MASK) << 32) | v;
}

//! Per-call control block (zeroed before each call).
struct SegControl {
    uint32_t n_warp, n_cta, n_large;  // list lengths
    uint32_t large_tiles;             // tiles of all large segments
    uint32_t warp_next, cta_next;     // work queue heads
    uint32_t tile_ctr[8];
    uint32_t n_sub_warp, n_sub_cta;      // sub-bucket list lengths (MSD route)
    uint32_t sub_warp_next, sub_cta_next;
    uint32_t barrier;                    // arrivals at the persistent batch's first grid barrier
    uint32_t large_barrier;              // ... and at those among its large-segment CTAs
};

template <typename K> struct SegArgs {
    const K* in_k;
    K* out_k;
    K* alt_k;
    const uint32_t* in_v;
    uint32_t* out_v;
    uint32_t* alt_v;
    const uint32_t* off;
    const uint8_t* skip;  // per segment: nonzero = already in order (in-place calls)
    uint32_t nseg;
    uint32_t cta_cap;
    dev::KeyXform<K> xf;
    SegControl* ctl;
    uint32_t* warp_list;
    uint32_t* cta_list;
    uint32_t* large_list;
    uint32_t* tile_begin;   // per large segment (n_large + 1)
    uint32_t* tile_seg;     // large tile -> index into large_list
    uint32_t* seg_hist;     // [large][PASSES][256]: bin start (absolute) per pass
    uint32_t max_large;
    uint32_t max_tiles;
    uint64_t* ring;
    uint64_t seq0;
    int* err;
    // MSD route of large segments: route[j] = the digit position of large
    // segment j's single pass, or NO_ROUTE for the full LSD passes; its
    // sub-buckets (begin, end pairs) are finished from alt into out by the
    // warp (<= WARP_CAP) and CTA (<= sub_cap) sorts.
    uint8_t* route;
    uint32_t* sub_warp_list;
    uint32_t* sub_cta_list;
    uint32_t max_sub;
    uint32_t sub_cap;
};

constexpr uint8_t NO_ROUTE = 0xFF;

// ---------------------------------------------------------------------------
// Classification
// ---------------------------------------------------------------------------
template <typename K> __device__ __forceinline__ void seg_classify(const SegArgs<K>& a)
{
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < a.nseg; i += stride) {
        const uint32_t b = a.off[i], e = a.off[i + 1];
        if (e < b) {
            dev::raise_error(a.err, dev::ERR_BAD_SEGMENT);
            continue;
        }
        const uint32_t len = e - b;
        if (len == 0 || (a.skip != nullptr && a.skip[i] != 0)) continue;
        if (len <= WARP_CAP) {
            a.warp_list[atomicAdd(&a.ctl->n_warp, 1u)] = i;
        } else if (len <= a.cta_cap) {
            a.cta_list[atomicAdd(&a.ctl->n_cta, 1u)] = i;
        } else {
            const uint32_t j = atomicAdd(&a.ctl->n_large, 1u);
            if (j < a.max_large) a.large_list[j] = i;
            else dev::raise_error(a.err, dev::ERR_BAD_SEGMENT);
        }
    }
}

template <typename K> __global__ void k_seg_classify(SegArgs<K> a) { seg_classify(a); }

// One CTA of NT threads: exclusive scan of the large segments' tile counts.
template <typename K, int TILE, int NT> __device__ __forceinline__ void seg_plan_scan(const SegArgs<K>& a)
{
    __shared__ uint32_t s_warp[NT / 32];
    __shared__ uint32_t s_carry;
    const uint32_t nl = min(a.ctl->n_large, a.max_large);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (threadIdx.x == 0) s_carry = 0;
    __syncthreads();
    for (uint32_t base = 0; base < nl; base += NT) {
        const uint32_t j = base + threadIdx.x;
        uint32_t cnt = 0;
        if (j < nl) {
            const uint32_t s = a.large_list[j];
            cnt = (a.off[s + 1] - a.off[s] + TILE - 1) / TILE;
        }
        uint32_t x = dev::warp_inclusive_scan(cnt, [](uint32_t p, uint32_t q) { return p + q; });
        if (lane == 31) s_warp[warp] = x;
        __syncthreads();
        uint32_t before = s_carry;
        for (int w = 0; w < warp; ++w) before += s_warp[w];
        if (j < nl) a.tile_begin[j] = before + x - cnt;
        __syncthreads();
        if (threadIdx.x == NT - 1) s_carry = before + x;
        __syncthreads();
    }
    const uint32_t total = min(s_carry, a.max_tiles);
    if (threadIdx.x == 0) {
        a.tile_begin[nl] = total;
        a.ctl->large_tiles = total;
    }
    __syncthreads();
}

// The tile -> segment map: the warps of the first `ctas` CTAs fill the tiles
// of one large segment at a time.
template <typename K> __device__ __forceinline__ void seg_plan_map(const SegArgs<K>& a, uint32_t ctas)
{
    const uint32_t nl = min(a.ctl->n_large, a.max_large);
    const uint32_t total = a.ctl->large_tiles;
    const int lane = threadIdx.x & 31;
    const uint32_t warps = ctas * (blockDim.x / 32);
    for (uint32_t j = blockIdx.x * (blockDim.x / 32) + (threadIdx.x >> 5); j < nl; j += warps) {
        const uint32_t t0 = a.tile_begin[j], t1 = min(a.tile_begin[j + 1], total);
        for (uint32_t t = t0 + lane; t < t1; t += 32) a.tile_seg[t] = j;
    }
}

template <typename K, int TILE> __global__ void __launch_bounds__(1024) k_seg_plan(SegArgs<K> a)
{
    seg_plan_scan<K, TILE, 1024>(a);
    seg_plan_map(a, gridDim.x);
}

// ---------------------------------------------------------------------------
// Shared-memory LSD sort of one segment by a group of GW warps (GW = 1: a
// warp on its own; GW = the CTA's warps: the whole CTA). Stable: items are ranked
// in index order (warp chunk, row, lane) and scattered by digit.
// ---------------------------------------------------------------------------
template <int GW> __device__ __forceinline__ void group_sync()
{
    if (GW == 1) __syncwarp();
    else __syncthreads();
}

// Ranking is by shared-memory peer masks, as in the digit pass: each lane ORs
// its bit into its digit's mask word (GW x 256 words in `masks`, all zero
// between rows), reads the word back (its peers) and the warp's count of the
// digit so far; the lowest peer stores the new count and clears the mask.
// (__match_any_sync ranked the same rows about 1.7x slower on this GPU.)
template <typename K, bool HAS_V, int GW>
__device__ void group_sort(K* k0, K* k1, uint32_t* v0, uint32_t* v1, uint32_t* rd, uint32_t* hist,
                           uint32_t* masks, uint32_t* scratch, uint32_t len, dev::KeyXform<K> xf, int gw, int lane,
                           bool& in_k1)
{
    constexpr int P = Traits<K>::PASSES;
    // Which digit positions vary inside the segment.
    K diff = 0;
    const K first = xf(k0[0]);
    for (uint32_t i = gw * 32 + lane; i < len; i += GW * 32) diff |= xf(k0[i]) ^ first;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) diff |= __shfl_xor_sync(FULL_MASK, diff, o);
    if (GW > 1) {
        // combine the warps' masks (scratch holds 2 x 32 words)
        if (lane == 0) {
            scratch[gw * 2] = (uint32_t)diff;
            scratch[gw * 2 + 1] = (uint32_t)((uint64_t)diff >> 32);
        }
        __syncthreads();
        uint64_t all = 0;
        for (int w = 0; w < GW; ++w) all |= (uint64_t)scratch[w * 2] | ((uint64_t)scratch[w * 2 + 1] << 32);
        diff = (K)all;
        __syncthreads();
    }
    const uint32_t chunk = ((len + GW * 32 - 1) / (GW * 32)) * 32;  // items per warp, whole rows
    const uint32_t rows = chunk / 32;
    in_k1 = false;
    for (int p = 0; p < P; ++p) {
        if ((((uint64_t)diff >> (8 * p)) & 0xFF) == 0) continue;
        const int shift = 8 * p;
        for (int i = (GW > 1 ? threadIdx.x : lane); i < GW * RADIX; i += GW * 32) hist[i] = 0;
        group_sync<GW>();
        uint32_t* wh = hist + gw * RADIX;
        uint32_t* wm = masks + gw * RADIX;
        const uint32_t lt = dev::lanemask_lt();
        for (uint32_t r = 0; r < rows; ++r) {
            const uint32_t idx = gw * chunk + r * 32 + lane;
            const bool valid = idx < len;
            // padding ranks in bin 255 (counted there, never placed)
            const uint32_t d = valid ? (uint32_t)(xf(k0[idx]) >> shift) & 0xFFu : 0xFFu;
            atomicOr(&wm[d], 1u << lane);
            __syncwarp();
            const uint32_t peers = wm[d];
            const uint32_t before = wh[d];
            __syncwarp();
            const uint32_t lower = peers & lt;
            if (lower == 0) {
                wh[d] = before + __popc(peers);
                wm[d] = 0;
            }
            __syncwarp();
            if (valid) rd[idx] = ((before + __popc(lower)) << 8) | d;
        }
        group_sync<GW>();
        // digit starts and per-warp offsets
        if (GW == 1) {
            uint32_t c[8], s = 0;
#pragma unroll
            for (int q = 0; q < 8; ++q) {
                c[q] = hist[lane * 8 + q];
                s += c[q];
            }
            const uint32_t incl = dev::warp_inclusive_scan(s, [](uint32_t x, uint32_t y) { return x + y; });
            uint32_t run = incl - s;
#pragma unroll
            for (int q = 0; q < 8; ++q) {
                hist[lane * 8 + q] = run;
                run += c[q];
            }
        } else {
            uint32_t count = 0;
            if (threadIdx.x < RADIX) {
                for (int w = 0; w < GW; ++w) {
                    const uint32_t c = hist[w * RADIX + threadIdx.x];
                    hist[w * RADIX + threadIdx.x] = count;
                    count += c;
                }
            }
            const uint32_t start = dev::bins_exclusive_sum(count, scratch + 64);
            if (threadIdx.x < RADIX)
                for (int w = 0; w < GW; ++w) hist[w * RADIX + threadIdx.x] += start;
        }
        group_sync<GW>();
        for (uint32_t r = 0; r < rows; ++r) {
            const uint32_t idx = gw * chunk + r * 32 + lane;
            if (idx < len) {
                const uint32_t x = rd[idx];
                const uint32_t pos = wh[x & 0xFF] + (x >> 8);
                k1[pos] = k0[idx];
                if (HAS_V) v1[pos] = v0[idx];
            }
        }
        group_sync<GW>();
        K* tk = k0;
        k0 = k1;
        k1 = tk;
        uint32_t* tv = v0;
        v0 = v1;
        v1 = tv;
        in_k1 = !in_k1;
    }
}

// SUB: the MSD route's sub-buckets (begin, end pairs, read from alt) instead
// of whole segments (read from the input).
template <typename K, bool HAS_V, bool SUB> __device__ __forceinline__ void seg_small_warp(const SegArgs<K>& a)
{
    extern __shared__ __align__(16) unsigned char smem[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    constexpr std::size_t per_warp =
        2 * WARP_CAP * sizeof(K) + (HAS_V ? 2 * WARP_CAP * 4 : 0) + WARP_CAP * 4 + 2 * RADIX * 4;
    unsigned char* base = smem + warp * per_warp;
    K* k0 = reinterpret_cast<K*>(base);
    K* k1 = k0 + WARP_CAP;
    uint32_t* v0 = reinterpret_cast<uint32_t*>(k1 + WARP_CAP);
    uint32_t* v1 = v0 + (HAS_V ? WARP_CAP : 0);
    uint32_t* rd = v1 + (HAS_V ? WARP_CAP : 0);
    uint32_t* hist = rd + WARP_CAP;
    uint32_t* masks = hist + RADIX;
    for (int i = lane; i < RADIX; i += 32) masks[i] = 0;
    __syncwarp();
    const uint32_t total = SUB ? min(a.ctl->n_sub_warp, a.max_sub) : a.ctl->n_warp;
    const K* src_k = SUB ? a.alt_k : a.in_k;
    const uint32_t* src_v = SUB ? a.alt_v : a.in_v;
    for (;;) {
        uint32_t w = 0;
        if (lane == 0) w = atomicAdd(SUB ? &a.ctl->sub_warp_next : &a.ctl->warp_next, 1u);
        w = __shfl_sync(FULL_MASK, w, 0);
        if (w >= total) break;
        uint32_t b, len;
        if (SUB) {
            b = a.sub_warp_list[2 * w];
            len = a.sub_warp_list[2 * w + 1] - b;
        } else {
            const uint32_t s = a.warp_list[w];
            b = a.off[s];
            len = a.off[s + 1] - b;
        }
        for (uint32_t i = lane; i < len; i += 32) {
            k0[i] = src_k[b + i];
            if (HAS_V) v0[i] = src_v[b + i];
        }
        __syncwarp();
        bool flipped = false;
        if (len > 1) group_sort<K, HAS_V, 1>(k0, k1, v0, v1, rd, hist, masks, nullptr, len, a.xf, 0, lane, flipped);
        const K* rk = flipped ? k1 : k0;
        const uint32_t* rv = flipped ? v1 : v0;
        for (uint32_t i = lane; i < len; i += 32) {
            a.out_k[b + i] = rk[i];
            if (HAS_V) a.out_v[b + i] = rv[i];
        }
        __syncwarp();
    }
}

template <typename K, bool HAS_V, bool SUB>
__global__ void __launch_bounds__(SMALL_THREADS) k_seg_small_warp(SegArgs<K> a)
{
    seg_small_warp<K, HAS_V, SUB>(a);
}

// THREADS: 256, or 512 where the shared memory allows (twice the warps in
// flight on the SM for the same shared-memory tile).
template <typename K, bool HAS_V, bool SUB, int THREADS = SMALL_THREADS>
__device__ __forceinline__ void seg_small_cta(const SegArgs<K>& a)
{
    constexpr int WARPS = THREADS / 32;
    static_assert(THREADS % 32 == 0 && THREADS >= RADIX && WARPS <= 32, "one thread per bin; scratch holds 32 warps");
    extern __shared__ __align__(16) unsigned char smem[];
    const uint32_t cap = SUB ? a.sub_cap : a.cta_cap;
    K* k0 = reinterpret_cast<K*>(smem);
    K* k1 = k0 + cap;
    uint32_t* v0 = reinterpret_cast<uint32_t*>(k1 + cap);
    uint32_t* v1 = v0 + (HAS_V ? cap : 0);
    uint32_t* rd = v1 + (HAS_V ? cap : 0);
    uint32_t* hist = rd + cap;
    uint32_t* masks = hist + WARPS * RADIX;
    for (int i = threadIdx.x; i < WARPS * RADIX; i += THREADS) masks[i] = 0;
    __shared__ uint32_t scratch[64 + 8];
    __shared__ uint32_t s_work;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint32_t total = SUB ? min(a.ctl->n_sub_cta, a.max_sub) : a.ctl->n_cta;
    const K* src_k = SUB ? a.alt_k : a.in_k;
    const uint32_t* src_v = SUB ? a.alt_v : a.in_v;
    for (;;) {
        if (threadIdx.x == 0) s_work = atomicAdd(SUB ? &a.ctl->sub_cta_next : &a.ctl->cta_next, 1u);
        __syncthreads();
        const uint32_t w = s_work;
        if (w >= total) break;
        uint32_t b, len;
        if (SUB) {
            b = a.sub_cta_list[2 * w];
            len = a.sub_cta_list[2 * w + 1] - b;
        } else {
            const uint32_t s = a.cta_list[w];
            b = a.off[s];
            len = a.off[s + 1] - b;
        }
        for (uint32_t i = threadIdx.x; i < len; i += THREADS) {
            k0[i] = src_k[b + i];
            if (HAS_V) v0[i] = src_v[b + i];
        }
        __syncthreads();
        bool flipped = false;
        group_sort<K, HAS_V, WARPS>(k0, k1, v0, v1, rd, hist, masks, scratch, len, a.xf, warp, lane, flipped);
        const K* rk = flipped ? k1 : k0;
        const uint32_t* rv = flipped ? v1 : v0;
        for (uint32_t i = threadIdx.x; i < len; i += THREADS) {
            a.out_k[b + i] = rk[i];
            if (HAS_V) a.out_v[b + i] = rv[i];
        }
        __syncthreads();
    }
}

template <typename K, bool HAS_V, bool SUB, int THREADS>
__global__ void __launch_bounds__(THREADS) k_seg_small_cta(SegArgs<K> a)
{
    seg_small_cta<K, HAS_V, SUB, THREADS>(a);
}

//! Shared memory of the one-CTA sort: two copies of keys (and values) and a
//! packed rank per element, then a histogram and a peer-mask array per warp.
template <typename K, bool HAS_V> constexpr std::size_t cta_sort_smem(uint32_t cap, int threads)
{
    return (std::size_t)cap * (2 * sizeof(K) + (HAS_V ? 8 : 0) + 4) + 2 * (std::size_t)(threads / 32) * RADIX * 4;
}

// ---------------------------------------------------------------------------
// Large segments: per-segment digit histograms -> absolute bin starts, in
// three steps over the large-segment tile sequence that the passes use (so
// a long segment is spread over many CTAs): zero the rows of the large
// segments present; count runs of HIST_TILES tiles in shared memory and add
// the counts to the segment's row whenever the segment changes or the run
// ends; turn every row into absolute bin starts.
// ---------------------------------------------------------------------------
constexpr uint32_t HIST_TILES = 8;

template <typename K> __device__ __forceinline__ void seg_large_zero(const SegArgs<K>& a, uint32_t ctas)
{
    constexpr int P = Traits<K>::PASSES;
    const uint32_t nl = min(a.ctl->n_large, a.max_large);
    const std::size_t words = (std::size_t)nl * P * RADIX;
    const std::size_t stride = (std::size_t)ctas * blockDim.x;
    for (std::size_t i = (std::size_t)blockIdx.x * blockDim.x + threadIdx.x; i < words; i += stride) a.seg_hist[i] = 0;
}

template <typename K> __global__ void k_seg_large_zero(SegArgs<K> a) { seg_large_zero(a, gridDim.x); }


template <typename K, int TILE> __device__ __forceinline__ void seg_large_count(const SegArgs<K>& a, uint32_t ctas)
{
    constexpr int P = Traits<K>::PASSES;
    constexpr int BATCH = 8;  // keys in flight per thread
    __shared__ uint32_t sh[2][P * RADIX];  // two copies (warp parity)
    uint32_t* my = sh[(threadIdx.x >> 5) & 1];
    const uint32_t total = a.ctl->large_tiles;
    const uint32_t runs = (total + HIST_TILES - 1) / HIST_TILES;
    auto flush = [&](uint32_t j) {  // adds the counts to row j and clears them
        __syncthreads();
        uint32_t* row = a.seg_hist + (std::size_t)j * P * RADIX;
        for (int i = threadIdx.x; i < P * RADIX; i += 256) {
            const uint32_t v = sh[0][i] + sh[1][i];
            if (v != 0) atomicAdd(&row[i], v);
            sh[0][i] = 0;
            sh[1][i] = 0;
        }
        __syncthreads();
    };
    for (int i = threadIdx.x; i < 2 * P * RADIX; i += 256) (&sh[0][0])[i] = 0;
    __syncthreads();
    for (uint32_t r = blockIdx.x; r < runs; r += ctas) {
        const uint32_t t0 = r * HIST_TILES, t1 = min(total, t0 + HIST_TILES);
        uint32_t j = a.tile_seg[t0];
        for (uint32_t t = t0; t < t1; ++t) {
            const uint32_t jt = a.tile_seg[t];  // the same for every thread
            if (jt != j) {
                flush(j);
                j = jt;
            }
            const uint32_t s = a.large_list[jt];
            const uint32_t b = a.off[s] + (t - a.tile_begin[jt]) * TILE;
            const uint32_t e = min(a.off[s + 1], b + TILE);
            for (uint32_t i0 = b; i0 < e; i0 += 256 * BATCH) {
                K k[BATCH];
#pragma unroll
                for (int q = 0; q < BATCH; ++q) {
                    const uint32_t i = i0 + q * 256 + threadIdx.x;
                    k[q] = i < e ? a.in_k[i] : K(0);
                }
#pragma unroll
                for (int q = 0; q < BATCH; ++q) {
                    if (i0 + q * 256 + threadIdx.x >= e) break;
                    const K x = a.xf(k[q]);
#pragma unroll
                    for (int p = 0; p < P; ++p) atomicAdd(&my[p * RADIX + (uint32_t)((x >> (8 * p)) & 0xFF)], 1u);
                }
            }
        }
        flush(j);
    }
}

template <typename K, int TILE> __global__ void __launch_bounds__(256) k_seg_large_count(SegArgs<K> a)
{
    seg_large_count<K, TILE>(a, gridDim.x);
}


template <typename K> __device__ __forceinline__ void seg_large_starts(const SegArgs<K>& a, uint32_t ctas)
{
    constexpr int P = Traits<K>::PASSES;
    __shared__ uint32_t s_scratch[8];
    const uint32_t nl = min(a.ctl->n_large, a.max_large);
    for (uint32_t j = blockIdx.x; j < nl; j += ctas) {
        const uint32_t b = a.off[a.large_list[j]];
        for (int p = 0; p < P; ++p) {
            uint32_t* row = a.seg_hist + ((std::size_t)j * P + p) * RADIX;
            const uint32_t ex = dev::bins_exclusive_sum(row[threadIdx.x], s_scratch);
            row[threadIdx.x] = b + ex;
        }
    }
}

template <typename K> __global__ void __launch_bounds__(256) k_seg_large_starts(SegArgs<K> a)
{
    seg_large_starts(a, gridDim.x);
}


// Per large segment (one CTA, thread d = bin d): the highest digit position
// that varies inside the segment (its bins are not all in one) and, when
// every bin there holds at most sub_cap keys, the MSD route: one pass on that
// digit partitions the segment into its bins (stable), which become
// sub-buckets for the warp and CTA sorts; else the full LSD passes. The bin
// starts in seg_hist are absolute, from k_seg_large_starts.
template <typename K> __device__ __forceinline__ void seg_route(const SegArgs<K>& a, uint32_t ctas)
{
    constexpr int P = Traits<K>::PASSES;
    __shared__ uint32_t s_max[8];
    __shared__ int s_top;
    const uint32_t nl = min(a.ctl->n_large, a.max_large);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (uint32_t j = blockIdx.x; j < nl; j += ctas) {
        const uint32_t s = a.large_list[j];
        const uint32_t segb = a.off[s], sege = a.off[s + 1], len = sege - segb;
        auto bin_size = [&](int p, uint32_t d) {
            const uint32_t* row = a.seg_hist + ((size_t)j * P + p) * RADIX;
            return (d == RADIX - 1 ? sege : row[d + 1]) - row[d];
        };
        if (threadIdx.x == 0) s_top = -1;
        __syncthreads();
        for (int p = P - 1; p >= 0; --p) {
            // a position varies when no bin holds the whole segment
            const bool whole = bin_size(p, threadIdx.x) == len;
            if (__syncthreads_or(whole) == 0) {
                if (threadIdx.x == 0) s_top = p;
                break;
            }
        }
        __syncthreads();
        const int top = s_top;
        uint32_t size = top >= 0 ? bin_size(top, threadIdx.x) : len;
        uint32_t m = size;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_xor_sync(FULL_MASK, m, o));
        if (lane == 0) s_max[warp] = m;
        __syncthreads();
        uint32_t biggest = 0;
#pragma unroll
        for (int w = 0; w < 8; ++w) biggest = max(biggest, s_max[w]);
        const bool msd = top >= 0 && biggest <= a.sub_cap;
        if (threadIdx.x == 0) a.route[j] = msd ? (uint8_t)top : NO_ROUTE;
        if (msd && size != 0) {  // a one-key bucket goes to the warp sort, which copies it
            const uint32_t b = a.seg_hist[((size_t)j * P + top) * RADIX + threadIdx.x];
            if (size <= (uint32_t)WARP_CAP) {
                const uint32_t q = atomicAdd(&a.ctl->n_sub_warp, 1u);
                if (q < a.max_sub) a.sub_warp_list[2 * q] = b, a.sub_warp_list[2 * q + 1] = b + size;
            } else {
                const uint32_t q = atomicAdd(&a.ctl->n_sub_cta, 1u);
                if (q < a.max_sub) a.sub_cta_list[2 * q] = b, a.sub_cta_list[2 * q + 1] = b + size;
            }
        }
        __syncthreads();
    }
}

template <typename K> __global__ void __launch_bounds__(256) k_seg_route(SegArgs<K> a) { seg_route(a, gridDim.x); }


// One digit pass over every large segment's tiles (cf. onesweep::k_pass2:
// shared-memory peer-mask ranking, place offsets folded into the per-warp
// counts, a look-back reading LBW predecessors per round trip, which stops at
// the segment's first tile (it publishes an inclusive count), an L2 prefetch
// of the tile a grid ahead and an unrolled write-out of full tiles).
constexpr int LARGE_PAD = 1;  // words between the half-warp count arrays of the large pass

template <typename K, bool HAS_V, int THREADS, int ITEMS, int LBW>
__device__ __forceinline__ void seg_large_pass(const SegArgs<K>& a, int slot, uint32_t ctas)
{
    constexpr int P = Traits<K>::PASSES;
    constexpr int WARPS = THREADS / 32;
    constexpr int TILE = THREADS * ITEMS;
    const uint32_t num_tiles = a.ctl->large_tiles;
    const int shift = 8 * slot;
    // pass s writes out when (P - 1 - s) is even; P is even, so pass 0 reads
    // the input and writes the scratch buffer.
    const bool dst_out = ((P - 1 - slot) & 1) == 0;
    K* dst_k = dst_out ? a.out_k : a.alt_k;
    uint32_t* dst_v = dst_out ? a.out_v : a.alt_v;
    const K* src_k = slot == 0 ? a.in_k : (dst_out ? a.alt_k : a.out_k);
    const uint32_t* src_v = slot == 0 ? a.in_v : (dst_out ? a.alt_v : a.out_v);
    const bool aligned_src =
        ((reinterpret_cast<uintptr_t>(src_k) | (HAS_V ? reinterpret_cast<uintptr_t>(src_v) : 0)) & 15) == 0;

    extern __shared__ __align__(16) unsigned char smem[];
    // Keys are ranked by half-warps (rows of 16, each half-warp a contiguous
    // run of the tile): one word per half-warp and digit holds the count
    // (high 16 bits) and the current row's peer mask (low 16 bits).
    // A half-warp's words sit LARGE_PAD banks from its partner's, so equal
    // digits in the two halves of a row do not meet in one bank.
    constexpr int GROUPS = 2 * WARPS, GSTRIDE = RADIX + LARGE_PAD;
    static_assert(16 * ITEMS < (1 << 16), "half-warp counts are 16-bit");
    uint32_t* warp_hist = reinterpret_cast<uint32_t*>(smem);  // GROUPS x GSTRIDE: counts, then place offsets
    K* s_keys = reinterpret_cast<K*>(warp_hist + GROUPS * GSTRIDE);
    uint32_t* s_vals = reinterpret_cast<uint32_t*>(s_keys + TILE);
    __shared__ uint32_t s_bin_off[RADIX], s_local[RADIX];
    __shared__ uint32_t s_scratch[8];
    __shared__ uint32_t s_tile;
    __shared__ int s_abort;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int grp = 2 * warp + (lane >> 4), gl = lane & 15;
    if (tid == 0) s_abort = 0;
    const uint64_t seq0 = a.seq0 + (uint64_t)slot * a.max_tiles;
    auto digit = [&](K k) -> uint32_t { return (uint32_t)(a.xf(k) >> shift) & 0xFFu; };

    for (;;) {
        if (tid == 0) {
            s_tile = atomicAdd(&a.ctl->tile_ctr[slot], 1u);
            // L2 prefetch of the tile a grid further on in the tile sequence
            // (from where this pass reads it, if it takes part)
            const uint32_t ahead = s_tile + ctas;
            if (aligned_src && ahead < num_tiles) {
                const uint32_t ja = a.tile_seg[ahead];
                const uint8_t ra = a.route[ja];
                const uint32_t sa = a.large_list[ja];
                const uint32_t ba = a.off[sa] + (ahead - a.tile_begin[ja]) * TILE;
                const K* pk = ra == NO_ROUTE ? src_k : a.in_k;
                const uint32_t* pv = ra == NO_ROUTE ? src_v : a.in_v;
                if ((ra == NO_ROUTE || ra == slot) && ba + TILE <= a.off[sa + 1] && (ba % (16 / sizeof(K))) == 0) {
                    dev::prefetch_l2(pk + ba, TILE * sizeof(K));
                    if (HAS_V && (ba & 3) == 0) dev::prefetch_l2(pv + ba, TILE * 4);
                }
            }
        }
        for (int i = tid; i < GROUPS * GSTRIDE; i += THREADS) warp_hist[i] = 0;
        __syncthreads();
        const uint32_t t = s_tile;
        if (t >= num_tiles) break;
        const uint32_t j = a.tile_seg[t];
        // a segment on the MSD route takes part in its one pass only, reading
        // the input and writing the scratch buffer (its sub-buckets are then
        // finished from there); its tiles publish nothing in the other passes,
        // and no tile of another segment looks back into it
        const uint8_t rt = a.route[j];
        if (rt != NO_ROUTE && rt != slot) {
            __syncthreads();  // every thread has read s_tile before thread 0 takes the next tile
            continue;
        }
        const K* tsrc_k = rt == NO_ROUTE ? src_k : a.in_k;
        const uint32_t* tsrc_v = rt == NO_ROUTE ? src_v : a.in_v;
        K* tdst_k = rt == NO_ROUTE ? dst_k : a.alt_k;
        uint32_t* tdst_v = rt == NO_ROUTE ? dst_v : a.alt_v;
        const uint32_t s = a.large_list[j];
        const uint32_t segb = a.off[s], sege = a.off[s + 1];
        const uint32_t lt = t - a.tile_begin[j];
        const uint32_t tile_base = segb + lt * TILE;
        const uint32_t valid = min((uint32_t)TILE, sege - tile_base);
        const bool first = lt == 0;

        const uint32_t wbase = tile_base + grp * 16 * ITEMS + gl;
        K key[ITEMS];
        uint32_t rd[ITEMS];
        uint32_t val[HAS_V ? ITEMS : 1];
        if (valid == (uint32_t)TILE) {
#pragma unroll
            for (int i = 0; i < ITEMS; ++i) key[i] = tsrc_k[wbase + i * 16];
            if (HAS_V) {
#pragma unroll
                for (int i = 0; i < ITEMS; ++i) val[i] = tsrc_v[wbase + i * 16];
            }
#pragma unroll
            for (int i = 0; i < ITEMS; ++i) rd[i] = digit(key[i]);
        } else {
#pragma unroll
            for (int i = 0; i < ITEMS; ++i) {
                const uint32_t idx = wbase + i * 16;
                const bool in = idx < sege;
                key[i] = in ? tsrc_k[idx] : K(0);
                if (HAS_V) val[i] = in ? tsrc_v[idx] : 0u;
                rd[i] = in ? digit(key[i]) : 0xFFu;  // padding ranks last
            }
        }

        uint32_t* wh = warp_hist + grp * GSTRIDE;
        const uint32_t hbit = 1u << gl, hlt = hbit - 1u;
#pragma unroll
        for (int i = 0; i < ITEMS; ++i) {
            const uint32_t d = rd[i];
            atomicOr(&wh[d], hbit);
            __syncwarp();
            const uint32_t x = wh[d];
            __syncwarp();
            const uint32_t peers = x & 0xFFFFu, before = x >> 16;
            if ((peers & hlt) == 0) wh[d] = (before + __popc(peers)) << 16;  // the new count; the mask cleared
            __syncwarp();
            rd[i] = ((before + __popc(peers & hlt)) << 8) | d;
        }
        __syncthreads();

        uint32_t count = 0;
        if (tid < RADIX) {
#pragma unroll
            for (int w = 0; w < GROUPS; ++w) {
                const uint32_t c = warp_hist[w * GSTRIDE + tid] >> 16;
                warp_hist[w * GSTRIDE + tid] = count;
                count += c;
            }
        }
        uint32_t agg = count;
        if (tid == RADIX - 1) agg -= (uint32_t)TILE - valid;
        uint64_t* my_status = a.ring + ((seq0 + t) & (RING_TILES - 1)) * RADIX;
        if (tid < RADIX) dev::st_relaxed(&my_status[tid], pack_status(first ? FLAG_PRE : FLAG_AGG, seq0 + t, agg));
        const uint32_t local = dev::bins_exclusive_sum(count, s_scratch);
        if (tid < RADIX) {
            s_local[tid] = local;
#pragma unroll
            for (int w = 0; w < GROUPS; ++w) warp_hist[w * GSTRIDE + tid] += local;
        }
        __syncthreads();
#pragma unroll
        for (int i = 0; i < ITEMS; ++i) {
            const uint32_t pos = warp_hist[grp * GSTRIDE + (rd[i] & 0xFFu)] + (rd[i] >> 8);
            s_keys[pos] = key[i];
            if (HAS_V) s_vals[pos] = val[i];
        }
        if (tid < RADIX) {
            uint32_t excl = 0;
            if (!first) {
                int64_t k = (int64_t)t - 1;
                bool done = false;
                while (!done) {
                    uint64_t w[LBW];
#pragma unroll
                    for (int q = 0; q < LBW; ++q)
                        if (k - q >= 0)
                            w[q] = dev::ld_relaxed(a.ring + ((seq0 + (uint64_t)(k - q)) & (RING_TILES - 1)) * RADIX +
                                                   tid);
#pragma unroll
                    for (int q = 0; q < LBW; ++q) {
                        if (done || k - q < 0) break;
                        const uint64_t seq = seq0 + (uint64_t)(k - q);
                        const uint64_t want = seq & TAG_MASK;
                        uint64_t x = w[q];
                        if ((x >> 62) == 0 || ((x >> 32) & TAG_MASK) != want) {
                            const uint64_t* pw = a.ring + (seq & (RING_TILES - 1)) * RADIX + tid;
                            const unsigned long long start = dev::globaltimer();
                            for (uint32_t spin = 1;; ++spin) {
                                x = dev::ld_relaxed(pw);
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
            s_bin_off[tid] = a.seg_hist[((size_t)j * P + slot) * RADIX + tid] + excl - s_local[tid];
        }
        __syncthreads();
        const uint32_t limit = s_abort ? 0u : valid;
        if (limit == (uint32_t)TILE) {
            uint32_t o[ITEMS];
#pragma unroll
            for (int i = 0; i < ITEMS; ++i) key[i] = s_keys[tid + i * THREADS];
            if (HAS_V) {
#pragma unroll
                for (int i = 0; i < ITEMS; ++i) val[i] = s_vals[tid + i * THREADS];
            }
#pragma unroll
            for (int i = 0; i < ITEMS; ++i) o[i] = s_bin_off[digit(key[i])] + tid + i * THREADS;
#pragma unroll
            for (int i = 0; i < ITEMS; ++i) {
                if (o[i] >= segb && o[i] < sege) {
                    tdst_k[o[i]] = key[i];
                    if (HAS_V) tdst_v[o[i]] = val[i];
                }
            }
        } else {
            for (uint32_t q = tid; q < limit; q += THREADS) {
                const K kk = s_keys[q];
                const uint32_t o = s_bin_off[digit(kk)] + q;
                if (o >= segb && o < sege) {
                    tdst_k[o] = kk;
                    if (HAS_V) tdst_v[o] = s_vals[q];
                }
            }
        }
        __syncthreads();
    }
}

template <typename K, bool HAS_V, int THREADS, int ITEMS, int MINB, int LBW>
__global__ void __launch_bounds__(THREADS, MINB) k_seg_large_pass(SegArgs<K> a, int slot)
{
    seg_large_pass<K, HAS_V, THREADS, ITEMS, LBW>(a, slot, gridDim.x);
}

// ---------------------------------------------------------------------------
// The whole batch in one persistent launch: every phase above in order, with
// a grid barrier wherever a phase reads what an earlier one wrote (the launch
// is cooperative, so every CTA is resident). After classification the first
// large_ctas CTAs take the large-segment phases -- the plan's scan (CTA 0)
// while they zero the histogram rows; the tile map; the histogram count; the
// bin starts; [the MSD route]; each digit pass; [the MSD route's bucket
// sorts] -- with barriers among themselves, and the other CTAs sort the
// small and medium segments meanwhile (the two paths share nothing). With
// large_ctas equal to the grid, every CTA takes both, the small and medium
// sorts after the histogram count. A barrier wait is bounded (about one
// second): a CTA that gives up records ERR_LOOKBACK_TIMEOUT and returns, so
// no later phase runs on incomplete data, and the others give up at their
// next barrier in turn.
// ---------------------------------------------------------------------------
// The first `parties` CTAs of the grid take part; `generation` counts the
// barriers passed (kept by thread 0).
__device__ __forceinline__ bool grid_barrier(uint32_t* arrivals, uint32_t& generation, uint32_t parties, int* err)
{
    __shared__ int s_ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        s_ok = 1;
        __threadfence();
        atomicAdd(arrivals, 1u);
        const uint32_t target = ++generation * parties;
        const unsigned long long t0 = dev::globaltimer();
        for (uint32_t spin = 1; dev::ld_acquire(arrivals) < target; ++spin) {
            if ((spin & 63) == 0 && dev::globaltimer() - t0 > dev::SPIN_LIMIT_NS) {
                dev::raise_error(err, dev::ERR_LOOKBACK_TIMEOUT);
                s_ok = 0;
                break;
            }
            if (spin > 16) __nanosleep(64);
        }
        __threadfence();
    }
    __syncthreads();
    return s_ok != 0;
}

template <typename K, bool HAS_V, int ITEMS, int LBW>
__global__ void __launch_bounds__(256, 2) k_seg_batch(SegArgs<K> a, int msd, uint32_t large_ctas)
{
    constexpr int P = Traits<K>::PASSES;
    constexpr int TILE = 256 * ITEMS;
    uint32_t gen = 0, lgen = 0;
    seg_classify(a);
    if (!grid_barrier(&a.ctl->barrier, gen, gridDim.x, a.err)) return;
    const bool split = large_ctas < gridDim.x;
    if (blockIdx.x >= large_ctas) {
        seg_small_warp<K, HAS_V, false>(a);
        __syncthreads();
        seg_small_cta<K, HAS_V, false>(a);
        return;
    }
    uint32_t* arrivals = &a.ctl->large_barrier;
    if (blockIdx.x == 0) seg_plan_scan<K, TILE, 256>(a);
    seg_large_zero(a, large_ctas);
    if (!grid_barrier(arrivals, lgen, large_ctas, a.err)) return;
    seg_plan_map(a, large_ctas);
    if (!grid_barrier(arrivals, lgen, large_ctas, a.err)) return;
    seg_large_count<K, TILE>(a, large_ctas);
    if (!split) {
        seg_small_warp<K, HAS_V, false>(a);
        __syncthreads();
        seg_small_cta<K, HAS_V, false>(a);
    }
    if (!grid_barrier(arrivals, lgen, large_ctas, a.err)) return;
    seg_large_starts(a, large_ctas);
    if (!grid_barrier(arrivals, lgen, large_ctas, a.err)) return;
    if (msd) {
        seg_route(a, large_ctas);
        if (!grid_barrier(arrivals, lgen, large_ctas, a.err)) return;
    }
    for (int slot = 0; slot < P; ++slot) {
        seg_large_pass<K, HAS_V, 256, ITEMS, LBW>(a, slot, large_ctas);
        if (!grid_barrier(arrivals, lgen, large_ctas, a.err)) return;
    }
    if (msd) {
        seg_small_warp<K, HAS_V, true>(a);
        __syncthreads();
        seg_small_cta<K, HAS_V, true>(a);
    }
}

// ---------------------------------------------------------------------------
// Host
// ---------------------------------------------------------------------------
template <typename K, bool HAS_V> struct LargeShape;
template <bool HV> struct LargeShape<uint32_t, HV> {
    static constexpr int THREADS = 256, ITEMS = 24, MINB = 2, LBW = HV ? 1 : 4;
};
template <bool HV> struct LargeShape<uint64_t, HV> {
    static constexpr int THREADS = 256, ITEMS = HV ? 20 : 24, MINB = 2, LBW = 4;
};

template <typename F> static void set_smem(F* kernel, std::size_t bytes)
{
    if (bytes > 0)  // static shared memory adds to this against the 48 KiB default
        check_cuda(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes),
                   "cudaFuncSetAttribute");
}

template <typename F> static int occupancy(F* kernel, int threads, std::size_t smem)
{
    int b = 0;
    check_cuda(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, kernel, threads, smem),
               "cudaOccupancyMaxActiveBlocksPerMultiprocessor");
    return std::max(b, 1);
}

// The one-CTA sorts of the segments (SUB: sub-buckets) of at most cap keys:
// 512 threads when threads == 512 and their shared memory fits the opt-in,
// else 256. (Keys-only u32 at the largest capacity: 16,384 keys in 224 KiB
// with 512 threads, one CTA per SM either way, so twice the warps hide the
// shared-memory round trips.)
template <typename K, bool HAS_V, bool SUB>
static void launch_cta_sort(device_context& ctx, const SegArgs<K>& a, uint32_t cap, int threads, cudaStream_t st)
{
    auto wide = &k_seg_small_cta<K, HAS_V, SUB, 512>;
    const std::size_t wsmem = cta_sort_smem<K, HAS_V>(cap, 512);
    cudaFuncAttributes fa{};
    check_cuda(cudaFuncGetAttributes(&fa, wide), "cudaFuncGetAttributes");
    if (threads == 512 && wsmem + fa.sharedSizeBytes <= ctx.smem_optin) {
        set_smem(wide, wsmem);
        wide<<<ctx.sm_count * occupancy(wide, 512, wsmem), 512, wsmem, st>>>(a);
    } else {
        auto kern = &k_seg_small_cta<K, HAS_V, SUB, SMALL_THREADS>;
        const std::size_t smem = cta_sort_smem<K, HAS_V>(cap, SMALL_THREADS);
        set_smem(kern, smem);
        kern<<<ctx.sm_count * occupancy(kern, SMALL_THREADS, smem), SMALL_THREADS, smem, st>>>(a);
    }
}

template <typename K, bool HAS_V>
void run(device_context& ctx, const K* in_k, K* out_k, const uint32_t* in_v, uint32_t* out_v, std::size_t n,
         const uint32_t* off, std::size_t nseg, dev::KeyXform<K> xf, const seg_options& opt)
{
    constexpr int P = Traits<K>::PASSES;
    using LS = LargeShape<K, HAS_V>;
    constexpr int TILE = LS::THREADS * LS::ITEMS;
    // Largest segment one CTA sorts in shared memory: two copies of keys (and
    // values) plus a packed rank per element, and 16 KiB of warp histograms
    // and peer masks (256 threads; 32 KiB with 512), must fit the 227 KiB
    // opt-in (u32: 12 B/elem keys-only, 20 B/elem with values; u64: 20 and
    // 28 B/elem).
    constexpr int MAX_CAP = sizeof(K) == 4 ? (HAS_V ? 10240 : 16384) : (HAS_V ? 7168 : 10240);
    const uint32_t cta_cap =
        (uint32_t)std::max<int>(WARP_CAP + 1, std::min<int>(opt.cta_cap > 0 ? opt.cta_cap : MAX_CAP, MAX_CAP));
    const uint32_t max_large = (uint32_t)std::min<std::size_t>(nseg, n / (cta_cap + 1) + 1);
    const uint32_t max_tiles = (uint32_t)(n / TILE + max_large + 1);

    temp_buffer ctl(ctx.resource, sizeof(SegControl));
    temp_buffer lists(ctx.resource, (2 * nseg + max_large + (max_large + 1)) * sizeof(uint32_t));
    temp_buffer tile_seg(ctx.resource, (std::size_t)max_tiles * sizeof(uint32_t));
    temp_buffer seg_hist(ctx.resource, (std::size_t)max_large * P * RADIX * sizeof(uint32_t));
    const bool maybe_large = n > cta_cap;
    temp_buffer alt_k(ctx.resource, maybe_large ? n * sizeof(K) : 0);
    temp_buffer alt_v(ctx.resource, maybe_large && HAS_V ? n * sizeof(uint32_t) : 0);
    // MSD route: per large segment its pass (or none), and at most 256
    // sub-buckets per large segment (never more than n)
    const uint32_t msd_cap = opt.msd_cap <= 0 ? 0u : (uint32_t)std::max<int>(WARP_CAP + 1, std::min(opt.msd_cap, MAX_CAP));
    const bool msd = maybe_large && msd_cap > 0;
    const uint32_t max_sub = msd ? (uint32_t)std::min<std::size_t>((std::size_t)max_large * RADIX, n) : 0;
    temp_buffer route(ctx.resource, maybe_large ? max_large : 0);
    temp_buffer sub_lists(ctx.resource, (std::size_t)max_sub * 4 * sizeof(uint32_t));
    check_cuda(cudaMemsetAsync(ctl.get(), 0, sizeof(SegControl), ctx.stream), "cudaMemsetAsync");
    if (maybe_large && !msd)
        check_cuda(cudaMemsetAsync(route.get(), NO_ROUTE, max_large, ctx.stream), "cudaMemsetAsync");

    SegArgs<K> a;
    a.in_k = in_k;
    a.out_k = out_k;
    a.alt_k = alt_k.as<K>();
    a.in_v = in_v;
    a.out_v = out_v;
    a.alt_v = alt_v.as<uint32_t>();
    a.off = off;
    a.skip = opt.skip;
    a.nseg = (uint32_t)nseg;
    a.cta_cap = cta_cap;
    a.xf = xf;
    a.ctl = ctl.as<SegControl>();
    uint32_t* l = lists.as<uint32_t>();
    a.warp_list = l;
    a.cta_list = l + nseg;
    a.large_list = l + 2 * nseg;
    a.tile_begin = l + 2 * nseg + max_large;
    a.tile_seg = tile_seg.as<uint32_t>();
    a.seg_hist = seg_hist.as<uint32_t>();
    a.max_large = max_large;
    a.max_tiles = max_tiles;
    a.ring = ctx.lookback_ring;
    a.seq0 = maybe_large ? ctx.reserve_seq((uint64_t)P * max_tiles) : 0;
    a.err = ctx.d_error;
    a.route = route.as<uint8_t>();
    a.sub_warp_list = sub_lists.as<uint32_t>();
    a.sub_cta_list = sub_lists.as<uint32_t>() + 2 * (std::size_t)max_sub;
    a.max_sub = max_sub;
    a.sub_cap = msd_cap;

    constexpr std::size_t per_warp_smem =
        2 * WARP_CAP * sizeof(K) + (HAS_V ? 2 * WARP_CAP * 4 : 0) + WARP_CAP * 4 + 2 * RADIX * 4;
    auto cta_smem = [](uint32_t cap) { return cta_sort_smem<K, HAS_V>(cap, SMALL_THREADS); };
    // the large pass: two half-warp count arrays of RADIX + LARGE_PAD words per warp, and a tile
    constexpr std::size_t large_pass_smem = (std::size_t)(LS::THREADS / 32) * (RADIX + LARGE_PAD) * 8 +
                                            (std::size_t)TILE * sizeof(K) + (HAS_V ? (std::size_t)TILE * 4 : 0);
    if (opt.persistent > 0) {
        // One cooperative launch of every phase; its shared memory is the
        // largest any phase needs. Falls through to the launch sequence below
        // when not even one CTA per SM fits.
        const std::size_t pass_smem = large_pass_smem;
        const std::size_t smem = std::max({per_warp_smem * SMALL_WARPS, cta_smem(cta_cap), pass_smem,
                                           msd ? cta_smem(msd_cap) : std::size_t(0)});
        auto kern = &k_seg_batch<K, HAS_V, LS::ITEMS, LS::LBW>;
        int per_sm = 0;
        if (smem + 32 * 1024 <= ctx.smem_optin) {
            set_smem(kern, smem);
            check_cuda(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, 256, smem),
                       "cudaOccupancyMaxActiveBlocksPerMultiprocessor");
        }
        if (per_sm > 0) {
            const uint32_t grid = (uint32_t)(ctx.sm_count * per_sm);
            // persistent >= 2: that many eighths (less one) of the grid sort
            // the small and medium segments while the rest take the large ones
            const uint32_t small_ctas = opt.persistent >= 2 ? grid * (uint32_t)std::min(opt.persistent - 1, 6) / 8 : 0;
            cudaLaunchConfig_t cfg = {};
            cfg.gridDim = dim3(grid);
            cfg.blockDim = dim3(256);
            cfg.dynamicSmemBytes = smem;
            cfg.stream = ctx.stream;
            cudaLaunchAttribute attr[1];
            attr[0].id = cudaLaunchAttributeCooperative;
            attr[0].val.cooperative = 1;
            cfg.attrs = attr;
            cfg.numAttrs = 1;
            kernel_timer kt(ctx, "segsort.batch");
            check_cuda(cudaLaunchKernelEx(&cfg, kern, a, msd ? 1 : 0, grid - small_ctas),
                       "segmented sort batch launch");
            return;
        }
    }

    {
        kernel_timer kt(ctx, "segsort.classify");
        const int grid = (int)std::max<std::size_t>(1, std::min<std::size_t>((nseg + 255) / 256, (std::size_t)ctx.sm_count * 4));
        k_seg_classify<K><<<grid, 256, 0, ctx.stream>>>(a);
        check_cuda(cudaGetLastError(), "segmented sort classify launch");
    }
    // Fork: the large-segment path runs on the auxiliary stream.
    cudaStream_t aux = ctx.aux_stream();
    check_cuda(cudaEventRecord(ctx.fork_event, ctx.stream), "cudaEventRecord");
    check_cuda(cudaStreamWaitEvent(aux, ctx.fork_event, 0), "cudaStreamWaitEvent");

    {
        kernel_timer kt(ctx, "segsort.small_warp");
        const std::size_t smem = per_warp_smem * SMALL_WARPS;
        auto kern = &k_seg_small_warp<K, HAS_V, false>;
        set_smem(kern, smem);
        const int grid = ctx.sm_count * occupancy(kern, SMALL_THREADS, smem);
        kern<<<grid, SMALL_THREADS, smem, ctx.stream>>>(a);
        check_cuda(cudaGetLastError(), "segmented sort warp launch");
    }
    {
        kernel_timer kt(ctx, "segsort.small_cta");
        launch_cta_sort<K, HAS_V, false>(ctx, a, cta_cap, opt.cta_threads, ctx.stream);
        check_cuda(cudaGetLastError(), "segmented sort cta launch");
    }
    if (maybe_large) {
        {
            kernel_timer kt(ctx, "segsort.large_histogram", aux);
            k_seg_plan<K, TILE><<<1, 1024, 0, aux>>>(a);
            check_cuda(cudaGetLastError(), "segmented sort plan launch");
            k_seg_large_zero<K><<<ctx.sm_count * 4, 256, 0, aux>>>(a);
            auto hk = &k_seg_large_count<K, TILE>;
            hk<<<ctx.sm_count * occupancy(hk, 256, 0), 256, 0, aux>>>(a);
            k_seg_large_starts<K><<<ctx.sm_count * 4, 256, 0, aux>>>(a);
            check_cuda(cudaGetLastError(), "segmented sort histogram launch");
        }
        if (msd) {
            k_seg_route<K><<<ctx.sm_count * 4, 256, 0, aux>>>(a);
            check_cuda(cudaGetLastError(), "segmented sort route launch");
        }
        auto pk = &k_seg_large_pass<K, HAS_V, LS::THREADS, LS::ITEMS, LS::MINB, LS::LBW>;
        const std::size_t psmem = large_pass_smem;
        set_smem(pk, psmem);
        const int pgrid = ctx.sm_count * occupancy(pk, LS::THREADS, psmem);
        for (int s = 0; s < P; ++s) {
            kernel_timer kt(ctx, "segsort.large_pass", aux);
            pk<<<pgrid, LS::THREADS, psmem, aux>>>(a, s);
            check_cuda(cudaGetLastError(), "segmented sort pass launch");
        }
        if (msd) {
            // the MSD route's sub-buckets: from the scratch buffer into the output
            constexpr std::size_t per_warp =
                2 * WARP_CAP * sizeof(K) + (HAS_V ? 2 * WARP_CAP * 4 : 0) + WARP_CAP * 4 + 2 * RADIX * 4;
            auto wk = &k_seg_small_warp<K, HAS_V, true>;
            set_smem(wk, per_warp * SMALL_WARPS);
            wk<<<ctx.sm_count * occupancy(wk, SMALL_THREADS, per_warp * SMALL_WARPS), SMALL_THREADS,
                 per_warp * SMALL_WARPS, aux>>>(a);
            launch_cta_sort<K, HAS_V, true>(ctx, a, msd_cap, opt.cta_threads, aux);
            check_cuda(cudaGetLastError(), "segmented sort sub-bucket launch");
        }
    }
    // Join.
    check_cuda(cudaEventRecord(ctx.join_event, aux), "cudaEventRecord");
    check_cuda(cudaStreamWaitEvent(ctx.stream, ctx.join_event, 0), "cudaStreamWaitEvent");
}

}  // namespace seg

uint32_t segsort_cta_cap(int key_bytes, bool has_values)
{
    return key_bytes == 4 ? (has_values ? 10240u : 16384u) : (has_values ? 7168u : 10240u);
}

std::string segsort_batch_tuning_key(int key_bytes, bool has_values, std::size_t n, std::size_t num_segments)
{
    return segsort_tuning_key(key_bytes, has_values, n, num_segments) + ":batch";
}

std::string segsort_cta_threads_tuning_key() { return "segsort:cta_threads"; }

std::string segsort_threads_tuning_key(int key_bytes, bool has_values, std::size_t n, std::size_t num_segments)
{
    return segsort_tuning_key(key_bytes, has_values, n, num_segments) + ":threads";
}

std::string segsort_msd_tuning_key(int key_bytes, bool has_values, std::size_t n, std::size_t num_segments)
{
    return segsort_tuning_key(key_bytes, has_values, n, num_segments) + ":msd";
}

std::string segsort_tuning_key(int key_bytes, bool has_values, std::size_t n, std::size_t num_segments)
{
    // distribution class: average segment length, as a power of two
    const std::size_t avg = num_segments ? n / num_segments : n;
    return std::string("segsort:") + (key_bytes == 4 ? "u32" : "u64") + (has_values ? "kv" : "k") + ":" +
           tuning_table::size_class(n) + ":avg" + tuning_table::size_class(avg);
}

void segmented_sort(device_context& ctx, const void* keys_in, void* keys_out, int key_bytes, int key_kind,
                    const uint32_t* vals_in, uint32_t* vals_out, std::size_t n, const uint32_t* offsets,
                    std::size_t num_segments, bool descending, const seg_options& opt)
{
    if (key_bytes != 4 && key_bytes != 8) throw std::invalid_argument("segmented_sort: keys must be 32 or 64 bits");
    if (key_kind < 0 || key_kind > 2) throw std::invalid_argument("segmented_sort: unknown key kind");
    if ((vals_in == nullptr) != (vals_out == nullptr))
        throw std::invalid_argument("segmented_sort: values need both an input and an output");
    check_size(n);
    if (num_segments == 0 || n == 0) return;
    if (offsets == nullptr || keys_in == nullptr || keys_out == nullptr)
        throw std::invalid_argument("segmented_sort: null argument");
    if (num_segments > 0x7FFFFFFFu) throw std::length_error("segmented_sort: too many segments");
    if (opt.skip != nullptr && (keys_in != keys_out || vals_in != vals_out))
        throw std::invalid_argument("segmented_sort: skipped segments need an in-place call");
    ctx.activate();
    seg_options o = opt;
    if (o.msd_cap < 0) {
        launch_shape shape;
        o.msd_cap = ctx.tuning.lookup(segsort_msd_tuning_key(key_bytes, vals_in != nullptr, n, num_segments), shape)
                        ? shape.variant
                        : 0;
    }
    if (o.cta_threads == 0) {
        launch_shape shape;
        if (ctx.tuning.lookup(segsort_threads_tuning_key(key_bytes, vals_in != nullptr, n, num_segments), shape) ||
            ctx.tuning.lookup(segsort_cta_threads_tuning_key(), shape))
            o.cta_threads = shape.variant;
    }
    if (o.persistent < 0) {
        launch_shape shape;
        o.persistent = ctx.tuning.lookup(segsort_batch_tuning_key(key_bytes, vals_in != nullptr, n, num_segments), shape)
                           ? shape.variant
                           : 0;
    }
    if (key_bytes == 4) {
        const auto xf = dev::make_xform<uint32_t>(key_kind, descending);
        if (vals_in)
            seg::run<uint32_t, true>(ctx, static_cast<const uint32_t*>(keys_in), static_cast<uint32_t*>(keys_out),
                                     vals_in, vals_out, n, offsets, num_segments, xf, o);
        else
            seg::run<uint32_t, false>(ctx, static_cast<const uint32_t*>(keys_in), static_cast<uint32_t*>(keys_out),
                                      nullptr, nullptr, n, offsets, num_segments, xf, o);
    } else {
        const auto xf = dev::make_xform<uint64_t>(key_kind, descending);
        if (vals_in)
            seg::run<uint64_t, true>(ctx, static_cast<const uint64_t*>(keys_in), static_cast<uint64_t*>(keys_out),
                                     vals_in, vals_out, n, offsets, num_segments, xf, o);
        else
            seg::run<uint64_t, false>(ctx, static_cast<const uint64_t*>(keys_in), static_cast<uint64_t*>(keys_out),
                                      nullptr, nullptr, n, offsets, num_segments, xf, o);
    }
}

}  // namespace gbc
