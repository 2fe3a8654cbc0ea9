// Bitpack compression of 32-bit integers: frame-of-reference bit packing per
// chunk, optionally after a delta + zigzag transform.
//
// Reference path replaced: compress_bitpack / decompress_bitpack
// (lib/src/Compute/Compression.cpp:139-200) with kernels clc_bitpack_analyze,
// clc_bitpack_pack and clc_bitpack_unpack (Compression.cpp:39-124). The
// device format is kept word for word, since compressed data outlives the
// library that wrote it (Compression.cpp:19-24): per chunk three words {base,
// width, offset of its packed words relative to the packed area}, then the
// packed area; element j of a chunk occupies bits [j * width, (j + 1) *
// width) of the chunk's words, least significant bits first; width = 32 -
// clz(max - min) of the chunk's encoded values (0 when they are all equal);
// delta mode stores zigzag(x[i] - x[i-1]) with wrapping arithmetic and
// x[-1] = 0, and decoding ends with a wrapping inclusive prefix sum over the
// whole array.
//
// How it runs here:
//   * analyze: one warp per chunk, 128-bit loads, warp min/max; the chunks'
//     word counts are turned into offsets by the library's single-pass scan
//     (the reference's scan client at Compression.cpp:178), which also
//     yields the total size;
//   * pack: one warp per chunk, in rounds of 2,048 elements. Lane l packs
//     elements 64 l .. 64 l + 63 of the round, which occupy exactly 2 x width
//     whole words, so no word is shared between lanes (the reference ORs
//     every element into global memory with atomics). The lanes' words are
//     staged in shared memory at an odd per-lane stride (2 width + 1: the
//     lanes hit different banks) and written out by the warp in order,
//     coalesced;
//   * unpack, delta mode with a mean width of at most 16 bits: one pass. A
//     thread decodes 32 consecutive elements from the `width` whole words
//     that hold them (width a compile-time constant: one funnel shift per
//     element), the tile sums its deltas, and its prefix comes from a
//     decoupled look-back;
//   * unpack, otherwise: one thread per 4 elements (a 128-bit store),
//     reading the 1-5 packed words that hold them; delta mode then runs the
//     library's scan in place.
#include <algorithm>
#include <cstring>
#include <functional>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/compute_c.h"
#include "device_common.cuh"
#include "runtime.hpp"
#include "sort_internal.hpp"

namespace gbc {
namespace bitpack {

using dev::FULL_MASK;

constexpr int THREADS = 256;
constexpr int WARPS = THREADS / 32;
constexpr int PACK_THREADS = 128;  // 4 warps x 8.1 KiB of staging: static shared memory
constexpr int PACK_WARPS = PACK_THREADS / 32;
constexpr uint32_t LANE_ELEMS = 64;          // per lane and round
constexpr uint32_t ROUND = 32 * LANE_ELEMS;  // per warp and round

__device__ __forceinline__ uint32_t zigzag(uint32_t d) { return (d << 1) ^ (0u - (d >> 31)); }
__device__ __forceinline__ uint32_t unzigzag(uint32_t v) { return (v >> 1) ^ (0u - (v & 1u)); }

// Encoded values in[i .. i+3] (i a multiple of 4; `prev` = in[i - 1], or 0).
template <bool DELTA> __device__ __forceinline__ void encode4(uint4 w, uint32_t prev, uint32_t (&e)[4])
{
    if (DELTA) {
        e[0] = zigzag(w.x - prev);
        e[1] = zigzag(w.y - w.x);
        e[2] = zigzag(w.z - w.y);
        e[3] = zigzag(w.w - w.z);
    } else {
        e[0] = w.x, e[1] = w.y, e[2] = w.z, e[3] = w.w;
    }
}

template <bool DELTA> __device__ __forceinline__ uint32_t encode_at(const uint32_t* in, uint32_t i)
{
    if (!DELTA) return in[i];
    return zigzag(in[i] - (i > 0 ? in[i - 1] : 0u));
}

// One warp per chunk: base and width into hdr[2c], hdr[2c + 1], the chunk's
// packed word count into words[c].
template <bool DELTA>
__global__ void __launch_bounds__(THREADS) k_bp_analyze(const uint32_t* __restrict__ in, uint32_t n, uint32_t chunk,
                                                        uint32_t chunks, uint32_t* __restrict__ hdr,
                                                        uint32_t* __restrict__ words)
{
    const int lane = threadIdx.x & 31;
    const bool vec = (reinterpret_cast<uintptr_t>(in) & 15) == 0;
    for (uint32_t c = blockIdx.x * WARPS + (threadIdx.x >> 5); c < chunks; c += gridDim.x * WARPS) {
        const uint32_t start = c * chunk, count = min(chunk, n - start);
        uint32_t lo = 0xFFFFFFFFu, hi = 0;
        uint32_t j = 0;
        if (vec) {
            for (; j + 4 * 32 <= count; j += 4 * 32) {
                const uint32_t i = start + j + 4 * lane;
                const uint4 w = dev::ld_stream(reinterpret_cast<const uint4*>(in + i));
                uint32_t e[4];
                encode4<DELTA>(w, DELTA && i > 0 ? in[i - 1] : 0u, e);
#pragma unroll
                for (int q = 0; q < 4; ++q) lo = min(lo, e[q]), hi = max(hi, e[q]);
            }
        }
        for (uint32_t k = j + lane; k < count; k += 32) {
            const uint32_t e = encode_at<DELTA>(in, start + k);
            lo = min(lo, e), hi = max(hi, e);
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            lo = min(lo, __shfl_xor_sync(FULL_MASK, lo, o));
            hi = max(hi, __shfl_xor_sync(FULL_MASK, hi, o));
        }
        if (lane == 0) {
            const uint32_t range = hi - lo;
            const uint32_t width = range == 0 ? 0u : 32u - __clz(range);
            hdr[2 * c] = lo;
            hdr[2 * c + 1] = width;
            words[c] = (uint32_t)(((uint64_t)count * width + 31) / 32);
        }
    }
}

// One warp per chunk: the header triple and the chunk's packed words.
template <bool DELTA>
__global__ void __launch_bounds__(PACK_THREADS) k_bp_pack(const uint32_t* __restrict__ in, uint32_t n, uint32_t chunk,
                                                     uint32_t chunks, const uint32_t* __restrict__ hdr,
                                                     const uint32_t* __restrict__ offsets, uint32_t* __restrict__ out)
{
    __shared__ uint32_t stage[PACK_WARPS][32 * 65];  // per lane 2 x width + 1 <= 65 words
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t* my = stage[warp];
    const bool vec = (reinterpret_cast<uintptr_t>(in) & 15) == 0;
    for (uint32_t c = blockIdx.x * PACK_WARPS + warp; c < chunks; c += gridDim.x * PACK_WARPS) {
        const uint32_t start = c * chunk, count = min(chunk, n - start);
        const uint32_t base = hdr[2 * c], width = hdr[2 * c + 1], off = offsets[c];
        if (lane == 0) {
            out[3 * c] = base;
            out[3 * c + 1] = width;
            out[3 * c + 2] = off;
        }
        if (width == 0) continue;
        uint32_t* packed = out + 3 * (size_t)chunks + off;
        const uint32_t lane_words = 2 * width, pitch = lane_words + 1;
        for (uint32_t r0 = 0; r0 < count; r0 += ROUND) {
            // this lane's elements of the round
            const uint32_t j0 = r0 + lane * LANE_ELEMS;
            const uint32_t mine = j0 < count ? min(LANE_ELEMS, count - j0) : 0u;
            uint64_t acc = 0;
            uint32_t bits = 0, k = 0;
            auto put = [&](uint32_t v) {
                acc |= (uint64_t)(v - base) << bits;
                bits += width;
                if (bits >= 32) {
                    my[lane * pitch + k++] = (uint32_t)acc;
                    acc >>= 32;
                    bits -= 32;
                }
            };
            const uint32_t i0 = start + j0;
            if (vec && mine == LANE_ELEMS) {
                uint32_t prev = DELTA && i0 > 0 ? in[i0 - 1] : 0u;
#pragma unroll 4
                for (uint32_t q = 0; q < LANE_ELEMS; q += 4) {
                    const uint4 w = *reinterpret_cast<const uint4*>(in + i0 + q);
                    uint32_t e[4];
                    encode4<DELTA>(w, prev, e);
                    prev = w.w;
#pragma unroll
                    for (int t = 0; t < 4; ++t) put(e[t]);
                }
            } else {
                for (uint32_t q = 0; q < mine; ++q) put(encode_at<DELTA>(in, i0 + q));
            }
            if (bits > 0) my[lane * pitch + k++] = (uint32_t)acc;  // the partial last word
            __syncwarp();
            // the round's words, in order: lane l's words are words
            // [l * 2 width, ...) of the round
            const uint32_t rcount = min(ROUND, count - r0);
            const uint32_t rwords = (uint32_t)(((uint64_t)rcount * width + 31) / 32);
            uint32_t* dst = packed + (size_t)(r0 / 32) * width;  // r0 * width / 32 (r0 is a multiple of 2048)
            for (uint32_t m = lane; m < rwords; m += 32) {
                const uint32_t l = m / lane_words, kk = m - l * lane_words;
                dst[m] = my[l * pitch + kk];
            }
            __syncwarp();
        }
    }
}

// One thread per 4 elements. Chunks hold a multiple of 4 elements (at least
// 256), so a group never straddles two chunks.
template <bool DELTA>
__global__ void __launch_bounds__(THREADS) k_bp_unpack(const uint32_t* __restrict__ data, uint32_t n,
                                                       uint32_t chunk_shift, uint32_t chunks,
                                                       uint32_t* __restrict__ out)
{
    const uint32_t groups = (n + 3) / 4;
    const bool vec = (reinterpret_cast<uintptr_t>(out) & 15) == 0;
    for (uint32_t g = blockIdx.x * THREADS + threadIdx.x; g < groups; g += gridDim.x * THREADS) {
        const uint32_t i = 4 * g;
        const uint32_t c = i >> chunk_shift, j = i & ((1u << chunk_shift) - 1u);
        const uint32_t base = __ldg(data + 3 * c), width = __ldg(data + 3 * c + 1);
        uint32_t v[4] = {base, base, base, base};
        if (width != 0) {
            const uint32_t* p = data + 3 * (size_t)chunks + __ldg(data + 3 * c + 2);
            const uint64_t first = (uint64_t)j * width;
            const uint32_t w0 = (uint32_t)(first >> 5);
            const uint32_t mask = width == 32 ? 0xFFFFFFFFu : ((1u << width) - 1u);
            // the group's elements below n lie in bits [first, first + valid
            // x width): at most 5 words from w0; words past the last of them
            // may lie beyond the chunk's packed words and are not read
            const uint32_t valid = min(4u, n - i);
            const uint32_t last_word = (uint32_t)((first + (uint64_t)valid * width - 1) >> 5);
            uint32_t wv[5];
#pragma unroll
            for (int q = 0; q < 5; ++q) wv[q] = (w0 + q <= last_word) ? __ldg(p + w0 + q) : 0u;
#pragma unroll
            for (int t = 0; t < 4; ++t) {
                const uint64_t bit = first + (uint64_t)t * width;
                const uint32_t q = (uint32_t)(bit >> 5) - w0, sh = (uint32_t)(bit & 31);
                const uint64_t both = (uint64_t)wv[q] | ((uint64_t)(q + 1 < 5 ? wv[q + 1] : 0u) << 32);
                v[t] = (uint32_t)(both >> sh) & mask;
                v[t] += base;
            }
        }
        if (DELTA) {
#pragma unroll
            for (int t = 0; t < 4; ++t) v[t] = unzigzag(v[t]);
        }
        if (vec && i + 4 <= n) {
            *reinterpret_cast<uint4*>(out + i) = make_uint4(v[0], v[1], v[2], v[3]);
        } else {
            for (int t = 0; t < 4 && i + t < n; ++t) out[i + t] = v[t];
        }
    }
}

// ---- fused unpack (and, in delta mode, the prefix sum that undoes it) -------
// Lane-private whole words: a thread decodes 32 consecutive elements of one
// chunk, which occupy exactly `width` whole words of the packed area (element
// j sits at bit j * width and 32 * width bits are width words), so with the
// width as a compile-time constant every shift and word index is a constant
// (one funnel shift, a mask and an add per element). A CTA's 8,192 elements
// form one tile. In delta mode the tile's deltas are scanned in place
// (thread, warp, CTA) and the tile's prefix comes from a decoupled look-back
// over the context's status ring, so the prefix sum costs no pass of its own.
// The decoded tile is staged in shared memory at an odd stride and written
// out coalesced.
constexpr int UT = 256;             // threads per CTA
constexpr int UE = 32;              // elements per thread
constexpr int UTILE = UT * UE;      // elements per tile
constexpr int U_LBL = 4;            // look-back: 32 x 4 tiles per round trip
constexpr uint64_t U_SLOTS = onesweep::RING_BYTES / 8;
constexpr uint64_t U_AGG = 1, U_PRE = 2, U_TAG = (1ull << 30) - 1;

__device__ __forceinline__ void u_publish(uint64_t* ring, uint64_t seq, uint64_t flag, uint32_t v)
{
    dev::st_relaxed(&ring[seq & (U_SLOTS - 1)], (flag << 62) | ((seq & U_TAG) << 32) | v);
}

__device__ __forceinline__ bool u_read(const uint64_t* ring, uint64_t seq, uint64_t& flag, uint32_t& v)
{
    const uint64_t w = dev::ld_relaxed(&ring[seq & (U_SLOTS - 1)]);
    flag = w >> 62;
    if (flag == 0 || ((w >> 32) & U_TAG) != (seq & U_TAG)) return false;
    v = (uint32_t)w;
    return true;
}

// Elements of the lane's 32 (all in one chunk) from its W packed words at p;
// `words_left` bounds the reads at the end of the buffer.
template <int W>
__device__ __forceinline__ void decode32(const uint32_t* __restrict__ p, uint64_t words_left, uint32_t base,
                                         uint32_t (&v)[UE])
{
    if constexpr (W == 0) {
#pragma unroll
        for (int e = 0; e < UE; ++e) v[e] = base;
    } else {
        uint32_t w[W];
        if (words_left >= (uint64_t)W) {
#pragma unroll
            for (int k = 0; k < W; ++k) w[k] = __ldg(p + k);
        } else {
#pragma unroll
            for (int k = 0; k < W; ++k) w[k] = (uint64_t)k < words_left ? __ldg(p + k) : 0u;
        }
#pragma unroll
        for (int e = 0; e < UE; ++e) {
            constexpr uint32_t mask = W == 32 ? 0xFFFFFFFFu : ((1u << (W & 31)) - 1u);
            const int bit = e * W, q = bit >> 5, sh = bit & 31;
            uint32_t x;
            if (W == 32) x = w[e];
            else if (sh + W <= 32) x = (w[q] >> sh) & mask;
            else x = __funnelshift_r(w[q], w[q + 1 < W ? q + 1 : q], sh) & mask;
            v[e] = x + base;
        }
    }
}

template <int W0>
__device__ __forceinline__ void decode_dispatch(uint32_t width, const uint32_t* p, uint64_t words_left, uint32_t base,
                                                uint32_t (&v)[UE])
{
    if constexpr (W0 <= 32) {
        if (width == (uint32_t)W0) decode32<W0>(p, words_left, base, v);
        else decode_dispatch<W0 + 1>(width, p, words_left, base, v);
    }
}

template <bool DELTA>
__global__ void __launch_bounds__(UT, 2)
    k_bp_unpack_tiles(const uint32_t* __restrict__ data, uint64_t words, uint32_t n, uint32_t chunk_shift,
                      uint32_t chunks, uint32_t* __restrict__ out, uint32_t num_tiles, uint32_t* tile_ctr,
                      uint64_t* ring, uint64_t seq0, int* err)
{
    __shared__ uint32_t s_out[UT * (UE + 1)];
    __shared__ uint32_t s_warp[UT / 32];
    __shared__ uint32_t s_prefix;
    __shared__ uint32_t s_tile;
    __shared__ int s_abort;  // a look-back wait gave up: the outputs are unknown, nothing is written
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const uint32_t* packed = data + 3 * (size_t)chunks;
    if (tid == 0) s_abort = 0;
    for (;;) {
        if (tid == 0) s_tile = atomicAdd(tile_ctr, 1u);
        __syncthreads();
        const uint32_t t = s_tile;
        if (t >= num_tiles) break;
        const uint32_t i0 = t * UTILE + tid * UE;  // the thread's first element
        uint32_t v[UE];
        if (i0 < n) {
            const uint32_t c = i0 >> chunk_shift, j0 = i0 & ((1u << chunk_shift) - 1u);
            const uint32_t base = __ldg(data + 3 * c), width = __ldg(data + 3 * c + 1);
            const uint64_t first = (uint64_t)__ldg(data + 3 * c + 2) + (uint64_t)(j0 / UE) * width;
            const uint64_t avail = 3 * (uint64_t)chunks + first < words ? words - 3 * (uint64_t)chunks - first : 0;
            if (width > 32) {  // corrupt header: the caller validated the blob, nothing is decoded
#pragma unroll
                for (int e = 0; e < UE; ++e) v[e] = 0;
            } else {
                decode_dispatch<0>(width, packed + first, avail, base, v);
            }
#pragma unroll
            for (int e = 0; e < UE; ++e)
                if (i0 + e >= n) v[e] = DELTA ? zigzag(0u) : 0u;  // past the end: a zero delta
        } else {
#pragma unroll
            for (int e = 0; e < UE; ++e) v[e] = 0;
        }
        if (DELTA) {
            // undo the zigzag, then the thread's, the warp's and the CTA's
            // inclusive sums (wrapping)
#pragma unroll
            for (int e = 0; e < UE; ++e) v[e] = unzigzag(v[e]);
#pragma unroll
            for (int e = 1; e < UE; ++e) v[e] += v[e - 1];
            uint32_t inc = v[UE - 1];
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const uint32_t y = __shfl_up_sync(FULL_MASK, inc, o);
                if (lane >= o) inc += y;
            }
            if (lane == 31) s_warp[warp] = inc;
            const uint32_t lane_excl = inc - v[UE - 1];
            __syncthreads();
            if (warp == 0) {
                uint32_t wt = lane < UT / 32 ? s_warp[lane] : 0u;
#pragma unroll
                for (int o = 1; o < UT / 32; o <<= 1) {
                    const uint32_t y = __shfl_up_sync(FULL_MASK, wt, o);
                    if (lane >= o) wt += y;
                }
                const uint32_t agg = __shfl_sync(FULL_MASK, wt, UT / 32 - 1);
                // exclusive warp offsets
                const uint32_t wexcl = __shfl_up_sync(FULL_MASK, wt, 1);
                if (lane < UT / 32) s_warp[lane] = lane == 0 ? 0u : wexcl;
                const uint64_t my_seq = seq0 + t;
                if (lane == 0) u_publish(ring, my_seq, t == 0 ? U_PRE : U_AGG, agg);
                uint32_t excl = 0;
                if (t > 0) {
                    bool gave_up = false;
                    int64_t w_end = t;
                    for (;;) {
                        uint64_t flag[U_LBL];
                        uint32_t val[U_LBL];
#pragma unroll
                        for (int q = 0; q < U_LBL; ++q) {
                            const int64_t k = w_end - 32 * U_LBL + lane * U_LBL + q;
                            flag[q] = U_PRE;  // before tile 0: an empty inclusive prefix
                            val[q] = 0;
                            if (k >= 0 && !u_read(ring, seq0 + (uint64_t)k, flag[q], val[q])) {
                                const unsigned long long start = dev::globaltimer();
                                for (uint32_t spin = 1;; ++spin) {
                                    if (u_read(ring, seq0 + (uint64_t)k, flag[q], val[q])) break;
                                    if ((spin & 255) == 0 && dev::globaltimer() - start > dev::SPIN_LIMIT_NS) {
                                        gave_up = true;
                                        flag[q] = U_PRE;
                                        val[q] = 0;
                                        break;
                                    }
                                    if (spin > 32) __nanosleep(64);
                                }
                            }
                        }
                        int hi = -1;  // this lane's nearest inclusive prefix
#pragma unroll
                        for (int q = 0; q < U_LBL; ++q)
                            if (flag[q] == U_PRE) hi = q;
                        const uint32_t pre = __ballot_sync(FULL_MASK, hi >= 0);
                        const int L = pre ? 31 - __clz(pre) : -1;
                        uint32_t contrib = 0;
                        if (lane >= L) {
                            const int q0 = lane == L ? hi : 0;
#pragma unroll
                            for (int q = 0; q < U_LBL; ++q)
                                if (q >= q0) contrib += val[q];
                        }
#pragma unroll
                        for (int o = 16; o > 0; o >>= 1) contrib += __shfl_xor_sync(FULL_MASK, contrib, o);
                        excl += contrib;
                        if (pre) break;
                        w_end -= 32 * U_LBL;
                    }
                    if (__any_sync(FULL_MASK, gave_up) && lane == 0) {
                        dev::raise_error(err, dev::ERR_LOOKBACK_TIMEOUT);
                        s_abort = 1;
                    }
                    if (lane == 0) u_publish(ring, my_seq, U_PRE, excl + agg);
                }
                if (lane == 0) s_prefix = excl;
            }
            __syncthreads();
            const uint32_t add = s_prefix + s_warp[warp] + lane_excl;
#pragma unroll
            for (int e = 0; e < UE; ++e) v[e] += add;
        }
        // stage at stride UE + 1 (conflict-free both ways) and write coalesced
#pragma unroll
        for (int e = 0; e < UE; ++e) s_out[tid * (UE + 1) + e] = v[e];
        __syncthreads();
        const uint32_t tb = t * UTILE;
        if (s_abort) {
            // after a timed-out wait the prefix is unknown: nothing is written
        } else if (tb + UTILE <= n) {
#pragma unroll 8
            for (int k = 0; k < UE; ++k) {
                const uint32_t idx = k * UT + tid;
                out[tb + idx] = s_out[(idx / UE) * (UE + 1) + idx % UE];
            }
        } else {
            for (int k = 0; k < UE; ++k) {
                const uint32_t idx = k * UT + tid;
                if (tb + idx < n) out[tb + idx] = s_out[(idx / UE) * (UE + 1) + idx % UE];
            }
        }
        __syncthreads();
    }
}

void check_chunk(std::size_t chunk)
{
    if (chunk < 256 || chunk > 65536 || (chunk & (chunk - 1)) != 0)
        throw std::invalid_argument("bitpack: chunk_size must be a power of two in [256, 65536]");
}

int grid_for(device_context& ctx, std::size_t work_warps, int warps_per_cta)
{
    const std::size_t ctas = (work_warps + warps_per_cta - 1) / warps_per_cta;
    return (int)std::max<std::size_t>(1, std::min<std::size_t>(ctas, (std::size_t)ctx.sm_count * 64 / warps_per_cta));
}

}  // namespace bitpack

std::size_t bitpack_words_bound(std::size_t n, std::size_t chunk)
{
    bitpack::check_chunk(chunk);
    return n == 0 ? 0 : 3 * ((n + chunk - 1) / chunk) + n;
}

std::size_t bitpack_compress(device_context& ctx, const uint32_t* in, std::size_t n, std::size_t chunk, bool delta,
                             const std::function<uint32_t*(std::size_t)>& make_output)
{
    using namespace bitpack;
    check_chunk(chunk);
    if (n == 0) return 0;
    check_size(n);
    if (in == nullptr) throw std::invalid_argument("bitpack: null input");
    ctx.activate();
    const uint32_t chunks = (uint32_t)((n + chunk - 1) / chunk);
    temp_buffer hdr(ctx.resource, (std::size_t)chunks * 2 * 4);
    temp_buffer words(ctx.resource, (std::size_t)chunks * 4);
    temp_buffer offs(ctx.resource, (std::size_t)chunks * 4);
    temp_buffer total(ctx.resource, 8);
    const int grid = grid_for(ctx, chunks, WARPS);
    {
        kernel_timer kt(ctx, "bitpack.analyze");
        if (delta)
            k_bp_analyze<true><<<grid, THREADS, 0, ctx.stream>>>(in, (uint32_t)n, (uint32_t)chunk, chunks,
                                                                 hdr.as<uint32_t>(), words.as<uint32_t>());
        else
            k_bp_analyze<false><<<grid, THREADS, 0, ctx.stream>>>(in, (uint32_t)n, (uint32_t)chunk, chunks,
                                                                  hdr.as<uint32_t>(), words.as<uint32_t>());
        check_cuda(cudaGetLastError(), "bitpack analyze launch");
    }
    const uint32_t zero = 0;
    scan(ctx, words.get(), offs.get(), chunks, elem::u32, op_kind::plus, &zero, true, total.get());
    uint64_t packed = 0;
    check_cuda(cudaMemcpyAsync(&packed, total.get(), 8, cudaMemcpyDeviceToHost, ctx.stream), "cudaMemcpyAsync");
    check_cuda(cudaStreamSynchronize(ctx.stream), "cudaStreamSynchronize");
    const std::size_t out_words = 3 * (std::size_t)chunks + packed;
    uint32_t* out = make_output(out_words);
    const int pgrid = grid_for(ctx, chunks, PACK_WARPS);
    {
        kernel_timer kt(ctx, "bitpack.pack");
        if (delta)
            k_bp_pack<true><<<pgrid, PACK_THREADS, 0, ctx.stream>>>(in, (uint32_t)n, (uint32_t)chunk, chunks,
                                                              hdr.as<uint32_t>(), offs.as<uint32_t>(), out);
        else
            k_bp_pack<false><<<pgrid, PACK_THREADS, 0, ctx.stream>>>(in, (uint32_t)n, (uint32_t)chunk, chunks,
                                                               hdr.as<uint32_t>(), offs.as<uint32_t>(), out);
        check_cuda(cudaGetLastError(), "bitpack pack launch");
    }
    return out_words;
}

void bitpack_decompress(device_context& ctx, const uint32_t* data, std::size_t words, std::size_t n,
                        std::size_t chunk, bool delta, uint32_t* out)
{
    using namespace bitpack;
    check_chunk(chunk);
    if (n == 0) return;
    check_size(n);
    if (data == nullptr || out == nullptr) throw std::invalid_argument("bitpack: null argument");
    const uint32_t chunks = (uint32_t)((n + chunk - 1) / chunk);
    if (words < 3 * (std::size_t)chunks) throw std::invalid_argument("bitpack: data shorter than its chunk headers");
    ctx.activate();
    uint32_t shift = 0;
    while ((std::size_t(1) << shift) < chunk) ++shift;
    // Delta mode with a mean packed width of at most 16 bits (known from the
    // compressed size): one pass that decodes and sums (the timestamp recipe
    // at 2^28: 0.73 ms against 0.91 for unpack + scan). Wider data, and plain
    // mode, decode faster as 4-element groups (the lane-private form issues
    // W scattered loads per lane: 1.1 ms against 0.42 at 32 bits).
    const uint64_t packed_words = words - 3 * (uint64_t)chunks;
    const bool one_pass = delta && packed_words * 32 <= (uint64_t)n * 16;
    launch_shape sh;
    const int forced = ctx.tuning.lookup("bitpack:unpack", sh) ? sh.variant : -1;  // 0: one pass, 1: two passes
    if (forced == 0 || (forced != 1 && one_pass)) {
        const uint32_t num_tiles = (uint32_t)((n + UTILE - 1) / UTILE);
        uint32_t* tile_ctr = reinterpret_cast<uint32_t*>(ctx.d_small + 3072);
        check_cuda(cudaMemsetAsync(tile_ctr, 0, 4, ctx.stream), "cudaMemsetAsync");
        const uint64_t seq0 = ctx.reserve_seq(num_tiles);
        auto kern = delta ? &k_bp_unpack_tiles<true> : &k_bp_unpack_tiles<false>;
        int per_sm = 1;
        check_cuda(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, UT, 0), "cudaOccupancy");
        const int grid = (int)std::max<std::size_t>(
            1, std::min<std::size_t>(num_tiles, (std::size_t)ctx.sm_count * std::max(per_sm, 1)));
        kernel_timer kt(ctx, "bitpack.unpack");
        kern<<<grid, UT, 0, ctx.stream>>>(data, (uint64_t)words, (uint32_t)n, shift, chunks, out, num_tiles, tile_ctr,
                                          ctx.lookback_ring, seq0, ctx.d_error);
        check_cuda(cudaGetLastError(), "bitpack unpack launch");
        return;
    }
    const std::size_t groups = (n + 3) / 4;
    const int grid = (int)std::max<std::size_t>(
        1, std::min<std::size_t>((groups + THREADS - 1) / THREADS, (std::size_t)ctx.sm_count * 16));
    {
        kernel_timer kt(ctx, "bitpack.unpack");
        if (delta)
            k_bp_unpack<true><<<grid, THREADS, 0, ctx.stream>>>(data, (uint32_t)n, shift, chunks, out);
        else
            k_bp_unpack<false><<<grid, THREADS, 0, ctx.stream>>>(data, (uint32_t)n, shift, chunks, out);
        check_cuda(cudaGetLastError(), "bitpack unpack launch");
    }
    if (delta) {
        const uint32_t zero = 0;
        scan(ctx, out, out, n, elem::u32, op_kind::plus, &zero, false, nullptr);
    }
}

}  // namespace gbc
