// Segmented scan: one single-pass decoupled look-back scan whose running value
// restarts at every segment start. No reference counterpart (the reference
// scans one array per call, lib/src/Compute/Algorithm.cpp:280-318); within a
// segment the semantics are the reference scan's: canonical operator combined
// in sequence order, exclusive output begins with the identity.
//
// Each element carries a head flag (it starts a segment); pairs combine as
//   (fa, va) (+) (fb, vb) = (fa | fb, fb ? vb : op(va, vb)),
// which is associative, so the tile machinery of the plain scan applies. A
// predecessor tile that contains a head already holds a complete prefix, so
// the look-back also stops there.
//
// Head flags come from the offsets: one binary search per tile for the first
// segment starting in the tile, then the tile's starts are set in a shared
// bitmask.
#include <cstring>

#include "device_common.cuh"
#include "ops.cuh"
#include "runtime.hpp"
#include "segmented.hpp"
#include "sort_internal.hpp"

namespace gbc {
namespace {

using dev::FULL_MASK;
constexpr int THREADS = 256;
constexpr uint64_t FLAG_AGG = 1, FLAG_PRE = 2;
constexpr uint64_t TAG_MASK = (1ull << 29) - 1;
constexpr uint64_t HEAD_BIT = 1ull << 61;

template <typename T> __device__ __forceinline__ uint64_t to_bits(T v)
{
    uint64_t b = 0;
    memcpy(&b, &v, sizeof(T));
    return b;
}
template <typename T> __device__ __forceinline__ T from_bits(uint64_t b)
{
    T v;
    memcpy(&v, &b, sizeof(T));
    return v;
}

template <typename T, bool WIDE = (sizeof(T) == 8)> struct SStatus;
template <typename T> struct SStatus<T, false> {
    static constexpr uint64_t SLOTS = onesweep::RING_BYTES / 8;
    __device__ static void publish(uint64_t* ring, uint64_t seq, uint64_t flag, bool head, T v)
    {
        dev::st_relaxed(&ring[seq & (SLOTS - 1)], (flag << 62) | (head ? HEAD_BIT : 0) |
                                                      ((seq & TAG_MASK) << 32) | (uint32_t)to_bits(v));
    }
    __device__ static bool read(const uint64_t* ring, uint64_t seq, uint64_t& flag, bool& head, T& v)
    {
        const uint64_t w = dev::ld_relaxed(&ring[seq & (SLOTS - 1)]);
        flag = w >> 62;
        if (flag == 0 || ((w >> 32) & TAG_MASK) != (seq & TAG_MASK)) return false;
        head = (w & HEAD_BIT) != 0;
        v = from_bits<T>((uint32_t)w);
        return true;
    }
};
template <typename T> struct SStatus<T, true> {
    static constexpr uint64_t SLOTS = onesweep::RING_BYTES / 32;
    __device__ static void publish(uint64_t* ring, uint64_t seq, uint64_t flag, bool head, T v)
    {
        uint64_t* s = ring + (seq & (SLOTS - 1)) * 4;
        dev::st_relaxed(&s[flag == FLAG_PRE ? 1 : 0], to_bits(v));
        dev::st_release(&s[2], (flag << 62) | (head ? HEAD_BIT : 0) | ((seq & TAG_MASK) << 32));
    }
    __device__ static bool read(const uint64_t* ring, uint64_t seq, uint64_t& flag, bool& head, T& v)
    {
        const uint64_t* s = ring + (seq & (SLOTS - 1)) * 4;
        const uint64_t w = dev::ld_acquire(&s[2]);
        flag = w >> 62;
        if (flag == 0 || ((w >> 32) & TAG_MASK) != (seq & TAG_MASK)) return false;
        head = (w & HEAD_BIT) != 0;
        v = from_bits<T>(dev::ld_relaxed(&s[flag == FLAG_PRE ? 1 : 0]));
        return true;
    }
};

template <typename T> struct SegScanArgs {
    const T* in;
    T* out;
    uint32_t n;
    T identity;
    int exclusive;
    int aligned;
    const uint32_t* off;
    uint32_t nseg;
    uint32_t num_tiles;
    uint64_t* ring;
    uint64_t seq0;
    uint32_t* tile_ctr;
    int* err;
};

// Inclusive scan of (flag, value) pairs across a warp, sequence order.
template <typename T, typename Op>
__device__ __forceinline__ void warp_seg_scan(uint32_t& f, T& v, Op op)
{
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const T yv = __shfl_up_sync(FULL_MASK, v, o);
        const uint32_t yf = __shfl_up_sync(FULL_MASK, f, o);
        if (lane >= o) {
            if (!f) v = op(yv, v);
            f |= yf;
        }
    }
}

template <typename T, typename Op>
__global__ void __launch_bounds__(THREADS) k_segscan(SegScanArgs<T> a)
{
    constexpr int VEC = 16 / sizeof(T);
    constexpr int ROWS = sizeof(T) == 4 ? 4 : 8;
    constexpr int TILE = THREADS * VEC * ROWS;
    constexpr int RW = ROWS * (THREADS / 32);
    constexpr int PER = RW / 32;

    __shared__ uint32_t s_head[TILE / 32];
    __shared__ T s_rw[RW];
    __shared__ uint32_t s_rwf[RW];
    __shared__ T s_prefix;
    __shared__ uint32_t s_tile, s_lo;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const Op op;
    const T identity = a.identity;

    for (;;) {
        if (tid == 0) s_tile = atomicAdd(a.tile_ctr, 1u);
        for (int i = tid; i < TILE / 32; i += THREADS) s_head[i] = 0;
        __syncthreads();
        const uint32_t t = s_tile;
        if (t >= a.num_tiles) break;
        const uint32_t base = t * TILE;
        const bool full = base + TILE <= a.n;

        // Segment starts inside [base, base + TILE).
        if (tid == 0) {
            uint32_t lo = 0, hi = a.nseg;  // first i in [0, nseg) with off[i] >= base, else nseg
            while (lo < hi) {
                const uint32_t mid = (lo + hi) >> 1;
                if (a.off[mid] < base) lo = mid + 1;
                else hi = mid;
            }
            s_lo = lo;
            if (base == 0) s_head[0] = 1u;  // position 0 always starts a segment
        }
        __syncthreads();
        for (uint32_t i = s_lo + tid; i < a.nseg; i += THREADS) {
            const uint32_t o = a.off[i];
            if (o >= base + TILE) break;
            if (o < base) continue;  // only with non-monotone offsets
            const uint32_t local = o - base;
            atomicOr(&s_head[local >> 5], 1u << (local & 31));
        }
        __syncthreads();

        T x[ROWS][VEC];
        uint32_t hb[ROWS];  // head bits of the thread's VEC elements, per row
        if (full && a.aligned) {
#pragma unroll
            for (int r = 0; r < ROWS; ++r) {
                const uint4 w = dev::ld_stream(reinterpret_cast<const uint4*>(a.in + base + (r * THREADS + tid) * VEC));
                memcpy(x[r], &w, 16);
            }
        } else {
#pragma unroll
            for (int r = 0; r < ROWS; ++r)
#pragma unroll
                for (int j = 0; j < VEC; ++j) {
                    const uint32_t idx = base + (r * THREADS + tid) * VEC + j;
                    x[r][j] = idx < a.n ? a.in[idx] : identity;
                }
        }
#pragma unroll
        for (int r = 0; r < ROWS; ++r) {
            const uint32_t l0 = (r * THREADS + tid) * VEC;
            hb[r] = (s_head[l0 >> 5] >> (l0 & 31)) & ((1u << VEC) - 1);
        }

        // Thread totals per row, then warp scans of the pairs.
        T wv[ROWS];
        uint32_t wf[ROWS];
#pragma unroll
        for (int r = 0; r < ROWS; ++r) {
            T v = x[r][0];
#pragma unroll
            for (int j = 1; j < VEC; ++j) v = ((hb[r] >> j) & 1) ? x[r][j] : op(v, x[r][j]);
            uint32_t f = hb[r] != 0;
            warp_seg_scan(f, v, op);
            wv[r] = v;
            wf[r] = f;
            if (lane == 31) {
                s_rw[r * (THREADS / 32) + warp] = v;
                s_rwf[r * (THREADS / 32) + warp] = f;
            }
        }
        __syncthreads();

        if (warp == 0) {
            T v[PER];
            uint32_t f[PER];
#pragma unroll
            for (int k = 0; k < PER; ++k) {
                v[k] = s_rw[lane * PER + k];
                f[k] = s_rwf[lane * PER + k];
            }
            T lv = v[0];
            uint32_t lf = f[0];
#pragma unroll
            for (int k = 1; k < PER; ++k) {
                lv = f[k] ? v[k] : op(lv, v[k]);
                lf |= f[k];
            }
            T iv = lv;
            uint32_t iff = lf;
            warp_seg_scan(iff, iv, op);
            const T uv = __shfl_up_sync(FULL_MASK, iv, 1);
            const uint32_t uf = __shfl_up_sync(FULL_MASK, iff, 1);
            // exclusive prefix of each row-warp (entry 0 has none)
            T rv = uv;
            uint32_t rf = lane == 0 ? 0u : uf;
#pragma unroll
            for (int k = 0; k < PER; ++k) {
                s_rw[lane * PER + k] = rv;
                s_rwf[lane * PER + k] = rf;
                if (lane == 0 && k == 0) {
                    rv = v[0];
                    rf = f[0];
                } else {
                    rv = f[k] ? v[k] : op(rv, v[k]);
                    rf |= f[k];
                }
            }
            const T agg = __shfl_sync(FULL_MASK, iv, 31);
            const bool agg_head = __shfl_sync(FULL_MASK, iff, 31) != 0;
            const uint64_t my_seq = a.seq0 + t;
            if (lane == 0) SStatus<T>::publish(a.ring, my_seq, t == 0 ? FLAG_PRE : FLAG_AGG, agg_head, agg);

            T excl = identity;
            if (t > 0) {
                bool have = false;
                int64_t w_end = t;
                for (;;) {
                    const int64_t k = w_end - 32 + lane;
                    uint64_t flag = FLAG_PRE;
                    bool head = true;
                    T val = identity;
                    bool gave_up = false;
                    if (k >= 0) {
                        if (!SStatus<T>::read(a.ring, a.seq0 + (uint64_t)k, flag, head, val)) {
                            const unsigned long long start = dev::globaltimer();
                            for (uint32_t spin = 1;; ++spin) {
                                if (SStatus<T>::read(a.ring, a.seq0 + (uint64_t)k, flag, head, val)) break;
                                if ((spin & 255) == 0 && dev::globaltimer() - start > dev::SPIN_LIMIT_NS) {
                                    gave_up = true;
                                    flag = FLAG_PRE;
                                    head = true;
                                    val = identity;
                                    break;
                                }
                                if (spin > 32) __nanosleep(64);
                            }
                        }
                    }
                    if (__any_sync(FULL_MASK, gave_up) && lane == 0) dev::raise_error(a.err, dev::ERR_LOOKBACK_TIMEOUT);
                    const bool stop = flag == FLAG_PRE || head;
                    const uint32_t stops = __ballot_sync(FULL_MASK, stop);
                    const int L = stops ? 31 - __clz(stops) : 0;
                    uint32_t cf = lane >= L ? (uint32_t)head : 0u;
                    T cv = lane >= L ? val : identity;
                    warp_seg_scan(cf, cv, op);
                    const T wsum = __shfl_sync(FULL_MASK, cv, 31);
                    const bool wflag = __shfl_sync(FULL_MASK, cf, 31) != 0;
                    (void)wflag;
                    // Nearer windows held no head and no prefix (else the walk
                    // would have stopped), so the farther window folds in
                    // front of what has been gathered so far.
                    excl = have ? op(wsum, excl) : wsum;
                    have = true;
                    if (stops) break;
                    w_end -= 32;
                }
                if (lane == 0)
                    SStatus<T>::publish(a.ring, my_seq, FLAG_PRE, true, agg_head ? agg : op(excl, agg));
            }
            if (lane == 0) s_prefix = excl;
        }
        __syncthreads();

        const T prefix = s_prefix;
#pragma unroll
        for (int r = 0; r < ROWS; ++r) {
            const int rw = r * (THREADS / 32) + warp;
            const T wexc = __shfl_up_sync(FULL_MASK, wv[r], 1);
            const uint32_t wexf = __shfl_up_sync(FULL_MASK, wf[r], 1);
            T run = prefix;  // placeholder when nothing precedes (position 0 is a head)
            if (rw != 0) run = s_rwf[rw] ? s_rw[rw] : op(run, s_rw[rw]);
            if (lane > 0) run = wexf ? wexc : op(run, wexc);
            T o[VEC];
#pragma unroll
            for (int j = 0; j < VEC; ++j) {
                const bool head = (hb[r] >> j) & 1;
                const T inc = head ? x[r][j] : op(run, x[r][j]);
                o[j] = a.exclusive ? (head ? identity : run) : inc;
                run = inc;
            }
            if (full && a.aligned) {
                uint4 w;
                memcpy(&w, o, 16);
                *reinterpret_cast<uint4*>(a.out + base + (r * THREADS + tid) * VEC) = w;
            } else {
#pragma unroll
                for (int j = 0; j < VEC; ++j) {
                    const uint32_t idx = base + (r * THREADS + tid) * VEC + j;
                    if (idx < a.n) a.out[idx] = o[j];
                }
            }
        }
        __syncthreads();
    }
}

struct SegScanLaunch {
    device_context& ctx;
    const void* in;
    void* out;
    std::size_t n;
    const void* identity;
    bool exclusive;
    const uint32_t* off;
    std::size_t nseg;

    template <typename T, typename Op> void run()
    {
        constexpr int VEC = 16 / sizeof(T);
        constexpr int ROWS = sizeof(T) == 4 ? 4 : 8;
        constexpr uint32_t TILE = THREADS * VEC * ROWS;
        SegScanArgs<T> a;
        a.in = static_cast<const T*>(in);
        a.out = static_cast<T*>(out);
        a.n = (uint32_t)n;
        std::memcpy(&a.identity, identity, sizeof(T));
        a.exclusive = exclusive ? 1 : 0;
        a.aligned = ((reinterpret_cast<uintptr_t>(in) | reinterpret_cast<uintptr_t>(out)) & 15) == 0;
        a.off = off;
        a.nseg = (uint32_t)nseg;
        a.num_tiles = (uint32_t)((n + TILE - 1) / TILE);
        a.ring = ctx.lookback_ring;
        a.seq0 = ctx.reserve_seq(a.num_tiles);
        a.err = ctx.d_error;
        unsigned char* ctl = ctx.d_small + 256;
        check_cuda(cudaMemsetAsync(ctl, 0, 64, ctx.stream), "cudaMemsetAsync");
        a.tile_ctr = reinterpret_cast<uint32_t*>(ctl);
        auto kernel = &k_segscan<T, Op>;
        int per_sm = 0;
        check_cuda(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, THREADS, 0),
                   "cudaOccupancyMaxActiveBlocksPerMultiprocessor");
        const int grid = (int)std::min<std::size_t>(a.num_tiles, (std::size_t)ctx.sm_count * std::max(per_sm, 1));
        kernel_timer kt(ctx, "segscan.lookback");
        kernel<<<grid, THREADS, 0, ctx.stream>>>(a);
        check_cuda(cudaGetLastError(), "segmented scan launch");
    }
};

}  // namespace

void segmented_scan(device_context& ctx, const void* in, void* out, std::size_t n, elem t, op_kind op,
                    const void* identity, bool exclusive, const uint32_t* offsets, std::size_t num_segments)
{
    if (n == 0) return;
    check_size(n);
    if (in == nullptr || out == nullptr || identity == nullptr || (num_segments > 0 && offsets == nullptr))
        throw std::invalid_argument("segmented_scan: null argument");
    if (num_segments > 0x7FFFFFFFu) throw std::length_error("segmented_scan: too many segments");
    ctx.activate();
    SegScanLaunch l{ctx, in, out, n, identity, exclusive, offsets, num_segments};
    ops::dispatch(t, op, l);
}

}  // namespace gbc
