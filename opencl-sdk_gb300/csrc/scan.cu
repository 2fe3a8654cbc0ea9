// Single-pass inclusive/exclusive scan with decoupled look-back.
//
// Reference path replaced: detail::scan -> scan_impl (lib/src/Compute/
// Algorithm.cpp:280-318, 444-451) with kernels clc_scan_tiles / clc_scan_add
// (79-127): every tile is scanned, the tile totals are scanned recursively and
// added back, i.e. about four passes over the data. Here each element is read
// once and written once: a tile publishes its aggregate as soon as it is
// known, looks back over its predecessors' status words for its exclusive
// prefix and writes its outputs.
//
// Semantics kept: any canonical associative operator, combined in sequence
// order (op(earlier, later)), so non-commutative operators such as the right
// projection work; out may alias in; exclusive output starts with identity.
// Added: a wide total (exact int64/uint64 sum for integer plus-scans of
// 32-bit elements, otherwise the last inclusive value widened).
//
// Tile layout (256 threads): row r, thread t holds VEC consecutive elements
// at tile_base + (r * 256 + t) * VEC, loaded as one 128-bit access. Sequence
// order is row, then thread, then element, so each row is a warp scan and the
// ROWS x 8 row-warp totals are scanned by one warp.
#include <cstring>
#include <map>
#include <mutex>

#include "../../include/compute_c.h"
#include "device_common.cuh"
#include "ops.cuh"
#include "runtime.hpp"
#include "sort_internal.hpp"

namespace gbc {
namespace {

using dev::FULL_MASK;

constexpr int THREADS = 256;
constexpr int LB_PER_LANE = 4;     // look-back window: 32 x 4 tiles per round trip
constexpr int PREFETCH_GRIDS = 1;  // L2 prefetch distance, in grids of tiles (2 measured slower)
constexpr uint64_t FLAG_AGG = 1, FLAG_PRE = 2;
constexpr uint64_t TAG_MASK = (1ull << 30) - 1;

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

// Status of one tile. 32-bit elements: one word (flag | tag | value) that is
// overwritten atomically from AGG to PRE. 64-bit elements: separate words for
// the aggregate and the inclusive prefix, published with release stores
// before the flag word, so a reader never pairs a flag with the wrong value.
template <typename T, bool WIDE = (sizeof(T) == 8)> struct Status;

template <typename T> struct Status<T, false> {
    static constexpr uint64_t SLOTS = onesweep::RING_BYTES / 8;
    __device__ static void publish(uint64_t* ring, uint64_t seq, uint64_t flag, T v)
    {
        dev::st_relaxed(&ring[seq & (SLOTS - 1)],
                        (flag << 62) | ((seq & TAG_MASK) << 32) | (uint32_t)to_bits(v));
    }
    __device__ static bool read(const uint64_t* ring, uint64_t seq, uint64_t& flag, T& v)
    {
        const uint64_t w = dev::ld_relaxed(&ring[seq & (SLOTS - 1)]);
        flag = w >> 62;
        if (flag == 0 || ((w >> 32) & TAG_MASK) != (seq & TAG_MASK)) return false;
        v = from_bits<T>((uint32_t)w);
        return true;
    }
};

template <typename T> struct Status<T, true> {
    static constexpr uint64_t SLOTS = onesweep::RING_BYTES / 32;
    __device__ static void publish(uint64_t* ring, uint64_t seq, uint64_t flag, T v)
    {
        uint64_t* s = ring + (seq & (SLOTS - 1)) * 4;
        dev::st_relaxed(&s[flag == FLAG_PRE ? 1 : 0], to_bits(v));
        dev::st_release(&s[2], (flag << 62) | ((seq & TAG_MASK) << 32));
    }
    __device__ static bool read(const uint64_t* ring, uint64_t seq, uint64_t& flag, T& v)
    {
        const uint64_t* s = ring + (seq & (SLOTS - 1)) * 4;
        const uint64_t w = dev::ld_acquire(&s[2]);
        flag = w >> 62;
        if (flag == 0 || ((w >> 32) & TAG_MASK) != (seq & TAG_MASK)) return false;
        v = from_bits<T>(dev::ld_relaxed(&s[flag == FLAG_PRE ? 1 : 0]));
        return true;
    }
};

template <typename T> struct ScanArgs {
    const T* in;
    T* out;
    uint32_t n;
    T identity;
    int exclusive;
    int aligned;  // in and out are 16-byte aligned
    uint32_t num_tiles;
    uint64_t* ring;
    uint64_t seq0;
    uint32_t* tile_ctr;
    unsigned long long* wide_sum;  // exact sum (integer plus, <= 32-bit), or null
    void* total;                   // last inclusive value widened to 8 bytes, or null
    int* err;
};

template <typename T> __device__ __forceinline__ void store_wide(void* dst, T v)
{
    if (std::is_floating_point<T>::value) {
        const double d = (double)v;
        memcpy(dst, &d, 8);
    } else if (std::is_signed<T>::value) {
        const long long w = (long long)v;
        memcpy(dst, &w, 8);
    } else {
        const unsigned long long w = (unsigned long long)v;
        memcpy(dst, &w, 8);
    }
}

template <typename T, int ROWS_ = 8> struct ScanShape {
    static constexpr int VEC = 16 / sizeof(T);
    static constexpr int ROWS = ROWS_;
    static constexpr int TILE = THREADS * VEC * ROWS;
    static constexpr int RW = ROWS * (THREADS / 32);
    static constexpr int PER = RW / 32;
    static_assert(RW % 32 == 0, "row-warp totals fill whole lanes");
};

// One tile after its elements x are in registers: wide sum, warp scans, the
// row-warp scan and look-back (warp 0), then the outputs. Contains CTA
// barriers: every thread of the CTA calls it.
template <typename T, typename Op, bool WIDE_SUM, int ROWS_>
__device__ __forceinline__ void scan_tile(const ScanArgs<T>& a, T (&x)[ROWS_][ScanShape<T, ROWS_>::VEC],
                                          uint32_t t, uint32_t base, bool full, T* s_rw, T& s_prefix,
                                          unsigned long long& wide)
{
    constexpr int VEC = ScanShape<T, ROWS_>::VEC;
    constexpr int ROWS = ROWS_;
    constexpr int PER = ScanShape<T, ROWS_>::PER;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const Op op;
    const T identity = a.identity;

    if (WIDE_SUM) {
        // Exact sum of the valid elements, widened (mod 2^64), accumulated by
        // the thread over all its tiles and added once at the kernel's end.
#pragma unroll
        for (int r = 0; r < ROWS; ++r)
#pragma unroll
            for (int j = 0; j < VEC; ++j) {
                const uint32_t idx = base + (r * THREADS + tid) * VEC + j;
                if (idx < a.n) {
                    if (std::is_signed<T>::value) wide += (unsigned long long)(long long)x[r][j];
                    else wide += (unsigned long long)x[r][j];
                }
            }
    }

    // Per-row warp scans of the thread totals.
    T winc[ROWS];
#pragma unroll
    for (int r = 0; r < ROWS; ++r) {
        T acc = x[r][0];
#pragma unroll
        for (int j = 1; j < VEC; ++j) acc = op(acc, x[r][j]);
        winc[r] = dev::warp_inclusive_scan(acc, op);
        if (lane == 31) s_rw[r * (THREADS / 32) + warp] = winc[r];
    }
    __syncthreads();

    if (warp == 0) {
        // Exclusive scan of the row-warp totals, in sequence order.
        T v[PER];
#pragma unroll
        for (int k = 0; k < PER; ++k) v[k] = s_rw[lane * PER + k];
        T lt = v[0];
#pragma unroll
        for (int k = 1; k < PER; ++k) lt = op(lt, v[k]);
        const T linc = dev::warp_inclusive_scan(lt, op);
        const T up = __shfl_up_sync(FULL_MASK, linc, 1);
        T run = lane == 0 ? identity : up;
#pragma unroll
        for (int k = 0; k < PER; ++k) {
            s_rw[lane * PER + k] = run;
            run = op(run, v[k]);
        }
        const T agg = __shfl_sync(FULL_MASK, linc, 31);
        const uint64_t my_seq = a.seq0 + t;
        if (lane == 0) Status<T>::publish(a.ring, my_seq, t == 0 ? FLAG_PRE : FLAG_AGG, agg);

        // Warp-cooperative look-back over windows of 32 * LB_PER_LANE
        // preceding tiles (lane l inspects LB_PER_LANE consecutive ones); the
        // nearest tile holding an inclusive prefix ends the walk. Tiles start
        // a few nanoseconds apart, so that prefix is typically a hundred or
        // more tiles back: a wide window finds it in one or two round trips.
        T excl = identity;
        if (t > 0) {
            bool have = false;
            int64_t w_end = t;
            bool gave_up = false;
            for (;;) {
                uint64_t flag[LB_PER_LANE];
                T val[LB_PER_LANE];
#pragma unroll
                for (int q = 0; q < LB_PER_LANE; ++q) {
                    const int64_t k = w_end - 32 * LB_PER_LANE + lane * LB_PER_LANE + q;
                    flag[q] = FLAG_PRE;  // before tile 0: an empty inclusive prefix
                    val[q] = identity;
                    if (k >= 0 && !Status<T>::read(a.ring, a.seq0 + (uint64_t)k, flag[q], val[q])) {
                        const unsigned long long start = dev::globaltimer();
                        for (uint32_t spin = 1;; ++spin) {
                            if (Status<T>::read(a.ring, a.seq0 + (uint64_t)k, flag[q], val[q])) break;
                            if ((spin & 255) == 0 && dev::globaltimer() - start > dev::SPIN_LIMIT_NS) {
                                gave_up = true;
                                flag[q] = FLAG_PRE;
                                val[q] = identity;
                                break;
                            }
                            if (spin > 32) __nanosleep(64);
                        }
                    }
                }
                int hi = -1;  // this lane's nearest inclusive prefix
#pragma unroll
                for (int q = 0; q < LB_PER_LANE; ++q)
                    if (flag[q] == FLAG_PRE) hi = q;
                const uint32_t pre = __ballot_sync(FULL_MASK, hi >= 0);
                const int L = pre ? 31 - __clz(pre) : -1;
                // This lane's part of the window, in sequence order.
                T contrib = identity;
                bool any = false;
                if (lane >= L) {
                    const int q0 = lane == L ? hi : 0;
#pragma unroll
                    for (int q = 0; q < LB_PER_LANE; ++q) {
                        if (q < q0) continue;
                        contrib = any ? op(contrib, val[q]) : val[q];
                        any = true;
                    }
                }
                const T wsum = dev::warp_reduce(contrib, op);
                excl = have ? op(wsum, excl) : wsum;
                have = true;
                if (pre) break;
                w_end -= 32 * LB_PER_LANE;
            }
            if (__any_sync(FULL_MASK, gave_up) && lane == 0) dev::raise_error(a.err, dev::ERR_LOOKBACK_TIMEOUT);
            if (lane == 0) Status<T>::publish(a.ring, my_seq, FLAG_PRE, op(excl, agg));
        }
        if (lane == 0) s_prefix = excl;
    }
    __syncthreads();

    const T prefix = s_prefix;
#pragma unroll
    for (int r = 0; r < ROWS; ++r) {
        const T wexc = __shfl_up_sync(FULL_MASK, winc[r], 1);
        // The first row-warp's exclusive value is the identity; combining
        // it on the right would break operators whose identity only works
        // from the left (the right projection), so it is skipped.
        T run = (r == 0 && warp == 0) ? prefix : op(prefix, s_rw[r * (THREADS / 32) + warp]);
        if (lane > 0) run = op(run, wexc);
        T o[VEC];
#pragma unroll
        for (int j = 0; j < VEC; ++j) {
            const T inc = op(run, x[r][j]);
            o[j] = a.exclusive ? run : inc;
            run = inc;
            if (a.total != nullptr && base + (r * THREADS + tid) * VEC + j == a.n - 1)
                store_wide<T>(a.total, inc);
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
}

// Latency-bound: each SM needs several tiles in flight, so the register
// budget is capped for MINB CTAs per SM (by default 4, 2 for 8-byte
// elements). PF: L2 prefetch distance in grids of tiles (0: none).
template <typename T, typename Op, bool WIDE_SUM, int ROWS_ = 8, int MINB = (sizeof(T) == 4 ? 4 : 2),
          int PF = PREFETCH_GRIDS>
__global__ void __launch_bounds__(THREADS, MINB) k_scan(ScanArgs<T> a)
{
    using S = ScanShape<T, ROWS_>;
    __shared__ T s_rw[S::RW];
    __shared__ T s_prefix;
    __shared__ uint32_t s_tile;
    const int tid = threadIdx.x;
    unsigned long long wide = 0;
    for (;;) {
        // The tile index is taken only when the CTA can start on it (taking
        // it earlier delays its status, measured slower). The tile
        // PREFETCH_GRIDS grids further on, which a CTA will take about that
        // many tile-times from now, is prefetched into L2.
        if (tid == 0) {
            s_tile = atomicAdd(a.tile_ctr, 1u);
            const uint64_t ahead = (uint64_t)s_tile + PF * gridDim.x;
            if (PF > 0 && a.aligned && (ahead + 1) * S::TILE <= a.n)
                dev::prefetch_l2(a.in + ahead * S::TILE, S::TILE * sizeof(T));
        }
        __syncthreads();
        const uint32_t t = s_tile;
        if (t >= a.num_tiles) break;
        const uint32_t base = t * S::TILE;
        const bool full = base + S::TILE <= a.n;
        T x[S::ROWS][S::VEC];
        if (full && a.aligned) {
#pragma unroll
            for (int r = 0; r < S::ROWS; ++r) {
                const uint4 w = dev::ld_stream(reinterpret_cast<const uint4*>(a.in + base + (r * THREADS + tid) * S::VEC));
                memcpy(x[r], &w, 16);
            }
        } else {
#pragma unroll
            for (int r = 0; r < S::ROWS; ++r)
#pragma unroll
                for (int j = 0; j < S::VEC; ++j) {
                    const uint32_t idx = base + (r * THREADS + tid) * S::VEC + j;
                    x[r][j] = idx < a.n ? a.in[idx] : a.identity;
                }
        }
        scan_tile<T, Op, WIDE_SUM, ROWS_>(a, x, t, base, full, s_rw, s_prefix, wide);
        __syncthreads();
    }
    if (WIDE_SUM) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) wide += __shfl_down_sync(FULL_MASK, wide, o);
        if ((tid & 31) == 0 && wide != 0) atomicAdd(a.wide_sum, wide);
    }
}

std::map<std::pair<int, const void*>, int> g_occ;  // (device, kernel): attributes and occupancy are per device
std::mutex g_occ_m;

template <typename F> int blocks_per_sm(F* kernel, std::size_t smem = 0)
{
    int dev = 0;
    check_cuda(cudaGetDevice(&dev), "cudaGetDevice");
    const std::pair<int, const void*> key(dev, (const void*)kernel);
    std::lock_guard<std::mutex> lock(g_occ_m);
    auto it = g_occ.find(key);
    if (it != g_occ.end()) return it->second;
    check_cuda(cudaFuncSetAttribute(kernel, cudaFuncAttributePreferredSharedMemoryCarveout,
                                    (int)cudaSharedmemCarveoutMaxShared),
               "cudaFuncSetAttribute");
    int b = 0;
    check_cuda(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, kernel, THREADS, smem),
               "cudaOccupancyMaxActiveBlocksPerMultiprocessor");
    b = std::max(b, 1);
    g_occ[key] = b;
    return b;
}

struct ScanLaunch {
    device_context& ctx;
    const void* in;
    void* out;
    std::size_t n;
    const void* identity;
    bool exclusive;
    void* total_dev;
    bool wide_plus;

    // Tile shape: 16 rows and 2 CTAs per SM for 4-byte elements, 8 rows for
    // 8-byte ones, L2 prefetch one grid ahead. Measured on GB300 (exclusive
    // int32 plus-scan of 2^30 with its int64 total, ms): 16 rows x 2 CTAs
    // 2.03; 8 x 4 (spills) 2.22; 12 x 3 2.33; 20 x 2 (spills) 2.36; 32 x 1
    // 2.28; 24 x 1 2.48; 4 x 6 2.77; 4 x 8 3.91; prefetch off 2.38, two grids
    // ahead 2.23. For int32 plus-scans the tuning table entry "scan:32"
    // selects 1: 8 rows x 4, 2: 32 rows x 1, 3: 16 rows x 2 without prefetch.
    template <typename T, typename Op> void run()
    {
        if constexpr (std::is_same<T, int32_t>::value && std::is_same<Op, ops::Plus>::value) {
            launch_shape sh;
            switch (ctx.tuning.lookup("scan:32", sh) ? sh.variant : 0) {
            case 1: run_shape<T, Op, 8, 4, 1>(); return;
            case 2: run_shape<T, Op, 32, 1, 1>(); return;
            case 3: run_shape<T, Op, 16, 2, 0>(); return;
            default: break;
            }
        }
        if constexpr (sizeof(T) == 4) run_shape<T, Op, 16, 2, PREFETCH_GRIDS>();
        else run_shape<T, Op, 8, 2, PREFETCH_GRIDS>();
    }

    template <typename T, typename Op, int ROWS_, int MINB, int PF> void run_shape()
    {
        constexpr int VEC = 16 / sizeof(T);
        constexpr uint32_t TILE = ScanShape<T, ROWS_>::TILE;
        constexpr bool can_wide = std::is_integral<T>::value && sizeof(T) == 4 &&
                                  std::is_same<Op, ops::Plus>::value;
        ScanArgs<T> a;
        a.in = static_cast<const T*>(in);
        a.out = static_cast<T*>(out);
        a.n = (uint32_t)n;
        std::memcpy(&a.identity, identity, sizeof(T));
        a.exclusive = exclusive ? 1 : 0;
        a.aligned = ((reinterpret_cast<uintptr_t>(in) | reinterpret_cast<uintptr_t>(out)) & 15) == 0;
        a.num_tiles = (uint32_t)((n + TILE - 1) / TILE);
        a.ring = ctx.lookback_ring;
        a.seq0 = ctx.reserve_seq(a.num_tiles);
        a.err = ctx.d_error;
        // Control block: tile counter + wide sum, in the context's small area.
        unsigned char* ctl = ctx.d_small;
        check_cuda(cudaMemsetAsync(ctl, 0, 64, ctx.stream), "cudaMemsetAsync");
        a.tile_ctr = reinterpret_cast<uint32_t*>(ctl);
        a.wide_sum = reinterpret_cast<unsigned long long*>(ctl + 8);
        const bool use_wide = can_wide && total_dev != nullptr;
        a.total = use_wide ? nullptr : total_dev;
        if (!use_wide) a.wide_sum = nullptr;

        // A bulk-copy staged form of this kernel measured slower: a CTA that
        // takes its next tile early publishes that tile's status late, which
        // stalls every successor's look-back.
        auto kernel = use_wide ? &k_scan<T, Op, can_wide, ROWS_, MINB, PF> : &k_scan<T, Op, false, ROWS_, MINB, PF>;
        const std::size_t smem = 0;
        const int grid =
            (int)std::min<std::size_t>(a.num_tiles, (std::size_t)ctx.sm_count * blocks_per_sm(kernel, smem));
        {
            kernel_timer kt(ctx, "scan.lookback");
            kernel<<<grid, THREADS, smem, ctx.stream>>>(a);
            check_cuda(cudaGetLastError(), "scan launch");
        }
        if (use_wide)
            check_cuda(cudaMemcpyAsync(total_dev, a.wide_sum, 8, cudaMemcpyDeviceToDevice, ctx.stream),
                       "cudaMemcpyAsync");
    }
};

}  // namespace

void selftest_lookback_timeout(device_context& ctx)
{
    // A two-tile int32 plus-scan whose only CTA starts at tile 1: tile 0 never
    // runs, so its status word never appears and the bounded wait must give
    // up, record ERR_LOOKBACK_TIMEOUT and let the kernel finish. Every access
    // stays inside the two-tile buffer.
    ctx.activate();
    constexpr uint32_t TILE = ScanShape<int32_t>::TILE;
    temp_buffer buf(ctx.resource, 2 * TILE * sizeof(int32_t));
    check_cuda(cudaMemsetAsync(buf.get(), 0, 2 * TILE * sizeof(int32_t), ctx.stream), "cudaMemsetAsync");
    unsigned char* ctl = ctx.d_small;
    check_cuda(cudaMemsetAsync(ctl, 0, 64, ctx.stream), "cudaMemsetAsync");
    check_cuda(cudaMemsetAsync(ctl, 1, 1, ctx.stream), "cudaMemsetAsync");  // tile counter = 1
    ScanArgs<int32_t> a;
    a.in = buf.as<int32_t>();
    a.out = buf.as<int32_t>();
    a.n = 2 * TILE;
    a.identity = 0;
    a.exclusive = 0;
    a.aligned = 1;
    a.num_tiles = 2;
    a.ring = ctx.lookback_ring;
    a.seq0 = ctx.reserve_seq(2);
    a.tile_ctr = reinterpret_cast<uint32_t*>(ctl);
    a.wide_sum = nullptr;
    a.total = nullptr;
    a.err = ctx.d_error;
    k_scan<int32_t, ops::Plus, false><<<1, THREADS, 0, ctx.stream>>>(a);
    check_cuda(cudaGetLastError(), "scan launch");
}

void scan(device_context& ctx, const void* in, void* out, std::size_t n, elem t, op_kind op,
          const void* identity, bool exclusive, void* total_dev)
{
    if (n == 0) return;
    check_size(n);
    if (in == nullptr || out == nullptr || identity == nullptr)
        throw std::invalid_argument("scan: null argument");
    ctx.activate();
    ScanLaunch l{ctx, in, out, n, identity, exclusive, total_dev, false};
    ops::dispatch(t, op, l);
}

// ---------------------------------------------------------------------------
// Allocation-free int32 scan (clc_scan_i32_noalloc).
//
// Some callers cannot allocate device memory when they need a scan: an
// embedder whose device memory belongs to another allocator (a framework's
// caching allocator, or a fixed arena on a GPU shared with other jobs) must
// not call cudaMalloc behind that allocator's back, and cudaFree synchronises
// the whole device, which a latency-bound caller cannot afford. This entry
// point therefore keeps its scratch -- the look-back status word of every
// tile, the tile counter and an error word -- in a fixed array compiled into
// the library, and it needs no clc_context (creating one allocates). The
// caller passes the input, the output and the stream.
//
// The array holds 16,384 tiles of 16,384 elements (the int32 tile shape of
// the pooled scan): at most 2^28 elements per call (128 KiB of status words,
// held by every GPU that loads the library until the process exits). Every
// call shares it and it keeps the last call's contents, so each call first
// clears the words it will read; calls whose work overlaps on the GPU
// (different streams, or different host threads) race on it and must be
// serialised by the caller.
//
// A look-back wait that runs out (about one second: only a GPU that stalls a
// predecessor tile that long) makes the kernel skip the writes that depend on
// it and set the error word; the call has already returned by then, so
// clc_scan_i32_noalloc_status reports it (and clears it) afterwards.
// ---------------------------------------------------------------------------
namespace noalloc {

constexpr int ROWS = 16, MINB = 2;  // the int32 shape of the pooled scan
constexpr uint32_t TILE = ScanShape<int32_t, ROWS>::TILE;
constexpr std::size_t MAX_ELEMENTS = std::size_t(1) << 28;
constexpr uint32_t MAX_TILES = (uint32_t)(MAX_ELEMENTS / TILE);

// [0, MAX_TILES): status word of each tile; [MAX_TILES]: the tile counter;
// [MAX_TILES + 1]: the error word (an int in its low half, sticky until
// clc_scan_i32_noalloc_status clears it).
constexpr uint32_t CTR_WORD = MAX_TILES, ERR_WORD = MAX_TILES + 1;
static __device__ __align__(256) uint64_t scan_scratch[MAX_TILES + 32];

struct device_setup {
    uint64_t* scratch = nullptr;  // device address of scan_scratch on this device
    int grid_cap = 0;             // SMs x resident CTAs of the scan kernel
};
std::mutex g_mutex;
std::map<int, device_setup> g_setup;

// Once per device, with that device current: the host-side name of
// scan_scratch is only a stand-in, so its device address is looked up here
// and handed to the kernel.
device_setup setup_current_device(int dev)
{
    std::lock_guard<std::mutex> lock(g_mutex);
    auto it = g_setup.find(dev);
    if (it != g_setup.end()) return it->second;
    device_setup s;
    void* p = nullptr;
    check_cuda(cudaGetSymbolAddress(&p, scan_scratch), "cudaGetSymbolAddress");
    s.scratch = static_cast<uint64_t*>(p);
    int sms = 0, blocks = 0;
    check_cuda(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev), "cudaDeviceGetAttribute");
    check_cuda(cudaOccupancyMaxActiveBlocksPerMultiprocessor(
                   &blocks, &k_scan<int32_t, ops::Plus, false, ROWS, MINB, PREFETCH_GRIDS>, THREADS, 0),
               "cudaOccupancyMaxActiveBlocksPerMultiprocessor");
    s.grid_cap = sms * std::max(blocks, 1);
    g_setup[dev] = s;
    return s;
}


// Argument checks shared by the entry points below: the stream and any
// device-memory pointer must belong to the current device, whose scratch
// array and grid size the call uses.
int check_device(void* stream, const void* const* ptrs, int count, std::string& why)
{
    int dev = 0;
    check_cuda(cudaGetDevice(&dev), "cudaGetDevice");
    int sdev = dev;
    if (stream != nullptr) check_cuda(cudaStreamGetDevice(static_cast<cudaStream_t>(stream), &sdev), "cudaStreamGetDevice");
    if (sdev != dev) {
        why = "the stream belongs to device " + std::to_string(sdev) + ", not the current device " + std::to_string(dev);
        return -1;
    }
    for (int i = 0; i < count; ++i) {
        cudaPointerAttributes pa{};
        if (cudaPointerGetAttributes(&pa, ptrs[i]) != cudaSuccess) {
            (void)cudaGetLastError();
            continue;  // not memory the runtime knows: the caller's responsibility
        }
        if (pa.type == cudaMemoryTypeDevice && pa.device != dev) {
            why = "a pointer is device memory of device " + std::to_string(pa.device) + ", not the current device " +
                  std::to_string(dev);
            return -1;
        }
    }
    return dev;
}

void launch(const device_setup& s, const int32_t* in, int32_t* out, std::size_t n, bool exclusive, cudaStream_t st,
            uint32_t first_tile)
{
    const uint32_t num_tiles = (uint32_t)((n + TILE - 1) / TILE);
    // Clear what this call reads before it is written: the tile counter
    // and the status words of its tiles (an earlier call left its own).
    // The error word is left alone: it stays set until it is read.
    check_cuda(cudaMemsetAsync(s.scratch, 0, (std::size_t)num_tiles * sizeof(uint64_t), st), "cudaMemsetAsync");
    check_cuda(cudaMemsetAsync(s.scratch + CTR_WORD, 0, sizeof(uint64_t), st), "cudaMemsetAsync");
    if (first_tile != 0)
        check_cuda(cudaMemsetAsync(s.scratch + CTR_WORD, (int)first_tile, 1, st), "cudaMemsetAsync");
    ScanArgs<int32_t> a;
    a.in = in;
    a.out = out;
    a.n = (uint32_t)n;
    a.identity = 0;
    a.exclusive = exclusive ? 1 : 0;
    a.aligned = ((reinterpret_cast<uintptr_t>(in) | reinterpret_cast<uintptr_t>(out)) & 15) == 0;
    a.num_tiles = num_tiles;
    a.ring = s.scratch;  // tile t uses word t (sequence numbers start at 0)
    a.seq0 = 0;
    a.tile_ctr = reinterpret_cast<uint32_t*>(s.scratch + CTR_WORD);
    a.wide_sum = nullptr;
    a.total = nullptr;
    a.err = reinterpret_cast<int*>(s.scratch + ERR_WORD);
    const uint32_t tiles_left = num_tiles - std::min(first_tile, num_tiles);
    const int grid = (int)std::max<uint32_t>(1, std::min<uint32_t>(tiles_left, (uint32_t)s.grid_cap));
    k_scan<int32_t, ops::Plus, false, ROWS, MINB, PREFETCH_GRIDS><<<grid, THREADS, 0, st>>>(a);
    check_cuda(cudaGetLastError(), "clc_scan_i32_noalloc launch");
}

template <typename F> clc_status guarded(F&& f)
{
    try {
        return f();
    } catch (const device_error& e) {
        return (clc_status)set_last_error(CLC_ERROR_OPENCL, e.what(), e.code);
    } catch (const std::exception& e) {
        return (clc_status)set_last_error(CLC_ERROR_INTERNAL, e.what(), 0);
    }
}

}  // namespace noalloc

}  // namespace gbc

extern "C" clc_status clc_scan_i32_noalloc(const int32_t* in, int32_t* out, size_t n, int exclusive, void* stream)
{
    using namespace gbc;
    return noalloc::guarded([&]() -> clc_status {
        if (n == 0) return (clc_status)set_last_error(CLC_SUCCESS, "", 0);
        if (n > noalloc::MAX_ELEMENTS)
            return (clc_status)set_last_error(
                CLC_ERROR_INVALID_ARGUMENT,
                ("clc_scan_i32_noalloc: n = " + std::to_string(n) +
                 " exceeds the 268435456 (2^28) elements its built-in scratch covers")
                    .c_str(),
                0);
        if (in == nullptr || out == nullptr)
            return (clc_status)set_last_error(CLC_ERROR_INVALID_ARGUMENT, "clc_scan_i32_noalloc: null pointer", 0);
        std::string why;
        const void* ptrs[2] = {in, out};
        const int dev = noalloc::check_device(stream, ptrs, 2, why);
        if (dev < 0)
            return (clc_status)set_last_error(CLC_ERROR_INVALID_ARGUMENT, ("clc_scan_i32_noalloc: " + why).c_str(), 0);
        const noalloc::device_setup s = noalloc::setup_current_device(dev);
        noalloc::launch(s, in, out, n, exclusive != 0, static_cast<cudaStream_t>(stream), 0);
        return (clc_status)set_last_error(CLC_SUCCESS, "", 0);
    });
}

extern "C" clc_status clc_scan_i32_noalloc_status(void* stream)
{
    using namespace gbc;
    return noalloc::guarded([&]() -> clc_status {
        std::string why;
        const int dev = noalloc::check_device(stream, nullptr, 0, why);
        if (dev < 0)
            return (clc_status)set_last_error(CLC_ERROR_INVALID_ARGUMENT,
                                              ("clc_scan_i32_noalloc_status: " + why).c_str(), 0);
        const noalloc::device_setup s = noalloc::setup_current_device(dev);
        cudaStream_t st = static_cast<cudaStream_t>(stream);
        int word = 0;  // pageable destination: the copy completes before it returns
        check_cuda(cudaMemcpyAsync(&word, s.scratch + noalloc::ERR_WORD, sizeof(int), cudaMemcpyDeviceToHost, st),
                   "cudaMemcpyAsync");
        check_cuda(cudaStreamSynchronize(st), "cudaStreamSynchronize");
        if (word == 0) return (clc_status)set_last_error(CLC_SUCCESS, "", 0);
        check_cuda(cudaMemsetAsync(s.scratch + noalloc::ERR_WORD, 0, sizeof(uint64_t), st), "cudaMemsetAsync");
        check_cuda(cudaStreamSynchronize(st), "cudaStreamSynchronize");
        return (clc_status)set_last_error(CLC_ERROR_OPENCL,
                                          "clc_scan_i32_noalloc: a look-back wait timed out; the output of an "
                                          "earlier call on this device is incomplete",
                                          0);
    });
}

extern "C" clc_status clc_selftest_noalloc_timeout(int32_t* buf, size_t n, void* stream)
{
    using namespace gbc;
    return noalloc::guarded([&]() -> clc_status {
        // Two or more tiles scanned with the tile counter starting at 1: tile
        // 0 never runs, so tile 1's bounded wait must give up and set the
        // error word. Every access stays inside the caller's n elements.
        if (buf == nullptr || n < 2 * (std::size_t)noalloc::TILE || n > noalloc::MAX_ELEMENTS)
            return (clc_status)set_last_error(CLC_ERROR_INVALID_ARGUMENT,
                                              "clc_selftest_noalloc_timeout: needs 2 to 16384 tiles of 16384 int32",
                                              0);
        std::string why;
        const void* ptrs[1] = {buf};
        const int dev = noalloc::check_device(stream, ptrs, 1, why);
        if (dev < 0)
            return (clc_status)set_last_error(CLC_ERROR_INVALID_ARGUMENT,
                                              ("clc_selftest_noalloc_timeout: " + why).c_str(), 0);
        const noalloc::device_setup s = noalloc::setup_current_device(dev);
        noalloc::launch(s, buf, buf, n, false, static_cast<cudaStream_t>(stream), 1);
        return (clc_status)set_last_error(CLC_SUCCESS, "", 0);
    });
}
