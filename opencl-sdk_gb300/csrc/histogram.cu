// histogram_even: counts in[i] into `bins` equal-width bins over [lower, upper).
//
// Reference path replaced: detail::histogram_even (lib/src/Compute/
// Algorithm.cpp:569-615) with kernel clc_histogram (240-273). The bin rule is
// kept operation for operation, because it decides bit-exact parity at bin
// edges: ACC is float unless the input is double; x = (ACC)in[i]; samples
// with !(x >= lower && x < upper) are ignored; b = (uint)((x - lower) * scale)
// with scale = (ACC)bins / (upper - lower) computed on the device in ACC;
// b >= bins is clamped to bins - 1. The histogram is zeroed first.
//
// The reference privatises the histogram in local memory when it fits and
// otherwise uses global atomics. Here: per-warp shared sub-histograms with
// shared atomics when bins x 8 warps fit in 64 KiB, one shared histogram per
// CTA while it fits in the opt-in shared memory, else global atomics; inputs
// are read with 128-bit loads (16 samples per load for u8). For 8- and 16-bit
// integer inputs whose bin rule reduces exactly to value - offset (checked on
// the host over every value of the type), the float arithmetic is skipped.
// (Lane-private 16-bit counters, bank-conflict free but 64 KiB per 4 warps,
// measured slower: occupancy. Four or eight interleaved copies of each
// warp's histogram, lane l counting into copy l % copies, measured no faster
// for 2^30 bytes (0.41 / 0.37 ms against 0.38) and slower for floats: the
// shared atomic instruction rate, not bank conflicts, is the limit.)
#include <cmath>
#include <cstring>
#include <limits>

#include "device_common.cuh"
#include "runtime.hpp"

namespace gbc {
namespace {

constexpr int THREADS = 256;
constexpr int WARPS = THREADS / 32;

enum class mode : int { per_warp = 0, per_cta = 1, global = 2 };

template <typename T, typename ACC, int MODE, bool OFFSET>
__global__ void __launch_bounds__(THREADS)
    k_histogram(const T* __restrict__ in, uint32_t n, uint32_t* __restrict__ hist, uint32_t bins,
                ACC lower, ACC upper, int offset)
{
    constexpr int VEC = 16 / sizeof(T);
    extern __shared__ uint32_t sh[];
    const uint32_t copies = MODE == 0 ? WARPS : 1;
    if (MODE != 2) {
        for (uint32_t i = threadIdx.x; i < bins * copies; i += THREADS) sh[i] = 0;
        __syncthreads();
    }
    uint32_t* target = MODE == 2 ? hist : sh + (MODE == 0 ? (threadIdx.x >> 5) * bins : 0);
    const ACC scale = (ACC)bins / (upper - lower);
    auto count = [&](T v) {
        if (OFFSET) {
            const uint32_t b = (uint32_t)((int)v - offset);
            if (b < bins) atomicAdd(&target[b], 1u);
            return;
        }
        const ACC x = (ACC)v;
        if (x >= lower && x < upper) {
            uint32_t b = (uint32_t)((x - lower) * scale);
            if (b >= bins) b = bins - 1;
            atomicAdd(&target[b], 1u);
        }
    };
    const uint32_t gtid = blockIdx.x * THREADS + threadIdx.x, stride = gridDim.x * THREADS;
    uint32_t head = 0;
    if ((reinterpret_cast<uintptr_t>(in) & 15) == 0) {
        const uint32_t nv = n / VEC;
        const uint4* vin = reinterpret_cast<const uint4*>(in);
        uint32_t v = gtid;
        // four 128-bit loads in flight per thread before they are counted
        for (; (uint64_t)v + 3ull * stride < nv; v += 4 * stride) {
            uint4 w[4];
#pragma unroll
            for (int q = 0; q < 4; ++q) w[q] = dev::ld_stream(vin + v + q * stride);
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                T e[VEC];
                memcpy(e, &w[q], 16);
#pragma unroll
                for (int j = 0; j < VEC; ++j) count(e[j]);
            }
        }
        for (; v < nv; v += stride) {
            const uint4 w = dev::ld_stream(vin + v);
            T e[VEC];
            memcpy(e, &w, 16);
#pragma unroll
            for (int j = 0; j < VEC; ++j) count(e[j]);
        }
        head = nv * VEC;
    }
    for (uint32_t i = head + gtid; i < n; i += stride) count(in[i]);
    if (MODE != 2) {
        __syncthreads();
        for (uint32_t b = threadIdx.x; b < bins; b += THREADS) {
            uint32_t s = 0;
            for (uint32_t c = 0; c < copies; ++c) s += sh[c * bins + b];
            if (s != 0) atomicAdd(&hist[b], s);
        }
    }
}

// True when, for every value v of T, the device's float rule gives exactly
// bin v - offset (or excludes v exactly when v - offset is outside [0, bins)).
// Evaluated over all 2^8 / 2^16 values with the same float operations the
// kernel performs.
template <typename T, typename ACC> bool offset_rule(uint32_t bins, ACC lo, ACC hi, int& offset)
{
    if (!std::is_integral<T>::value || sizeof(T) > 2) return false;
    if (!(std::floor((double)lo) == (double)lo) || std::fabs((double)lo) > 65536.0) return false;
    offset = (int)lo;
    const ACC scale = (ACC)bins / (hi - lo);
    const int64_t first = std::numeric_limits<T>::min(), last = std::numeric_limits<T>::max();
    for (int64_t v = first; v <= last; ++v) {
        const ACC x = (ACC)(T)v;
        int64_t fb = -1;
        if (x >= lo && x < hi) {
            volatile ACC d = x - lo;  // one rounding per operation, as on the device
            volatile ACC p = d * scale;
            uint32_t b = (uint32_t)p;
            if (b >= bins) b = bins - 1;
            fb = b;
        }
        const int64_t ib = v - offset;
        const int64_t want = (ib >= 0 && ib < (int64_t)bins) ? ib : -1;
        if (fb != want) return false;
    }
    return true;
}

template <typename T>
void launch(device_context& ctx, const void* in, uint32_t n, uint32_t* hist, uint32_t bins,
            double lower, double upper)
{
    using ACC = typename std::conditional<std::is_same<T, double>::value, double, float>::type;
    const ACC lo = static_cast<ACC>(lower), hi = static_cast<ACC>(upper);
    constexpr int VEC = 16 / sizeof(T);
    const std::size_t warp_bytes = (std::size_t)bins * 4 * WARPS;
    const std::size_t cta_bytes = (std::size_t)bins * 4;
    int m;
    std::size_t smem;
    if (warp_bytes <= 64 * 1024) m = 0, smem = warp_bytes;
    else if (cta_bytes + 1024 <= ctx.smem_optin) m = 1, smem = cta_bytes;
    else m = 2, smem = 0;
    int offset = 0;
    const bool use_offset = offset_rule<T, ACC>(bins, lo, hi, offset);
    void (*kernel)(const T*, uint32_t, uint32_t*, uint32_t, ACC, ACC, int) =
        use_offset ? (m == 0 ? &k_histogram<T, ACC, 0, true> : m == 1 ? &k_histogram<T, ACC, 1, true>
                                                                       : &k_histogram<T, ACC, 2, true>)
                   : (m == 0 ? &k_histogram<T, ACC, 0, false> : m == 1 ? &k_histogram<T, ACC, 1, false>
                                                                        : &k_histogram<T, ACC, 2, false>);
    if (smem > 0)  // static shared memory adds to this against the 48 KiB default
        check_cuda(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem),
                   "cudaFuncSetAttribute");
    int per_sm = 0;
    check_cuda(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, THREADS, smem),
               "cudaOccupancyMaxActiveBlocksPerMultiprocessor");
    const std::size_t work = ((std::size_t)n + (std::size_t)THREADS * VEC - 1) / ((std::size_t)THREADS * VEC);
    const int grid = (int)std::max<std::size_t>(1, std::min<std::size_t>(work, (std::size_t)ctx.sm_count * std::max(per_sm, 1)));
    kernel_timer kt(ctx, "histogram.even");
    kernel<<<grid, THREADS, smem, ctx.stream>>>(static_cast<const T*>(in), n, hist, bins, lo, hi, offset);
    check_cuda(cudaGetLastError(), "histogram launch");
}

}  // namespace

void histogram_even(device_context& ctx, const void* in, std::size_t n, elem t, uint32_t* hist,
                    std::size_t bins, double lower, double upper)
{
    if (bins == 0) return;
    if (!(lower < upper)) throw std::invalid_argument("histogram_even: lower must be below upper");
    check_size(n);
    if (bins > 0xFFFFFFFFu) throw std::invalid_argument("histogram_even: too many bins");
    ctx.activate();
    check_cuda(cudaMemsetAsync(hist, 0, bins * sizeof(uint32_t), ctx.stream), "cudaMemsetAsync");
    if (n == 0) return;
    const uint32_t nn = (uint32_t)n, b = (uint32_t)bins;
    switch (t) {
    case elem::i8: launch<int8_t>(ctx, in, nn, hist, b, lower, upper); break;
    case elem::u8: launch<uint8_t>(ctx, in, nn, hist, b, lower, upper); break;
    case elem::i16: launch<int16_t>(ctx, in, nn, hist, b, lower, upper); break;
    case elem::u16: launch<uint16_t>(ctx, in, nn, hist, b, lower, upper); break;
    case elem::i32: launch<int32_t>(ctx, in, nn, hist, b, lower, upper); break;
    case elem::u32: launch<uint32_t>(ctx, in, nn, hist, b, lower, upper); break;
    case elem::i64: launch<int64_t>(ctx, in, nn, hist, b, lower, upper); break;
    case elem::u64: launch<uint64_t>(ctx, in, nn, hist, b, lower, upper); break;
    case elem::f32: launch<float>(ctx, in, nn, hist, b, lower, upper); break;
    case elem::f64: launch<double>(ctx, in, nn, hist, b, lower, upper); break;
    }
}

}  // namespace gbc
