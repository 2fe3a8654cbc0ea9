// Device-side building blocks shared by every gbcompute kernel: memory-model
// helpers for the decoupled look-back status words, bounded spin waits,
// order-preserving key bijections and warp/CTA collectives.
//
// The CTA collectives replace the OpenCL work-group macros of the reference
// (CLC_DEFINE_WG_REDUCE / CLC_DEFINE_WG_SCAN in lib/src/Compute/
// DeviceHeaders.cpp:30-85). Those are a local-memory tree reduction and a
// Hillis-Steele scan with two barriers per step; here the same sequence-ordered
// semantics (a precedes b in every `op(a, b)`) come from warp shuffles plus one
// shared-memory exchange of warp totals.
#pragma once

#include <cstdint>
#include <type_traits>
#include <cuda_runtime.h>

namespace gbc {
namespace dev {

constexpr unsigned FULL_MASK = 0xffffffffu;

// Error codes a kernel can leave in the context's device error word. The host
// reads the word at the next synchronising call and reports it.
enum : int {
    ERR_NONE = 0,
    ERR_LOOKBACK_TIMEOUT = 1,  // a decoupled look-back wait gave up
    ERR_BAD_SEGMENT = 2,       // a segment offset table was not monotone
    ERR_LEARNED_OVERFLOW = 3,  // informational: learned sort used its fallback
};

// How long a spin wait on another CTA may last before it records
// ERR_LOOKBACK_TIMEOUT and returns (nanoseconds of %globaltimer).
constexpr unsigned long long SPIN_LIMIT_NS = 1000000000ull;

__device__ __forceinline__ unsigned lanemask_lt()
{
    unsigned m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

__device__ __forceinline__ unsigned long long globaltimer()
{
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ uint32_t ld_relaxed(const uint32_t* p)
{
    uint32_t v;
    asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ uint64_t ld_relaxed(const uint64_t* p)
{
    uint64_t v;
    asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_relaxed(uint32_t* p, uint32_t v)
{
    asm volatile("st.relaxed.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ void st_relaxed(uint64_t* p, uint64_t v)
{
    asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
__device__ __forceinline__ uint32_t ld_acquire(const uint32_t* p)
{
    uint32_t v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_release(uint32_t* p, uint32_t v)
{
    asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ uint64_t ld_acquire(const uint64_t* p)
{
    uint64_t v;
    asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_release(uint64_t* p, uint64_t v)
{
    asm volatile("st.release.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}

// Streaming 128-bit load that does not allocate in L1 (the data is read once).
__device__ __forceinline__ uint4 ld_stream(const uint4* p)
{
    uint4 v;
    asm volatile("ld.global.nc.L1::no_allocate.v4.u32 {%0,%1,%2,%3}, [%4];"
                 : "=r"(v.x), "=r"(v.y), "=r"(v.z), "=r"(v.w)
                 : "l"(p));
    return v;
}

// ---------------------------------------------------------------------------
// Bulk (TMA engine) copies global -> shared, completed on an mbarrier.
// Both addresses must be 16-byte aligned and the size a multiple of 16.
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t smem_addr(const void* p)
{
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void fence_mbar_init()
{
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
// Orders this thread's earlier shared-memory accesses (and, after a CTA
// barrier, the other threads') before a following async-proxy copy.
__device__ __forceinline__ void fence_proxy_async()
{
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar)
{
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smem_addr(dst)),
        "l"(src), "r"(bytes), "r"(smem_addr(bar))
        : "memory");
}
// Bulk prefetch of [p, p + bytes) into L2 (16-byte aligned, size a multiple
// of 16); nothing waits for it.
__device__ __forceinline__ void prefetch_l2(const void* p, uint32_t bytes)
{
    asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(p), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity)
{
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
// Waits for the given phase parity, at most SPIN_LIMIT_NS; false if it gave up.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity)
{
    if (mbar_try_wait(bar, parity)) return true;
    const unsigned long long start = globaltimer();
    for (uint32_t spin = 1;; ++spin) {
        if (mbar_try_wait(bar, parity)) return true;
        if ((spin & 63) == 0 && globaltimer() - start > SPIN_LIMIT_NS) return false;
    }
}

// Records `code` in the error word unless an earlier error is already there.
__device__ __forceinline__ void raise_error(int* err, int code)
{
    if (err != nullptr) atomicCAS(err, ERR_NONE, code);
}

// ---------------------------------------------------------------------------
// Order-preserving bijections to unsigned integers (Algorithm.cpp:459-469):
//   unsigned: k                     signed: k ^ signbit
//   float:    sign ? ~k : k | signbit      descending: ~(the above)
// All four are written as  k ^ (smear(sign(k)) & a) ^ b  so that one kernel
// serves every key type and both orders with two runtime constants.
// ---------------------------------------------------------------------------
template <typename K> struct KeyXform {
    K a, b;
    __host__ __device__ __forceinline__ K operator()(K k) const
    {
        using S = typename std::conditional<sizeof(K) == 4, int32_t, int64_t>::type;
        const K smear = static_cast<K>(static_cast<S>(k) >> (sizeof(K) * 8 - 1));
        return k ^ (smear & a) ^ b;
    }
};

// kind: 0 unsigned, 1 signed, 2 floating point.
template <typename K> inline KeyXform<K> make_xform(int kind, bool descending)
{
    const K sign = K(1) << (sizeof(K) * 8 - 1);
    KeyXform<K> x{0, 0};
    if (kind == 1) x.b = sign;
    if (kind == 2) {
        x.a = ~sign;  // negative: k ^ ~sign ^ sign == ~k
        x.b = sign;   // non-negative: k ^ sign == k | sign
    }
    if (descending) x.b = ~x.b;
    return x;
}

// ---------------------------------------------------------------------------
// Warp collectives with sequence-ordered combination: op(earlier, later).
// ---------------------------------------------------------------------------
template <typename T, typename Op>
__device__ __forceinline__ T warp_inclusive_scan(T x, Op op)
{
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const T y = __shfl_up_sync(FULL_MASK, x, o);
        if (lane >= o) x = op(y, x);
    }
    return x;
}

template <typename T, typename Op>
__device__ __forceinline__ T warp_reduce(T x, Op op)
{
    // Tree over lanes in index order: lane i combines with lane i+o so the
    // left operand always precedes the right one.
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const T y = __shfl_down_sync(FULL_MASK, x, o);
        if (((threadIdx.x & 31) & (2 * o - 1)) == 0) x = op(x, y);
    }
    return __shfl_sync(FULL_MASK, x, 0);
}

// Exclusive sum of one value per thread over the first 256 threads of the CTA
// (the 256 radix bins). Every thread of the CTA must call it; threads >= 256
// contribute nothing. `scratch` holds 8 words.
__device__ __forceinline__ uint32_t bins_exclusive_sum(uint32_t v, uint32_t* scratch,
                                                       uint32_t* total = nullptr)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t x = threadIdx.x < 256 ? v : 0u;
    x = warp_inclusive_scan(x, [](uint32_t a, uint32_t b) { return a + b; });
    if (warp < 8 && lane == 31) scratch[warp] = x;
    __syncthreads();
    uint32_t before = 0, all = 0;
#pragma unroll
    for (int w = 0; w < 8; ++w) {
        const uint32_t s = scratch[w];
        if (w < warp) before += s;
        all += s;
    }
    __syncthreads();
    if (total != nullptr) *total = all;
    return before + x - (threadIdx.x < 256 ? v : 0u);
}

}  // namespace dev
}  // namespace gbc
