// Single-launch reduce: result = op(init, fold(in)).
//
// Reference path replaced: detail::reduce (lib/src/Compute/Algorithm.cpp:
// 400-442) with kernel clc_reduce (58-74): up to 256 work-groups fold a
// grid-stride slice each, a second launch folds the partials and applies
// init, and the result is read back blocking. Here one launch does both: each
// CTA folds a grid-stride slice with 128-bit loads, the last CTA to finish
// (an atomic ticket) folds the partials in CTA order and applies init once.
// Like the reference, the combination order is fixed but unspecified, so the
// operator must be commutative; integer results are exact, floating-point
// sums are deterministic run to run but may round differently from a
// sequential sum.
#include <cstring>

#include "device_common.cuh"
#include "ops.cuh"
#include "runtime.hpp"

namespace gbc {
namespace {

using dev::FULL_MASK;
constexpr int THREADS = 256;

template <typename T, typename Op>
__global__ void __launch_bounds__(THREADS)
    k_reduce(const T* __restrict__ in, uint32_t n, T identity, T init, T* partials,
             uint32_t* ticket, T* result)
{
    constexpr int VEC = 16 / sizeof(T);
    const Op op;
    __shared__ T s_warp[THREADS / 32];
    __shared__ bool s_last;
    T acc = identity;
    const uint32_t gtid = blockIdx.x * THREADS + threadIdx.x, stride = gridDim.x * THREADS;
    uint32_t head = 0;
    if ((reinterpret_cast<uintptr_t>(in) & 15) == 0) {
        const uint32_t nv = n / VEC;
        const uint4* vin = reinterpret_cast<const uint4*>(in);
        uint32_t v = gtid;
        // four 128-bit loads in flight per thread before they are folded
        for (; (uint64_t)v + 3ull * stride < nv; v += 4 * stride) {
            uint4 w[4];
#pragma unroll
            for (int q = 0; q < 4; ++q) w[q] = dev::ld_stream(vin + v + q * stride);
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                T e[VEC];
                memcpy(e, &w[q], 16);
#pragma unroll
                for (int j = 0; j < VEC; ++j) acc = op(acc, e[j]);
            }
        }
        for (; v < nv; v += stride) {
            const uint4 w = dev::ld_stream(vin + v);
            T e[VEC];
            memcpy(e, &w, 16);
#pragma unroll
            for (int j = 0; j < VEC; ++j) acc = op(acc, e[j]);
        }
        head = nv * VEC;
    }
    for (uint32_t i = head + gtid; i < n; i += stride) acc = op(acc, in[i]);

    acc = dev::warp_reduce(acc, op);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) s_warp[warp] = acc;
    __syncthreads();
    if (warp == 0) {
        T v = lane < THREADS / 32 ? s_warp[lane] : identity;
        v = dev::warp_reduce(v, op);
        if (lane == 0) {
            partials[blockIdx.x] = v;
            __threadfence();
            s_last = atomicAdd(ticket, 1u) == gridDim.x - 1;
        }
    }
    __syncthreads();
    if (!s_last) return;
    __threadfence();
    // Last CTA: fold the partials in CTA order.
    if (warp == 0) {
        T v = identity;
        for (uint32_t b = lane; b < gridDim.x; b += 32) {
            volatile T* p = partials + b;
            v = op(v, *p);
        }
        v = dev::warp_reduce(v, op);
        if (lane == 0) *result = op(init, v);
    }
}

struct ReduceLaunch {
    device_context& ctx;
    const void* in;
    std::size_t n;
    const void* identity;
    const void* init;
    void* result_host;

    template <typename T, typename Op> void run()
    {
        T id, ini;
        std::memcpy(&id, identity, sizeof(T));
        std::memcpy(&ini, init, sizeof(T));
        constexpr int VEC = 16 / sizeof(T);
        const std::size_t work = (n + (std::size_t)THREADS * VEC - 1) / ((std::size_t)THREADS * VEC);
        const int grid = (int)std::max<std::size_t>(1, std::min<std::size_t>(work, (std::size_t)ctx.sm_count * 4));
        temp_buffer partials(ctx.resource, (std::size_t)grid * sizeof(T));
        unsigned char* ctl = ctx.d_small;
        check_cuda(cudaMemsetAsync(ctl, 0, 64, ctx.stream), "cudaMemsetAsync");
        T* dres = reinterpret_cast<T*>(ctl + 16);
        {
            kernel_timer kt(ctx, "reduce.single_pass");
            k_reduce<T, Op><<<grid, THREADS, 0, ctx.stream>>>(static_cast<const T*>(in), (uint32_t)n, id, ini,
                                                              partials.as<T>(), reinterpret_cast<uint32_t*>(ctl), dres);
            check_cuda(cudaGetLastError(), "reduce launch");
        }
        check_cuda(cudaMemcpyAsync(ctx.pinned, dres, sizeof(T), cudaMemcpyDeviceToHost, ctx.stream),
                   "cudaMemcpyAsync");
        ctx.finish();
        std::memcpy(result_host, ctx.pinned, sizeof(T));
    }
};

}  // namespace

void reduce(device_context& ctx, const void* in, std::size_t n, elem t, op_kind op,
            const void* identity, const void* init, void* result_host)
{
    if (n == 0) {
        std::memcpy(result_host, init, elem_size(t));
        return;
    }
    check_size(n);
    ctx.activate();
    ReduceLaunch l{ctx, in, n, identity, init, result_host};
    ops::dispatch(t, op, l);
}

}  // namespace gbc
