// fill and sequence (lib/src/Compute/Algorithm.cpp:16-27 kernels clc_fill /
// clc_sequence, host side 331-359): out[i] = value and out[i] = start + i *
// step. One grid-stride kernel per element size; sequence computes in the
// element type, like the reference's `start + (T)i * step`.
#include <cstring>

#include "device_common.cuh"
#include "runtime.hpp"

namespace gbc {
namespace {

template <typename W>
__global__ void k_fill(W* __restrict__ out, std::size_t n, W value)
{
    const std::size_t stride = (std::size_t)gridDim.x * blockDim.x;
    for (std::size_t i = (std::size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride)
        out[i] = value;
}

template <typename T>
__global__ void k_sequence(T* __restrict__ out, std::size_t n, T start, T step)
{
    const std::size_t stride = (std::size_t)gridDim.x * blockDim.x;
    for (std::size_t i = (std::size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride)
        out[i] = start + (T)(uint32_t)i * step;
}

int grid_for(const device_context& ctx, std::size_t n)
{
    const std::size_t want = (n + 255) / 256;
    return (int)std::max<std::size_t>(1, std::min<std::size_t>(want, (std::size_t)ctx.sm_count * 8));
}

template <typename T>
void launch_sequence(device_context& ctx, void* out, std::size_t n, const void* start,
                     const void* step)
{
    T s, d;
    std::memcpy(&s, start, sizeof(T));
    std::memcpy(&d, step, sizeof(T));
    k_sequence<T><<<grid_for(ctx, n), 256, 0, ctx.stream>>>(static_cast<T*>(out), n, s, d);
}

}  // namespace

void fill(device_context& ctx, void* out, std::size_t n, elem t, const void* value)
{
    if (n == 0) return;
    check_size(n);
    ctx.activate();
    const std::size_t sz = elem_size(t);
    // A 1-, 2- or 4-byte pattern is replicated to 4 bytes when n allows;
    // otherwise fill element by element.
    kernel_timer kt(ctx, "fill");
    switch (sz) {
    case 1: {
        uint8_t v;
        std::memcpy(&v, value, 1);
        check_cuda(cudaMemsetAsync(out, v, n, ctx.stream), "cudaMemsetAsync");
        return;
    }
    case 2: {
        uint16_t v;
        std::memcpy(&v, value, 2);
        k_fill<uint16_t><<<grid_for(ctx, n), 256, 0, ctx.stream>>>(static_cast<uint16_t*>(out), n, v);
        break;
    }
    case 4: {
        uint32_t v;
        std::memcpy(&v, value, 4);
        k_fill<uint32_t><<<grid_for(ctx, n), 256, 0, ctx.stream>>>(static_cast<uint32_t*>(out), n, v);
        break;
    }
    default: {
        uint64_t v;
        std::memcpy(&v, value, 8);
        k_fill<uint64_t><<<grid_for(ctx, n), 256, 0, ctx.stream>>>(static_cast<uint64_t*>(out), n, v);
        break;
    }
    }
    check_cuda(cudaGetLastError(), "fill launch");
}

void sequence(device_context& ctx, void* out, std::size_t n, elem t, const void* start,
              const void* step)
{
    if (n == 0) return;
    check_size(n);
    ctx.activate();
    kernel_timer kt(ctx, "sequence");
    switch (t) {
    case elem::i8: launch_sequence<int8_t>(ctx, out, n, start, step); break;
    case elem::u8: launch_sequence<uint8_t>(ctx, out, n, start, step); break;
    case elem::i16: launch_sequence<int16_t>(ctx, out, n, start, step); break;
    case elem::u16: launch_sequence<uint16_t>(ctx, out, n, start, step); break;
    case elem::i32: launch_sequence<int32_t>(ctx, out, n, start, step); break;
    case elem::u32: launch_sequence<uint32_t>(ctx, out, n, start, step); break;
    case elem::i64: launch_sequence<int64_t>(ctx, out, n, start, step); break;
    case elem::u64: launch_sequence<uint64_t>(ctx, out, n, start, step); break;
    case elem::f32: launch_sequence<float>(ctx, out, n, start, step); break;
    case elem::f64: launch_sequence<double>(ctx, out, n, start, step); break;
    }
    check_cuda(cudaGetLastError(), "sequence launch");
}

}  // namespace gbc
