// static_map: a fixed-capacity GPU hash map from 32-bit keys to 32-bit values.
//
// Reference path replaced: cl::compute::static_map (lib/include/CL/Compute/
// HashMap.hpp, lib/src/Compute/HashMap.cpp:16-184) with kernels
// clc_map_insert / clc_map_find / clc_map_contains. Kept, because callers
// observe them: open addressing with linear probing over a power-of-two table
// (capacity rounded up, at least 2, at most 2^31), the MurmurHash3 32-bit
// finalizer as the hash (the reference's clc_hash_u32, DeviceHeaders.cpp:
// 136-145, the published fmix32), empty_key marking free slots and never
// inserted, empty_value returned for missing keys, the first value stored for
// a key kept by later inserts (which count nothing), a probe walk that ends at
// an empty slot, and insert reporting how many keys were new while a full
// table fails the call with the number it could not place.
//
// Here each slot is one 64-bit word, key in the low half and value in the
// high half, claimed with one 64-bit compare-and-swap: a lookup reads one
// word per probe (the reference reads the key array, then the value array),
// and a slot's key and value appear together. Inserted and failed counts are
// aggregated per warp (one atomic per warp instead of one per key). The
// separate key and value arrays of the reference (slot_keys(), slot_values())
// are produced on request by an unzip kernel.
#include <algorithm>
#include <stdexcept>
#include <string>

#include "device_common.cuh"
#include "runtime.hpp"

namespace gbc {
namespace hashmap {

constexpr int THREADS = 256;

__device__ __forceinline__ uint32_t fmix32(uint32_t k)
{
    k ^= k >> 16;
    k *= 0x85ebca6bu;
    k ^= k >> 13;
    k *= 0xc2b2ae35u;
    k ^= k >> 16;
    return k;
}

__device__ __forceinline__ uint64_t pack(uint32_t key, uint32_t value) { return ((uint64_t)value << 32) | key; }

__global__ void __launch_bounds__(THREADS) k_map_fill(unsigned long long* slots, uint64_t count, uint64_t empty)
{
    for (uint64_t i = (uint64_t)blockIdx.x * THREADS + threadIdx.x; i < count; i += (uint64_t)gridDim.x * THREADS)
        slots[i] = empty;
}

// counters[0]: keys newly inserted, counters[1]: keys not placed (table full)
__global__ void __launch_bounds__(THREADS)
    k_map_insert(const uint32_t* __restrict__ keys, const uint32_t* __restrict__ values, uint32_t n,
                 unsigned long long* slots, uint32_t mask, uint32_t empty_key, uint32_t empty_value,
                 unsigned int* counters)
{
    const unsigned long long empty = pack(empty_key, empty_value);
    const uint32_t stride = gridDim.x * THREADS;
    const uint32_t rounds = (n + stride - 1) / stride;
    const int lane = threadIdx.x & 31;
    for (uint32_t r = 0; r < rounds; ++r) {
        const uint32_t i = r * stride + blockIdx.x * THREADS + threadIdx.x;
        bool added = false, failed = false;
        if (i < n) {
            const uint32_t key = keys[i];
            if (key != empty_key) {
                const unsigned long long mine = pack(key, values[i]);
                uint32_t slot = fmix32(key) & mask;
                failed = true;
                for (uint32_t probe = 0; probe <= mask; ++probe) {
                    unsigned long long seen = slots[slot];
                    if ((uint32_t)seen == empty_key) seen = atomicCAS(&slots[slot], empty, mine);
                    if (seen == empty) {
                        added = true, failed = false;
                        break;
                    }
                    if ((uint32_t)seen == key) {  // present: the first value stays
                        failed = false;
                        break;
                    }
                    slot = (slot + 1) & mask;
                }
            }
        }
        const uint32_t a = __ballot_sync(dev::FULL_MASK, added), f = __ballot_sync(dev::FULL_MASK, failed);
        if (lane == 0) {
            if (a) atomicAdd(&counters[0], (unsigned)__popc(a));
            if (f) atomicAdd(&counters[1], (unsigned)__popc(f));
        }
    }
}

// The slot holding key, or mask + 1 when absent (the walk ends at an empty slot).
__device__ __forceinline__ uint64_t probe(const unsigned long long* __restrict__ slots, uint32_t mask, uint32_t key,
                                          uint32_t empty_key, uint32_t& value)
{
    if (key == empty_key) return (uint64_t)mask + 1;
    uint32_t slot = fmix32(key) & mask;
    for (uint32_t p = 0; p <= mask; ++p) {
        const unsigned long long w = __ldg(slots + slot);
        if ((uint32_t)w == key) {
            value = (uint32_t)(w >> 32);
            return slot;
        }
        if ((uint32_t)w == empty_key) break;
        slot = (slot + 1) & mask;
    }
    return (uint64_t)mask + 1;
}

__global__ void __launch_bounds__(THREADS)
    k_map_find(const uint32_t* __restrict__ keys, uint32_t n, const unsigned long long* __restrict__ slots,
               uint32_t mask, uint32_t empty_key, uint32_t empty_value, uint32_t* __restrict__ out)
{
    for (uint32_t i = blockIdx.x * THREADS + threadIdx.x; i < n; i += gridDim.x * THREADS) {
        uint32_t v = empty_value;
        probe(slots, mask, keys[i], empty_key, v);
        out[i] = v;
    }
}

__global__ void __launch_bounds__(THREADS)
    k_map_contains(const uint32_t* __restrict__ keys, uint32_t n, const unsigned long long* __restrict__ slots,
                   uint32_t mask, uint32_t empty_key, uint8_t* __restrict__ out)
{
    for (uint32_t i = blockIdx.x * THREADS + threadIdx.x; i < n; i += gridDim.x * THREADS) {
        uint32_t v = 0;
        out[i] = probe(slots, mask, keys[i], empty_key, v) <= mask ? 1 : 0;
    }
}

__global__ void __launch_bounds__(THREADS)
    k_map_unzip(const unsigned long long* __restrict__ slots, uint64_t count, uint32_t* __restrict__ keys,
                uint32_t* __restrict__ values)
{
    for (uint64_t i = (uint64_t)blockIdx.x * THREADS + threadIdx.x; i < count; i += (uint64_t)gridDim.x * THREADS) {
        const unsigned long long w = slots[i];
        if (keys != nullptr) keys[i] = (uint32_t)w;
        if (values != nullptr) values[i] = (uint32_t)(w >> 32);
    }
}

int grid(device_context& ctx, uint64_t work)
{
    return (int)std::max<uint64_t>(1, std::min<uint64_t>((work + THREADS - 1) / THREADS, (uint64_t)ctx.sm_count * 8));
}

}  // namespace hashmap

std::size_t static_map_slots(std::size_t capacity)
{
    if (capacity > (std::size_t(1) << 31)) throw std::length_error("static_map: capacity above 2^31");
    std::size_t c = 2;
    while (c < capacity) c <<= 1;
    return c;
}

void static_map_clear(device_context& ctx, void* slots, std::size_t capacity, uint32_t empty_key,
                      uint32_t empty_value)
{
    using namespace hashmap;
    ctx.activate();
    kernel_timer kt(ctx, "static_map.clear");
    k_map_fill<<<grid(ctx, capacity), THREADS, 0, ctx.stream>>>(static_cast<unsigned long long*>(slots), capacity,
                                                              ((uint64_t)empty_value << 32) | empty_key);
    check_cuda(cudaGetLastError(), "static_map clear launch");
}

std::size_t static_map_insert(device_context& ctx, void* slots, std::size_t capacity, uint32_t empty_key,
                              uint32_t empty_value, const uint32_t* keys, const uint32_t* values, std::size_t n,
                              std::size_t& not_placed)
{
    using namespace hashmap;
    not_placed = 0;
    if (n == 0) return 0;
    check_size(n);
    if (keys == nullptr || values == nullptr) throw std::invalid_argument("static_map::insert: null keys or values");
    ctx.activate();
    unsigned int* counters = reinterpret_cast<unsigned int*>(ctx.d_small);
    check_cuda(cudaMemsetAsync(counters, 0, 8, ctx.stream), "cudaMemsetAsync");
    {
        kernel_timer kt(ctx, "static_map.insert");
        k_map_insert<<<grid(ctx, n), THREADS, 0, ctx.stream>>>(keys, values, (uint32_t)n,
                                                             static_cast<unsigned long long*>(slots),
                                                             (uint32_t)(capacity - 1), empty_key, empty_value,
                                                             counters);
        check_cuda(cudaGetLastError(), "static_map insert launch");
    }
    unsigned int* h = static_cast<unsigned int*>(ctx.pinned);
    check_cuda(cudaMemcpyAsync(h, counters, 8, cudaMemcpyDeviceToHost, ctx.stream), "cudaMemcpyAsync");
    check_cuda(cudaStreamSynchronize(ctx.stream), "cudaStreamSynchronize");
    not_placed = h[1];
    return h[0];
}

void static_map_find(device_context& ctx, const void* slots, std::size_t capacity, uint32_t empty_key,
                     uint32_t empty_value, const uint32_t* keys, std::size_t n, uint32_t* out)
{
    using namespace hashmap;
    if (n == 0) return;
    check_size(n);
    if (keys == nullptr || out == nullptr) throw std::invalid_argument("static_map::find: null argument");
    ctx.activate();
    kernel_timer kt(ctx, "static_map.find");
    k_map_find<<<grid(ctx, n), THREADS, 0, ctx.stream>>>(keys, (uint32_t)n,
                                                        static_cast<const unsigned long long*>(slots),
                                                        (uint32_t)(capacity - 1), empty_key, empty_value, out);
    check_cuda(cudaGetLastError(), "static_map find launch");
}

void static_map_contains(device_context& ctx, const void* slots, std::size_t capacity, uint32_t empty_key,
                         const uint32_t* keys, std::size_t n, uint8_t* out)
{
    using namespace hashmap;
    if (n == 0) return;
    check_size(n);
    if (keys == nullptr || out == nullptr) throw std::invalid_argument("static_map::contains: null argument");
    ctx.activate();
    kernel_timer kt(ctx, "static_map.contains");
    k_map_contains<<<grid(ctx, n), THREADS, 0, ctx.stream>>>(keys, (uint32_t)n,
                                                            static_cast<const unsigned long long*>(slots),
                                                            (uint32_t)(capacity - 1), empty_key, out);
    check_cuda(cudaGetLastError(), "static_map contains launch");
}

void static_map_unzip(device_context& ctx, const void* slots, std::size_t capacity, uint32_t* keys, uint32_t* values)
{
    using namespace hashmap;
    ctx.activate();
    kernel_timer kt(ctx, "static_map.unzip");
    k_map_unzip<<<grid(ctx, capacity), THREADS, 0, ctx.stream>>>(static_cast<const unsigned long long*>(slots),
                                                               capacity, keys, values);
    check_cuda(cudaGetLastError(), "static_map unzip launch");
}

}  // namespace gbc
