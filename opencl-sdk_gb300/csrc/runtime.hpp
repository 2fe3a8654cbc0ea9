// Host runtime of gbcompute: the execution context (device + stream + memory
// resource + tuning table + resident scratch), the CUDA upstream memory
// resource, error types and the internal C++ entry points of every algorithm.
//
// The reference's compute_context bundles an in-order cl::CommandQueue, a
// memory_resource and a JIT program_cache
// (lib/include/CL/Compute/Context.hpp:25-59, MemoryResource.cpp:169-197).
// Here the queue is a CUDA stream, temporaries come from a stream-ordered
// slab arena over cudaMallocAsync, and the program cache is replaced by
// kernels compiled ahead of time for sm_103a plus a tuning table of launch
// shapes.
#pragma once

#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>
#include <functional>
#include <map>
#include <memory>
#include <mutex>
#include <stdexcept>
#include <string>
#include <vector>

#include "arena.hpp"

namespace gbc {

// ---- errors ---------------------------------------------------------------

//! A CUDA runtime failure (the reference's cl::Error); code is the
//! cudaError_t, reported through clc_last_cl_error().
struct device_error : std::runtime_error {
    int code;
    device_error(const std::string& what, int c) : std::runtime_error(what), code(c) {}
};
struct unsupported_error : std::runtime_error {
    using std::runtime_error::runtime_error;
};
struct no_device_error : std::runtime_error {
    using std::runtime_error::runtime_error;
};
//! An expression that OpenCL C would reject (the reference's build_error,
//! ProgramCache.hpp:28); the message carries a "build log" line.
struct build_error : std::runtime_error {
    using std::runtime_error::runtime_error;
};

//! Throws out_of_memory for allocation failures and device_error otherwise.
void check_cuda(cudaError_t e, const char* what);

//! True the first time it is called for `kernel` on the current device
//! (thread-safe): for one-time per-device kernel setup such as the
//! shared-memory opt-in, which CUDA keeps per device.
bool first_use_on_device(const void* kernel);

//! Kernels index elements with 32-bit integers: at most 2^31-1 per call
//! (lib/src/Compute/Detail.hpp:18-23).
void check_size(std::size_t n);

// ---- memory ---------------------------------------------------------------

//! Owns the CUDA stream. Held by the context and by every memory resource
//! built on it, so buffers may outlive the context that made them.
struct stream_holder {
    int device = 0;
    cudaStream_t stream = nullptr;
    bool owned = false;
    ~stream_holder();
};

//! Stream-ordered upstream: cudaMallocAsync / cudaFreeAsync on the context's
//! stream (rmm::mr::cuda_async_memory_resource analogue).
class cuda_async_resource final : public memory_resource {
public:
    explicit cuda_async_resource(std::shared_ptr<stream_holder> s) : s_(std::move(s)) {}
    //! Frees what was handed back while the stream was being captured.
    void flush_deferred();

protected:
    // While the stream is being captured into a CUDA graph, an allocation
    // would become a graph node whose memory the pool must not keep: it is
    // refused (warm the pool by running the call once first), and frees are
    // deferred until the capture ends.
    void* do_allocate(std::size_t bytes) override;
    void do_deallocate(void* p, std::size_t bytes) noexcept override;

private:
    bool capturing() const;
    std::shared_ptr<stream_holder> s_;
    std::mutex m_;
    std::vector<void*> deferred_;
};

// ---- tuning table (replaces the JIT program cache) ------------------------

//! Launch shape of one kernel family, picked by the autotuner.
struct launch_shape {
    int variant = 0;  // index into the family's compiled variant list
};

class tuning_table {
public:
    //! Key: "<op>:<dtype>:<size class>[:<distribution>]".
    bool lookup(const std::string& key, launch_shape& out) const;
    void store(const std::string& key, const launch_shape& s);
    void load(const std::string& path);   // missing file is not an error
    void save(const std::string& path) const;
    std::size_t size() const;
    static std::string size_class(std::size_t n);  // "2^k" of the next power of two

private:
    mutable std::mutex m_;
    std::map<std::string, launch_shape> entries_;
};

// ---- profiler -------------------------------------------------------------

//! Optional per-kernel timing: when enabled, every kernel launch of the
//! library is bracketed by CUDA events on the context's stream and its
//! duration is accumulated under the kernel family's name. Off by default;
//! reading the totals synchronises the stream.
class profiler {
public:
    struct total {
        unsigned long long launches = 0;
        double ms = 0;
    };
    bool enabled() const { return enabled_; }
    void enable(bool on) { enabled_ = on; }
    //! Returns a slot to pass to stop(), or -1 when disabled.
    int start(cudaStream_t s, const char* name);
    void stop(cudaStream_t s, int slot);
    //! Resolves pending events (blocking) and returns the totals.
    std::map<std::string, total> totals(cudaStream_t s);
    void reset(cudaStream_t s);
    ~profiler();

private:
    struct pending {
        std::string name;
        cudaEvent_t a, b;
    };
    cudaEvent_t get_event();
    void resolve(cudaStream_t s);
    bool enabled_ = false;
    std::vector<pending> pending_;
    std::vector<cudaEvent_t> free_;
    std::map<std::string, total> totals_;
    std::mutex m_;
};

struct device_context;

//! Brackets one kernel launch for the context's profiler.
class kernel_timer {
public:
    kernel_timer(device_context& ctx, const char* name);                       // on the context's stream
    kernel_timer(device_context& ctx, const char* name, cudaStream_t stream);  // on another stream of it
    ~kernel_timer();
    kernel_timer(const kernel_timer&) = delete;
    kernel_timer& operator=(const kernel_timer&) = delete;

private:
    device_context& ctx_;
    cudaStream_t stream_;
    int slot_;
};

// ---- context --------------------------------------------------------------

struct device_context {
    int device = 0;
    int sm_count = 0;
    std::size_t smem_optin = 0;
    std::size_t global_memory = 0;
    std::string name;
    std::shared_ptr<stream_holder> holder;
    cudaStream_t stream = nullptr;
    std::shared_ptr<stream_arena> arena;        // temporaries and buffers
    std::shared_ptr<memory_resource> resource;  // == arena: what algorithms allocate from
    tuning_table tuning;
    std::string tuning_path;
    profiler prof;

    // Resident scratch, allocated once per context.
    int* d_error = nullptr;         // device error word (see dev::ERR_*)
    uint64_t* lookback_ring = nullptr;  // decoupled look-back status ring
    uint64_t ring_seq = 0;          // next look-back sequence number
    unsigned char* d_small = nullptr;   // 64 KiB of per-call control blocks
    void* pinned = nullptr;         // 64 KiB of pinned host staging

    // A second stream for independent work inside one call (forked from and
    // joined back to `stream` with the two events), created on first use.
    cudaStream_t aux = nullptr;
    cudaEvent_t fork_event = nullptr, join_event = nullptr;
    cudaStream_t aux_stream();

    device_context(int device, cudaStream_t external_stream,
                   const stream_arena::config& arena_cfg, const std::string& tuning_dir);
    ~device_context();
    device_context(const device_context&) = delete;
    device_context& operator=(const device_context&) = delete;

    void activate() const;  // cudaSetDevice(device)
    //! Reserves `count` consecutive look-back sequence numbers. Tags are 30
    //! bits wide: before they would wrap, the ring is cleared (stream-ordered)
    //! so that no stale word can carry a matching tag.
    uint64_t reserve_seq(uint64_t count);
    //! True while the context's stream is being captured into a CUDA graph.
    bool capturing() const;
    std::shared_ptr<cuda_async_resource> upstream;
    //! Synchronises the stream and reports a kernel-recorded error, if any.
    void finish();
    //! Reads and clears the device error word (synchronises the stream).
    int take_device_error();
};

//! The arena's settings on a device with `global_memory` bytes: idle space
//! kept for reuse up to 1/8 of HBM (at least 1 GiB; one 2^28-pair sort needs
//! 2 GiB of temporaries); CLC_POOL_MAX_CACHED_BYTES overrides the limit.
stream_arena::config default_arena_config(std::size_t global_memory);

// ---- algorithms (internal C++ entry points) -------------------------------
// Every function enqueues on ctx.stream and returns without synchronising
// unless stated otherwise. Pointers are device pointers.

enum class elem : int { i8, u8, i16, u16, i32, u32, i64, u64, f32, f64 };
std::size_t elem_size(elem t);

enum class op_kind : int { plus, multiplies, bit_and, bit_or, bit_xor, minimum, maximum, right, left };

void fill(device_context& ctx, void* out, std::size_t n, elem t, const void* value);
void sequence(device_context& ctx, void* out, std::size_t n, elem t, const void* start,
              const void* step);

//! Stable LSD radix sort. key_kind: 0 unsigned, 1 signed, 2 float; key_bytes
//! 4 or 8. keys_in == keys_out (and vals_in == vals_out) sorts in place.
//! vals may be null. Values are 32-bit.
void radix_sort(device_context& ctx, const void* keys_in, void* keys_out, int key_bytes,
                int key_kind, const uint32_t* vals_in, uint32_t* vals_out, std::size_t n,
                bool descending);

//! Scan with a canonical operator. `identity` points to one element; `total`
//! (device, may be null) receives the wide (int64/uint64/double) sum of the
//! whole input for plus-scans of 8/16/32-bit integers, else the last
//! inclusive value widened.
void scan(device_context& ctx, const void* in, void* out, std::size_t n, elem t, op_kind op,
          const void* identity, bool exclusive, void* total_dev);

//! Reduce: op(init, fold(in)); blocking, result to host.
void reduce(device_context& ctx, const void* in, std::size_t n, elem t, op_kind op,
            const void* identity, const void* init, void* result_host);

void histogram_even(device_context& ctx, const void* in, std::size_t n, elem t,
                    uint32_t* hist, std::size_t bins, double lower, double upper);

//! Runs of equal adjacent keys (4- or 8-byte): per run its key, the uint64
//! sum of its uint32 values and (if counts_out) its length, in run order;
//! hist (65536 bins, or null) counts key & 0xFFFF of every key; the number of
//! runs goes to num_runs_device (or nowhere if null). Asynchronous.
void reduce_by_key(device_context& ctx, const void* keys, int key_bytes, const uint32_t* vals, std::size_t n,
                   void* keys_out, unsigned long long* sums_out, uint32_t* counts_out, uint32_t* hist,
                   uint32_t* num_runs_device);

//! Bitpack compression of n uint32 (the reference's chunk format, see
//! bitpack.cu): analyzes and scans, then asks make_output for a device
//! buffer of the exact compressed size in words, packs into it and returns
//! that size. Synchronises once (to learn the size).
std::size_t bitpack_compress(device_context& ctx, const uint32_t* in, std::size_t n, std::size_t chunk, bool delta,
                             const std::function<uint32_t*(std::size_t)>& make_output);
//! Decodes n elements of compressed data (`words` words) into out. Asynchronous.
void bitpack_decompress(device_context& ctx, const uint32_t* data, std::size_t words, std::size_t n,
                        std::size_t chunk, bool delta, uint32_t* out);
//! Upper bound of the compressed size in words (3 per chunk + n).
std::size_t bitpack_words_bound(std::size_t n, std::size_t chunk);

//! static_map (static_map.cu): slots are `capacity` 64-bit words (key low,
//! value high); capacity is a power of two from static_map_slots.
std::size_t static_map_slots(std::size_t capacity);
void static_map_clear(device_context& ctx, void* slots, std::size_t capacity, uint32_t empty_key,
                      uint32_t empty_value);
//! Blocks; returns the keys newly inserted, the keys it could not place in not_placed.
std::size_t static_map_insert(device_context& ctx, void* slots, std::size_t capacity, uint32_t empty_key,
                              uint32_t empty_value, const uint32_t* keys, const uint32_t* values, std::size_t n,
                              std::size_t& not_placed);
void static_map_find(device_context& ctx, const void* slots, std::size_t capacity, uint32_t empty_key,
                     uint32_t empty_value, const uint32_t* keys, std::size_t n, uint32_t* out);
void static_map_contains(device_context& ctx, const void* slots, std::size_t capacity, uint32_t empty_key,
                         const uint32_t* keys, std::size_t n, uint8_t* out);
void static_map_unzip(device_context& ctx, const void* slots, std::size_t capacity, uint32_t* keys,
                      uint32_t* values);

//! Launches one scan tile whose predecessor never publishes (the failure
//! path of the bounded look-back wait); the next finish() reports it.
void selftest_lookback_timeout(device_context& ctx);

//! Records a clc_status and message as the calling thread's last error (for
//! C entry points defined outside capi.cpp); returns the status.
int set_last_error(int status, const char* msg, int native);

}  // namespace gbc
