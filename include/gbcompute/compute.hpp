/*
 * gbcompute C++ interface: the reference's C++ algorithm API
 * (lib/include/CL/Compute/Algorithm.hpp:27-250, DeviceBuffer.hpp:26-132,
 * Context.hpp:25-59 of the OpenCL Compute library) written over this
 * library's C ABI (compute_c.h), header-only.
 *
 * Same namespace (cl::compute), function names, template signatures,
 * default arguments, static_asserts and exceptions as the reference:
 *   - sizes that do not fit (an output smaller than its input, too few
 *     values) throw std::invalid_argument before anything is enqueued;
 *   - more than 2^31-1 elements throw std::length_error;
 *   - a device_buffer range outside the buffer throws std::out_of_range;
 *   - an expression that does not parse throws build_error (its message has
 *     the "build log" line), one outside the compiled subset
 *     unsupported_error, a device failure device_error (with the
 *     cudaError_t), an allocation failure out_of_memory.
 * What differs, because the device is a CUDA GPU instead of an OpenCL queue:
 *   - compute_context is made from a device index (and optionally a tuning
 *     directory, the program cache's replacement) instead of a
 *     cl::CommandQueue; ctx.queue() returns the context's command_queue,
 *     which device_buffer's copy_from_host / copy_to_host take as the
 *     reference's take a cl::CommandQueue, and whose finish() waits;
 *   - device_buffer::get() is the clc_buffer handle, data() the device
 *     pointer; copies always block (the blocking flag is accepted);
 *   - memory resources and the program cache are not exposed: temporaries
 *     come from the context's stream-ordered arena, kernels are compiled
 *     ahead of time.
 *
 * Link with -lgbcompute (opencl-sdk_gb300/libgbcompute.so).
 */
#ifndef GBCOMPUTE_COMPUTE_HPP
#define GBCOMPUTE_COMPUTE_HPP

#include <cstddef>
#include <cstdint>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <utility>
#include <vector>

#include "../compute_c.h"

/* The OpenCL scalar names the reference's API is written with, unless the
 * OpenCL headers have already declared them (the same types). */
#ifndef __CL_PLATFORM_H
typedef int8_t cl_char;
typedef uint8_t cl_uchar;
typedef int16_t cl_short;
typedef uint16_t cl_ushort;
typedef int32_t cl_int;
typedef uint32_t cl_uint;
typedef int64_t cl_long;
typedef uint64_t cl_ulong;
typedef float cl_float;
typedef double cl_double;
#endif

namespace cl {
namespace compute {

// ---- errors ----------------------------------------------------------------

//! A device runtime failure; native() is the cudaError_t (the reference
//! reports OpenCL failures as cl::Error with the cl_int code).
class device_error : public std::runtime_error {
public:
    device_error(const std::string& what, int native) : std::runtime_error(what), native_(native) {}
    int native() const { return native_; }

private:
    int native_;
};
//! An expression that is not valid OpenCL C (the reference's build_error,
//! ProgramCache.hpp:28): the message carries a "build log" line.
struct build_error : std::runtime_error {
    using std::runtime_error::runtime_error;
};
//! Valid OpenCL C outside what the ahead-of-time kernels implement, or an
//! unsupported element type.
struct unsupported_error : std::runtime_error {
    using std::runtime_error::runtime_error;
};
struct out_of_memory : std::runtime_error {
    using std::runtime_error::runtime_error;
};
struct no_device_error : std::runtime_error {
    using std::runtime_error::runtime_error;
};

namespace detail {

//! Turns a C status into the exception the reference throws for that case.
inline void check(clc_status s)
{
    if (s == CLC_SUCCESS) return;
    const std::string msg = clc_last_error();
    switch (s) {
    case CLC_ERROR_INVALID_ARGUMENT: throw std::invalid_argument(msg);
    case CLC_ERROR_BUILD: throw build_error(msg);
    case CLC_ERROR_UNSUPPORTED: throw unsupported_error(msg);
    case CLC_ERROR_OUT_OF_MEMORY: throw out_of_memory(msg);
    case CLC_ERROR_NO_DEVICE: throw no_device_error(msg);
    case CLC_ERROR_OPENCL: throw device_error(msg, clc_last_cl_error());
    default: throw std::runtime_error(msg);
    }
}

//! Kernels index with 32-bit integers (Detail.hpp:18-23).
inline void check_size(std::size_t n)
{
    if (n > 0x7FFFFFFFu) throw std::length_error("gbcompute: at most 2^31-1 elements per call");
}

template <typename T> struct type_of;
template <> struct type_of<int8_t> { static constexpr clc_type value = CLC_TYPE_I8; };
template <> struct type_of<uint8_t> { static constexpr clc_type value = CLC_TYPE_U8; };
template <> struct type_of<int16_t> { static constexpr clc_type value = CLC_TYPE_I16; };
template <> struct type_of<uint16_t> { static constexpr clc_type value = CLC_TYPE_U16; };
template <> struct type_of<int32_t> { static constexpr clc_type value = CLC_TYPE_I32; };
template <> struct type_of<uint32_t> { static constexpr clc_type value = CLC_TYPE_U32; };
template <> struct type_of<int64_t> { static constexpr clc_type value = CLC_TYPE_I64; };
template <> struct type_of<uint64_t> { static constexpr clc_type value = CLC_TYPE_U64; };
template <> struct type_of<float> { static constexpr clc_type value = CLC_TYPE_F32; };
template <> struct type_of<double> { static constexpr clc_type value = CLC_TYPE_F64; };

}  // namespace detail

// ---- operators (Algorithm.hpp:27-65) -----------------------------------------

//! Associative binary operator: an OpenCL C expression of a and b and its
//! identity. The C interface matches the expression against its table of
//! canonical operators; anything else is unsupported_error.
struct binary_op {
    std::string expression;
    std::string identity;
};

namespace ops {
template <typename T> struct limits;
template <> struct limits<int8_t> {
    static const char* lowest() { return "CHAR_MIN"; }
    static const char* highest() { return "CHAR_MAX"; }
};
template <> struct limits<uint8_t> {
    static const char* lowest() { return "0"; }
    static const char* highest() { return "UCHAR_MAX"; }
};
template <> struct limits<int16_t> {
    static const char* lowest() { return "SHRT_MIN"; }
    static const char* highest() { return "SHRT_MAX"; }
};
template <> struct limits<uint16_t> {
    static const char* lowest() { return "0"; }
    static const char* highest() { return "USHRT_MAX"; }
};
template <> struct limits<int32_t> {
    static const char* lowest() { return "INT_MIN"; }
    static const char* highest() { return "INT_MAX"; }
};
template <> struct limits<uint32_t> {
    static const char* lowest() { return "0"; }
    static const char* highest() { return "UINT_MAX"; }
};
template <> struct limits<int64_t> {
    static const char* lowest() { return "LONG_MIN"; }
    static const char* highest() { return "LONG_MAX"; }
};
template <> struct limits<uint64_t> {
    static const char* lowest() { return "0"; }
    static const char* highest() { return "ULONG_MAX"; }
};
template <> struct limits<float> {
    static const char* lowest() { return "(-INFINITY)"; }
    static const char* highest() { return "INFINITY"; }
};
template <> struct limits<double> {
    static const char* lowest() { return "(-INFINITY)"; }
    static const char* highest() { return "INFINITY"; }
};

inline binary_op plus() { return {"(a + b)", "0"}; }
inline binary_op multiplies() { return {"(a * b)", "1"}; }
inline binary_op bit_and() { return {"(a & b)", "(~0)"}; }
inline binary_op bit_or() { return {"(a | b)", "0"}; }
inline binary_op bit_xor() { return {"(a ^ b)", "0"}; }
template <typename T> binary_op minimum() { return {"((b < a) ? b : a)", limits<T>::highest()}; }
template <typename T> binary_op maximum() { return {"((a < b) ? b : a)", limits<T>::lowest()}; }
}  // namespace ops

// ---- context (Context.hpp:25-59) ---------------------------------------------

class compute_context;

//! The context's in-order queue: a CUDA stream. copy_from_host and
//! copy_to_host take it where the reference takes a cl::CommandQueue.
class command_queue {
public:
    //! Waits for everything enqueued; reports a kernel-recorded failure (a
    //! look-back wait that timed out) as device_error.
    void finish() { detail::check(clc_finish(ctx_)); }
    clc_context context_handle() const { return ctx_; }
    //! The cudaStream_t.
    void* stream() const { return clc_context_stream(ctx_); }

private:
    friend class compute_context;
    explicit command_queue(clc_context c) : ctx_(c) {}
    clc_context ctx_;
};

//! One GPU, one CUDA stream, a stream-ordered arena for temporaries and the
//! tuning table of launch shapes. Not thread-safe: one per host thread.
class compute_context {
public:
    //! device: index among the CUDA devices (CLC_DEFAULT_DEVICE: the first);
    //! tuning_dir: where the tuning table is kept (NULL: CLC_TUNING_DIR,
    //! then CL_COMPUTE_CACHE_DIR).
    explicit compute_context(std::size_t device = CLC_DEFAULT_DEVICE, const char* tuning_dir = nullptr)
        : queue_(nullptr)
    {
        clc_context c = nullptr;
        detail::check(clc_context_create_with_cache(device, tuning_dir, &c));
        queue_ = command_queue(c);
    }
    ~compute_context()
    {
        if (queue_.ctx_ != nullptr) clc_context_release(queue_.ctx_);
    }
    compute_context(const compute_context&) = delete;
    compute_context& operator=(const compute_context&) = delete;
    compute_context(compute_context&& o) noexcept : queue_(o.queue_.ctx_) { o.queue_.ctx_ = nullptr; }
    compute_context& operator=(compute_context&& o) noexcept
    {
        if (this != &o) {
            if (queue_.ctx_ != nullptr) clc_context_release(queue_.ctx_);
            queue_.ctx_ = o.queue_.ctx_;
            o.queue_.ctx_ = nullptr;
        }
        return *this;
    }

    command_queue& queue() { return queue_; }
    clc_context handle() const { return queue_.ctx_; }
    clc_device_info device() const
    {
        clc_device_info info;
        detail::check(clc_context_get_info(queue_.ctx_, &info));
        return info;
    }
    clc_memory_stats memory_stats() const
    {
        clc_memory_stats s;
        detail::check(clc_context_memory_stats(queue_.ctx_, &s));
        return s;
    }

private:
    command_queue queue_;
};

// ---- device_buffer (DeviceBuffer.hpp:26-132) ----------------------------------

//! Typed, move-only device allocation from the context's arena. A buffer
//! keeps the arena (and the stream) alive, so it may outlive its context.
template <typename T> class device_buffer {
public:
    device_buffer() = default;
    device_buffer(const compute_context& ctx, std::size_t size) : size_(size)
    {
        detail::check(clc_buffer_alloc(ctx.handle(), bytes(), &buf_));
    }
    device_buffer(const device_buffer&) = delete;
    device_buffer& operator=(const device_buffer&) = delete;
    device_buffer(device_buffer&& o) noexcept : buf_(o.buf_), size_(o.size_)
    {
        o.buf_ = nullptr;
        o.size_ = 0;
    }
    device_buffer& operator=(device_buffer&& o) noexcept
    {
        if (this != &o) {
            reset();
            buf_ = o.buf_;
            size_ = o.size_;
            o.buf_ = nullptr;
            o.size_ = 0;
        }
        return *this;
    }
    ~device_buffer() { reset(); }

    //! Returns the allocation to the arena.
    void reset() noexcept
    {
        clc_buffer_release(buf_);
        buf_ = nullptr;
        size_ = 0;
    }

    std::size_t size() const { return size_; }
    std::size_t bytes() const { return size_ * sizeof(T); }
    bool empty() const { return size_ == 0; }
    clc_buffer get() const { return buf_; }
    T* data() const { return static_cast<T*>(clc_buffer_device_pointer(buf_)); }

    void copy_from_host(command_queue& queue, const T* src, std::size_t count, std::size_t offset = 0,
                        bool /*blocking*/ = true)
    {
        check_range(offset, count);
        if (count != 0)
            detail::check(clc_buffer_write(queue.context_handle(), buf_, offset * sizeof(T), count * sizeof(T), src));
    }
    void copy_to_host(command_queue& queue, T* dst, std::size_t count, std::size_t offset = 0,
                      bool /*blocking*/ = true) const
    {
        check_range(offset, count);
        if (count != 0)
            detail::check(clc_buffer_read(queue.context_handle(), buf_, offset * sizeof(T), count * sizeof(T), dst));
    }
    std::vector<T> to_host(compute_context& ctx) const
    {
        std::vector<T> out(size_);
        copy_to_host(ctx.queue(), out.data(), size_);
        return out;
    }
    //! Takes ownership of a buffer handle from the C interface.
    static device_buffer adopt(clc_buffer handle, std::size_t size)
    {
        device_buffer b;
        b.buf_ = handle;
        b.size_ = size;
        return b;
    }
    static device_buffer from_host(compute_context& ctx, const std::vector<T>& values)
    {
        device_buffer b(ctx, values.size());
        b.copy_from_host(ctx.queue(), values.data(), values.size());
        return b;
    }

private:
    void check_range(std::size_t offset, std::size_t count) const
    {
        if (offset > size_ || count > size_ - offset) throw std::out_of_range("device_buffer: range out of bounds");
    }
    clc_buffer buf_ = nullptr;
    std::size_t size_ = 0;
};

// ---- algorithms (Algorithm.hpp:119-250) ----------------------------------------

//! out[i] = value (thrust::fill).
template <typename T> void fill(compute_context& ctx, device_buffer<T>& out, T value)
{
    detail::check_size(out.size());
    detail::check(clc_fill(ctx.handle(), out.get(), out.size(), detail::type_of<T>::value, &value));
}

//! out[i] = start + i * step (thrust::sequence).
template <typename T> void sequence(compute_context& ctx, device_buffer<T>& out, T start = T(0), T step = T(1))
{
    detail::check_size(out.size());
    detail::check(clc_sequence(ctx.handle(), out.get(), out.size(), detail::type_of<T>::value, &start, &step));
}

//! out[i] = expression(in[i]); the expression uses x (thrust::transform).
template <typename In, typename Out>
void transform(compute_context& ctx, const device_buffer<In>& in, device_buffer<Out>& out,
               const std::string& expression)
{
    if (out.size() < in.size()) throw std::invalid_argument("transform: output too small");
    detail::check_size(in.size());
    detail::check(clc_transform(ctx.handle(), in.get(), detail::type_of<In>::value, out.get(),
                                detail::type_of<Out>::value, in.size(), expression.c_str()));
}

//! out[i] = expression(in1[i], in2[i]); the expression uses x and y; out may
//! alias an input (binary thrust::transform).
template <typename In1, typename In2, typename Out>
void transform(compute_context& ctx, const device_buffer<In1>& in1, const device_buffer<In2>& in2,
               device_buffer<Out>& out, const std::string& expression)
{
    if (in2.size() < in1.size() || out.size() < in1.size()) throw std::invalid_argument("transform: size mismatch");
    detail::check_size(in1.size());
    detail::check(clc_transform2(ctx.handle(), in1.get(), detail::type_of<In1>::value, in2.get(),
                                 detail::type_of<In2>::value, out.get(), detail::type_of<Out>::value, in1.size(),
                                 expression.c_str()));
}

//! op(init, fold of in with op); the order of combination is unspecified, so
//! op must be associative and commutative (thrust::reduce). Blocks.
template <typename T>
T reduce(compute_context& ctx, const device_buffer<T>& in, const binary_op& op = ops::plus(), T init = T(0))
{
    detail::check_size(in.size());
    T result = init;
    detail::check(clc_reduce(ctx.handle(), in.get(), in.size(), detail::type_of<T>::value, op.expression.c_str(),
                             op.identity.c_str(), &init, &result));
    return result;
}

//! out[i] = in[0] op ... op in[i]; out may alias in (thrust::inclusive_scan).
template <typename T>
void inclusive_scan(compute_context& ctx, const device_buffer<T>& in, device_buffer<T>& out,
                    const binary_op& op = ops::plus())
{
    if (out.size() < in.size()) throw std::invalid_argument("inclusive_scan: output too small");
    detail::check_size(in.size());
    detail::check(clc_scan(ctx.handle(), in.get(), out.get(), in.size(), detail::type_of<T>::value,
                           op.expression.c_str(), op.identity.c_str(), 0));
}

//! out[i] = identity op in[0] op ... op in[i-1]; out may alias in
//! (thrust::exclusive_scan).
template <typename T>
void exclusive_scan(compute_context& ctx, const device_buffer<T>& in, device_buffer<T>& out,
                    const binary_op& op = ops::plus())
{
    if (out.size() < in.size()) throw std::invalid_argument("exclusive_scan: output too small");
    detail::check_size(in.size());
    detail::check(clc_scan(ctx.handle(), in.get(), out.get(), in.size(), detail::type_of<T>::value,
                           op.expression.c_str(), op.identity.c_str(), 1));
}

//! Stable radix sort of 32-bit keys in place (cl_uint, cl_int or cl_float;
//! floats in the order of their sign/bit flip, so -0 sorts before +0).
template <typename Key> void sort(compute_context& ctx, device_buffer<Key>& keys, bool descending = false)
{
    static_assert(sizeof(Key) == 4, "sort: keys must be 32-bit");
    detail::check_size(keys.size());
    detail::check(clc_sort(ctx.handle(), keys.get(), detail::type_of<Key>::value, nullptr, keys.size(),
                           descending ? 1 : 0));
}

//! Sorts keys and permutes 32-bit values alongside (thrust::sort_by_key).
template <typename Key, typename Value>
void sort_by_key(compute_context& ctx, device_buffer<Key>& keys, device_buffer<Value>& values, bool descending = false)
{
    static_assert(sizeof(Key) == 4, "sort_by_key: keys must be 32-bit");
    static_assert(sizeof(Value) == 4, "sort_by_key: values must be 32-bit");
    if (values.size() < keys.size()) throw std::invalid_argument("sort_by_key: too few values");
    detail::check_size(keys.size());
    detail::check(clc_sort(ctx.handle(), keys.get(), detail::type_of<Key>::value, values.get(), keys.size(),
                           descending ? 1 : 0));
}

//! Copies the elements of in for which predicate (an expression of x) holds
//! to the front of out, in order; returns how many (thrust::copy_if). Blocks.
template <typename T>
std::size_t copy_if(compute_context& ctx, const device_buffer<T>& in, device_buffer<T>& out,
                    const std::string& predicate)
{
    if (out.size() < in.size()) throw std::invalid_argument("copy_if: output too small");
    detail::check_size(in.size());
    std::size_t count = 0;
    detail::check(clc_copy_if(ctx.handle(), in.get(), out.get(), in.size(), detail::type_of<T>::value,
                              predicate.c_str(), &count));
    return count;
}

//! Counts in into histogram.size() equal-width bins over [lower, upper);
//! samples outside are ignored (cub::DeviceHistogram::HistogramEven).
template <typename T>
void histogram_even(compute_context& ctx, const device_buffer<T>& in, device_buffer<cl_uint>& histogram, double lower,
                    double upper)
{
    detail::check_size(in.size());
    detail::check(clc_histogram_even(ctx.handle(), in.get(), in.size(), detail::type_of<T>::value, histogram.get(),
                                     histogram.size(), lower, upper));
}

// ---- bitpack compression (Compression.hpp) ----------------------------------

//! Options of compress_bitpack: delta coding of consecutive elements, and the
//! chunk size (a power of two in [256, 65536]).
struct bitpack_options {
    bool delta = false;
    std::size_t chunk_size = 2048;
};

//! The reference's compressed_buffer: the device words of its chunk format
//! (per chunk {base, width, offset}, then the packed words).
struct compressed_buffer {
    device_buffer<cl_uint> data;
    std::size_t num_elements = 0;
    std::size_t chunk_size = 0;
    bool delta = false;

    std::size_t num_chunks() const { return chunk_size == 0 ? 0 : (num_elements + chunk_size - 1) / chunk_size; }
    std::size_t compressed_bytes() const { return data.bytes(); }
    std::size_t uncompressed_bytes() const { return num_elements * sizeof(cl_uint); }

    //! Host blob: an 8-word header, then the device words.
    std::vector<unsigned char> serialize(compute_context& ctx) const
    {
        std::size_t needed = 0;
        detail::check(clc_bitpack_serialize(ctx.handle(), data.get(), num_elements, chunk_size, delta ? 1 : 0,
                                            nullptr, 0, &needed));
        std::vector<unsigned char> blob(needed);
        detail::check(clc_bitpack_serialize(ctx.handle(), data.get(), num_elements, chunk_size, delta ? 1 : 0,
                                            blob.data(), blob.size(), &needed));
        return blob;
    }
    //! Validates the blob (std::invalid_argument when it is not one) and
    //! uploads its words.
    static compressed_buffer deserialize(compute_context& ctx, const std::vector<unsigned char>& blob)
    {
        clc_buffer h = nullptr;
        std::size_t n = 0, chunk = 0;
        int d = 0;
        detail::check(clc_bitpack_deserialize(ctx.handle(), blob.data(), blob.size(), &h, &n, &chunk, &d));
        compressed_buffer r;
        r.data = device_buffer<cl_uint>::adopt(h, clc_buffer_size(h) / sizeof(cl_uint));
        r.num_elements = n;
        r.chunk_size = chunk;
        r.delta = d != 0;
        return r;
    }
};

inline compressed_buffer compress_bitpack(compute_context& ctx, const device_buffer<cl_uint>& in,
                                          bitpack_options options = bitpack_options())
{
    clc_buffer h = nullptr;
    std::size_t words = 0;
    detail::check(clc_bitpack_compress(ctx.handle(), in.get(), in.size(), options.chunk_size, options.delta ? 1 : 0,
                                       &h, &words));
    compressed_buffer r;
    r.data = device_buffer<cl_uint>::adopt(h, words);
    r.num_elements = in.size();
    r.chunk_size = options.chunk_size;
    r.delta = options.delta;
    return r;
}

//! Decompresses into out, which must hold in.num_elements values.
inline void decompress_bitpack(compute_context& ctx, const compressed_buffer& in, device_buffer<cl_uint>& out)
{
    if (out.size() < in.num_elements) throw std::invalid_argument("decompress_bitpack: output too small");
    detail::check(clc_bitpack_decompress(ctx.handle(), in.data.get(), in.num_elements, in.chunk_size,
                                         in.delta ? 1 : 0, out.get()));
}

// ---- static_map (HashMap.hpp) --------------------------------------------------

//! Fixed-capacity hash map from cl_uint keys to cl_uint values: linear
//! probing over a power-of-two table, MurmurHash3 finalizer; empty_key marks
//! free slots, find returns empty_value for absent keys, insert keeps a
//! key's first value and throws std::overflow_error when the table is full.
class static_map {
public:
    static_map(compute_context& ctx, std::size_t capacity, cl_uint empty_key = 0xFFFFFFFFu,
               cl_uint empty_value = 0xFFFFFFFFu)
        : ctx_(ctx)
    {
        detail::check(clc_map_create(ctx.handle(), capacity, empty_key, empty_value, &map_));
    }
    ~static_map() { clc_map_release(map_); }
    static_map(const static_map&) = delete;
    static_map& operator=(const static_map&) = delete;

    //! Inserts n pairs; returns how many keys were new.
    std::size_t insert(const device_buffer<cl_uint>& keys, const device_buffer<cl_uint>& values, std::size_t n)
    {
        if (n > keys.size() || n > values.size()) throw std::invalid_argument("static_map::insert: n out of range");
        std::size_t added = 0;
        const clc_status s = clc_map_insert(ctx_.handle(), map_, keys.get(), values.get(), n, &added);
        if (s == CLC_ERROR_OUT_OF_MEMORY) throw std::overflow_error(clc_last_error());
        detail::check(s);
        return added;
    }
    std::size_t insert(const device_buffer<cl_uint>& keys, const device_buffer<cl_uint>& values)
    {
        return insert(keys, values, keys.size());
    }
    //! values[i] = map[keys[i]], or empty_value when absent.
    void find(const device_buffer<cl_uint>& keys, device_buffer<cl_uint>& values) const
    {
        if (values.size() < keys.size()) throw std::invalid_argument("static_map::find: output too small");
        detail::check(clc_map_find(ctx_.handle(), map_, keys.get(), keys.size(), values.get()));
    }
    //! found[i] = 1 when keys[i] is present, else 0.
    void contains(const device_buffer<cl_uint>& keys, device_buffer<cl_uchar>& found) const
    {
        if (found.size() < keys.size()) throw std::invalid_argument("static_map::contains: output too small");
        detail::check(clc_map_contains(ctx_.handle(), map_, keys.get(), keys.size(), found.get()));
    }
    void clear() { detail::check(clc_map_clear(ctx_.handle(), map_)); }

    std::size_t size() const { return info().size; }
    std::size_t capacity() const { return info().capacity; }
    double load_factor() const { return double(size()) / double(capacity()); }
    cl_uint empty_key() const { return info().empty_key; }
    cl_uint empty_value() const { return info().empty_value; }
    //! The table's slot keys and values (copies of the device table).
    device_buffer<cl_uint> slot_keys() const { return slots(true); }
    device_buffer<cl_uint> slot_values() const { return slots(false); }

private:
    struct info_t {
        std::size_t size, capacity;
        cl_uint empty_key, empty_value;
    };
    info_t info() const
    {
        info_t i{};
        detail::check(clc_map_info(map_, &i.size, &i.capacity, &i.empty_key, &i.empty_value));
        return i;
    }
    device_buffer<cl_uint> slots(bool keys) const
    {
        device_buffer<cl_uint> b(ctx_, capacity());
        detail::check(clc_map_slots(ctx_.handle(), map_, keys ? b.get() : nullptr, keys ? nullptr : b.get()));
        return b;
    }
    compute_context& ctx_;
    clc_map map_ = nullptr;
};

// ---- extensions (no counterpart in the reference's C++ API) -----------------

//! exclusive_scan plus the exact 64-bit sum of all inputs (8/16/32-bit
//! integer plus-scans; otherwise the last inclusive value widened). Blocks.
template <typename T, typename Wide = typename std::conditional<std::is_signed<T>::value, int64_t, uint64_t>::type>
Wide exclusive_scan_total(compute_context& ctx, const device_buffer<T>& in, device_buffer<T>& out,
                          const binary_op& op = ops::plus())
{
    if (out.size() < in.size()) throw std::invalid_argument("exclusive_scan_total: output too small");
    detail::check_size(in.size());
    Wide total = 0;
    detail::check(clc_scan_ex(ctx.handle(), in.get(), out.get(), in.size(), detail::type_of<T>::value,
                              op.expression.c_str(), op.identity.c_str(), 1, &total));
    return total;
}

//! Stable sort of 32- or 64-bit keys with optional 32-bit values (the
//! reference sorts 32-bit keys only).
template <typename Key> void sort_wide(compute_context& ctx, device_buffer<Key>& keys, bool descending = false)
{
    static_assert(sizeof(Key) == 4 || sizeof(Key) == 8, "sort_wide: keys must be 32- or 64-bit");
    detail::check_size(keys.size());
    detail::check(clc_sort_ex(ctx.handle(), keys.get(), detail::type_of<Key>::value, nullptr, keys.size(),
                              descending ? 1 : 0));
}
template <typename Key, typename Value>
void sort_by_key_wide(compute_context& ctx, device_buffer<Key>& keys, device_buffer<Value>& values,
                      bool descending = false)
{
    static_assert(sizeof(Key) == 4 || sizeof(Key) == 8, "sort_by_key_wide: keys must be 32- or 64-bit");
    static_assert(sizeof(Value) == 4, "sort_by_key_wide: values must be 32-bit");
    if (values.size() < keys.size()) throw std::invalid_argument("sort_by_key_wide: too few values");
    detail::check_size(keys.size());
    detail::check(clc_sort_ex(ctx.handle(), keys.get(), detail::type_of<Key>::value, values.get(), keys.size(),
                              descending ? 1 : 0));
}

}  // namespace compute
}  // namespace cl

#endif  // GBCOMPUTE_COMPUTE_HPP
