// The C ABI: clc_* entry points over the gbcompute runtime.
//
// Reference: lib/src/Compute/CApi.cpp:1-643 (over lib/include/CL/Compute/
// compute_c.h). Kept: opaque handles; buffers share the memory resource (and
// here the stream) with their context and may outlive it (CApi.cpp:21-26,
// 301-320); zero-byte buffers are valid and releasing NULL is a no-op;
// thread-local last error and native error code (49-57); no exception
// crosses the boundary, each is mapped to a status by type (60-115);
// require_fits bounds checks (213-218); clc_sort accepts only 32-bit keys
// (517-531); device enumeration and context creation are serialised (117-124).
// Changed: OpenCL C expressions become a table of canonical operators
// (parse_op) and identity literals (parse_identity); the user-kernel and
// file-I/O entry points exist so C callers link, and report
// CLC_ERROR_UNSUPPORTED.
#include "../../include/compute_c.h"

#include <cctype>
#include <cerrno>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <limits>
#include <memory>
#include <mutex>
#include <new>
#include <string>

#include "autotune.hpp"
#include "expr.hpp"
#include "select.hpp"
#include "learned.hpp"
#include "runtime.hpp"
#include "segmented.hpp"
#include "sort_internal.hpp"

struct clc_context_s {
    std::unique_ptr<gbc::device_context> ctx;
};

struct clc_buffer_s {
    std::shared_ptr<gbc::memory_resource> resource;  // null for wrapped memory
    std::shared_ptr<gbc::stream_holder> holder;
    void* ptr;
    std::size_t bytes;
};

struct clc_kernel_s {
    int unused;
};

struct clc_map_s {
    std::shared_ptr<gbc::memory_resource> resource;
    std::shared_ptr<gbc::stream_holder> holder;
    void* slots;
    std::size_t capacity;
    uint32_t empty_key, empty_value;
    std::size_t size;
};

struct clc_graph_s {
    cudaGraph_t graph;
    cudaGraphExec_t exec;
    int device;
};

namespace {

using gbc::build_error;

thread_local std::string last_error;
thread_local int last_native_error = 0;

clc_status fail(clc_status s, const std::string& msg, int native = 0)
{
    last_error = msg;
    last_native_error = native;
    return s;
}

}  // namespace

namespace gbc {
// Sets the thread's last error for entry points defined outside this file.
int set_last_error(int status, const char* msg, int native)
{
    if (status == CLC_SUCCESS) {
        last_error.clear();
        last_native_error = 0;
        return status;
    }
    return fail(static_cast<clc_status>(status), msg, native);
}
}  // namespace gbc

namespace {

template <typename F> clc_status guarded(F&& body)
{
    try {
        body();
        last_error.clear();
        last_native_error = 0;
        return CLC_SUCCESS;
    } catch (const gbc::no_device_error& e) {
        return fail(CLC_ERROR_NO_DEVICE, e.what());
    } catch (const gbc::unsupported_error& e) {
        return fail(CLC_ERROR_UNSUPPORTED, e.what());
    } catch (const build_error& e) {
        return fail(CLC_ERROR_BUILD, e.what());
    } catch (const gbc::out_of_memory& e) {
        return fail(CLC_ERROR_OUT_OF_MEMORY, e.what());
    } catch (const gbc::device_error& e) {
        return fail(CLC_ERROR_OPENCL, e.what(), e.code);
    } catch (const std::bad_alloc&) {
        return fail(CLC_ERROR_OUT_OF_MEMORY, "host allocation failed");
    } catch (const std::invalid_argument& e) {
        return fail(CLC_ERROR_INVALID_ARGUMENT, e.what());
    } catch (const std::out_of_range& e) {
        return fail(CLC_ERROR_INVALID_ARGUMENT, e.what());
    } catch (const std::length_error& e) {
        return fail(CLC_ERROR_INVALID_ARGUMENT, e.what());
    } catch (const std::overflow_error& e) {
        return fail(CLC_ERROR_OUT_OF_MEMORY, e.what());
    } catch (const std::exception& e) {
        return fail(CLC_ERROR_INTERNAL, e.what());
    } catch (...) {
        return fail(CLC_ERROR_INTERNAL, "unknown error");
    }
}

std::mutex& init_mutex()
{
    static std::mutex m;
    return m;
}

// CUDA devices; 0 when there is no driver or no device (not an error).
int device_count()
{
    std::lock_guard<std::mutex> lock(init_mutex());
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess) {
        (void)cudaGetLastError();
        return 0;
    }
    return n;
}

void copy_text(char (&dst)[256], const std::string& src)
{
    const std::size_t n = std::min<std::size_t>(src.size(), 255);
    std::memcpy(dst, src.data(), n);
    dst[n] = '\0';
}

void fill_info(int device, clc_device_info* info)
{
    cudaDeviceProp p;
    gbc::check_cuda(cudaGetDeviceProperties(&p, device), "cudaGetDeviceProperties");
    copy_text(info->name, p.name);
    copy_text(info->platform, "NVIDIA CUDA");
    info->is_gpu = 1;
    info->has_fp64 = 1;
    info->global_memory = (unsigned long long)p.totalGlobalMem;
    info->max_work_group_size = (size_t)p.maxThreadsPerBlock;
}

gbc::elem elem_of(clc_type t)
{
    switch (t) {
    case CLC_TYPE_I8: return gbc::elem::i8;
    case CLC_TYPE_U8: return gbc::elem::u8;
    case CLC_TYPE_I16: return gbc::elem::i16;
    case CLC_TYPE_U16: return gbc::elem::u16;
    case CLC_TYPE_I32: return gbc::elem::i32;
    case CLC_TYPE_U32: return gbc::elem::u32;
    case CLC_TYPE_I64: return gbc::elem::i64;
    case CLC_TYPE_U64: return gbc::elem::u64;
    case CLC_TYPE_F32: return gbc::elem::f32;
    case CLC_TYPE_F64: return gbc::elem::f64;
    }
    throw std::invalid_argument("clc: unknown element type");
}

void require(bool c, const char* msg)
{
    if (!c) throw std::invalid_argument(msg);
}

void require_fits(clc_buffer b, std::size_t n, clc_type t)
{
    require(b != nullptr, "clc: null buffer");
    require(n <= b->bytes / gbc::elem_size(elem_of(t)), "clc: buffer too small for the element count");
}

// ---- operator and identity tables ----------------------------------------

std::string normalise(const char* s)
{
    std::string r;
    for (const char* p = s; *p; ++p)
        if (!std::isspace((unsigned char)*p)) r += *p;
    // Strip parentheses that enclose the whole expression.
    for (;;) {
        if (r.size() < 2 || r.front() != '(' || r.back() != ')') break;
        int depth = 0;
        bool encloses = true;
        for (std::size_t i = 0; i < r.size(); ++i) {
            if (r[i] == '(') ++depth;
            if (r[i] == ')') --depth;
            if (depth == 0 && i + 1 < r.size()) {
                encloses = false;
                break;
            }
        }
        if (!encloses) break;
        r = r.substr(1, r.size() - 2);
    }
    return r;
}

gbc::op_kind parse_op(const char* expr)
{
    const std::string e = normalise(expr);
    if (e == "a+b") return gbc::op_kind::plus;
    if (e == "a*b") return gbc::op_kind::multiplies;
    if (e == "a&b") return gbc::op_kind::bit_and;
    if (e == "a|b") return gbc::op_kind::bit_or;
    if (e == "a^b") return gbc::op_kind::bit_xor;
    if (e == "(b<a)?b:a" || e == "min(a,b)" || e == "fmin(a,b)") return gbc::op_kind::minimum;
    if (e == "(a<b)?b:a" || e == "max(a,b)" || e == "fmax(a,b)") return gbc::op_kind::maximum;
    if (e == "b") return gbc::op_kind::right;
    if (e == "a") return gbc::op_kind::left;
    throw gbc::unsupported_error(std::string("clc: operator \"") + expr +
                                 "\" is not one of the compiled operators (a + b, a * b, a & b, "
                                 "a | b, a ^ b, min, max, b)");
}

// Writes the identity literal as one element of type t into out (8 bytes).
void parse_identity(const char* lit, clc_type t, void* out)
{
    const std::string s = normalise(lit);
    const gbc::elem e = elem_of(t);
    const bool is_float = e == gbc::elem::f32 || e == gbc::elem::f64;
    long double v = 0;
    bool is_bits = false;
    uint64_t bits = 0;
    struct named {
        const char* name;
        long double value;
    };
    static const named table[] = {
        {"CHAR_MIN", -128.0L},
        {"CHAR_MAX", 127.0L},
        {"UCHAR_MAX", 255.0L},
        {"SHRT_MIN", -32768.0L},
        {"SHRT_MAX", 32767.0L},
        {"USHRT_MAX", 65535.0L},
        {"INT_MIN", -2147483648.0L},
        {"INT_MAX", 2147483647.0L},
        {"UINT_MAX", 4294967295.0L},
        {"LONG_MIN", -9223372036854775808.0L},
        {"LONG_MAX", 9223372036854775807.0L},
        {"ULONG_MAX", 18446744073709551615.0L},
        {"INFINITY", std::numeric_limits<long double>::infinity()},
        {"-INFINITY", -std::numeric_limits<long double>::infinity()},
    };
    bool found = false;
    for (const auto& n : table)
        if (s == n.name) {
            v = n.value;
            found = true;
        }
    if (!found && (s == "~0" || s == "~0u" || s == "~0U")) {
        is_bits = true;
        bits = ~uint64_t(0);
        found = true;
    }
    if (!found) {
        std::string num = s;
        while (!num.empty() && std::strchr("uUlLfF", num.back()) != nullptr &&
               !(num.size() > 2 && (num[1] == 'x' || num[1] == 'X') && std::isxdigit((unsigned char)num.back())))
            num.pop_back();
        if (num.empty()) throw gbc::unsupported_error(std::string("clc: identity \"") + lit + "\" is not a literal");
        char* end = nullptr;
        errno = 0;
        const bool hex = num.size() > 2 && num[0] == '0' && (num[1] == 'x' || num[1] == 'X');
        if (!is_float && (hex || num.find_first_of(".eE") == std::string::npos)) {
            if (num[0] == '-') v = (long double)std::strtoll(num.c_str(), &end, 0);
            else {
                is_bits = true;
                bits = std::strtoull(num.c_str(), &end, 0);
            }
        } else {
            v = std::strtold(num.c_str(), &end);
        }
        if (end == nullptr || *end != '\0')
            throw gbc::unsupported_error(std::string("clc: identity \"") + lit + "\" is not a literal");
    }
    uint64_t raw = 0;
    switch (e) {
    case gbc::elem::f32: {
        const float f = is_bits ? (float)bits : (float)v;
        std::memcpy(&raw, &f, 4);
        break;
    }
    case gbc::elem::f64: {
        const double d = is_bits ? (double)bits : (double)v;
        std::memcpy(&raw, &d, 8);
        break;
    }
    default: {
        // Integers: two's complement truncation to the element width, like
        // an OpenCL C conversion of the literal.
        if (is_bits) raw = bits;
        else if (v < 0) raw = (uint64_t)(int64_t)v;
        else raw = (uint64_t)v;
        break;
    }
    }
    std::memcpy(out, &raw, gbc::elem_size(e));
}

void key_kind_of(clc_type t, int& bytes, int& kind)
{
    switch (t) {
    case CLC_TYPE_U32: bytes = 4, kind = 0; return;
    case CLC_TYPE_I32: bytes = 4, kind = 1; return;
    case CLC_TYPE_F32: bytes = 4, kind = 2; return;
    case CLC_TYPE_U64: bytes = 8, kind = 0; return;
    case CLC_TYPE_I64: bytes = 8, kind = 1; return;
    case CLC_TYPE_F64: bytes = 8, kind = 2; return;
    default: break;
    }
    throw std::invalid_argument("clc_sort: keys must be I32, U32, F32, I64, U64 or F64");
}

void require_same_device(clc_context ctx, clc_buffer b)
{
    if (b != nullptr && b->holder && b->holder->device != ctx->ctx->device)
        throw std::invalid_argument("clc: buffer belongs to another device");
}

}  // namespace

extern "C" {

const char* clc_last_error(void) { return last_error.c_str(); }
int clc_last_cl_error(void) { return last_native_error; }

clc_status clc_device_count(size_t* count)
{
    if (count == nullptr) return fail(CLC_ERROR_INVALID_ARGUMENT, "clc: null count");
    return guarded([&] { *count = (size_t)device_count(); });
}

clc_status clc_device_get_info(size_t index, clc_device_info* info)
{
    if (info == nullptr) return fail(CLC_ERROR_INVALID_ARGUMENT, "clc: null info");
    return guarded([&] {
        require(index < (size_t)device_count(), "clc: device index out of range");
        fill_info((int)index, info);
    });
}

clc_status clc_context_create(size_t index, clc_context* out)
{
    return clc_context_create_with_cache(index, nullptr, out);
}

clc_status clc_context_create_with_cache(size_t index, const char* cache_dir, clc_context* out)
{
    if (out == nullptr) return fail(CLC_ERROR_INVALID_ARGUMENT, "clc: null output");
    *out = nullptr;
    return guarded([&] {
        const int n = device_count();
        if (n == 0) throw gbc::no_device_error("clc: no CUDA device available");
        if (index == CLC_DEFAULT_DEVICE) index = 0;
        if (index >= (size_t)n) throw gbc::no_device_error("clc: device index out of range");
        std::lock_guard<std::mutex> lock(init_mutex());
        cudaDeviceProp p;
        gbc::check_cuda(cudaGetDeviceProperties(&p, (int)index), "cudaGetDeviceProperties");
        auto ctx = std::make_unique<gbc::device_context>(
            (int)index, nullptr, gbc::default_arena_config(p.totalGlobalMem),
            cache_dir != nullptr ? cache_dir : "");
        *out = new clc_context_s{std::move(ctx)};
    });
}

void clc_context_release(clc_context ctx) { delete ctx; }

clc_status clc_context_get_info(clc_context ctx, clc_device_info* info)
{
    if (ctx == nullptr || info == nullptr) return fail(CLC_ERROR_INVALID_ARGUMENT, "clc: null argument");
    return guarded([&] { fill_info(ctx->ctx->device, info); });
}

clc_status clc_finish(clc_context ctx)
{
    if (ctx == nullptr) return fail(CLC_ERROR_INVALID_ARGUMENT, "clc: null context");
    return guarded([&] { ctx->ctx->finish(); });
}

clc_status clc_buffer_alloc(clc_context ctx, size_t bytes, clc_buffer* out)
{
    if (ctx == nullptr || out == nullptr) return fail(CLC_ERROR_INVALID_ARGUMENT, "clc: null argument");
    *out = nullptr;
    return guarded([&] {
        ctx->ctx->activate();
        std::unique_ptr<clc_buffer_s> b(new clc_buffer_s{ctx->ctx->resource, ctx->ctx->holder, nullptr, bytes});
        if (bytes != 0) b->ptr = b->resource->allocate(bytes);
        *out = b.release();
    });
}

void clc_buffer_release(clc_buffer buffer)
{
    if (buffer == nullptr) return;
    if (buffer->bytes != 0 && buffer->resource) buffer->resource->deallocate(buffer->ptr, buffer->bytes);
    delete buffer;
}

size_t clc_buffer_size(clc_buffer buffer) { return buffer == nullptr ? 0 : buffer->bytes; }

clc_status clc_buffer_write(clc_context ctx, clc_buffer buffer, size_t offset, size_t bytes, const void* src)
{
    return guarded([&] {
        require(ctx != nullptr && buffer != nullptr, "clc: null argument");
        require(offset <= buffer->bytes && bytes <= buffer->bytes - offset, "clc: write out of bounds");
        require(bytes == 0 || src != nullptr, "clc: null source");
        require_same_device(ctx, buffer);
        if (bytes == 0) return;
        auto& c = *ctx->ctx;
        c.activate();
        gbc::check_cuda(cudaMemcpyAsync(static_cast<char*>(buffer->ptr) + offset, src, bytes,
                                        cudaMemcpyHostToDevice, c.stream),
                        "cudaMemcpyAsync");
        gbc::check_cuda(cudaStreamSynchronize(c.stream), "cudaStreamSynchronize");
    });
}

clc_status clc_buffer_read(clc_context ctx, clc_buffer buffer, size_t offset, size_t bytes, void* dst)
{
    return guarded([&] {
        require(ctx != nullptr && buffer != nullptr, "clc: null argument");
        require(offset <= buffer->bytes && bytes <= buffer->bytes - offset, "clc: read out of bounds");
        require(bytes == 0 || dst != nullptr, "clc: null destination");
        require_same_device(ctx, buffer);
        auto& c = *ctx->ctx;
        c.activate();
        if (bytes != 0)
            gbc::check_cuda(cudaMemcpyAsync(dst, static_cast<const char*>(buffer->ptr) + offset, bytes,
                                            cudaMemcpyDeviceToHost, c.stream),
                            "cudaMemcpyAsync");
        c.finish();  // waits, and reports a kernel-recorded error
    });
}

clc_status clc_buffer_copy(clc_context ctx, clc_buffer src, size_t src_offset, clc_buffer dst,
                           size_t dst_offset, size_t bytes)
{
    return guarded([&] {
        require(ctx != nullptr && src != nullptr && dst != nullptr, "clc: null argument");
        require(src_offset <= src->bytes && bytes <= src->bytes - src_offset, "clc: copy source out of bounds");
        require(dst_offset <= dst->bytes && bytes <= dst->bytes - dst_offset,
                "clc: copy destination out of bounds");
        if (bytes == 0) return;
        auto& c = *ctx->ctx;
        c.activate();
        gbc::check_cuda(cudaMemcpyAsync(static_cast<char*>(dst->ptr) + dst_offset,
                                        static_cast<const char*>(src->ptr) + src_offset, bytes,
                                        cudaMemcpyDeviceToDevice, c.stream),
                        "cudaMemcpyAsync");
    });
}

// ---- out-of-scope entry points (link, then report UNSUPPORTED) -----------

#define GBC_UNSUPPORTED(what) \
    return fail(CLC_ERROR_UNSUPPORTED, "clc: " what " is outside gbcompute's primitive core")

clc_status clc_file_size(const char*, size_t*) { GBC_UNSUPPORTED("file I/O"); }
clc_status clc_file_read(clc_context, const char*, size_t, clc_buffer, size_t, size_t, size_t* done)
{
    if (done) *done = 0;
    GBC_UNSUPPORTED("file I/O");
}
clc_status clc_file_write(clc_context, const char*, int, size_t, clc_buffer, size_t, size_t, size_t* done)
{
    if (done) *done = 0;
    GBC_UNSUPPORTED("file I/O");
}
// transform / transform2 (CApi.cpp:455-486): the expression is compiled on
// the host into a program for the ahead-of-time interpreter kernel (expr.hpp);
// a malformed expression is CLC_ERROR_BUILD with "build log" in the message,
// OpenCL C outside the supported subset CLC_ERROR_UNSUPPORTED.
clc_status clc_transform(clc_context ctx, clc_buffer in, clc_type in_type, clc_buffer out, clc_type out_type,
                         size_t n, const char* expression)
{
    return guarded([&] {
        require(ctx != nullptr && expression != nullptr, "clc: null argument");
        require_fits(in, n, in_type);
        require_fits(out, n, out_type);
        const gbc::xp::program p =
            gbc::xp::compile(expression, elem_of(in_type), false, elem_of(in_type), elem_of(out_type));
        gbc::transform(*ctx->ctx, p, in->ptr, nullptr, out->ptr, n);
    });
}
clc_status clc_transform2(clc_context ctx, clc_buffer in1, clc_type type1, clc_buffer in2, clc_type type2,
                          clc_buffer out, clc_type out_type, size_t n, const char* expression)
{
    return guarded([&] {
        require(ctx != nullptr && expression != nullptr, "clc: null argument");
        require_fits(in1, n, type1);
        require_fits(in2, n, type2);
        require_fits(out, n, out_type);
        const gbc::xp::program p =
            gbc::xp::compile(expression, elem_of(type1), true, elem_of(type2), elem_of(out_type));
        gbc::transform(*ctx->ctx, p, in1->ptr, in2->ptr, out->ptr, n);
    });
}
clc_status clc_transform_compile(const char* expression, clc_type in_type, int has_in2, clc_type in2_type,
                                 clc_type out_type, char* listing, size_t capacity)
{
    return guarded([&] {
        require(expression != nullptr, "clc: null argument");
        const gbc::xp::program p = gbc::xp::compile(expression, elem_of(in_type), has_in2 != 0,
                                                    elem_of(has_in2 ? in2_type : in_type), elem_of(out_type));
        if (listing != nullptr && capacity > 0) {
            const std::string text = gbc::xp::listing(p);
            const std::size_t k = std::min(capacity - 1, text.size());
            std::memcpy(listing, text.data(), k);
            listing[k] = '\0';
        }
    });
}
// copy_if (CApi.cpp:533-545): the predicate is compiled from the expression
// subset transform uses (expr.hpp); a malformed one is CLC_ERROR_BUILD, one
// outside the subset CLC_ERROR_UNSUPPORTED.
clc_status clc_copy_if(clc_context ctx, clc_buffer in, clc_buffer out, size_t n, clc_type type, const char* predicate,
                       size_t* count)
{
    return guarded([&] {
        require(ctx != nullptr && predicate != nullptr && count != nullptr, "clc: null argument");
        *count = 0;
        require_fits(in, n, type);
        require_fits(out, n, type);
        const gbc::xp::program p = gbc::xp::compile_predicate(predicate, elem_of(type));
        *count = gbc::copy_if(*ctx->ctx, in->ptr, out->ptr, n, elem_of(type), p);
    });
}
clc_status clc_add_header(clc_context, const char*, const char*) { GBC_UNSUPPORTED("run-time kernel source"); }
clc_status clc_kernel_create(clc_context, const char*, const char*, const char*, const char* const*,
                             const char* const*, size_t, clc_kernel* out)
{
    if (out) *out = nullptr;
    GBC_UNSUPPORTED("run-time kernel source");
}
void clc_kernel_release(clc_kernel kernel) { delete kernel; }
clc_status clc_kernel_set_buffer(clc_kernel, unsigned, clc_buffer) { GBC_UNSUPPORTED("run-time kernel source"); }
clc_status clc_kernel_set_value(clc_kernel, unsigned, size_t, const void*) { GBC_UNSUPPORTED("run-time kernel source"); }
clc_status clc_kernel_set_local(clc_kernel, unsigned, size_t) { GBC_UNSUPPORTED("run-time kernel source"); }
clc_status clc_kernel_work_group_size(clc_context, clc_kernel, size_t, size_t*)
{
    GBC_UNSUPPORTED("run-time kernel source");
}
clc_status clc_kernel_launch(clc_context, clc_kernel, size_t, size_t) { GBC_UNSUPPORTED("run-time kernel source"); }
#undef GBC_UNSUPPORTED

// ---- algorithms -----------------------------------------------------------

clc_status clc_fill(clc_context ctx, clc_buffer out, size_t n, clc_type type, const void* value)
{
    return guarded([&] {
        require(ctx != nullptr && value != nullptr, "clc: null argument");
        require_fits(out, n, type);
        gbc::fill(*ctx->ctx, out->ptr, n, elem_of(type), value);
    });
}

clc_status clc_sequence(clc_context ctx, clc_buffer out, size_t n, clc_type type, const void* start,
                        const void* step)
{
    return guarded([&] {
        require(ctx != nullptr && start != nullptr && step != nullptr, "clc: null argument");
        require_fits(out, n, type);
        gbc::sequence(*ctx->ctx, out->ptr, n, elem_of(type), start, step);
    });
}

clc_status clc_reduce(clc_context ctx, clc_buffer in, size_t n, clc_type type, const char* op,
                      const char* identity, const void* init, void* result)
{
    return guarded([&] {
        require(ctx != nullptr && op != nullptr && identity != nullptr && init != nullptr && result != nullptr,
                "clc: null argument");
        require_fits(in, n, type);
        const gbc::op_kind k = parse_op(op);
        unsigned char id[8];
        parse_identity(identity, type, id);
        gbc::reduce(*ctx->ctx, in->ptr, n, elem_of(type), k, id, init, result);
    });
}

clc_status clc_reduce_raw(clc_context ctx, const void* in, size_t n, clc_type type, const char* op,
                          const char* identity, const void* init, void* result)
{
    return guarded([&] {
        require(ctx != nullptr && op != nullptr && identity != nullptr && init != nullptr && result != nullptr,
                "clc: null argument");
        require(n == 0 || in != nullptr, "clc: null input");
        const gbc::op_kind k = parse_op(op);
        unsigned char id[8];
        parse_identity(identity, type, id);
        gbc::reduce(*ctx->ctx, in, n, elem_of(type), k, id, init, result);
    });
}

clc_status clc_scan_ex(clc_context ctx, clc_buffer in, clc_buffer out, size_t n, clc_type type,
                       const char* op, const char* identity, int exclusive, void* total)
{
    return guarded([&] {
        require(ctx != nullptr && op != nullptr && identity != nullptr, "clc: null argument");
        require_fits(in, n, type);
        require_fits(out, n, type);
        const gbc::op_kind k = parse_op(op);
        unsigned char id[8];
        parse_identity(identity, type, id);
        auto& c = *ctx->ctx;
        if (total == nullptr) {
            gbc::scan(c, in->ptr, out->ptr, n, elem_of(type), k, id, exclusive != 0, nullptr);
            return;
        }
        if (n == 0) {
            std::memset(total, 0, 8);
            return;
        }
        gbc::temp_buffer t(c.resource, 8);
        gbc::scan(c, in->ptr, out->ptr, n, elem_of(type), k, id, exclusive != 0, t.get());
        gbc::check_cuda(cudaMemcpyAsync(c.pinned, t.get(), 8, cudaMemcpyDeviceToHost, c.stream), "cudaMemcpyAsync");
        c.finish();
        std::memcpy(total, c.pinned, 8);
    });
}

clc_status clc_scan(clc_context ctx, clc_buffer in, clc_buffer out, size_t n, clc_type type, const char* op,
                    const char* identity, int exclusive)
{
    return clc_scan_ex(ctx, in, out, n, type, op, identity, exclusive, nullptr);
}

clc_status clc_scan_raw(clc_context ctx, const void* in, void* out, size_t n, clc_type type, const char* op,
                        const char* identity, int exclusive, void* total_device)
{
    return guarded([&] {
        require(ctx != nullptr && op != nullptr && identity != nullptr, "clc: null argument");
        require(n == 0 || (in != nullptr && out != nullptr), "clc: null buffer");
        const gbc::op_kind k = parse_op(op);
        unsigned char id[8];
        parse_identity(identity, type, id);
        gbc::scan(*ctx->ctx, in, out, n, elem_of(type), k, id, exclusive != 0, total_device);
    });
}

clc_status clc_sort(clc_context ctx, clc_buffer keys, clc_type key_type, clc_buffer values, size_t n,
                    int descending)
{
    return guarded([&] {
        require(ctx != nullptr, "clc: null context");
        require(key_type == CLC_TYPE_I32 || key_type == CLC_TYPE_U32 || key_type == CLC_TYPE_F32,
                "clc_sort: keys must be I32, U32 or F32");
        require_fits(keys, n, key_type);
        if (values != nullptr) require_fits(values, n, CLC_TYPE_U32);
        int bytes, kind;
        key_kind_of(key_type, bytes, kind);
        uint32_t* v = values != nullptr ? static_cast<uint32_t*>(values->ptr) : nullptr;
        gbc::radix_sort(*ctx->ctx, keys->ptr, keys->ptr, bytes, kind, v, v, n, descending != 0);
    });
}

clc_status clc_sort_ex(clc_context ctx, clc_buffer keys, clc_type key_type, clc_buffer values, size_t n,
                       int descending)
{
    return guarded([&] {
        require(ctx != nullptr, "clc: null context");
        int bytes, kind;
        key_kind_of(key_type, bytes, kind);
        require_fits(keys, n, key_type);
        if (values != nullptr) require_fits(values, n, CLC_TYPE_U32);
        uint32_t* v = values != nullptr ? static_cast<uint32_t*>(values->ptr) : nullptr;
        gbc::radix_sort(*ctx->ctx, keys->ptr, keys->ptr, bytes, kind, v, v, n, descending != 0);
    });
}

clc_status clc_sort_keys_raw(clc_context ctx, const void* keys_in, void* keys_out, clc_type key_type,
                             const uint32_t* vals_in, uint32_t* vals_out, size_t n, int descending)
{
    return guarded([&] {
        require(ctx != nullptr, "clc: null context");
        int bytes, kind;
        key_kind_of(key_type, bytes, kind);
        gbc::radix_sort(*ctx->ctx, keys_in, keys_out, bytes, kind, vals_in, vals_out, n, descending != 0);
    });
}

clc_status clc_histogram_even(clc_context ctx, clc_buffer in, size_t n, clc_type type, clc_buffer hist,
                              size_t bins, double lower, double upper)
{
    return guarded([&] {
        require(ctx != nullptr, "clc: null context");
        require_fits(in, n, type);
        require_fits(hist, bins, CLC_TYPE_U32);
        gbc::histogram_even(*ctx->ctx, in->ptr, n, elem_of(type), static_cast<uint32_t*>(hist->ptr), bins,
                            lower, upper);
    });
}

clc_status clc_histogram_even_raw(clc_context ctx, const void* in, size_t n, clc_type type, uint32_t* hist,
                                  size_t bins, double lower, double upper)
{
    return guarded([&] {
        require(ctx != nullptr, "clc: null context");
        require(n == 0 || in != nullptr, "clc: null input");
        require(bins == 0 || hist != nullptr, "clc: null histogram");
        gbc::histogram_even(*ctx->ctx, in, n, elem_of(type), hist, bins, lower, upper);
    });
}

// ---- batched / segmented --------------------------------------------------

clc_status clc_segmented_sort_raw(clc_context ctx, const void* keys_in, void* keys_out, clc_type key_type,
                                  const uint32_t* vals_in, uint32_t* vals_out, size_t n, const uint32_t* offsets,
                                  size_t num_segments, int descending)
{
    return guarded([&] {
        require(ctx != nullptr, "clc: null context");
        int bytes, kind;
        key_kind_of(key_type, bytes, kind);
        gbc::seg_options opt;
        gbc::launch_shape shape;
        if (ctx->ctx->tuning.lookup(gbc::segsort_tuning_key(bytes, vals_in != nullptr, n, num_segments), shape))
            opt.cta_cap = shape.variant;
        gbc::segmented_sort(*ctx->ctx, keys_in, keys_out, bytes, kind, vals_in, vals_out, n, offsets,
                            num_segments, descending != 0, opt);
    });
}

clc_status clc_segmented_sort(clc_context ctx, clc_buffer keys, clc_type key_type, clc_buffer values, size_t n,
                              clc_buffer offsets, size_t num_segments, int descending)
{
    return guarded([&] {
        require(ctx != nullptr, "clc: null context");
        require_fits(keys, n, key_type);
        if (values != nullptr) require_fits(values, n, CLC_TYPE_U32);
        if (num_segments > 0) require_fits(offsets, num_segments + 1, CLC_TYPE_U32);
        uint32_t* v = values != nullptr ? static_cast<uint32_t*>(values->ptr) : nullptr;
        const clc_status s =
            clc_segmented_sort_raw(ctx, keys->ptr, keys->ptr, key_type, v, v, n,
                                   num_segments > 0 ? static_cast<const uint32_t*>(offsets->ptr) : nullptr,
                                   num_segments, descending);
        if (s != CLC_SUCCESS) throw std::runtime_error(last_error);
    });
}

clc_status clc_segmented_scan_raw(clc_context ctx, const void* in, void* out, size_t n, clc_type type,
                                  const char* op, const char* identity, int exclusive, const uint32_t* offsets,
                                  size_t num_segments)
{
    return guarded([&] {
        require(ctx != nullptr && op != nullptr && identity != nullptr, "clc: null argument");
        const gbc::op_kind k = parse_op(op);
        unsigned char id[8];
        parse_identity(identity, type, id);
        gbc::segmented_scan(*ctx->ctx, in, out, n, elem_of(type), k, id, exclusive != 0, offsets, num_segments);
    });
}

clc_status clc_segmented_scan(clc_context ctx, clc_buffer in, clc_buffer out, size_t n, clc_type type,
                              const char* op, const char* identity, int exclusive, clc_buffer offsets,
                              size_t num_segments)
{
    return guarded([&] {
        require(ctx != nullptr && op != nullptr && identity != nullptr, "clc: null argument");
        require_fits(in, n, type);
        require_fits(out, n, type);
        if (num_segments > 0) require_fits(offsets, num_segments + 1, CLC_TYPE_U32);
        const gbc::op_kind k = parse_op(op);
        unsigned char id[8];
        parse_identity(identity, type, id);
        gbc::segmented_scan(*ctx->ctx, in->ptr, out->ptr, n, elem_of(type), k, id, exclusive != 0,
                            num_segments > 0 ? static_cast<const uint32_t*>(offsets->ptr) : nullptr, num_segments);
    });
}

clc_status clc_reduce_by_key_raw(clc_context ctx, const void* keys, clc_type key_type, const uint32_t* values,
                                 size_t n, void* keys_out, unsigned long long* sums_out, uint32_t* counts_out,
                                 uint32_t* hist16, size_t* num_runs)
{
    return guarded([&] {
        require(ctx != nullptr, "clc: null context");
        const std::size_t kb = gbc::elem_size(elem_of(key_type));
        require(kb == 4 || kb == 8, "clc_reduce_by_key: keys must be 4 or 8 bytes");
        auto& c = *ctx->ctx;
        uint32_t* dcount = num_runs != nullptr ? reinterpret_cast<uint32_t*>(c.d_small + 1024) : nullptr;
        gbc::reduce_by_key(c, keys, (int)kb, values, n, keys_out, sums_out, counts_out, hist16, dcount);
        if (num_runs != nullptr) {
            gbc::check_cuda(cudaMemcpyAsync(c.pinned, dcount, 4, cudaMemcpyDeviceToHost, c.stream), "cudaMemcpyAsync");
            c.finish();
            uint32_t r;
            std::memcpy(&r, c.pinned, 4);
            *num_runs = r;
        }
    });
}

// ---- learned-CDF sort -------------------------------------------------------

void clc_learned_default_options(clc_learned_options* o)
{
    if (o == nullptr) return;
    *o = clc_learned_options{0, 0, 0, -1, 0.f, 1, nullptr, nullptr, nullptr, -1};
}

int clc_learned_param_count(void) { return gbc::learned::NPARAM; }

clc_status clc_sort_learned(clc_context ctx, const void* keys_in, void* keys_out, clc_type key_type, size_t n,
                            const clc_learned_options* options, clc_learned_stats* stats)
{
    return guarded([&] {
        require(ctx != nullptr, "clc: null context");
        require(key_type == CLC_TYPE_U32 || key_type == CLC_TYPE_I32 || key_type == CLC_TYPE_F32,
                "clc_sort_learned: keys must be U32, I32 or F32");
        int bytes, kind;
        key_kind_of(key_type, bytes, kind);
        gbc::learned_options o;
        if (options != nullptr) {
            o.sample = options->sample;
            o.points = options->points;
            o.buckets = options->buckets;
            o.steps = options->steps;
            o.lr = options->lr;
            o.use_model = options->use_model != 0;
            o.params_in = options->params_in;
            o.params_out = options->params_out;
            o.splitters_in = options->splitters_in;
            o.refine = options->refine;
        }
        gbc::learned_stats s;
        gbc::learned_sort(*ctx->ctx, keys_in, keys_out, kind, n, o, &s);
        if (stats != nullptr)
            *stats = clc_learned_stats{s.buckets,       s.nonempty_buckets,         s.largest_bucket,
                                       s.oversized_buckets, s.oversized_keys,      s.constant_keys,
                                       s.estimated_oversized_keys, s.violation,    s.fallback,
                                       s.first_loss,    s.last_loss,               s.refined_splitters};
    });
}

clc_status clc_sort_learned_pairs(clc_context ctx, const void* keys_in, void* keys_out, clc_type key_type,
                                  const unsigned* vals_in, unsigned* vals_out, size_t n,
                                  const clc_learned_options* options, clc_learned_stats* stats)
{
    return guarded([&] {
        require(ctx != nullptr, "clc: null context");
        require(key_type == CLC_TYPE_U32 || key_type == CLC_TYPE_I32 || key_type == CLC_TYPE_F32 ||
                    key_type == CLC_TYPE_U64 || key_type == CLC_TYPE_I64,
                "clc_sort_learned_pairs: keys must be U32, I32, F32, U64 or I64");
        int bytes, kind;
        key_kind_of(key_type, bytes, kind);
        gbc::learned_options o;
        if (options != nullptr) {
            o.sample = options->sample;
            o.points = options->points;
            o.buckets = options->buckets;
            o.steps = options->steps;
            o.lr = options->lr;
            o.use_model = options->use_model != 0;
            o.params_in = options->params_in;
            o.params_out = options->params_out;
            o.splitters_in = options->splitters_in;
            o.refine = options->refine;
        }
        gbc::learned_stats s;
        gbc::learned_sort_pairs(*ctx->ctx, keys_in, keys_out, bytes, kind, vals_in, vals_out, n, o, &s);
        if (stats != nullptr)
            *stats = clc_learned_stats{s.buckets,       s.nonempty_buckets,         s.largest_bucket,
                                       s.oversized_buckets, s.oversized_keys,      s.constant_keys,
                                       s.estimated_oversized_keys, s.violation,    s.fallback,
                                       s.first_loss,    s.last_loss,               s.refined_splitters};
    });
}

clc_status clc_learned_mlp_gradients(clc_context ctx, const float* params, const unsigned* centres, float inv_span,
                                     const unsigned* keys, const float* ys, size_t m, float* grad, float* loss)
{
    return guarded([&] {
        require(ctx != nullptr && params != nullptr && centres != nullptr && keys != nullptr && ys != nullptr &&
                    grad != nullptr && loss != nullptr,
                "clc: null argument");
        gbc::mlp_gradients(*ctx->ctx, params, centres, inv_span, keys, ys, m, grad, loss);
    });
}

// ---- CUDA graphs ------------------------------------------------------------

clc_status clc_graph_begin(clc_context ctx)
{
    if (ctx == nullptr) return fail(CLC_ERROR_INVALID_ARGUMENT, "clc: null context");
    return guarded([&] {
        ctx->ctx->activate();
        gbc::check_cuda(cudaStreamBeginCapture(ctx->ctx->stream, cudaStreamCaptureModeThreadLocal),
                        "cudaStreamBeginCapture");
    });
}

clc_status clc_graph_end(clc_context ctx, clc_graph* out)
{
    if (ctx == nullptr || out == nullptr) return fail(CLC_ERROR_INVALID_ARGUMENT, "clc: null argument");
    *out = nullptr;
    return guarded([&] {
        ctx->ctx->activate();
        cudaGraph_t g = nullptr;
        const cudaError_t e = cudaStreamEndCapture(ctx->ctx->stream, &g);
        ctx->ctx->upstream->flush_deferred();
        gbc::check_cuda(e, "cudaStreamEndCapture");
        cudaGraphExec_t exec = nullptr;
        const cudaError_t ei = cudaGraphInstantiate(&exec, g, 0);
        if (ei != cudaSuccess) cudaGraphDestroy(g);
        gbc::check_cuda(ei, "cudaGraphInstantiate");
        *out = new clc_graph_s{g, exec, ctx->ctx->device};
    });
}

clc_status clc_graph_launch(clc_context ctx, clc_graph graph)
{
    if (ctx == nullptr || graph == nullptr) return fail(CLC_ERROR_INVALID_ARGUMENT, "clc: null argument");
    return guarded([&] {
        require(graph->device == ctx->ctx->device, "clc: graph belongs to another device");
        ctx->ctx->activate();
        gbc::check_cuda(cudaGraphLaunch(graph->exec, ctx->ctx->stream), "cudaGraphLaunch");
    });
}

void clc_graph_release(clc_graph graph)
{
    if (graph == nullptr) return;
    cudaSetDevice(graph->device);
    cudaGraphExecDestroy(graph->exec);
    cudaGraphDestroy(graph->graph);
    delete graph;
}

// ---- buffers and context extras ------------------------------------------

void* clc_buffer_device_pointer(clc_buffer buffer) { return buffer == nullptr ? nullptr : buffer->ptr; }

clc_status clc_buffer_wrap(clc_context ctx, void* device_pointer, size_t bytes, clc_buffer* out)
{
    if (ctx == nullptr || out == nullptr) return fail(CLC_ERROR_INVALID_ARGUMENT, "clc: null argument");
    *out = nullptr;
    return guarded([&] {
        require(bytes == 0 || device_pointer != nullptr, "clc: null device pointer");
        *out = new clc_buffer_s{nullptr, ctx->ctx->holder, bytes == 0 ? nullptr : device_pointer, bytes};
    });
}

void* clc_context_stream(clc_context ctx) { return ctx == nullptr ? nullptr : (void*)ctx->ctx->stream; }

clc_status clc_context_memory_stats(clc_context ctx, clc_memory_stats* out)
{
    if (ctx == nullptr || out == nullptr) return fail(CLC_ERROR_INVALID_ARGUMENT, "clc: null argument");
    return guarded([&] {
        const gbc::stream_arena::usage u = ctx->ctx->arena->stats();
        out->current_bytes = u.current_bytes;
        out->peak_bytes = u.peak_bytes;
        out->total_bytes = u.total_bytes;
        out->current_allocations = u.current_allocations;
        out->total_allocations = u.total_allocations;
        out->cached_bytes = u.idle_bytes;
    });
}

clc_status clc_context_arena_info(clc_context ctx, size_t* held_bytes, size_t* slabs, size_t* slab_allocations,
                                  size_t* slab_releases)
{
    if (ctx == nullptr) return fail(CLC_ERROR_INVALID_ARGUMENT, "clc: null argument");
    return guarded([&] {
        const gbc::stream_arena::usage u = ctx->ctx->arena->stats();
        if (held_bytes != nullptr) *held_bytes = u.held_bytes;
        if (slabs != nullptr) *slabs = u.slabs;
        if (slab_allocations != nullptr) *slab_allocations = u.slab_allocations;
        if (slab_releases != nullptr) *slab_releases = u.slab_releases;
    });
}

clc_status clc_context_release_cache(clc_context ctx)
{
    if (ctx == nullptr) return fail(CLC_ERROR_INVALID_ARGUMENT, "clc: null argument");
    return guarded([&] {
        ctx->ctx->activate();
        ctx->ctx->arena->trim();
    });
}

clc_status clc_selftest_lookback_timeout(clc_context ctx)
{
    if (ctx == nullptr) return fail(CLC_ERROR_INVALID_ARGUMENT, "clc: null context");
    return guarded([&] {
        gbc::selftest_lookback_timeout(*ctx->ctx);
        ctx->ctx->finish();
    });
}

// ---- profiling ------------------------------------------------------------

clc_status clc_profile_enable(clc_context ctx, int enable)
{
    if (ctx == nullptr) return fail(CLC_ERROR_INVALID_ARGUMENT, "clc: null context");
    return guarded([&] { ctx->ctx->prof.enable(enable != 0); });
}

clc_status clc_profile_reset(clc_context ctx)
{
    if (ctx == nullptr) return fail(CLC_ERROR_INVALID_ARGUMENT, "clc: null context");
    return guarded([&] {
        ctx->ctx->activate();
        ctx->ctx->prof.reset(ctx->ctx->stream);
    });
}

clc_status clc_profile_count(clc_context ctx, size_t* count)
{
    if (ctx == nullptr || count == nullptr) return fail(CLC_ERROR_INVALID_ARGUMENT, "clc: null argument");
    return guarded([&] {
        ctx->ctx->activate();
        *count = ctx->ctx->prof.totals(ctx->ctx->stream).size();
    });
}

clc_status clc_profile_entry(clc_context ctx, size_t index, char* name, size_t name_bytes,
                             unsigned long long* launches, double* total_ms)
{
    return guarded([&] {
        require(ctx != nullptr && name != nullptr && name_bytes > 0 && launches != nullptr && total_ms != nullptr,
                "clc: null argument");
        ctx->ctx->activate();
        const auto t = ctx->ctx->prof.totals(ctx->ctx->stream);
        require(index < t.size(), "clc: profile index out of range");
        auto it = t.begin();
        std::advance(it, index);
        const std::size_t k = std::min(it->first.size(), name_bytes - 1);
        std::memcpy(name, it->first.data(), k);
        name[k] = '\0';
        *launches = it->second.launches;
        *total_ms = it->second.ms;
    });
}

// ---- tuning -------------------------------------------------------------

int clc_tuning_sort_variants(int key_bytes, int has_values)
{
    if (key_bytes != 4 && key_bytes != 8) return 0;
    return gbc::sort_variant_count(key_bytes, has_values != 0);
}

clc_status clc_tuning_sort_key(int key_bytes, int has_values, size_t n, char* out, size_t out_bytes)
{
    return guarded([&] {
        require(key_bytes == 4 || key_bytes == 8, "clc: key_bytes must be 4 or 8");
        require(out != nullptr && out_bytes > 0, "clc: null output");
        const std::string k = gbc::sort_tuning_key(key_bytes, has_values != 0, n);
        require(k.size() < out_bytes, "clc: output too small");
        std::memcpy(out, k.c_str(), k.size() + 1);
    });
}

clc_status clc_tuning_set(clc_context ctx, const char* key, int variant)
{
    return guarded([&] {
        require(ctx != nullptr && key != nullptr, "clc: null argument");
        gbc::launch_shape s;
        s.variant = variant;
        ctx->ctx->tuning.store(key, s);
    });
}

clc_status clc_tuning_get(clc_context ctx, const char* key, int* variant)
{
    return guarded([&] {
        require(ctx != nullptr && key != nullptr && variant != nullptr, "clc: null argument");
        gbc::launch_shape s;
        *variant = ctx->ctx->tuning.lookup(key, s) ? s.variant : -1;
    });
}

clc_status clc_autotune_sort(clc_context ctx, const void* keys_in, void* keys_out, clc_type key_type,
                             const uint32_t* vals_in, uint32_t* vals_out, size_t n, int repetitions, int* best_variant,
                             double* best_ms)
{
    return guarded([&] {
        require(ctx != nullptr, "clc: null context");
        int bytes, kind;
        key_kind_of(key_type, bytes, kind);
        const gbc::autotune_result r =
            gbc::autotune_sort(*ctx->ctx, keys_in, keys_out, bytes, kind, vals_in, vals_out, n, repetitions);
        if (best_variant != nullptr) *best_variant = r.best;
        if (best_ms != nullptr) *best_ms = r.best_ms;
    });
}

clc_status clc_autotune_segmented_sort(clc_context ctx, const void* keys_in, void* keys_out, clc_type key_type,
                                       const uint32_t* vals_in, uint32_t* vals_out, size_t n, const uint32_t* offsets,
                                       size_t num_segments, int repetitions, int* best_cta_cap, double* best_ms)
{
    return guarded([&] {
        require(ctx != nullptr, "clc: null context");
        int bytes, kind;
        key_kind_of(key_type, bytes, kind);
        const gbc::autotune_result r = gbc::autotune_segmented_sort(
            *ctx->ctx, keys_in, keys_out, bytes, kind, vals_in, vals_out, n, offsets, num_segments, repetitions);
        if (best_cta_cap != nullptr) *best_cta_cap = r.best;
        if (best_ms != nullptr) *best_ms = r.best_ms;
    });
}

clc_status clc_tuning_save(clc_context ctx, const char* path)
{
    return guarded([&] {
        require(ctx != nullptr, "clc: null context");
        std::string p = path != nullptr && *path ? std::string(path) : ctx->ctx->tuning_path;
        require(!p.empty(), "clc: no tuning table path (pass one, or create the context with a cache dir)");
        ctx->ctx->tuning.save(p);
    });
}

// ---- bitpack compression ---------------------------------------------------
// The reference's compressed_buffer (Compression.hpp, Compression.cpp:
// 139-278) has no C interface; these entry points carry its operations and
// its serialized form: an 8-word header {magic "CLBP", version 1, delta,
// chunk size, element count (2 words, low first), data words (2 words)}
// followed by the device words, validated on load as the reference does
// (Compression.cpp:226-275).

namespace {
constexpr uint32_t BITPACK_MAGIC = 0x50424C43u;  // "CLBP"
constexpr uint32_t BITPACK_VERSION = 1;
constexpr std::size_t BITPACK_HEADER_WORDS = 8;
}  // namespace

size_t clc_bitpack_words_bound(size_t n, size_t chunk_size)
{
    try {
        return gbc::bitpack_words_bound(n, chunk_size);
    } catch (...) {
        return 0;
    }
}

clc_status clc_bitpack_compress(clc_context ctx, clc_buffer in, size_t n, size_t chunk_size, int delta,
                                clc_buffer* out, size_t* out_words)
{
    if (ctx == nullptr || out == nullptr || out_words == nullptr)
        return fail(CLC_ERROR_INVALID_ARGUMENT, "clc: null argument");
    *out = nullptr;
    *out_words = 0;
    return guarded([&] {
        require_fits(in, n, CLC_TYPE_U32);
        require_same_device(ctx, in);
        std::unique_ptr<clc_buffer_s> b(new clc_buffer_s{ctx->ctx->resource, ctx->ctx->holder, nullptr, 0});
        const std::size_t words = gbc::bitpack_compress(
            *ctx->ctx, static_cast<const uint32_t*>(in->ptr), n, chunk_size, delta != 0, [&](std::size_t w) {
                b->bytes = w * 4;
                if (b->bytes != 0) b->ptr = b->resource->allocate(b->bytes);
                return static_cast<uint32_t*>(b->ptr);
            });
        if (n == 0) gbc::bitpack_words_bound(0, chunk_size);  // validates chunk_size
        *out_words = words;
        *out = b.release();
    });
}

clc_status clc_bitpack_decompress(clc_context ctx, clc_buffer data, size_t n, size_t chunk_size, int delta,
                                  clc_buffer out)
{
    return guarded([&] {
        require(ctx != nullptr, "clc: null context");
        require(data != nullptr, "clc: null buffer");
        require_fits(out, n, CLC_TYPE_U32);
        require_same_device(ctx, data);
        require_same_device(ctx, out);
        gbc::bitpack_decompress(*ctx->ctx, static_cast<const uint32_t*>(data->ptr), data->bytes / 4, n, chunk_size,
                                delta != 0, static_cast<uint32_t*>(out->ptr));
    });
}

clc_status clc_bitpack_compress_raw(clc_context ctx, const uint32_t* in, size_t n, size_t chunk_size, int delta,
                                    uint32_t* out, size_t out_capacity_words, size_t* out_words)
{
    if (ctx == nullptr || out_words == nullptr) return fail(CLC_ERROR_INVALID_ARGUMENT, "clc: null argument");
    *out_words = 0;
    return guarded([&] {
        require(n == 0 || in != nullptr, "clc: null input");
        std::size_t words = gbc::bitpack_compress(*ctx->ctx, in, n, chunk_size, delta != 0, [&](std::size_t w) {
            if (w > out_capacity_words || out == nullptr)
                throw std::invalid_argument("clc_bitpack_compress_raw: output capacity below the compressed size "
                                            "(clc_bitpack_words_bound gives a sufficient one)");
            return out;
        });
        if (n == 0) gbc::bitpack_words_bound(0, chunk_size);
        *out_words = words;
    });
}

clc_status clc_bitpack_decompress_raw(clc_context ctx, const uint32_t* data, size_t words, size_t n,
                                      size_t chunk_size, int delta, uint32_t* out)
{
    return guarded([&] {
        require(ctx != nullptr, "clc: null context");
        gbc::bitpack_decompress(*ctx->ctx, data, words, n, chunk_size, delta != 0, out);
    });
}

clc_status clc_bitpack_serialize(clc_context ctx, clc_buffer data, size_t n, size_t chunk_size, int delta, void* blob,
                                 size_t blob_bytes, size_t* needed)
{
    return guarded([&] {
        require(ctx != nullptr && data != nullptr, "clc: null argument");
        gbc::bitpack_words_bound(0, chunk_size);  // validates chunk_size
        const std::size_t words = data->bytes / 4;
        const std::size_t bytes = (BITPACK_HEADER_WORDS + words) * 4;
        if (needed != nullptr) *needed = bytes;
        if (blob == nullptr) return;
        require(blob_bytes >= bytes, "clc_bitpack_serialize: blob too small");
        const uint64_t n64 = n, w64 = words;
        const uint32_t header[BITPACK_HEADER_WORDS] = {
            BITPACK_MAGIC, BITPACK_VERSION, delta ? 1u : 0u, (uint32_t)chunk_size,
            (uint32_t)(n64 & 0xFFFFFFFFu), (uint32_t)(n64 >> 32), (uint32_t)(w64 & 0xFFFFFFFFu), (uint32_t)(w64 >> 32)};
        std::memcpy(blob, header, sizeof header);
        if (words != 0) {
            ctx->ctx->activate();
            gbc::check_cuda(cudaMemcpyAsync(static_cast<char*>(blob) + sizeof header, data->ptr, words * 4,
                                            cudaMemcpyDeviceToHost, ctx->ctx->stream),
                            "cudaMemcpyAsync");
            gbc::check_cuda(cudaStreamSynchronize(ctx->ctx->stream), "cudaStreamSynchronize");
        }
    });
}

clc_status clc_bitpack_deserialize(clc_context ctx, const void* blob, size_t blob_bytes, clc_buffer* data,
                                   size_t* n, size_t* chunk_size, int* delta)
{
    if (ctx == nullptr || blob == nullptr || data == nullptr || n == nullptr || chunk_size == nullptr ||
        delta == nullptr)
        return fail(CLC_ERROR_INVALID_ARGUMENT, "clc: null argument");
    *data = nullptr;
    return guarded([&] {
        uint32_t h[BITPACK_HEADER_WORDS];
        require(blob_bytes >= sizeof h, "bitpack: truncated header");
        std::memcpy(h, blob, sizeof h);
        require(h[0] == BITPACK_MAGIC && h[1] == BITPACK_VERSION, "bitpack: not a bitpack stream");
        const uint64_t count = h[4] | ((uint64_t)h[5] << 32), words = h[6] | ((uint64_t)h[7] << 32);
        require(blob_bytes == (BITPACK_HEADER_WORDS + words) * 4, "bitpack: size mismatch");
        const uint64_t chunk = h[3];
        const bool pow2 = chunk >= 256 && chunk <= 65536 && (chunk & (chunk - 1)) == 0;
        const uint64_t chunks = pow2 ? (count + chunk - 1) / chunk : 0;
        require(pow2 && (count == 0 || words >= 3 * chunks), "bitpack: corrupt header");
        require(count <= 0x7FFFFFFFu, "bitpack: more than 2^31-1 elements");
        // every chunk header must keep the unpack kernel inside the data
        const uint32_t* body = reinterpret_cast<const uint32_t*>(static_cast<const char*>(blob) + sizeof h);
        const uint64_t packed = words - 3 * chunks;
        for (uint64_t c = 0; c < chunks; ++c) {
            const uint64_t elems = std::min<uint64_t>(chunk, count - c * chunk);
            const uint32_t width = body[3 * c + 1];
            require(width <= 32 && (uint64_t)body[3 * c + 2] + (elems * width + 31) / 32 <= packed,
                    "bitpack: corrupt chunk header");
        }
        std::unique_ptr<clc_buffer_s> b(
            new clc_buffer_s{ctx->ctx->resource, ctx->ctx->holder, nullptr, (std::size_t)words * 4});
        ctx->ctx->activate();
        if (words != 0) {
            b->ptr = b->resource->allocate(b->bytes);
            gbc::check_cuda(cudaMemcpyAsync(b->ptr, body, b->bytes, cudaMemcpyHostToDevice, ctx->ctx->stream),
                            "cudaMemcpyAsync");
            gbc::check_cuda(cudaStreamSynchronize(ctx->ctx->stream), "cudaStreamSynchronize");
        }
        *n = (std::size_t)count;
        *chunk_size = (std::size_t)chunk;
        *delta = h[2] != 0 ? 1 : 0;
        *data = b.release();
    });
}

// ---- static_map --------------------------------------------------------------
// The reference's static_map (HashMap.hpp, HashMap.cpp:16-184) has no C
// interface; these entry points carry its operations.

clc_status clc_map_create(clc_context ctx, size_t capacity, uint32_t empty_key, uint32_t empty_value, clc_map* out)
{
    if (ctx == nullptr || out == nullptr) return fail(CLC_ERROR_INVALID_ARGUMENT, "clc: null argument");
    *out = nullptr;
    return guarded([&] {
        const std::size_t slots = gbc::static_map_slots(std::max<std::size_t>(capacity, 2));
        ctx->ctx->activate();
        std::unique_ptr<clc_map_s> m(
            new clc_map_s{ctx->ctx->resource, ctx->ctx->holder, nullptr, slots, empty_key, empty_value, 0});
        m->slots = m->resource->allocate(slots * 8);
        try {
            gbc::static_map_clear(*ctx->ctx, m->slots, slots, empty_key, empty_value);
        } catch (...) {
            m->resource->deallocate(m->slots, slots * 8);
            throw;
        }
        *out = m.release();
    });
}

void clc_map_release(clc_map map)
{
    if (map == nullptr) return;
    cudaSetDevice(map->holder->device);
    map->resource->deallocate(map->slots, map->capacity * 8);
    delete map;
}

clc_status clc_map_info(clc_map map, size_t* size, size_t* capacity, uint32_t* empty_key, uint32_t* empty_value)
{
    if (map == nullptr) return fail(CLC_ERROR_INVALID_ARGUMENT, "clc: null map");
    if (size != nullptr) *size = map->size;
    if (capacity != nullptr) *capacity = map->capacity;
    if (empty_key != nullptr) *empty_key = map->empty_key;
    if (empty_value != nullptr) *empty_value = map->empty_value;
    return fail(CLC_SUCCESS, "");
}

clc_status clc_map_clear(clc_context ctx, clc_map map)
{
    return guarded([&] {
        require(ctx != nullptr && map != nullptr, "clc: null argument");
        require(map->holder->device == ctx->ctx->device, "clc: map belongs to another device");
        gbc::static_map_clear(*ctx->ctx, map->slots, map->capacity, map->empty_key, map->empty_value);
        map->size = 0;
    });
}

clc_status clc_map_insert_raw(clc_context ctx, clc_map map, const uint32_t* keys, const uint32_t* values, size_t n,
                              size_t* inserted)
{
    if (inserted != nullptr) *inserted = 0;
    return guarded([&] {
        require(ctx != nullptr && map != nullptr, "clc: null argument");
        require(map->holder->device == ctx->ctx->device, "clc: map belongs to another device");
        std::size_t not_placed = 0;
        const std::size_t added = gbc::static_map_insert(*ctx->ctx, map->slots, map->capacity, map->empty_key,
                                                         map->empty_value, keys, values, n, not_placed);
        map->size += added;
        if (inserted != nullptr) *inserted = added;
        if (not_placed != 0)
            throw std::overflow_error("static_map::insert: table is full (" + std::to_string(not_placed) +
                                      " keys not inserted)");
    });
}

clc_status clc_map_insert(clc_context ctx, clc_map map, clc_buffer keys, clc_buffer values, size_t n,
                          size_t* inserted)
{
    if (keys == nullptr || values == nullptr) return fail(CLC_ERROR_INVALID_ARGUMENT, "clc: null buffer");
    if (n > keys->bytes / 4 || n > values->bytes / 4)
        return fail(CLC_ERROR_INVALID_ARGUMENT, "static_map::insert: n out of range");
    return clc_map_insert_raw(ctx, map, static_cast<const uint32_t*>(keys->ptr), static_cast<const uint32_t*>(values->ptr),
                              n, inserted);
}

clc_status clc_map_find_raw(clc_context ctx, clc_map map, const uint32_t* keys, size_t n, uint32_t* values)
{
    return guarded([&] {
        require(ctx != nullptr && map != nullptr, "clc: null argument");
        require(map->holder->device == ctx->ctx->device, "clc: map belongs to another device");
        gbc::static_map_find(*ctx->ctx, map->slots, map->capacity, map->empty_key, map->empty_value, keys, n, values);
    });
}

clc_status clc_map_find(clc_context ctx, clc_map map, clc_buffer keys, size_t n, clc_buffer values)
{
    if (keys == nullptr || values == nullptr) return fail(CLC_ERROR_INVALID_ARGUMENT, "clc: null buffer");
    if (n > keys->bytes / 4 || n > values->bytes / 4)
        return fail(CLC_ERROR_INVALID_ARGUMENT, "static_map::find: output too small");
    return clc_map_find_raw(ctx, map, static_cast<const uint32_t*>(keys->ptr), n, static_cast<uint32_t*>(values->ptr));
}

clc_status clc_map_contains_raw(clc_context ctx, clc_map map, const uint32_t* keys, size_t n, uint8_t* found)
{
    return guarded([&] {
        require(ctx != nullptr && map != nullptr, "clc: null argument");
        require(map->holder->device == ctx->ctx->device, "clc: map belongs to another device");
        gbc::static_map_contains(*ctx->ctx, map->slots, map->capacity, map->empty_key, keys, n, found);
    });
}

clc_status clc_map_contains(clc_context ctx, clc_map map, clc_buffer keys, size_t n, clc_buffer found)
{
    if (keys == nullptr || found == nullptr) return fail(CLC_ERROR_INVALID_ARGUMENT, "clc: null buffer");
    if (n > keys->bytes / 4 || n > found->bytes)
        return fail(CLC_ERROR_INVALID_ARGUMENT, "static_map::contains: output too small");
    return clc_map_contains_raw(ctx, map, static_cast<const uint32_t*>(keys->ptr), n, static_cast<uint8_t*>(found->ptr));
}

clc_status clc_map_slots(clc_context ctx, clc_map map, clc_buffer slot_keys, clc_buffer slot_values)
{
    return guarded([&] {
        require(ctx != nullptr && map != nullptr, "clc: null argument");
        require(slot_keys == nullptr || slot_keys->bytes >= map->capacity * 4, "clc: slot key buffer too small");
        require(slot_values == nullptr || slot_values->bytes >= map->capacity * 4, "clc: slot value buffer too small");
        gbc::static_map_unzip(*ctx->ctx, map->slots, map->capacity,
                              slot_keys ? static_cast<uint32_t*>(slot_keys->ptr) : nullptr,
                              slot_values ? static_cast<uint32_t*>(slot_values->ptr) : nullptr);
    });
}

}  // extern "C"
