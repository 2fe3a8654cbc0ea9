/*
 * gbcompute C interface: the drop-in boundary for the OpenCL Compute
 * library's primitive core (radix sort, scan, reduce, histogram), built for
 * one NVIDIA GB300 (sm_103a).
 *
 * The first part of this header keeps the names, enum values and argument
 * meaning of the reference C interface (lib/include/CL/Compute/compute_c.h)
 * so that a caller written against it relinks against libgbcompute.so:
 *   - every fallible call returns a clc_status and never lets a C++ exception
 *     escape; clc_last_error() holds a thread-local message;
 *   - handles are opaque; a buffer keeps its context's memory resource (and
 *     CUDA stream) alive, so it may outlive the context;
 *   - a context is not thread-safe: one per thread, or serialise;
 *   - sort, scan, fill, sequence and histogram are asynchronous on the
 *     context's stream; reduce and buffer reads/writes block; clc_finish waits.
 * CUDA replaces OpenCL underneath: clc_last_cl_error() reports the
 * cudaError_t of the last CLC_ERROR_OPENCL, a context owns one CUDA stream,
 * and operators are not compiled at run time but matched against a table of
 * canonical expressions (see clc_reduce).
 *
 * The second part adds what the reference does not have (64-bit keys,
 * segmented and learned sorts, reduce_by_key, histogram through C, raw device
 * pointers, graph capture, autotuning). Those functions say so.
 */
#ifndef GBCOMPUTE_COMPUTE_C_H
#define GBCOMPUTE_COMPUTE_C_H

#include <stddef.h>
#include <stdint.h>

#if defined(_WIN32)
#define GBC_EXPORT __declspec(dllexport)
#else
#define GBC_EXPORT __attribute__((visibility("default")))
#endif

#ifdef __cplusplus
extern "C" {
#endif

typedef struct clc_context_s* clc_context;
typedef struct clc_buffer_s* clc_buffer;
typedef struct clc_kernel_s* clc_kernel;
typedef struct clc_map_s* clc_map; /* extension: static_map */

/* Numeric values as in the reference (compute_c.h:30-41). */
typedef enum clc_status {
    CLC_SUCCESS = 0,
    CLC_ERROR_OPENCL = 1, /* device runtime error: clc_last_cl_error() has the cudaError_t */
    CLC_ERROR_INVALID_ARGUMENT = 2,
    CLC_ERROR_BUILD = 3, /* kept for ABI compatibility; kernels are compiled ahead of time */
    CLC_ERROR_NO_DEVICE = 4,
    CLC_ERROR_OUT_OF_MEMORY = 5,
    CLC_ERROR_UNSUPPORTED = 6, /* operator, type or feature without a kernel here */
    CLC_ERROR_INTERNAL = 7,
    CLC_ERROR_IO = 8
} clc_status;

/* Element types, numeric values as in the reference (compute_c.h:44-56). */
typedef enum clc_type {
    CLC_TYPE_I8 = 0,
    CLC_TYPE_U8 = 1,
    CLC_TYPE_I16 = 2,
    CLC_TYPE_U16 = 3,
    CLC_TYPE_I32 = 4,
    CLC_TYPE_U32 = 5,
    CLC_TYPE_I64 = 6,
    CLC_TYPE_U64 = 7,
    CLC_TYPE_F32 = 8,
    CLC_TYPE_F64 = 9
} clc_type;

/* Device index meaning "the first GPU" (compute_c.h:58-60). */
#define CLC_DEFAULT_DEVICE ((size_t)-1)

/* ---- errors (replaces compute_c.h:64-66) -------------------------------- */

GBC_EXPORT const char* clc_last_error(void);
/* cudaError_t of the last CLC_ERROR_OPENCL on this thread, else 0. */
GBC_EXPORT int clc_last_cl_error(void);

/* ---- devices and contexts (replaces compute_c.h:70-99) ------------------ */

typedef struct clc_device_info {
    char name[256];
    char platform[256];
    int is_gpu;
    int has_fp64;
    unsigned long long global_memory;
    size_t max_work_group_size;
} clc_device_info;

/* CUDA devices. *count = 0 with CLC_SUCCESS when there is no device or no
 * driver (compute_c.h:80-82). */
GBC_EXPORT clc_status clc_device_count(size_t* count);
GBC_EXPORT clc_status clc_device_get_info(size_t index, clc_device_info* info);

/* Creates a context: one CUDA stream, a pooled stream-ordered memory resource
 * and the tuning table (compute_c.h:86-89). */
GBC_EXPORT clc_status clc_context_create(size_t index, clc_context* out);
/* cache_dir holds the tuning table (gbcompute_tuning.txt); NULL or "" falls
 * back to CLC_TUNING_DIR, then CL_COMPUTE_CACHE_DIR (compute_c.h:90-94). */
GBC_EXPORT clc_status clc_context_create_with_cache(size_t index, const char* cache_dir,
                                                    clc_context* out);
GBC_EXPORT void clc_context_release(clc_context ctx);
GBC_EXPORT clc_status clc_context_get_info(clc_context ctx, clc_device_info* info);
/* Waits for the context's stream; reports an error a kernel recorded
 * (e.g. a look-back wait that timed out) as CLC_ERROR_OPENCL. */
GBC_EXPORT clc_status clc_finish(clc_context ctx);

/* ---- buffers (replaces compute_c.h:101-118) ----------------------------- */

GBC_EXPORT clc_status clc_buffer_alloc(clc_context ctx, size_t bytes, clc_buffer* out);
GBC_EXPORT void clc_buffer_release(clc_buffer buffer);
GBC_EXPORT size_t clc_buffer_size(clc_buffer buffer);
/* Blocking; offset + bytes must stay within the buffer. */
GBC_EXPORT clc_status clc_buffer_write(clc_context ctx, clc_buffer buffer, size_t offset,
                                       size_t bytes, const void* src);
GBC_EXPORT clc_status clc_buffer_read(clc_context ctx, clc_buffer buffer, size_t offset,
                                      size_t bytes, void* dst);
/* Asynchronous device-to-device copy on the context's stream. */
GBC_EXPORT clc_status clc_buffer_copy(clc_context ctx, clc_buffer src, size_t src_offset,
                                      clc_buffer dst, size_t dst_offset, size_t bytes);

/* ---- file I/O: outside this library's scope; return CLC_ERROR_UNSUPPORTED  */
GBC_EXPORT clc_status clc_file_size(const char* path, size_t* bytes);
GBC_EXPORT clc_status clc_file_read(clc_context ctx, const char* path, size_t file_offset,
                                    clc_buffer buffer, size_t buffer_offset, size_t bytes,
                                    size_t* done);
GBC_EXPORT clc_status clc_file_write(clc_context ctx, const char* path, int truncate,
                                     size_t file_offset, clc_buffer buffer, size_t buffer_offset,
                                     size_t bytes, size_t* done);

/* ---- typed algorithms (replaces compute_c.h:137-171) -------------------- */
/* Operators: a precedes b. Accepted spellings (whitespace-insensitive, outer
 * parentheses optional): "a + b", "a * b", "a & b", "a | b", "a ^ b",
 * "(b < a) ? b : a" / "min(a, b)", "(a < b) ? b : a" / "max(a, b)",
 * "b" (right projection) and "a" (left projection). Any other expression
 * returns CLC_ERROR_UNSUPPORTED. Identities: decimal or hex literals (with
 * an optional u/l suffix or float syntax), "(~0)", INT_MIN, INT_MAX, UINT_MAX,
 * LONG_MIN, LONG_MAX, ULONG_MAX, CHAR_MIN, CHAR_MAX, UCHAR_MAX, SHRT_MIN,
 * SHRT_MAX, USHRT_MAX, INFINITY, (-INFINITY). */

GBC_EXPORT clc_status clc_fill(clc_context ctx, clc_buffer out, size_t n, clc_type type,
                               const void* value);
GBC_EXPORT clc_status clc_sequence(clc_context ctx, clc_buffer out, size_t n, clc_type type,
                                   const void* start, const void* step);
/* out[i] = (out_type)(expression) with x = in[i] (and y = in2[i]); out may
 * alias an input of the same type. Replaces compute_c.h:147-154. The
 * expression is OpenCL C from a subset (operators, casts, literals, min/max/
 * clamp/abs/fabs/as_T/convert_T) compiled for an ahead-of-time interpreter:
 * malformed text is CLC_ERROR_BUILD with "build log" in clc_last_error(),
 * OpenCL C outside the subset CLC_ERROR_UNSUPPORTED. Asynchronous. */
GBC_EXPORT clc_status clc_transform(clc_context ctx, clc_buffer in, clc_type in_type,
                                    clc_buffer out, clc_type out_type, size_t n,
                                    const char* expression);
GBC_EXPORT clc_status clc_transform2(clc_context ctx, clc_buffer in1, clc_type type1,
                                     clc_buffer in2, clc_type type2, clc_buffer out,
                                     clc_type out_type, size_t n, const char* expression);
/* result = op(init, in[0] op ... op in[n-1]); blocks. n = 0 gives init. */
GBC_EXPORT clc_status clc_reduce(clc_context ctx, clc_buffer in, size_t n, clc_type type,
                                 const char* op, const char* identity, const void* init,
                                 void* result);
/* out may be in (in-place). Exclusive: out[0] = identity. */
GBC_EXPORT clc_status clc_scan(clc_context ctx, clc_buffer in, clc_buffer out, size_t n,
                               clc_type type, const char* op, const char* identity,
                               int exclusive);
/* Stable radix sort of 32-bit keys (I32, U32, F32) in place; values may be
 * NULL, else n 32-bit elements permuted alongside. Other key types give
 * CLC_ERROR_INVALID_ARGUMENT as in the reference (CApi.cpp:517-531). */
GBC_EXPORT clc_status clc_sort(clc_context ctx, clc_buffer keys, clc_type key_type,
                               clc_buffer values, size_t n, int descending);
/* Extension (no reference counterpart): compiles a transform expression
 * without a device and writes the program listing (one operation per line)
 * into listing[capacity] when listing is not NULL. Same statuses as
 * clc_transform. */
GBC_EXPORT clc_status clc_transform_compile(const char* expression, clc_type in_type, int has_in2,
                                            clc_type in2_type, clc_type out_type, char* listing,
                                            size_t capacity);
/* out[0 .. *count) = the elements x of in, in order, for which predicate
 * (an expression over x from the clc_transform subset) is nonzero; blocks.
 * Replaces compute_c.h:169-171 (copy_if). in and out must differ. */
GBC_EXPORT clc_status clc_copy_if(clc_context ctx, clc_buffer in, clc_buffer out, size_t n,
                                  clc_type type, const char* predicate, size_t* count);

/* ---- user kernels: need an OpenCL C compiler; CLC_ERROR_UNSUPPORTED ------ */
GBC_EXPORT clc_status clc_add_header(clc_context ctx, const char* name, const char* content);
GBC_EXPORT clc_status clc_kernel_create(clc_context ctx, const char* source, const char* name,
                                        const char* options, const char* const* define_names,
                                        const char* const* define_values, size_t ndefines,
                                        clc_kernel* out);
GBC_EXPORT void clc_kernel_release(clc_kernel kernel);
GBC_EXPORT clc_status clc_kernel_set_buffer(clc_kernel kernel, unsigned index, clc_buffer buffer);
GBC_EXPORT clc_status clc_kernel_set_value(clc_kernel kernel, unsigned index, size_t size,
                                           const void* value);
GBC_EXPORT clc_status clc_kernel_set_local(clc_kernel kernel, unsigned index, size_t bytes);
GBC_EXPORT clc_status clc_kernel_work_group_size(clc_context ctx, clc_kernel kernel, size_t limit,
                                                 size_t* out);
GBC_EXPORT clc_status clc_kernel_launch(clc_context ctx, clc_kernel kernel, size_t global,
                                        size_t local);

/* ======================================================================== */
/* Extensions (no counterpart in the reference C interface).               */
/* ======================================================================== */

/* Counts in[i] into bins equal-width bins over [lower, upper) exactly as the
 * reference's C++ histogram_even (Algorithm.hpp:243-250, Algorithm.cpp:
 * 240-273, 569-615): hist is zeroed first; for non-double input the bin is
 * (uint)(((float)x - lower) * scale) with scale = (float)bins / (upper -
 * lower) in float, clamped to bins - 1; out-of-range samples are ignored.
 * Asynchronous. */
GBC_EXPORT clc_status clc_histogram_even(clc_context ctx, clc_buffer in, size_t n, clc_type type,
                                         clc_buffer hist, size_t bins, double lower, double upper);

/* clc_scan plus a wide total: for 8/16/32-bit integer plus-scans, *total
 * (host, int64_t or uint64_t) receives the exact sum of all n inputs without
 * wrap-around; for other scans, the last inclusive value widened. Blocks when
 * total != NULL. */
GBC_EXPORT clc_status clc_scan_ex(clc_context ctx, clc_buffer in, clc_buffer out, size_t n,
                                  clc_type type, const char* op, const char* identity,
                                  int exclusive, void* total);

/* Stable sort of 32- or 64-bit keys (I32, U32, F32, I64, U64, F64) with
 * optional 32-bit values, in place. */
GBC_EXPORT clc_status clc_sort_ex(clc_context ctx, clc_buffer keys, clc_type key_type,
                                  clc_buffer values, size_t n, int descending);

/* Batched segmented sort: every segment [offsets[i], offsets[i+1]) of the
 * keys (and values) is sorted independently and stably, all segments in one
 * call. offsets holds num_segments + 1 monotone uint32 entries in device
 * memory. Keys: I32, U32, F32, I64, U64, F64; values: 32-bit or NULL. The
 * launch sequence does not depend on the data (small, medium and large
 * segments are told apart on the device), so the call can be captured with
 * clc_graph_begin/end once it has run (the pool must be warm). */
GBC_EXPORT clc_status clc_segmented_sort(clc_context ctx, clc_buffer keys, clc_type key_type, clc_buffer values,
                                         size_t n, clc_buffer offsets, size_t num_segments, int descending);
GBC_EXPORT clc_status clc_segmented_sort_raw(clc_context ctx, const void* keys_in, void* keys_out,
                                             clc_type key_type, const uint32_t* vals_in, uint32_t* vals_out,
                                             size_t n, const uint32_t* offsets, size_t num_segments,
                                             int descending);
/* Scan restarted at every segment start (position 0 always starts one);
 * exclusive: each segment's first output is the identity. */
GBC_EXPORT clc_status clc_segmented_scan(clc_context ctx, clc_buffer in, clc_buffer out, size_t n, clc_type type,
                                         const char* op, const char* identity, int exclusive, clc_buffer offsets,
                                         size_t num_segments);
GBC_EXPORT clc_status clc_segmented_scan_raw(clc_context ctx, const void* in, void* out, size_t n, clc_type type,
                                             const char* op, const char* identity, int exclusive,
                                             const uint32_t* offsets, size_t num_segments);

/* Learned-CDF sort of 32-bit keys (U32, I32, F32), out of place (keys_in is
 * left unchanged): a monotone 1 -> 32 -> 32 -> 1 fp32 network is fitted on the
 * GPU to a sample of the keys (fitting time is part of the call) and compiled
 * into bucket splitters; one counting pass and one scatter pass partition the
 * keys into the buckets, the segmented sort finishes them, and a boundary
 * check proves the result ordered. A model that would leave more than half of
 * the keys in buckets too large for one CTA's shared-memory sort (judged on
 * the sample, before the partition), or a failed check, sends the input to
 * the plain radix sort. The output is bit-identical to clc_sort's. Blocks
 * twice (to read the estimate and the statistics). options and stats may be
 * NULL. */
typedef struct clc_learned_options {
    int sample;   /* sampled keys (0: 2^20) */
    int points;   /* training points from the sorted sample (0: 8192) */
    int buckets;  /* partition buckets (0: about n / 8192, at least 4096, as many as shared memory holds) */
    int steps;    /* Adam steps (-1: none, the data-driven initial network as fitted) */
    float lr;     /* Adam learning rate (0: 0.01) */
    int use_model;                 /* 0: equal-width buckets over the sampled key range (no network) */
    const float* params_in;        /* host, clc_learned_param_count() floats, or NULL (data-driven init) */
    float* params_out;             /* host, receives the fitted parameters, or NULL */
    const unsigned* splitters_in;  /* host, buckets - 1 order-preserving keys replacing the compiled ones, or NULL */
    int refine; /* second model level: 1/refine of the buckets split the network's buckets that the sample predicts
                   oversized, at the sample's quantiles (-1: 3, the default; 0: off) */
} clc_learned_options;
typedef struct clc_learned_stats {
    unsigned buckets, nonempty_buckets, largest_bucket;
    unsigned oversized_buckets, oversized_keys; /* buckets beyond one CTA's shared-memory sort */
    unsigned constant_keys;                     /* keys in oversized buckets holding one key value */
    unsigned estimated_oversized_keys;          /* the same, predicted from the sample */
    unsigned violation;                         /* the boundary check failed */
    unsigned fallback;                          /* the plain radix sort produced the output */
    float first_loss, last_loss;                /* training loss at the first and last step */
    unsigned refined_splitters;                 /* splitters added by the second model level */
} clc_learned_stats;
GBC_EXPORT void clc_learned_default_options(clc_learned_options* options);
GBC_EXPORT clc_status clc_sort_learned(clc_context ctx, const void* keys_in, void* keys_out, clc_type key_type,
                                       size_t n, const clc_learned_options* options, clc_learned_stats* stats);
/* Extension: the learned-CDF sort of key-value pairs, stable, out of place:
 * keys U32 / I32 / F32 / U64 / I64 with 32-bit values; output identical to
 * clc_sort_ex's. 64-bit keys are bucketed through a monotone 32-bit
 * projection of the sample's key range. Synchronises. */
GBC_EXPORT clc_status clc_sort_learned_pairs(clc_context ctx, const void* keys_in, void* keys_out, clc_type key_type,
                                             const unsigned* vals_in, unsigned* vals_out, size_t n,
                                             const clc_learned_options* options, clc_learned_stats* stats);
/* One forward/backward pass of the network on the GPU over m points (host
 * arrays): keys in the order-preserving 32-bit domain and target CDF values;
 * the first layer sees (key - centres[j]) * inv_span. Returns the gradient of
 * the mean squared error with respect to the raw parameters (weights are
 * stored as v with w = exp(v)) and the loss. */
GBC_EXPORT int clc_learned_param_count(void);
GBC_EXPORT clc_status clc_learned_mlp_gradients(clc_context ctx, const float* params, const unsigned* centres,
                                                float inv_span, const unsigned* keys, const float* ys, size_t m,
                                                float* grad, float* loss);

/* reduce_by_key over grouped keys (equal keys adjacent, e.g. after a sort):
 * for run r, keys_out[r] is its key, sums_out[r] the sum of its uint32 values
 * as uint64 and counts_out[r] (if not NULL) its length. hist16 (NULL or 65,536
 * uint32 bins, zeroed by the call) counts the low 16 bits of every key.
 * Keys: any 4- or 8-byte type (equality of bit patterns). *num_runs (if not
 * NULL) receives the number of runs and makes the call blocking; otherwise it
 * is asynchronous. All pointers are device pointers except num_runs. */
GBC_EXPORT clc_status clc_reduce_by_key_raw(clc_context ctx, const void* keys, clc_type key_type,
                                            const uint32_t* values, size_t n, void* keys_out,
                                            unsigned long long* sums_out, uint32_t* counts_out, uint32_t* hist16,
                                            size_t* num_runs);

/* CUDA graphs: calls made on ctx between clc_graph_begin and clc_graph_end
 * are captured (not run) into a graph that clc_graph_launch replays on the
 * context's stream. Every call captured must have run once before on the same
 * context with the same sizes, so that its temporaries come from the pool;
 * a call that would allocate during capture fails with CLC_ERROR_UNSUPPORTED.
 * Blocking calls (reads, reduce, finish) cannot be captured. */
typedef struct clc_graph_s* clc_graph;
GBC_EXPORT clc_status clc_graph_begin(clc_context ctx);
GBC_EXPORT clc_status clc_graph_end(clc_context ctx, clc_graph* out);
GBC_EXPORT clc_status clc_graph_launch(clc_context ctx, clc_graph graph);
GBC_EXPORT void clc_graph_release(clc_graph graph);

/* Device pointer of a buffer (NULL for a zero-byte buffer). */
GBC_EXPORT void* clc_buffer_device_pointer(clc_buffer buffer);
/* Wraps existing device memory of the context's device as a buffer that does
 * not own it (the memory must outlive the buffer). */
GBC_EXPORT clc_status clc_buffer_wrap(clc_context ctx, void* device_pointer, size_t bytes,
                                      clc_buffer* out);
/* The context's CUDA stream (a cudaStream_t). */
GBC_EXPORT void* clc_context_stream(clc_context ctx);
/* Memory statistics of the context's arena: bytes and allocations live,
 * their peak and totals (of the sizes asked for), and cached_bytes, the
 * device memory the arena holds idle for reuse. */
typedef struct clc_memory_stats {
    size_t current_bytes, peak_bytes, total_bytes;
    size_t current_allocations, total_allocations;
    size_t cached_bytes;
} clc_memory_stats;
GBC_EXPORT clc_status clc_context_memory_stats(clc_context ctx, clc_memory_stats* out);
/* The arena's slabs: device bytes held, slab count, and how many slabs it
 * has taken from and handed back to the device so far. */
GBC_EXPORT clc_status clc_context_arena_info(clc_context ctx, size_t* held_bytes, size_t* slabs,
                                             size_t* slab_allocations, size_t* slab_releases);
/* Hands every idle slab of the context's arena back to the device. */
GBC_EXPORT clc_status clc_context_release_cache(clc_context ctx);

/* Raw-pointer forms: the same algorithms on device pointers, asynchronous on
 * the context's stream. keys_in == keys_out sorts in place. vals may be NULL. */
GBC_EXPORT clc_status clc_sort_keys_raw(clc_context ctx, const void* keys_in, void* keys_out,
                                        clc_type key_type, const uint32_t* vals_in,
                                        uint32_t* vals_out, size_t n, int descending);
GBC_EXPORT clc_status clc_scan_raw(clc_context ctx, const void* in, void* out, size_t n,
                                   clc_type type, const char* op, const char* identity,
                                   int exclusive, void* total_device);
GBC_EXPORT clc_status clc_histogram_even_raw(clc_context ctx, const void* in, size_t n,
                                             clc_type type, uint32_t* hist, size_t bins,
                                             double lower, double upper);
GBC_EXPORT clc_status clc_reduce_raw(clc_context ctx, const void* in, size_t n, clc_type type,
                                     const char* op, const char* identity, const void* init,
                                     void* result);

/* Bitpack compression of uint32 data: the reference's compress_bitpack /
 * decompress_bitpack and compressed_buffer::serialize / deserialize
 * (lib/include/CL/Compute/Compression.hpp, Compression.cpp:139-278), which
 * have no C entry points there. The device format is the reference's: per
 * chunk of chunk_size elements (a power of two in [256, 65536]) three words
 * {base, bit width, offset of its packed words}, then the packed words;
 * delta != 0 packs zigzag-encoded differences of consecutive elements.
 *
 * clc_bitpack_compress allocates *out (exactly *out_words words) from the
 * context and blocks once to learn the size. clc_bitpack_decompress writes n
 * elements to out, asynchronously. clc_bitpack_serialize writes the blob
 * (8-word header + data words) when blob is not NULL and reports its size in
 * *needed; clc_bitpack_deserialize validates a blob (magic, version, sizes,
 * and that every chunk header stays inside the data) and uploads its data.
 * The _raw forms work on device pointers: clc_bitpack_compress_raw needs an
 * output capacity of at least the compressed size, which
 * clc_bitpack_words_bound(n, chunk_size) bounds (0 for an invalid
 * chunk_size). */
GBC_EXPORT size_t clc_bitpack_words_bound(size_t n, size_t chunk_size);
GBC_EXPORT clc_status clc_bitpack_compress(clc_context ctx, clc_buffer in, size_t n, size_t chunk_size,
                                           int delta, clc_buffer* out, size_t* out_words);
GBC_EXPORT clc_status clc_bitpack_decompress(clc_context ctx, clc_buffer data, size_t n, size_t chunk_size,
                                             int delta, clc_buffer out);
GBC_EXPORT clc_status clc_bitpack_compress_raw(clc_context ctx, const uint32_t* in, size_t n, size_t chunk_size,
                                               int delta, uint32_t* out, size_t out_capacity_words,
                                               size_t* out_words);
GBC_EXPORT clc_status clc_bitpack_decompress_raw(clc_context ctx, const uint32_t* data, size_t words, size_t n,
                                                 size_t chunk_size, int delta, uint32_t* out);
GBC_EXPORT clc_status clc_bitpack_serialize(clc_context ctx, clc_buffer data, size_t n, size_t chunk_size,
                                            int delta, void* blob, size_t blob_bytes, size_t* needed);
GBC_EXPORT clc_status clc_bitpack_deserialize(clc_context ctx, const void* blob, size_t blob_bytes,
                                              clc_buffer* data, size_t* n, size_t* chunk_size, int* delta);

/* static_map: a fixed-capacity hash map from uint32 keys to uint32 values,
 * the reference's cl::compute::static_map (lib/include/CL/Compute/
 * HashMap.hpp, HashMap.cpp) through C, which the reference does not offer.
 * Open addressing with linear probing over a power-of-two table (capacity
 * rounded up, at least 2, at most 2^31), hashed with the MurmurHash3
 * finalizer; empty_key marks free slots and is never inserted; find returns
 * empty_value for absent keys; inserting a key already present keeps its
 * first value. Keep the load factor below ~0.7 for short probes.
 *
 * clc_map_insert blocks and reports how many keys were new; a full table
 * returns CLC_ERROR_OUT_OF_MEMORY ("table is full", as the reference throws
 * std::overflow_error) after inserting what fits. find/contains run
 * asynchronously on the context's stream and see every earlier insert;
 * found[i] is a byte, 1 when keys[i] is present. clc_map_slots copies the
 * table into separate slot-key and slot-value arrays (either may be NULL),
 * the reference's slot_keys()/slot_values(). A map holds its device memory
 * until clc_map_release and may outlive its context. */
GBC_EXPORT clc_status clc_map_create(clc_context ctx, size_t capacity, uint32_t empty_key, uint32_t empty_value,
                                     clc_map* out);
GBC_EXPORT void clc_map_release(clc_map map);
GBC_EXPORT clc_status clc_map_info(clc_map map, size_t* size, size_t* capacity, uint32_t* empty_key,
                                   uint32_t* empty_value);
GBC_EXPORT clc_status clc_map_clear(clc_context ctx, clc_map map);
GBC_EXPORT clc_status clc_map_insert(clc_context ctx, clc_map map, clc_buffer keys, clc_buffer values, size_t n,
                                     size_t* inserted);
GBC_EXPORT clc_status clc_map_find(clc_context ctx, clc_map map, clc_buffer keys, size_t n, clc_buffer values);
GBC_EXPORT clc_status clc_map_contains(clc_context ctx, clc_map map, clc_buffer keys, size_t n, clc_buffer found);
GBC_EXPORT clc_status clc_map_slots(clc_context ctx, clc_map map, clc_buffer slot_keys, clc_buffer slot_values);
GBC_EXPORT clc_status clc_map_insert_raw(clc_context ctx, clc_map map, const uint32_t* keys, const uint32_t* values,
                                         size_t n, size_t* inserted);
GBC_EXPORT clc_status clc_map_find_raw(clc_context ctx, clc_map map, const uint32_t* keys, size_t n,
                                       uint32_t* values);
GBC_EXPORT clc_status clc_map_contains_raw(clc_context ctx, clc_map map, const uint32_t* keys, size_t n,
                                           uint8_t* found);

/* Allocation-free int32 plus-scan. No counterpart in the reference.
 *
 * For callers that cannot allocate device memory when they need a scan: code
 * whose device memory belongs to another allocator (a framework's caching
 * allocator, a fixed arena on a shared GPU) and code that cannot afford the
 * device-wide synchronisation of cudaFree. The call allocates nothing and
 * needs no clc_context: its scratch (one look-back status word per tile of
 * 16,384 elements, and a tile counter) is a fixed 128 KiB array inside the
 * library, so n is limited to 2^28 elements; larger n returns
 * CLC_ERROR_INVALID_ARGUMENT without launching anything.
 *
 * in and out are device pointers of the current device (out may equal in);
 * exclusive != 0 gives an exclusive scan (out[0] = 0). The scan is enqueued on
 * `stream` (a cudaStream_t; NULL is the legacy default stream) and the call
 * returns without waiting. Sums wrap modulo 2^32, as clc_scan's do.
 *
 * The first call on a device looks up the device address of the scratch
 * array (cudaGetSymbolAddress) with that device current; make that first call
 * before any stream capture. Every call shares the one array and clears the
 * part it uses before its kernel runs, so calls whose work may overlap on the
 * GPU (other streams, other host threads) race and must be serialised by the
 * caller. The stream, in and out must belong to the current device
 * (CLC_ERROR_INVALID_ARGUMENT otherwise).
 *
 * The scan's look-back waits are bounded (about one second). A wait that runs
 * out sets an error word in the same array and leaves that call's output
 * incomplete; since the call has returned by then, ask
 * clc_scan_i32_noalloc_status afterwards. */
GBC_EXPORT clc_status clc_scan_i32_noalloc(const int32_t* in, int32_t* out, size_t n, int exclusive,
                                           void* stream);

/* Companion of clc_scan_i32_noalloc, allocating nothing either: waits for
 * `stream`, then returns CLC_ERROR_OPENCL if any clc_scan_i32_noalloc call on
 * the current device had a look-back wait run out since the last status
 * query (and clears that error word), CLC_SUCCESS otherwise. */
GBC_EXPORT clc_status clc_scan_i32_noalloc_status(void* stream);

/* Failure-path self-test of the allocation-free scan: scans buf (2 to 16,384
 * tiles of 16,384 int32, device memory of the current device) with its first
 * tile never run, so the next tile's bounded wait gives up after about one
 * second and sets the error word; clc_scan_i32_noalloc_status then reports
 * it. buf's contents are overwritten. */
GBC_EXPORT clc_status clc_selftest_noalloc_timeout(int32_t* buf, size_t n, void* stream);

/* Failure-path self-test: runs one scan tile whose predecessor never
 * publishes its status, so the tile's bounded look-back wait gives up after
 * about one second instead of hanging. Returns what the next synchronising
 * call reports: CLC_ERROR_OPENCL with a "timed out" message. The context
 * stays usable. */
GBC_EXPORT clc_status clc_selftest_lookback_timeout(clc_context ctx);

/* Profiling: when enabled, every kernel launch is bracketed by CUDA events on
 * the context's stream and its time accumulated per kernel family
 * ("sort.digit_pass", "scan.lookback", ...). Reading entries synchronises. */
GBC_EXPORT clc_status clc_profile_enable(clc_context ctx, int enable);
GBC_EXPORT clc_status clc_profile_reset(clc_context ctx);
GBC_EXPORT clc_status clc_profile_count(clc_context ctx, size_t* count);
GBC_EXPORT clc_status clc_profile_entry(clc_context ctx, size_t index, char* name, size_t name_bytes,
                                        unsigned long long* launches, double* total_ms);

/* Tuning: entries of the context's table and how many compiled variants a
 * sort family has; clc_autotune_* time them and store the fastest (or set an
 * entry with clc_tuning_set); clc_tuning_save writes the table. */
GBC_EXPORT int clc_tuning_sort_variants(int key_bytes, int has_values);
GBC_EXPORT clc_status clc_tuning_sort_key(int key_bytes, int has_values, size_t n, char* out,
                                          size_t out_bytes);
GBC_EXPORT clc_status clc_tuning_set(clc_context ctx, const char* key, int variant);
GBC_EXPORT clc_status clc_tuning_get(clc_context ctx, const char* key, int* variant);
GBC_EXPORT clc_status clc_tuning_save(clc_context ctx, const char* path);

/* Autotuner: times every compiled launch shape of the plain sort (the
 * variants differ in threads per CTA, keys per thread, CTAs per SM, look-back
 * window and bulk-copy staging; digits are 8 bits throughout) on the
 * caller's device data, stores the fastest in the context's tuning table
 * under the workload's key (element type and size class) and returns it with
 * its time per call. The entry applies to every key distribution of that
 * class, so the default variant (the one used without an entry, a shape
 * that holds up on skewed keys) is kept unless another is more than 2%
 * faster. keys_in must differ from keys_out, which receives the sorted keys.
 * Blocks. */
GBC_EXPORT clc_status clc_autotune_sort(clc_context ctx, const void* keys_in, void* keys_out, clc_type key_type,
                                        const uint32_t* vals_in, uint32_t* vals_out, size_t n, int repetitions,
                                        int* best_variant, double* best_ms);
/* The same for the segmented sort: the candidates are capacities of its
 * one-CTA size class; the key adds the class of the average segment length.
 * The MSD route's capacity, the one-CTA sorts' thread count and the launch
 * form are tuned after it and stored under the same key with ":msd",
 * ":threads" and ":batch". */
GBC_EXPORT clc_status clc_autotune_segmented_sort(clc_context ctx, const void* keys_in, void* keys_out,
                                                  clc_type key_type, const uint32_t* vals_in, uint32_t* vals_out,
                                                  size_t n, const uint32_t* offsets, size_t num_segments,
                                                  int repetitions, int* best_cta_cap, double* best_ms);

#ifdef __cplusplus
}
#endif

#endif
