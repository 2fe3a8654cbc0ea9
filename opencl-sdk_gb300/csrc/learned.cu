// Learned-CDF sort: a small monotone MLP fitted on the GPU to a sample of the
// keys predicts each key's CDF and scatters the keys into buckets in one pass;
// the buckets are then finished by the segmented sort (shared-memory sorts,
// with oversized buckets routed to its batched onesweep radix sort), and any
// monotonicity violation sends the whole input to the plain radix sort.
//
// No reference counterpart. The output is the plain radix sort's output bit
// for bit (the reference's key order, Algorithm.cpp:459-469): bucket order is a
// monotone function of the key, each bucket is sorted exactly, and the check
// proves the concatenation ordered.
//
// Steps (all on the context's stream):
//   1. sample S keys at a fixed stride, in the order-preserving u32 form, and
//      sort the sample with the plain radix sort;
//   2. training points: x = the normalised key of sample quantile i/M,
//      y = (i + 0.5) / M;
//   3. fit 1 -> H -> H -> 1 (ReLU, weights w = v^2 >= 0, so the network is
//      monotone non-decreasing by construction) with full-batch Adam, one
//      kernel launch per step: each CTA runs forward and backward for its
//      points, the last CTA to finish sums the partial gradients and updates;
//   4. compile: evaluate alpha * network(x) + (1 - alpha) * x on a GRID + 1
//      point table; a key's bucket is floor(B * interp(table, x(key))),
//      monotone in the key;
//   5. count keys per (CTA chunk, bucket), exclusive offsets bucket-major,
//      scatter (shared-memory cursors per bucket);
//   6. segmented sort of the B buckets; 7. boundary check; fallback if needed.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "device_common.cuh"
#include "learned.hpp"
#include "runtime.hpp"
#include "segmented.hpp"

namespace gbc {
namespace learned {

// ---- parameter layout (floats) ---------------------------------------------
constexpr int OFF_V1 = 0, OFF_B1 = H, OFF_V2 = 2 * H, OFF_B2 = 2 * H + H * H, OFF_V3 = 3 * H + H * H,
              OFF_B3 = 4 * H + H * H;
static_assert(OFF_B3 + 1 == NPARAM, "parameter layout");

constexpr int TRAIN_THREADS = 256;  // one training point per thread
constexpr int PSTRIDE = TRAIN_THREADS + 1;  // padded row of per-point activations

__device__ __forceinline__ float relu(float z) { return z > 0.f ? z : 0.f; }

// Order-preserving u32 view of a key (floats: sign ? ~k : k | sign).
__device__ __forceinline__ uint32_t ordered(uint32_t k, int kind)
{
    if (kind == 1) return k ^ 0x80000000u;
    if (kind == 2) return (k & 0x80000000u) ? ~k : (k | 0x80000000u);
    return k;
}

struct Norm {
    uint32_t umin;
    float inv_range;
    __device__ __forceinline__ float operator()(uint32_t u) const
    {
        const uint32_t d = u > umin ? u - umin : 0u;
        return fminf((float)d * inv_range, 1.0f);
    }
};

// ---- 1. sample ---------------------------------------------------------------
__global__ void k_sample(const uint32_t* __restrict__ keys, uint32_t n, uint32_t* __restrict__ sample, uint32_t s,
                         int kind)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < s) {
        const uint32_t idx = (uint32_t)(((uint64_t)i * n) / s);
        sample[i] = ordered(keys[idx], kind);
    }
}

// ---- 2. training points --------------------------------------------------
// stats[0] = umin, stats[1] = umax (ordered), from the sorted sample.
__global__ void k_points(const uint32_t* __restrict__ sorted, uint32_t s, float* __restrict__ xs,
                         float* __restrict__ ys, uint32_t m, uint32_t* __restrict__ range)
{
    const uint32_t umin = sorted[0], umax = sorted[s - 1];
    const float inv = umax > umin ? 1.0f / (float)(umax - umin) : 0.f;
    const Norm norm{umin, inv};
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i == 0) {
        range[0] = umin;
        range[1] = umax;
    }
    if (i < m) {
        const uint32_t q = (uint32_t)(((uint64_t)(2 * i + 1) * s) / (2 * (uint64_t)m));
        xs[i] = norm(sorted[min(q, s - 1)]);
        ys[i] = ((float)i + 0.5f) / (float)m;
    }
}

// ---- 3. training -------------------------------------------------------------
__global__ void k_init_params(float* p, float* adam_m, float* adam_s)
{
    for (int i = threadIdx.x; i < NPARAM; i += blockDim.x) {
        float v = 0.f;
        if (i < OFF_B1) v = 1.0f;                                                     // w1 = 1
        else if (i < OFF_V2) v = -((float)(i - OFF_B1) + 0.5f) / (float)H;            // ramps across [0, 1]
        else if (i < OFF_B2) {                                                        // w2 ~ (0.25 .. 2.25) / H
            const uint32_t h = (uint32_t)(i - OFF_V2) * 2654435761u;
            v = sqrtf((0.25f + 2.0f * (float)(h >> 8) / 16777216.0f) / (float)H);
        } else if (i < OFF_V3) v = 0.f;
        else if (i < OFF_B3) v = sqrtf(1.0f / (float)H);
        else v = 0.f;
        p[i] = v;
        adam_m[i] = 0.f;
        adam_s[i] = 0.f;
    }
}

// Forward and backward for one point per thread; per-CTA gradient sums to
// partial[blockIdx.x]; the last CTA sums the partials and (when lr > 0)
// applies one Adam step. grad_out (optional) receives the summed gradient with
// respect to the raw parameters, loss_out[step] the mean squared error.
struct TrainArgs {
    float* params;
    float* adam_m;
    float* adam_s;
    const float* xs;
    const float* ys;
    uint32_t m;
    float* partial;  // [gridDim.x][NPARAM + 1]
    uint32_t* ticket;
    float* grad_out;
    float* loss_out;
    int step;  // 1-based Adam step
    float lr;
};

__global__ void __launch_bounds__(TRAIN_THREADS) k_train_step(TrainArgs a)
{
    extern __shared__ float sm[];
    float* w = sm;                                 // NPARAM: weights squared, biases copied
    float* H1 = w + NPARAM;                        // [H][PSTRIDE]
    float* D2 = H1 + H * PSTRIDE;                  // [H][PSTRIDE]
    float* D1 = D2 + H * PSTRIDE;                  // [H][PSTRIDE]
    float* H2 = D1 + H * PSTRIDE;                  // [H][PSTRIDE]
    float* X = H2 + H * PSTRIDE;                   // [PSTRIDE]
    float* G = X + PSTRIDE;                        // [PSTRIDE]
    __shared__ float s_red[TRAIN_THREADS / 32];
    __shared__ bool s_last;
    const int tid = threadIdx.x;
    for (int i = tid; i < NPARAM; i += TRAIN_THREADS) {
        const float v = a.params[i];
        const bool is_w = i < OFF_B1 || (i >= OFF_V2 && i < OFF_B2) || (i >= OFF_V3 && i < OFF_B3);
        w[i] = is_w ? v * v : v;
    }
    __syncthreads();

    const uint32_t p = blockIdx.x * TRAIN_THREADS + tid;
    const bool valid = p < a.m;
    const float x = valid ? a.xs[p] : 0.f;
    const float y = valid ? a.ys[p] : 0.f;
    float h1[H], h2[H];
    uint32_t on1 = 0, on2 = 0;
#pragma unroll
    for (int j = 0; j < H; ++j) {
        const float z = w[OFF_V1 + j] * x + w[OFF_B1 + j];
        h1[j] = relu(z);
        on1 |= (z > 0.f ? 1u : 0u) << j;
    }
    float yhat = w[OFF_B3];
#pragma unroll 4
    for (int k = 0; k < H; ++k) {
        float z = w[OFF_B2 + k];
#pragma unroll
        for (int j = 0; j < H; ++j) z += w[OFF_V2 + k * H + j] * h1[j];
        h2[k] = relu(z);
        on2 |= (z > 0.f ? 1u : 0u) << k;
        yhat += w[OFF_V3 + k] * h2[k];
    }
    const float err = valid ? yhat - y : 0.f;
    const float g = 2.f * err / (float)a.m;
    float d2[H];
#pragma unroll
    for (int k = 0; k < H; ++k) d2[k] = ((on2 >> k) & 1) ? g * w[OFF_V3 + k] : 0.f;
#pragma unroll
    for (int j = 0; j < H; ++j) {
        float s = 0.f;
#pragma unroll
        for (int k = 0; k < H; ++k) s += d2[k] * w[OFF_V2 + k * H + j];
        D1[j * PSTRIDE + tid] = ((on1 >> j) & 1) ? s : 0.f;
        H1[j * PSTRIDE + tid] = h1[j];
        D2[j * PSTRIDE + tid] = d2[j];
        H2[j * PSTRIDE + tid] = h2[j];
    }
    X[tid] = x;
    G[tid] = g;
    // loss partial
    float l = err * err;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) l += __shfl_down_sync(dev::FULL_MASK, l, o);
    if ((tid & 31) == 0) s_red[tid >> 5] = l;
    __syncthreads();

    // Gradient sums over this CTA's points, with respect to the weights w
    // (converted to the raw v = sqrt(w) parameters by the last CTA).
    float* out = a.partial + (size_t)blockIdx.x * (NPARAM + 1);
    {
        // dW2[k][j] = sum_p D2[k][p] H1[j][p]: thread t owns k = t / 8, j = 4 (t % 8) .. + 3
        const int k = tid >> 3, j0 = (tid & 7) * 4;
        float acc[4] = {0.f, 0.f, 0.f, 0.f};
        for (int q = 0; q < TRAIN_THREADS; ++q) {
            const float d = D2[k * PSTRIDE + q];
#pragma unroll
            for (int r = 0; r < 4; ++r) acc[r] += d * H1[(j0 + r) * PSTRIDE + q];
        }
#pragma unroll
        for (int r = 0; r < 4; ++r) out[OFF_V2 + k * H + j0 + r] = acc[r];
    }
    if (tid < 5 * H + 1) {
        // 0..H-1: dW1, H..2H-1: db1, 2H..3H-1: db2, 3H..4H-1: dW3, 4H..5H-1: unused, 5H: db3
        const int kind = tid / H, u = tid % H;
        float acc = 0.f;
        for (int q = 0; q < TRAIN_THREADS; ++q) {
            switch (kind) {
            case 0: acc += D1[u * PSTRIDE + q] * X[q]; break;
            case 1: acc += D1[u * PSTRIDE + q]; break;
            case 2: acc += D2[u * PSTRIDE + q]; break;
            case 3: acc += G[q] * H2[u * PSTRIDE + q]; break;
            default: acc += G[q]; break;
            }
        }
        if (kind == 0) out[OFF_V1 + u] = acc;
        else if (kind == 1) out[OFF_B1 + u] = acc;
        else if (kind == 2) out[OFF_B2 + u] = acc;
        else if (kind == 3) out[OFF_V3 + u] = acc;
        else if (kind == 5) out[OFF_B3] = acc;
    }
    if (tid == 0) {
        float l2 = 0.f;
        for (int i = 0; i < TRAIN_THREADS / 32; ++i) l2 += s_red[i];
        out[NPARAM] = l2;
    }
    __threadfence();
    __syncthreads();
    if (tid == 0) s_last = atomicAdd(a.ticket, 1u) == gridDim.x - 1;
    __syncthreads();
    if (!s_last) return;
    __threadfence();

    // Last CTA: sum the partials in CTA order and update.
    const float b1c = 1.f - powf(0.9f, (float)a.step), b2c = 1.f - powf(0.999f, (float)a.step);
    for (int i = tid; i <= NPARAM; i += TRAIN_THREADS) {
        float sum = 0.f;
        for (uint32_t c = 0; c < gridDim.x; ++c) sum += *((volatile float*)(a.partial + (size_t)c * (NPARAM + 1) + i));
        if (i == NPARAM) {
            if (a.loss_out) a.loss_out[a.step - 1] = sum / (float)a.m;
            continue;
        }
        const float v = a.params[i];
        const bool is_w = i < OFF_B1 || (i >= OFF_V2 && i < OFF_B2) || (i >= OFF_V3 && i < OFF_B3);
        const float grad = is_w ? sum * 2.f * v : sum;  // d/dv of w = v^2
        if (a.grad_out) a.grad_out[i] = grad;
        if (a.lr > 0.f) {
            const float m1 = 0.9f * a.adam_m[i] + 0.1f * grad;
            const float s1 = 0.999f * a.adam_s[i] + 0.001f * grad * grad;
            a.adam_m[i] = m1;
            a.adam_s[i] = s1;
            a.params[i] = v - a.lr * (m1 / b1c) / (sqrtf(s1 / b2c) + 1e-8f);
        }
    }
    if (tid == 0) *a.ticket = 0;  // ready for the next step's launch
}

// ---- 4. compile the network into a CDF table -----------------------------
__global__ void k_table(const float* __restrict__ params, float* __restrict__ table, int grid_pts, float alpha)
{
    __shared__ float w[NPARAM];
    for (int i = threadIdx.x; i < NPARAM; i += blockDim.x) {
        const float v = params[i];
        const bool is_w = i < OFF_B1 || (i >= OFF_V2 && i < OFF_B2) || (i >= OFF_V3 && i < OFF_B3);
        w[i] = is_w ? v * v : v;
    }
    __syncthreads();
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i > grid_pts) return;
    const float x = (float)i / (float)grid_pts;
    float h1[H];
#pragma unroll
    for (int j = 0; j < H; ++j) h1[j] = relu(w[OFF_V1 + j] * x + w[OFF_B1 + j]);
    float y = w[OFF_B3];
    for (int k = 0; k < H; ++k) {
        float z = w[OFF_B2 + k];
#pragma unroll
        for (int j = 0; j < H; ++j) z += w[OFF_V2 + k * H + j] * h1[j];
        y += w[OFF_V3 + k] * relu(z);
    }
    // alpha * F(x) + (1 - alpha) * x: the linear share bounds the slope from
    // below, so modes the network cannot resolve are never merged.
    table[i] = alpha * fminf(fmaxf(y, 0.f), 1.f) + (1.f - alpha) * x;
}

// The identity table: bucket by the normalised key alone (the method without
// the network, for comparison).
__global__ void k_table_linear(float* table, int grid_pts)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i <= grid_pts) table[i] = (float)i / (float)grid_pts;
}

// ---- 5. partition ----------------------------------------------------------
struct PartArgs {
    const uint32_t* keys;
    uint32_t* out;
    uint32_t n;
    int kind;
    const uint32_t* range;  // umin, umax
    const float* table;
    int grid_pts;
    uint32_t buckets;
    uint32_t* counts;   // [gridDim.x][buckets]: counts, then absolute start offsets
    uint32_t* bucket_off;  // [buckets + 1]
};

struct BucketFn {
    Norm norm;
    const float* table;
    int grid_pts;
    uint32_t buckets;
    __device__ __forceinline__ uint32_t operator()(uint32_t u) const
    {
        const float s = norm(u) * (float)grid_pts;
        const int i = min((int)s, grid_pts - 1);
        const float f = s - (float)i;
        const float lo = table[i];
        const float c = lo + (table[i + 1] - lo) * f;
        return min((uint32_t)(c * (float)buckets), buckets - 1);
    }
};

__device__ __forceinline__ BucketFn make_bucket_fn(const PartArgs& a, const float* table)
{
    const uint32_t umin = a.range[0], umax = a.range[1];
    return BucketFn{Norm{umin, umax > umin ? 1.0f / (float)(umax - umin) : 0.f}, table, a.grid_pts, a.buckets};
}

constexpr int PART_THREADS = 1024;

__global__ void __launch_bounds__(PART_THREADS) k_count(PartArgs a)
{
    extern __shared__ uint32_t sh[];
    uint32_t* hist = sh;                                          // buckets
    float* table = reinterpret_cast<float*>(sh + a.buckets);      // grid + 1
    for (uint32_t i = threadIdx.x; i < a.buckets; i += PART_THREADS) hist[i] = 0;
    for (int i = threadIdx.x; i <= a.grid_pts; i += PART_THREADS) table[i] = a.table[i];
    __syncthreads();
    const BucketFn bf = make_bucket_fn(a, table);
    const uint32_t chunk = (a.n + gridDim.x - 1) / gridDim.x;
    const uint32_t b0 = blockIdx.x * chunk, b1 = min(a.n, b0 + chunk);
    for (uint32_t i = b0 + threadIdx.x; i < b1; i += PART_THREADS)
        atomicAdd(&hist[bf(ordered(a.keys[i], a.kind))], 1u);
    __syncthreads();
    uint32_t* row = a.counts + (size_t)blockIdx.x * a.buckets;
    for (uint32_t i = threadIdx.x; i < a.buckets; i += PART_THREADS) row[i] = hist[i];
}

// Column prefix over CTAs (per bucket) and bucket totals; one thread per bucket.
__global__ void k_columns(uint32_t* counts, uint32_t rows, uint32_t buckets, uint32_t* totals)
{
    const uint32_t b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= buckets) return;
    uint32_t run = 0;
    for (uint32_t r = 0; r < rows; ++r) {
        const uint32_t c = counts[(size_t)r * buckets + b];
        counts[(size_t)r * buckets + b] = run;
        run += c;
    }
    totals[b] = run;
}

// Exclusive scan of the bucket totals (one CTA), bucket_off[buckets] = n.
__global__ void __launch_bounds__(1024) k_bucket_scan(const uint32_t* totals, uint32_t buckets, uint32_t* bucket_off)
{
    __shared__ uint32_t s_warp[32], s_carry;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (threadIdx.x == 0) s_carry = 0;
    __syncthreads();
    for (uint32_t base = 0; base < buckets; base += 1024) {
        const uint32_t i = base + threadIdx.x;
        const uint32_t c = i < buckets ? totals[i] : 0u;
        const uint32_t x = dev::warp_inclusive_scan(c, [](uint32_t p, uint32_t q) { return p + q; });
        if (lane == 31) s_warp[warp] = x;
        __syncthreads();
        uint32_t before = s_carry;
        for (int w = 0; w < warp; ++w) before += s_warp[w];
        if (i < buckets) bucket_off[i] = before + x - c;
        __syncthreads();
        if (threadIdx.x == 1023) s_carry = before + x;
        __syncthreads();
    }
    if (threadIdx.x == 0) bucket_off[buckets] = s_carry;
}

__global__ void __launch_bounds__(PART_THREADS) k_scatter(PartArgs a)
{
    extern __shared__ uint32_t sh[];
    uint32_t* cursor = sh;
    float* table = reinterpret_cast<float*>(sh + a.buckets);
    const uint32_t* row = a.counts + (size_t)blockIdx.x * a.buckets;
    for (uint32_t i = threadIdx.x; i < a.buckets; i += PART_THREADS) cursor[i] = a.bucket_off[i] + row[i];
    for (int i = threadIdx.x; i <= a.grid_pts; i += PART_THREADS) table[i] = a.table[i];
    __syncthreads();
    const BucketFn bf = make_bucket_fn(a, table);
    const uint32_t chunk = (a.n + gridDim.x - 1) / gridDim.x;
    const uint32_t b0 = blockIdx.x * chunk, b1 = min(a.n, b0 + chunk);
    for (uint32_t i = b0 + threadIdx.x; i < b1; i += PART_THREADS) {
        const uint32_t k = a.keys[i];
        const uint32_t pos = atomicAdd(&cursor[bf(ordered(k, a.kind))], 1u);
        if (pos < a.n) a.out[pos] = k;
    }
}

// ---- 6/7. statistics and the boundary check ----------------------------------
// stats: [0] violation flag, [1] keys in oversized buckets, [2] oversized
// buckets, [3] largest bucket, [4] non-empty buckets.
__global__ void k_check(const uint32_t* __restrict__ out, const uint32_t* __restrict__ bucket_off, uint32_t buckets,
                        int kind, uint32_t cap, uint32_t* stats)
{
    const uint32_t b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= buckets) return;
    const uint32_t s = bucket_off[b], e = bucket_off[b + 1];
    const uint32_t len = e - s;
    if (len > cap) {
        atomicAdd(&stats[1], len);
        atomicAdd(&stats[2], 1u);
    }
    if (len > 0) atomicAdd(&stats[4], 1u);
    atomicMax(&stats[3], len);
    // every bucket's first key must not precede the previous key
    if (s > 0 && len > 0 && ordered(out[s - 1], kind) > ordered(out[s], kind)) atomicExch(&stats[0], 1u);
}

}  // namespace learned

void learned_sort(device_context& ctx, const void* keys_in, void* keys_out, int key_kind, std::size_t n,
                  const learned_options& opt, learned_stats* stats_host)
{
    using namespace learned;
    if (key_kind < 0 || key_kind > 2) throw std::invalid_argument("sort_learned: unknown key kind");
    check_size(n);
    if (keys_in == nullptr || keys_out == nullptr) {
        if (n == 0) return;
        throw std::invalid_argument("sort_learned: null keys");
    }
    if (keys_in == keys_out) throw std::invalid_argument("sort_learned: keys_in and keys_out must differ");
    ctx.activate();
    learned_stats st;
    if (n <= 1) {
        if (n == 1)
            check_cuda(cudaMemcpyAsync(keys_out, keys_in, 4, cudaMemcpyDeviceToDevice, ctx.stream), "cudaMemcpyAsync");
        if (stats_host) *stats_host = st;
        return;
    }
    const uint32_t nn = (uint32_t)n;
    const uint32_t S = (uint32_t)std::min<std::size_t>(opt.sample > 0 ? opt.sample : (1u << 20), n);
    const uint32_t M = (uint32_t)std::max<uint32_t>(TRAIN_THREADS, std::min<uint32_t>(opt.points > 0 ? opt.points : 8192, S));
    const uint32_t buckets = (uint32_t)std::max<int>(2, opt.buckets > 0 ? opt.buckets : 32768);
    const int grid_pts = opt.grid > 0 ? opt.grid : 8192;
    const int steps = opt.steps >= 0 ? opt.steps : 64;
    const int G = (int)((M + TRAIN_THREADS - 1) / TRAIN_THREADS);
    const std::size_t part_smem = (std::size_t)buckets * 4 + (std::size_t)(grid_pts + 1) * 4;
    if (part_smem > ctx.smem_optin)
        throw std::invalid_argument("sort_learned: buckets + table do not fit in shared memory");

    // Scratch: sample, points, params (+ Adam), partials, table, counts, offsets.
    const std::size_t rows = (std::size_t)ctx.sm_count;
    temp_buffer sample(ctx.resource, (std::size_t)S * 4);
    temp_buffer pts(ctx.resource, (std::size_t)2 * M * 4);
    temp_buffer prm(ctx.resource, (std::size_t)3 * NPARAM * 4);
    temp_buffer partial(ctx.resource, (std::size_t)G * (NPARAM + 1) * 4);
    temp_buffer table(ctx.resource, (std::size_t)(grid_pts + 1) * 4);
    temp_buffer counts(ctx.resource, rows * buckets * 4);
    temp_buffer boff(ctx.resource, ((std::size_t)buckets + 1) * 4);
    temp_buffer totals(ctx.resource, (std::size_t)buckets * 4);
    temp_buffer misc(ctx.resource, 64 + (std::size_t)std::max(steps, 1) * 4);
    uint32_t* range = misc.as<uint32_t>();          // [0..1]
    uint32_t* ticket = range + 2;                   // [2]
    uint32_t* dstats = range + 4;                   // [4..8]
    float* losses = reinterpret_cast<float*>(misc.as<unsigned char>() + 64);
    check_cuda(cudaMemsetAsync(misc.get(), 0, 64 + (std::size_t)std::max(steps, 1) * 4, ctx.stream), "cudaMemsetAsync");

    const uint32_t* in = static_cast<const uint32_t*>(keys_in);
    uint32_t* out = static_cast<uint32_t*>(keys_out);
    {
        kernel_timer kt(ctx, "learned.sample");
        k_sample<<<(S + 255) / 256, 256, 0, ctx.stream>>>(in, nn, sample.as<uint32_t>(), S, key_kind);
        check_cuda(cudaGetLastError(), "learned sample launch");
    }
    radix_sort(ctx, sample.get(), sample.get(), 4, 0, nullptr, nullptr, S, false);
    float* xs = pts.as<float>();
    float* ys = xs + M;
    k_points<<<(M + 255) / 256, 256, 0, ctx.stream>>>(sample.as<uint32_t>(), S, xs, ys, M, range);
    check_cuda(cudaGetLastError(), "learned points launch");

    float* params = prm.as<float>();
    if (opt.params_in != nullptr) {
        check_cuda(cudaMemcpyAsync(params, opt.params_in, NPARAM * 4, cudaMemcpyHostToDevice, ctx.stream),
                   "cudaMemcpyAsync");
        check_cuda(cudaMemsetAsync(params + NPARAM, 0, 2 * NPARAM * 4, ctx.stream), "cudaMemsetAsync");
    } else {
        k_init_params<<<1, 256, 0, ctx.stream>>>(params, params + NPARAM, params + 2 * NPARAM);
        check_cuda(cudaGetLastError(), "learned init launch");
    }
    const std::size_t train_smem = (std::size_t)(NPARAM + 4 * H * PSTRIDE + 2 * PSTRIDE) * 4;
    static bool smem_set = false;
    if (!smem_set) {
        check_cuda(cudaFuncSetAttribute(k_train_step, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)train_smem),
                   "cudaFuncSetAttribute");
        smem_set = true;
    }
    if (opt.use_model) {
        for (int s = 1; s <= steps; ++s) {
            kernel_timer kt(ctx, "learned.train_step");
            TrainArgs ta{params, params + NPARAM, params + 2 * NPARAM, xs, ys, M, partial.as<float>(), ticket, nullptr,
                         losses, s, opt.lr > 0 ? opt.lr : 0.02f};
            k_train_step<<<G, TRAIN_THREADS, train_smem, ctx.stream>>>(ta);
            check_cuda(cudaGetLastError(), "learned train launch");
        }
        kernel_timer kt(ctx, "learned.table");
        k_table<<<(grid_pts + 1 + 255) / 256, 256, 0, ctx.stream>>>(params, table.as<float>(), grid_pts,
                                                                   opt.model_weight);
    } else {
        k_table_linear<<<(grid_pts + 1 + 255) / 256, 256, 0, ctx.stream>>>(table.as<float>(), grid_pts);
    }
    check_cuda(cudaGetLastError(), "learned table launch");
    if (opt.table_in != nullptr)
        check_cuda(cudaMemcpyAsync(table.get(), opt.table_in, (std::size_t)(grid_pts + 1) * 4, cudaMemcpyHostToDevice,
                                   ctx.stream),
                   "cudaMemcpyAsync");

    PartArgs pa{in, out, nn, key_kind, range, table.as<float>(), grid_pts, buckets, counts.as<uint32_t>(),
                boff.as<uint32_t>()};
    static std::size_t smem_part_set = 0;
    if (smem_part_set < part_smem) {
        check_cuda(cudaFuncSetAttribute(k_count, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)part_smem),
                   "cudaFuncSetAttribute");
        check_cuda(cudaFuncSetAttribute(k_scatter, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)part_smem),
                   "cudaFuncSetAttribute");
        smem_part_set = part_smem;
    }
    {
        kernel_timer kt(ctx, "learned.count");
        k_count<<<(int)rows, PART_THREADS, part_smem, ctx.stream>>>(pa);
        check_cuda(cudaGetLastError(), "learned count launch");
    }
    k_columns<<<(buckets + 255) / 256, 256, 0, ctx.stream>>>(counts.as<uint32_t>(), (uint32_t)rows, buckets,
                                                              totals.as<uint32_t>());
    k_bucket_scan<<<1, 1024, 0, ctx.stream>>>(totals.as<uint32_t>(), buckets, boff.as<uint32_t>());
    check_cuda(cudaGetLastError(), "learned offsets launch");
    {
        kernel_timer kt(ctx, "learned.scatter");
        k_scatter<<<(int)rows, PART_THREADS, part_smem, ctx.stream>>>(pa);
        check_cuda(cudaGetLastError(), "learned scatter launch");
    }
    // Finish every bucket in place (shared-memory sorts; oversized buckets
    // take the batched onesweep path).
    seg_options so;
    segmented_sort(ctx, out, out, 4, key_kind, nullptr, nullptr, n, boff.as<uint32_t>(), buckets, false, so);
    {
        kernel_timer kt(ctx, "learned.check");
        k_check<<<(buckets + 255) / 256, 256, 0, ctx.stream>>>(out, boff.as<uint32_t>(), buckets, key_kind,
                                                                segsort_cta_cap(4, false), dstats);
        check_cuda(cudaGetLastError(), "learned check launch");
    }
    // Read the statistics (and losses); a violation sends the input to the
    // plain radix sort.
    std::vector<uint32_t> hs(5);
    check_cuda(cudaMemcpyAsync(hs.data(), dstats, 5 * 4, cudaMemcpyDeviceToHost, ctx.stream), "cudaMemcpyAsync");
    std::vector<float> hl(std::max(steps, 1));
    if (steps > 0 && opt.use_model)
        check_cuda(cudaMemcpyAsync(hl.data(), losses, steps * 4, cudaMemcpyDeviceToHost, ctx.stream), "cudaMemcpyAsync");
    if (opt.params_out != nullptr)
        check_cuda(cudaMemcpyAsync(opt.params_out, params, NPARAM * 4, cudaMemcpyDeviceToHost, ctx.stream),
                   "cudaMemcpyAsync");
    ctx.finish();
    st.violation = hs[0];
    st.oversized_keys = hs[1];
    st.oversized_buckets = hs[2];
    st.largest_bucket = hs[3];
    st.nonempty_buckets = hs[4];
    st.buckets = buckets;
    st.first_loss = (steps > 0 && opt.use_model) ? hl[0] : 0.f;
    st.last_loss = (steps > 0 && opt.use_model) ? hl[steps - 1] : 0.f;
    if (st.violation) {
        st.fallback = 1;
        radix_sort(ctx, keys_in, keys_out, 4, key_kind, nullptr, nullptr, n, false);
    }
    if (stats_host) *stats_host = st;
}

void mlp_gradients(device_context& ctx, const float* params_host, const float* xs_host, const float* ys_host,
                   std::size_t m, float* grad_host, float* loss_host)
{
    using namespace learned;
    if (m == 0 || m > (1u << 24)) throw std::invalid_argument("mlp_gradients: 0 < m <= 2^24");
    ctx.activate();
    const int G = (int)((m + TRAIN_THREADS - 1) / TRAIN_THREADS);
    temp_buffer prm(ctx.resource, (std::size_t)3 * NPARAM * 4);
    temp_buffer pts(ctx.resource, (std::size_t)2 * m * 4);
    temp_buffer partial(ctx.resource, (std::size_t)G * (NPARAM + 1) * 4);
    temp_buffer misc(ctx.resource, 64 + 2 * NPARAM * 4);
    float* params = prm.as<float>();
    float* xs = pts.as<float>();
    float* ys = xs + m;
    uint32_t* ticket = misc.as<uint32_t>();
    float* loss = reinterpret_cast<float*>(misc.as<unsigned char>() + 16);
    float* grad = reinterpret_cast<float*>(misc.as<unsigned char>() + 64);
    check_cuda(cudaMemsetAsync(misc.get(), 0, 64 + 2 * NPARAM * 4, ctx.stream), "cudaMemsetAsync");
    check_cuda(cudaMemsetAsync(params, 0, 3 * NPARAM * 4, ctx.stream), "cudaMemsetAsync");
    check_cuda(cudaMemcpyAsync(params, params_host, NPARAM * 4, cudaMemcpyHostToDevice, ctx.stream), "cudaMemcpyAsync");
    check_cuda(cudaMemcpyAsync(xs, xs_host, m * 4, cudaMemcpyHostToDevice, ctx.stream), "cudaMemcpyAsync");
    check_cuda(cudaMemcpyAsync(ys, ys_host, m * 4, cudaMemcpyHostToDevice, ctx.stream), "cudaMemcpyAsync");
    const std::size_t train_smem = (std::size_t)(NPARAM + 4 * H * PSTRIDE + 2 * PSTRIDE) * 4;
    check_cuda(cudaFuncSetAttribute(k_train_step, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)train_smem),
               "cudaFuncSetAttribute");
    TrainArgs ta{params, params + NPARAM, params + 2 * NPARAM, xs, ys, (uint32_t)m, partial.as<float>(), ticket, grad,
                 loss, 1, 0.f};
    k_train_step<<<G, TRAIN_THREADS, train_smem, ctx.stream>>>(ta);
    check_cuda(cudaGetLastError(), "mlp gradient launch");
    check_cuda(cudaMemcpyAsync(grad_host, grad, NPARAM * 4, cudaMemcpyDeviceToHost, ctx.stream), "cudaMemcpyAsync");
    check_cuda(cudaMemcpyAsync(loss_host, loss, 4, cudaMemcpyDeviceToHost, ctx.stream), "cudaMemcpyAsync");
    ctx.finish();
}

}  // namespace gbc
