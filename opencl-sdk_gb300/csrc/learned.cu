// Learned-CDF sort: a small monotone MLP fitted on the GPU to a sample of the
// keys models their CDF; the model is compiled into bucket splitters, the keys
// are partitioned into the buckets in one counting pass and one scatter pass,
// the buckets are finished by the segmented sort (shared-memory sorts, with
// oversized buckets routed to its batched onesweep radix sort), and any
// monotonicity violation sends the whole input to the plain radix sort.
//
// No reference counterpart. The output is the plain radix sort's output bit
// for bit (the reference's key order, Algorithm.cpp:459-469): the bucket of a
// key is a monotone function of the key, each bucket is sorted exactly, and
// the boundary check proves the concatenation ordered.
//
// The network, 1 -> H -> H -> 1 on a key u in the order-preserving 32-bit
// domain:
//   d_j  = (float)(u - c_j) * inv_span          (the difference is exact)
//   h1_j = clamp(w1_j * d_j + b1_j, 0, 1)
//   h2_k = clamp(b2_k + sum_j w2_kj * h1_j, 0, 1)
//   F(u) = b3 + sum_k w3_k * h2_k
// with every weight w = exp(v) > 0, so F is non-decreasing in u by
// construction (round-to-nearest float arithmetic is monotone too). The
// centres c_j sit at the sample quantiles (j + 1/2) / H, so the first layer
// resolves clusters far narrower than float precision over the whole key
// range; clamp rather than ReLU keeps F from being convex, so it can follow
// a multi-modal CDF.
//
// Steps (all on the context's stream):
//   1. sample S keys at a fixed stride (order-preserving form) and sort them
//      with the plain radix sort;
//   2. frame (key range, centres), data-driven initial parameters (the ramps
//      of layer 1 span consecutive sample quantiles, layer 2 ~ identity, so
//      the initial F interpolates the sample CDF) and M training points
//      (x = sample quantile i/M, y = (i + 1/2)/M);
//   3. full-batch Adam on the mean squared error, all steps in one
//      cooperative launch: every CTA runs forward and backward for its
//      points, writes its gradient sums, and after one grid barrier every CTA
//      sums all partial gradients in the same order and applies the same
//      update to its own copy of the parameters;
//   4. splitters: s_b = min{u : F(u) >= b / B} by bisection over the key
//      domain, b = 1 .. B-1; a lookup table over the top bits of (u - umin)
//      narrows each key's search to the splitters inside its cell;
//   5. count keys per (CTA chunk, bucket), storing every key's bucket,
//      exclusive offsets, then the keys partitioned in two levels (groups
//      of buckets, then buckets) by the stored buckets;
//   6. segmented sort of the B buckets, except those holding one key value;
//   7. boundary check; fallback if needed.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <type_traits>
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

constexpr int TRAIN_THREADS = 256;          // one training point per thread and round
constexpr int PSTR = (NPARAM + 1 + 3) / 4 * 4;  // a CTA's partial row (gradient sums, loss), 16-byte multiple
constexpr int PSTRIDE = TRAIN_THREADS + 1;  // padded row of per-point activations
constexpr int LUT_BITS = 12;                // splitter lookup table: 2^12 cells
constexpr int NCELLS = 1 << LUT_BITS;
constexpr int PART_THREADS = 1024;
constexpr int PART_ITEMS = 8;               // keys in flight per thread in the partition passes
constexpr uint32_t PART_GROUP = 128;        // buckets per group of the first partition level

__host__ __device__ __forceinline__ bool is_weight(int i)
{
    return i < OFF_B1 || (i >= OFF_V2 && i < OFF_B2) || (i >= OFF_V3 && i < OFF_B3);
}

__device__ __forceinline__ float clamp01(float z) { return fminf(fmaxf(z, 0.f), 1.f); }

// Order-preserving u32 view of a key (floats: sign ? ~k : k | sign).
__device__ __forceinline__ uint32_t ordered(uint32_t k, int kind)
{
    if (kind == 1) return k ^ 0x80000000u;
    if (kind == 2) return (k & 0x80000000u) ? ~k : (k | 0x80000000u);
    return k;
}

// Key range of the sample and the first layer's centres.
struct Frame {
    uint32_t umin, umax;
    float inv_span;
    uint32_t pad;
    uint32_t c[H];
};

__device__ __forceinline__ float feature(uint32_t u, uint32_t c, float inv_span)
{
    return (float)((long long)u - (long long)c) * inv_span;
}

// F(u) with the effective weights w (exp applied) and centres c in shared memory.
__device__ float network(const float* w, const uint32_t* c, float inv_span, uint32_t u)
{
    float h1[H];
#pragma unroll
    for (int j = 0; j < H; ++j) h1[j] = clamp01(fmaf(w[OFF_V1 + j], feature(u, c[j], inv_span), w[OFF_B1 + j]));
    float y = w[OFF_B3];
#pragma unroll 4
    for (int k = 0; k < H; ++k) {
        float z = w[OFF_B2 + k];
#pragma unroll
        for (int j = 0; j < H; ++j) z = fmaf(w[OFF_V2 + k * H + j], h1[j], z);
        y = fmaf(w[OFF_V3 + k], clamp01(z), y);
    }
    return y;
}

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

// ---- 2. frame, initial parameters, training points ---------------------------
__global__ void k_frame(const uint32_t* __restrict__ sorted, uint32_t s, Frame* fr, float* params, int init_params)
{
    const uint32_t umin = sorted[0], umax = sorted[s - 1];
    const float span = (float)max(umax - umin, 1u);
    const int t = threadIdx.x;
    if (t == 0) {
        fr->umin = umin;
        fr->umax = umax;
        fr->inv_span = 1.0f / span;
        fr->pad = 0;
    }
    if (t < H) {
        const uint32_t qa = sorted[min((uint32_t)(((uint64_t)t * s) / H), s - 1)];
        const uint32_t qb = sorted[min((uint32_t)(((uint64_t)(t + 1) * s) / H), s - 1)];
        fr->c[t] = qa + (qb - qa) / 2;
        if (init_params) {
            // ramp from 0 at qa to 1 at qb: w1 = span / width, b1 = 1/2
            params[OFF_V1 + t] = logf(span / (float)max(qb - qa, 1u));
            params[OFF_B1 + t] = 0.5f;
        }
    }
    if (!init_params) return;
    for (int i = t; i < H * H; i += blockDim.x)
        params[OFF_V2 + i] = (i / H == i % H) ? 0.f : logf(1e-3f);  // w2 ~ identity
    if (t < H) {
        params[OFF_B2 + t] = 0.f;
        params[OFF_V3 + t] = logf(1.0f / (float)H);  // output = mean of h2
    }
    if (t == 0) params[OFF_B3] = 0.f;
}

__global__ void k_points(const uint32_t* __restrict__ sorted, uint32_t s, uint32_t* __restrict__ xs,
                         float* __restrict__ ys, uint32_t m)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < m) {
        const uint32_t q = (uint32_t)(((uint64_t)(2 * i + 1) * s) / (2 * (uint64_t)m));
        xs[i] = sorted[min(q, s - 1)];
        ys[i] = ((float)i + 0.5f) / (float)m;
    }
}

// ---- 3. training -------------------------------------------------------------
struct TrainArgs {
    float* params;       // NPARAM raw parameters: read at the start, written by CTA 0 at the end
    const Frame* frame;
    const uint32_t* xs;  // m training keys (order-preserving form)
    const float* ys;
    uint32_t m;
    float* partial;      // [2][gridDim.x][PSTR]: gradient sums and the loss
    uint32_t* barrier;   // zero before the launch
    float* grad_out;     // optional: gradient at the starting parameters
    float* loss_out;     // optional: [steps] loss before each update
    int steps;           // >= 1
    float lr;            // 0: gradients only
    int* err;
};

__global__ void __launch_bounds__(TRAIN_THREADS, 1) k_train(TrainArgs a)
{
    extern __shared__ float sm[];
    float* p = sm;              // this CTA's copy of the raw parameters
    float* am = p + NPARAM;     // Adam first moment
    float* as = am + NPARAM;    // Adam second moment
    float* w = as + NPARAM;     // effective parameters: exp(v) for weights
    float* H1 = w + NPARAM;     // [H][PSTRIDE] per-point activations and deltas
    float* D2 = H1 + H * PSTRIDE;
    float* D1 = D2 + H * PSTRIDE;
    float* P1 = D1 + H * PSTRIDE;  // d1 * feature
    float* H2 = P1 + H * PSTRIDE;
    float* G = H2 + H * PSTRIDE;   // [PSTRIDE] output deltas
    __shared__ uint32_t s_c[H];
    __shared__ float s_red[TRAIN_THREADS / 32];
    __shared__ int s_abort;
    const int tid = threadIdx.x;
    for (int i = tid; i < NPARAM; i += TRAIN_THREADS) {
        p[i] = a.params[i];
        am[i] = 0.f;
        as[i] = 0.f;
    }
    if (tid < H) s_c[tid] = a.frame->c[tid];
    if (tid == 0) s_abort = 0;
    const float inv_span = a.frame->inv_span;
    const uint32_t per_round = gridDim.x * TRAIN_THREADS;
    const uint32_t rounds = (a.m + per_round - 1) / per_round;
    const float inv_m = 1.0f / (float)a.m;
    __syncthreads();

    for (int step = 0; step < a.steps; ++step) {
        for (int i = tid; i < NPARAM; i += TRAIN_THREADS) w[i] = is_weight(i) ? expf(p[i]) : p[i];
        __syncthreads();
        // This CTA's gradient sums with respect to the effective parameters:
        // thread t owns dW2[t / 8][4 (t % 8) .. + 3] and, for t < 5H + 1, one
        // of dw1, db1, db2, dw3 (kinds 0..3) or db3 (t = 5H).
        const int k2 = tid >> 3, j2 = (tid & 7) * 4;
        float acc2[4] = {0.f, 0.f, 0.f, 0.f};
        float acc1 = 0.f, lsum = 0.f;
        for (uint32_t r = 0; r < rounds; ++r) {
            const uint32_t pi = (r * gridDim.x + blockIdx.x) * TRAIN_THREADS + tid;
            const bool valid = pi < a.m;
            const uint32_t u = valid ? a.xs[pi] : s_c[0];
            const float yv = valid ? a.ys[pi] : 0.f;
            float h1[H], h2[H];
            uint32_t on1 = 0, on2 = 0;
#pragma unroll
            for (int j = 0; j < H; ++j) {
                const float z = fmaf(w[OFF_V1 + j], feature(u, s_c[j], inv_span), w[OFF_B1 + j]);
                h1[j] = clamp01(z);
                on1 |= (z > 0.f && z < 1.f ? 1u : 0u) << j;
            }
            float yhat = w[OFF_B3];
#pragma unroll 4
            for (int k = 0; k < H; ++k) {
                float z = w[OFF_B2 + k];
#pragma unroll
                for (int j = 0; j < H; ++j) z = fmaf(w[OFF_V2 + k * H + j], h1[j], z);
                h2[k] = clamp01(z);
                on2 |= (z > 0.f && z < 1.f ? 1u : 0u) << k;
                yhat = fmaf(w[OFF_V3 + k], h2[k], yhat);
            }
            const float e = valid ? yhat - yv : 0.f;
            lsum += e * e;
            const float g = 2.f * e * inv_m;
            float d2[H];
#pragma unroll
            for (int k = 0; k < H; ++k) d2[k] = ((on2 >> k) & 1) ? g * w[OFF_V3 + k] : 0.f;
#pragma unroll
            for (int j = 0; j < H; ++j) {
                float s = 0.f;
#pragma unroll
                for (int k = 0; k < H; ++k) s = fmaf(d2[k], w[OFF_V2 + k * H + j], s);
                const float d1 = ((on1 >> j) & 1) ? s : 0.f;
                D1[j * PSTRIDE + tid] = d1;
                P1[j * PSTRIDE + tid] = d1 * feature(u, s_c[j], inv_span);
                H1[j * PSTRIDE + tid] = h1[j];
                D2[j * PSTRIDE + tid] = d2[j];
                H2[j * PSTRIDE + tid] = h2[j];
            }
            G[tid] = g;
            __syncthreads();
#pragma unroll 8
            for (int q = 0; q < TRAIN_THREADS; ++q) {
                const float d = D2[k2 * PSTRIDE + q];
#pragma unroll
                for (int i = 0; i < 4; ++i) acc2[i] = fmaf(d, H1[(j2 + i) * PSTRIDE + q], acc2[i]);
            }
            if (tid < 5 * H + 1) {
                // one loop per kind (the kind is fixed per thread): the same
                // sums in the same order, with the loads pipelined
                const int kind = tid / H, u1 = tid % H;
                if (kind == 3) {
                    const float* h2 = H2 + u1 * PSTRIDE;
#pragma unroll 8
                    for (int q = 0; q < TRAIN_THREADS; ++q) acc1 = fmaf(G[q], h2[q], acc1);
                } else {
                    const float* row = kind == 0 ? P1 + u1 * PSTRIDE
                                     : kind == 1 ? D1 + u1 * PSTRIDE
                                     : kind == 2 ? D2 + u1 * PSTRIDE
                                                 : G;
#pragma unroll 8
                    for (int q = 0; q < TRAIN_THREADS; ++q) acc1 += row[q];
                }
            }
            __syncthreads();  // the buffers are rewritten by the next round
        }
        float* out = a.partial + ((size_t)(step & 1) * gridDim.x + blockIdx.x) * PSTR;
#pragma unroll
        for (int i = 0; i < 4; ++i) out[OFF_V2 + k2 * H + j2 + i] = acc2[i];
        if (tid < 5 * H + 1) {
            const int kind = tid / H, u1 = tid % H;
            if (kind == 0) out[OFF_V1 + u1] = acc1;
            else if (kind == 1) out[OFF_B1 + u1] = acc1;
            else if (kind == 2) out[OFF_B2 + u1] = acc1;
            else if (kind == 3) out[OFF_V3 + u1] = acc1;
            else out[OFF_B3] = acc1;
        }
        lsum = dev::warp_reduce(lsum, [](float x, float y) { return x + y; });
        if ((tid & 31) == 0) s_red[tid >> 5] = lsum;
        __syncthreads();
        if (tid == 0) {
            float l = 0.f;
            for (int i = 0; i < TRAIN_THREADS / 32; ++i) l += s_red[i];
            out[NPARAM] = l;
        }
        // Grid barrier (the launch is cooperative, so every CTA is resident);
        // the partial buffers alternate between steps, so one barrier a step
        // suffices. The wait is bounded.
        __threadfence();
        __syncthreads();
        if (tid == 0) {
            atomicAdd(a.barrier, 1u);
            const uint32_t target = (uint32_t)(step + 1) * gridDim.x;
            const unsigned long long t0 = dev::globaltimer();
            uint32_t spin = 0;
            while (dev::ld_acquire(a.barrier) < target) {
                if ((++spin & 63) == 0 && dev::globaltimer() - t0 > dev::SPIN_LIMIT_NS) {
                    dev::raise_error(a.err, dev::ERR_LOOKBACK_TIMEOUT);
                    s_abort = 1;
                    break;
                }
            }
            __threadfence();
        }
        __syncthreads();
        if (s_abort) return;
        // Every CTA sums the partials in CTA order and applies the same update.
        const float b1c = 1.f - powf(0.9f, (float)(step + 1)), b2c = 1.f - powf(0.999f, (float)(step + 1));
        const float4* base = reinterpret_cast<const float4*>(a.partial + (size_t)(step & 1) * gridDim.x * PSTR);
        for (int c4 = tid; c4 < PSTR / 4; c4 += TRAIN_THREADS) {
            // four sums per thread, 16 partial vectors in flight per round
            // trip to L2; each sum taken in CTA order
            const float4* col = base + c4;
            float4 sum = make_float4(0.f, 0.f, 0.f, 0.f);
            uint32_t c = 0;
            for (; c + 16 <= gridDim.x; c += 16) {
                float4 v[16];
#pragma unroll
                for (int q = 0; q < 16; ++q) v[q] = __ldcg(col + (size_t)(c + q) * (PSTR / 4));
#pragma unroll
                for (int q = 0; q < 16; ++q) {
                    sum.x += v[q].x;
                    sum.y += v[q].y;
                    sum.z += v[q].z;
                    sum.w += v[q].w;
                }
            }
            for (; c < gridDim.x; ++c) {
                const float4 v = __ldcg(col + (size_t)c * (PSTR / 4));
                sum.x += v.x;
                sum.y += v.y;
                sum.z += v.z;
                sum.w += v.w;
            }
            const float sums[4] = {sum.x, sum.y, sum.z, sum.w};
#pragma unroll
            for (int e = 0; e < 4; ++e) {
                const int i = 4 * c4 + e;
                if (i > NPARAM) break;
                if (i == NPARAM) {
                    if (blockIdx.x == 0 && a.loss_out != nullptr) a.loss_out[step] = sums[e] * inv_m;
                    break;
                }
                const float grad = is_weight(i) ? sums[e] * w[i] : sums[e];  // d exp(v) / dv = exp(v)
                if (step == 0 && blockIdx.x == 0 && a.grad_out != nullptr) a.grad_out[i] = grad;
                if (a.lr > 0.f) {
                    const float m1 = 0.9f * am[i] + 0.1f * grad;
                    const float s1 = 0.999f * as[i] + 0.001f * grad * grad;
                    am[i] = m1;
                    as[i] = s1;
                    p[i] -= a.lr * (m1 / b1c) / (sqrtf(s1 / b2c) + 1e-8f);
                }
            }
        }
        __syncthreads();
    }
    if (blockIdx.x == 0)
        for (int i = tid; i < NPARAM; i += TRAIN_THREADS) a.params[i] = p[i];
}

// ---- 4. splitters and their lookup table -----------------------------------
// sp[b - 1] = min{u in [umin, umax + 1] : F(u) >= b / B}, saturated to 2^32-1;
// without the model, equal-width buckets over [umin, umax].
__global__ void k_splitters(const float* __restrict__ params, const Frame* __restrict__ fr, uint32_t buckets,
                            uint32_t* __restrict__ sp, int use_model)
{
    __shared__ float w[NPARAM];
    __shared__ uint32_t c[H];
    for (int i = threadIdx.x; i < NPARAM; i += blockDim.x) w[i] = is_weight(i) ? expf(params[i]) : params[i];
    if (threadIdx.x < H) c[threadIdx.x] = fr->c[threadIdx.x];
    __syncthreads();
    const uint32_t b = blockIdx.x * blockDim.x + threadIdx.x + 1;
    if (b >= buckets) return;
    const uint32_t umin = fr->umin, umax = fr->umax;
    uint64_t lo = umin, hi = (uint64_t)umax + 1;
    if (!use_model) {
        lo = umin + ((uint64_t)b * ((uint64_t)(umax - umin) + 1)) / buckets;
    } else {
        const float target = (float)b / (float)buckets;
        const float inv_span = fr->inv_span;
        while (lo < hi) {
            const uint64_t mid = (lo + hi) >> 1;
            if (network(w, c, inv_span, (uint32_t)mid) >= target) hi = mid;
            else lo = mid + 1;
        }
    }
    sp[b - 1] = (uint32_t)min(lo, (uint64_t)0xFFFFFFFFu);
}

__device__ __forceinline__ int lut_shift(uint32_t umin, uint32_t umax)
{
    const uint32_t span = umax - umin;
    const int bits = span == 0 ? 0 : 32 - __clz(span);
    return max(0, bits - LUT_BITS);
}

// lut[c] = number of splitters <= the first key of cell c; lut[NCELLS] = B - 1.
__global__ void k_lut(const uint32_t* __restrict__ sp, uint32_t buckets, const Frame* __restrict__ fr,
                      uint16_t* __restrict__ lut)
{
    const uint32_t c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c > (uint32_t)NCELLS) return;
    if (c == (uint32_t)NCELLS) {
        lut[c] = (uint16_t)(buckets - 1);
        return;
    }
    const uint64_t start = (uint64_t)fr->umin + ((uint64_t)c << lut_shift(fr->umin, fr->umax));
    uint32_t lo = 0, hi = buckets - 1;
    if (start > 0xFFFFFFFFull) {
        lo = hi;
    } else {
        while (lo < hi) {
            const uint32_t m = (lo + hi) >> 1;
            if (sp[m] <= (uint32_t)start) lo = m + 1;
            else hi = m;
        }
    }
    lut[c] = (uint16_t)lo;
}

// ---- 4b. second model level: oversized root buckets split at sample quantiles
// The root model's bm - 1 splitters spm partition the sorted sample. A root
// bucket whose expected size (its sample count scaled to n) exceeds cap and
// whose sample keys are not all equal asks for ceil(size / target) - 1 more
// splitters, placed at equally spaced positions of its own sample keys: a
// piecewise model of the bucket's CDF, the leaf level of a recursive model
// index whose root is the network. At most buckets - bm are added (scaled
// down in proportion when more are asked); the final buckets - 1 splitters
// are non-decreasing, the unused tail set to 2^32 - 1 (empty buckets).

// want[b] = splitters root bucket b asks for; lo[b] = its first sample index.
__global__ void k_refine_want(const uint32_t* __restrict__ sorted, uint32_t s, const uint32_t* __restrict__ spm,
                              uint32_t bm, uint32_t n, uint32_t cap, uint32_t target, uint32_t* __restrict__ lo_out,
                              uint32_t* __restrict__ want)
{
    const uint32_t b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= bm) return;
    auto lower = [&](uint32_t v) {
        uint32_t lo = 0, hi = s;
        while (lo < hi) {
            const uint32_t m = (lo + hi) >> 1;
            if (sorted[m] < v) lo = m + 1;
            else hi = m;
        }
        return lo;
    };
    const uint32_t lo = b == 0 ? 0u : lower(spm[b - 1]);
    const uint32_t hi = b + 1 == bm ? s : lower(spm[b]);
    uint32_t r = 0;
    if (hi > lo + 1 && sorted[lo] != sorted[hi - 1]) {
        const uint64_t size = (uint64_t)(hi - lo) * n / s;
        if (size > cap) {
            const uint64_t ask = (size + target - 1) / target - 1;
            r = (uint32_t)(ask < (uint64_t)(hi - lo - 1) ? ask : (uint64_t)(hi - lo - 1));
        }
    }
    lo_out[b] = lo;
    want[b] = r;
}

constexpr int REFINE_THREADS = 1024;

// One CTA: the granted count of every root bucket (want scaled to the budget)
// replaced in place by its exclusive prefix; *added = the total granted.
__global__ void __launch_bounds__(REFINE_THREADS) k_refine_plan(uint32_t* __restrict__ want, uint32_t bm,
                                                                uint32_t budget, uint32_t* __restrict__ added)
{
    __shared__ uint32_t s_part[REFINE_THREADS];
    __shared__ unsigned long long s_total;
    const uint32_t per = (bm + REFINE_THREADS - 1) / REFINE_THREADS;
    const uint32_t b0 = min(bm, threadIdx.x * per), b1 = min(bm, b0 + per);
    if (threadIdx.x == 0) s_total = 0;
    __syncthreads();
    unsigned long long mine = 0;
    for (uint32_t b = b0; b < b1; ++b) mine += want[b];
    atomicAdd(&s_total, mine);
    __syncthreads();
    const unsigned long long total = s_total;
    auto grant = [&](uint32_t w) -> uint32_t {
        return total <= budget ? w : (uint32_t)(((unsigned long long)w * budget) / total);
    };
    uint32_t sum = 0;
    for (uint32_t b = b0; b < b1; ++b) sum += grant(want[b]);
    // exclusive scan of the per-thread sums (Hillis-Steele over 1024 words)
    s_part[threadIdx.x] = sum;
    __syncthreads();
    for (int d = 1; d < REFINE_THREADS; d <<= 1) {
        const uint32_t v = threadIdx.x >= (uint32_t)d ? s_part[threadIdx.x - d] : 0u;
        __syncthreads();
        s_part[threadIdx.x] += v;
        __syncthreads();
    }
    uint32_t run = s_part[threadIdx.x] - sum;
    for (uint32_t b = b0; b < b1; ++b) {
        const uint32_t g = grant(want[b]);
        want[b] = run;
        run += g;
    }
    if (threadIdx.x == REFINE_THREADS - 1) *added = s_part[REFINE_THREADS - 1];
}

// The final splitters, one thread per output position i. Root bucket b's
// group (its granted splitters, then spm[b] unless b is the last) starts at
// position b + off[b]; a thread finds its group by binary search, so a root
// bucket granted thousands of splitters does not leave them to one thread.
// Positions past the last group are 2^32 - 1 (empty buckets).
__global__ void k_refine_write(const uint32_t* __restrict__ sorted, uint32_t s, const uint32_t* __restrict__ spm,
                               uint32_t bm, uint32_t buckets, const uint32_t* __restrict__ lo_in,
                               const uint32_t* __restrict__ off, const uint32_t* __restrict__ added,
                               uint32_t* __restrict__ sp)
{
    const uint32_t total = *added;
    const uint32_t used = bm - 1 + total;  // positions the groups fill
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i + 1 < buckets; i += stride) {
        if (i >= used) {
            sp[i] = 0xFFFFFFFFu;
            continue;
        }
        // the last root bucket whose group starts at or before i (group 0 starts at 0)
        uint32_t lo_b = 1, hi_b = bm;
        while (lo_b < hi_b) {
            const uint32_t m = (lo_b + hi_b) >> 1;
            if (m + off[m] <= i) lo_b = m + 1;
            else hi_b = m;
        }
        const uint32_t b = lo_b - 1;
        const uint32_t j = i - (b + off[b]);
        const uint32_t r = (b + 1 < bm ? off[b + 1] : total) - off[b];
        if (j < r) {
            const uint32_t l = lo_in[b], h = b + 1 < bm ? lo_in[b + 1] : s;
            sp[i] = sorted[l + (uint32_t)(((uint64_t)(j + 1) * (h - l)) / (r + 1))];
        } else {
            sp[i] = spm[b];  // j == r: the root splitter closing group b (b + 1 < bm)
        }
    }
}

// ---- 5. partition ----------------------------------------------------------
struct PartArgs {
    const uint32_t* keys;
    uint32_t n;
    int kind;
    const Frame* frame;
    const uint32_t* sp;     // buckets - 1 splitters
    const uint16_t* lut;    // NCELLS + 1 entries
    uint32_t buckets;
    uint32_t* counts;       // [gridDim.x][buckets]: per-CTA counts
    uint16_t* ids;          // [n]: every key's bucket, written by the counting pass
};

// Bucket of a key: the number of splitters <= u, searched among the splitters
// of u's lookup cell only.
struct Bucketer {
    const uint32_t* sp;
    const uint16_t* lut;
    uint32_t umin;
    int shift;
    __device__ __forceinline__ uint32_t operator()(uint32_t u) const
    {
        if (u < umin) return 0;
        const uint32_t c = min((u - umin) >> shift, (uint32_t)NCELLS - 1);
        uint32_t lo = lut[c], hi = lut[c + 1];
        while (lo < hi) {
            const uint32_t m = (lo + hi) >> 1;
            if (sp[m] <= u) lo = m + 1;
            else hi = m;
        }
        return lo;
    }
};

__host__ __device__ constexpr std::size_t part_smem_bytes(uint32_t buckets)
{
    return (std::size_t)buckets * 4 + (std::size_t)(buckets - 1) * 4 + (std::size_t)(NCELLS + 1) * 2;
}

// k_partition_buckets with T threads: 2 x (2T) words (the staged bucket
// range), the staged chunk's keys and buckets.
__host__ __device__ constexpr std::size_t bucket_smem_bytes(int T)
{
    return ((std::size_t)2 * (2 * T) + (std::size_t)PART_ITEMS * T) * 4 + (std::size_t)PART_ITEMS * T * 2;
}

// k_partition_groups with T threads: 2 x groups words, the staged chunk's
// keys and buckets.
__host__ __device__ constexpr std::size_t group_smem_bytes(uint32_t buckets, int T)
{
    return ((std::size_t)2 * ((buckets + PART_GROUP - 1) / PART_GROUP) + (std::size_t)PART_ITEMS * T) * 4 +
           (std::size_t)PART_ITEMS * T * 2;
}

// Loads the splitters and the table into shared memory after a buckets-word
// array (the counts); returns the bucketer.
__device__ __forceinline__ Bucketer load_bucketer(const PartArgs& a, uint32_t* sh)
{
    uint32_t* sp = sh + a.buckets;
    uint16_t* lut = reinterpret_cast<uint16_t*>(sp + (a.buckets - 1));
    for (uint32_t i = threadIdx.x; i + 1 < a.buckets; i += PART_THREADS) sp[i] = a.sp[i];
    for (int i = threadIdx.x; i <= NCELLS; i += PART_THREADS) lut[i] = a.lut[i];
    const uint32_t umin = a.frame->umin, umax = a.frame->umax;
    return Bucketer{sp, lut, umin, lut_shift(umin, umax)};
}

__global__ void __launch_bounds__(PART_THREADS, 1) k_count(PartArgs a)
{
    extern __shared__ uint32_t sh[];
    uint32_t* hist = sh;  // buckets
    for (uint32_t i = threadIdx.x; i < a.buckets; i += PART_THREADS) hist[i] = 0;
    const Bucketer bk = load_bucketer(a, sh);
    __syncthreads();
    const uint32_t chunk = (a.n + gridDim.x - 1) / gridDim.x;
    const uint32_t b0 = min(a.n, blockIdx.x * chunk), b1 = min(a.n, b0 + chunk);
    uint32_t i = b0 + threadIdx.x;
    for (; i + (PART_ITEMS - 1) * PART_THREADS < b1; i += PART_ITEMS * PART_THREADS) {
        uint32_t k[PART_ITEMS];
#pragma unroll
        for (int j = 0; j < PART_ITEMS; ++j) k[j] = a.keys[i + j * PART_THREADS];
#pragma unroll
        for (int j = 0; j < PART_ITEMS; ++j) {
            const uint32_t b = bk(ordered(k[j], a.kind));
            atomicAdd(&hist[b], 1u);
            a.ids[i + j * PART_THREADS] = (uint16_t)b;
        }
    }
    for (; i < b1; i += PART_THREADS) {
        const uint32_t b = bk(ordered(a.keys[i], a.kind));
        atomicAdd(&hist[b], 1u);
        a.ids[i] = (uint16_t)b;
    }
    __syncthreads();
    uint32_t* row = a.counts + (size_t)blockIdx.x * a.buckets;
    for (uint32_t i = threadIdx.x; i < a.buckets; i += PART_THREADS) row[i] = hist[i];
}

// Bucket totals: the column sums of the per-CTA counts; one thread per bucket.
__global__ void k_columns(const uint32_t* __restrict__ counts, uint32_t rows, uint32_t buckets,
                          uint32_t* __restrict__ totals)
{
    const uint32_t b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= buckets) return;
    uint32_t run = 0;
    for (uint32_t r = 0; r < rows; ++r) run += counts[(size_t)r * buckets + b];
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

// Start of every bucket group (GROUP consecutive buckets) and of every
// bucket: the write cursors of the two partition levels.
__global__ void k_cursors(const uint32_t* __restrict__ bucket_off, uint32_t buckets, uint32_t* __restrict__ group_cur,
                          uint32_t* __restrict__ bucket_cur)
{
    const uint32_t b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= buckets) return;
    bucket_cur[b] = bucket_off[b];
    if (b % PART_GROUP == 0) group_cur[b / PART_GROUP] = bucket_off[b];
}

// Second partition level, keys only (the order inside a bucket is free):
// src holds the keys grouped by bucket group, so a chunk of PART_ITEMS x T
// keys (T threads per CTA) spans a narrow bucket range [L, R]. Per chunk: ranks
// within each bucket by shared atomics over that range, the chunk staged in
// shared memory in bucket order, one global reservation per bucket present,
// then written out run by run with consecutive threads on consecutive
// addresses. A chunk wider than 2T buckets (groups much smaller than a
// chunk) takes one global cursor increment per key instead. The buckets come
// with the keys (src_ids), so there is no search. Shared memory: 2 x 2T
// words, the staged keys and their buckets relative to L (u16).
template <int T>
__global__ void __launch_bounds__(T, 1024 / T) k_partition_buckets(PartArgs a, const uint32_t* __restrict__ src,
                                                                const uint16_t* __restrict__ src_ids,
                                                                uint32_t* __restrict__ dst,
                                                                uint32_t* __restrict__ cursor)
{
    extern __shared__ uint32_t sh[];
    constexpr uint32_t PER = PART_ITEMS * T;
    constexpr uint32_t NONE = 0xFFFFFFFFu;
    constexpr uint32_t PART_RANGE = 2 * T;  // two range entries per thread
    uint32_t* hist = sh;                                       // [PART_RANGE]: counts, then chunk offsets
    uint32_t* delta = hist + PART_RANGE;                       // [PART_RANGE]: global start - chunk offset
    uint32_t* stage = delta + PART_RANGE;                      // [PER]
    uint16_t* sbkt = reinterpret_cast<uint16_t*>(stage + PER); // [PER]
    __shared__ uint32_t s_warp[T / 32], s_lo, s_hi;
    const uint32_t tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    if (tid == 0) {
        s_lo = NONE;
        s_hi = 0;
    }
    const uint32_t chunks = (a.n + PER - 1) / PER;
    for (uint32_t c = blockIdx.x; c < chunks; c += gridDim.x) {
        const uint32_t first = c * PER;
        const uint32_t count = min(PER, a.n - first);
        uint32_t k[PART_ITEMS], b[PART_ITEMS], r[PART_ITEMS];
#pragma unroll
        for (int j = 0; j < PART_ITEMS; ++j) {
            const uint32_t i = j * T + tid;
            k[j] = i < count ? src[first + i] : 0u;
            b[j] = i < count ? (uint32_t)src_ids[first + i] : NONE;
        }
        __syncthreads();  // the previous chunk is done (and s_lo/s_hi are reset)
        uint32_t lo = NONE, hi = 0;
#pragma unroll
        for (int j = 0; j < PART_ITEMS; ++j) {
            if (b[j] != NONE) {
                lo = min(lo, b[j]);
                hi = max(hi, b[j]);
            }
        }
        lo = __reduce_min_sync(0xffffffffu, lo);
        hi = __reduce_max_sync(0xffffffffu, hi);
        if (lane == 0 && lo != NONE) {
            atomicMin(&s_lo, lo);
            atomicMax(&s_hi, hi);
        }
        __syncthreads();
        const uint32_t L = s_lo, span = s_hi - s_lo + 1;  // every chunk holds at least one key
        const bool wide = span > PART_RANGE;
        if (!wide)
            for (uint32_t e = tid; e < span; e += T) hist[e] = 0;
        __syncthreads();
        if (tid == 0) {  // for the next chunk: every thread has read L and span
            s_lo = NONE;
            s_hi = 0;
        }
        if (wide) {
#pragma unroll
            for (int j = 0; j < PART_ITEMS; ++j)
                if (b[j] != NONE) {
                    const uint32_t pos = atomicAdd(&cursor[b[j]], 1u);
                    if (pos < a.n) dst[pos] = k[j];
                }
            continue;
        }
#pragma unroll
        for (int j = 0; j < PART_ITEMS; ++j) r[j] = b[j] != NONE ? atomicAdd(&hist[b[j] - L], 1u) : 0u;
        __syncthreads();
        // chunk offsets (exclusive scan over the range, two entries per thread) and reservations
        const uint32_t e0 = 2 * tid, e1 = e0 + 1;
        const uint32_t v0 = e0 < span ? hist[e0] : 0u, v1 = e1 < span ? hist[e1] : 0u;
        const uint32_t incl = dev::warp_inclusive_scan(v0 + v1, [](uint32_t p, uint32_t q) { return p + q; });
        if (lane == 31) s_warp[warp] = incl;
        __syncthreads();
        uint32_t before = 0;
        for (uint32_t w = 0; w < warp; ++w) before += s_warp[w];
        const uint32_t off0 = before + incl - v0 - v1, off1 = off0 + v0;
        if (e0 < span) {
            const uint32_t start = v0 != 0 ? atomicAdd(&cursor[L + e0], v0) : 0u;
            hist[e0] = off0;
            delta[e0] = start - off0;
        }
        if (e1 < span) {
            const uint32_t start = v1 != 0 ? atomicAdd(&cursor[L + e1], v1) : 0u;
            hist[e1] = off1;
            delta[e1] = start - off1;
        }
        __syncthreads();
#pragma unroll
        for (int j = 0; j < PART_ITEMS; ++j)
            if (b[j] != NONE) {
                const uint32_t slot = hist[b[j] - L] + r[j];
                stage[slot] = k[j];
                sbkt[slot] = (uint16_t)(b[j] - L);
            }
        __syncthreads();
        for (uint32_t i = tid; i < count; i += T) {
            const uint32_t pos = delta[sbkt[i]] + i;
            if (pos < a.n) dst[pos] = stage[i];
        }
    }
}

// First partition level, keys only: every key, with its bucket, to its
// bucket group (bucket / PART_GROUP; the buckets are those the counting pass
// stored, so the group regions hold exactly their counted keys). Per chunk
// of PART_ITEMS x T keys (T threads per CTA, T >= groups): ranks within each group by shared
// atomics, the chunk staged in shared memory in group order, one global
// reservation per group present, then written out run by run with
// consecutive threads on consecutive addresses. Shared memory: 2 x groups
// words, the staged keys and their buckets (u16).
template <int T>
__global__ void __launch_bounds__(T, 1024 / T) k_partition_groups(PartArgs a, uint32_t groups,
                                                               uint32_t* __restrict__ dst,
                                                               uint16_t* __restrict__ dst_ids,
                                                               uint32_t* __restrict__ cursor)
{
    extern __shared__ uint32_t sh[];
    constexpr uint32_t PER = PART_ITEMS * T;
    constexpr uint32_t NONE = 0xFFFFFFFFu;
    uint32_t* hist = sh;                                       // [groups]: counts, then chunk offsets
    uint32_t* delta = hist + groups;                           // [groups]: global start - chunk offset
    uint32_t* stage = delta + groups;                          // [PER]
    uint16_t* sbkt = reinterpret_cast<uint16_t*>(stage + PER); // [PER]
    __shared__ uint32_t s_warp[T / 32];
    const uint32_t tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const uint32_t chunks = (a.n + PER - 1) / PER;
    for (uint32_t c = blockIdx.x; c < chunks; c += gridDim.x) {
        const uint32_t first = c * PER;
        const uint32_t count = min(PER, a.n - first);
        uint32_t k[PART_ITEMS], bb[PART_ITEMS], g[PART_ITEMS], r[PART_ITEMS];
#pragma unroll
        for (int j = 0; j < PART_ITEMS; ++j) {
            const uint32_t i = j * T + tid;
            k[j] = i < count ? a.keys[first + i] : 0u;
            bb[j] = i < count ? (uint32_t)a.ids[first + i] : 0u;
        }
        __syncthreads();  // the previous chunk's write-out is done
#pragma unroll
        for (int j = 0; j < PART_ITEMS; ++j) g[j] = j * T + tid < count ? bb[j] / PART_GROUP : NONE;
        for (uint32_t i = tid; i < groups; i += T) hist[i] = 0;
        __syncthreads();
#pragma unroll
        for (int j = 0; j < PART_ITEMS; ++j) r[j] = g[j] != NONE ? atomicAdd(&hist[g[j]], 1u) : 0u;
        __syncthreads();
        // chunk offsets (exclusive scan over groups <= T) and reservations
        const uint32_t v = tid < groups ? hist[tid] : 0u;
        const uint32_t incl = dev::warp_inclusive_scan(v, [](uint32_t p, uint32_t q) { return p + q; });
        if (lane == 31) s_warp[warp] = incl;
        __syncthreads();
        if (tid < groups) {
            uint32_t before = 0;
            for (uint32_t w = 0; w < warp; ++w) before += s_warp[w];
            const uint32_t off = before + incl - v;
            const uint32_t start = v != 0 ? atomicAdd(&cursor[tid], v) : 0u;
            hist[tid] = off;
            delta[tid] = start - off;
        }
        __syncthreads();
#pragma unroll
        for (int j = 0; j < PART_ITEMS; ++j)
            if (g[j] != NONE) {
                const uint32_t slot = hist[g[j]] + r[j];
                stage[slot] = k[j];
                sbkt[slot] = (uint16_t)bb[j];
            }
        __syncthreads();
        for (uint32_t i = tid; i < count; i += T) {
            const uint32_t b = sbkt[i];
            const uint32_t pos = delta[b / PART_GROUP] + i;
            if (pos < a.n) {
                dst[pos] = stage[i];
                dst_ids[pos] = (uint16_t)b;
            }
        }
    }
}

// skip[b] = 1 when bucket b holds at most one distinct key (already in
// order, so the segmented sort leaves it alone); one CTA per bucket, leaving
// at the first key that differs from the bucket's first.
__global__ void __launch_bounds__(256) k_constant_buckets(const uint32_t* __restrict__ out,
                                                          const uint32_t* __restrict__ bucket_off,
                                                          uint8_t* __restrict__ skip)
{
    const uint32_t b = blockIdx.x;
    const uint32_t s = bucket_off[b], e = bucket_off[b + 1];
    if (e - s >= 2) {
        const uint32_t first = out[s];
        for (uint32_t base = s + 1; base < e; base += 256 * 8) {
            bool diff = false;
#pragma unroll
            for (int j = 0; j < 8; ++j) {
                const uint32_t i = base + j * 256 + threadIdx.x;
                if (i < e && out[i] != first) diff = true;
            }
            if (__syncthreads_or(diff)) {
                if (threadIdx.x == 0) skip[b] = 0;
                return;
            }
        }
    }
    if (threadIdx.x == 0) skip[b] = 1;
}

// ---- 6/7. statistics and the boundary check ----------------------------------
// stats: [0] violation flag, [1] keys in oversized buckets, [2] oversized
// buckets, [3] largest bucket, [4] non-empty buckets, [5] keys in oversized
// buckets that hold one key value.
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
        if (out[s] == out[e - 1]) atomicAdd(&stats[5], len);
    }
    if (len > 0) atomicAdd(&stats[4], 1u);
    atomicMax(&stats[3], len);
    // every bucket's first key must not precede the previous key
    if (s > 0 && len > 0 && ordered(out[s - 1], kind) > ordered(out[s], kind)) atomicExch(&stats[0], 1u);
}

// Expected bucket sizes from the sorted sample (S keys): the sample keys of
// bucket b are those in [sp[b-1], sp[b]). est[0] receives the sample keys in
// buckets whose size scaled to n would exceed cap.
__global__ void k_estimate(const uint32_t* __restrict__ sorted, uint32_t s, const uint32_t* __restrict__ sp,
                           uint32_t buckets, uint32_t n, uint32_t cap, int skip_constant, uint32_t* est)
{
    const uint32_t b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= buckets) return;
    auto lower = [&](uint32_t v) {
        uint32_t lo = 0, hi = s;
        while (lo < hi) {
            const uint32_t m = (lo + hi) >> 1;
            if (sorted[m] < v) lo = m + 1;
            else hi = m;
        }
        return lo;
    };
    const uint32_t lo = b == 0 ? 0u : lower(sp[b - 1]);
    const uint32_t hi = b + 1 == buckets ? s : lower(sp[b]);
    const uint32_t cnt = hi > lo ? hi - lo : 0u;
    // skip_constant: a bucket whose sample keys are all equal needs no sort
    if (skip_constant && cnt > 0 && sorted[lo] == sorted[hi - 1]) return;
    if ((uint64_t)cnt * n > (uint64_t)cap * s) atomicAdd(est, cnt);
}

// ---- key-value form: 64-bit keys through a monotone 32-bit projection --------
// The sample of 64-bit keys (order-preserving form) is sorted; keys are
// projected to 32 bits as p(u) = min(2^32 - 1, (u - kmin) >> shift) (0 below
// kmin), shift chosen so that the sample's range [kmin, kmax] fits: p is
// non-decreasing, so buckets over p are buckets over the keys. 32-bit keys
// use p(u) = u.
struct Proj {
    unsigned long long kmin;
    int shift;
    int pad;
};

__device__ __forceinline__ uint64_t ordered64(uint64_t k, int kind)
{
    return kind == 1 ? k ^ 0x8000000000000000ull : k;
}
template <typename K> __device__ __forceinline__ uint64_t ordered_any(K k, int kind)
{
    if constexpr (sizeof(K) == 8) return ordered64(k, kind);
    else return ordered(k, kind);
}
__device__ __forceinline__ uint32_t project(uint64_t u, const Proj& p)
{
    if (u <= p.kmin) return 0;
    const uint64_t d = (u - p.kmin) >> p.shift;
    return d > 0xFFFFFFFFull ? 0xFFFFFFFFu : (uint32_t)d;
}

__global__ void k_sample64(const uint64_t* __restrict__ keys, uint32_t n, uint64_t* __restrict__ sample, uint32_t s,
                           int kind)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < s) sample[i] = ordered64(keys[(uint32_t)(((uint64_t)i * n) / s)], kind);
}

// One CTA: the projection from the sorted 64-bit sample, and the sample
// projected (still sorted).
__global__ void k_project(const uint64_t* __restrict__ sorted, uint32_t s, Proj* __restrict__ pj,
                          uint32_t* __restrict__ sorted32)
{
    __shared__ Proj p;
    if (threadIdx.x == 0) {
        const uint64_t kmin = sorted[0], span = sorted[s - 1] - kmin;
        const int bits = span == 0 ? 0 : 64 - __clzll((long long)span);
        p.kmin = kmin;
        p.shift = bits > 32 ? bits - 32 : 0;
        p.pad = 0;
        *pj = p;
    }
    __syncthreads();
    for (uint32_t i = threadIdx.x; i < s; i += blockDim.x) sorted32[i] = project(sorted[i], p);
}

// Bucket of every key (and its index), for the stable partition.
template <typename K>
__global__ void __launch_bounds__(PART_THREADS) k_bucket_ids(const K* __restrict__ keys, uint32_t n, int kind,
                                                             const Proj* __restrict__ pj,
                                                             const Frame* __restrict__ fr,
                                                             const uint32_t* __restrict__ gsp,
                                                             const uint16_t* __restrict__ glut, uint32_t buckets,
                                                             uint32_t* __restrict__ ids, uint32_t* __restrict__ idx)
{
    extern __shared__ uint32_t sh[];
    uint32_t* sp = sh;
    uint16_t* lut = reinterpret_cast<uint16_t*>(sp + (buckets - 1));
    for (uint32_t i = threadIdx.x; i + 1 < buckets; i += PART_THREADS) sp[i] = gsp[i];
    for (int i = threadIdx.x; i <= NCELLS; i += PART_THREADS) lut[i] = glut[i];
    const Proj p = *pj;
    const Bucketer bk{sp, lut, fr->umin, lut_shift(fr->umin, fr->umax)};
    __syncthreads();
    const uint32_t stride = gridDim.x * PART_THREADS;
    uint32_t i = blockIdx.x * PART_THREADS + threadIdx.x;
    for (; i + 3 * stride < n; i += 4 * stride) {
        K k[4];
#pragma unroll
        for (int j = 0; j < 4; ++j) k[j] = keys[i + j * stride];
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            ids[i + j * stride] = bk(project(ordered_any<K>(k[j], kind), p));
            idx[i + j * stride] = i + j * stride;
        }
    }
    for (; i < n; i += stride) {
        ids[i] = bk(project(ordered_any<K>(keys[i], kind), p));
        idx[i] = i;
    }
}

// bucket_off[b] = first position of bucket b in the sorted bucket ids.
__global__ void k_bucket_offsets(const uint32_t* __restrict__ ids, uint32_t n, uint32_t buckets,
                                 uint32_t* __restrict__ bucket_off)
{
    const uint32_t b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b > buckets) return;
    uint32_t lo = 0, hi = n;
    while (lo < hi) {
        const uint32_t m = (lo + hi) >> 1;
        if (ids[m] < b) lo = m + 1;
        else hi = m;
    }
    bucket_off[b] = lo;
}

// skip[b] = 0 for every bucket b holding two different keys (skip starts at 1):
// ids are the sorted bucket numbers, aligned with the gathered keys.
template <typename K>
__global__ void k_mixed_buckets(const K* __restrict__ keys, const uint32_t* __restrict__ ids, uint32_t n,
                                uint8_t* __restrict__ skip)
{
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x + 1; i < n; i += stride) {
        const uint32_t b = ids[i];
        if (ids[i - 1] == b && keys[i - 1] != keys[i] && skip[b] != 0) skip[b] = 0;
    }
}

template <typename K>
__global__ void k_gather(const K* __restrict__ keys, const uint32_t* __restrict__ vals, const uint32_t* __restrict__ perm,
                         uint32_t n, K* __restrict__ keys_out, uint32_t* __restrict__ vals_out)
{
    const uint32_t stride = gridDim.x * blockDim.x;
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    for (; i + 3 * stride < n; i += 4 * stride) {
        uint32_t j[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) j[q] = perm[i + q * stride];
        K k[4];
        uint32_t v[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            k[q] = keys[j[q]];
            v[q] = vals[j[q]];
        }
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            keys_out[i + q * stride] = k[q];
            vals_out[i + q * stride] = v[q];
        }
    }
    for (; i < n; i += stride) {
        const uint32_t j = perm[i];
        keys_out[i] = keys[j];
        vals_out[i] = vals[j];
    }
}

// The statistics and boundary check of k_check for either key width.
template <typename K>
__global__ void k_check_any(const K* __restrict__ out, const uint32_t* __restrict__ bucket_off, uint32_t buckets,
                            int kind, uint32_t cap, uint32_t* stats)
{
    const uint32_t b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= buckets) return;
    const uint32_t s = bucket_off[b], e = bucket_off[b + 1];
    const uint32_t len = e - s;
    if (len > cap) {
        atomicAdd(&stats[1], len);
        atomicAdd(&stats[2], 1u);
        if (out[s] == out[e - 1]) atomicAdd(&stats[5], len);
    }
    if (len > 0) atomicAdd(&stats[4], 1u);
    atomicMax(&stats[3], len);
    if (s > 0 && len > 0 && ordered_any<K>(out[s - 1], kind) > ordered_any<K>(out[s], kind))
        atomicExch(&stats[0], 1u);
}

// Points per cooperative training launch: at most one CTA per SM.
static uint32_t train_grid(const device_context& ctx, uint32_t m)
{
    return std::max<uint32_t>(1, std::min<uint32_t>((m + TRAIN_THREADS - 1) / TRAIN_THREADS, ctx.sm_count));
}

constexpr std::size_t TRAIN_SMEM = (std::size_t)(4 * NPARAM + 5 * H * PSTRIDE + PSTRIDE) * 4;

static void launch_train(device_context& ctx, TrainArgs& ta, uint32_t grid)
{
    // per device, so set on every call
    check_cuda(cudaFuncSetAttribute(k_train, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)TRAIN_SMEM),
               "cudaFuncSetAttribute");
    int per_sm = 0;
    check_cuda(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_train, TRAIN_THREADS, TRAIN_SMEM),
               "cudaOccupancyMaxActiveBlocksPerMultiprocessor");
    if ((uint64_t)per_sm * ctx.sm_count < grid) throw std::invalid_argument("learned training: grid does not fit on the device");
    void* args[] = {&ta};
    check_cuda(cudaLaunchCooperativeKernel((const void*)k_train, dim3(grid), dim3(TRAIN_THREADS), args, TRAIN_SMEM,
                                           ctx.stream),
               "learned train launch");
}

// Stages 2-4 on a sorted sample of S keys (order-preserving 32-bit form):
// frame, parameters (fitted unless the model is off), splitters and lookup
// table; returns the sample keys that would fall in buckets above cap
// (reads it back: synchronises).
struct model_scratch {
    float* params;
    Frame* frame;
    float* partial;
    uint32_t* barrier;
    float* losses;
    uint32_t* xs;
    float* ys;
    uint32_t* sp;
    uint16_t* lut;
    uint32_t* est;     // [0] the sample estimate, [1] splitters added by the second level
    uint32_t* refine;  // 3 x buckets words: root splitters, first sample index and grants per root bucket
};

uint32_t build_model(device_context& ctx, const uint32_t* sorted, uint32_t S, uint32_t M, uint32_t G,
                     uint32_t buckets, uint32_t n, uint32_t cap, bool skip_constant, const learned_options& opt,
                     int steps, float lr, const model_scratch& m, uint32_t* refined)
{
    const bool own_init = opt.params_in == nullptr;
    if (!own_init)
        check_cuda(cudaMemcpyAsync(m.params, opt.params_in, NPARAM * 4, cudaMemcpyHostToDevice, ctx.stream),
                   "cudaMemcpyAsync");
    k_frame<<<1, 256, 0, ctx.stream>>>(sorted, S, m.frame, m.params, own_init ? 1 : 0);
    k_points<<<(M + 255) / 256, 256, 0, ctx.stream>>>(sorted, S, m.xs, m.ys, M);
    check_cuda(cudaGetLastError(), "learned frame launch");
    if (opt.use_model && steps > 0) {
        kernel_timer kt(ctx, "learned.train");
        TrainArgs ta{m.params, m.frame, m.xs, m.ys, M, m.partial, m.barrier, nullptr, m.losses, steps, lr,
                     ctx.d_error};
        launch_train(ctx, ta, G);
    }
    {
        kernel_timer kt(ctx, "learned.splitters");
        // second level: a share 1/refine of the buckets splits oversized root buckets
        const int refine = opt.refine < 0 ? 3 : opt.refine;
        const uint32_t budget = opt.splitters_in == nullptr && refine > 0 ? buckets / (uint32_t)refine : 0u;
        const uint32_t bm = buckets - budget;
        if (opt.splitters_in != nullptr) {
            check_cuda(cudaMemcpyAsync(m.sp, opt.splitters_in, (std::size_t)(buckets - 1) * 4,
                                       cudaMemcpyHostToDevice, ctx.stream),
                       "cudaMemcpyAsync");
        } else if (budget == 0) {
            k_splitters<<<(buckets + 127) / 128, 128, 0, ctx.stream>>>(m.params, m.frame, buckets, m.sp,
                                                                       opt.use_model ? 1 : 0);
        } else {
            uint32_t* spm = m.refine;      // bm - 1 root splitters
            uint32_t* lo = spm + buckets;  // bm words
            uint32_t* want = lo + buckets; // bm words
            k_splitters<<<(bm + 127) / 128, 128, 0, ctx.stream>>>(m.params, m.frame, bm, spm, opt.use_model ? 1 : 0);
            k_refine_want<<<(bm + 255) / 256, 256, 0, ctx.stream>>>(sorted, S, spm, bm, n, cap, std::max(1u, cap / 2),
                                                                     lo, want);
            k_refine_plan<<<1, REFINE_THREADS, 0, ctx.stream>>>(want, bm, budget, m.est + 1);
            k_refine_write<<<std::max(1u, (buckets + 254) / 256), 256, 0, ctx.stream>>>(sorted, S, spm, bm, buckets, lo, want,
                                                                           m.est + 1, m.sp);
        }
        k_lut<<<(NCELLS + 1 + 255) / 256, 256, 0, ctx.stream>>>(m.sp, buckets, m.frame, m.lut);
        check_cuda(cudaGetLastError(), "learned splitter launch");
    }
    // A model that would leave most keys in oversized buckets cannot beat the
    // plain sort: the callers decide from the sample, before the partition.
    k_estimate<<<(buckets + 255) / 256, 256, 0, ctx.stream>>>(sorted, S, m.sp, buckets, n, cap,
                                                               skip_constant ? 1 : 0, m.est);
    check_cuda(cudaGetLastError(), "learned estimate launch");
    uint32_t est[2] = {0, 0};  // the estimate, the splitters the second level added
    check_cuda(cudaMemcpyAsync(est, m.est, 8, cudaMemcpyDeviceToHost, ctx.stream), "cudaMemcpyAsync");
    ctx.finish();
    if (refined != nullptr) *refined = est[1];
    return est[0];
}

// Training losses (and the parameters, when asked) back to the host.
void read_training(device_context& ctx, const learned_options& opt, int steps, const float* losses,
                   const float* params, learned_stats& st)
{
    std::vector<float> hl(std::max(steps, 1));
    check_cuda(cudaMemcpyAsync(hl.data(), losses, steps * 4, cudaMemcpyDeviceToHost, ctx.stream), "cudaMemcpyAsync");
    if (opt.params_out != nullptr)
        check_cuda(cudaMemcpyAsync(opt.params_out, params, NPARAM * 4, cudaMemcpyDeviceToHost, ctx.stream),
                   "cudaMemcpyAsync");
    ctx.finish();
    st.first_loss = hl[0];
    st.last_loss = hl[steps - 1];
}

// Sizes shared by both forms: sample S, training points M, buckets, training grid.
struct learned_shape {
    uint32_t S, M, buckets, G;
    int steps;
    float lr;
};

learned_shape shape_for(const device_context& ctx, std::size_t n, const learned_options& opt)
{
    learned_shape sh;
    sh.S = (uint32_t)std::min<std::size_t>(opt.sample > 0 ? opt.sample : (1u << 20), n);
    sh.M = std::max<uint32_t>(1, std::min<uint32_t>({(uint32_t)(opt.points > 0 ? opt.points : 8192), sh.S,
                                                     (uint32_t)(TRAIN_THREADS * ctx.sm_count)}));
    // Buckets: about 8192 keys each by default, as many as the partition
    // kernels' shared memory holds (counters, splitters and the table).
    const uint32_t max_buckets =
        (uint32_t)std::min<std::size_t>(65536, (ctx.smem_optin - (std::size_t)(NCELLS + 1) * 2 + 4) / 8);
    if (opt.buckets > 0) {
        sh.buckets = (uint32_t)opt.buckets;
        if (sh.buckets < 2 || sh.buckets > max_buckets)
            throw std::invalid_argument("sort_learned: buckets must be in [2, " + std::to_string(max_buckets) + "]");
    } else {
        const uint32_t want = (uint32_t)((n / 8192 + 1023) / 1024 * 1024);
        sh.buckets = std::max<uint32_t>(4096, std::min<uint32_t>(want, max_buckets / 1024 * 1024));
    }
    // Adam steps: none by default. The data-driven initial network (ramps
    // between sample quantiles) is already a fit of the sample's CDF, and on
    // the 2^28-key mixture gradient steps cost more than they save downstream
    // (0, 8, 16, 32, 64 steps: 8.2, 8.4, 8.6, 8.9, 9.5 ms without the second
    // level; 7.8 against 8.5 ms with it at 32 steps).
    sh.steps = opt.steps >= 0 ? opt.steps : 0;
    sh.lr = opt.lr > 0 ? opt.lr : 0.01f;
    sh.G = train_grid(ctx, sh.M);
    return sh;
}

// The model stages' scratch: points, parameters and frame, training
// partials, splitters and table, small words (barrier, statistics, losses).
struct model_buffers {
    temp_buffer pts, prm, partial, spl, misc, refine;
    model_scratch m;
    uint32_t* dstats;  // [0..5] k_check statistics, [6] estimate, [7] splitters added by the second level
    model_buffers(device_context& ctx, const learned_shape& sh)
        : pts(ctx.resource, (std::size_t)2 * sh.M * 4),
          prm(ctx.resource, (std::size_t)NPARAM * 4 + sizeof(Frame) + 16),
          partial(ctx.resource, (std::size_t)2 * sh.G * PSTR * 4),
          spl(ctx.resource, (std::size_t)sh.buckets * 4 + (std::size_t)(NCELLS + 1) * 2 + 16),
          misc(ctx.resource, 64 + (std::size_t)std::max(sh.steps, 1) * 4),
          refine(ctx.resource, (std::size_t)3 * sh.buckets * 4)
    {
        check_cuda(cudaMemsetAsync(misc.get(), 0, 64 + (std::size_t)std::max(sh.steps, 1) * 4, ctx.stream),
                   "cudaMemsetAsync");
        m.params = prm.as<float>();
        m.frame = reinterpret_cast<Frame*>(
            (reinterpret_cast<uintptr_t>(prm.as<unsigned char>() + (std::size_t)NPARAM * 4) + 15) & ~(uintptr_t)15);
        m.partial = partial.as<float>();
        m.barrier = misc.as<uint32_t>();  // [0]
        dstats = m.barrier + 4;           // [4..10]
        m.losses = reinterpret_cast<float*>(misc.as<unsigned char>() + 64);
        m.xs = pts.as<uint32_t>();
        m.ys = reinterpret_cast<float*>(m.xs + sh.M);
        m.sp = spl.as<uint32_t>();
        m.lut = reinterpret_cast<uint16_t*>(m.sp + sh.buckets);
        m.est = dstats + 6;
        m.refine = refine.as<uint32_t>();
    }
};

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
    const learned_shape sh = shape_for(ctx, n, opt);
    const uint32_t S = sh.S, buckets = sh.buckets;
    const int steps = sh.steps;
    const std::size_t part_smem = part_smem_bytes(buckets);

    // Scratch: the model's, the sample, per-(CTA, bucket) counts, offsets, totals.
    const std::size_t rows = (std::size_t)ctx.sm_count;
    model_buffers mb(ctx, sh);
    temp_buffer sample(ctx.resource, (std::size_t)S * 4);
    temp_buffer counts(ctx.resource, rows * buckets * 4);
    temp_buffer boff(ctx.resource, ((std::size_t)buckets + 1) * 4);
    temp_buffer totals(ctx.resource, (std::size_t)buckets * 4);
    uint32_t* dstats = mb.dstats;
    Frame* frame = mb.m.frame;
    uint32_t* sp = mb.m.sp;
    uint16_t* lut = mb.m.lut;

    const uint32_t* in = static_cast<const uint32_t*>(keys_in);
    uint32_t* out = static_cast<uint32_t*>(keys_out);
    {
        kernel_timer kt(ctx, "learned.sample");
        k_sample<<<(S + 255) / 256, 256, 0, ctx.stream>>>(in, nn, sample.as<uint32_t>(), S, key_kind);
        check_cuda(cudaGetLastError(), "learned sample launch");
    }
    radix_sort(ctx, sample.get(), sample.get(), 4, 0, nullptr, nullptr, S, false);
    const bool train = opt.use_model && steps > 0;
    const uint32_t cap = segsort_cta_cap(4, false);
    // buckets holding one key value need no sort, so they do not count
    // against the model
    const uint32_t est = build_model(ctx, sample.as<uint32_t>(), S, sh.M, sh.G, buckets, nn, cap, true, opt, steps,
                                     sh.lr, mb.m, &st.refined_splitters);
    auto read_losses = [&] {
        if (train) read_training(ctx, opt, steps, mb.m.losses, mb.m.params, st);
    };
    st.buckets = buckets;
    st.estimated_oversized_keys = (uint32_t)std::min<uint64_t>(n, (uint64_t)est * n / S);
    if ((uint64_t)est * 2 > S) {
        read_losses();
        st.fallback = 1;
        radix_sort(ctx, keys_in, keys_out, 4, key_kind, nullptr, nullptr, n, false);
        if (stats_host) *stats_host = st;
        return;
    }

    temp_buffer ids(ctx.resource, (std::size_t)n * 2);  // every key's bucket (u16: buckets <= 65536)
    PartArgs pa{in, nn, key_kind, frame, sp, lut, buckets, counts.as<uint32_t>(), ids.as<uint16_t>()};
    // shared-memory opt-in is per device: set on every call
    check_cuda(cudaFuncSetAttribute(k_count, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)part_smem),
               "cudaFuncSetAttribute");
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
        // two levels: bucket groups into tmp, then buckets into out
        const uint32_t groups = (buckets + PART_GROUP - 1) / PART_GROUP;
        temp_buffer tmp(ctx.resource, (std::size_t)n * 4), tmp_ids(ctx.resource, (std::size_t)n * 2);
        temp_buffer cur(ctx.resource, ((std::size_t)buckets + groups) * 4);
        uint32_t* bucket_cur = cur.as<uint32_t>();
        uint32_t* group_cur = bucket_cur + buckets;
        k_cursors<<<(buckets + 255) / 256, 256, 0, ctx.stream>>>(boff.as<uint32_t>(), buckets, group_cur, bucket_cur);
        // Threads per partition CTA, per level: 1024 (one CTA per SM), 512
        // or 256 (two or four per SM, each CTA's barriers and reservation
        // round trips overlapping the others' work; a chunk is 8 keys per
        // thread). The first level needs groups <= threads. Measured at 2^28
        // mixture keys (1024 / 512 / 256 threads): group level 1.36 / 1.11 /
        // 1.53 ms (at 256, chunks of 2,048 keys leave ~10 keys per group and
        // chunk), bucket level 1.12 / 0.98 / 0.91 ms. Defaults 512 and 256;
        // the tuning table's "learned:group_threads" and
        // "learned:bucket_threads" entries override them.
        auto threads_of = [&](const char* key, int dflt, uint32_t need) {
            launch_shape sh;
            int t = ctx.tuning.lookup(key, sh) ? sh.variant : dflt;
            if (t != 256 && t != 512) t = PART_THREADS;
            return (uint32_t)t < need ? PART_THREADS : t;
        };
        const int gt = threads_of("learned:group_threads", 512, groups);
        const int bt = threads_of("learned:bucket_threads", 256, 0);
        auto group_level = [&](auto tc) {
            constexpr int T = decltype(tc)::value;
            kernel_timer kt(ctx, "learned.partition_groups");
            const std::size_t gsmem = group_smem_bytes(buckets, T);
            check_cuda(cudaFuncSetAttribute(k_partition_groups<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                            (int)gsmem),
                       "cudaFuncSetAttribute");
            k_partition_groups<T><<<(int)rows * (PART_THREADS / T), T, gsmem, ctx.stream>>>(
                pa, groups, tmp.as<uint32_t>(), tmp_ids.as<uint16_t>(), group_cur);
        };
        auto bucket_level = [&](auto tc) {
            constexpr int T = decltype(tc)::value;
            kernel_timer kt(ctx, "learned.partition_buckets");
            const std::size_t bsmem = bucket_smem_bytes(T);
            check_cuda(cudaFuncSetAttribute(k_partition_buckets<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                            (int)bsmem),
                       "cudaFuncSetAttribute");
            k_partition_buckets<T><<<(int)rows * (PART_THREADS / T), T, bsmem, ctx.stream>>>(
                pa, tmp.as<uint32_t>(), tmp_ids.as<uint16_t>(), out, bucket_cur);
        };
        if (gt == 256) group_level(std::integral_constant<int, 256>());
        else if (gt == 512) group_level(std::integral_constant<int, 512>());
        else group_level(std::integral_constant<int, PART_THREADS>());
        if (bt == 256) bucket_level(std::integral_constant<int, 256>());
        else if (bt == 512) bucket_level(std::integral_constant<int, 512>());
        else bucket_level(std::integral_constant<int, PART_THREADS>());
        check_cuda(cudaGetLastError(), "learned partition launch");
    }
    // Finish every bucket that holds two different keys in place
    // (shared-memory sorts; oversized buckets take the batched onesweep
    // path); buckets of one key value are already in order.
    temp_buffer skip(ctx.resource, buckets);
    {
        kernel_timer kt(ctx, "learned.check");
        k_constant_buckets<<<buckets, 256, 0, ctx.stream>>>(out, boff.as<uint32_t>(), skip.as<uint8_t>());
        check_cuda(cudaGetLastError(), "learned bucket check launch");
    }
    seg_options so;
    so.skip = skip.as<uint8_t>();
    // Buckets are mostly near the one-CTA capacity: twice the warps per CTA
    // (one CTA per SM either way) finish them faster (2^28 mixture keys:
    // 2.50 -> 1.92 ms for the one-CTA sorts, 7.72 -> 7.22 ms for the sort).
    so.cta_threads = 512;
    segmented_sort(ctx, out, out, 4, key_kind, nullptr, nullptr, n, boff.as<uint32_t>(), buckets, false, so);
    {
        kernel_timer kt(ctx, "learned.check");
        k_check<<<(buckets + 255) / 256, 256, 0, ctx.stream>>>(out, boff.as<uint32_t>(), buckets, key_kind, cap,
                                                                dstats);
        check_cuda(cudaGetLastError(), "learned check launch");
    }
    // Read the statistics (and losses); a violation sends the input to the
    // plain radix sort. (The bucket of a key is the result of a binary search
    // over the splitters, which is monotone in the key for any splitter
    // array, so the check guards the implementation rather than the model.)
    std::vector<uint32_t> hs(6);
    check_cuda(cudaMemcpyAsync(hs.data(), dstats, 6 * 4, cudaMemcpyDeviceToHost, ctx.stream), "cudaMemcpyAsync");
    read_losses();
    st.violation = hs[0];
    st.oversized_keys = hs[1];
    st.oversized_buckets = hs[2];
    st.largest_bucket = hs[3];
    st.nonempty_buckets = hs[4];
    st.constant_keys = hs[5];
    if (st.violation) {
        st.fallback = 1;
        radix_sort(ctx, keys_in, keys_out, 4, key_kind, nullptr, nullptr, n, false);
    }
    if (stats_host) *stats_host = st;
}

void learned_sort_pairs(device_context& ctx, const void* keys_in, void* keys_out, int key_bytes, int key_kind,
                        const uint32_t* vals_in, uint32_t* vals_out, std::size_t n, const learned_options& opt,
                        learned_stats* stats_host)
{
    using namespace learned;
    if (key_bytes != 4 && key_bytes != 8) throw std::invalid_argument("sort_learned_pairs: keys must be 4 or 8 bytes");
    if (key_kind < 0 || key_kind > (key_bytes == 4 ? 2 : 1))
        throw std::invalid_argument("sort_learned_pairs: unknown key kind");
    check_size(n);
    if (n == 0) {
        if (stats_host) *stats_host = learned_stats{};
        return;
    }
    if (keys_in == nullptr || keys_out == nullptr || vals_in == nullptr || vals_out == nullptr)
        throw std::invalid_argument("sort_learned_pairs: null argument");
    if (keys_in == keys_out || vals_in == vals_out)
        throw std::invalid_argument("sort_learned_pairs: inputs and outputs must differ");
    ctx.activate();
    learned_stats st;
    if (n == 1) {
        check_cuda(cudaMemcpyAsync(keys_out, keys_in, key_bytes, cudaMemcpyDeviceToDevice, ctx.stream),
                   "cudaMemcpyAsync");
        check_cuda(cudaMemcpyAsync(vals_out, vals_in, 4, cudaMemcpyDeviceToDevice, ctx.stream), "cudaMemcpyAsync");
        if (stats_host) *stats_host = st;
        return;
    }
    const uint32_t nn = (uint32_t)n;
    const learned_shape sh = shape_for(ctx, n, opt);
    const uint32_t S = sh.S, buckets = sh.buckets;
    const int steps = sh.steps;
    model_buffers mb(ctx, sh);
    temp_buffer sample(ctx.resource, (std::size_t)S * 8 + 16);
    temp_buffer sample32(ctx.resource, (std::size_t)S * 4);
    temp_buffer proj(ctx.resource, sizeof(Proj));
    Proj* pj = proj.as<Proj>();

    // 1. the sorted sample in the order-preserving form, projected to 32 bits
    {
        kernel_timer kt(ctx, "learned.sample");
        if (key_bytes == 8) {
            k_sample64<<<(S + 255) / 256, 256, 0, ctx.stream>>>(static_cast<const uint64_t*>(keys_in), nn,
                                                                 sample.as<uint64_t>(), S, key_kind);
        } else {
            k_sample<<<(S + 255) / 256, 256, 0, ctx.stream>>>(static_cast<const uint32_t*>(keys_in), nn,
                                                               sample32.as<uint32_t>(), S, key_kind);
        }
        check_cuda(cudaGetLastError(), "learned sample launch");
    }
    if (key_bytes == 8) {
        radix_sort(ctx, sample.get(), sample.get(), 8, 0, nullptr, nullptr, S, false);
        k_project<<<1, 1024, 0, ctx.stream>>>(sample.as<uint64_t>(), S, pj, sample32.as<uint32_t>());
        check_cuda(cudaGetLastError(), "learned projection launch");
    } else {
        radix_sort(ctx, sample32.get(), sample32.get(), 4, 0, nullptr, nullptr, S, false);
        const Proj identity{0ull, 0, 0};
        check_cuda(cudaMemcpyAsync(pj, &identity, sizeof(Proj), cudaMemcpyHostToDevice, ctx.stream), "cudaMemcpyAsync");
    }

    // 2-4. the model, its splitters, and the decision from the sample
    const bool train = opt.use_model && steps > 0;
    const uint32_t cap = segsort_cta_cap(key_bytes, true);
    // buckets holding one key value are left as the stable partition leaves
    // them (already in order), so they do not count against the model
    const uint32_t est = build_model(ctx, sample32.as<uint32_t>(), S, sh.M, sh.G, buckets, nn, cap, true, opt, steps,
                                     sh.lr, mb.m, &st.refined_splitters);
    st.buckets = buckets;
    st.estimated_oversized_keys = (uint32_t)std::min<uint64_t>(n, (uint64_t)est * n / S);
    auto plain = [&] {
        st.fallback = 1;
        radix_sort(ctx, keys_in, keys_out, key_bytes, key_kind, vals_in, vals_out, n, false);
    };
    if ((uint64_t)est * 2 > S) {
        if (train) read_training(ctx, opt, steps, mb.m.losses, mb.m.params, st);
        plain();
        if (stats_host) *stats_host = st;
        return;
    }

    // 5. stable partition: bucket of every key, the indices stably sorted by
    // bucket (the plain radix sort, whose pass plan skips the digits that no
    // bucket number uses), keys and values gathered in that order
    temp_buffer ids(ctx.resource, (std::size_t)n * 4), idx(ctx.resource, (std::size_t)n * 4);
    temp_buffer ids_sorted(ctx.resource, (std::size_t)n * 4), perm(ctx.resource, (std::size_t)n * 4);
    temp_buffer boff(ctx.resource, ((std::size_t)buckets + 1) * 4);
    const std::size_t ids_smem = (std::size_t)(buckets - 1) * 4 + (std::size_t)(NCELLS + 1) * 2;
    {
        kernel_timer kt(ctx, "learned.count");
        const int grid = ctx.sm_count * 2;
        if (key_bytes == 8) {
            check_cuda(cudaFuncSetAttribute(k_bucket_ids<uint64_t>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                            (int)ids_smem),
                       "cudaFuncSetAttribute");
            k_bucket_ids<uint64_t><<<grid, PART_THREADS, ids_smem, ctx.stream>>>(
                static_cast<const uint64_t*>(keys_in), nn, key_kind, pj, mb.m.frame, mb.m.sp, mb.m.lut, buckets,
                ids.as<uint32_t>(), idx.as<uint32_t>());
        } else {
            check_cuda(cudaFuncSetAttribute(k_bucket_ids<uint32_t>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                            (int)ids_smem),
                       "cudaFuncSetAttribute");
            k_bucket_ids<uint32_t><<<grid, PART_THREADS, ids_smem, ctx.stream>>>(
                static_cast<const uint32_t*>(keys_in), nn, key_kind, pj, mb.m.frame, mb.m.sp, mb.m.lut, buckets,
                ids.as<uint32_t>(), idx.as<uint32_t>());
        }
        check_cuda(cudaGetLastError(), "learned bucket launch");
    }
    radix_sort(ctx, ids.get(), ids_sorted.get(), 4, 0, idx.as<uint32_t>(), perm.as<uint32_t>(), n, false);
    {
        kernel_timer kt(ctx, "learned.scatter");
        k_bucket_offsets<<<(buckets + 1 + 255) / 256, 256, 0, ctx.stream>>>(ids_sorted.as<uint32_t>(), nn, buckets,
                                                                            boff.as<uint32_t>());
        const int grid = ctx.sm_count * 8;
        if (key_bytes == 8)
            k_gather<uint64_t><<<grid, 256, 0, ctx.stream>>>(static_cast<const uint64_t*>(keys_in), vals_in,
                                                             perm.as<uint32_t>(), nn,
                                                             static_cast<uint64_t*>(keys_out), vals_out);
        else
            k_gather<uint32_t><<<grid, 256, 0, ctx.stream>>>(static_cast<const uint32_t*>(keys_in), vals_in,
                                                             perm.as<uint32_t>(), nn,
                                                             static_cast<uint32_t*>(keys_out), vals_out);
        check_cuda(cudaGetLastError(), "learned gather launch");
    }
    // 6. every bucket that holds two different keys finished in place by the
    // stable segmented sort; the others are already in order
    temp_buffer skip(ctx.resource, buckets);
    check_cuda(cudaMemsetAsync(skip.get(), 1, buckets, ctx.stream), "cudaMemsetAsync");
    {
        kernel_timer kt(ctx, "learned.scatter");
        if (key_bytes == 8)
            k_mixed_buckets<uint64_t><<<ctx.sm_count * 8, 256, 0, ctx.stream>>>(
                static_cast<const uint64_t*>(keys_out), ids_sorted.as<uint32_t>(), nn, skip.as<uint8_t>());
        else
            k_mixed_buckets<uint32_t><<<ctx.sm_count * 8, 256, 0, ctx.stream>>>(
                static_cast<const uint32_t*>(keys_out), ids_sorted.as<uint32_t>(), nn, skip.as<uint8_t>());
        check_cuda(cudaGetLastError(), "learned bucket check launch");
    }
    seg_options so;
    so.skip = skip.as<uint8_t>();
    segmented_sort(ctx, keys_out, keys_out, key_bytes, key_kind, vals_out, vals_out, n, boff.as<uint32_t>(), buckets,
                   false, so);
    // 7. statistics and the boundary check
    {
        kernel_timer kt(ctx, "learned.check");
        if (key_bytes == 8)
            k_check_any<uint64_t><<<(buckets + 255) / 256, 256, 0, ctx.stream>>>(
                static_cast<const uint64_t*>(keys_out), boff.as<uint32_t>(), buckets, key_kind, cap, mb.dstats);
        else
            k_check_any<uint32_t><<<(buckets + 255) / 256, 256, 0, ctx.stream>>>(
                static_cast<const uint32_t*>(keys_out), boff.as<uint32_t>(), buckets, key_kind, cap, mb.dstats);
        check_cuda(cudaGetLastError(), "learned check launch");
    }
    std::vector<uint32_t> hs(6);
    check_cuda(cudaMemcpyAsync(hs.data(), mb.dstats, 6 * 4, cudaMemcpyDeviceToHost, ctx.stream), "cudaMemcpyAsync");
    if (train) read_training(ctx, opt, steps, mb.m.losses, mb.m.params, st);
    ctx.finish();
    st.violation = hs[0];
    st.oversized_keys = hs[1];
    st.oversized_buckets = hs[2];
    st.largest_bucket = hs[3];
    st.nonempty_buckets = hs[4];
    st.constant_keys = hs[5];
    if (st.violation) plain();
    if (stats_host) *stats_host = st;
}

void mlp_gradients(device_context& ctx, const float* params_host, const uint32_t* centres_host, float inv_span,
                   const uint32_t* keys_host, const float* ys_host, std::size_t m, float* grad_host, float* loss_host)
{
    using namespace learned;
    if (m == 0 || m > (1u << 24)) throw std::invalid_argument("mlp_gradients: 0 < m <= 2^24");
    ctx.activate();
    const uint32_t G = train_grid(ctx, (uint32_t)m);
    temp_buffer prm(ctx.resource, (std::size_t)NPARAM * 4 + sizeof(Frame) + 16);
    temp_buffer pts(ctx.resource, (std::size_t)2 * m * 4);
    temp_buffer partial(ctx.resource, (std::size_t)2 * G * PSTR * 4);
    temp_buffer misc(ctx.resource, 64 + (std::size_t)NPARAM * 4);
    float* params = prm.as<float>();
    Frame* frame = reinterpret_cast<Frame*>(
        (reinterpret_cast<uintptr_t>(prm.as<unsigned char>() + (std::size_t)NPARAM * 4) + 15) & ~(uintptr_t)15);
    uint32_t* xs = pts.as<uint32_t>();
    float* ys = reinterpret_cast<float*>(xs + m);
    uint32_t* barrier = misc.as<uint32_t>();
    float* loss = reinterpret_cast<float*>(misc.as<unsigned char>() + 16);
    float* grad = reinterpret_cast<float*>(misc.as<unsigned char>() + 64);
    Frame hf{};
    hf.inv_span = inv_span;
    std::memcpy(hf.c, centres_host, sizeof(hf.c));
    check_cuda(cudaMemsetAsync(misc.get(), 0, 64 + (std::size_t)NPARAM * 4, ctx.stream), "cudaMemsetAsync");
    check_cuda(cudaMemcpyAsync(params, params_host, NPARAM * 4, cudaMemcpyHostToDevice, ctx.stream), "cudaMemcpyAsync");
    check_cuda(cudaMemcpyAsync(frame, &hf, sizeof(Frame), cudaMemcpyHostToDevice, ctx.stream), "cudaMemcpyAsync");
    check_cuda(cudaMemcpyAsync(xs, keys_host, m * 4, cudaMemcpyHostToDevice, ctx.stream), "cudaMemcpyAsync");
    check_cuda(cudaMemcpyAsync(ys, ys_host, m * 4, cudaMemcpyHostToDevice, ctx.stream), "cudaMemcpyAsync");
    TrainArgs ta{params, frame, xs, ys, (uint32_t)m, partial.as<float>(), barrier, grad, loss, 1, 0.f, ctx.d_error};
    launch_train(ctx, ta, G);
    check_cuda(cudaMemcpyAsync(grad_host, grad, NPARAM * 4, cudaMemcpyDeviceToHost, ctx.stream), "cudaMemcpyAsync");
    check_cuda(cudaMemcpyAsync(loss_host, loss, 4, cudaMemcpyDeviceToHost, ctx.stream), "cudaMemcpyAsync");
    ctx.finish();
}

}  // namespace gbc
