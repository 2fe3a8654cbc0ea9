// CPU ORACLE — test infrastructure only.
//
// This file is the reference oracle for gbcompute's parity tests and the CPU
// baseline of bench.py. It is never linked into libgbcompute.so and nothing on the
// product path calls it. Only tests/, __graft_entry__.smoke() and bench.py's
// CPU-baseline leg load it.
//
// Two layers:
//  1. std:: ground truth, exactly as the reference's own tests compute their
//     host references (lib/test/Compute/main.cpp): std::stable_sort of
//     (key, index) pairs by the order-preserving key bijection (main.cpp:
//     257-263), sequential scans (215-222), std::accumulate (188-189) and the
//     histogram bin formula of the device code (Algorithm.cpp:251-258).
//     The seeded generators reproduce main.cpp:45-52 (std::mt19937 +
//     uniform_int_distribution) and main.cpp:297-300 bit for bit with
//     libstdc++.
//  2. A CPU restatement of the reference algorithms, multi-threaded, used as
//     the timed CPU baseline and as a second opinion:
//       - radix sort: 8 passes of 4 bits over tiles of 128 x 8 keys, a
//         digit-major per-tile count table, its exclusive scan and a stable
//         scatter (Algorithm.cpp:133-213, 453-527);
//       - scan: tiles of 256 x 4, tile totals scanned recursively and added
//         back (Algorithm.cpp:79-127, 280-318);
//       - reduce: at most 256 groups of 256 work-items folding a grid-stride
//         slice, tree reductions, init applied once (Algorithm.cpp:58-74,
//         400-442) — operation order identical, so float results match the
//         reference's bit for bit as long as the OpenCL compiler does not
//         reassociate;
//       - histogram_even: private bins per thread, same bin rule
//         (Algorithm.cpp:240-273, 569-615).
//
// Pinning: tests/test_oracle.py checks layer 2 against layer 1 and both
// against the known answers in the reference's tests (capi.c:103-141: sum,
// max 499, sorted ascending; main.cpp:274-311: stability with 16 distinct
// keys, signed extremes, float -0.0/inf descending).
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <functional>
#include <numeric>
#include <random>
#include <thread>
#include <vector>

namespace {

enum { T_I8, T_U8, T_I16, T_U16, T_I32, T_U32, T_I64, T_U64, T_F32, T_F64 };
enum { OP_PLUS, OP_MUL, OP_AND, OP_OR, OP_XOR, OP_MIN, OP_MAX, OP_RIGHT };

template <typename K> K xform(K k, int kind, int desc)
{
    constexpr K sign = K(1) << (sizeof(K) * 8 - 1);
    K t = k;
    if (kind == 1) t = k ^ sign;
    if (kind == 2) t = (k & sign) ? K(~k) : K(k | sign);
    if (desc) t = ~t;
    return t;
}

int hw_threads(int requested)
{
    if (requested > 0) return requested;
    const unsigned h = std::thread::hardware_concurrency();
    return h == 0 ? 1 : (int)h;
}

void parallel_for(std::size_t n, int threads, const std::function<void(std::size_t, std::size_t)>& body)
{
    threads = std::max(1, std::min<int>(threads, (int)std::max<std::size_t>(n, 1)));
    if (threads == 1) {
        body(0, n);
        return;
    }
    std::vector<std::thread> pool;
    const std::size_t chunk = (n + threads - 1) / threads;
    for (int t = 0; t < threads; ++t) {
        const std::size_t b = std::min(n, t * chunk), e = std::min(n, b + chunk);
        pool.emplace_back([&body, b, e] { body(b, e); });
    }
    for (auto& th : pool) th.join();
}

template <typename T> T apply(int op, T a, T b)
{
    switch (op) {
    case OP_PLUS: return (T)(a + b);
    case OP_MUL: return (T)(a * b);
    case OP_MIN: return (b < a) ? b : a;
    case OP_MAX: return (a < b) ? b : a;
    case OP_RIGHT: return b;
    default: break;
    }
    if constexpr (std::is_integral<T>::value) {
        switch (op) {
        case OP_AND: return (T)(a & b);
        case OP_OR: return (T)(a | b);
        case OP_XOR: return (T)(a ^ b);
        default: break;
        }
    }
    return a;
}

// Integer arithmetic wraps: compute plus/mul in the unsigned counterpart.
template <typename T> T wrap_apply(int op, T a, T b)
{
    if constexpr (std::is_integral<T>::value && std::is_signed<T>::value) {
        using U = typename std::make_unsigned<T>::type;
        if (op == OP_PLUS) return (T)(U)((U)a + (U)b);
        if (op == OP_MUL) return (T)(U)((U)a * (U)b);
    }
    if constexpr (std::is_integral<T>::value && sizeof(T) < sizeof(int)) {
        if (op == OP_PLUS) return (T)(unsigned)((unsigned)a + (unsigned)b);
        if (op == OP_MUL) return (T)(unsigned)((unsigned)a * (unsigned)b);
    }
    return apply<T>(op, a, b);
}

template <typename F> void by_type(int type, F&& f)
{
    switch (type) {
    case T_I8: f(int8_t{}); break;
    case T_U8: f(uint8_t{}); break;
    case T_I16: f(int16_t{}); break;
    case T_U16: f(uint16_t{}); break;
    case T_I32: f(int32_t{}); break;
    case T_U32: f(uint32_t{}); break;
    case T_I64: f(int64_t{}); break;
    case T_U64: f(uint64_t{}); break;
    case T_F32: f(float{}); break;
    case T_F64: f(double{}); break;
    }
}

template <typename K>
void std_sort_pairs(K* keys, uint32_t* vals, std::size_t n, int kind, int desc)
{
    std::vector<uint32_t> idx(n);
    std::iota(idx.begin(), idx.end(), 0u);
    std::stable_sort(idx.begin(), idx.end(), [&](uint32_t a, uint32_t b) {
        return xform<K>(keys[a], kind, desc) < xform<K>(keys[b], kind, desc);
    });
    std::vector<K> k2(n);
    for (std::size_t i = 0; i < n; ++i) k2[i] = keys[idx[i]];
    std::memcpy(keys, k2.data(), n * sizeof(K));
    if (vals) {
        std::vector<uint32_t> v2(n);
        for (std::size_t i = 0; i < n; ++i) v2[i] = vals[idx[i]];
        std::memcpy(vals, v2.data(), n * 4);
    }
}

// Restated reference radix sort: 4-bit digits, tiles of WG*ITEMS keys.
template <typename K>
void ref_radix_sort(K* keys, uint32_t* vals, std::size_t n, int kind, int desc, int threads)
{
    if (n <= 1) return;
    constexpr std::size_t WG = 128, ITEMS = 8, TILE = WG * ITEMS, RADIX = 16;
    constexpr int PASSES = (int)(sizeof(K) * 2);
    const std::size_t groups = (n + TILE - 1) / TILE;
    std::vector<K> kalt(n);
    std::vector<uint32_t> valt(vals ? n : 0);
    std::vector<uint32_t> counts(RADIX * groups), offsets(RADIX * groups);
    K* kb[2] = {keys, kalt.data()};
    uint32_t* vb[2] = {vals, vals ? valt.data() : nullptr};
    threads = hw_threads(threads);
    for (int pass = 0; pass < PASSES; ++pass) {
        const int shift = pass * 4, src = pass & 1, dst = src ^ 1;
        const K* in = kb[src];
        // clc_radix_histogram: digit-major table histogram[digit * groups + group]
        parallel_for(groups, threads, [&](std::size_t g0, std::size_t g1) {
            for (std::size_t g = g0; g < g1; ++g) {
                uint32_t c[RADIX] = {0};
                const std::size_t b = g * TILE, e = std::min(n, b + TILE);
                for (std::size_t i = b; i < e; ++i) ++c[(xform<K>(in[i], kind, desc) >> shift) & 15];
                for (std::size_t d = 0; d < RADIX; ++d) counts[d * groups + g] = c[d];
            }
        });
        // scan_impl(exclusive, plus) over the table
        uint32_t run = 0;
        for (std::size_t i = 0; i < RADIX * groups; ++i) {
            offsets[i] = run;
            run += counts[i];
        }
        // clc_radix_scatter: stable, in index order within a tile
        parallel_for(groups, threads, [&](std::size_t g0, std::size_t g1) {
            for (std::size_t g = g0; g < g1; ++g) {
                uint32_t base[RADIX];
                for (std::size_t d = 0; d < RADIX; ++d) base[d] = offsets[d * groups + g];
                const std::size_t b = g * TILE, e = std::min(n, b + TILE);
                for (std::size_t i = b; i < e; ++i) {
                    const uint32_t d = (xform<K>(in[i], kind, desc) >> shift) & 15;
                    const uint32_t o = base[d]++;
                    kb[dst][o] = in[i];
                    if (vals) vb[dst][o] = vb[src][i];
                }
            }
        });
    }
    // An even pass count leaves the result in the caller's buffers.
}

template <typename T>
void std_scan(const T* in, T* out, std::size_t n, int op, T identity, int exclusive)
{
    T run = identity;
    for (std::size_t i = 0; i < n; ++i) {
        const T x = in[i];
        const T next = wrap_apply<T>(op, run, x);
        out[i] = exclusive ? run : next;
        run = next;
    }
}

// Restated three-phase scan (tiles of 256 x 4, recursive on tile totals).
template <typename T>
void ref_scan(const T* in, T* out, std::size_t n, int op, T identity, int exclusive, int threads)
{
    if (n == 0) return;
    constexpr std::size_t TILE = 256 * 4;
    const std::size_t tiles = (n + TILE - 1) / TILE;
    std::vector<T> totals(tiles);
    std::vector<T> tmp(in, in + n);  // in may alias out
    parallel_for(tiles, hw_threads(threads), [&](std::size_t t0, std::size_t t1) {
        for (std::size_t t = t0; t < t1; ++t) {
            T run = identity;
            const std::size_t b = t * TILE, e = std::min(n, b + TILE);
            for (std::size_t i = b; i < e; ++i) {
                const T next = wrap_apply<T>(op, run, tmp[i]);
                out[i] = exclusive ? run : next;
                run = next;
            }
            // pad with identity like the reference so the tile total matches
            for (std::size_t i = e; i < b + TILE; ++i) run = wrap_apply<T>(op, run, identity);
            totals[t] = run;
        }
    });
    if (tiles == 1) return;
    std::vector<T> offs(tiles);
    ref_scan<T>(totals.data(), offs.data(), tiles, op, identity, 1, 1);
    parallel_for(tiles, hw_threads(threads), [&](std::size_t t0, std::size_t t1) {
        for (std::size_t t = std::max<std::size_t>(t0, 1); t < t1; ++t) {
            const std::size_t b = t * TILE, e = std::min(n, b + TILE);
            for (std::size_t i = b; i < e; ++i) out[i] = wrap_apply<T>(op, offs[t], out[i]);
        }
    });
}

// Restated two-level reduce with the reference's exact combination order.
template <typename T>
T ref_reduce(const T* in, std::size_t n, int op, T identity, T init, int threads)
{
    if (n == 0) return init;
    constexpr std::size_t WG = 256;
    auto level = [&](const T* src, std::size_t m, std::size_t groups, bool apply_init) {
        std::vector<T> part(groups);
        parallel_for(groups, hw_threads(threads), [&](std::size_t g0, std::size_t g1) {
            std::vector<T> scratch(WG);
            for (std::size_t g = g0; g < g1; ++g) {
                for (std::size_t l = 0; l < WG; ++l) {
                    T acc = identity;
                    for (std::size_t i = g * WG + l; i < m; i += groups * WG) acc = wrap_apply<T>(op, acc, src[i]);
                    scratch[l] = acc;
                }
                for (std::size_t s = WG / 2; s > 0; s >>= 1)
                    for (std::size_t l = 0; l < s; ++l) scratch[l] = wrap_apply<T>(op, scratch[l], scratch[l + s]);
                part[g] = apply_init ? wrap_apply<T>(op, init, scratch[0]) : scratch[0];
            }
        });
        return part;
    };
    const std::size_t groups = std::min<std::size_t>((n + WG - 1) / WG, 256);
    const std::vector<T> partials = level(in, n, groups, false);
    return level(partials.data(), groups, 1, true)[0];
}

template <typename T>
void histogram_even(const T* in, std::size_t n, uint32_t* hist, std::size_t bins, double lower, double upper,
                    int threads)
{
    using ACC = typename std::conditional<std::is_same<T, double>::value, double, float>::type;
    std::fill(hist, hist + bins, 0u);
    if (bins == 0 || n == 0) return;
    const ACC lo = (ACC)lower, hi = (ACC)upper;
    const ACC scale = (ACC)bins / (hi - lo);
    const int nt = hw_threads(threads);
    std::vector<std::vector<uint32_t>> priv(nt, std::vector<uint32_t>(bins, 0));
    std::atomic<int> next{0};
    parallel_for(n, nt, [&](std::size_t b, std::size_t e) {
        auto& h = priv[next++];
        for (std::size_t i = b; i < e; ++i) {
            const ACC x = (ACC)in[i];
            if (x >= lo && x < hi) {
                // volatile keeps the float product from being contracted
                volatile ACC d = x - lo;
                volatile ACC prod = d * scale;
                uint32_t bin = (uint32_t)prod;
                if (bin >= bins) bin = (uint32_t)bins - 1;
                ++h[bin];
            }
        }
    });
    for (const auto& h : priv)
        for (std::size_t b = 0; b < bins; ++b) hist[b] += h[b];
}

}  // namespace

extern "C" {

// ---- generators (reference test recipes) -------------------------------

// main.cpp:45-52 random_uints(n, max, seed)
void orc_random_uints(uint32_t* out, std::size_t n, uint32_t max, unsigned seed)
{
    std::mt19937 rng(seed);
    std::uniform_int_distribution<uint32_t> dist(0, max);
    for (std::size_t i = 0; i < n; ++i) out[i] = dist(rng);
}

// main.cpp:297-300: uniform_real_distribution<float>(lo, hi) over mt19937(seed)
void orc_random_floats(float* out, std::size_t n, float lo, float hi, unsigned seed)
{
    std::mt19937 rng(seed);
    std::uniform_real_distribution<float> dist(lo, hi);
    for (std::size_t i = 0; i < n; ++i) out[i] = dist(rng);
}

// ---- ground truth --------------------------------------------------------

// kind: 0 unsigned, 1 signed, 2 float. vals may be null.
void orc_std_sort(void* keys, uint32_t* vals, std::size_t n, int key_bytes, int kind, int desc)
{
    if (key_bytes == 4) std_sort_pairs<uint32_t>(static_cast<uint32_t*>(keys), vals, n, kind, desc);
    else std_sort_pairs<uint64_t>(static_cast<uint64_t*>(keys), vals, n, kind, desc);
}

void orc_std_scan(const void* in, void* out, std::size_t n, int type, int op, const void* identity, int exclusive)
{
    by_type(type, [&](auto tag) {
        using T = decltype(tag);
        T id;
        std::memcpy(&id, identity, sizeof(T));
        std_scan<T>(static_cast<const T*>(in), static_cast<T*>(out), n, op, id, exclusive);
    });
}

// Sequential fold: op(init, in[0] op ... op in[n-1]).
void orc_std_reduce(const void* in, std::size_t n, int type, int op, const void* identity, const void* init,
                    void* result)
{
    by_type(type, [&](auto tag) {
        using T = decltype(tag);
        T id, ini;
        std::memcpy(&id, identity, sizeof(T));
        std::memcpy(&ini, init, sizeof(T));
        const T* p = static_cast<const T*>(in);
        T acc = id;
        for (std::size_t i = 0; i < n; ++i) acc = wrap_apply<T>(op, acc, p[i]);
        const T r = n == 0 ? ini : wrap_apply<T>(op, ini, acc);
        std::memcpy(result, &r, sizeof(T));
    });
}

// Exact 64-bit sum of 32-bit integers (the scan's wide total).
long long orc_sum_i32(const int32_t* in, std::size_t n)
{
    long long s = 0;
    for (std::size_t i = 0; i < n; ++i) s += in[i];
    return s;
}

void orc_histogram_even(const void* in, std::size_t n, int type, uint32_t* hist, std::size_t bins, double lower,
                        double upper, int threads)
{
    by_type(type, [&](auto tag) {
        using T = decltype(tag);
        histogram_even<T>(static_cast<const T*>(in), n, hist, bins, lower, upper, threads);
    });
}

// ---- restated reference algorithms ---------------------------------------

void orc_ref_radix_sort(void* keys, uint32_t* vals, std::size_t n, int key_bytes, int kind, int desc, int threads)
{
    if (key_bytes == 4) ref_radix_sort<uint32_t>(static_cast<uint32_t*>(keys), vals, n, kind, desc, threads);
    else ref_radix_sort<uint64_t>(static_cast<uint64_t*>(keys), vals, n, kind, desc, threads);
}

void orc_ref_scan(const void* in, void* out, std::size_t n, int type, int op, const void* identity, int exclusive,
                  int threads)
{
    by_type(type, [&](auto tag) {
        using T = decltype(tag);
        T id;
        std::memcpy(&id, identity, sizeof(T));
        ref_scan<T>(static_cast<const T*>(in), static_cast<T*>(out), n, op, id, exclusive, threads);
    });
}

void orc_ref_reduce(const void* in, std::size_t n, int type, int op, const void* identity, const void* init,
                    void* result, int threads)
{
    by_type(type, [&](auto tag) {
        using T = decltype(tag);
        T id, ini;
        std::memcpy(&id, identity, sizeof(T));
        std::memcpy(&ini, init, sizeof(T));
        const T r = ref_reduce<T>(static_cast<const T*>(in), n, op, id, ini, threads);
        std::memcpy(result, &r, sizeof(T));
    });
}

int orc_hardware_threads(void) { return hw_threads(0); }

// ---- learned-CDF network (no reference counterpart) -----------------------
// 1 -> H -> H -> 1 on a key u (order-preserving u32 domain):
//   d_j = (u - c_j) * inv_span, h1_j = clamp(w1_j d_j + b1_j, 0, 1),
//   h2_k = clamp(b2_k + sum_j w2_kj h1_j, 0, 1), yhat = b3 + sum_k w3_k h2_k,
// weights stored as v with w = exp(v); loss = mean of (yhat - y)^2. Gradient
// with respect to the raw parameters, in double (clamp' = 1 strictly inside
// (0, 1)). Layout: v1[H], b1[H], v2[H][H] (row = output unit), b2[H], v3[H], b3.
void orc_mlp_grad(const float* params, const uint32_t* centres, float inv_span, const uint32_t* keys,
                  const float* ys, std::size_t m, int h, float* grad, double* loss)
{
    const int H = h;
    const int OV1 = 0, OB1 = H, OV2 = 2 * H, OB2 = 2 * H + H * H, OV3 = 3 * H + H * H, OB3 = 4 * H + H * H;
    const int NP = OB3 + 1;
    auto is_w = [&](int i) { return i < OB1 || (i >= OV2 && i < OB2) || (i >= OV3 && i < OB3); };
    std::vector<double> w(NP), g(NP, 0.0);
    for (int i = 0; i < NP; ++i) w[i] = is_w(i) ? std::exp((double)params[i]) : (double)params[i];
    double l = 0;
    std::vector<double> d(H), z1(H), h1(H), z2(H), h2(H), d2(H);
    auto inside = [](double z) { return z > 0 && z < 1; };
    auto clamp01 = [](double z) { return z < 0 ? 0.0 : (z > 1 ? 1.0 : z); };
    for (std::size_t p = 0; p < m; ++p) {
        for (int j = 0; j < H; ++j) {
            d[j] = (double)((int64_t)keys[p] - (int64_t)centres[j]) * (double)inv_span;
            z1[j] = w[OV1 + j] * d[j] + w[OB1 + j];
            h1[j] = clamp01(z1[j]);
        }
        double yhat = w[OB3];
        for (int k = 0; k < H; ++k) {
            double z = w[OB2 + k];
            for (int j = 0; j < H; ++j) z += w[OV2 + k * H + j] * h1[j];
            z2[k] = z;
            h2[k] = clamp01(z);
            yhat += w[OV3 + k] * h2[k];
        }
        const double err = yhat - ys[p];
        l += err * err;
        const double gy = 2 * err / (double)m;
        g[OB3] += gy;
        for (int k = 0; k < H; ++k) {
            g[OV3 + k] += gy * h2[k];
            d2[k] = inside(z2[k]) ? gy * w[OV3 + k] : 0;
            g[OB2 + k] += d2[k];
            for (int j = 0; j < H; ++j) g[OV2 + k * H + j] += d2[k] * h1[j];
        }
        for (int j = 0; j < H; ++j) {
            double s = 0;
            for (int k = 0; k < H; ++k) s += d2[k] * w[OV2 + k * H + j];
            const double d1 = inside(z1[j]) ? s : 0;
            g[OV1 + j] += d1 * d[j];
            g[OB1 + j] += d1;
        }
    }
    for (int i = 0; i < NP; ++i) grad[i] = (float)(is_w(i) ? g[i] * w[i] : g[i]);
    *loss = l / (double)m;
}

// ---- batched forms (no reference counterpart; std:: ground truth) ---------

// Every segment [off[i], off[i+1]) sorted independently, stably.
void orc_std_segmented_sort(void* keys, uint32_t* vals, std::size_t n, int key_bytes, int kind, int desc,
                            const uint32_t* off, std::size_t nseg, int threads)
{
    (void)n;
    parallel_for(nseg, hw_threads(threads), [&](std::size_t s0, std::size_t s1) {
        for (std::size_t s = s0; s < s1; ++s) {
            const std::size_t b = off[s], len = off[s + 1] - off[s];
            if (key_bytes == 4)
                std_sort_pairs<uint32_t>(static_cast<uint32_t*>(keys) + b, vals ? vals + b : nullptr, len, kind,
                                         desc);
            else
                std_sort_pairs<uint64_t>(static_cast<uint64_t*>(keys) + b, vals ? vals + b : nullptr, len, kind,
                                         desc);
        }
    });
}

// Scan restarted at position 0 and at every off[i] (i < nseg).
void orc_std_segmented_scan(const void* in, void* out, std::size_t n, int type, int op, const void* identity,
                            int exclusive, const uint32_t* off, std::size_t nseg)
{
    std::vector<char> head(n, 0);
    if (n) head[0] = 1;
    for (std::size_t i = 0; i < nseg; ++i)
        if (off[i] < n) head[off[i]] = 1;
    by_type(type, [&](auto tag) {
        using T = decltype(tag);
        T id;
        std::memcpy(&id, identity, sizeof(T));
        const T* p = static_cast<const T*>(in);
        T* o = static_cast<T*>(out);
        T run = id;
        for (std::size_t i = 0; i < n; ++i) {
            if (head[i]) run = id;
            const T next = head[i] ? p[i] : wrap_apply<T>(op, run, p[i]);
            o[i] = exclusive ? (head[i] ? id : run) : next;
            run = next;
        }
    });
}

}  // extern "C"

extern "C" {
// Runs of equal adjacent keys: key, uint64 sum of values, length; histogram of
// the low 16 key bits (65536 bins). Returns the number of runs.
std::size_t orc_std_reduce_by_key(const void* keys, int key_bytes, const uint32_t* vals, std::size_t n,
                                  void* keys_out, unsigned long long* sums, uint32_t* counts, uint32_t* hist)
{
    auto key = [&](std::size_t i) -> uint64_t {
        return key_bytes == 4 ? static_cast<const uint32_t*>(keys)[i] : static_cast<const uint64_t*>(keys)[i];
    };
    std::fill(hist, hist + 65536, 0u);
    std::size_t r = 0;
    for (std::size_t i = 0; i < n;) {
        std::size_t j = i;
        unsigned long long s = 0;
        while (j < n && key(j) == key(i)) s += vals[j++];
        if (key_bytes == 4) static_cast<uint32_t*>(keys_out)[r] = (uint32_t)key(i);
        else static_cast<uint64_t*>(keys_out)[r] = key(i);
        sums[r] = s;
        counts[r] = (uint32_t)(j - i);
        hist[key(i) & 0xFFFF] += (uint32_t)(j - i);
        ++r;
        i = j;
    }
    return r;
}
}

// ---- bitpack compression (restated from lib/src/Compute/Compression.cpp) ----
// Chunk format of Compression.cpp:19-24, 88-106: for every chunk of `chunk`
// elements three words {base, width, offset of the packed words relative to
// the packed area}, then the packed area; a chunk's values are stored as
// (encoded value - base) in `width` bits each, least significant bits first,
// element j at bit j * width of the chunk's words. width = 32 - clz(max -
// min) of the encoded values (0 when they are all equal). Delta mode encodes
// zigzag(x[i] - x[i-1]) with wrapping 32-bit arithmetic and x[-1] = 0
// (Compression.cpp:30-37); decoding undoes the zigzag and takes a wrapping
// inclusive prefix sum over the whole array (Compression.cpp:121-123, 178).
namespace {
uint32_t bp_encode(const uint32_t* in, std::size_t i, int delta)
{
    if (!delta) return in[i];
    const uint32_t d = in[i] - (i > 0 ? in[i - 1] : 0u);
    return (d << 1) ^ (0u - (d >> 31));
}
}  // namespace

extern "C" {
// Writes the compressed words into out (when not null); returns their count.
std::size_t orc_bitpack_compress(const uint32_t* in, std::size_t n, std::size_t chunk, int delta, uint32_t* out)
{
    if (n == 0) return 0;
    const std::size_t chunks = (n + chunk - 1) / chunk;
    std::vector<uint32_t> base(chunks), width(chunks), offset(chunks);
    std::size_t packed = 0;
    for (std::size_t c = 0; c < chunks; ++c) {
        const std::size_t b = c * chunk, e = std::min(n, b + chunk);
        uint32_t lo = 0xFFFFFFFFu, hi = 0;
        for (std::size_t i = b; i < e; ++i) {
            const uint32_t v = bp_encode(in, i, delta);
            lo = std::min(lo, v);
            hi = std::max(hi, v);
        }
        const uint32_t range = hi - lo;
        uint32_t w = 0;
        while (w < 32 && (range >> w) != 0) ++w;  // 32 - clz(range), 0 for range 0
        base[c] = lo;
        width[c] = w;
        offset[c] = (uint32_t)packed;
        packed += ((e - b) * w + 31) / 32;
    }
    const std::size_t total = 3 * chunks + packed;
    if (out == nullptr) return total;
    std::fill(out, out + total, 0u);
    for (std::size_t c = 0; c < chunks; ++c) {
        out[3 * c] = base[c];
        out[3 * c + 1] = width[c];
        out[3 * c + 2] = offset[c];
        const uint32_t w = width[c];
        if (w == 0) continue;
        uint32_t* words = out + 3 * chunks + offset[c];
        const std::size_t b = c * chunk, e = std::min(n, b + chunk);
        for (std::size_t i = b; i < e; ++i) {
            const uint64_t v = bp_encode(in, i, delta) - base[c];
            const uint64_t bit = (uint64_t)(i - b) * w;
            const uint64_t bits = v << (bit & 31);
            words[bit >> 5] |= (uint32_t)bits;
            if ((bit & 31) + w > 32) words[(bit >> 5) + 1] |= (uint32_t)(bits >> 32);
        }
    }
    return total;
}

// Decodes n elements from data (`words` words); returns 0, or -1 when a
// chunk header points outside the data.
int orc_bitpack_decompress(const uint32_t* data, std::size_t words, std::size_t n, std::size_t chunk, int delta,
                           uint32_t* out)
{
    if (n == 0) return 0;
    const std::size_t chunks = (n + chunk - 1) / chunk;
    if (words < 3 * chunks) return -1;
    const std::size_t packed = words - 3 * chunks;
    uint32_t run = 0;
    for (std::size_t c = 0; c < chunks; ++c) {
        const uint32_t base = data[3 * c], w = data[3 * c + 1], off = data[3 * c + 2];
        const std::size_t b = c * chunk, e = std::min(n, b + chunk);
        if (w > 32 || (uint64_t)off + ((e - b) * (uint64_t)w + 31) / 32 > packed) return -1;
        const uint32_t* p = data + 3 * chunks + off;
        for (std::size_t i = b; i < e; ++i) {
            uint32_t v = 0;
            if (w != 0) {
                const uint64_t bit = (uint64_t)(i - b) * w;
                uint64_t both = p[bit >> 5];
                if ((bit & 31) + w > 32) both |= (uint64_t)p[(bit >> 5) + 1] << 32;
                v = (uint32_t)((both >> (bit & 31)) & (w == 32 ? 0xFFFFFFFFull : ((1ull << w) - 1)));
            }
            v += base;
            if (delta) {
                run += (v >> 1) ^ (0u - (v & 1u));
                out[i] = run;
            } else {
                out[i] = v;
            }
        }
    }
    return 0;
}
}  // extern "C"
