// copy_if: out gets, in order, the elements of in that satisfy a predicate;
// returns how many.
//
// Reference path replaced: detail::copy_if (lib/src/Compute/Algorithm.cpp:
// 529-567) with its kernels clc_select_flags / clc_select_scatter (216-237):
// a flag pass, an exclusive scan of the flags into positions and a scatter
// pass, then a blocking read of the last position and flag. The reference
// compiles the predicate as an OpenCL C expression over x; here it is parsed
// from a fixed grammar (comparisons of x, (x % c) or (x & c) with a constant,
// joined by && or ||) and evaluated with OpenCL C's usual arithmetic
// conversions. One single-pass kernel: each tile counts its kept elements,
// finds the count of all earlier tiles by a decoupled look-back and writes
// its kept elements in order.
#include <cctype>
#include <cmath>
#include <cstring>

#include "device_common.cuh"
#include "select.hpp"
#include "sort_internal.hpp"

namespace gbc {

// ---- predicate grammar ------------------------------------------------------
namespace {

struct lexer {
    const std::string& s;
    std::size_t i = 0;
    void skip()
    {
        while (i < s.size() && std::isspace((unsigned char)s[i])) ++i;
    }
    bool eat(const char* tok)
    {
        skip();
        const std::size_t k = std::strlen(tok);
        if (s.compare(i, k, tok) == 0) {
            i += k;
            return true;
        }
        return false;
    }
    bool done()
    {
        skip();
        return i == s.size();
    }
};

[[noreturn]] void bad(const std::string& text)
{
    throw unsupported_error("copy_if: predicate \"" + text +
                            "\" is outside the supported grammar (comparisons of x, (x % c) or (x & c) with a "
                            "constant, joined by && or ||)");
}

// literal type: 0 int, 1 uint, 2 long, 3 ulong, 4 float, 5 double
struct literal {
    int type = 0;
    int64_t i = 0;
    double f = 0;
};

literal parse_literal(lexer& lx, const std::string& text)
{
    lx.skip();
    const char* b = lx.s.c_str() + lx.i;
    bool neg = false;
    if (*b == '-' || *b == '+') {
        neg = *b == '-';
        ++b;
    }
    const char* p = b;
    literal L;
    bool is_float = false;
    while (std::isdigit((unsigned char)*p) || *p == '.' || *p == 'e' || *p == 'E' ||
           ((*p == '-' || *p == '+') && (p[-1] == 'e' || p[-1] == 'E')) || (*p == 'x' || *p == 'X') ||
           (std::isxdigit((unsigned char)*p) && (b[0] == '0' && (b[1] == 'x' || b[1] == 'X')))) {
        if (*p == '.' || ((*p == 'e' || *p == 'E') && !(b[0] == '0' && (b[1] == 'x' || b[1] == 'X')))) is_float = true;
        ++p;
    }
    if (p == b) bad(text);
    const std::string digits(b, p);
    bool u = false, l = false, f = false;
    while (*p == 'u' || *p == 'U' || *p == 'l' || *p == 'L' || *p == 'f' || *p == 'F') {
        if (*p == 'u' || *p == 'U') u = true;
        else if (*p == 'l' || *p == 'L') l = true;
        else f = true;
        ++p;
    }
    if (std::isalnum((unsigned char)*p) || *p == '_') bad(text);
    lx.i = (std::size_t)(p - lx.s.c_str());
    if (is_float || f) {
        if (u || l) bad(text);
        L.type = f ? 4 : 5;
        L.f = std::strtod(digits.c_str(), nullptr);
        if (f) L.f = (double)(float)L.f;
        if (neg) L.f = -L.f;
        return L;
    }
    errno = 0;
    const unsigned long long v = std::strtoull(digits.c_str(), nullptr, 0);
    if (errno != 0) bad(text);
    // the type of an integer constant: the first of int, uint, long, ulong
    // (decimal without u: int, long) that holds it, as in C
    const bool decimal = !(digits.size() > 1 && digits[0] == '0');
    if (!u && !l && v <= 0x7FFFFFFFull) L.type = 0;
    else if (!l && (u || !decimal) && v <= 0xFFFFFFFFull) L.type = 1;
    else if (!u && v <= 0x7FFFFFFFFFFFFFFFull) L.type = 2;
    else L.type = 3;
    L.i = (int64_t)v;
    if (neg) L.i = -L.i;  // unary minus applies in the literal's type below
    return L;
}

// element type -> operand type after integer promotion
int promoted(elem t)
{
    switch (t) {
    case elem::i8: case elem::u8: case elem::i16: case elem::u16: case elem::i32: return 0;
    case elem::u32: return 1;
    case elem::i64: return 2;
    case elem::u64: return 3;
    case elem::f32: return 4;
    default: return 5;
    }
}

// usual arithmetic conversions for the type codes above
int common(int a, int b)
{
    if (a >= 4 || b >= 4) return std::max(a, b);
    const int ra = a >> 1, rb = b >> 1;  // rank: 0 (32-bit), 1 (64-bit)
    const bool ua = a & 1, ub = b & 1;
    if (ra == rb) return (ra << 1) | (ua || ub);
    const int hi = ra > rb ? a : b, lo = ra > rb ? b : a;
    // the 64-bit type holds every 32-bit value, so signedness follows it
    (void)lo;
    return hi;
}

pred_clause parse_clause(lexer& lx, elem t, const std::string& text)
{
    pred_clause c;
    int lhs_type = promoted(t);
    if (lx.eat("(")) {
        if (!lx.eat("x")) bad(text);
        if (lx.eat("%")) c.lhs = 1;
        else if (lx.eat("&")) c.lhs = 2;
        else bad(text);
        const literal m = parse_literal(lx, text);
        if (!lx.eat(")")) bad(text);
        if (lhs_type >= 4 || m.type >= 4) bad(text);  // % and & need integers
        lhs_type = common(lhs_type, m.type);
        c.m_i = m.i;
        if (c.lhs == 1 && m.i == 0) bad(text);
    } else if (!lx.eat("x")) {
        bad(text);
    }
    if (lx.eat("<=")) c.cmp = 1;
    else if (lx.eat(">=")) c.cmp = 3;
    else if (lx.eat("==")) c.cmp = 4;
    else if (lx.eat("!=")) c.cmp = 5;
    else if (lx.eat("<")) c.cmp = 0;
    else if (lx.eat(">")) c.cmp = 2;
    else bad(text);
    const literal k = parse_literal(lx, text);
    c.ctype = common(lhs_type, k.type);
    c.c_i = k.type >= 4 ? (int64_t)k.f : k.i;
    c.c_f = k.type >= 4 ? k.f : (double)k.i;
    if (k.type < 4 && (k.type & 1) && k.i < 0) c.c_f = (double)(uint64_t)k.i;
    return c;
}

}  // namespace

predicate parse_predicate(const std::string& text, elem t)
{
    lexer lx{text};
    predicate p;
    for (;;) {
        if (p.count == 4) bad(text);
        p.c[p.count++] = parse_clause(lx, t, text);
        if (lx.done()) break;
        const int join = lx.eat("&&") ? 0 : lx.eat("||") ? 1 : -1;
        if (join < 0 || (p.count > 1 && join != p.join)) bad(text);
        p.join = join;
    }
    return p;
}

// ---- device -------------------------------------------------------------------
namespace {

using dev::FULL_MASK;
constexpr int THREADS = 256;
constexpr int LB_PER_LANE = 4;
constexpr uint64_t FLAG_AGG = 1, FLAG_PRE = 2;
constexpr uint64_t TAG_MASK = (1ull << 30) - 1;
constexpr uint64_t SLOTS = onesweep::RING_BYTES / 8;

// A clause flattened for the device: the operand path (0 int32, 1 uint32,
// 2 int64, 3 uint64, 4 double, which is exact for float operands and
// literals), the left side, and the result for each ordering of lhs against
// the constant (less, equal, greater, unordered: NaN), so that no switch on
// the comparison is needed.
struct dclause {
    int kind;
    int lhs;  // 0: x, 1: x % m, 2: x & m
    int64_t m, c;
    double cf;
    bool lt, eq, gt, un;
};
struct dpredicate {
    int count, join;
    dclause c[4];
};

template <typename I, typename T> __device__ __forceinline__ int order_int(T x, const dclause& c)
{
    I v = (I)x;
    if (c.lhs == 1) v = (I)(v % (I)c.m);
    else if (c.lhs == 2) v = (I)(v & (I)c.m);
    const I k = (I)c.c;
    return v < k ? 0 : (v == k ? 1 : 2);
}

// (if-else rather than switch: a jump table costs an indirect branch per
// element and stalls instruction fetch)
template <typename T> __device__ __forceinline__ bool clause_eval(T x, const dclause& c)
{
    int o;
    if (c.kind == 0) o = order_int<int32_t>(x, c);
    else if (c.kind == 1) o = order_int<uint32_t>(x, c);
    else if (c.kind == 2) o = order_int<int64_t>(x, c);
    else if (c.kind == 3) o = order_int<uint64_t>(x, c);
    else {
        const double v = (double)x;
        o = v < c.cf ? 0 : (v == c.cf ? 1 : (v > c.cf ? 2 : 3));
    }
    return o == 0 ? c.lt : (o == 1 ? c.eq : (o == 2 ? c.gt : c.un));
}

template <typename T> __device__ __forceinline__ bool eval(T x, const dpredicate& p)
{
    bool r = clause_eval(x, p.c[0]);
    // unrolled with guards: constant indices keep the clauses in the
    // parameter space (a run-time index would copy them to local memory)
#pragma unroll
    for (int k = 1; k < 4; ++k)
        if (k < p.count) r = p.join ? (r || clause_eval(x, p.c[k])) : (r && clause_eval(x, p.c[k]));
    return r;
}

template <typename T> struct SelArgs {
    const T* in;
    T* out;
    uint32_t n;
    dpredicate p;
    uint32_t num_tiles;
    uint64_t* ring;
    uint64_t seq0;
    uint32_t* tile_ctr;
    uint32_t* total;  // written by the last tile
    int* err;
};

__device__ __forceinline__ void publish(uint64_t* ring, uint64_t seq, uint64_t flag, uint32_t v)
{
    dev::st_relaxed(&ring[seq & (SLOTS - 1)], (flag << 62) | ((seq & TAG_MASK) << 32) | v);
}
__device__ __forceinline__ bool read_status(const uint64_t* ring, uint64_t seq, uint64_t& flag, uint32_t& v)
{
    const uint64_t w = dev::ld_relaxed(&ring[seq & (SLOTS - 1)]);
    flag = w >> 62;
    if (flag == 0 || ((w >> 32) & TAG_MASK) != (seq & TAG_MASK)) return false;
    v = (uint32_t)w;
    return true;
}

// Tile: THREADS x ITEMS elements; warp w owns ROWS = ITEMS / V rows of 32 x V
// consecutive elements (V = 16 / sizeof(T): one 128-bit load per lane and
// row), row r at tile_base + (w * ROWS + r) * 32 V, lane l holding elements
// l V .. l V + V - 1 of the row. A ballot per element slot gives the row's
// keep masks; an element's place among the row's kept ones is the number of
// kept elements in lower lanes (sum over the slots of popc(mask & lower
// lanes)) plus the lane's own kept elements before it. The rows are visited
// by loops that are not unrolled, so the predicate's evaluator appears once
// in the code (unrolled, its copies overflowed the instruction cache).
template <typename T, int ITEMS> __global__ void __launch_bounds__(THREADS) k_copy_if(SelArgs<T> a)
{
    constexpr int WARPS = THREADS / 32;
    constexpr int TILE = THREADS * ITEMS;
    constexpr int V = 16 / sizeof(T);
    constexpr int ROWS = ITEMS / V;
    static_assert(ITEMS % V == 0, "whole 128-bit rows");
    __shared__ __align__(16) T s_in[TILE];
    __shared__ uint32_t s_mask[WARPS * ROWS * V];
    __shared__ uint32_t s_warp[WARPS];
    __shared__ uint32_t s_prefix;
    __shared__ uint32_t s_tile;
    __shared__ dpredicate s_p;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    if (tid == 0) s_p = a.p;
    const uint32_t lt_mask = dev::lanemask_lt();
    const bool aligned = (reinterpret_cast<uintptr_t>(a.in) & 15) == 0;
    for (;;) {
        if (tid == 0) {
            // taken only when the CTA can start on it; the tile a grid ahead
            // is prefetched into L2 (cf. the scan)
            s_tile = atomicAdd(a.tile_ctr, 1u);
            const uint64_t ahead = (uint64_t)s_tile + gridDim.x;
            if (aligned && (ahead + 1) * TILE <= a.n) dev::prefetch_l2(a.in + ahead * TILE, TILE * sizeof(T));
        }
        __syncthreads();
        const uint32_t t = s_tile;
        if (t >= a.num_tiles) break;
        const uint32_t wbase = t * TILE + warp * ROWS * 32 * V;
        T* srow = s_in + warp * ROWS * 32 * V;
        uint32_t count = 0;
#pragma unroll 1
        for (int r = 0; r < ROWS; ++r) {
            const uint32_t first = wbase + (r * 32 + lane) * V;
            T x[V];
            if (aligned && first + V <= a.n) {
                const uint4 w = *reinterpret_cast<const uint4*>(a.in + first);
                memcpy(x, &w, 16);
            } else {
#pragma unroll
                for (int q = 0; q < V; ++q) x[q] = first + q < a.n ? a.in[first + q] : T(0);
            }
            *reinterpret_cast<uint4*>(srow + (r * 32 + lane) * V) = *reinterpret_cast<const uint4*>(x);
#pragma unroll
            for (int q = 0; q < V; ++q) {
                const uint32_t m = __ballot_sync(FULL_MASK, first + q < a.n && eval(x[q], s_p));
                if (lane == 0) s_mask[(warp * ROWS + r) * V + q] = m;
                count += __popc(m);
            }
        }
        if (lane == 0) s_warp[warp] = count;
        __syncthreads();
        if (warp == 0) {
            const uint32_t wv = lane < WARPS ? s_warp[lane] : 0u;
            const uint32_t wi = dev::warp_inclusive_scan(wv, [](uint32_t p, uint32_t q) { return p + q; });
            if (lane < WARPS) s_warp[lane] = wi - wv;
            const uint32_t agg = __shfl_sync(FULL_MASK, wi, 31);
            const uint64_t my_seq = a.seq0 + t;
            if (lane == 0) publish(a.ring, my_seq, t == 0 ? FLAG_PRE : FLAG_AGG, agg);
            uint32_t excl = 0;
            if (t > 0) {
                int64_t w_end = t;
                bool gave_up = false;
                for (;;) {
                    uint64_t flag[LB_PER_LANE];
                    uint32_t val[LB_PER_LANE];
#pragma unroll
                    for (int q = 0; q < LB_PER_LANE; ++q) {
                        const int64_t k = w_end - 32 * LB_PER_LANE + lane * LB_PER_LANE + q;
                        flag[q] = FLAG_PRE;
                        val[q] = 0;
                        if (k >= 0 && !read_status(a.ring, a.seq0 + (uint64_t)k, flag[q], val[q])) {
                            const unsigned long long start = dev::globaltimer();
                            for (uint32_t spin = 1;; ++spin) {
                                if (read_status(a.ring, a.seq0 + (uint64_t)k, flag[q], val[q])) break;
                                if ((spin & 255) == 0 && dev::globaltimer() - start > dev::SPIN_LIMIT_NS) {
                                    gave_up = true;
                                    flag[q] = FLAG_PRE;
                                    val[q] = 0;
                                    break;
                                }
                                if (spin > 32) __nanosleep(64);
                            }
                        }
                    }
                    int hi = -1;
#pragma unroll
                    for (int q = 0; q < LB_PER_LANE; ++q)
                        if (flag[q] == FLAG_PRE) hi = q;
                    const uint32_t pre = __ballot_sync(FULL_MASK, hi >= 0);
                    const int L = pre ? 31 - __clz(pre) : -1;
                    uint32_t contrib = 0;
                    if (lane >= L) {
                        const int q0 = lane == L ? hi : 0;
#pragma unroll
                        for (int q = 0; q < LB_PER_LANE; ++q)
                            if (q >= q0) contrib += val[q];
                    }
                    excl += dev::warp_reduce(contrib, [](uint32_t p, uint32_t q) { return p + q; });
                    if (pre) break;
                    w_end -= 32 * LB_PER_LANE;
                }
                if (__any_sync(FULL_MASK, gave_up) && lane == 0) dev::raise_error(a.err, dev::ERR_LOOKBACK_TIMEOUT);
                if (lane == 0) publish(a.ring, my_seq, FLAG_PRE, excl + agg);
            }
            if (lane == 0) {
                s_prefix = excl;
                if (t == a.num_tiles - 1) *a.total = excl + agg;
            }
        }
        __syncthreads();
        uint32_t pos = s_prefix + s_warp[warp];
#pragma unroll 1
        for (int r = 0; r < ROWS; ++r) {
            uint32_t m[V], below = 0, row_total = 0;
#pragma unroll
            for (int q = 0; q < V; ++q) {
                m[q] = s_mask[(warp * ROWS + r) * V + q];
                below += __popc(m[q] & lt_mask);
                row_total += __popc(m[q]);
            }
            uint32_t o = pos + below;
            const T* src = srow + (r * 32 + lane) * V;
#pragma unroll
            for (int q = 0; q < V; ++q)
                if ((m[q] >> lane) & 1u) {
                    if (o < a.n) a.out[o] = src[q];
                    ++o;
                }
            pos += row_total;
        }
        __syncthreads();
    }
}

template <typename T>
void launch_select(device_context& ctx, const void* in, void* out, uint32_t n, const predicate& p, uint32_t* total)
{
    constexpr int ITEMS = sizeof(T) <= 4 ? 32 : 16;
    constexpr uint32_t TILE = THREADS * ITEMS;
    SelArgs<T> a;
    a.in = static_cast<const T*>(in);
    a.out = static_cast<T*>(out);
    a.n = n;
    a.p.count = p.count;
    a.p.join = p.join;
    for (int k = 0; k < p.count; ++k) {
        const pred_clause& q = p.c[k];
        dclause& d = a.p.c[k];
        d.kind = q.ctype >= 4 ? 4 : q.ctype;
        d.lhs = q.lhs;
        d.m = q.m_i;
        d.c = q.c_i;
        d.cf = q.ctype == 4 ? (double)(float)q.c_f : q.c_f;  // float compare: the constant in float
        d.lt = q.cmp == 0 || q.cmp == 1 || q.cmp == 5;
        d.eq = q.cmp == 1 || q.cmp == 3 || q.cmp == 4;
        d.gt = q.cmp == 2 || q.cmp == 3 || q.cmp == 5;
        d.un = q.cmp == 5;  // only != holds for NaN
    }
    a.num_tiles = (n + TILE - 1) / TILE;
    a.ring = ctx.lookback_ring;
    a.seq0 = ctx.reserve_seq(a.num_tiles);
    unsigned char* ctl = ctx.d_small + 2048;
    check_cuda(cudaMemsetAsync(ctl, 0, 16, ctx.stream), "cudaMemsetAsync");
    a.tile_ctr = reinterpret_cast<uint32_t*>(ctl);
    a.total = total;
    a.err = ctx.d_error;
    int per_sm = 0;
    check_cuda(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, &k_copy_if<T, ITEMS>, THREADS, 0),
               "cudaOccupancyMaxActiveBlocksPerMultiprocessor");
    const int grid = (int)std::min<std::size_t>(a.num_tiles, (std::size_t)ctx.sm_count * std::max(per_sm, 1));
    kernel_timer kt(ctx, "select.copy_if");
    k_copy_if<T, ITEMS><<<grid, THREADS, 0, ctx.stream>>>(a);
    check_cuda(cudaGetLastError(), "copy_if launch");
}

}  // namespace

std::size_t copy_if(device_context& ctx, const void* in, void* out, std::size_t n, elem t, const predicate& p)
{
    if (n == 0) return 0;
    check_size(n);
    if (in == nullptr || out == nullptr) throw std::invalid_argument("copy_if: null argument");
    if (in == out) throw std::invalid_argument("copy_if: in and out must differ");
    ctx.activate();
    uint32_t* total = reinterpret_cast<uint32_t*>(ctx.d_small + 2048 + 16);
    const uint32_t nn = (uint32_t)n;
    switch (t) {
    case elem::i8: launch_select<int8_t>(ctx, in, out, nn, p, total); break;
    case elem::u8: launch_select<uint8_t>(ctx, in, out, nn, p, total); break;
    case elem::i16: launch_select<int16_t>(ctx, in, out, nn, p, total); break;
    case elem::u16: launch_select<uint16_t>(ctx, in, out, nn, p, total); break;
    case elem::i32: launch_select<int32_t>(ctx, in, out, nn, p, total); break;
    case elem::u32: launch_select<uint32_t>(ctx, in, out, nn, p, total); break;
    case elem::i64: launch_select<int64_t>(ctx, in, out, nn, p, total); break;
    case elem::u64: launch_select<uint64_t>(ctx, in, out, nn, p, total); break;
    case elem::f32: launch_select<float>(ctx, in, out, nn, p, total); break;
    case elem::f64: launch_select<double>(ctx, in, out, nn, p, total); break;
    }
    check_cuda(cudaMemcpyAsync(ctx.pinned, total, 4, cudaMemcpyDeviceToHost, ctx.stream), "cudaMemcpyAsync");
    ctx.finish();
    uint32_t r = 0;
    std::memcpy(&r, ctx.pinned, 4);
    return r;
}

}  // namespace gbc
