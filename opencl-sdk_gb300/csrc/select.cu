// copy_if: out gets, in order, the elements of in that satisfy a predicate;
// returns how many.
//
// Reference path replaced: detail::copy_if (lib/src/Compute/Algorithm.cpp:
// 529-567) with its kernels clc_select_flags / clc_select_scatter (216-237):
// `flags[i] = (PRED) ? 1u : 0u`, an exclusive scan of the flags into
// positions, a scatter pass, then a blocking read of the last position and
// flag. The reference compiles the predicate as OpenCL C over `x`; here it is
// compiled on the host from the expression subset that transform uses
// (xp::compile_predicate: the expression's truth value in its own type) and
// run by the shared interpreter (interp.cuh).
//
// Three streaming passes, each warp working alone on its part of a tile (no
// CTA barrier): evaluate the predicate, store the warp's keep masks (one bit
// per element) and its count of kept elements; the library's scan turns the
// counts into offsets and their exact total; read the part and its masks
// again, compact the kept elements in the warp's shared memory and write
// them as one run at the warp's offset.
// Each thread runs the program over RUN elements at a time, so an
// operation's dispatch is shared by RUN elements. (Measured on
// GB300, 2^30 int32 "x > 0": a single-pass form with a decoupled look-back
// and a per-element evaluator of a fixed grammar took 3.25 ms; the evaluator,
// not the look-back, was the cost.)
#include <cstring>

#include "device_common.cuh"
#include "interp.cuh"
#include "select.hpp"

namespace gbc {
namespace {

using namespace xp;
using namespace xp::interp;
using dev::FULL_MASK;

constexpr int THREADS = 256;
constexpr int WARPS = THREADS / 32;

// Elements of SZ bytes; each thread holds ITEMS of them as ROWS rows of V =
// 16 / SZ (one 128-bit access per row). Row r of warp w covers tile elements
// (w * ROWS + r) * 32 V + lane V + q, q < V; the thread's element j = r V + q.
// All of a thread's loads are issued first; the predicate then runs over
// RUN elements at a time (fewer registers than all ITEMS at once).
template <int SZ> struct SelShape {
    static constexpr int ITEMS = SZ == 8 ? 8 : 16;
    static constexpr int RUN = 8;
    static constexpr int V = 16 / SZ;
    static constexpr int ROWS = ITEMS / V;
    static constexpr int TILE = THREADS * ITEMS;
    static constexpr int WARP_ELEMS = ROWS * 32 * V;
    static constexpr int WORDS = ITEMS * SZ / 4;  // 32-bit words per thread
    static_assert(ITEMS % RUN == 0 && ITEMS <= 32, "whole runs; one mask word per lane");
};

struct SelArgs {
    const unsigned char* in;
    unsigned char* out;
    uint32_t n;
    uint32_t* tiles;  // per tile and warp: kept elements (count pass), then their exclusive offsets
    uint32_t* masks;  // per tile and warp: ITEMS keep masks (count pass), read by the scatter pass
};

template <int SZ, int WORDS>
__device__ __forceinline__ uint64_t raw_elem(const uint32_t (&w)[WORDS], int j)
{
    if constexpr (SZ == 1) return (w[j / 4] >> (8 * (j % 4))) & 0xFFu;
    else if constexpr (SZ == 2) return (w[j / 2] >> (16 * (j % 2))) & 0xFFFFu;
    else if constexpr (SZ == 4) return w[j];
    else return ((uint64_t)w[2 * j + 1] << 32) | w[2 * j];
}

// The thread's elements as raw words; elements past n are 0 (the callers
// flag them out).
template <int SZ>
__device__ __forceinline__ void load_raw(const SelArgs& a, uint32_t wbase, int lane, uint32_t (&w)[SelShape<SZ>::WORDS])
{
    using S = SelShape<SZ>;
    if (((reinterpret_cast<uintptr_t>(a.in) & 15) == 0) && wbase + S::WARP_ELEMS <= a.n) {
#pragma unroll
        for (int r = 0; r < S::ROWS; ++r) {
            const uint4 u = dev::ld_stream(
                reinterpret_cast<const uint4*>(a.in + ((std::size_t)wbase + (r * 32 + lane) * S::V) * SZ));
            w[4 * r] = u.x, w[4 * r + 1] = u.y, w[4 * r + 2] = u.z, w[4 * r + 3] = u.w;
        }
        return;
    }
#pragma unroll
    for (int k = 0; k < S::WORDS; ++k) w[k] = 0;
#pragma unroll
    for (int r = 0; r < S::ROWS; ++r)
#pragma unroll
        for (int q = 0; q < S::V; ++q) {
            const uint32_t idx = wbase + (r * 32 + lane) * S::V + q;
            if (idx < a.n) {
                const unsigned char* s = a.in + (std::size_t)idx * SZ;
                const int j = r * S::V + q;
                if constexpr (SZ == 1) w[j / 4] |= (uint32_t)*s << (8 * (j % 4));
                else if constexpr (SZ == 2) w[j / 2] |= (uint32_t)*reinterpret_cast<const uint16_t*>(s) << (16 * (j % 2));
                else if constexpr (SZ == 4) w[j] = *reinterpret_cast<const uint32_t*>(s);
                else {
                    const uint64_t v = *reinterpret_cast<const uint64_t*>(s);
                    w[2 * j] = (uint32_t)v;
                    w[2 * j + 1] = (uint32_t)(v >> 32);
                }
            }
        }
}

// Elements first .. first + RUN - 1 of the thread, promoted to the program's
// registers (char and short sign-extended, unsigned narrow types zero-extended).
template <int SZ, typename W, int FIRST>
__device__ __forceinline__ void promote_run(uint8_t e, const uint32_t (&w)[SelShape<SZ>::WORDS],
                                            W (&xv)[SelShape<SZ>::RUN])
{
    using S = SelShape<SZ>;
    if constexpr (SZ >= 4) {
#pragma unroll
        for (int i = 0; i < S::RUN; ++i) xv[i] = (W)raw_elem<SZ, S::WORDS>(w, FIRST + i);
    } else if (e == (uint8_t)elem::i8 || e == (uint8_t)elem::i16) {
#pragma unroll
        for (int i = 0; i < S::RUN; ++i) {
            const uint32_t r = (uint32_t)raw_elem<SZ, S::WORDS>(w, FIRST + i);
            xv[i] = put<W>(SZ == 1 ? (int32_t)(int8_t)(uint8_t)r : (int32_t)(int16_t)(uint16_t)r);
        }
    } else {
#pragma unroll
        for (int i = 0; i < S::RUN; ++i) xv[i] = (W)raw_elem<SZ, S::WORDS>(w, FIRST + i);
    }
}

// The program over elements FIRST .. FIRST + RUN - 1; a ballot per element
// slot; lane j keeps slot j's mask.
template <int SZ, typename W, bool STK, int FIRST>
__device__ __forceinline__ void flag_run(const program& p, const uint32_t (&w)[SelShape<SZ>::WORDS], W* st,
                                         uint32_t wbase, uint32_t n, bool whole, int lane, uint32_t& count,
                                         uint32_t& mine)
{
    using S = SelShape<SZ>;
    W xv[S::RUN], acc[S::RUN];
    promote_run<SZ, W, FIRST>(p.x_elem, w, xv);
    run_program<W, S::RUN, STK, THREADS>(p, acc, xv, xv, st);
#pragma unroll
    for (int i = 0; i < S::RUN; ++i) {
        const int j = FIRST + i;
        const bool keep = (uint32_t)acc[i] != 0u && (whole || wbase + ((j / S::V) * 32 + lane) * S::V + j % S::V < n);
        const uint32_t m = __ballot_sync(FULL_MASK, keep);
        count += __popc(m);
        if (lane == j) mine = m;
    }
}

// Pass 1, per warp (no CTA barrier): the keep masks of the warp's ITEMS
// element slots, stored for pass 3 (which then evaluates nothing), and its
// count of kept elements.
template <int SZ, typename W, bool STK>
__global__ void __launch_bounds__(THREADS) k_sel_count(SelArgs a, const __grid_constant__ program p)
{
    using S = SelShape<SZ>;
    extern __shared__ __align__(16) unsigned char sel_smem[];  // STK: the program's stack slots
    W* st = reinterpret_cast<W*>(sel_smem);
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const uint32_t t = blockIdx.x;
    const uint32_t wbase = t * S::TILE + warp * S::WARP_ELEMS;
    uint32_t w[S::WORDS];
    load_raw<SZ>(a, wbase, lane, w);
    const bool whole = wbase + S::WARP_ELEMS <= a.n;
    uint32_t count = 0, mine = 0;
    flag_run<SZ, W, STK, 0>(p, w, st, wbase, a.n, whole, lane, count, mine);
    if constexpr (S::ITEMS > S::RUN) flag_run<SZ, W, STK, S::RUN>(p, w, st, wbase, a.n, whole, lane, count, mine);
    const std::size_t wi = (std::size_t)t * WARPS + warp;
    if (lane < S::ITEMS) a.masks[wi * S::ITEMS + lane] = mine;
    if (lane == 0) a.tiles[wi] = count;
}

// Pass 1 for the commonest predicates, `x OP literal` on 4-byte elements
// (OP a comparison, the literal in x's own type: the program is a load of x
// and one comparison with an immediate), with the comparison inlined instead
// of interpreted: the interpreter's dispatch made the pass issue-bound (0.73
// warp instructions per element for "x > 0"). Same masks and counts.
template <typename T, int CMP> __device__ __forceinline__ bool compare(T x, T c)
{
    if constexpr (CMP == K_LT) return x < c;
    else if constexpr (CMP == K_LE) return x <= c;
    else if constexpr (CMP == K_GT) return x > c;
    else if constexpr (CMP == K_GE) return x >= c;
    else if constexpr (CMP == K_EQ) return x == c;
    else return x != c;
}

template <typename T, int CMP>
__global__ void __launch_bounds__(THREADS) k_sel_count_cmp(SelArgs a, T imm)
{
    using S = SelShape<4>;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const uint32_t t = blockIdx.x;
    const uint32_t wbase = t * S::TILE + warp * S::WARP_ELEMS;
    uint32_t w[S::WORDS];
    load_raw<4>(a, wbase, lane, w);
    const bool whole = wbase + S::WARP_ELEMS <= a.n;
    uint32_t count = 0, mine = 0;
#pragma unroll
    for (int j = 0; j < S::ITEMS; ++j) {
        T x;
        memcpy(&x, &w[j], 4);
        const bool keep = compare<T, CMP>(x, imm) && (whole || wbase + ((j / S::V) * 32 + lane) * S::V + j % S::V < a.n);
        const uint32_t m = __ballot_sync(FULL_MASK, keep);
        count += __popc(m);
        if (lane == j) mine = m;
    }
    const std::size_t wi = (std::size_t)t * WARPS + warp;
    if (lane < S::ITEMS) a.masks[wi * S::ITEMS + lane] = mine;
    if (lane == 0) a.tiles[wi] = count;
}

// The comparison kind when the program is `load x; compare with an immediate
// of x's type` over a 4-byte element type, else -1.
int simple_compare(const program& p)
{
    if (p.nops != 2) return -1;
    const op& l = p.ops[0];
    const op& c = p.ops[1];
    if (l.kind != K_LOAD || l.src != S_X || l.t != p.x_ty) return -1;
    if (c.kind < K_LT || c.kind > K_NE || c.src != S_IMM || c.t != p.x_ty) return -1;
    if (p.x_ty != I32 && p.x_ty != U32 && p.x_ty != F32) return -1;
    return c.kind;
}

template <typename T>
void launch_count_cmp(device_context& ctx, const SelArgs& a, uint32_t num_tiles, int kind, uint64_t imm_bits)
{
    T imm;
    const uint32_t b = (uint32_t)imm_bits;
    memcpy(&imm, &b, 4);
    switch (kind) {
    case K_LT: k_sel_count_cmp<T, K_LT><<<num_tiles, THREADS, 0, ctx.stream>>>(a, imm); break;
    case K_LE: k_sel_count_cmp<T, K_LE><<<num_tiles, THREADS, 0, ctx.stream>>>(a, imm); break;
    case K_GT: k_sel_count_cmp<T, K_GT><<<num_tiles, THREADS, 0, ctx.stream>>>(a, imm); break;
    case K_GE: k_sel_count_cmp<T, K_GE><<<num_tiles, THREADS, 0, ctx.stream>>>(a, imm); break;
    case K_EQ: k_sel_count_cmp<T, K_EQ><<<num_tiles, THREADS, 0, ctx.stream>>>(a, imm); break;
    default: k_sel_count_cmp<T, K_NE><<<num_tiles, THREADS, 0, ctx.stream>>>(a, imm); break;
    }
}

// Pass 3 (after the exclusive scan of the warp counts), per warp: an
// element's place among the warp's kept ones is the kept elements of earlier
// rows, of lower lanes in its row (sum over the slots of popc(mask & lower
// lanes)) and of its own earlier slots; the warp compacts its kept elements
// in its part of shared memory and writes them as one run at its offset.
template <int SZ>
__global__ void __launch_bounds__(THREADS) k_sel_scatter(SelArgs a)
{
    using S = SelShape<SZ>;
    __shared__ __align__(16) unsigned char s_out[WARPS][S::WARP_ELEMS * SZ];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const uint32_t lt_mask = dev::lanemask_lt();
    const uint32_t t = blockIdx.x;
    const uint32_t wbase = t * S::TILE + warp * S::WARP_ELEMS;
    const std::size_t wi = (std::size_t)t * WARPS + warp;
    const uint32_t mword = lane < S::ITEMS ? a.masks[wi * S::ITEMS + lane] : 0u;
    const uint32_t base = a.tiles[wi];
    uint32_t w[S::WORDS];
    load_raw<SZ>(a, wbase, lane, w);
    unsigned char* so = s_out[warp];
    uint32_t pos = 0;
#pragma unroll
    for (int r = 0; r < S::ROWS; ++r) {
        uint32_t m[S::V], below = 0, row_total = 0;
#pragma unroll
        for (int q = 0; q < S::V; ++q) {
            m[q] = __shfl_sync(FULL_MASK, mword, r * S::V + q);
            below += __popc(m[q] & lt_mask);
            row_total += __popc(m[q]);
        }
        uint32_t o = pos + below;
#pragma unroll
        for (int q = 0; q < S::V; ++q)
            if ((m[q] >> lane) & 1u) {
                const uint64_t v = raw_elem<SZ, S::WORDS>(w, r * S::V + q);
                unsigned char* d = so + (std::size_t)o * SZ;
                if constexpr (SZ == 1) *d = (uint8_t)v;
                else if constexpr (SZ == 2) *reinterpret_cast<uint16_t*>(d) = (uint16_t)v;
                else if constexpr (SZ == 4) *reinterpret_cast<uint32_t*>(d) = (uint32_t)v;
                else *reinterpret_cast<uint64_t*>(d) = v;
                ++o;
            }
        pos += row_total;
    }
    __syncwarp();
    for (uint32_t i = lane; i < pos; i += 32) {
        if (base + i >= a.n) break;
        const unsigned char* s = so + (std::size_t)i * SZ;
        unsigned char* d = a.out + ((std::size_t)base + i) * SZ;
        if constexpr (SZ == 1) *d = *s;
        else if constexpr (SZ == 2) *reinterpret_cast<uint16_t*>(d) = *reinterpret_cast<const uint16_t*>(s);
        else if constexpr (SZ == 4) *reinterpret_cast<uint32_t*>(d) = *reinterpret_cast<const uint32_t*>(s);
        else *reinterpret_cast<uint64_t*>(d) = *reinterpret_cast<const uint64_t*>(s);
    }
}

template <int SZ, typename W, bool STK>
void run_select(device_context& ctx, const SelArgs& a0, const program& p, unsigned long long* total)
{
    using S = SelShape<SZ>;
    SelArgs a = a0;
    const uint32_t num_tiles = (a.n + S::TILE - 1) / S::TILE;
    const std::size_t slot_bytes = STK ? (std::size_t)STACK * S::RUN * THREADS * sizeof(W) : 0;
    if (first_use_on_device((const void*)&k_sel_count<SZ, W, STK>))
        check_cuda(cudaFuncSetAttribute(&k_sel_count<SZ, W, STK>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        (int)slot_bytes),
                   "cudaFuncSetAttribute");
    temp_buffer tiles(ctx.resource, (std::size_t)num_tiles * WARPS * sizeof(uint32_t));
    temp_buffer masks(ctx.resource, (std::size_t)num_tiles * WARPS * S::ITEMS * sizeof(uint32_t));
    a.tiles = tiles.as<uint32_t>();
    a.masks = masks.as<uint32_t>();
    {
        kernel_timer kt(ctx, "select.count");
        const int cmp = SZ == 4 ? simple_compare(p) : -1;
        if (cmp < 0)
            k_sel_count<SZ, W, STK><<<num_tiles, THREADS, slot_bytes, ctx.stream>>>(a, p);
        else if (p.x_ty == I32)
            launch_count_cmp<int32_t>(ctx, a, num_tiles, cmp, p.ops[1].imm);
        else if (p.x_ty == U32)
            launch_count_cmp<uint32_t>(ctx, a, num_tiles, cmp, p.ops[1].imm);
        else
            launch_count_cmp<float>(ctx, a, num_tiles, cmp, p.ops[1].imm);
        check_cuda(cudaGetLastError(), "copy_if count launch");
    }
    const uint32_t zero = 0;
    scan(ctx, a.tiles, a.tiles, (std::size_t)num_tiles * WARPS, elem::u32, op_kind::plus, &zero, true, total);
    {
        kernel_timer kt(ctx, "select.scatter");
        k_sel_scatter<SZ><<<num_tiles, THREADS, 0, ctx.stream>>>(a);
        check_cuda(cudaGetLastError(), "copy_if scatter launch");
    }
}

template <int SZ>
void dispatch(device_context& ctx, const SelArgs& a, const program& p, unsigned long long* total)
{
    const bool stk = uses_stack(p);
    if constexpr (SZ == 8) {
        if (stk) run_select<SZ, uint64_t, true>(ctx, a, p, total);
        else run_select<SZ, uint64_t, false>(ctx, a, p, total);
    } else {
        if (all_32bit(p)) {
            if (stk) run_select<SZ, uint32_t, true>(ctx, a, p, total);
            else run_select<SZ, uint32_t, false>(ctx, a, p, total);
        } else {
            if (stk) run_select<SZ, uint64_t, true>(ctx, a, p, total);
            else run_select<SZ, uint64_t, false>(ctx, a, p, total);
        }
    }
}

}  // namespace

std::size_t copy_if(device_context& ctx, const void* in, void* out, std::size_t n, elem t, const program& p)
{
    if (n == 0) return 0;
    check_size(n);
    if (in == nullptr || out == nullptr) throw std::invalid_argument("copy_if: null argument");
    if (in == out) throw std::invalid_argument("copy_if: in and out must differ");
    if (p.nops == 0 || p.nops > (uint32_t)MAX_OPS || p.x_elem != (uint8_t)t)
        throw std::invalid_argument("copy_if: the predicate was compiled for another element type");
    ctx.activate();
    auto* total = reinterpret_cast<unsigned long long*>(ctx.d_small + 2048 + 16);  // exact sum of the tile counts
    SelArgs a;
    a.in = static_cast<const unsigned char*>(in);
    a.out = static_cast<unsigned char*>(out);
    a.n = (uint32_t)n;
    a.tiles = nullptr;
    a.masks = nullptr;
    switch (elem_size(t)) {
    case 1: dispatch<1>(ctx, a, p, total); break;
    case 2: dispatch<2>(ctx, a, p, total); break;
    case 4: dispatch<4>(ctx, a, p, total); break;
    default: dispatch<8>(ctx, a, p, total); break;
    }
    check_cuda(cudaMemcpyAsync(ctx.pinned, total, 8, cudaMemcpyDeviceToHost, ctx.stream), "cudaMemcpyAsync");
    ctx.finish();
    unsigned long long r = 0;
    std::memcpy(&r, ctx.pinned, 8);
    return (std::size_t)r;
}

}  // namespace gbc
