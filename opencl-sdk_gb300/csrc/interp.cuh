// The element-wise expression interpreter shared by transform and copy_if:
// conversions (host and device, so that literals folded on the host and
// values converted on the device agree bit for bit) and the device
// evaluation of an xp::program over V values held by one thread. The
// program is uniform across the CTA, so every dispatch branch is uniform.
#pragma once

#include <algorithm>
#include <cstddef>
#include <cstdint>
#include <cstring>
#include <limits>
#include <type_traits>

#include "expr.hpp"

namespace gbc {
namespace xp {

// ---------------------------------------------------------------------------
// Conversions, shared by the host (folding literals into immediates) and the
// device (CVT), so both give identical bits. Values travel as raw bits; 32-bit
// types use the low 32 bits.
// ---------------------------------------------------------------------------
namespace cv {

template <typename T> __host__ __device__ __forceinline__ T from_bits(uint64_t r)
{
    T v;
    if constexpr (sizeof(T) == 4) {
        const uint32_t u = (uint32_t)r;
        memcpy(&v, &u, 4);
    } else {
        memcpy(&v, &r, 8);
    }
    return v;
}
template <typename T> __host__ __device__ __forceinline__ uint64_t to_bits(T v)
{
    if constexpr (sizeof(T) == 4) {
        uint32_t u;
        memcpy(&u, &v, 4);
        return u;
    } else {
        uint64_t u;
        memcpy(&u, &v, 8);
        return u;
    }
}

// integer -> floating point, round to nearest even
template <typename F, typename I> __host__ __device__ __forceinline__ F i2f(I v)
{
#ifdef __CUDA_ARCH__
    if constexpr (sizeof(F) == 4) {
        if constexpr (std::is_same<I, int32_t>::value) return __int2float_rn((int)v);
        else if constexpr (std::is_same<I, uint32_t>::value) return __uint2float_rn((unsigned)v);
        else if constexpr (std::is_same<I, int64_t>::value) return __ll2float_rn((long long)v);
        else return __ull2float_rn((unsigned long long)v);
    } else {
        if constexpr (std::is_same<I, int32_t>::value) return __int2double_rn((int)v);
        else if constexpr (std::is_same<I, uint32_t>::value) return __uint2double_rn((unsigned)v);
        else if constexpr (std::is_same<I, int64_t>::value) return __ll2double_rn((long long)v);
        else return __ull2double_rn((unsigned long long)v);
    }
#else
    return (F)v;  // the host's conversions round to nearest even
#endif
}

// floating point -> integer: toward zero, saturating, NaN -> 0. The bounds
// are powers of two, exact in both float and double.
template <typename I, typename F> __host__ __device__ __forceinline__ I f2i(F f)
{
    if (!(f == f)) return 0;
    if constexpr (std::is_signed<I>::value) {
        const F hi = sizeof(I) == 4 ? (F)2147483648.0 : (F)9223372036854775808.0;
        if (f >= hi) return std::numeric_limits<I>::max();
        if (f < -hi) return std::numeric_limits<I>::min();
    } else {
        const F hi = sizeof(I) == 4 ? (F)4294967296.0 : (F)18446744073709551616.0;
        if (!(f > (F)-1.0)) return 0;
        if (f >= hi) return std::numeric_limits<I>::max();
    }
    return (I)f;  // in range: truncation is exact
}

template <typename F> __host__ __device__ __forceinline__ float d2f(F d)
{
#ifdef __CUDA_ARCH__
    return __double2float_rn((double)d);
#else
    return (float)d;
#endif
}

template <typename TO, typename FROM> __host__ __device__ __forceinline__ TO conv(FROM v)
{
    if constexpr (std::is_floating_point<TO>::value) {
        if constexpr (std::is_floating_point<FROM>::value) {
            if constexpr (sizeof(TO) >= sizeof(FROM)) return (TO)v;  // same type, or float -> double: exact
            else return d2f(v);
        } else {
            return i2f<TO>(v);
        }
    } else if constexpr (std::is_floating_point<FROM>::value) {
        return f2i<TO>(v);
    } else {
        return (TO)v;  // integer -> integer: modulo 2^bits (two's complement)
    }
}

template <typename TO> __host__ __device__ __forceinline__ uint64_t conv_from(uint8_t from, uint64_t r)
{
    switch (from) {
    case I32: return to_bits(conv<TO>(from_bits<int32_t>(r)));
    case U32: return to_bits(conv<TO>(from_bits<uint32_t>(r)));
    case I64: return to_bits(conv<TO>(from_bits<int64_t>(r)));
    case U64: return to_bits(conv<TO>(from_bits<uint64_t>(r)));
    case F32: return to_bits(conv<TO>(from_bits<float>(r)));
    default: return to_bits(conv<TO>(from_bits<double>(r)));
    }
}

__host__ __device__ __forceinline__ uint64_t convert(uint8_t from, uint8_t to, uint64_t r)
{
    switch (to) {
    case I32: return conv_from<int32_t>(from, r);
    case U32: return conv_from<uint32_t>(from, r);
    case I64: return conv_from<int64_t>(from, r);
    case U64: return conv_from<uint64_t>(from, r);
    case F32: return conv_from<float>(from, r);
    default: return conv_from<double>(from, r);
    }
}

}  // namespace cv

// ---------------------------------------------------------------------------
// Device interpreter
// ---------------------------------------------------------------------------
namespace interp {

// bytes of an elem code (i8 u8 i16 u16 i32 u32 i64 u64 f32 f64)
__device__ __forceinline__ int elem_size_dev(uint8_t e) { return e <= 1 ? 1 : e <= 3 ? 2 : (e <= 5 || e == 8) ? 4 : 8; }

template <typename T, typename W> __device__ __forceinline__ T get(W r) { return cv::from_bits<T>((uint64_t)r); }
template <typename W, typename T> __device__ __forceinline__ W put(T v) { return (W)cv::to_bits(v); }

template <typename T> struct ops_int {
    using U = typename std::make_unsigned<T>::type;
    static constexpr int BITS = sizeof(T) * 8;
    __device__ static T add(T a, T b) { return (T)((U)a + (U)b); }
    __device__ static T sub(T a, T b) { return (T)((U)a - (U)b); }
    __device__ static T mul(T a, T b) { return (T)((U)a * (U)b); }
    __device__ static T div(T a, T b)
    {
        if (b == 0) return 0;
        if (std::is_signed<T>::value && b == (T)-1) return (T)(U)(0 - (U)a);
        return a / b;
    }
    __device__ static T rem(T a, T b)
    {
        if (b == 0 || (std::is_signed<T>::value && b == (T)-1)) return 0;
        return a % b;
    }
    __device__ static T shl(T a, T b) { return (T)((U)a << ((U)b & (BITS - 1))); }
    __device__ static T shr(T a, T b) { return a >> ((U)b & (BITS - 1)); }  // arithmetic for signed T
    __device__ static T neg(T a) { return (T)(U)(0 - (U)a); }
    __device__ static T bnot(T a) { return (T)~(U)a; }
    __device__ static T babs(T a) { return (std::is_signed<T>::value && a < 0) ? (T)(U)(0 - (U)a) : a; }
    __device__ static T mn(T a, T b) { return b < a ? b : a; }
    __device__ static T mx(T a, T b) { return a < b ? b : a; }
};

template <typename T> struct ops_fp {
    static constexpr bool F = sizeof(T) == 4;
    __device__ static T add(T a, T b)
    {
        if constexpr (F) return __fadd_rn(a, b);
        else return __dadd_rn(a, b);
    }
    __device__ static T sub(T a, T b)
    {
        if constexpr (F) return __fsub_rn(a, b);
        else return __dsub_rn(a, b);
    }
    __device__ static T mul(T a, T b)
    {
        if constexpr (F) return __fmul_rn(a, b);
        else return __dmul_rn(a, b);
    }
    __device__ static T div(T a, T b)
    {
        if constexpr (F) return __fdiv_rn(a, b);
        else return __ddiv_rn(a, b);
    }
    __device__ static T neg(T a) { return -a; }
    __device__ static T babs(T a)
    {
        if constexpr (F) return cv::from_bits<float>(cv::to_bits(a) & 0x7FFFFFFFu);
        else return cv::from_bits<double>(cv::to_bits(a) & 0x7FFFFFFFFFFFFFFFull);
    }
    // "y if y < x, else x", and a NaN operand gives the other one
    __device__ static T mn(T a, T b) { return a != a ? b : (b != b ? a : (b < a ? b : a)); }
    __device__ static T mx(T a, T b) { return a != a ? b : (b != b ? a : (a < b ? b : a)); }
};

// Operands: a broadcast immediate, or one register per value.
template <typename W> struct imm_operand {
    W v;
    __device__ __forceinline__ W operator()(int) const { return v; }
};
template <typename W, int V> struct reg_operand {
    const W (&r)[V];
    __device__ __forceinline__ W operator()(int j) const { return r[j]; }
};

#define GBC_EACH(BODY)                  \
    _Pragma("unroll") for (int j = 0; j < V; ++j) \
    {                                   \
        const T a = get<T>(acc[j]);     \
        const T b = get<T>(opd(j));     \
        (void)b;                        \
        BODY;                           \
    }                                   \
    break;

template <typename T, typename W, int V, typename OPD>
__device__ __forceinline__ void exec_int(uint8_t kind, W (&acc)[V], const OPD& opd)
{
    using O = ops_int<T>;
    switch (kind) {
    case K_ADD: GBC_EACH(acc[j] = put<W>(O::add(a, b)))
    case K_SUB: GBC_EACH(acc[j] = put<W>(O::sub(a, b)))
    case K_RSUB: GBC_EACH(acc[j] = put<W>(O::sub(b, a)))
    case K_MUL: GBC_EACH(acc[j] = put<W>(O::mul(a, b)))
    case K_DIV: GBC_EACH(acc[j] = put<W>(O::div(a, b)))
    case K_RDIV: GBC_EACH(acc[j] = put<W>(O::div(b, a)))
    case K_REM: GBC_EACH(acc[j] = put<W>(O::rem(a, b)))
    case K_RREM: GBC_EACH(acc[j] = put<W>(O::rem(b, a)))
    case K_AND: GBC_EACH(acc[j] = put<W>((T)(a & b)))
    case K_OR: GBC_EACH(acc[j] = put<W>((T)(a | b)))
    case K_XOR: GBC_EACH(acc[j] = put<W>((T)(a ^ b)))
    case K_SHL: GBC_EACH(acc[j] = put<W>(O::shl(a, b)))
    case K_RSHL: GBC_EACH(acc[j] = put<W>(O::shl(b, a)))
    case K_SHR: GBC_EACH(acc[j] = put<W>(O::shr(a, b)))
    case K_RSHR: GBC_EACH(acc[j] = put<W>(O::shr(b, a)))
    case K_LT: GBC_EACH(acc[j] = put<W>((int32_t)(a < b)))
    case K_LE: GBC_EACH(acc[j] = put<W>((int32_t)(a <= b)))
    case K_GT: GBC_EACH(acc[j] = put<W>((int32_t)(a > b)))
    case K_GE: GBC_EACH(acc[j] = put<W>((int32_t)(a >= b)))
    case K_EQ: GBC_EACH(acc[j] = put<W>((int32_t)(a == b)))
    case K_NE: GBC_EACH(acc[j] = put<W>((int32_t)(a != b)))
    case K_MIN: GBC_EACH(acc[j] = put<W>(O::mn(a, b)))
    case K_MAX: GBC_EACH(acc[j] = put<W>(O::mx(a, b)))
    case K_NEG: GBC_EACH(acc[j] = put<W>(O::neg(a)))
    case K_NOT: GBC_EACH(acc[j] = put<W>(O::bnot(a)))
    case K_ABS: GBC_EACH(acc[j] = put<W>(O::babs(a)))
    default: break;
    }
}

template <typename T, typename W, int V, typename OPD>
__device__ __forceinline__ void exec_fp(uint8_t kind, W (&acc)[V], const OPD& opd)
{
    using O = ops_fp<T>;
    switch (kind) {
    case K_ADD: GBC_EACH(acc[j] = put<W>(O::add(a, b)))
    case K_SUB: GBC_EACH(acc[j] = put<W>(O::sub(a, b)))
    case K_RSUB: GBC_EACH(acc[j] = put<W>(O::sub(b, a)))
    case K_MUL: GBC_EACH(acc[j] = put<W>(O::mul(a, b)))
    case K_DIV: GBC_EACH(acc[j] = put<W>(O::div(a, b)))
    case K_RDIV: GBC_EACH(acc[j] = put<W>(O::div(b, a)))
    case K_LT: GBC_EACH(acc[j] = put<W>((int32_t)(a < b)))
    case K_LE: GBC_EACH(acc[j] = put<W>((int32_t)(a <= b)))
    case K_GT: GBC_EACH(acc[j] = put<W>((int32_t)(a > b)))
    case K_GE: GBC_EACH(acc[j] = put<W>((int32_t)(a >= b)))
    case K_EQ: GBC_EACH(acc[j] = put<W>((int32_t)(a == b)))
    case K_NE: GBC_EACH(acc[j] = put<W>((int32_t)(a != b)))
    case K_MIN: GBC_EACH(acc[j] = put<W>(O::mn(a, b)))
    case K_MAX: GBC_EACH(acc[j] = put<W>(O::mx(a, b)))
    case K_NEG: GBC_EACH(acc[j] = put<W>(O::neg(a)))
    case K_ABS: GBC_EACH(acc[j] = put<W>(O::babs(a)))
    default: break;
    }
}
#undef GBC_EACH

template <typename TO, typename W, int V> __device__ __forceinline__ void cvt_to(uint8_t from, W (&acc)[V])
{
#define GBC_CVT(TY, CT)                                                   \
    case TY:                                                              \
        _Pragma("unroll") for (int j = 0; j < V; ++j) acc[j] = put<W>(cv::conv<TO>(get<CT>(acc[j]))); \
        break;
    switch (from) {
        GBC_CVT(I32, int32_t)
        GBC_CVT(U32, uint32_t)
        GBC_CVT(F32, float)
    default:
        if constexpr (sizeof(W) == 8) {
            switch (from) {
                GBC_CVT(I64, int64_t)
                GBC_CVT(U64, uint64_t)
                GBC_CVT(F64, double)
            default: break;
            }
        }
        break;
    }
#undef GBC_CVT
}

// Stack slots live in shared memory, [slot][element][thread] (conflict-free:
// consecutive threads touch consecutive words); only programs that push use
// them.
template <typename W, int V, int NT>
__device__ __forceinline__ W* slot_ptr(W* st, int slot)
{
    return st + (std::size_t)slot * V * NT + threadIdx.x;
}

// acc = acc OP operand for the arithmetic kinds, by element type
template <typename W, int V, typename OPD>
__device__ __forceinline__ void exec_arith(uint8_t kind, uint8_t t, W (&acc)[V], const OPD& opd)
{
    switch (t) {
    case I32: exec_int<int32_t>(kind, acc, opd); return;
    case U32: exec_int<uint32_t>(kind, acc, opd); return;
    case F32: exec_fp<float>(kind, acc, opd); return;
    default:
        if constexpr (sizeof(W) == 8) {
            if (t == I64) exec_int<int64_t>(kind, acc, opd);
            else if (t == U64) exec_int<uint64_t>(kind, acc, opd);
            else exec_fp<double>(kind, acc, opd);
        }
        return;
    }
}

// acc / d or acc % d for an integer literal d (|d| >= 2) by a multiply-high:
// the multiplier is o.aux, l = o.slot (see K_DIVC).
template <typename W, int V> __device__ __forceinline__ void exec_divc(const op& o, W (&acc)[V])
{
    const bool rem = o.kind == K_REMC;
    const int l = o.slot;
    const int sh1 = l > 0 ? 1 : 0, sh2 = l > 0 ? l - 1 : 0;
    switch (o.t) {
    case U32: {
        const uint32_t m = (uint32_t)o.aux, d = (uint32_t)o.imm;
#pragma unroll
        for (int j = 0; j < V; ++j) {
            const uint32_t n = get<uint32_t>(acc[j]);
            const uint32_t t1 = __umulhi(m, n);
            const uint32_t q = (t1 + ((n - t1) >> sh1)) >> sh2;
            acc[j] = put<W>(rem ? n - q * d : q);
        }
        return;
    }
    case I32: {
        const int32_t m = (int32_t)(uint32_t)o.aux, d = (int32_t)(uint32_t)o.imm, ds = d < 0 ? -1 : 0;
#pragma unroll
        for (int j = 0; j < V; ++j) {
            const int32_t n = get<int32_t>(acc[j]);
            int32_t q = (int32_t)((uint32_t)n + (uint32_t)__mulhi(m, n));
            q = (q >> (l - 1)) - (n >> 31);
            q = (q ^ ds) - ds;
            acc[j] = put<W>(rem ? (int32_t)((uint32_t)n - (uint32_t)q * (uint32_t)d) : q);
        }
        return;
    }
    default:
        if constexpr (sizeof(W) == 8) {
            if (o.t == U64) {
                const uint64_t m = o.aux, d = o.imm;
#pragma unroll
                for (int j = 0; j < V; ++j) {
                    const uint64_t n = get<uint64_t>(acc[j]);
                    const uint64_t t1 = __umul64hi(m, n);
                    const uint64_t q = (t1 + ((n - t1) >> sh1)) >> sh2;
                    acc[j] = put<W>(rem ? n - q * d : q);
                }
            } else if (o.t == I64) {
                const long long m = (long long)o.aux, d = (long long)o.imm, ds = d < 0 ? -1 : 0;
#pragma unroll
                for (int j = 0; j < V; ++j) {
                    const long long n = get<int64_t>(acc[j]);
                    long long q = (long long)((unsigned long long)n + (unsigned long long)__mul64hi(m, n));
                    q = (q >> (l - 1)) - (n >> 63);
                    q = (q ^ ds) - ds;
                    acc[j] = put<W>((int64_t)(rem ? (long long)((unsigned long long)n - (unsigned long long)q *
                                                                                         (unsigned long long)d)
                                                  : q));
                }
            }
        }
        return;
    }
}

// STK: the program uses stack slots; NT: threads of the CTA (the slot
// layout's stride). The arithmetic kinds are tested first; an immediate
// operand is used as a scalar.
template <typename W, int V, bool STK, int NT>
__device__ __forceinline__ void exec_op(const op& o, W (&acc)[V], const W (&xv)[V], const W (&yv)[V], W* st)
{
    if (o.kind >= K_ADD && o.kind <= K_ABS) {
        if (o.src == S_IMM || o.src == S_ACC) {
            exec_arith<W, V>(o.kind, o.t, acc, imm_operand<W>{(W)o.imm});
        } else {
            W opd[V];
            if (o.src == S_X) {
#pragma unroll
                for (int j = 0; j < V; ++j) opd[j] = xv[j];
            } else if (o.src == S_Y) {
#pragma unroll
                for (int j = 0; j < V; ++j) opd[j] = yv[j];
            } else if constexpr (STK) {
                const W* r = slot_ptr<W, V, NT>(st, o.slot);
#pragma unroll
                for (int j = 0; j < V; ++j) opd[j] = r[j * NT];
            } else {
#pragma unroll
                for (int j = 0; j < V; ++j) opd[j] = 0;
            }
            exec_arith<W, V>(o.kind, o.t, acc, reg_operand<W, V>{opd});
        }
        return;
    }
    switch (o.kind) {
    case K_LOAD:
        if (o.src == S_X) {
#pragma unroll
            for (int j = 0; j < V; ++j) acc[j] = xv[j];
        } else if (o.src == S_Y) {
#pragma unroll
            for (int j = 0; j < V; ++j) acc[j] = yv[j];
        } else {
#pragma unroll
            for (int j = 0; j < V; ++j) acc[j] = (W)o.imm;
        }
        return;
    case K_PUSH:
        if constexpr (STK) {
            W* r = slot_ptr<W, V, NT>(st, o.slot);
#pragma unroll
            for (int j = 0; j < V; ++j) r[j * NT] = acc[j];
        }
        return;
    case K_SEL:
        if constexpr (STK) {
            // condition in slot, value-if-true in slot + 1
            const W* c = slot_ptr<W, V, NT>(st, o.slot);
            const W* t = slot_ptr<W, V, NT>(st, o.slot + 1);
#pragma unroll
            for (int j = 0; j < V; ++j) acc[j] = (uint32_t)c[j * NT] != 0u ? t[j * NT] : acc[j];
        }
        return;
    case K_EXT8S:
#pragma unroll
        for (int j = 0; j < V; ++j) acc[j] = put<W>((int32_t)(int8_t)(uint8_t)acc[j]);
        return;
    case K_EXT8U:
#pragma unroll
        for (int j = 0; j < V; ++j) acc[j] = put<W>((int32_t)(uint8_t)acc[j]);
        return;
    case K_EXT16S:
#pragma unroll
        for (int j = 0; j < V; ++j) acc[j] = put<W>((int32_t)(int16_t)(uint16_t)acc[j]);
        return;
    case K_EXT16U:
#pragma unroll
        for (int j = 0; j < V; ++j) acc[j] = put<W>((int32_t)(uint16_t)acc[j]);
        return;
    case K_DIVC:
    case K_REMC: exec_divc<W, V>(o, acc); return;
    case K_CVT:
        switch (o.t2) {
        case I32: cvt_to<int32_t>(o.t, acc); return;
        case U32: cvt_to<uint32_t>(o.t, acc); return;
        case F32: cvt_to<float>(o.t, acc); return;
        default:
            if constexpr (sizeof(W) == 8) {
                if (o.t2 == I64) cvt_to<int64_t>(o.t, acc);
                else if (o.t2 == U64) cvt_to<uint64_t>(o.t, acc);
                else cvt_to<double>(o.t, acc);
            }
            return;
        }
    default: return;
    }
}

// raw element -> promoted arithmetic value
template <typename W> __device__ __forceinline__ W promote(uint8_t e, uint32_t raw)
{
    switch (e) {
    case (uint8_t)elem::i8: return put<W>((int32_t)(int8_t)(uint8_t)raw);
    case (uint8_t)elem::i16: return put<W>((int32_t)(int16_t)(uint16_t)raw);
    default: return (W)raw;  // unsigned narrow types zero-extended, 32-bit as is
    }
}

// ---- host-side shape of a program ----

// widest element, in bytes
inline int widest(const program& p)
{
    const std::size_t a = elem_size((elem)p.x_elem), b = elem_size((elem)(p.has_y ? p.y_elem : p.x_elem)),
                      c = elem_size((elem)p.out_elem);
    return (int)std::max(a, std::max(b, c));
}

inline bool all_32bit(const program& p)
{
    auto small = [](uint8_t t) { return t == I32 || t == U32 || t == F32; };
    if (widest(p) > 4) return false;
    for (uint32_t k = 0; k < p.nops; ++k) {
        const op& o = p.ops[k];
        if (!small(o.t)) return false;
        if (o.kind == K_CVT && !small(o.t2)) return false;
    }
    return true;
}

// the program keeps temporaries in stack slots
inline bool uses_stack(const program& p)
{
    for (uint32_t k = 0; k < p.nops; ++k)
        if (p.ops[k].kind == K_PUSH) return true;
    return false;
}

// acc = the program over xv (and yv); the first operation is always a load,
// done without a dispatch. Every program writes a stack slot (PUSH) before
// it reads it; st: the CTA's slots in shared memory (STK only).
template <typename W, int V, bool STK, int NT>
__device__ __forceinline__ void run_program(const program& p, W (&acc)[V], const W (&xv)[V], const W (&yv)[V], W* st)
{
    const op& first = p.ops[0];
    if (first.src == S_X) {
#pragma unroll
        for (int j = 0; j < V; ++j) acc[j] = xv[j];
    } else if (first.src == S_Y) {
#pragma unroll
        for (int j = 0; j < V; ++j) acc[j] = yv[j];
    } else {
        const W imm = (W)first.imm;
#pragma unroll
        for (int j = 0; j < V; ++j) acc[j] = imm;
    }
    for (uint32_t k = 1; k < p.nops; ++k) exec_op<W, V, STK, NT>(p.ops[k], acc, xv, yv, st);
}

}  // namespace interp
}  // namespace xp
}  // namespace gbc
