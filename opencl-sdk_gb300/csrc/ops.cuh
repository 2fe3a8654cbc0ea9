// The canonical binary operators behind the reference's ops:: helpers
// (lib/include/CL/Compute/Algorithm.hpp:53-65) and the expressions its tests
// use ("(a + b)", "max(a, b)", "b"). Each is a functor op(a, b) where a
// precedes b in sequence order; minimum/maximum are the reference's ternaries
// ((b < a) ? b : a and (a < b) ? b : a), so ties and NaNs resolve the same way.
#pragma once

#include <cstdint>
#include <type_traits>

#include "runtime.hpp"

namespace gbc {
namespace ops {

struct Plus {
    template <typename T> __host__ __device__ __forceinline__ T operator()(T a, T b) const { return a + b; }
};
struct Mul {
    template <typename T> __host__ __device__ __forceinline__ T operator()(T a, T b) const { return a * b; }
};
struct And {
    template <typename T> __host__ __device__ __forceinline__ T operator()(T a, T b) const { return a & b; }
};
struct Or {
    template <typename T> __host__ __device__ __forceinline__ T operator()(T a, T b) const { return a | b; }
};
struct Xor {
    template <typename T> __host__ __device__ __forceinline__ T operator()(T a, T b) const { return a ^ b; }
};
struct Min {
    template <typename T> __host__ __device__ __forceinline__ T operator()(T a, T b) const { return (b < a) ? b : a; }
};
struct Max {
    template <typename T> __host__ __device__ __forceinline__ T operator()(T a, T b) const { return (a < b) ? b : a; }
};
// Right projection: scanning with it reproduces the input, which the
// reference's tests use to prove sequence-ordered combination
// (lib/test/Compute/main.cpp:231-238). Its identity works from the left only.
struct Right {
    template <typename T> __host__ __device__ __forceinline__ T operator()(T, T b) const { return b; }
};

// Calls f.template operator()<T, Op>() for the runtime (elem, op_kind) pair,
// over the element types and operators that have compiled kernels:
// 32- and 64-bit integers with every operator, float/double without the
// bitwise ones.
template <typename F> void dispatch(elem t, op_kind op, F&& f)
{
    auto with_type = [&](auto tag) {
        using T = decltype(tag);
        constexpr bool is_int = !std::is_floating_point<T>::value;
        switch (op) {
        case op_kind::plus: f.template run<T, Plus>(); return;
        case op_kind::multiplies: f.template run<T, Mul>(); return;
        case op_kind::minimum: f.template run<T, Min>(); return;
        case op_kind::maximum: f.template run<T, Max>(); return;
        case op_kind::right: f.template run<T, Right>(); return;
        case op_kind::left:
            throw unsupported_error("gbcompute: the left projection has no identity element");
        case op_kind::bit_and:
            if constexpr (is_int) { f.template run<T, And>(); return; }
            break;
        case op_kind::bit_or:
            if constexpr (is_int) { f.template run<T, Or>(); return; }
            break;
        case op_kind::bit_xor:
            if constexpr (is_int) { f.template run<T, Xor>(); return; }
            break;
        }
        throw unsupported_error("gbcompute: bitwise operator on a floating-point type");
    };
    switch (t) {
    case elem::i32: with_type(int32_t{}); return;
    case elem::u32: with_type(uint32_t{}); return;
    case elem::i64: with_type(int64_t{}); return;
    case elem::u64: with_type(uint64_t{}); return;
    case elem::f32: with_type(float{}); return;
    case elem::f64: with_type(double{}); return;
    default: break;
    }
    throw unsupported_error("gbcompute: scan/reduce support 32- and 64-bit element types only");
}

}  // namespace ops
}  // namespace gbc
