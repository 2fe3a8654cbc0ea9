// Element-wise expressions for transform / transform2: an OpenCL C expression
// over x (and y) is compiled on the host into a short accumulator program that
// one ahead-of-time kernel interprets. The program is the same for every
// element, so the interpreter's branches are uniform across a warp and its
// dispatch is paid once per group of elements a thread holds.
//
// Reference path replaced: detail::transform / detail::transform2
// (lib/src/Compute/Algorithm.cpp:361-398), which paste the expression into the
// kernels clc_transform / clc_transform2 (30-56) as `out[i] = (T_OUT)(EXPR)`
// with `const T_IN x = in[i]` (and `const T_IN2 y`) and compile them at run
// time. Here the expression language is a subset of OpenCL C:
//   - operands x, y, integer and floating literals (C suffixes u, l, f), the
//     limits INT_MIN ... ULONG_MAX, FLT_MAX, DBL_MAX, INFINITY, NAN;
//   - unary + - ~ !, binary * / % + - << >> < <= > >= == != & ^ | && ||, ?:;
//   - casts to char, uchar, short, ushort, int, uint, long, ulong, size_t,
//     float, double (with the "unsigned ..." spellings);
//   - min, max, clamp, abs, fabs, fmin, fmax, as_int/uint/long/ulong/float/
//     double, convert_<type>.
// Types follow OpenCL C: integer promotion of char/short, the usual arithmetic
// conversions, int results for comparisons and logic, shift counts masked to
// the width of the left operand, abs of an integer giving the unsigned type.
// Where OpenCL C leaves a result undefined the interpreter defines it:
// integer division or remainder by zero gives 0, INT_MIN / -1 wraps,
// float-to-integer conversion saturates (NaN gives 0), min/max of a NaN give
// the other operand. Float arithmetic is IEEE with round-to-nearest and no
// contraction into fused multiply-adds.
// A malformed expression throws build_error (the reference's build failure,
// CLC_ERROR_BUILD); well-formed OpenCL C outside the subset (sqrt, vector
// types, ...) throws unsupported_error.
#pragma once

#include <cstddef>
#include <cstdint>
#include <string>

#include "runtime.hpp"

namespace gbc {
namespace xp {

// arithmetic types after integer promotion
enum ty : uint8_t { I32 = 0, U32 = 1, I64 = 2, U64 = 3, F32 = 4, F64 = 5 };

// operand sources
enum src : uint8_t { S_ACC = 0, S_IMM = 1, S_X = 2, S_Y = 3, S_POP = 4 };

// Operations. Binary kinds compute acc = acc OP operand; the R* kinds compute
// acc = operand OP acc. Comparisons take operands of type t and leave an I32
// 0/1. CVT converts acc from t to t2. EXT8S/EXT8U/EXT16S/EXT16U keep the low
// 8/16 bits of an I32 (a cast to char/uchar/short/ushort, promoted back).
// PUSH stores acc in stack slot `slot`; SEL sets acc = st[slot] ? st[slot+1] :
// acc (slot holds an I32 condition). DIVC / REMC divide by an integer literal
// without a division (Granlund and Montgomery, "Division by Invariant
// Integers using Multiplication", PLDI 1994: figure 4.1 for unsigned, 5.2 for
// signed operands), with the same results as DIV / REM.
enum kind : uint8_t {
    K_LOAD = 0,
    K_PUSH,
    K_ADD,
    K_SUB,
    K_RSUB,
    K_MUL,
    K_DIV,
    K_RDIV,
    K_REM,
    K_RREM,
    K_AND,
    K_OR,
    K_XOR,
    K_SHL,
    K_RSHL,
    K_SHR,
    K_RSHR,
    K_LT,
    K_LE,
    K_GT,
    K_GE,
    K_EQ,
    K_NE,
    K_MIN,
    K_MAX,
    K_NEG,
    K_NOT,
    K_ABS,
    K_CVT,
    K_EXT8S,
    K_EXT8U,
    K_EXT16S,
    K_EXT16U,
    K_SEL,
    K_DIVC,  // acc / imm and acc % imm for an integer literal |imm| >= 2, by
    K_REMC,  // multiplication with a precomputed multiplier (aux) and shift (slot)
    K_COUNT
};

constexpr int MAX_OPS = 48;
constexpr int STACK = 4;

struct op {
    uint8_t kind, t, src, slot, t2, pad[3];
    uint64_t imm;  // raw bits of the immediate in type t
    uint64_t aux;  // K_DIVC / K_REMC: the multiplier
};

struct program {
    uint32_t nops = 0;
    uint8_t x_elem = 0, y_elem = 0, out_elem = 0, has_y = 0;  // elem codes
    uint8_t x_ty = 0, y_ty = 0, out_ty = 0, pad = 0;            // promoted types
    op ops[MAX_OPS];
};

//! Compiles `text` for inputs of element type tx (and ty2 when has_y) and an
//! output of type tout. Throws build_error or unsupported_error.
program compile(const std::string& text, elem tx, bool has_y, elem ty2, elem tout);

//! Compiles a copy_if predicate over x of element type tx: the program leaves
//! an int 1 where the expression is nonzero in its own type (the reference's
//! `(PRED) ? 1u : 0u`), else 0.
program compile_predicate(const std::string& text, elem tx);

//! Human-readable listing of a compiled program (tests and diagnostics).
std::string listing(const program& p);

}  // namespace xp

//! out[i] = (T_OUT)(expr(x[i] [, y[i]])) for i < n; asynchronous.
void transform(device_context& ctx, const xp::program& p, const void* x, const void* y, void* out,
               std::size_t n);

}  // namespace gbc
