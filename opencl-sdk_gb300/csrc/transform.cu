// transform / transform2: out[i] = (T_OUT)(expr(x[i] [, y[i]])).
//
// Reference path replaced: detail::transform / detail::transform2
// (lib/src/Compute/Algorithm.cpp:361-398) and their kernels clc_transform /
// clc_transform2 (30-56), which compile the expression at run time. Here the
// expression is compiled on the host (recursive descent over the OpenCL C
// expression grammar, typed with OpenCL C's rules) into an accumulator
// program that one ahead-of-time kernel interprets. The language subset and
// the results the interpreter defines where OpenCL C leaves them undefined
// are listed in expr.hpp.
//
// Kernel: one CTA per chunk; each thread loads K groups of E consecutive
// elements of x (and y), one vector access per group with a warp's groups
// contiguous, promotes them to their arithmetic type, runs the program over
// all V = E * K values at once (one dispatch per operation per V elements,
// branches uniform across the warp) and stores V results. Programs whose
// types are all 32-bit run with 32-bit registers, the rest with 64-bit ones;
// E makes a group one 16-byte vector of the widest element. Programs that
// need temporaries keep them in shared memory.
#include <cctype>
#include <cerrno>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <limits>
#include <memory>
#include <sstream>
#include <type_traits>
#include <vector>

#include "device_common.cuh"
#include "expr.hpp"
#include "interp.cuh"

namespace gbc {
namespace xp {

// ---------------------------------------------------------------------------
// Host: lexer, parser with OpenCL C typing, code generation.
// ---------------------------------------------------------------------------
namespace {

bool is_int(elem t) { return t != elem::f32 && t != elem::f64; }
bool is_narrow(elem t) { return elem_size(t) < 4; }

ty arith(elem t)
{
    switch (t) {
    case elem::i8:
    case elem::u8:
    case elem::i16:
    case elem::u16:
    case elem::i32: return I32;  // char, uchar, short, ushort promote to int
    case elem::u32: return U32;
    case elem::i64: return I64;
    case elem::u64: return U64;
    case elem::f32: return F32;
    case elem::f64: return F64;
    }
    return I32;
}

elem of_ty(ty t)
{
    switch (t) {
    case I32: return elem::i32;
    case U32: return elem::u32;
    case I64: return elem::i64;
    case U64: return elem::u64;
    case F32: return elem::f32;
    default: return elem::f64;
    }
}

const char* elem_name(elem t)
{
    static const char* names[] = {"char", "uchar", "short", "ushort", "int", "uint", "long", "ulong", "float", "double"};
    return names[(int)t];
}

// usual arithmetic conversions (C99 6.3.1.8 with 32-bit int, 64-bit long)
elem common(elem a, elem b)
{
    if (a == elem::f64 || b == elem::f64) return elem::f64;
    if (a == elem::f32 || b == elem::f32) return elem::f32;
    const ty pa = arith(a), pb = arith(b);
    if (pa == pb) return of_ty(pa);
    const bool ua = pa == U32 || pa == U64, ub = pb == U32 || pb == U64;
    const int ra = (pa == I64 || pa == U64) ? 2 : 1, rb = (pb == I64 || pb == U64) ? 2 : 1;
    if (ua == ub) return of_ty(ra >= rb ? pa : pb);
    const ty u = ua ? pa : pb, s = ua ? pb : pa;
    const int ru = ua ? ra : rb, rs = ua ? rb : ra;
    if (ru >= rs) return of_ty(u);
    if (rs > ru) return of_ty(s);  // long holds every uint
    return of_ty(s == I32 ? U32 : U64);
}

// Division by an invariant integer d (Granlund and Montgomery, PLDI 1994).
// Unsigned N-bit (figure 4.1), 1 <= d < 2^N: l = ceil(log2 d), m = floor(2^N
// (2^l - d) / d) + 1; then q = SRL(t1 + SRL(n - t1, min(l, 1)), max(l - 1, 0))
// with t1 = MULUH(m, n).
void magic_unsigned(int bits, uint64_t d, uint64_t& m, int& l)
{
    using u128 = unsigned __int128;
    l = 0;
    while (((u128)1 << l) < d) ++l;
    const u128 num = ((u128)1 << bits) * (((u128)1 << l) - d);
    m = (uint64_t)(num / d + 1);
}
// Signed N-bit (figure 5.2), |d| >= 2: l = max(ceil(log2 |d|), 1), m = 1 +
// floor(2^(N + l - 1) / |d|) - 2^N (a negative N-bit value); then q0 = n +
// MULSH(m, n), q0 = SRA(q0, l - 1) - XSIGN(n), q = EOR(q0, dsign) - dsign.
void magic_signed(int bits, int64_t d, uint64_t& m, int& l)
{
    using u128 = unsigned __int128;
    const uint64_t ad = d < 0 ? (uint64_t)(-(d + 1)) + 1u : (uint64_t)d;
    l = 0;
    while (((u128)1 << l) < ad) ++l;
    if (l < 1) l = 1;
    const u128 big = 1 + (((u128)1 << (bits + l - 1)) / ad);
    m = (uint64_t)(big - ((u128)1 << bits));  // two's complement, low `bits` bits meaningful
    if (bits == 32) m &= 0xFFFFFFFFull;
}

struct token {
    enum kind { END, NUM, ID, PUNCT } k = END;
    std::string s;
    std::size_t pos = 0;
};

enum node_kind { N_X, N_Y, N_LIT, N_UN, N_BIN, N_CAST, N_TERN, N_MINMAX, N_CLAMP, N_ABS, N_BITCAST };

struct node {
    node_kind k;
    int op = 0;              // token code for N_UN/N_BIN; K_MIN/K_MAX for N_MINMAX
    elem t = elem::i32;      // C type of the result
    elem opt = elem::i32;    // operation type (binary / comparison operands, min/max/clamp)
    uint64_t bits = 0;       // N_LIT: value in arith(t)
    std::unique_ptr<node> a, b, c;
};
using node_ptr = std::unique_ptr<node>;

class compiler {
public:
    compiler(const std::string& text, elem tx, bool has_y, elem ty2, const char* who)
        : text_(text), tx_(tx), has_y_(has_y), ty_(ty2), who_(who)
    {
        // bounds the token list before lexing; a program of MAX_OPS
        // operations needs far less text
        if (text.size() > MAX_TEXT)
            fail_unsupported("an expression text longer than " + std::to_string(MAX_TEXT) + " characters");
        lex();
    }

    node_ptr parse()
    {
        if (toks_.size() == 1) fail_build(0, "expected an expression");
        node_ptr e = expression();
        if (peek().k != token::END) fail_build(peek().pos, "unexpected '" + peek().s + "'");
        return e;
    }

    program emit(const node& root, elem tout)
    {
        gen(root, 0);
        convert_to(arith(root.t), tout);
        prog_.out_ty = is_narrow(tout) ? (uint8_t)I32 : (uint8_t)arith(tout);
        return prog_;
    }

    // the expression's truth value (nonzero, in its own type) as an int 0/1
    program emit_truth(const node& root)
    {
        gen_truth(root, 0);
        prog_.out_ty = I32;
        return prog_;
    }

private:
    const std::string& text_;
    elem tx_;
    bool has_y_;
    elem ty_;
    const char* who_;
    std::vector<token> toks_;
    std::size_t at_ = 0;
    // Bounds on the recursion of the parser, the code generator and the
    // tree's destructor, so that hostile text is refused, not a stack
    // overflow: nesting levels (parentheses, prefix operators, casts,
    // ternaries, call arguments) and nodes created. A program has at most
    // MAX_OPS operations, far fewer than MAX_NODES nodes.
    static constexpr int MAX_NEST = 128;
    static constexpr std::size_t MAX_NODES = 256;
    static constexpr std::size_t MAX_TEXT = 65536;
    int nest_ = 0;
    std::size_t nodes_ = 0;

    struct nest_guard {
        compiler& c;
        explicit nest_guard(compiler& cc) : c(cc)
        {
            if (++c.nest_ > MAX_NEST)
                c.fail_unsupported("an expression nested deeper than " + std::to_string(MAX_NEST) + " levels");
        }
        ~nest_guard() { --c.nest_; }
        nest_guard(const nest_guard&) = delete;
        nest_guard& operator=(const nest_guard&) = delete;
    };
    program prog_;

    // the expression as quoted in messages: at most 200 characters
    std::string quoted() const { return text_.size() <= 200 ? text_ : text_.substr(0, 200) + "..."; }

    [[noreturn]] void fail_build(std::size_t pos, const std::string& what) const
    {
        throw build_error(std::string(who_) + ": build log: error at column " + std::to_string(pos + 1) + ": " + what +
                          " in \"" + quoted() + "\"");
    }
    [[noreturn]] void fail_unsupported(const std::string& what) const
    {
        throw unsupported_error(std::string(who_) + ": " + what + " in \"" + quoted() +
                                "\" is outside the supported expression subset");
    }

    // ---- lexer ----
    void lex()
    {
        static const char* puncts[] = {"<<", ">>", "<=", ">=", "==", "!=", "&&", "||", "++", "--", "+=", "-=",
                                       "*=", "/=", "%=", "&=", "|=", "^=", "->", "+", "-", "*", "/", "%",
                                       "&", "|", "^", "~", "!", "<", ">", "(", ")", ",", "?", ":", "=",
                                       "[", "]", ".", "{", "}", ";", "#"};
        const std::string& s = text_;
        std::size_t i = 0;
        while (true) {
            while (i < s.size() && std::isspace((unsigned char)s[i])) ++i;
            token t;
            t.pos = i;
            if (i == s.size()) {
                toks_.push_back(t);
                return;
            }
            const char c = s[i];
            if (std::isdigit((unsigned char)c) || (c == '.' && i + 1 < s.size() && std::isdigit((unsigned char)s[i + 1]))) {
                std::size_t j = i;
                if (c == '0' && j + 1 < s.size() && (s[j + 1] == 'x' || s[j + 1] == 'X')) {
                    j += 2;
                    while (j < s.size() && (std::isalnum((unsigned char)s[j]) || s[j] == '.')) ++j;
                } else {
                    while (j < s.size()) {
                        const char d = s[j];
                        if (std::isalnum((unsigned char)d) || d == '.' || d == '_') {
                            ++j;
                        } else if ((d == '+' || d == '-') && (s[j - 1] == 'e' || s[j - 1] == 'E')) {
                            ++j;
                        } else {
                            break;
                        }
                    }
                }
                t.k = token::NUM;
                t.s = s.substr(i, j - i);
                i = j;
            } else if (std::isalpha((unsigned char)c) || c == '_') {
                std::size_t j = i;
                while (j < s.size() && (std::isalnum((unsigned char)s[j]) || s[j] == '_')) ++j;
                t.k = token::ID;
                t.s = s.substr(i, j - i);
                i = j;
            } else {
                bool found = false;
                for (const char* p : puncts) {
                    const std::size_t len = std::strlen(p);
                    if (s.compare(i, len, p) == 0) {
                        t.k = token::PUNCT;
                        t.s = p;
                        i += len;
                        found = true;
                        break;
                    }
                }
                if (!found) fail_build(i, std::string("invalid character '") + c + "'");
            }
            toks_.push_back(t);
        }
    }

    const token& peek(std::size_t ahead = 0) const
    {
        const std::size_t k = std::min(at_ + ahead, toks_.size() - 1);
        return toks_[k];
    }
    bool is(const char* p, std::size_t ahead = 0) const
    {
        const token& t = peek(ahead);
        return t.k == token::PUNCT && t.s == p;
    }
    bool accept(const char* p)
    {
        if (!is(p)) return false;
        ++at_;
        return true;
    }
    void expect(const char* p)
    {
        if (!accept(p)) {
            const token& t = peek();
            fail_build(t.pos, std::string("expected '") + p + "'" +
                                  (t.k == token::END ? " at end of expression" : " before '" + t.s + "'"));
        }
    }

    // ---- node builders ----
    node_ptr make(node_kind k, elem t)
    {
        if (++nodes_ > MAX_NODES) fail_unsupported("an expression longer than " + std::to_string(MAX_OPS) + " operations");
        node_ptr n(new node);
        n->k = k;
        n->t = t;
        return n;
    }
    node_ptr literal(elem t, uint64_t bits)
    {
        node_ptr n = make(N_LIT, t);
        n->bits = bits;
        return n;
    }

    void require_int(const node& e, std::size_t pos, const char* what) const
    {
        if (!is_int(e.t)) fail_build(pos, std::string("invalid operand of type '") + elem_name(e.t) + "' to " + what);
    }

    // ---- grammar (C precedence) ----
    node_ptr expression()
    {
        node_ptr e = conditional();
        if (is(",")) fail_unsupported("the comma operator");
        return e;
    }

    node_ptr conditional()
    {
        const nest_guard guard(*this);
        node_ptr c = binary(0);
        if (!is("?")) return c;
        ++at_;
        node_ptr a = expression();
        expect(":");
        node_ptr b = conditional();
        node_ptr n = make(N_TERN, common(a->t, b->t));
        n->opt = n->t;
        n->a = std::move(c);
        n->b = std::move(a);
        n->c = std::move(b);
        return n;
    }

    // binary operators by precedence level, loosest first
    int level_of(const token& t) const
    {
        if (t.k != token::PUNCT) return -1;
        static const char* levels[][4] = {{"||"}, {"&&"}, {"|"}, {"^"}, {"&"}, {"==", "!="},
                                          {"<", ">", "<=", ">="}, {"<<", ">>"}, {"+", "-"}, {"*", "/", "%"}};
        for (int l = 0; l < 10; ++l)
            for (const char* p : levels[l])
                if (p != nullptr && t.s == p) return l;
        return -1;
    }

    node_ptr binary(int level)
    {
        if (level == 10) return unary();
        node_ptr lhs = binary(level + 1);
        while (level_of(peek()) == level) {
            const token op = peek();
            ++at_;
            node_ptr rhs = binary(level + 1);
            lhs = make_binary(op, std::move(lhs), std::move(rhs));
        }
        return lhs;
    }

    node_ptr make_binary(const token& op, node_ptr a, node_ptr b)
    {
        const std::string& s = op.s;
        node_ptr n;
        if (s == "||" || s == "&&") {
            n = make(N_BIN, elem::i32);
        } else if (s == "<<" || s == ">>") {
            require_int(*a, op.pos, "a shift");
            require_int(*b, op.pos, "a shift");
            n = make(N_BIN, of_ty(arith(a->t)));
            n->opt = n->t;
        } else if (s == "==" || s == "!=" || s == "<" || s == ">" || s == "<=" || s == ">=") {
            n = make(N_BIN, elem::i32);
            n->opt = common(a->t, b->t);
        } else {
            if (s == "%" || s == "&" || s == "|" || s == "^") {
                require_int(*a, op.pos, ("'" + s + "'").c_str());
                require_int(*b, op.pos, ("'" + s + "'").c_str());
            }
            n = make(N_BIN, common(a->t, b->t));
            n->opt = n->t;
        }
        n->op = kind_of(s);
        n->a = std::move(a);
        n->b = std::move(b);
        return n;
    }

    static int kind_of(const std::string& s)
    {
        if (s == "+") return K_ADD;
        if (s == "-") return K_SUB;
        if (s == "*") return K_MUL;
        if (s == "/") return K_DIV;
        if (s == "%") return K_REM;
        if (s == "&") return K_AND;
        if (s == "|") return K_OR;
        if (s == "^") return K_XOR;
        if (s == "<<") return K_SHL;
        if (s == ">>") return K_SHR;
        if (s == "<") return K_LT;
        if (s == "<=") return K_LE;
        if (s == ">") return K_GT;
        if (s == ">=") return K_GE;
        if (s == "==") return K_EQ;
        if (s == "!=") return K_NE;
        if (s == "&&") return 100;
        return 101;  // ||
    }

    // type names a cast may use; false when the tokens at the cursor are not one
    bool type_name(elem& t, std::size_t& len) const
    {
        const token& a = peek();
        if (a.k != token::ID) return false;
        static const struct {
            const char* name;
            elem t;
        } simple[] = {{"char", elem::i8},  {"uchar", elem::u8},   {"short", elem::i16}, {"ushort", elem::u16},
                      {"int", elem::i32},  {"uint", elem::u32},   {"long", elem::i64},  {"ulong", elem::u64},
                      {"float", elem::f32}, {"double", elem::f64}, {"size_t", elem::u64}};
        if (a.s == "unsigned" || a.s == "signed") {
            const bool u = a.s == "unsigned";
            const token& b = peek(1);
            if (b.k == token::ID && (b.s == "char" || b.s == "short" || b.s == "int" || b.s == "long")) {
                len = 2;
                if (b.s == "char") t = u ? elem::u8 : elem::i8;
                else if (b.s == "short") t = u ? elem::u16 : elem::i16;
                else if (b.s == "int") t = u ? elem::u32 : elem::i32;
                else t = u ? elem::u64 : elem::i64;
                return true;
            }
            len = 1;
            t = u ? elem::u32 : elem::i32;
            return true;
        }
        for (const auto& e : simple)
            if (a.s == e.name) {
                t = e.t;
                len = 1;
                return true;
            }
        static const char* other[] = {"bool", "half", "void", "size_t2", "intptr_t", "uintptr_t", "ptrdiff_t"};
        for (const char* o : other)
            if (a.s == o) fail_unsupported(std::string("the type '") + a.s + "'");
        // vector types (float4, int2, ...)
        for (const auto& e : simple) {
            const std::size_t k = std::strlen(e.name);
            if (a.s.size() > k && a.s.compare(0, k, e.name) == 0 && std::isdigit((unsigned char)a.s[k]))
                fail_unsupported("the vector type '" + a.s + "'");
        }
        return false;
    }

    node_ptr unary()
    {
        const nest_guard guard(*this);
        const token t = peek();
        if (is("+") || is("-") || is("~") || is("!")) {
            ++at_;
            node_ptr e = unary();
            if (t.s == "~") require_int(*e, t.pos, "'~'");
            return make_unary(t.s[0], std::move(e));
        }
        if (is("++") || is("--")) fail_build(t.pos, "cannot modify a const value");
        if (is("(")) {
            elem ct;
            std::size_t len = 0;
            ++at_;
            const bool cast = type_name(ct, len);
            --at_;
            if (cast && peek(1 + len).k == token::PUNCT && peek(1 + len).s == ")") {
                at_ += 2 + len;
                node_ptr e = unary();
                return make_cast(ct, std::move(e));
            }
        }
        return primary();
    }

    node_ptr make_unary(char op, node_ptr e)
    {
        if (op == '!') {
            node_ptr n = make(N_UN, elem::i32);
            n->op = '!';
            n->opt = e->t;
            n->a = std::move(e);
            return n;
        }
        const elem pt = of_ty(arith(e->t));
        if (op == '+') {
            if (e->k == N_LIT) return literal(pt, e->bits);
            node_ptr n = make(N_UN, pt);
            n->op = '+';
            n->a = std::move(e);
            return n;
        }
        if (e->k == N_LIT) return literal(pt, fold_unary(op, arith(pt), e->bits));
        node_ptr n = make(N_UN, pt);
        n->op = op;
        n->a = std::move(e);
        return n;
    }

    static uint64_t fold_unary(char op, ty t, uint64_t r)
    {
        switch (t) {
        case F32: return cv::to_bits(-cv::from_bits<float>(r));
        case F64: return cv::to_bits(-cv::from_bits<double>(r));
        case I32:
        case U32: return op == '-' ? (uint64_t)(uint32_t)(0u - (uint32_t)r) : (uint64_t)(uint32_t)~(uint32_t)r;
        default: return op == '-' ? 0ull - r : ~r;
        }
    }

    node_ptr make_cast(elem ct, node_ptr e)
    {
        if (e->k == N_LIT) {
            const uint64_t v = cv::convert(arith(e->t), is_narrow(ct) ? (uint8_t)I32 : (uint8_t)arith(ct), e->bits);
            return literal(ct, narrow_bits(ct, v));
        }
        node_ptr n = make(N_CAST, ct);
        n->a = std::move(e);
        return n;
    }

    // value of a narrow type kept as a promoted int (sign- or zero-extended)
    static uint64_t narrow_bits(elem t, uint64_t v)
    {
        switch (t) {
        case elem::i8: return (uint32_t)(int32_t)(int8_t)(uint8_t)v;
        case elem::u8: return (uint8_t)v;
        case elem::i16: return (uint32_t)(int32_t)(int16_t)(uint16_t)v;
        case elem::u16: return (uint16_t)v;
        default: return v;
        }
    }

    node_ptr number(const token& t)
    {
        const std::string& s = t.s;
        std::size_t end = s.size();
        while (end > 0 && std::strchr("uUlLfF", s[end - 1]) != nullptr) {
            // an 'f' ending a hex literal is a digit
            if ((s[end - 1] == 'f' || s[end - 1] == 'F') && s.size() > 2 && (s[1] == 'x' || s[1] == 'X')) break;
            --end;
        }
        const std::string digits = s.substr(0, end), suffix = s.substr(end);
        int u = 0, l = 0, f = 0;
        for (char c : suffix) {
            if (c == 'u' || c == 'U') ++u;
            else if (c == 'l' || c == 'L') ++l;
            else ++f;
        }
        const bool hex = digits.size() > 1 && digits[0] == '0' && (digits[1] == 'x' || digits[1] == 'X');
        const bool floating = !hex && (digits.find_first_of(".eE") != std::string::npos);
        if (hex && digits.find_first_of(".pP") != std::string::npos) fail_unsupported("the hexadecimal float literal " + s);
        if (floating || f > 0) {
            if (u > 0 || f > 1 || (f == 1 && l > 0) || !floating) fail_build(t.pos, "invalid suffix on literal " + s);
            if (l > 0) fail_unsupported("the long double literal " + s);
            char* stop = nullptr;
            if (f == 1) {
                const float v = std::strtof(digits.c_str(), &stop);
                if (stop != digits.c_str() + digits.size()) fail_build(t.pos, "invalid literal " + s);
                return literal(elem::f32, cv::to_bits(v));
            }
            const double v = std::strtod(digits.c_str(), &stop);
            if (stop != digits.c_str() + digits.size()) fail_build(t.pos, "invalid literal " + s);
            return literal(elem::f64, cv::to_bits(v));
        }
        if (u > 1 || l > 1) fail_build(t.pos, "invalid suffix on literal " + s);
        for (std::size_t i = hex ? 2 : 0; i < digits.size(); ++i) {
            const char c = digits[i];
            const bool ok = hex ? std::isxdigit((unsigned char)c) != 0
                                : (std::isdigit((unsigned char)c) && !(digits[0] == '0' && c > '7'));
            if (!ok) fail_build(t.pos, "invalid digit in literal " + s);
        }
        if (hex && digits.size() == 2) fail_build(t.pos, "invalid literal " + s);
        errno = 0;
        const unsigned long long v = std::strtoull(digits.c_str(), nullptr, 0);
        if (errno != 0) fail_build(t.pos, "integer literal " + s + " is too large");
        const bool decimal = !(digits.size() > 1 && digits[0] == '0');
        // the first type that holds the value (C99 6.4.4.1; int 32-bit, long 64-bit)
        elem lt;
        if (!u && !l && v <= 0x7FFFFFFFull) lt = elem::i32;
        else if (!l && (u || !decimal) && v <= 0xFFFFFFFFull) lt = elem::u32;
        else if (!u && v <= 0x7FFFFFFFFFFFFFFFull) lt = elem::i64;
        else lt = elem::u64;
        return literal(lt, (lt == elem::i32 || lt == elem::u32) ? (uint64_t)(uint32_t)v : (uint64_t)v);
    }

    node_ptr constant(const std::string& name)
    {
        using fl = std::numeric_limits<float>;
        using dl = std::numeric_limits<double>;
        if (name == "INT_MAX") return literal(elem::i32, 0x7FFFFFFFu);
        if (name == "INT_MIN") return literal(elem::i32, 0x80000000u);
        if (name == "UINT_MAX") return literal(elem::u32, 0xFFFFFFFFu);
        if (name == "LONG_MAX") return literal(elem::i64, 0x7FFFFFFFFFFFFFFFull);
        if (name == "LONG_MIN") return literal(elem::i64, 0x8000000000000000ull);
        if (name == "ULONG_MAX") return literal(elem::u64, ~0ull);
        if (name == "CHAR_MAX" || name == "SCHAR_MAX") return literal(elem::i32, 127);
        if (name == "CHAR_MIN" || name == "SCHAR_MIN") return literal(elem::i32, (uint32_t)-128);
        if (name == "UCHAR_MAX") return literal(elem::i32, 255);
        if (name == "SHRT_MAX") return literal(elem::i32, 32767);
        if (name == "SHRT_MIN") return literal(elem::i32, (uint32_t)-32768);
        if (name == "USHRT_MAX") return literal(elem::i32, 65535);
        if (name == "CHAR_BIT") return literal(elem::i32, 8);
        if (name == "FLT_MAX" || name == "MAXFLOAT") return literal(elem::f32, cv::to_bits(fl::max()));
        if (name == "FLT_MIN") return literal(elem::f32, cv::to_bits(fl::min()));
        if (name == "FLT_EPSILON") return literal(elem::f32, cv::to_bits(fl::epsilon()));
        if (name == "DBL_MAX") return literal(elem::f64, cv::to_bits(dl::max()));
        if (name == "DBL_MIN") return literal(elem::f64, cv::to_bits(dl::min()));
        if (name == "DBL_EPSILON") return literal(elem::f64, cv::to_bits(dl::epsilon()));
        if (name == "INFINITY" || name == "HUGE_VALF") return literal(elem::f32, cv::to_bits(fl::infinity()));
        if (name == "HUGE_VAL") return literal(elem::f64, cv::to_bits(dl::infinity()));
        if (name == "NAN") return literal(elem::f32, cv::to_bits(fl::quiet_NaN()));
        return nullptr;
    }

    std::vector<node_ptr> call_args(std::size_t pos, const std::string& fn, std::size_t want)
    {
        std::vector<node_ptr> args;
        expect("(");
        if (!is(")")) {
            args.push_back(conditional());
            while (accept(",")) args.push_back(conditional());
        }
        expect(")");
        if (args.size() != want)
            fail_build(pos, (args.size() < want ? "too few" : "too many") + std::string(" arguments to '") + fn + "'");
        return args;
    }

    node_ptr call(const token& t)
    {
        const std::string& f = t.s;
        if (f == "min" || f == "max" || f == "fmin" || f == "fmax") {
            auto args = call_args(t.pos, f, 2);
            const bool fp = f[0] == 'f';
            if (fp && (is_int(args[0]->t) || is_int(args[1]->t)))
                fail_build(t.pos, "call to '" + f + "' with an integer argument is ambiguous");
            const elem c = args[0]->t == args[1]->t ? args[0]->t : common(args[0]->t, args[1]->t);
            node_ptr n = make(N_MINMAX, c);
            n->opt = of_ty(arith(c));
            n->op = (f == "min" || f == "fmin") ? K_MIN : K_MAX;
            n->a = std::move(args[0]);
            n->b = std::move(args[1]);
            return n;
        }
        if (f == "clamp") {
            auto args = call_args(t.pos, f, 3);
            elem c = args[0]->t;
            if (!(args[1]->t == c && args[2]->t == c)) c = common(common(c, args[1]->t), args[2]->t);
            node_ptr n = make(N_CLAMP, c);
            n->opt = of_ty(arith(c));
            n->a = std::move(args[0]);
            n->b = std::move(args[1]);
            n->c = std::move(args[2]);
            return n;
        }
        if (f == "abs" || f == "fabs") {
            auto args = call_args(t.pos, f, 1);
            const elem a = args[0]->t;
            if ((f == "abs") != is_int(a))
                fail_build(t.pos, "no matching function for call to '" + f + "' with an argument of type '" +
                                      elem_name(a) + "'");
            static const elem unsigned_of[] = {elem::u8,  elem::u8,  elem::u16, elem::u16, elem::u32,
                                               elem::u32, elem::u64, elem::u64, elem::f32, elem::f64};
            node_ptr n = make(N_ABS, unsigned_of[(int)a]);
            n->opt = a;
            n->a = std::move(args[0]);
            return n;
        }
        static const struct {
            const char* name;
            elem t;
        } types[] = {{"char", elem::i8},  {"uchar", elem::u8},   {"short", elem::i16}, {"ushort", elem::u16},
                     {"int", elem::i32},  {"uint", elem::u32},   {"long", elem::i64},  {"ulong", elem::u64},
                     {"float", elem::f32}, {"double", elem::f64}};
        if (f.compare(0, 3, "as_") == 0 || f.compare(0, 8, "convert_") == 0) {
            const bool as = f[0] == 'a';
            const std::string tn = f.substr(as ? 3 : 8);
            for (const auto& e : types)
                if (tn == e.name) {
                    auto args = call_args(t.pos, f, 1);
                    if (!as) return make_cast(e.t, std::move(args[0]));
                    if (elem_size(args[0]->t) != elem_size(e.t))
                        fail_build(t.pos, "invalid reinterpretation: sizes of '" + std::string(elem_name(args[0]->t)) +
                                              "' and '" + e.name + "' differ");
                    node_ptr n = make(N_BITCAST, e.t);
                    n->a = std::move(args[0]);
                    return n;
                }
            fail_unsupported("the built-in '" + f + "'");
        }
        static const char* known[] = {"sqrt", "rsqrt", "cbrt", "exp", "exp2", "exp10", "expm1", "log", "log2",
                                      "log10", "log1p", "pow", "pown", "powr", "sin", "cos", "tan", "asin",
                                      "acos", "atan", "atan2", "sinh", "cosh", "tanh", "floor", "ceil", "round",
                                      "trunc", "rint", "fmod", "remainder", "hypot", "mad", "fma", "mix", "step",
                                      "smoothstep", "sign", "select", "popcount", "clz", "ctz", "rotate",
                                      "hadd", "rhadd", "mul24", "mad24", "mul_hi", "mad_hi", "mad_sat",
                                      "add_sat", "sub_sat", "abs_diff", "upsample", "copysign", "fdim",
                                      "isnan", "isinf", "isfinite", "signbit", "native_sqrt", "native_exp",
                                      "native_log", "native_sin", "native_cos", "half_sqrt", "degrees",
                                      "radians", "ldexp", "frexp", "ilogb", "logb", "nextafter", "maxmag",
                                      "minmag", "erf", "erfc", "tgamma", "lgamma", "bitselect", "any", "all",
                                      "dot", "length", "distance", "normalize", "cross", "shuffle", "vload4",
                                      "get_global_id", "get_local_id"};
        for (const char* k : known)
            if (f == k) fail_unsupported("the built-in '" + f + "'");
        fail_build(t.pos, "implicit declaration of function '" + f + "'");
    }

    node_ptr primary()
    {
        const token t = peek();
        if (t.k == token::NUM) {
            ++at_;
            return number(t);
        }
        if (t.k == token::ID) {
            ++at_;
            if (is("(")) return call(t);
            if (t.s == "x") return make(N_X, tx_);
            if (t.s == "y" && has_y_) return make(N_Y, ty_);
            if (node_ptr c = constant(t.s)) return c;
            if (t.s == "M_PI" || t.s == "M_PI_F" || t.s == "M_E" || t.s == "M_E_F")
                fail_unsupported("the constant '" + t.s + "'");
            fail_build(t.pos, "use of undeclared identifier '" + t.s + "'");
        }
        if (accept("(")) {
            node_ptr e = expression();
            expect(")");
            if (is("[") || is(".") || is("->") || is("++") || is("--")) fail_build(peek().pos, "invalid postfix operator");
            return e;
        }
        if (t.k == token::END) fail_build(t.pos, "expected an expression at end of input");
        fail_build(t.pos, "expected an expression before '" + t.s + "'");
    }

    // ---- code generation ----
    void push_op(uint8_t kind, uint8_t t, uint8_t src = S_ACC, uint64_t imm = 0, uint8_t slot = 0, uint8_t t2 = 0)
    {
        if (prog_.nops >= (uint32_t)MAX_OPS) fail_unsupported("an expression longer than " + std::to_string(MAX_OPS) + " operations");
        op& o = prog_.ops[prog_.nops++];
        std::memset(&o, 0, sizeof(o));
        o.kind = kind;
        o.t = t;
        o.src = src;
        o.imm = imm;
        o.slot = slot;
        o.t2 = t2;
    }
    void need_slots(int sp, int count) const
    {
        if (sp + count > STACK) fail_unsupported("an expression nested deeper than " + std::to_string(STACK) + " temporaries");
    }

    // acc (holding a value of arithmetic type `from`) becomes a value of C type `to`
    void convert_to(ty from, elem to)
    {
        if (is_narrow(to)) {
            if (from != I32 && from != U32) push_op(K_CVT, from, S_ACC, 0, 0, I32);
            const uint8_t k = to == elem::i8 ? K_EXT8S : to == elem::u8 ? K_EXT8U : to == elem::i16 ? K_EXT16S : K_EXT16U;
            push_op(k, I32);
            return;
        }
        const ty t = arith(to);
        if (t == from) return;
        const bool same_bits = (t == I32 && from == U32) || (t == U32 && from == I32) || (t == I64 && from == U64) ||
                               (t == U64 && from == I64);
        if (!same_bits) push_op(K_CVT, from, S_ACC, 0, 0, t);
    }

    // a leaf usable directly as the operand of an operation of type t
    bool leaf(const node& e, ty t, uint8_t& src, uint64_t& imm) const
    {
        if (e.k == N_LIT) {
            src = S_IMM;
            imm = cv::convert(arith(e.t), t, e.bits);
            return true;
        }
        if ((e.k == N_X || e.k == N_Y) && arith(e.t) == t) {
            src = e.k == N_X ? S_X : S_Y;
            imm = 0;
            return true;
        }
        return false;
    }

    // acc = acc OP leaf; an integer literal divisor with |d| >= 2 divides by
    // multiplication
    void push_leaf_op(uint8_t kind, ty t, uint8_t src, uint64_t imm)
    {
        const bool integer = t == I32 || t == U32 || t == I64 || t == U64;
        if ((kind == K_DIV || kind == K_REM) && src == S_IMM && integer) {
            const int bits = (t == I32 || t == U32) ? 32 : 64;
            const bool sgn = t == I32 || t == I64;
            const int64_t sd = bits == 32 ? (int64_t)(int32_t)(uint32_t)imm : (int64_t)imm;
            const uint64_t ud = bits == 32 ? (uint64_t)(uint32_t)imm : imm;
            const bool ok = sgn ? (sd >= 2 || sd <= -2) : ud >= 2;
            if (ok) {
                uint64_t m = 0;
                int l = 0;
                if (sgn) magic_signed(bits, sd, m, l);
                else magic_unsigned(bits, ud, m, l);
                push_op(kind == K_DIV ? K_DIVC : K_REMC, t, S_IMM, imm, (uint8_t)l);
                prog_.ops[prog_.nops - 1].aux = m;
                return;
            }
        }
        push_op(kind, t, src, imm);
    }

    static uint8_t reversed(uint8_t k)
    {
        switch (k) {
        case K_SUB: return K_RSUB;
        case K_RSUB: return K_SUB;
        case K_DIV: return K_RDIV;
        case K_RDIV: return K_DIV;
        case K_REM: return K_RREM;
        case K_RREM: return K_REM;
        case K_SHL: return K_RSHL;
        case K_RSHL: return K_SHL;
        case K_SHR: return K_RSHR;
        case K_RSHR: return K_SHR;
        case K_LT: return K_GT;
        case K_GT: return K_LT;
        case K_LE: return K_GE;
        case K_GE: return K_LE;
        default: return k;  // commutative
        }
    }

    // acc = value of e converted to arithmetic type t
    void gen_as(const node& e, ty t, int sp)
    {
        gen(e, sp);
        convert_to(arith(e.t), of_ty(t));
    }

    // acc = a OP b, both converted to t
    // min / max of floating-point values keep their operand order: with a +0
    // and a -0 the first operand wins (OpenCL C max: y if x < y, otherwise x)
    static bool ordered_minmax(uint8_t kind, ty t) { return (kind == K_MIN || kind == K_MAX) && (t == F32 || t == F64); }

    void gen_binary(uint8_t kind, ty t, const node& a, const node& b, int sp)
    {
        uint8_t src;
        uint64_t imm;
        if (leaf(b, t, src, imm)) {
            gen_as(a, t, sp);
            push_leaf_op(kind, t, src, imm);
        } else if (ordered_minmax(kind, t)) {
            // b into a slot first, then acc = a OP slot
            gen_as(b, t, sp);
            need_slots(sp, 1);
            push_op(K_PUSH, t, S_ACC, 0, (uint8_t)sp);
            gen_as(a, t, sp + 1);
            push_op(kind, t, S_POP, 0, (uint8_t)sp);
        } else if (leaf(a, t, src, imm)) {
            gen_as(b, t, sp);
            push_op(reversed(kind), t, src, imm);
        } else {
            gen_as(a, t, sp);
            need_slots(sp, 1);
            push_op(K_PUSH, t, S_ACC, 0, (uint8_t)sp);
            gen_as(b, t, sp + 1);
            push_op(reversed(kind), t, S_POP, 0, (uint8_t)sp);
        }
    }

    // acc (already of type t) = acc OP b
    void gen_rhs(uint8_t kind, ty t, const node& b, int sp)
    {
        uint8_t src;
        uint64_t imm;
        if (leaf(b, t, src, imm)) {
            push_leaf_op(kind, t, src, imm);
            return;
        }
        need_slots(sp, 1);
        push_op(K_PUSH, t, S_ACC, 0, (uint8_t)sp);
        gen_as(b, t, sp + 1);
        push_op(reversed(kind), t, S_POP, 0, (uint8_t)sp);
    }

    // comparisons and logic already give an int 0 or 1
    static bool is_bool(const node& e)
    {
        return (e.k == N_BIN && ((e.op >= K_LT && e.op <= K_NE) || e.op == 100 || e.op == 101)) ||
               (e.k == N_UN && e.op == '!');
    }

    // acc = (e != 0) as an int 0 or 1
    void gen_truth(const node& e, int sp)
    {
        gen(e, sp);
        if (!is_bool(e)) push_op(K_NE, arith(e.t), S_IMM, 0);
    }

    void gen(const node& e, int sp)
    {
        switch (e.k) {
        case N_X: push_op(K_LOAD, arith(e.t), S_X); return;
        case N_Y: push_op(K_LOAD, arith(e.t), S_Y); return;
        case N_LIT: push_op(K_LOAD, arith(e.t), S_IMM, e.bits); return;
        case N_CAST: gen(*e.a, sp); convert_to(arith(e.a->t), e.t); return;
        case N_BITCAST:
            gen(*e.a, sp);
            if (is_narrow(e.t)) convert_to(I32, e.t);  // re-extend the low bits by the new signedness
            return;
        case N_UN: {
            const ty t = arith(e.t);
            if (e.op == '!') {
                gen(*e.a, sp);
                push_op(K_EQ, arith(e.a->t), S_IMM, 0);
            } else {
                gen_as(*e.a, t, sp);
                if (e.op == '-') push_op(K_NEG, t);
                else if (e.op == '~') push_op(K_NOT, t);
            }
            return;
        }
        case N_BIN: {
            if (e.op == 100 || e.op == 101) {  // && and || on truth values (no side effects to skip)
                gen_truth(*e.a, sp);
                need_slots(sp, 1);
                push_op(K_PUSH, I32, S_ACC, 0, (uint8_t)sp);
                gen_truth(*e.b, sp + 1);
                push_op(e.op == 100 ? K_AND : K_OR, I32, S_POP, 0, (uint8_t)sp);
                return;
            }
            gen_binary((uint8_t)e.op, arith(e.opt), *e.a, *e.b, sp);
            return;
        }
        case N_MINMAX: gen_binary((uint8_t)e.op, arith(e.opt), *e.a, *e.b, sp); return;
        case N_CLAMP: {  // min(max(a, b), c)
            const ty t = arith(e.opt);
            uint8_t src;
            uint64_t imm;
            if (ordered_minmax(K_MIN, t) && !leaf(*e.c, t, src, imm)) {
                // the upper bound into a slot first, so that min keeps its order
                gen_as(*e.c, t, sp);
                need_slots(sp, 1);
                push_op(K_PUSH, t, S_ACC, 0, (uint8_t)sp);
                gen_binary(K_MAX, t, *e.a, *e.b, sp + 1);
                push_op(K_MIN, t, S_POP, 0, (uint8_t)sp);
            } else {
                gen_binary(K_MAX, t, *e.a, *e.b, sp);
                gen_rhs(K_MIN, t, *e.c, sp);
            }
            if (is_narrow(e.t)) convert_to(I32, e.t);
            return;
        }
        case N_ABS: {
            gen(*e.a, sp);
            push_op(K_ABS, arith(e.opt));
            return;
        }
        case N_TERN: {
            const ty t = arith(e.opt);
            need_slots(sp, 2);
            gen(*e.a, sp);  // SEL tests the low 32 bits for nonzero
            if (arith(e.a->t) != I32 && arith(e.a->t) != U32) push_op(K_NE, arith(e.a->t), S_IMM, 0);
            push_op(K_PUSH, I32, S_ACC, 0, (uint8_t)sp);
            gen_as(*e.b, t, sp + 1);
            push_op(K_PUSH, t, S_ACC, 0, (uint8_t)(sp + 1));
            gen_as(*e.c, t, sp + 2);
            push_op(K_SEL, t, S_ACC, 0, (uint8_t)sp);
            return;
        }
        }
    }
};

}  // namespace

program compile(const std::string& text, elem tx, bool has_y, elem ty2, elem tout)
{
    compiler c(text, tx, has_y, ty2, "transform");
    node_ptr root = c.parse();
    program p = c.emit(*root, tout);
    p.x_elem = (uint8_t)tx;
    p.y_elem = (uint8_t)(has_y ? ty2 : tx);
    p.out_elem = (uint8_t)tout;
    p.has_y = has_y ? 1 : 0;
    p.x_ty = (uint8_t)arith(tx);
    p.y_ty = (uint8_t)arith(has_y ? ty2 : tx);
    return p;
}

program compile_predicate(const std::string& text, elem tx)
{
    compiler c(text, tx, false, tx, "copy_if");
    node_ptr root = c.parse();
    program p = c.emit_truth(*root);
    p.x_elem = p.y_elem = (uint8_t)tx;
    p.out_elem = (uint8_t)elem::i32;
    p.has_y = 0;
    p.x_ty = p.y_ty = (uint8_t)arith(tx);
    return p;
}

std::string listing(const program& p)
{
    static const char* kinds[] = {"load", "push", "add", "sub", "rsub", "mul", "div", "rdiv", "rem", "rrem", "and", "or",
                                  "xor", "shl", "rshl", "shr", "rshr", "lt", "le", "gt", "ge", "eq", "ne", "min",
                                  "max", "neg", "not", "abs", "cvt", "ext8s", "ext8u", "ext16s", "ext16u", "sel",
                                  "divc", "remc"};
    static const char* tys[] = {"i32", "u32", "i64", "u64", "f32", "f64"};
    std::ostringstream os;
    for (uint32_t k = 0; k < p.nops; ++k) {
        const op& o = p.ops[k];
        os << kinds[o.kind] << '.' << tys[o.t];
        if (o.kind == K_CVT) os << "->" << tys[o.t2];
        switch (o.src) {
        case S_IMM: os << " #0x" << std::hex << o.imm << std::dec; break;
        case S_X: os << " x"; break;
        case S_Y: os << " y"; break;
        case S_POP: os << " st" << (int)o.slot; break;
        default: break;
        }
        if (o.kind == K_PUSH || o.kind == K_SEL) os << " st" << (int)o.slot;
        if (o.kind == K_DIVC || o.kind == K_REMC) os << " m=0x" << std::hex << o.aux << std::dec << " l=" << (int)o.slot;
        os << '\n';
    }
    return os.str();
}

}  // namespace xp

// ---------------------------------------------------------------------------
// Device kernel
// ---------------------------------------------------------------------------
namespace {

using namespace xp;
using namespace xp::interp;

constexpr int THREADS = 256;

// One group: E consecutive elements of SZ bytes (E * SZ <= 16, a power of
// two, so one aligned vector access).
template <int SZ, typename W, int E> constexpr bool group_fits()
{
    return E * SZ <= 16 && (SZ < 8 || sizeof(W) == 8);
}

template <int BYTES> __device__ __forceinline__ void load_vec(const unsigned char* q, uint32_t (&w)[4])
{
    if constexpr (BYTES == 16) {
        const uint4 u = *reinterpret_cast<const uint4*>(q);
        w[0] = u.x, w[1] = u.y, w[2] = u.z, w[3] = u.w;
    } else if constexpr (BYTES == 8) {
        const uint2 u = *reinterpret_cast<const uint2*>(q);
        w[0] = u.x, w[1] = u.y;
    } else if constexpr (BYTES == 4) {
        w[0] = *reinterpret_cast<const uint32_t*>(q);
    } else {
        w[0] = *reinterpret_cast<const uint16_t*>(q);
    }
}

template <int BYTES> __device__ __forceinline__ void store_vec(unsigned char* q, const uint32_t (&w)[4])
{
    if constexpr (BYTES == 16) {
        *reinterpret_cast<uint4*>(q) = make_uint4(w[0], w[1], w[2], w[3]);
    } else if constexpr (BYTES == 8) {
        *reinterpret_cast<uint2*>(q) = make_uint2(w[0], w[1]);
    } else if constexpr (BYTES == 4) {
        *reinterpret_cast<uint32_t*>(q) = w[0];
    } else {
        *reinterpret_cast<uint16_t*>(q) = (uint16_t)w[0];
    }
}

// E elements starting at element index i (aligned), promoted into v[0..E)
template <typename W, int E>
__device__ __forceinline__ void load_group(const unsigned char* p, uint8_t e, int sz, std::size_t i, W* v)
{
    uint32_t w[4] = {0u, 0u, 0u, 0u};
    const unsigned char* q = p + i * sz;
    if (sz == 1) {
        if constexpr (group_fits<1, W, E>()) {
            load_vec<E>(q, w);
#pragma unroll
            for (int j = 0; j < E; ++j) v[j] = promote<W>(e, (w[j / 4] >> (8 * (j % 4))) & 0xFFu);
        }
    } else if (sz == 2) {
        if constexpr (group_fits<2, W, E>()) {
            load_vec<2 * E>(q, w);
#pragma unroll
            for (int j = 0; j < E; ++j) v[j] = promote<W>(e, (w[j / 2] >> (16 * (j % 2))) & 0xFFFFu);
        }
    } else if (sz == 4) {
        if constexpr (group_fits<4, W, E>()) {
            load_vec<4 * E>(q, w);
#pragma unroll
            for (int j = 0; j < E; ++j) v[j] = (W)w[j];
        }
    } else {
        if constexpr (group_fits<8, W, E>()) {
            load_vec<8 * E>(q, w);
#pragma unroll
            for (int j = 0; j < E; ++j) v[j] = (W)(((uint64_t)w[2 * j + 1] << 32) | w[2 * j]);
        }
    }
}

template <typename W, int E>
__device__ __forceinline__ void store_group(unsigned char* p, int sz, std::size_t i, const W* v)
{
    uint32_t w[4] = {0u, 0u, 0u, 0u};
    unsigned char* q = p + i * sz;
    if (sz == 1) {
        if constexpr (group_fits<1, W, E>()) {
#pragma unroll
            for (int j = 0; j < E; ++j) w[j / 4] |= ((uint32_t)v[j] & 0xFFu) << (8 * (j % 4));
            store_vec<E>(q, w);
        }
    } else if (sz == 2) {
        if constexpr (group_fits<2, W, E>()) {
#pragma unroll
            for (int j = 0; j < E; ++j) w[j / 2] |= ((uint32_t)v[j] & 0xFFFFu) << (16 * (j % 2));
            store_vec<2 * E>(q, w);
        }
    } else if (sz == 4) {
        if constexpr (group_fits<4, W, E>()) {
#pragma unroll
            for (int j = 0; j < E; ++j) w[j] = (uint32_t)v[j];
            store_vec<4 * E>(q, w);
        }
    } else {
        if constexpr (group_fits<8, W, E>()) {
#pragma unroll
            for (int j = 0; j < E; ++j) {
                w[2 * j] = (uint32_t)(uint64_t)v[j];
                w[2 * j + 1] = (uint32_t)((uint64_t)v[j] >> 32);
            }
            store_vec<8 * E>(q, w);
        }
    }
}

__device__ __forceinline__ uint64_t load_one(const unsigned char* p, int sz, std::size_t i)
{
    const unsigned char* q = p + i * sz;
    if (sz == 1) return *q;
    if (sz == 2) return *reinterpret_cast<const uint16_t*>(q);
    if (sz == 4) return *reinterpret_cast<const uint32_t*>(q);
    return *reinterpret_cast<const uint64_t*>(q);
}

__device__ __forceinline__ void store_one(unsigned char* p, int sz, std::size_t i, uint64_t r)
{
    unsigned char* q = p + i * sz;
    if (sz == 1) *q = (uint8_t)r;
    else if (sz == 2) *reinterpret_cast<uint16_t*>(q) = (uint16_t)r;
    else if (sz == 4) *reinterpret_cast<uint32_t*>(q) = (uint32_t)r;
    else *reinterpret_cast<uint64_t*>(q) = r;
}

// One CTA per chunk of THREADS x E x K elements. Element (k, j) of thread t
// is chunk + (k * THREADS + t) * E + j: each group of E consecutive elements
// is one vector access and a warp's groups are contiguous, so every warp
// access is a run of 32 vectors. All loads of a thread are issued before
// the program runs. (Measured on GB300 copies: this one-shot, lane-strided
// form reaches the copy peak; grid-stride loops, 32 contiguous bytes per
// thread and L2 bulk prefetch ahead each lose 10-25%.)
template <typename W, int E, int K, bool HAS_Y, bool STK>
__global__ void __launch_bounds__(THREADS)
    k_transform(const unsigned char* x, const unsigned char* y, unsigned char* out, std::size_t n, int aligned,
                const __grid_constant__ program p)
{
    constexpr int V = E * K;
    extern __shared__ __align__(16) unsigned char transform_smem[];
    W* st = reinterpret_cast<W*>(transform_smem);
    const int sx = elem_size_dev(p.x_elem), sy = elem_size_dev(p.y_elem), so = elem_size_dev(p.out_elem);
    const std::size_t chunk = (std::size_t)blockIdx.x * THREADS * V;
    const bool whole = aligned && chunk + (std::size_t)THREADS * V <= n;
    W xv[V], yv[V], acc[V];
    if (whole) {
#pragma unroll
        for (int k = 0; k < K; ++k) {
            const std::size_t i = chunk + ((std::size_t)k * THREADS + threadIdx.x) * E;
            load_group<W, E>(x, p.x_elem, sx, i, xv + k * E);
            if (HAS_Y) load_group<W, E>(y, p.y_elem, sy, i, yv + k * E);
        }
    } else {
#pragma unroll
        for (int k = 0; k < K; ++k)
#pragma unroll
            for (int j = 0; j < E; ++j) {
                const std::size_t i = chunk + ((std::size_t)k * THREADS + threadIdx.x) * E + j;
                uint64_t rx = 0, ry = 0;
                if (i < n) {
                    rx = load_one(x, sx, i);
                    if (HAS_Y) ry = load_one(y, sy, i);
                }
                xv[k * E + j] = sx == 8 ? (W)rx : promote<W>(p.x_elem, (uint32_t)rx);
                if (HAS_Y) yv[k * E + j] = sy == 8 ? (W)ry : promote<W>(p.y_elem, (uint32_t)ry);
            }
    }
    if (!HAS_Y) {
#pragma unroll
        for (int j = 0; j < V; ++j) yv[j] = 0;
    }
    run_program<W, V, STK, THREADS>(p, acc, xv, yv, st);
    if (whole) {
#pragma unroll
        for (int k = 0; k < K; ++k)
            store_group<W, E>(out, so, chunk + ((std::size_t)k * THREADS + threadIdx.x) * E, acc + k * E);
    } else {
#pragma unroll
        for (int k = 0; k < K; ++k)
#pragma unroll
            for (int j = 0; j < E; ++j) {
                const std::size_t i = chunk + ((std::size_t)k * THREADS + threadIdx.x) * E + j;
                if (i < n) store_one(out, so, i, (uint64_t)acc[k * E + j]);
            }
    }
}

template <typename W, int E, int K, bool HAS_Y, bool STK>
void launch_variant(device_context& ctx, const program& p, const void* x, const void* y, void* out, std::size_t n,
                    int aligned)
{
    constexpr int V = E * K;
    auto kernel = &k_transform<W, E, K, HAS_Y, STK>;
    const std::size_t smem = STK ? (std::size_t)STACK * V * THREADS * sizeof(W) : 0;
    if (smem > 48 * 1024 && first_use_on_device((const void*)kernel))
        check_cuda(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem),
                   "cudaFuncSetAttribute");
    const std::size_t chunks = (n + (std::size_t)THREADS * V - 1) / ((std::size_t)THREADS * V);
    kernel<<<(unsigned)chunks, THREADS, smem, ctx.stream>>>(static_cast<const unsigned char*>(x),
                                                           static_cast<const unsigned char*>(y),
                                                           static_cast<unsigned char*>(out), n, aligned, p);
    check_cuda(cudaGetLastError(), "transform launch");
}

template <bool HAS_Y>
void launch(device_context& ctx, const program& p, const void* x, const void* y, void* out, std::size_t n, int aligned)
{
    // Registers: 32-bit when every type is 32-bit, else 64-bit. Group width
    // E: one 16-byte vector of the widest element type. Groups per thread K
    // for the common shapes (no stack, widest element 4 or 8 bytes): the
    // tuning table's "transform:32" / "transform:64" variant v gives K = 2^v.
    // Defaults measured on GB300 over 2^30 elements: K = 2 for 32-bit
    // programs (copy and x + y at the copy peak; K = 1 and 4 lose 4-7%),
    // K = 1 for 64-bit ones (f64 x + y: 0.73 of peak against 0.61 at K = 2).
    const bool stack = uses_stack(p);
    const int wide = widest(p);
    const bool w32 = all_32bit(p);
    launch_shape shape;
    const int kv = ctx.tuning.lookup(w32 ? "transform:32" : "transform:64", shape) ? shape.variant : (w32 ? 1 : 0);
    if (!w32) {
        if (wide == 8) {
            if (stack) launch_variant<uint64_t, 2, 2, HAS_Y, true>(ctx, p, x, y, out, n, aligned);
            else if (kv == 0) launch_variant<uint64_t, 2, 1, HAS_Y, false>(ctx, p, x, y, out, n, aligned);
            else if (kv == 2) launch_variant<uint64_t, 2, 4, HAS_Y, false>(ctx, p, x, y, out, n, aligned);
            else launch_variant<uint64_t, 2, 2, HAS_Y, false>(ctx, p, x, y, out, n, aligned);
        } else {
            if (stack) launch_variant<uint64_t, 4, 1, HAS_Y, true>(ctx, p, x, y, out, n, aligned);
            else launch_variant<uint64_t, 4, 1, HAS_Y, false>(ctx, p, x, y, out, n, aligned);
        }
    } else if (wide == 4) {
        if (stack) launch_variant<uint32_t, 4, 2, HAS_Y, true>(ctx, p, x, y, out, n, aligned);
        else if (kv == 0) launch_variant<uint32_t, 4, 1, HAS_Y, false>(ctx, p, x, y, out, n, aligned);
        else if (kv == 2) launch_variant<uint32_t, 4, 4, HAS_Y, false>(ctx, p, x, y, out, n, aligned);
        else launch_variant<uint32_t, 4, 2, HAS_Y, false>(ctx, p, x, y, out, n, aligned);
    } else if (stack || wide == 2) {
        if (stack) launch_variant<uint32_t, 8, 1, HAS_Y, true>(ctx, p, x, y, out, n, aligned);
        else launch_variant<uint32_t, 8, 1, HAS_Y, false>(ctx, p, x, y, out, n, aligned);
    } else {
        launch_variant<uint32_t, 16, 1, HAS_Y, false>(ctx, p, x, y, out, n, aligned);
    }
}

}  // namespace

void transform(device_context& ctx, const program& p, const void* x, const void* y, void* out, std::size_t n)
{
    if (n == 0) return;
    check_size(n);
    if (p.nops == 0 || p.nops > (uint32_t)MAX_OPS) throw std::invalid_argument("transform: empty program");
    if (p.has_y && y == nullptr) throw std::invalid_argument("transform: missing second input");
    ctx.activate();
    auto al = [](const void* q) { return q == nullptr || (reinterpret_cast<uintptr_t>(q) & 15) == 0; };
    const int aligned = (al(x) && al(y) && al(out)) ? 1 : 0;
    kernel_timer kt(ctx, "transform");
    if (p.has_y) launch<true>(ctx, p, x, y, out, n, aligned);
    else launch<false>(ctx, p, x, nullptr, out, n, aligned);
}

}  // namespace gbc
