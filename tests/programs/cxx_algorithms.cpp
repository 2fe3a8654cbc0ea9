// A C++ caller of the reference's algorithm API, compiled against
// include/gbcompute/compute.hpp and linked with libgbcompute.so. It runs the
// algorithm cases of the reference's C++ test (lib/test/Compute/
// main.cpp:184-451) with the same recipes -- sizes {0, 1, 7, 255, 256, 1000,
// 4097, 100003, 2^20}, mt19937(seed) + uniform_int_distribution inputs,
// seeds n (reduce), n+1 (scan), n+2 (sort), n+3 (copy_if and histogram) --
// and checks every result on the host: sequence/transform/fill, reduce with
// plus/min/max, inclusive/exclusive/in-place scans with the right projection
// and the max operator, sort_by_key against std::stable_sort, stability with
// many duplicates, signed and float keys (descending, with -0 and +-inf),
// copy_if and a 10-bin histogram; the static_map and bitpack compression
// cases of main.cpp:337-451 (a 200,000-key map, finds of present and absent
// keys, the overflow of a 4-slot table; three inputs x delta x two chunk
// sizes round-tripped through compression and serialization, the > 4x ratio
// of delta-coded timestamps, a rejected blob); plus the facade's
// exceptions. Exit status = failed checks.
#include <gbcompute/compute.hpp>

#include <algorithm>
#include <climits>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <numeric>
#include <random>
#include <utility>
#include <vector>

namespace cc = cl::compute;

namespace {

int failed = 0, total = 0;

void expect(bool ok, const char* what, int line)
{
    ++total;
    if (!ok) {
        ++failed;
        std::fprintf(stderr, "check failed at line %d: %s\n", line, what);
    }
}
#define EXPECT(c) expect(static_cast<bool>(c), #c, __LINE__)

template <typename F> bool throws_invalid(F&& f)
{
    try {
        f();
    } catch (const std::invalid_argument&) {
        return true;
    } catch (...) {
    }
    return false;
}

std::vector<cl_uint> uniform(std::size_t n, cl_uint hi, unsigned seed)
{
    std::mt19937 gen(seed);
    std::uniform_int_distribution<cl_uint> d(0, hi);
    std::vector<cl_uint> v(n);
    for (auto& x : v) x = d(gen);
    return v;
}

const std::size_t kSizes[] = {0, 1, 7, 255, 256, 1000, 4097, 100003, std::size_t(1) << 20};

void elementwise(cc::compute_context& ctx)
{
    for (std::size_t n : kSizes) {
        cc::device_buffer<cl_int> seq(ctx, n);
        cc::sequence(ctx, seq, cl_int(5), cl_int(3));
        std::vector<cl_int> want(n);
        for (std::size_t i = 0; i < n; ++i) want[i] = 5 + 3 * cl_int(i);
        EXPECT(seq.to_host(ctx) == want);

        cc::device_buffer<cl_float> half(ctx, n);
        cc::transform(ctx, seq, half, "(float)x * 0.5f");
        std::vector<cl_float> hw(n);
        for (std::size_t i = 0; i < n; ++i) hw[i] = float(want[i]) * 0.5f;
        EXPECT(half.to_host(ctx) == hw);

        cc::device_buffer<cl_int> sq(ctx, n);
        cc::transform(ctx, seq, seq, sq, "x * y - 1");
        std::vector<cl_int> sw(n);
        for (std::size_t i = 0; i < n; ++i)
            sw[i] = cl_int(uint32_t(want[i]) * uint32_t(want[i]) - 1u);  // wraps as OpenCL C int does
        EXPECT(sq.to_host(ctx) == sw);

        cc::fill(ctx, half, 2.5f);
        EXPECT(half.to_host(ctx) == std::vector<cl_float>(n, 2.5f));
    }
}

void reductions(cc::compute_context& ctx)
{
    for (std::size_t n : kSizes) {
        const auto h = uniform(n, 1000, unsigned(n));
        auto b = cc::device_buffer<cl_uint>::from_host(ctx, h);
        EXPECT(cc::reduce(ctx, b, cc::ops::plus(), cl_uint(7)) == std::accumulate(h.begin(), h.end(), cl_uint(7)));
        if (n != 0) {
            EXPECT(cc::reduce(ctx, b, cc::ops::maximum<cl_uint>(), cl_uint(0)) == *std::max_element(h.begin(), h.end()));
            EXPECT(cc::reduce(ctx, b, cc::ops::minimum<cl_uint>(), cl_uint(0xFFFFFFFFu)) ==
                   *std::min_element(h.begin(), h.end()));
        }
    }
    std::vector<cl_float> f(10000);
    for (std::size_t i = 0; i < f.size(); ++i) f[i] = float(int(i % 17) - 8);
    auto fb = cc::device_buffer<cl_float>::from_host(ctx, f);
    EXPECT(cc::reduce(ctx, fb, cc::ops::maximum<cl_float>(), -INFINITY) == 8.0f);
    EXPECT(cc::reduce(ctx, fb, cc::ops::minimum<cl_float>(), INFINITY) == -8.0f);
}

void scans(cc::compute_context& ctx)
{
    for (std::size_t n : kSizes) {
        const auto h = uniform(n, 100, unsigned(n) + 1);
        auto in = cc::device_buffer<cl_uint>::from_host(ctx, h);
        cc::device_buffer<cl_uint> out(ctx, n);
        std::vector<cl_uint> inc(n), exc(n);
        cl_uint acc = 0;
        for (std::size_t i = 0; i < n; ++i) {
            exc[i] = acc;
            inc[i] = acc += h[i];
        }
        cc::inclusive_scan(ctx, in, out);
        EXPECT(out.to_host(ctx) == inc);
        cc::exclusive_scan(ctx, in, out);
        EXPECT(out.to_host(ctx) == exc);
        cc::inclusive_scan(ctx, in, in);
        EXPECT(in.to_host(ctx) == inc);
    }
    // the right projection reproduces its input only when operands are
    // combined in sequence order
    std::vector<cl_int> v(5000);
    for (std::size_t i = 0; i < v.size(); ++i) v[i] = cl_int(i * 7 % 101);
    auto vb = cc::device_buffer<cl_int>::from_host(ctx, v);
    cc::device_buffer<cl_int> vo(ctx, v.size());
    cc::inclusive_scan(ctx, vb, vo, cc::binary_op{"b", "0"});
    EXPECT(vo.to_host(ctx) == v);
    cc::inclusive_scan(ctx, vb, vo, cc::ops::maximum<cl_int>());
    std::vector<cl_int> running(v.size());
    cl_int m = INT_MIN;
    for (std::size_t i = 0; i < v.size(); ++i) running[i] = m = std::max(m, v[i]);
    EXPECT(vo.to_host(ctx) == running);

    // extension: the exact 64-bit total beside an exclusive scan
    std::vector<cl_int> big(300001);
    for (std::size_t i = 0; i < big.size(); ++i) big[i] = cl_int(2000000000 - int(i % 7));
    auto bb = cc::device_buffer<cl_int>::from_host(ctx, big);
    cc::device_buffer<cl_int> bo(ctx, big.size());
    const int64_t t = cc::exclusive_scan_total(ctx, bb, bo);
    EXPECT(t == std::accumulate(big.begin(), big.end(), int64_t(0)));
}

void sorts(cc::compute_context& ctx)
{
    for (std::size_t n : kSizes) {
        const auto keys = uniform(n, 0xFFFFFFFFu, unsigned(n) + 2);
        std::vector<cl_uint> idx(n);
        std::iota(idx.begin(), idx.end(), 0u);
        auto kb = cc::device_buffer<cl_uint>::from_host(ctx, keys);
        auto vb = cc::device_buffer<cl_uint>::from_host(ctx, idx);
        cc::sort_by_key(ctx, kb, vb);
        std::vector<cl_uint> order(idx);
        std::stable_sort(order.begin(), order.end(), [&](cl_uint a, cl_uint b) { return keys[a] < keys[b]; });
        std::vector<cl_uint> sk(n);
        for (std::size_t i = 0; i < n; ++i) sk[i] = keys[order[i]];
        EXPECT(kb.to_host(ctx) == sk);
        EXPECT(vb.to_host(ctx) == order);
    }

    // stability: 50,000 keys in [0, 15]
    const auto dup = uniform(50000, 15, 99);
    std::vector<cl_uint> pos(dup.size());
    std::iota(pos.begin(), pos.end(), 0u);
    auto db = cc::device_buffer<cl_uint>::from_host(ctx, dup);
    auto pb = cc::device_buffer<cl_uint>::from_host(ctx, pos);
    cc::sort_by_key(ctx, db, pb);
    const auto k = db.to_host(ctx), p = pb.to_host(ctx);
    bool stable = true;
    for (std::size_t i = 1; i < k.size(); ++i)
        if (k[i - 1] > k[i] || (k[i - 1] == k[i] && p[i - 1] > p[i])) stable = false;
    EXPECT(stable);

    // signed keys
    std::vector<cl_int> ints{5, -3, 0, INT_MIN, 7, -1, INT_MAX, 2};
    auto ib = cc::device_buffer<cl_int>::from_host(ctx, ints);
    cc::sort(ctx, ib);
    auto si = ints;
    std::sort(si.begin(), si.end());
    EXPECT(ib.to_host(ctx) == si);

    // float keys, descending, with -0, +inf and -inf; compared by bit pattern
    // in the order of the reference's key bijection (+0 before -0 descending)
    std::vector<cl_float> fl(3000);
    std::mt19937 gen(5);
    std::uniform_real_distribution<float> d(-1e6f, 1e6f);
    for (auto& x : fl) x = d(gen);
    fl[0] = -0.0f;
    fl[1] = INFINITY;
    fl[2] = -INFINITY;
    auto fb = cc::device_buffer<cl_float>::from_host(ctx, fl);
    cc::sort(ctx, fb, true);
    auto ordered = [](float x) {
        uint32_t u;
        std::memcpy(&u, &x, 4);
        return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
    };
    auto sf = fl;
    std::stable_sort(sf.begin(), sf.end(), [&](float a, float b) { return ordered(a) > ordered(b); });
    const auto got = fb.to_host(ctx);
    EXPECT(got.size() == sf.size() && std::memcmp(got.data(), sf.data(), 4 * sf.size()) == 0);
}

void select_and_histogram(cc::compute_context& ctx)
{
    for (std::size_t n : kSizes) {
        const auto h = uniform(n, 1000, unsigned(n) + 3);
        auto in = cc::device_buffer<cl_uint>::from_host(ctx, h);
        cc::device_buffer<cl_uint> out(ctx, n);
        const std::size_t kept = cc::copy_if(ctx, in, out, "(x % 3u) == 0u");
        std::vector<cl_uint> want;
        for (cl_uint x : h)
            if (x % 3 == 0) want.push_back(x);
        EXPECT(kept == want.size());
        auto got = out.to_host(ctx);
        got.resize(kept);
        EXPECT(got == want);

        cc::device_buffer<cl_uint> hist(ctx, 10);
        cc::histogram_even(ctx, in, hist, 0.0, 1000.0);
        std::vector<cl_uint> hw(10, 0);
        for (cl_uint x : h)
            if (x < 1000) ++hw[x / 100];
        EXPECT(hist.to_host(ctx) == hw);
    }
}

void hash_map(cc::compute_context& ctx)
{
    const std::size_t n = 200000;
    std::vector<cl_uint> keys(n), values(n);
    for (std::size_t i = 0; i < n; ++i) {
        keys[i] = cl_uint(uint64_t(i) * 2654435761u % 0xFFFFFFF0u);  // distinct
        values[i] = cl_uint(i);
    }
    cc::static_map map(ctx, n * 2);
    auto kb = cc::device_buffer<cl_uint>::from_host(ctx, keys);
    auto vb = cc::device_buffer<cl_uint>::from_host(ctx, values);
    EXPECT(map.insert(kb, vb) == n);
    EXPECT(map.size() == n);
    EXPECT(map.insert(kb, vb) == 0);  // present keys keep their values
    std::vector<cl_uint> q(keys.begin(), keys.begin() + 1000);
    for (cl_uint i = 0; i < 1000; ++i) q.push_back(0xFFFFFFF1u + i % 14);
    auto qb = cc::device_buffer<cl_uint>::from_host(ctx, q);
    cc::device_buffer<cl_uint> found(ctx, q.size());
    map.find(qb, found);
    const auto fv = found.to_host(ctx);
    bool ok = true;
    for (std::size_t i = 0; i < q.size(); ++i) ok = ok && fv[i] == (i < 1000 ? values[i] : map.empty_value());
    EXPECT(ok);
    cc::device_buffer<cl_uchar> present(ctx, q.size());
    map.contains(qb, present);
    const auto pv = present.to_host(ctx);
    EXPECT(std::count(pv.begin(), pv.end(), cl_uchar(1)) == 1000);
    EXPECT(map.slot_keys().size() == map.capacity());

    cc::static_map tiny(ctx, 4);
    bool overflow = false;
    try {
        tiny.insert(kb, vb, 10);
    } catch (const std::overflow_error&) {
        overflow = true;
    }
    EXPECT(overflow && tiny.size() == 4);
    tiny.clear();
    EXPECT(tiny.size() == 0);
}

void compression(cc::compute_context& ctx)
{
    std::mt19937 ticks(11);
    for (std::size_t n : kSizes) {
        std::vector<cl_uint> ts(n);  // slowly increasing timestamps
        cl_uint t = 1700000000u;
        for (auto& x : ts) x = t += ticks() % 50;
        auto small = uniform(n, 300, unsigned(n) + 4);  // small range
        for (auto& x : small) x += 5000000u;
        const auto noise = uniform(n, 0xFFFFFFFFu, unsigned(n) + 5);  // incompressible
        const std::vector<cl_uint>* inputs[] = {&ts, &small, &noise};
        for (const auto* input : inputs)
            for (bool delta : {false, true})
                for (std::size_t chunk : {std::size_t(256), std::size_t(2048)}) {
                    auto in = cc::device_buffer<cl_uint>::from_host(ctx, *input);
                    cc::bitpack_options opt;
                    opt.delta = delta;
                    opt.chunk_size = chunk;
                    const auto packed = cc::compress_bitpack(ctx, in, opt);
                    cc::device_buffer<cl_uint> out(ctx, n);
                    cc::decompress_bitpack(ctx, packed, out);
                    EXPECT(out.to_host(ctx) == *input);
                    const auto restored = cc::compressed_buffer::deserialize(ctx, packed.serialize(ctx));
                    cc::device_buffer<cl_uint> out2(ctx, n);
                    cc::decompress_bitpack(ctx, restored, out2);
                    EXPECT(out2.to_host(ctx) == *input);
                }
        if (n == (std::size_t(1) << 20)) {
            auto in = cc::device_buffer<cl_uint>::from_host(ctx, ts);
            cc::bitpack_options opt;
            opt.delta = true;
            const auto packed = cc::compress_bitpack(ctx, in, opt);
            EXPECT(double(packed.uncompressed_bytes()) / double(packed.compressed_bytes()) > 4.0);
        }
    }
    bool rejected = false;
    try {
        cc::compressed_buffer::deserialize(ctx, std::vector<unsigned char>(64, 0));
    } catch (const std::invalid_argument&) {
        rejected = true;
    }
    EXPECT(rejected);
}

void facade_errors(cc::compute_context& ctx)
{
    cc::device_buffer<cl_uint> small(ctx, 10), large(ctx, 20);
    EXPECT(throws_invalid([&] { cc::inclusive_scan(ctx, large, small); }));
    EXPECT(throws_invalid([&] { cc::sort_by_key(ctx, large, small); }));
    EXPECT(throws_invalid([&] { cc::copy_if(ctx, large, small, "x > 1u"); }));
    bool range = false;
    try {
        cl_uint tmp[4] = {0, 0, 0, 0};
        small.copy_to_host(ctx.queue(), tmp, 4, 8);
    } catch (const std::out_of_range&) {
        range = true;
    }
    EXPECT(range);
    bool build = false;
    try {
        cc::transform(ctx, small, small, "x +* nonsense");
    } catch (const cc::build_error& e) {
        build = std::strstr(e.what(), "build log") != nullptr;
    }
    EXPECT(build);
    bool unsupported = false;
    try {
        cc::reduce(ctx, small, cc::binary_op{"(a - b)", "0"}, cl_uint(0));
    } catch (const cc::unsupported_error&) {
        unsupported = true;
    }
    EXPECT(unsupported);
    // buffers move; the moved-from one is empty
    cc::device_buffer<cl_uint> moved(std::move(large));
    EXPECT(large.empty() && moved.size() == 20);
    ctx.queue().finish();
    EXPECT(ctx.memory_stats().current_allocations >= 2);
}

}  // namespace

int main()
{
    try {
        cc::compute_context ctx;
        elementwise(ctx);
        reductions(ctx);
        scans(ctx);
        sorts(ctx);
        select_and_histogram(ctx);
        hash_map(ctx);
        compression(ctx);
        facade_errors(ctx);
    } catch (const std::exception& e) {
        std::fprintf(stderr, "unexpected exception: %s\n", e.what());
        return 100;
    }
    std::printf("%d of %d checks failed\n", failed, total);
    return failed;
}
