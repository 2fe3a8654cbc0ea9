// Host-only checks of the stream-ordered slab arena (opencl-sdk_gb300/csrc/
// arena.hpp) over a fake upstream whose allocations can be made to fail: slab
// sharing, best fit, merging of freed neighbours, the retain limit, the
// statistics a caller reads, and one retry after idle slabs are handed back
// when the upstream runs out of memory (the observable behaviour of the
// reference's pool, lib/src/Compute/MemoryResource.cpp:77-88). Exit status =
// number of failed checks.
#include "arena.hpp"

#include <cstdio>
#include <cstdlib>
#include <iterator>
#include <map>
#include <random>
#include <vector>

static int failures = 0;
#define CHECK(c)                                                           \
    do {                                                                   \
        if (!(c)) {                                                        \
            ++failures;                                                    \
            std::fprintf(stderr, "FAILED: %s at line %d\n", #c, __LINE__); \
        }                                                                  \
    } while (0)

struct fake_upstream : gbc::memory_resource {
    std::size_t live_bytes = 0, allocs = 0, frees = 0, limit = ~std::size_t(0);
    std::map<void*, std::size_t> live;
    void* do_allocate(std::size_t b) override
    {
        if (live_bytes + b > limit) throw gbc::out_of_memory("fake upstream: out of memory");
        void* p = std::aligned_alloc(256, (b + 255) / 256 * 256);
        live[p] = b;
        live_bytes += b;
        ++allocs;
        return p;
    }
    void do_deallocate(void* p, std::size_t b) noexcept override
    {
        if (live.count(p) == 0 || live[p] != b) std::abort();  // a slab handed back twice or resized
        live.erase(p);
        live_bytes -= b;
        ++frees;
        std::free(p);
    }
};

static const std::size_t KiB = 1024, MiB = 1024 * 1024;

int main()
{
    auto up = std::make_shared<fake_upstream>();
    gbc::stream_arena::config cfg;
    cfg.slab_bytes = 1 * MiB;
    cfg.own_slab_round = 64 * KiB;
    cfg.retain_bytes = 8 * MiB;
    auto arena = std::make_shared<gbc::stream_arena>(up, cfg);

    // small requests share one slab, at 256-byte alignment
    char* a = static_cast<char*>(arena->allocate(100));
    char* b = static_cast<char*>(arena->allocate(300));
    CHECK(up->allocs == 1);
    CHECK(b == a + 256);
    CHECK(reinterpret_cast<std::uintptr_t>(a) % 256 == 0);
    auto u = arena->stats();
    CHECK(u.current_bytes == 400 && u.current_allocations == 2 && u.held_bytes == 1 * MiB);
    CHECK(u.idle_bytes == 1 * MiB - 256 - 512);

    // a freed block is taken again at once (stream-ordered reuse)
    arena->deallocate(a, 100);
    char* c = static_cast<char*>(arena->allocate(200));
    CHECK(c == a);

    // freed neighbours merge: a block spanning both is carved where they were
    arena->deallocate(c, 200);
    arena->deallocate(b, 300);
    CHECK(arena->stats().idle_bytes == 1 * MiB);
    char* d = static_cast<char*>(arena->allocate(700));
    CHECK(d == a);
    arena->deallocate(d, 700);

    // best fit: the smallest free range that holds the request is used
    std::vector<char*> p;
    for (int i = 0; i < 6; ++i) p.push_back(static_cast<char*>(arena->allocate(KiB)));
    arena->deallocate(p[1], KiB);                         // a 1 KiB hole
    arena->deallocate(p[3], KiB);
    arena->deallocate(p[4], KiB);                         // a 2 KiB hole
    char* e = static_cast<char*>(arena->allocate(1500));  // fits only the 2 KiB hole
    CHECK(e == p[3]);
    char* f = static_cast<char*>(arena->allocate(900));  // the 1 KiB hole is the best fit
    CHECK(f == p[1]);
    for (char* q : {p[0], f, p[2], e, p[5]}) arena->deallocate(q, 0);
    CHECK(arena->stats().current_allocations == 0);
    CHECK(up->allocs == 1);

    // a large request gets a slab of its own, rounded to own_slab_round
    void* big = arena->allocate(3 * MiB + 1);
    CHECK(up->allocs == 2);
    CHECK(up->live[big] == 3 * MiB + 64 * KiB);
    arena->deallocate(big, 3 * MiB + 1);
    // ... and serves a smaller large request later without a new slab
    void* big2 = arena->allocate(2 * MiB);
    CHECK(big2 == big && up->allocs == 2);
    arena->deallocate(big2, 2 * MiB);

    // beyond the retain limit, empty slabs go back to the upstream
    void* huge = arena->allocate(6 * MiB);
    CHECK(up->allocs == 3);
    arena->deallocate(huge, 6 * MiB);
    CHECK(arena->stats().idle_bytes <= 8 * MiB);
    CHECK(up->frees >= 1);

    // statistics over everything so far
    u = arena->stats();
    CHECK(u.current_bytes == 0 && u.current_allocations == 0);
    CHECK(u.peak_bytes == 6 * MiB);
    CHECK(u.total_allocations == 15);

    // out of memory: idle slabs are handed back and the request retried once
    CHECK(up->live_bytes > 0);
    up->limit = 5 * MiB;  // with the idle slabs held (4 MiB + 64 KiB), a 4 MiB slab does not fit
    void* g = arena->allocate(4 * MiB);
    CHECK(g != nullptr);
    CHECK(up->live_bytes == 4 * MiB);
    arena->deallocate(g, 4 * MiB);

    // out of memory with nothing idle to hand back: the error reaches the caller
    arena->trim();
    CHECK(up->live_bytes == 0);
    up->limit = 0;
    bool threw = false;
    try {
        arena->allocate(10);
    } catch (const gbc::out_of_memory&) {
        threw = true;
    }
    CHECK(threw);
    CHECK(arena->stats().current_allocations == 0);

    // a shared slab that does not fit falls back to a slab of the request's size
    up->limit = 4 * KiB;
    void* h = arena->allocate(1000);
    CHECK(h != nullptr && up->live_bytes == 1024);
    arena->deallocate(h, 1000);
    up->limit = ~std::size_t(0);
    arena->trim();

    // temp_buffer hands its block back on scope exit; zero bytes take nothing
    {
        gbc::temp_buffer t(arena, 100);
        CHECK(t.get() != nullptr);
        gbc::temp_buffer z(arena, 0);
        CHECK(z.get() == nullptr);
        CHECK(arena->stats().current_allocations == 1);
    }
    CHECK(arena->stats().current_allocations == 0);

    // random churn: live blocks never overlap, everything is accounted for
    std::mt19937 rng(7);
    std::map<char*, std::size_t> live;
    for (int step = 0; step < 20000; ++step) {
        if (live.empty() || rng() % 3 != 0) {
            const std::size_t n = 1 + rng() % (rng() % 8 == 0 ? 3 * MiB : 64 * KiB);
            char* q = static_cast<char*>(arena->allocate(n));
            auto next = live.lower_bound(q);
            if (next != live.end()) CHECK(q + n <= next->first);
            if (next != live.begin()) {
                auto prev = std::prev(next);
                CHECK(prev->first + prev->second <= q);
            }
            live[q] = n;
        } else {
            auto it = live.begin();
            std::advance(it, rng() % live.size());
            arena->deallocate(it->first, it->second);
            live.erase(it);
        }
    }
    std::size_t want = 0;
    for (auto& kv : live) want += kv.second;
    CHECK(arena->stats().current_bytes == want);
    CHECK(arena->stats().current_allocations == live.size());
    for (auto& kv : live) arena->deallocate(kv.first, kv.second);
    CHECK(arena->stats().idle_bytes == arena->stats().held_bytes);

    // the destructor hands every slab back
    arena.reset();
    CHECK(up->live.empty());

    std::printf("%d failures\n", failures);
    return failures;
}
