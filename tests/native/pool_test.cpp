// Host-only checks of the memory resources (opencl-sdk_gb300/csrc/pool.hpp)
// with a fake upstream whose allocations can be made to fail on demand: the
// release-and-retry path of pool_resource (reference MemoryResource.cpp:
// 77-88) is exercised without a GPU. Exit status = number of failed checks.
#include "pool.hpp"

#include <cstdio>
#include <cstdlib>
#include <set>

static int failures = 0;
#define CHECK(c)                                                             \
    do {                                                                     \
        if (!(c)) {                                                          \
            ++failures;                                                      \
            std::fprintf(stderr, "FAILED: %s at line %d\n", #c, __LINE__);   \
        }                                                                    \
    } while (0)

struct fake_upstream : gbc::memory_resource {
    std::size_t live_bytes = 0, allocs = 0, frees = 0, limit = ~std::size_t(0);
    std::set<void*> live;
    void* do_allocate(std::size_t b) override
    {
        if (live_bytes + b > limit) throw gbc::out_of_memory("fake upstream: out of memory");
        void* p = std::malloc(b);
        live.insert(p);
        live_bytes += b;
        ++allocs;
        return p;
    }
    void do_deallocate(void* p, std::size_t b) noexcept override
    {
        live.erase(p);
        live_bytes -= b;
        ++frees;
        std::free(p);
    }
};

int main()
{
    auto up = std::make_shared<fake_upstream>();
    gbc::pool_resource::options o;
    o.max_cached_bytes = 1 << 20;
    auto pool = std::make_shared<gbc::pool_resource>(up, o);
    auto stats = std::make_shared<gbc::statistics_adaptor>(pool);

    // size classes (MemoryResource.cpp:47-58)
    CHECK(pool->size_class(1) == 256);
    CHECK(pool->size_class(257) == 512);
    CHECK(pool->size_class(16 << 20) == (16u << 20));
    CHECK(pool->size_class((16 << 20) + 1) == (17u << 20));

    // reuse of a freed block of the same class, no new upstream allocation
    void* a = stats->allocate(1000);
    stats->deallocate(a, 1000);
    CHECK(pool->cached_bytes() == 1024);
    void* b = stats->allocate(900);
    CHECK(b == a);
    CHECK(up->allocs == 1);
    stats->deallocate(b, 900);

    // blocks beyond max_cached_bytes go back upstream
    void* big = stats->allocate(2 << 20);
    stats->deallocate(big, 2 << 20);
    CHECK(pool->cached_bytes() == 1024);
    CHECK(up->frees == 1);

    // statistics adaptor (MemoryResource.cpp:141-166)
    auto s = stats->statistics();
    CHECK(s.total_allocations == 3);
    CHECK(s.current_allocations == 0);
    CHECK(s.peak_bytes == (2u << 20));
    CHECK(s.current_bytes == 0);

    // out of memory: cache released, allocation retried once and succeeds
    up->limit = up->live_bytes + 3072;  // 1024 cached + 3 KiB: 4 KiB fits only without the cache
    void* c = stats->allocate(4000);    // class 4096 does not fit with the cache held
    CHECK(c != nullptr);
    CHECK(pool->cached_bytes() == 0);
    stats->deallocate(c, 4000);

    // out of memory with nothing cached: the error reaches the caller
    pool->release();
    up->limit = 0;
    bool threw = false;
    try {
        stats->allocate(10);
    } catch (const gbc::out_of_memory&) {
        threw = true;
    }
    CHECK(threw);
    CHECK(stats->statistics().current_allocations == 0);

    // temp_buffer returns its block on scope exit; zero bytes hold nothing
    up->limit = ~std::size_t(0);
    {
        gbc::temp_buffer t(stats, 100);
        CHECK(t.get() != nullptr);
        gbc::temp_buffer z(stats, 0);
        CHECK(z.get() == nullptr);
        CHECK(stats->statistics().current_allocations == 1);
    }
    CHECK(stats->statistics().current_allocations == 0);

    // the destructor hands every cached block back upstream
    pool.reset();
    stats.reset();
    CHECK(up->live.empty());

    std::printf("%d failures\n", failures);
    return failures;
}
