// Device memory for temporaries: a stream-ordered slab arena.
//
// Every user of a context enqueues its work on the context's one stream
// (helper streams are forked from it and joined back inside a call), so a
// block handed back after a call was enqueued may be handed out again at once:
// whatever the next user enqueues runs after the previous user's work on the
// same stream. The arena therefore needs no events and no deferred frees.
//
// Memory comes from the upstream in slabs. A request below half a slab shares
// a slab with others (blocks carved at 256-byte alignment); a larger one gets
// a slab of its own, rounded up to 2 MiB. Free space is kept as address
// ranges; a range freed next to another free range of the same slab merges
// with it, and a request takes the smallest free range that holds it (best
// fit), so the space of several freed temporaries can serve one larger
// request. A slab whose blocks are all free goes back to the upstream once
// more idle space is held than the retain limit (1/8 of HBM on a GB300 by
// default: one sort of 2^28 key-value pairs alone needs 2 GiB of temporaries,
// which then stay resident between calls).
//
// What a caller of the reference's memory resources can observe is kept
// (lib/include/CL/Compute/MemoryResource.hpp:78-150, lib/src/Compute/
// MemoryResource.cpp:77-88): the statistics it reads (bytes and allocations
// live, peak and total, and the bytes held idle), and one retry, after every
// idle slab has been handed back, when the upstream runs out of memory.
// Zero-byte temporaries hold nothing. Refusing allocations while the stream
// is captured into a CUDA graph is the CUDA upstream's job (runtime.hpp).
//
// No CUDA dependency: the logic is tested on a host with a fake upstream.
#pragma once

#include <algorithm>
#include <cstddef>
#include <cstdint>
#include <map>
#include <memory>
#include <mutex>
#include <stdexcept>
#include <unordered_map>
#include <vector>

namespace gbc {

//! Thrown by an upstream resource when the device is out of memory.
struct out_of_memory : std::runtime_error {
    using std::runtime_error::runtime_error;
};

//! Where device memory comes from: allocate/deallocate of byte counts.
class memory_resource {
public:
    virtual ~memory_resource() = default;
    void* allocate(std::size_t bytes) { return do_allocate(bytes); }
    void deallocate(void* p, std::size_t bytes) noexcept { do_deallocate(p, bytes); }

protected:
    virtual void* do_allocate(std::size_t bytes) = 0;
    virtual void do_deallocate(void* p, std::size_t bytes) noexcept = 0;
};

class stream_arena final : public memory_resource {
public:
    struct config {
        std::size_t slab_bytes = std::size_t(64) << 20;   // a shared slab
        std::size_t alignment = 256;                      // of every block (a power of two)
        std::size_t own_slab_round = std::size_t(2) << 20;  // rounding of a slab of its own
        std::size_t retain_bytes = std::size_t(1) << 30;  // idle space kept for reuse
    };
    //! Byte and allocation counts are of the sizes callers asked for; held
    //! and idle bytes are of whole slabs.
    struct usage {
        std::size_t current_bytes = 0, peak_bytes = 0, total_bytes = 0;
        std::size_t current_allocations = 0, total_allocations = 0;
        std::size_t held_bytes = 0, idle_bytes = 0, slabs = 0;
        std::size_t slab_allocations = 0, slab_releases = 0;  // upstream calls so far
    };

    stream_arena(std::shared_ptr<memory_resource> upstream, config c) : up_(std::move(upstream)), cfg_(c)
    {
        if (!up_) throw std::invalid_argument("stream_arena: an upstream resource is required");
        const std::size_t a = cfg_.alignment;
        if (a == 0 || (a & (a - 1)) != 0 || cfg_.slab_bytes < a || cfg_.own_slab_round == 0)
            throw std::invalid_argument("stream_arena: alignment must be a power of two no larger than a slab");
    }
    ~stream_arena() override
    {
        std::lock_guard<std::mutex> g(m_);
        for (auto& s : slabs_) up_->deallocate(s->base, s->bytes);
    }
    stream_arena(const stream_arena&) = delete;
    stream_arena& operator=(const stream_arena&) = delete;

    usage stats() const
    {
        std::lock_guard<std::mutex> g(m_);
        usage u = use_;
        u.held_bytes = held_;
        u.idle_bytes = held_ - carved_;
        u.slabs = slabs_.size();
        return u;
    }
    std::size_t idle_bytes() const
    {
        std::lock_guard<std::mutex> g(m_);
        return held_ - carved_;
    }
    //! Hands every slab with no live block back to the upstream; returns the
    //! bytes handed back.
    std::size_t trim()
    {
        std::lock_guard<std::mutex> g(m_);
        return drop_empty_slabs(0);
    }
    const config& settings() const { return cfg_; }

protected:
    void* do_allocate(std::size_t bytes) override
    {
        const std::size_t need = round_up(std::max<std::size_t>(bytes, 1), cfg_.alignment);
        std::lock_guard<std::mutex> g(m_);
        auto fit = by_size_.lower_bound(need);
        if (fit == by_size_.end()) {
            grow(need);
            fit = by_size_.lower_bound(need);
        }
        char* p = fit->second;
        slab* owner = by_addr_.at(p).owner;
        take(p, need);
        live_.emplace(p, block{need, bytes, owner});
        owner->carved += need;
        carved_ += need;
        use_.current_bytes += bytes;
        use_.total_bytes += bytes;
        use_.peak_bytes = std::max(use_.peak_bytes, use_.current_bytes);
        ++use_.current_allocations;
        ++use_.total_allocations;
        return p;
    }

    void do_deallocate(void* p, std::size_t) noexcept override
    {
        std::lock_guard<std::mutex> g(m_);
        auto it = live_.find(p);
        if (it == live_.end()) return;  // not from this arena: nothing to give back
        const block b = it->second;
        live_.erase(it);
        b.owner->carved -= b.carved;
        carved_ -= b.carved;
        use_.current_bytes -= b.requested;
        --use_.current_allocations;
        give_back(static_cast<char*>(p), b.carved, b.owner);
        if (held_ - carved_ > cfg_.retain_bytes) drop_empty_slabs(cfg_.retain_bytes);
    }

private:
    struct slab {
        char* base;
        std::size_t bytes;
        std::size_t carved;  // bytes of live blocks
    };
    struct span {
        std::size_t bytes;
        slab* owner;
    };
    struct block {
        std::size_t carved, requested;
        slab* owner;
    };

    static std::size_t round_up(std::size_t x, std::size_t g) { return (x + g - 1) / g * g; }

    void index_free(char* p, std::size_t bytes, slab* owner)
    {
        by_addr_.emplace(p, span{bytes, owner});
        by_size_.emplace(bytes, p);
    }
    void unindex_free(std::map<char*, span>::iterator it)
    {
        auto range = by_size_.equal_range(it->second.bytes);
        for (auto s = range.first; s != range.second; ++s)
            if (s->second == it->first) {
                by_size_.erase(s);
                break;
            }
        by_addr_.erase(it);
    }
    //! Carves `bytes` off the front of the free range starting at p.
    void take(char* p, std::size_t bytes)
    {
        auto it = by_addr_.find(p);
        const span s = it->second;
        unindex_free(it);
        if (s.bytes > bytes) index_free(p + bytes, s.bytes - bytes, s.owner);
    }
    //! Returns a block to its slab's free ranges, merged with free neighbours.
    void give_back(char* p, std::size_t bytes, slab* owner)
    {
        auto next = by_addr_.find(p + bytes);
        if (next != by_addr_.end() && next->second.owner == owner) {
            bytes += next->second.bytes;
            unindex_free(next);
        }
        auto after = by_addr_.upper_bound(p);
        if (after != by_addr_.begin()) {
            auto prev = std::prev(after);
            if (prev->second.owner == owner && prev->first + prev->second.bytes == p) {
                p = prev->first;
                bytes += prev->second.bytes;
                unindex_free(prev);
            }
        }
        index_free(p, bytes, owner);
    }
    //! A new slab that holds at least `need` bytes. On out of memory: every
    //! empty slab is handed back and one more request is made (for `need`
    //! alone when a shared slab was asked for); a second failure reaches the
    //! caller.
    void grow(std::size_t need)
    {
        const bool shared = need <= cfg_.slab_bytes / 2;
        std::size_t bytes = shared ? cfg_.slab_bytes : round_up(need, cfg_.own_slab_round);
        void* mem = nullptr;
        try {
            mem = up_->allocate(bytes);
        } catch (const out_of_memory&) {
            const std::size_t freed = drop_empty_slabs(0);
            const std::size_t exact = shared ? need : bytes;  // need is a multiple of the alignment
            if (freed == 0 && exact == bytes) throw;          // nothing changed: the same request would fail
            bytes = exact;
            mem = up_->allocate(bytes);
        }
        slabs_.push_back(std::unique_ptr<slab>(new slab{static_cast<char*>(mem), bytes, 0}));
        held_ += bytes;
        ++use_.slab_allocations;
        index_free(slabs_.back()->base, bytes, slabs_.back().get());
    }
    //! Hands empty slabs back, largest first, until at most `keep` idle bytes
    //! are held; returns the bytes handed back.
    std::size_t drop_empty_slabs(std::size_t keep)
    {
        std::vector<slab*> empty;
        for (auto& s : slabs_)
            if (s->carved == 0) empty.push_back(s.get());
        std::sort(empty.begin(), empty.end(), [](const slab* a, const slab* b) { return a->bytes > b->bytes; });
        std::size_t freed = 0;
        for (slab* s : empty) {
            if (held_ - carved_ <= keep) break;
            unindex_free(by_addr_.find(s->base));  // an empty slab is one free range
            up_->deallocate(s->base, s->bytes);
            held_ -= s->bytes;
            freed += s->bytes;
            ++use_.slab_releases;
            slabs_.erase(std::find_if(slabs_.begin(), slabs_.end(),
                                      [s](const std::unique_ptr<slab>& q) { return q.get() == s; }));
        }
        return freed;
    }

    std::shared_ptr<memory_resource> up_;
    config cfg_;
    mutable std::mutex m_;
    std::vector<std::unique_ptr<slab>> slabs_;
    std::map<char*, span> by_addr_;              // free ranges by start address
    std::multimap<std::size_t, char*> by_size_;  // the same ranges by size (best fit)
    std::unordered_map<void*, block> live_;
    std::size_t held_ = 0, carved_ = 0;
    usage use_;
};

//! A temporary for the duration of one call (the reference's
//! internal::temp_buffer, lib/src/Compute/Detail.hpp:37-57): taken from a
//! resource on construction, handed back on destruction; zero bytes take
//! nothing.
class temp_buffer {
public:
    temp_buffer(std::shared_ptr<memory_resource> r, std::size_t bytes) : r_(std::move(r)), bytes_(bytes)
    {
        if (bytes_ != 0) p_ = r_->allocate(bytes_);
    }
    ~temp_buffer()
    {
        if (p_ != nullptr) r_->deallocate(p_, bytes_);
    }
    temp_buffer(const temp_buffer&) = delete;
    temp_buffer& operator=(const temp_buffer&) = delete;

    void* get() const { return p_; }
    template <typename T> T* as() const { return static_cast<T*>(p_); }

private:
    std::shared_ptr<memory_resource> r_;
    std::size_t bytes_;
    void* p_ = nullptr;
};

}  // namespace gbc
