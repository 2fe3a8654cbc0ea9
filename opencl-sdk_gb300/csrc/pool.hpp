// Memory resources for temporary storage: a caching size-class pool and a
// statistics adaptor over an abstract upstream. The header has no CUDA
// dependency so that its logic is testable on a host without a GPU (with a
// fake upstream); the CUDA upstream lives in runtime.hpp.
//
// Semantics follow the reference memory resources
// (lib/include/CL/Compute/MemoryResource.hpp:31-150,
//  lib/src/Compute/MemoryResource.cpp:31-166):
//   * size classes: powers of two up to pow2_limit, then multiples of
//     large_granularity, never below min_block_bytes;
//   * freed blocks wait in per-class free lists while the cache stays under
//     max_cached_bytes, otherwise they go back upstream;
//   * when the upstream runs out of memory the cache is released and the
//     allocation is retried once;
//   * reuse is stream-ordered: a block handed back by deallocate() may be
//     returned by the next allocate() at once, which is safe because every
//     user of a context enqueues on the context's one stream.
#pragma once

#include <algorithm>
#include <cstddef>
#include <map>
#include <memory>
#include <mutex>
#include <stdexcept>
#include <vector>

namespace gbc {

//! Thrown by an upstream resource when the device is out of memory.
struct out_of_memory : std::runtime_error {
    using std::runtime_error::runtime_error;
};

class memory_resource {
public:
    virtual ~memory_resource() = default;
    void* allocate(std::size_t bytes) { return do_allocate(bytes); }
    void deallocate(void* p, std::size_t bytes) noexcept { do_deallocate(p, bytes); }

protected:
    virtual void* do_allocate(std::size_t bytes) = 0;
    virtual void do_deallocate(void* p, std::size_t bytes) noexcept = 0;
};

class pool_resource final : public memory_resource {
public:
    struct options {
        std::size_t min_block_bytes = 256;
        std::size_t pow2_limit = std::size_t(16) << 20;
        std::size_t large_granularity = std::size_t(1) << 20;
        std::size_t max_cached_bytes = std::size_t(1) << 30;
    };

    explicit pool_resource(std::shared_ptr<memory_resource> upstream)
        : pool_resource(std::move(upstream), options())
    {
    }
    pool_resource(std::shared_ptr<memory_resource> upstream, options opts)
        : upstream_(std::move(upstream)), opts_(opts)
    {
        if (!upstream_) throw std::invalid_argument("pool_resource: null upstream");
        if (opts_.min_block_bytes == 0 || opts_.large_granularity == 0)
            throw std::invalid_argument("pool_resource: zero block size");
    }
    ~pool_resource() override
    {
        std::lock_guard<std::mutex> lock(mutex_);
        release_locked();
    }

    std::size_t size_class(std::size_t bytes) const
    {
        bytes = std::max(bytes, opts_.min_block_bytes);
        if (bytes <= opts_.pow2_limit) {
            std::size_t size = 1;
            while (size < bytes) size <<= 1;
            return size;
        }
        const std::size_t g = opts_.large_granularity;
        return (bytes + g - 1) / g * g;
    }

    //! Hands every cached block back to the upstream resource.
    void release()
    {
        std::lock_guard<std::mutex> lock(mutex_);
        release_locked();
    }

    std::size_t cached_bytes() const
    {
        std::lock_guard<std::mutex> lock(mutex_);
        return cached_bytes_;
    }

    const options& opts() const { return opts_; }

protected:
    void* do_allocate(std::size_t bytes) override
    {
        const std::size_t size = size_class(bytes);
        {
            std::lock_guard<std::mutex> lock(mutex_);
            auto it = free_lists_.find(size);
            if (it != free_lists_.end() && !it->second.empty()) {
                void* p = it->second.back();
                it->second.pop_back();
                cached_bytes_ -= size;
                return p;
            }
        }
        try {
            return upstream_->allocate(size);
        } catch (const out_of_memory&) {
            {
                std::lock_guard<std::mutex> lock(mutex_);
                if (cached_bytes_ == 0) throw;
                release_locked();
            }
            return upstream_->allocate(size);
        }
    }

    void do_deallocate(void* p, std::size_t bytes) noexcept override
    {
        const std::size_t size = size_class(bytes);
        std::lock_guard<std::mutex> lock(mutex_);
        if (cached_bytes_ + size <= opts_.max_cached_bytes) {
            try {
                free_lists_[size].push_back(p);
                cached_bytes_ += size;
                return;
            } catch (...) {
                // No host memory for the list entry: give the block back.
            }
        }
        upstream_->deallocate(p, size);
    }

private:
    void release_locked()
    {
        for (auto& entry : free_lists_)
            for (void* p : entry.second) upstream_->deallocate(p, entry.first);
        free_lists_.clear();
        cached_bytes_ = 0;
    }

    std::shared_ptr<memory_resource> upstream_;
    options opts_;
    mutable std::mutex mutex_;
    std::map<std::size_t, std::vector<void*>> free_lists_;
    std::size_t cached_bytes_ = 0;
};

class statistics_adaptor final : public memory_resource {
public:
    struct counters {
        std::size_t current_bytes = 0;
        std::size_t peak_bytes = 0;
        std::size_t total_bytes = 0;
        std::size_t current_allocations = 0;
        std::size_t total_allocations = 0;
    };

    explicit statistics_adaptor(std::shared_ptr<memory_resource> upstream)
        : upstream_(std::move(upstream))
    {
        if (!upstream_) throw std::invalid_argument("statistics_adaptor: null upstream");
    }

    counters statistics() const
    {
        std::lock_guard<std::mutex> lock(mutex_);
        return counters_;
    }

protected:
    void* do_allocate(std::size_t bytes) override
    {
        void* p = upstream_->allocate(bytes);
        std::lock_guard<std::mutex> lock(mutex_);
        counters_.current_bytes += bytes;
        counters_.peak_bytes = std::max(counters_.peak_bytes, counters_.current_bytes);
        counters_.total_bytes += bytes;
        ++counters_.current_allocations;
        ++counters_.total_allocations;
        return p;
    }
    void do_deallocate(void* p, std::size_t bytes) noexcept override
    {
        upstream_->deallocate(p, bytes);
        std::lock_guard<std::mutex> lock(mutex_);
        counters_.current_bytes -= bytes;
        --counters_.current_allocations;
    }

private:
    std::shared_ptr<memory_resource> upstream_;
    mutable std::mutex mutex_;
    counters counters_;
};

//! RAII temporary from a resource (the reference's internal::temp_buffer,
//! lib/src/Compute/Detail.hpp:37-57). Zero bytes hold nothing.
class temp_buffer {
public:
    temp_buffer(std::shared_ptr<memory_resource> r, std::size_t bytes)
        : resource_(std::move(r)), bytes_(bytes)
    {
        if (bytes_ != 0) p_ = resource_->allocate(bytes_);
    }
    ~temp_buffer()
    {
        if (bytes_ != 0) resource_->deallocate(p_, bytes_);
    }
    temp_buffer(const temp_buffer&) = delete;
    temp_buffer& operator=(const temp_buffer&) = delete;

    void* get() const { return p_; }
    template <typename T> T* as() const { return static_cast<T*>(p_); }

private:
    std::shared_ptr<memory_resource> resource_;
    void* p_ = nullptr;
    std::size_t bytes_;
};

}  // namespace gbc
