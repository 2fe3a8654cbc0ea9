// Host runtime: context lifetime, the CUDA upstream memory resource, device
// error reporting and the tuning table that replaces the reference's JIT
// program cache (lib/src/Compute/ProgramCache.cpp:17-283: it hashed OpenCL C
// source + options + device identity and kept built binaries in memory and in
// CL_COMPUTE_CACHE_DIR). Kernels here are compiled ahead of time for sm_103a;
// what remains to choose at run time is a launch shape per (operation, element
// type, size class, distribution), which the autotuner measures and this
// table stores in <cache_dir>/gbcompute_tuning.txt.
#include "runtime.hpp"

#include <cstdlib>
#include <cstring>
#include <fstream>
#include <sstream>
#include <set>
#include <utility>

#include "sort_internal.hpp"

namespace gbc {

void check_cuda(cudaError_t e, const char* what)
{
    if (e == cudaSuccess) return;
    if (e == cudaErrorMemoryAllocation) {
        (void)cudaGetLastError();  // not sticky: clear it
        throw out_of_memory(std::string(what) + ": out of device memory");
    }
    throw device_error(std::string(what) + " failed: " + cudaGetErrorString(e) + " (" +
                           std::to_string((int)e) + ")",
                       (int)e);
}

void check_size(std::size_t n)
{
    if (n > 0x7FFFFFFFu) throw std::length_error("gbcompute: at most 2^31-1 elements per call");
}

std::size_t elem_size(elem t)
{
    switch (t) {
    case elem::i8:
    case elem::u8: return 1;
    case elem::i16:
    case elem::u16: return 2;
    case elem::i32:
    case elem::u32:
    case elem::f32: return 4;
    case elem::i64:
    case elem::u64:
    case elem::f64: return 8;
    }
    throw std::invalid_argument("gbcompute: unknown element type");
}

stream_holder::~stream_holder()
{
    if (owned && stream != nullptr) {
        cudaSetDevice(device);
        cudaStreamSynchronize(stream);
        cudaStreamDestroy(stream);
    }
}

bool cuda_async_resource::capturing() const
{
    cudaStreamCaptureStatus st = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(s_->stream, &st) != cudaSuccess) {
        (void)cudaGetLastError();
        return false;
    }
    return st != cudaStreamCaptureStatusNone;
}

void* cuda_async_resource::do_allocate(std::size_t bytes)
{
    void* p = nullptr;
    cudaSetDevice(s_->device);
    if (capturing())
        throw unsupported_error(
            "gbcompute: a temporary is not in the pool while the stream is being captured; run the same "
            "call once before capturing it");
    check_cuda(cudaMallocAsync(&p, std::max<std::size_t>(bytes, 1), s_->stream), "cudaMallocAsync");
    return p;
}

void cuda_async_resource::do_deallocate(void* p, std::size_t) noexcept
{
    cudaSetDevice(s_->device);
    if (capturing()) {
        std::lock_guard<std::mutex> lock(m_);
        try {
            deferred_.push_back(p);
            return;
        } catch (...) {
            // no host memory for the list: fall through
        }
    }
    cudaFreeAsync(p, s_->stream);
}

void cuda_async_resource::flush_deferred()
{
    std::lock_guard<std::mutex> lock(m_);
    cudaSetDevice(s_->device);
    for (void* p : deferred_) cudaFreeAsync(p, s_->stream);
    deferred_.clear();
}

stream_arena::config default_arena_config(std::size_t global_memory)
{
    stream_arena::config c;
    c.retain_bytes = std::max<std::size_t>(c.retain_bytes, global_memory / 8);
    if (const char* env = std::getenv("CLC_POOL_MAX_CACHED_BYTES")) {
        char* end = nullptr;
        const unsigned long long v = std::strtoull(env, &end, 10);
        if (end != env) c.retain_bytes = (std::size_t)v;
    }
    return c;
}

device_context::device_context(int dev, cudaStream_t external_stream,
                               const stream_arena::config& arena_cfg, const std::string& tuning_dir)
    : device(dev)
{
    check_cuda(cudaSetDevice(dev), "cudaSetDevice");
    cudaDeviceProp prop;
    check_cuda(cudaGetDeviceProperties(&prop, dev), "cudaGetDeviceProperties");
    sm_count = prop.multiProcessorCount;
    smem_optin = prop.sharedMemPerBlockOptin;
    global_memory = prop.totalGlobalMem;
    name = prop.name;

    holder = std::make_shared<stream_holder>();
    holder->device = dev;
    if (external_stream != nullptr) {
        holder->stream = external_stream;
        holder->owned = false;
    } else {
        check_cuda(cudaStreamCreateWithFlags(&holder->stream, cudaStreamNonBlocking),
                   "cudaStreamCreate");
        holder->owned = true;
    }
    stream = holder->stream;
    upstream = std::make_shared<cuda_async_resource>(holder);
    arena = std::make_shared<stream_arena>(upstream, arena_cfg);
    resource = arena;

    try {
        check_cuda(cudaMalloc(&d_error, sizeof(int)), "cudaMalloc");
        check_cuda(cudaMalloc(&lookback_ring, onesweep::RING_BYTES), "cudaMalloc");
        check_cuda(cudaMalloc(&d_small, 64 * 1024), "cudaMalloc");
        check_cuda(cudaMallocHost(&pinned, 64 * 1024), "cudaMallocHost");
        check_cuda(cudaMemsetAsync(d_error, 0, sizeof(int), stream), "cudaMemsetAsync");
        check_cuda(cudaMemsetAsync(lookback_ring, 0, onesweep::RING_BYTES, stream), "cudaMemsetAsync");
        check_cuda(cudaMemsetAsync(d_small, 0, 64 * 1024, stream), "cudaMemsetAsync");
        check_cuda(cudaStreamSynchronize(stream), "cudaStreamSynchronize");
    } catch (...) {
        if (d_error) cudaFree(d_error);
        if (lookback_ring) cudaFree(lookback_ring);
        if (d_small) cudaFree(d_small);
        if (pinned) cudaFreeHost(pinned);
        throw;
    }

    std::string dir = tuning_dir;
    if (dir.empty()) {
        if (const char* env = std::getenv("CLC_TUNING_DIR")) dir = env;
        else if (const char* env2 = std::getenv("CL_COMPUTE_CACHE_DIR")) dir = env2;
    }
    if (!dir.empty()) {
        tuning_path = dir + "/gbcompute_tuning.txt";
        tuning.load(tuning_path);
    }
}

cudaStream_t device_context::aux_stream()
{
    if (aux == nullptr) {
        activate();
        check_cuda(cudaStreamCreateWithFlags(&aux, cudaStreamNonBlocking), "cudaStreamCreate");
        check_cuda(cudaEventCreateWithFlags(&fork_event, cudaEventDisableTiming), "cudaEventCreate");
        check_cuda(cudaEventCreateWithFlags(&join_event, cudaEventDisableTiming), "cudaEventCreate");
    }
    return aux;
}

device_context::~device_context()
{
    cudaSetDevice(device);
    cudaStreamSynchronize(stream);
    if (aux != nullptr) {
        cudaStreamSynchronize(aux);
        cudaStreamDestroy(aux);
        cudaEventDestroy(fork_event);
        cudaEventDestroy(join_event);
    }
    cudaFree(d_error);
    cudaFree(lookback_ring);
    cudaFree(d_small);
    cudaFreeHost(pinned);
}

void device_context::activate() const { check_cuda(cudaSetDevice(device), "cudaSetDevice"); }

bool device_context::capturing() const
{
    cudaStreamCaptureStatus st = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(stream, &st) != cudaSuccess) {
        (void)cudaGetLastError();
        return false;
    }
    return st != cudaStreamCaptureStatusNone;
}

uint64_t device_context::reserve_seq(uint64_t count)
{
    constexpr uint64_t WRAP = uint64_t(1) << 30;
    if (capturing()) {
        // A graph replays the sequence numbers it was captured with, so the
        // words of the previous replay would carry matching tags: a captured
        // call clears the ring first (one 16 MiB memset node).
        check_cuda(cudaMemsetAsync(lookback_ring, 0, onesweep::RING_BYTES, stream), "cudaMemsetAsync");
    } else if ((ring_seq % WRAP) + count >= WRAP) {
        check_cuda(cudaMemsetAsync(lookback_ring, 0, onesweep::RING_BYTES, stream), "cudaMemsetAsync");
        ring_seq = (ring_seq / WRAP + 1) * WRAP;
    }
    const uint64_t s = ring_seq;
    ring_seq += count;
    return s;
}

int device_context::take_device_error()
{
    activate();
    // The upper half of the pinned page is reserved for the error word; the
    // lower half stages algorithm results.
    int* h = reinterpret_cast<int*>(static_cast<char*>(pinned) + 32 * 1024);
    check_cuda(cudaMemcpyAsync(h, d_error, sizeof(int), cudaMemcpyDeviceToHost, stream), "cudaMemcpyAsync");
    check_cuda(cudaStreamSynchronize(stream), "cudaStreamSynchronize");
    const int e = *h;
    if (e != 0) {
        check_cuda(cudaMemsetAsync(d_error, 0, sizeof(int), stream), "cudaMemsetAsync");
        check_cuda(cudaStreamSynchronize(stream), "cudaStreamSynchronize");
    }
    return e;
}

void device_context::finish()
{
    const int e = take_device_error();
    if (e == 1)
        throw device_error("gbcompute: a decoupled look-back wait timed out; results of the last "
                           "calls are invalid",
                           (int)cudaErrorLaunchTimeout);
    if (e == 2) throw std::invalid_argument("gbcompute: segment offsets are not monotone");
}

// ---- profiler -------------------------------------------------------------

cudaEvent_t profiler::get_event()
{
    if (!free_.empty()) {
        cudaEvent_t e = free_.back();
        free_.pop_back();
        return e;
    }
    cudaEvent_t e;
    check_cuda(cudaEventCreate(&e), "cudaEventCreate");
    return e;
}

int profiler::start(cudaStream_t s, const char* name)
{
    if (!enabled_) return -1;
    cudaStreamCaptureStatus st = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(s, &st) != cudaSuccess || st != cudaStreamCaptureStatusNone) {
        (void)cudaGetLastError();
        return -1;  // events recorded inside a capture cannot be timed
    }
    std::lock_guard<std::mutex> lock(m_);
    pending p{name, get_event(), get_event()};
    check_cuda(cudaEventRecord(p.a, s), "cudaEventRecord");
    pending_.push_back(p);
    return (int)pending_.size() - 1;
}

void profiler::stop(cudaStream_t s, int slot)
{
    if (slot < 0) return;
    std::lock_guard<std::mutex> lock(m_);
    if (slot < (int)pending_.size()) cudaEventRecord(pending_[slot].b, s);
}

void profiler::resolve(cudaStream_t s)
{
    if (pending_.empty()) return;
    check_cuda(cudaStreamSynchronize(s), "cudaStreamSynchronize");
    for (auto& p : pending_) {
        float ms = 0;
        if (cudaEventElapsedTime(&ms, p.a, p.b) == cudaSuccess) {
            auto& t = totals_[p.name];
            t.launches += 1;
            t.ms += ms;
        } else {
            (void)cudaGetLastError();
        }
        free_.push_back(p.a);
        free_.push_back(p.b);
    }
    pending_.clear();
}

std::map<std::string, profiler::total> profiler::totals(cudaStream_t s)
{
    std::lock_guard<std::mutex> lock(m_);
    resolve(s);
    return totals_;
}

void profiler::reset(cudaStream_t s)
{
    std::lock_guard<std::mutex> lock(m_);
    resolve(s);
    totals_.clear();
}

profiler::~profiler()
{
    for (auto& p : pending_) {
        cudaEventDestroy(p.a);
        cudaEventDestroy(p.b);
    }
    for (auto e : free_) cudaEventDestroy(e);
}

kernel_timer::kernel_timer(device_context& ctx, const char* name) : kernel_timer(ctx, name, ctx.stream) {}

kernel_timer::kernel_timer(device_context& ctx, const char* name, cudaStream_t stream)
    : ctx_(ctx), stream_(stream), slot_(ctx.prof.start(stream, name))
{
}

kernel_timer::~kernel_timer() { ctx_.prof.stop(stream_, slot_); }

// ---- tuning table ---------------------------------------------------------

bool tuning_table::lookup(const std::string& key, launch_shape& out) const
{
    std::lock_guard<std::mutex> lock(m_);
    auto it = entries_.find(key);
    if (it == entries_.end()) return false;
    out = it->second;
    return true;
}

void tuning_table::store(const std::string& key, const launch_shape& s)
{
    std::lock_guard<std::mutex> lock(m_);
    entries_[key] = s;
}

std::size_t tuning_table::size() const
{
    std::lock_guard<std::mutex> lock(m_);
    return entries_.size();
}

void tuning_table::load(const std::string& path)
{
    std::ifstream f(path);
    if (!f) return;
    std::string line;
    std::lock_guard<std::mutex> lock(m_);
    while (std::getline(f, line)) {
        if (line.empty() || line[0] == '#') continue;
        std::istringstream ss(line);
        std::string key;
        launch_shape s;
        if (ss >> key >> s.variant) entries_[key] = s;
    }
}

void tuning_table::save(const std::string& path) const
{
    std::ofstream f(path, std::ios::trunc);
    if (!f) throw std::runtime_error("gbcompute: cannot write tuning table " + path);
    std::lock_guard<std::mutex> lock(m_);
    f << "# gbcompute tuning table: <op:dtype:size class[:distribution]> <variant>\n";
    for (const auto& e : entries_) f << e.first << ' ' << e.second.variant << '\n';
}

std::string tuning_table::size_class(std::size_t n)
{
    int k = 0;
    while ((std::size_t(1) << k) < n && k < 63) ++k;
    return "2^" + std::to_string(k);
}

bool first_use_on_device(const void* kernel)
{
    static std::mutex m;
    static std::set<std::pair<int, const void*>> seen;
    int dev = 0;
    check_cuda(cudaGetDevice(&dev), "cudaGetDevice");
    std::lock_guard<std::mutex> lock(m);
    return seen.emplace(dev, kernel).second;
}

}  // namespace gbc
