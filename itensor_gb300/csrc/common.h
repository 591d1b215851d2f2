// Shared host-side plumbing for the GB300 DMRG hot path: error handling,
// stream-ordered device buffers, and the per-context state.
#pragma once
#include <cuda_runtime.h>
#include <cuda_bf16.h>
#include <atomic>
#include <cstdint>
#include <cstdio>
#include <map>
#include <memory>
#include <mutex>
#include <stdexcept>
#include <string>
#include <unordered_map>
#include <vector>

namespace itg {

// Status codes returned through the C-ABI (include/itg.h).
enum Status : int {
    OK = 0,
    ERR_ARG = 1,        // malformed arguments / block metadata
    ERR_CUDA = 2,       // CUDA runtime error
    ERR_OOM = 3,        // device allocation failed
    ERR_NOCONV = 4,     // eigensolver did not converge within its sweep cap
    ERR_TIMEOUT = 5,    // device-side bounded wait gave up
    ERR_INTERNAL = 6,
    ERR_RANGE = 7,      // size beyond a stated maximum
};

struct Error : std::runtime_error {
    int code;
    Error(int c, std::string const& m) : std::runtime_error(m), code(c) {}
};

#define ITG_CHECK_CUDA(expr)                                                                      \
    do {                                                                                          \
        cudaError_t e_ = (expr);                                                                  \
        if (e_ != cudaSuccess) {                                                                  \
            throw ::itg::Error(e_ == cudaErrorMemoryAllocation ? ::itg::ERR_OOM : ::itg::ERR_CUDA, \
                               std::string(#expr) + ": " + cudaGetErrorString(e_));               \
        }                                                                                         \
    } while (0)

#define ITG_REQUIRE(cond, msg)                                  \
    do {                                                        \
        if (!(cond)) throw ::itg::Error(::itg::ERR_ARG, (msg)); \
    } while (0)

// Streams of live contexts. A buffer that outlives its context (a tensor
// handle released after itg_destroy) is freed synchronously instead of on the
// destroyed stream.
struct BlockCache;
void stream_register(cudaStream_t s, std::shared_ptr<BlockCache> cache);
void stream_unregister(cudaStream_t s);
bool stream_alive(cudaStream_t s);
// The block cache of the context that owns stream s (null: none).
std::shared_ptr<BlockCache> stream_cache(cudaStream_t s);
// Set while allocating buffers that outlive the current solve (shared plan
// tables): they bypass every block cache.
bool& cache_bypass();

// Cooperative solve multiplexing (fiber.cpp). A solver-pool worker thread runs
// several solves as fibers; a fiber that must wait for its stream yields to
// the others instead of blocking the thread.
bool fiber_active();                    // the calling code runs inside a pool fiber
void fiber_wait_event(cudaEvent_t ev);  // yield until ev has completed (errors throw)

// Device bytes held by one solve: the solver pool charges every buffer that a
// solve allocates to its account and reports the peak beside the admission
// estimate.
struct MemAccount {
    std::atomic<int64_t> cur{0}, peak{0};
    void add(int64_t n) {
        const int64_t c = cur.fetch_add(n) + n;
        int64_t p = peak.load();
        while (c > p && !peak.compare_exchange_weak(p, c)) {}
    }
    void sub(int64_t n) { cur.fetch_sub(n); }
};
// Account charged by the calling thread's allocations (empty: none).
std::shared_ptr<MemAccount>& current_account();

// Device allocations are rounded up to size classes: eight per power of two
// (at most 12.5% over the request), 512 B at least. Blocks freed by one
// tensor then fit the next request of about the same size, so caches hit.
inline size_t alloc_class(size_t n) {
    if (n <= 512) return 512;
    const int k = 63 - __builtin_clzll((unsigned long long)(n - 1));  // 2^k < n <= 2^(k+1)
    const size_t step = size_t(1) << (k - 3);
    return (n + step - 1) / step * step;
}

// Process-wide allocator counters (diagnostics): requests served by a block
// cache, and the driver's allocation and free calls.
struct AllocCounters {
    std::atomic<uint64_t> cached{0}, driver_allocs{0}, driver_frees{0};
    std::atomic<uint64_t> bypass{0}, nocache{0}, full{0};  // driver allocations without a cache; frees a full cache refused
};
AllocCounters& alloc_counters();

// Blocks freed on a context's stream, kept for its next allocations on that
// stream: reuse in stream order needs no synchronisation, and the solver
// pool's many threads then make far fewer allocator calls (which serialise
// on the driver). Blocks are reused for requests of half their size or more;
// the cache holds at most `limit` bytes. In the solver pool it outlives the
// solves of its slot and is trimmed when each solve ends.
struct BlockCache {
    std::mutex mu;
    cudaStream_t stream = nullptr;
    std::multimap<size_t, void*> free;
    size_t held = 0, limit = size_t(1) << 30;
    explicit BlockCache(cudaStream_t s) : stream(s) {}
    void* take(size_t n, size_t* got) {
        std::lock_guard<std::mutex> g(mu);
        auto it = free.lower_bound(n);
        if (it == free.end() || it->first > 2 * n) return nullptr;
        void* p = it->second;
        *got = it->first;
        held -= it->first;
        free.erase(it);
        return p;
    }
    bool put(void* p, size_t n) {
        std::lock_guard<std::mutex> g(mu);
        if (held + n > limit) return false;
        free.emplace(n, p);
        held += n;
        return true;
    }
    void release() { trim(0); }  // frees every cached block (on the stream while it lives)
    void trim(size_t keep);       // frees the largest blocks until at most `keep` bytes stay
    ~BlockCache() { release(); }
};
// Cache serving the calling thread's allocations (empty: none).
std::shared_ptr<BlockCache>& current_cache();

// Device buffer from the stream-ordered pool (cudaMallocAsync). Freed on the
// stream it was allocated on, so reuse is ordered after every prior use.
struct DevBuf {
    void* p = nullptr;
    size_t bytes = 0;
    cudaStream_t stream = nullptr;
    std::shared_ptr<MemAccount> acct;
    std::shared_ptr<BlockCache> cache;
    DevBuf() = default;
    DevBuf(size_t n, cudaStream_t s) : bytes(n), stream(s) {
        if (n) {
            const size_t cls = alloc_class(n);
            std::shared_ptr<BlockCache> c;
            if (!cache_bypass()) {
                c = current_cache();                // the cache of a pool solve's slot
                if (!c || c->stream != s) c = stream_cache(s);  // else the stream's context cache
            }
            if (c && c->stream == s) {
                cache = c;
                size_t got = 0;
                if ((p = c->take(cls, &got))) {
                    bytes = got;
                    alloc_counters().cached.fetch_add(1, std::memory_order_relaxed);
                }
            }
            if (!p) {
                ITG_CHECK_CUDA(cudaMallocAsync(&p, cls, s));
                bytes = cls;
                alloc_counters().driver_allocs.fetch_add(1, std::memory_order_relaxed);
                if (cache_bypass()) alloc_counters().bypass.fetch_add(1, std::memory_order_relaxed);
                else if (!cache) alloc_counters().nocache.fetch_add(1, std::memory_order_relaxed);
            }
            acct = current_account();
            if (acct) acct->add((int64_t)bytes);
        }
    }
    ~DevBuf() {
        if (!p) return;
        if (acct) acct->sub((int64_t)bytes);
        // (a cache frees its blocks itself, checking its stream then)
        if (cache && cache->put(p, bytes)) return;
        alloc_counters().driver_frees.fetch_add(1, std::memory_order_relaxed);
        if (cache) alloc_counters().full.fetch_add(1, std::memory_order_relaxed);
        if (stream_alive(stream)) cudaFreeAsync(p, stream);
        else cudaFree(p);
    }
    DevBuf(DevBuf const&) = delete;
    DevBuf& operator=(DevBuf const&) = delete;
    template <typename T> T* as() const { return static_cast<T*>(p); }
};
using DevBufPtr = std::shared_ptr<DevBuf>;

inline DevBufPtr dev_alloc(size_t bytes, cudaStream_t s) { return std::make_shared<DevBuf>(bytes, s); }

// Arithmetic used by the block GEMMs.
enum Precision : int {
    PREC_F64 = 0,        // plain FP64 (FFMA) -- the drop-in path
    PREC_OZAKI_BF16 = 1, // FP64 operands split into exact BF16 integer slices, FP32-exact accumulation
    PREC_TF32X3 = 2,     // 3xTF32 split, FP32 accumulate (FP32-level accuracy)
};

}  // namespace itg
