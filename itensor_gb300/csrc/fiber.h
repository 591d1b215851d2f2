// Fibers for the solver pool: each worker thread runs several DMRG solves as
// cooperative fibers (ucontext, one private stack each). A solve only gives
// up the thread where it waits for its own stream (Ctx::sync), so the host
// work of one solve overlaps the device work of the others, and the solve's
// code stays the plain sequential sweep loop.
#pragma once
#include "common.h"
#include <exception>
#include <functional>
#include <ucontext.h>

namespace itg {

struct Fiber {
    ucontext_t uc;
    void* stack = nullptr;          // mmap'd, lowest page a guard page
    size_t stack_bytes = 0;
    std::function<void()> fn;
    bool running = false;           // started and not finished
    cudaEvent_t wait = nullptr;     // event the fiber waits for (null: runnable)
    cudaError_t wait_status = cudaSuccess;
    std::shared_ptr<MemAccount> acct;       // the solve's account
    std::shared_ptr<MemAccount> live_acct;  // the thread's account when the fiber last yielded
    std::shared_ptr<BlockCache> cache;      // the solve's block cache
    std::shared_ptr<BlockCache> live_cache; // the thread's cache when the fiber last yielded
    bool live_bypass = false;               // the thread's cache bypass when the fiber last yielded
    bool group_wait = false;                // handed a contraction to the next grouped launch
    cudaEvent_t group_ready = nullptr;      // its inputs are ready on its stream
    std::string group_error;                // set when the grouped launch failed
    Fiber();
    ~Fiber();
    Fiber(Fiber const&) = delete;
    Fiber& operator=(Fiber const&) = delete;
};

struct Ctx;
struct Plan;
// A split-precision contraction a fiber handed to the thread's next grouped launch.
struct GroupRequest {
    Fiber* fiber;
    Ctx* ctx;
    Plan const* plan;
    double const* A;
    double const* B;
    double* C;
    int S;
    __nv_bfloat16* panels;
    int32_t* exps;
    bool prep_b;
};

// One per worker thread.
struct FiberScheduler {
    ucontext_t main_uc;
    Fiber* current = nullptr;
    // Starts f running fn (f must not be running); returns at its first wait or end.
    void start(Fiber& f, std::function<void()> fn);
    // Resumes f if its wait is over; returns true if it ran.
    bool poll(Fiber& f);
    static FiberScheduler*& of_thread();

    // Cross-solve grouping: while `grouping` is on, the fibers' split-precision
    // contractions wait in `pending` (each fiber yields) until the thread has
    // nothing else to run; flush() then enqueues all of them as one grouped
    // prep launch and one grouped GEMM launch on the thread's group stream,
    // ordered after each contraction's inputs and before each stream's next work.
    bool grouping = false;
    std::vector<GroupRequest> pending;
    void flush();
    uint64_t grouped_launches = 0, grouped_contractions = 0;
    ~FiberScheduler();

private:
    cudaStream_t gstream_ = nullptr;
    cudaEvent_t gdone_ = nullptr;
    void* ref_dev_ = nullptr;                // device GroupRef array
    size_t ref_cap_ = 0;                     // its capacity (records)
    static constexpr int NSTAGE = 4;         // pinned staging slots for the records
    void* ref_host_[NSTAGE] = {};
    cudaEvent_t ref_ev_[NSTAGE] = {};
    int ref_slot_ = 0;
};

}  // namespace itg
