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
    Fiber();
    ~Fiber();
    Fiber(Fiber const&) = delete;
    Fiber& operator=(Fiber const&) = delete;
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
};

}  // namespace itg
