// Cooperative fibers of the solver pool (see fiber.h).
#include "fiber.h"
#include <sys/mman.h>
#include <unistd.h>

namespace itg {

namespace {
constexpr size_t FIBER_STACK_BYTES = 2u << 20;  // touched lazily; sweeps use well under 256 KB
size_t page_bytes() { return (size_t)sysconf(_SC_PAGESIZE); }

void fiber_entry() {
    FiberScheduler* s = FiberScheduler::of_thread();
    Fiber* f = s->current;
    f->fn();  // the pool's solve wrapper catches every exception
    f->running = false;
    // returning resumes uc_link: the scheduler
}

void resume(FiberScheduler& s, Fiber& f) {
    s.current = &f;
    current_account() = f.live_acct;  // as the fiber left it (a section may have suspended charging)
    current_cache() = f.live_cache;
    cache_bypass() = f.live_bypass;
    if (swapcontext(&s.main_uc, &f.uc) != 0) throw Error(ERR_INTERNAL, "fiber: context switch failed");
    current_account().reset();
    current_cache().reset();
    cache_bypass() = false;
    s.current = nullptr;
}
}  // namespace

Fiber::Fiber() {
    const size_t page = page_bytes();
    stack_bytes = FIBER_STACK_BYTES;
    void* p = mmap(nullptr, stack_bytes + page, PROT_READ | PROT_WRITE, MAP_PRIVATE | MAP_ANONYMOUS | MAP_NORESERVE, -1, 0);
    if (p == MAP_FAILED) throw Error(ERR_INTERNAL, "fiber: stack allocation failed");
    mprotect(p, page, PROT_NONE);  // an overflow faults on the guard page instead of corrupting memory
    stack = p;
}

Fiber::~Fiber() {
    if (stack) munmap(stack, stack_bytes + page_bytes());
}

FiberScheduler*& FiberScheduler::of_thread() {
    thread_local FiberScheduler* s = nullptr;
    return s;
}

void FiberScheduler::start(Fiber& f, std::function<void()> fn) {
    ITG_REQUIRE(!f.running, "fiber: already running");
    if (getcontext(&f.uc) != 0) throw Error(ERR_INTERNAL, "fiber: getcontext failed");
    f.uc.uc_stack.ss_sp = static_cast<char*>(f.stack) + page_bytes();
    f.uc.uc_stack.ss_size = f.stack_bytes;
    f.uc.uc_link = &main_uc;
    makecontext(&f.uc, fiber_entry, 0);
    f.fn = std::move(fn);
    f.running = true;
    f.wait = nullptr;
    f.wait_status = cudaSuccess;
    f.live_acct = f.acct;
    f.live_cache = f.cache;
    f.live_bypass = false;
    resume(*this, f);
}

bool FiberScheduler::poll(Fiber& f) {
    if (!f.running) return false;
    if (f.wait) {
        const cudaError_t e = cudaEventQuery(f.wait);
        if (e == cudaErrorNotReady) return false;
        f.wait_status = e;
        f.wait = nullptr;
    }
    resume(*this, f);
    return true;
}

bool fiber_active() {
    FiberScheduler* s = FiberScheduler::of_thread();
    return s && s->current;
}

void fiber_wait_event(cudaEvent_t ev) {
    FiberScheduler* s = FiberScheduler::of_thread();
    Fiber* f = s->current;
    f->wait = ev;
    f->live_acct = current_account();
    f->live_cache = current_cache();
    f->live_bypass = cache_bypass();
    if (swapcontext(&f->uc, &s->main_uc) != 0) throw Error(ERR_INTERNAL, "fiber: context switch failed");
    // resumed by poll() once the event completed (or reported an error)
    const cudaError_t e = f->wait_status;
    f->wait_status = cudaSuccess;
    if (e != cudaSuccess) throw Error(ERR_CUDA, std::string("stream wait: ") + cudaGetErrorString(e));
}

}  // namespace itg
