// Cooperative fibers of the solver pool (see fiber.h).
#include "fiber.h"
#include "engine.h"
#include <algorithm>
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
    if (group_ready) cudaEventDestroy(group_ready);
}

FiberScheduler::~FiberScheduler() {
    if (gstream_) cudaStreamSynchronize(gstream_);
    for (int i = 0; i < NSTAGE; ++i) {
        if (ref_ev_[i]) cudaEventDestroy(ref_ev_[i]);
        if (ref_host_[i]) cudaFreeHost(ref_host_[i]);
    }
    if (ref_dev_) cudaFree(ref_dev_);
    if (gdone_) cudaEventDestroy(gdone_);
    if (gstream_) cudaStreamDestroy(gstream_);
}

void FiberScheduler::flush() {
    if (pending.empty()) return;
    std::vector<GroupRequest> reqs;
    reqs.swap(pending);
    try {
        if (!gstream_) {
            ITG_CHECK_CUDA(cudaStreamCreateWithFlags(&gstream_, cudaStreamNonBlocking));
            ITG_CHECK_CUDA(cudaEventCreateWithFlags(&gdone_, cudaEventDisableTiming));
            for (int i = 0; i < NSTAGE; ++i) ITG_CHECK_CUDA(cudaEventCreateWithFlags(&ref_ev_[i], cudaEventDisableTiming));
        }
        // every contraction's inputs (and scratch) are ready on its own stream first
        for (auto const& r : reqs) ITG_CHECK_CUDA(cudaStreamWaitEvent(gstream_, r.fiber->group_ready, 0));
        // one group per slice count (normally all requests share one)
        std::vector<int> order(reqs.size());
        for (size_t i = 0; i < reqs.size(); ++i) order[i] = (int)i;
        std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return reqs[a].S < reqs[b].S; });
        for (size_t i0 = 0; i0 < order.size();) {
            size_t i1 = i0;
            while (i1 < order.size() && reqs[order[i1]].S == reqs[order[i0]].S) ++i1;
            const int n = (int)(i1 - i0);
            if ((size_t)n > ref_cap_) {
                // grow the record arrays (the group stream is idle once synchronised)
                ITG_CHECK_CUDA(cudaStreamSynchronize(gstream_));
                if (ref_dev_) cudaFree(ref_dev_);
                for (int k = 0; k < NSTAGE; ++k)
                    if (ref_host_[k]) { cudaFreeHost(ref_host_[k]); ref_host_[k] = nullptr; }
                ref_cap_ = std::max<size_t>(2 * n, 64);
                ITG_CHECK_CUDA(cudaMalloc(&ref_dev_, sizeof(GroupRef) * ref_cap_));
                for (int k = 0; k < NSTAGE; ++k) ITG_CHECK_CUDA(cudaHostAlloc(&ref_host_[k], sizeof(GroupRef) * ref_cap_, 0));
            }
            const int slot = ref_slot_;
            ref_slot_ = (ref_slot_ + 1) % NSTAGE;
            ITG_CHECK_CUDA(cudaEventSynchronize(ref_ev_[slot]));  // its previous copy has been read
            GroupRef* refs = static_cast<GroupRef*>(ref_host_[slot]);
            int total_prep = 0, total_tiles = 0;
            for (int j = 0; j < n; ++j) {
                GroupRequest const& r = reqs[order[i0 + j]];
                Plan const& p = *r.plan;
                GroupRef g;
                g.prep = p.d_prep;
                g.ops = p.d_ops;
                g.tab = p.d_tab;
                g.items = p.d_items;
                g.pairs = p.d_pairs;
                g.cblk = p.d_cblk;
                g.A = r.A;
                g.B = r.B;
                g.C = r.C;
                g.panels = r.panels;
                g.exps = r.exps;
                g.plane = (p.panel_elems + 15) / 16 * 16;
                g.prep_start = total_prep;
                g.tile_start = total_tiles;
                if (r.S > 0) total_prep += r.prep_b ? p.nprep : p.nprepA;
                total_tiles += p.nitems;
                refs[j] = g;
            }
            ITG_CHECK_CUDA(cudaMemcpyAsync(ref_dev_, refs, sizeof(GroupRef) * n, cudaMemcpyHostToDevice, gstream_));
            ITG_CHECK_CUDA(cudaEventRecord(ref_ev_[slot], gstream_));
            // S > 0: split precision with S slices; S == 0: FP64 tiles
            if (reqs[order[i0]].S > 0)
                launch_ozaki_group(gstream_, static_cast<GroupRef const*>(ref_dev_), n, total_prep, total_tiles,
                                   reqs[order[i0]].S);
            else
                launch_f64_group(gstream_, static_cast<GroupRef const*>(ref_dev_), n, total_tiles);
            grouped_launches += (total_prep > 0) + (total_tiles > 0);
            grouped_contractions += n;
            i0 = i1;
        }
        ITG_CHECK_CUDA(cudaEventRecord(gdone_, gstream_));
        // each stream's next work comes after the grouped launches
        for (auto const& r : reqs) {
            ITG_CHECK_CUDA(cudaStreamWaitEvent(r.ctx->stream, gdone_, 0));
            r.ctx->kernel_launches += r.S > 0 ? 2 : 1;
        }
    } catch (std::exception const& e) {
        for (auto const& r : reqs) r.fiber->group_error = e.what();
    }
    for (auto const& r : reqs) r.fiber->group_wait = false;
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
    if (!f.running || f.group_wait) return false;
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

bool fiber_group_contract(Ctx& ctx, Plan const& p, double const* A, double const* B, double* C, int S,
                       __nv_bfloat16* panels, int32_t* exps, bool prep_b) {
    FiberScheduler* s = FiberScheduler::of_thread();
    if (!s || !s->current || !s->grouping) return false;
    Fiber* f = s->current;
    if (!f->group_ready) ITG_CHECK_CUDA(cudaEventCreateWithFlags(&f->group_ready, cudaEventDisableTiming));
    ITG_CHECK_CUDA(cudaEventRecord(f->group_ready, ctx.stream));
    s->pending.push_back(GroupRequest{f, &ctx, &p, A, B, C, S, panels, exps, prep_b});
    f->group_wait = true;
    f->live_acct = current_account();
    f->live_cache = current_cache();
    f->live_bypass = cache_bypass();
    if (swapcontext(&f->uc, &s->main_uc) != 0) throw Error(ERR_INTERNAL, "fiber: context switch failed");
    // resumed once flush() has enqueued the grouped launch (the stream waits for it)
    if (!f->group_error.empty()) {
        std::string msg = "grouped launch: " + f->group_error;
        f->group_error.clear();
        throw Error(ERR_CUDA, msg);
    }
    return true;
}

}  // namespace itg
