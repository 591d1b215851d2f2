// Solver pool (see pool.h).
#include "pool.h"
#include <algorithm>
#include <cmath>

namespace itg {

int64_t solve_footprint_estimate(ModelSpec const& m, std::vector<SweepSpec> const& sweeps, int prec) {
    Hamiltonian H = make_hamiltonian(m);
    return solve_footprint_estimate(H.N, H.st.d(), mpo_bond_dim(H), sweeps, prec);
}

namespace {
// Sites, local dimension and MPO bond dimension of a request.
void request_dims(SolveRequest const& r, int& N, int& d, int& D) {
    if (!r.mpo) {
        Hamiltonian H = make_hamiltonian(r.model);
        N = H.N;
        d = H.st.d();
        D = mpo_bond_dim(H);
        return;
    }
    N = (int)r.mpo->W.size();
    d = 1;
    D = 1;
    for (int j = 0; j < N; ++j) {
        auto const& W = *r.mpo->W[j].lay;
        for (auto const& I : W.inds) {
            bool site = false;
            for (auto const& J : r.mpo->psi0[j].lay->inds) site = site || J.id == I.id;
            if (site) d = std::max<int>(d, (int)I.dim());
            else D = std::max<int>(D, (int)I.dim());
        }
    }
}

std::string request_family(SolveRequest const& r, int d, int D) {
    return (r.mpo ? std::string("mpo") : "model" + std::to_string(r.model.type)) + ":d" + std::to_string(d) + ":D" +
           std::to_string(D) + ":p" + std::to_string(r.prec);
}

bool out_of_memory(SolveRecord const& r) { return r.status == ERR_OOM; }
}  // namespace

int64_t solve_footprint_estimate(SolveRequest const& r) {
    int N, d, D;
    request_dims(r, N, d, D);
    return solve_footprint_estimate(N, d, D, r.sweeps, r.prec);
}

int64_t solve_footprint_estimate(int N, int d, int D, std::vector<SweepSpec> const& sweeps, int prec) {
    long maxdim = 1;
    int niter = 2;
    for (auto const& s : sweeps) {
        maxdim = std::max(maxdim, s.maxdim);
        niter = std::max(niter, s.niter);
    }
    // m_b: largest dimension of link b allowed by the schedule and by the half-chains' Hilbert spaces
    std::vector<double> mb(N + 1, 1.0);
    for (int b = 1; b < N; ++b) {
        const double left = std::pow((double)d, std::min(b, 60)), right = std::pow((double)d, std::min(N - b, 60));
        mb[b] = std::min<double>((double)maxdim, std::min(left, right));
    }
    double mps = 0, env = 0, work = 0;
    for (int n = 1; n <= N; ++n) mps += mb[n - 1] * d * mb[n];
    for (int b = 1; b < N; ++b) env += mb[b] * D * mb[b];
    const int S = 6;  // digit planes of the split form
    for (int b = 1; b < N; ++b) {
        const double ml = mb[b - 1], mr = mb[b + 1 <= N ? b + 1 : N];
        const double phi = ml * d * d * mr;
        const double fused = std::max(ml, mr) * d;
        // Davidson: V and H V for every iteration; H_eff intermediates (two of D x phi);
        // bond split: combined copy, density matrix and eigenvectors (or U, V), and
        // the eigensolver's rotation log (30 sweeps x n^2/2 rotations x 16 B per block)
        double w = phi * (2.0 * (niter + 2) + 2.0 * D + 3.0) + 3.0 * fused * fused + 30.0 * fused * fused;
        if (prec == PREC_OZAKI_BF16) w += (2.0 * S / 8.0) * (2.0 * phi + 2.0 * ml * D * ml + 2.0 * mr * D * mr);
        work = std::max(work, w);
    }
    return (int64_t)(8.0 * (mps + env + work)) + (4 << 20);
}

SolverPool::SolverPool(int device, int workers, int slots_per_worker, int64_t budget_bytes)
    : device_(device), workers_(workers), slots_(slots_per_worker), budget_(budget_bytes) {
    ITG_REQUIRE(workers >= 1 && slots_per_worker >= 1, "pool: need at least one worker and one slot");
    ITG_REQUIRE(budget_bytes > 0, "pool: memory budget must be positive");
}

SolverPool::~SolverPool() {
    {
        std::lock_guard<std::mutex> g(mu_);
        stop_ = true;
    }
    cv_work_.notify_all();
    for (auto& t : threads_) t.join();
    if (started_ && std::getenv("ITG_ALLOC_LOG"))
        std::fprintf(stderr,
                     "itg pool allocations: %llu from block caches, %llu driver allocations (%llu bypassing the caches, "
                     "%llu on streams without one), %llu driver frees (%llu refused by a full cache)\n",
                     (unsigned long long)(alloc_counters().cached.load() - alloc0_[0]),
                     (unsigned long long)(alloc_counters().driver_allocs.load() - alloc0_[1]),
                     (unsigned long long)(alloc_counters().bypass.load() - alloc0_[3]),
                     (unsigned long long)(alloc_counters().nocache.load() - alloc0_[4]),
                     (unsigned long long)(alloc_counters().driver_frees.load() - alloc0_[2]),
                     (unsigned long long)(alloc_counters().full.load() - alloc0_[5]));
}

double SolverPool::now() const {
    if (!started_) return 0.0;
    return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0_).count();
}

int64_t SolverPool::submit(SolveRequest req) {
    auto rec = std::make_shared<SolveRecord>();
    {
        int N, d, D;
        request_dims(req, N, d, D);
        rec->est_bytes = solve_footprint_estimate(N, d, D, req.sweeps, req.prec);
        rec->family = request_family(req, d, D);
    }
    ITG_REQUIRE(!req.sweeps.empty(), "pool: empty sweep schedule");
    {
        std::lock_guard<std::mutex> g(mu_);
        rec->id = (int64_t)records_.size();
        rec->t_arrive = std::max(req.arrival, now());
        rec->req = std::move(req);
        records_.push_back(rec);
        st_.submitted++;
        if (rec->est_bytes > budget_) {
            rec->status = ERR_RANGE;
            rec->error = "pool: the request's memory estimate (" + std::to_string(rec->est_bytes) +
                         " bytes) exceeds the pool budget";
            st_.failed++;
            cv_done_.notify_all();
            return rec->id;
        }
        auto pos = std::upper_bound(queue_.begin(), queue_.end(), rec,
                                    [](auto const& a, auto const& b) { return a->t_arrive < b->t_arrive; });
        queue_.insert(pos, rec);
    }
    cv_work_.notify_all();
    return rec->id;
}

void SolverPool::start() {
    {
        std::lock_guard<std::mutex> g(mu_);
        ITG_REQUIRE(!started_, "pool: already started");
        t0_ = std::chrono::steady_clock::now();
        started_ = true;
        alloc0_[0] = alloc_counters().cached.load();
        alloc0_[1] = alloc_counters().driver_allocs.load();
        alloc0_[2] = alloc_counters().driver_frees.load();
        alloc0_[3] = alloc_counters().bypass.load();
        alloc0_[4] = alloc_counters().nocache.load();
        alloc0_[5] = alloc_counters().full.load();
        init_pending_ = workers_;
    }
    for (int w = 0; w < workers_; ++w) threads_.emplace_back(&SolverPool::worker_main, this, w);
    std::unique_lock<std::mutex> lk(mu_);
    cv_done_.wait(lk, [&] { return init_pending_ == 0; });
    if (!init_error_.empty()) {
        stop_ = true;
        lk.unlock();
        cv_work_.notify_all();
        for (auto& t : threads_) t.join();
        threads_.clear();
        throw Error(ERR_CUDA, "pool: worker setup failed: " + init_error_);
    }
}

void SolverPool::set_calibration(int min_solves, double safety) {
    std::lock_guard<std::mutex> g(mu_);
    ITG_REQUIRE(!started_, "pool: calibration is set before start");
    ITG_REQUIRE(min_solves >= 0 && safety >= 1.0, "pool: calibration needs min_solves >= 0 and safety >= 1");
    cal_min_ = min_solves;
    cal_safety_ = safety;
}

void SolverPool::set_grouping(bool on) {
    std::lock_guard<std::mutex> g(mu_);
    ITG_REQUIRE(!started_, "pool: grouping is set before start");
    grouping_ = on;
}

void SolverPool::drain() {
    std::unique_lock<std::mutex> lk(mu_);
    ITG_REQUIRE(started_, "pool: drain before start");
    cv_done_.wait(lk, [&] { return st_.done + st_.failed == st_.submitted; });
}

SolveRecord SolverPool::record(int64_t id) {
    std::lock_guard<std::mutex> g(mu_);
    ITG_REQUIRE(id >= 0 && id < (int64_t)records_.size(), "pool: unknown request id");
    return *records_[id];
}

PoolStats SolverPool::stats() {
    std::lock_guard<std::mutex> g(mu_);
    PoolStats s = st_;
    s.elapsed = now();
    s.grouped_launches = grouped_launches_.load();
    s.grouped_contractions = grouped_contractions_.load();
    return s;
}

std::shared_ptr<SolveRecord> SolverPool::try_admit() {
    std::lock_guard<std::mutex> g(mu_);
    if (queue_.empty() || stop_) return nullptr;
    auto rec = queue_.front();
    const double t = now();
    if (rec->t_arrive > t) return nullptr;
    // first come, first served: the head waits until its memory estimate fits
    int64_t eff = rec->est_bytes;
    if (cal_min_ > 0 && !rec->full_est) {
        auto it = fam_.find(rec->family);
        if (it != fam_.end() && it->second.second >= cal_min_) {
            const double cal = (double)rec->est_bytes * it->second.first * cal_safety_;
            eff = std::min<int64_t>(rec->est_bytes, std::max<int64_t>(int64_t(16) << 20, (int64_t)cal));
        }
    }
    if (st_.running > 0 && st_.reserved_bytes + eff > budget_) return nullptr;
    queue_.pop_front();
    rec->t_admit = t;
    rec->status = -2;
    rec->adm_bytes = eff;
    if (eff < rec->est_bytes) st_.calibrated++;
    st_.reserved_bytes += eff;
    st_.peak_reserved_bytes = std::max(st_.peak_reserved_bytes, st_.reserved_bytes);
    st_.running++;
    st_.peak_running = std::max(st_.peak_running, st_.running);
    return rec;
}

void SolverPool::finish(std::shared_ptr<SolveRecord> const& rec) {
    {
        std::lock_guard<std::mutex> g(mu_);
        st_.reserved_bytes -= rec->adm_bytes;
        st_.running--;
        if (rec->status == 0) {
            st_.done++;
            if (rec->est_bytes > 0) {
                auto& f = fam_[rec->family];
                f.first = std::max(f.first, (double)rec->peak_bytes / (double)rec->est_bytes);
                f.second++;
            }
        } else if (out_of_memory(*rec) && rec->adm_bytes < rec->est_bytes && rec->retries == 0) {
            // admitted below its full estimate and out of memory: again, first in line, by the full estimate
            rec->status = -1;
            rec->error.clear();
            rec->result = DmrgResult{};
            rec->full_est = true;
            rec->retries++;
            st_.retried++;
            queue_.push_front(rec);
        } else {
            st_.failed++;
        }
    }
    cv_done_.notify_all();
    cv_work_.notify_all();
}

namespace {
void run_solve(Ctx& ctx, SolveRecord& rec, SolverPool const& pool) {
    try {
        if (rec.req.mpo) {
            // the caller's MPO and initial MPS, uploaded on this solve's stream
            std::vector<Tensor> W, psi;
            for (auto const& h : rec.req.mpo->W) W.push_back(upload_tensor(ctx, h.lay, h.data.data()));
            for (auto const& h : rec.req.mpo->psi0) psi.push_back(upload_tensor(ctx, h.lay, h.data.data()));
            MPO mpo = mpo_from_tensors(W, psi);
            rec.result = dmrg(ctx, mpo, std::move(psi), rec.req.sweeps, rec.req.prec);
        } else {
            Hamiltonian H = make_hamiltonian(rec.req.model);
            ITG_REQUIRE(H.N >= 2, "pool: need at least two sites");
            MPO mpo = build_mpo(ctx, H);
            auto psi = product_mps(ctx, mpo, H.st, default_state(rec.req.model));
            rec.result = dmrg(ctx, mpo, std::move(psi), rec.req.sweeps, rec.req.prec);
        }
        // the record keeps energies and links; the state only when asked for
        if (!rec.req.keep_mps) rec.result.psi.clear();
        rec.status = 0;
    } catch (Error const& e) {
        rec.status = e.code;
        rec.error = e.what();
    } catch (std::exception const& e) {
        rec.status = ERR_INTERNAL;
        rec.error = e.what();
    }
    ctx.split_scratch.reset();
    try {
        ctx.sync();
    } catch (std::exception const& e) {
        if (rec.status == 0) { rec.status = ERR_CUDA; rec.error = e.what(); }
    }
    rec.t_done = pool.now();
}
}  // namespace

void SolverPool::worker_main(int w) {
    std::vector<std::unique_ptr<Slot>> slots;
    FiberScheduler sched;
    sched.grouping = grouping_;
    try {
        ITG_CHECK_CUDA(cudaSetDevice(device_));
        for (int i = 0; i < slots_; ++i) {
            auto s = std::make_unique<Slot>();
            s->ctx = std::make_unique<Ctx>(device_);
            s->ctx->ensure_pin(1 << 20);
            s->ctx->ensure_stage(8 << 20);
            slots.push_back(std::move(s));
        }
    } catch (std::exception const& e) {
        std::lock_guard<std::mutex> g(mu_);
        init_error_ = e.what();
        slots.clear();
    }
    {
        std::lock_guard<std::mutex> g(mu_);
        --init_pending_;
    }
    cv_done_.notify_all();
    if (slots.empty()) return;
    FiberScheduler::of_thread() = &sched;
    // freed blocks a slot keeps between its solves: an eighth of its share of
    // the budget, at most 256 MiB (not counted against the budget)
    const size_t retain = (size_t)std::min<int64_t>(int64_t(256) << 20, budget_ / (8 * (int64_t)workers_ * slots_));
    int idle_spins = 0;
    for (;;) {
        bool progressed = false;
        int busy = 0;
        for (int i = 0; i < (int)slots.size(); ++i) {
            Slot& s = *slots[i];
            if (!s.rec) {
                if (auto rec = try_admit()) {
                    s.rec = rec;
                    rec->worker = w;
                    rec->slot = i;
                    s.fiber.acct = std::make_shared<MemAccount>();
                    s.fiber.cache = s.ctx->cache;  // the slot's cache, kept across its solves
                    Ctx* ctx = s.ctx.get();
                    SolveRecord* r = rec.get();
                    sched.start(s.fiber, [ctx, r, this] { run_solve(*ctx, *r, *this); });
                    progressed = true;
                }
            } else if (sched.poll(s.fiber)) {
                progressed = true;
            }
            if (s.rec && !s.fiber.running) {
                s.rec->peak_bytes = s.fiber.acct->peak.load();
                finish(s.rec);
                s.rec.reset();
                s.fiber.acct.reset();
                s.fiber.live_acct.reset();
                // the next solve on this slot reuses the freed blocks; what the cache
                // keeps beyond the slot's share of the budget goes back to the driver
                // plans are per slot (their tables are read on its stream only);
                // a finished solve's plans rarely fit the next one
                s.ctx->plans->clear();
                if (s.fiber.cache) s.fiber.cache->trim(retain);
                s.fiber.cache.reset();
                s.fiber.live_cache.reset();
            }
            busy += s.rec ? 1 : 0;
        }
        if (busy == 0) {
            std::unique_lock<std::mutex> lk(mu_);
            if (stop_) break;
            // nothing running here: sleep until a request is submitted, memory is
            // returned, or the next request arrives
            double wait_s = 0.05;
            if (!queue_.empty()) wait_s = std::clamp(queue_.front()->t_arrive - now(), 2e-4, 0.05);
            cv_work_.wait_for(lk, std::chrono::duration<double>(wait_s));
            continue;
        }
        if (!progressed && !sched.pending.empty()) {
            // every solve here waits (for its stream or for a grouped launch):
            // enqueue the waiting contractions as one grouped launch
            const uint64_t l0 = sched.grouped_launches, c0 = sched.grouped_contractions;
            sched.flush();
            grouped_launches_ += (int64_t)(sched.grouped_launches - l0);
            grouped_contractions_ += (int64_t)(sched.grouped_contractions - c0);
            progressed = true;
        }
        if (progressed) {
            idle_spins = 0;
        } else if (++idle_spins > 64) {
            std::this_thread::sleep_for(std::chrono::microseconds(5));
        } else {
            std::this_thread::yield();
        }
    }
    FiberScheduler::of_thread() = nullptr;
}

}  // namespace itg
