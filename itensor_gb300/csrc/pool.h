// Solver pool: many independent ground-state solves on one GPU.
//
// Requests (model, sweep schedule, precision, arrival time) wait in an
// arrival-ordered queue. A request is admitted when its arrival time has
// passed, a solve slot is free, and its device-memory estimate fits in what
// the budget has left; slots free up and memory returns as solves finish, so
// requests that arrive while others run join them (continuous batching).
// Each worker thread owns several slots; a slot is a context (its own stream)
// and a fiber that runs the plain DMRG sweep loop (itensor/mps/dmrg.h:336-467).
// While one solve waits for its stream the thread runs the others, so the
// device sees the kernels of every admitted solve at once. Each slot keeps its
// own contraction plans and freed device blocks (read and reused on its own
// stream only). A solve's result does not depend on what runs beside it:
// kernels are deterministic and solves share no device state.
#pragma once
#include "algo.h"
#include "fiber.h"
#include <condition_variable>
#include <deque>
#include <map>
#include <thread>

namespace itg {

// A caller's MPO and initial MPS, copied to host memory when submitted (the
// solve uploads them on its own stream, so the caller's tensors may be freed
// or changed after submission).
struct HostTensor {
    std::shared_ptr<Layout> lay;
    std::vector<double> data;
};
struct MpoInput {
    std::vector<HostTensor> W, psi0;
};

struct SolveRequest {
    ModelSpec model;                      // used when mpo is empty
    std::shared_ptr<const MpoInput> mpo;  // else the caller's MPO and initial MPS
    bool keep_mps = false;                // the record keeps the final MPS (device memory until freed)
    std::vector<SweepSpec> sweeps;
    int prec = PREC_F64;
    double arrival = 0;          // seconds after the pool started (<= 0: at once)
};

struct SolveRecord {
    int64_t id = 0;
    SolveRequest req;
    int status = -1;             // -1 queued, -2 running, 0 done, else an error code
    std::string error;
    DmrgResult result;
    double t_arrive = 0, t_admit = 0, t_done = 0;   // seconds after the pool started
    int64_t est_bytes = 0, peak_bytes = 0;
    int64_t adm_bytes = 0;       // what admission reserved (the estimate, or its calibrated form)
    std::string family;          // model family and precision (calibration key)
    bool full_est = false;       // admit by the full estimate (after an out-of-memory retry)
    int retries = 0;
    int worker = -1, slot = -1;
};

// Upper bound of the device memory of one solve: dense blocks at the bond
// dimensions the sweep schedule allows (capped by the Hilbert space of each
// half-chain), for the MPS, the environments and one bond step's workspace
// (Davidson vectors, H_eff intermediates, density matrix, split-precision
// digit panels).
int64_t solve_footprint_estimate(ModelSpec const& m, std::vector<SweepSpec> const& sweeps, int prec);
// The same bound for N sites of local dimension d and an MPO of bond dimension D.
int64_t solve_footprint_estimate(int N, int d, int D, std::vector<SweepSpec> const& sweeps, int prec);
int64_t solve_footprint_estimate(SolveRequest const& r);

struct PoolStats {
    int64_t submitted = 0, done = 0, failed = 0;
    int64_t reserved_bytes = 0, peak_reserved_bytes = 0;
    int running = 0, peak_running = 0;
    double elapsed = 0;          // seconds since start
    // grouped launches (split-precision prep + GEMM of several solves' contractions each)
    int64_t grouped_launches = 0, grouped_contractions = 0;
    // admissions by a calibrated estimate; solves re-run after running out of memory
    int64_t calibrated = 0, retried = 0;
};

class SolverPool {
public:
    SolverPool(int device, int workers, int slots_per_worker, int64_t budget_bytes);
    ~SolverPool();
    int64_t submit(SolveRequest req);  // thread-safe, before or after start()
    void start();
    // Cross-solve grouping (before start; off by default): the block GEMMs
    // (FP64 or split precision) that a worker's solves reach while all of them
    // wait run as one grouped launch instead of one launch each.
    void set_grouping(bool on);
    // Calibrated admission (before start; off with min_solves 0, the default).
    // Once min_solves requests of a model family (model type, local and MPO
    // bond dimensions, precision) have finished, the family's requests are
    // admitted by estimate x safety x the largest measured peak/estimate ratio
    // of that family (at least 16 MiB, at most the estimate). A solve admitted
    // that way that runs out of device memory is queued again, first in line,
    // with its full estimate.
    void set_calibration(int min_solves, double safety);
    void drain();                      // blocks until every submitted request has finished
    SolveRecord record(int64_t id);
    PoolStats stats();
    double now() const;

private:
    struct Slot {
        std::unique_ptr<Ctx> ctx;
        Fiber fiber;
        std::shared_ptr<SolveRecord> rec;
    };
    void worker_main(int w);
    std::shared_ptr<SolveRecord> try_admit();
    void finish(std::shared_ptr<SolveRecord> const& rec);

    int device_, workers_, slots_;
    bool grouping_ = false;
    int cal_min_ = 0;
    double cal_safety_ = 2.0;
    std::map<std::string, std::pair<double, int>> fam_;    // family -> (largest peak/estimate, finished)
    std::atomic<int64_t> grouped_launches_{0}, grouped_contractions_{0};
    int64_t budget_;
    std::mutex mu_;
    std::condition_variable cv_done_, cv_work_;
    std::deque<std::shared_ptr<SolveRecord>> queue_;        // by arrival time
    std::vector<std::shared_ptr<SolveRecord>> records_;     // by id
    PoolStats st_;
    bool started_ = false, stop_ = false;
    std::chrono::steady_clock::time_point t0_;
    uint64_t alloc0_[6] = {0, 0, 0, 0, 0, 0};  // allocator counters at start (ITG_ALLOC_LOG)
    std::vector<std::thread> threads_;
    std::string init_error_;
    int init_pending_ = 0;
};

}  // namespace itg
