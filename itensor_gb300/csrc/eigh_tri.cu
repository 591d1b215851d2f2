// Large-block path of the batched symmetric eigensolver. The reference
// diagonalises each density-matrix block with LAPACK dsyev
// (itensor/tensor/algs.cc:34-41): Householder reduction to tridiagonal form,
// then implicit QL/QR with the transformations accumulated. This file does the
// same three stages, laid out for the GPU:
//
//   1. tri_reduce_kernel: Householder tridiagonalisation of one block by a
//      cluster of CTAs (columns dealt round-robin to the CTAs; per column k the
//      owner builds the reflector, all CTAs form p = tau A v over their columns,
//      then apply the rank-2 update A -= v w^T + w v^T with w = p - (tau/2)(p.v) v;
//      two cluster barriers per column). Reflectors are kept below the subdiagonal.
//   2. the implicit QL recurrence on (d, e) (tridiag_ql.cpp): a chain of
//      dependent scalar FP64 operations, ~n^2 rotations per block with a square
//      root and two divisions each. On this part an SM issues ~2 FP64 FMAs per
//      clock, so one thread's dependent FP64 chain advances by one operation
//      every few tens of cycles (measured: ~1.7 us per rotation on the SM); the
//      host core runs it in nanoseconds per operation. It records the plane
//      rotations; the eigenvalues go back to the caller, which truncates;
//   3. tri_rot_kernel: only the kept eigenvectors of the tridiagonal matrices:
//      the recorded rotations applied in reverse to unit vectors, a tile of
//      vectors per CTA in shared memory, the CTA's 32 warps applying
//      rotations of 32 sweeps at once on a lockstep schedule from the host;
//   4. tri_applyq_kernel: the Householder reflectors applied to each kept
//      vector (one warp per vector), written to the output in eigenvalue order.
// The FP64 work is ~n^3 FMA for the reduction, then ~n^2 rotations and ~2n^2
// reflector FMAs per kept vector, against ~4n^3 per Jacobi sweep for every vector.
#include "ops.h"
#include "eigh_tri.h"
#include "tridiag_ql.h"
#include <cooperative_groups.h>
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <numeric>
#include <condition_variable>
#include <functional>
#include <mutex>
#include <unistd.h>
#include <thread>

namespace cg = cooperative_groups;

namespace itg {

namespace {
constexpr int TRI_THREADS = 256;
constexpr int TRI_APPLYQ_WARPS = 4;       // kept vectors per CTA in the reflector stage (one warp each)
constexpr int TRI_ROT_WARPS = 32;        // sweeps applied at once to one row tile
constexpr int TRI_ROT_WINDOW = 4;        // lockstep steps between barriers
constexpr size_t TRI_SMEM_LIMIT = 200 * 1024;

struct TriJob {
    int64_t a_off;     // input block (n x n, column-major) in src
    int64_t v_off;     // eigenvectors (columns, eigenvalues descending) in vout
    int64_t w_off;     // eigenvalues (descending) in wout
    int64_t s_off;     // 2 n^2 doubles: reduced matrix + reflectors, then Q
    int64_t aux_off;   // tri_aux_doubles(n) doubles in aux: d, e, tau, v, p, partial sums
    int32_t n, keep;   // keep: eigenvectors wanted (the largest eigenvalues), set before the vector stage
};
struct ColJob { int32_t job, c0; };
struct RowJob { int32_t job, r0; };

__host__ __device__ inline int64_t tri_aux_doubles(int n) { return 5 * (int64_t)n + 16; }

__device__ __forceinline__ double warp_sum(double v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// sum_i x[i] y[i] over i = i0, i0 + step, ... < n with four independent
// accumulators (a single chain of dependent FP64 FMAs leaves the FP64 pipe
// mostly idle: each FMA waits for the previous one), added in a fixed order.
__device__ __forceinline__ double dot4(double const* __restrict__ x, double const* __restrict__ y, int i0, int n,
                                       int step) {
    double a0 = 0.0, a1 = 0.0, a2 = 0.0, a3 = 0.0;
    int i = i0;
    const int step4 = 4 * step;
    for (; i + 3 * step < n; i += step4) {
        double const* xp = x + i;
        double const* yp = y + i;
        a0 = fma(xp[0], yp[0], a0);
        a1 = fma(xp[step], yp[step], a1);
        a2 = fma(xp[2 * step], yp[2 * step], a2);
        a3 = fma(xp[3 * step], yp[3 * step], a3);
    }
    for (; i < n; i += step) a0 = fma(x[i], y[i], a0);
    return (a0 + a1) + (a2 + a3);
}

// Sum over the CTA (a fixed tree: lanes, then the warps' sums); every thread
// gets the same value. The warps' sums are combined by shuffles, not by a
// serial loop in every warp: each FP64 instruction costs a warp tens of cycles.
__device__ double cta_sum(double v, double* red) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    v = warp_sum(v);
    __syncthreads();
    if (lane == 0) red[warp] = v;
    __syncthreads();
    double s = lane < nw ? red[lane] : 0.0;
    for (int o = 4; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);   // nw <= 8
    return __shfl_sync(0xffffffffu, s, 0);
}

// Householder reflector for column k (rows k+1..n-1), dlarfg's convention:
// H = I - tau v v^T with v[k+1] = 1 and H [alpha; x] = [beta; 0]. Run by every
// thread of the owning CTA.
__device__ void tri_reflector(int k, int n, double* A, double* d, double* e, double* tau, double* vg, double* red) {
    __shared__ double sc[3];   // beta, tau, 1 / (alpha - beta): computed once, by thread 0
    double* col = A + (size_t)k * n;
    const double alpha = col[k + 1];
    double ss = dot4(col, col, k + 2 + threadIdx.x, n, blockDim.x);
    ss = cta_sum(ss, red);
    if (threadIdx.x == 0) {
        double t = 0.0, beta = alpha, scal = 0.0;
        if (ss > 0.0) {
            beta = -copysign(sqrt(fma(alpha, alpha, ss)), alpha);
            t = (beta - alpha) / beta;
            scal = 1.0 / (alpha - beta);
        }
        sc[0] = beta;
        sc[1] = t;
        sc[2] = scal;
    }
    __syncthreads();
    const double beta = sc[0], t = sc[1], scal = sc[2];
    for (int i = k + 2 + threadIdx.x; i < n; i += blockDim.x) {
        const double v = col[i] * scal;
        col[i] = v;
        __stcg(vg + i, v);
    }
    if (threadIdx.x == 0) {
        __stcg(vg + k + 1, 1.0);
        __stcg(tau + k, t);
        __stcg(d + k, col[k]);
        __stcg(e + k, beta);
    }
}

__global__ void __launch_bounds__(TRI_THREADS, 1) tri_reduce_kernel(TriJob const* __restrict__ jobs,
                                                                 double const* __restrict__ src,
                                                                 double* __restrict__ scratch,
                                                                 double* __restrict__ aux) {
    extern __shared__ double sm[];
    __shared__ double red[TRI_THREADS / 32];
    cg::cluster_group cl = cg::this_cluster();
    const int C = (int)cl.num_blocks();
    const int rank = (int)cl.block_rank();
    const TriJob jb = jobs[blockIdx.x / C];
    const int n = jb.n;
    double* A = scratch + jb.s_off;
    double* d = aux + jb.aux_off;
    double* e = d + n;
    double* tau = e + n;
    double* vg = tau + n;
    double* pg = vg + n;
    double* part = pg + n;
    double* vs = sm;
    double* ws = sm + n;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;

    for (int j = rank; j < n; j += C)
        for (int i = threadIdx.x; i < n; i += blockDim.x) A[(size_t)j * n + i] = src[jb.a_off + (size_t)j * n + i];
    __syncthreads();
    if (n >= 3 && rank == 0) tri_reflector(0, n, A, d, e, tau, vg, red);
    cl.sync();
    for (int k = 0; k + 2 < n; ++k) {
        const double tk = __ldcg(tau + k);
        // first column > k owned by this CTA
        const int j0 = k + 1 + (((rank - (k + 1)) % C) + C) % C;
        for (int i = k + 1 + threadIdx.x; i < n; i += blockDim.x) vs[i] = __ldcg(vg + i);
        __syncthreads();
        double mine = 0.0;
        if (tk != 0.0) {
            // two columns at a time: their dot products and warp reductions
            // interleave (each reduction is a chain of dependent shuffles and adds)
            const int js = nw * C;
            int j = j0 + warp * C;
            for (; j + js < n; j += 2 * js) {
                double s1 = dot4(A + (size_t)j * n, vs, k + 1 + lane, n, 32);
                double s2 = dot4(A + (size_t)(j + js) * n, vs, k + 1 + lane, n, 32);
                for (int o = 16; o > 0; o >>= 1) {
                    s1 += __shfl_xor_sync(0xffffffffu, s1, o);
                    s2 += __shfl_xor_sync(0xffffffffu, s2, o);
                }
                if (lane == 0) {
                    const double p1 = tk * s1, p2 = tk * s2;
                    __stcg(pg + j, p1);
                    mine = fma(p1, vs[j], mine);
                    __stcg(pg + j + js, p2);
                    mine = fma(p2, vs[j + js], mine);
                }
            }
            if (j < n) {
                const double pj = tk * warp_sum(dot4(A + (size_t)j * n, vs, k + 1 + lane, n, 32));
                if (lane == 0) {
                    __stcg(pg + j, pj);
                    mine = fma(pj, vs[j], mine);
                }
            }
        }
        const double psum = cta_sum(mine, red);
        if (threadIdx.x == 0) __stcg(part + rank, psum);
        cl.sync();
        if (tk != 0.0) {
            // sum of the C partial dot products, as a shuffle tree (C <= 16)
            double K = lane < C ? __ldcg(part + lane) : 0.0;
            for (int o = 8; o > 0; o >>= 1) K += __shfl_xor_sync(0xffffffffu, K, o);
            K = __shfl_sync(0xffffffffu, K, 0) * (-0.5 * tk);
            for (int i = k + 1 + threadIdx.x; i < n; i += blockDim.x) ws[i] = fma(K, vs[i], __ldcg(pg + i));
            __syncthreads();
            for (int j = j0 + warp * C; j < n; j += nw * C) {
                double* col = A + (size_t)j * n;
                const double vj = vs[j], wj = ws[j];
#pragma unroll 4
                for (int i = k + 1 + lane; i < n; i += 32) col[i] = fma(-vs[i], wj, fma(-ws[i], vj, col[i]));
            }
        }
        __syncthreads();
        if (k + 3 < n && rank == (k + 1) % C) tri_reflector(k + 1, n, A, d, e, tau, vg, red);
        cl.sync();
    }
    if (rank == 0 && threadIdx.x == 0) {
        if (n >= 2) {
            d[n - 2] = __ldcg(A + (size_t)(n - 2) * n + (n - 2));
            e[n - 2] = __ldcg(A + (size_t)(n - 2) * n + (n - 1));
            d[n - 1] = __ldcg(A + (size_t)(n - 1) * n + (n - 1));
            tau[n - 2] = 0.0;
        } else {
            d[0] = __ldcg(A);
        }
        e[n - 1] = 0.0;
        tau[n - 1] = 0.0;
    }
}

// z = H_0 (H_1 (... H_{n-3} y)) for the kept columns y of Y (n x k, column-major,
// in the second half of the block's scratch): the eigenvectors of the block,
// written to vout in eigenvalue order. One warp per column; H_k acts on rows
// k+1..n-1 with v[k+1] = 1 and v[i] stored below the subdiagonal of column k.
__global__ void __launch_bounds__(TRI_APPLYQ_WARPS * 32) tri_applyq_kernel(ColJob const* __restrict__ cjobs,
                                                                          TriJob const* __restrict__ jobs,
                                                                          double const* __restrict__ scratch,
                                                                          double const* __restrict__ aux,
                                                                          double* __restrict__ vout, int nmax) {
    pdl_wait();
    extern __shared__ double sm[];
    const ColJob cj = cjobs[blockIdx.x];
    const TriJob jb = jobs[cj.job];
    const int n = jb.n;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int j = cj.c0 + warp;
    if (j >= jb.keep) return;
    double const* Rf = scratch + jb.s_off;               // reflectors below the subdiagonal
    double const* Y = scratch + jb.s_off + (size_t)n * n;
    double const* tau = aux + jb.aux_off + 2 * (size_t)n;
    double* y = sm + (size_t)warp * nmax;
    for (int i = lane; i < n; i += 32) y[i] = Y[(size_t)j * n + i];
    __syncwarp();
    for (int k = n - 3; k >= 0; --k) {
        const double t = tau[k];
        if (t == 0.0) continue;
        double const* v = Rf + (size_t)k * n;
        const double dt = t * (warp_sum(dot4(v, y, k + 2 + lane, n, 32)) + y[k + 1]);
        __syncwarp();
        if (lane == 0) y[k + 1] -= dt;
#pragma unroll 4
        for (int i = k + 2 + lane; i < n; i += 32) y[i] = fma(-dt, v[i], y[i]);
        __syncwarp();
    }
    for (int i = lane; i < n; i += 32) vout[jb.v_off + (size_t)j * n + i] = y[i];
}

// The vector stage's per-block records (offsets into the uploaded blob).
struct QlOut {
    int64_t hdr_off;   // sweeps (QlSweep = int4: l, m, rotation offset, 0), mirrored and reversed
    int64_t rot_off;   // rotations (QlRot = double2: c, s) in that order
    int64_t sched_off; // TRI_ROT_WARPS + 1 entry offsets, then entries (QlStart = int2: start step, sweep)
    int64_t sel_off;   // kept eigenvalues' positions in the QL output (int32), descending eigenvalue order
    int32_t nsweeps, nsteps;
};

// Kept eigenvectors of the tridiagonal matrix: rows r0..r0+R-1 of Y^T, row r
// starting as the unit vector of the r-th kept eigenvalue, times the QL
// rotations in reverse order (G e_j = G_1 (G_2 (... G_T e_j))). In mirrored
// column order (column c holds component n-1-c) the reversed sequence is again
// a series of sweeps that run down the columns with the recorded (c, s), so the
// same lockstep schedule applies: the CTA's warps apply rotations of different
// sweeps at once, a barrier every TRI_ROT_WINDOW steps, and the host's schedule
// keeps the warps of one window on disjoint columns. Rotation at column i:
// (z_i, z_{i+1}) <- (c z_i - s z_{i+1}, s z_i + c z_{i+1}). The tile lives in
// shared memory as tile[col * R + row], lane = row; Y (n x keep) is written to
// the second half of the block's scratch.
__global__ void __launch_bounds__(TRI_ROT_WARPS * 32) tri_rot_kernel(RowJob const* __restrict__ rjobs,
                                                                     TriJob const* __restrict__ jobs,
                                                                     double* __restrict__ scratch,
                                                                     QlOut const* __restrict__ qo,
                                                                     char const* __restrict__ blob, int R) {
    pdl_wait();
    extern __shared__ double tile[];
    const RowJob rj = rjobs[blockIdx.x];
    const TriJob jb = jobs[rj.job];
    const QlOut o = qo[rj.job];
    const int n = jb.n;
    const int rows = min(R, jb.keep - rj.r0);
    int32_t const* sel = reinterpret_cast<int32_t const*>(blob + o.sel_off);
    for (int idx = threadIdx.x; idx < n * R; idx += blockDim.x) {
        const int c = idx / R, r = idx % R;
        tile[idx] = (r < rows && c == n - 1 - __ldg(sel + rj.r0 + r)) ? 1.0 : 0.0;
    }
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    int4 const* hd = reinterpret_cast<int4 const*>(blob + o.hdr_off);
    double2 const* lg = reinterpret_cast<double2 const*>(blob + o.rot_off);
    int32_t const* woff = reinterpret_cast<int32_t const*>(blob + o.sched_off);
    int2 const* ent = reinterpret_cast<int2 const*>(blob + o.sched_off + 8 * ((TRI_ROT_WARPS + 2) / 2));
    int e = __ldg(woff + warp);
    const int e_end = __ldg(woff + warp + 1);
    int S = 0, len = 0, m = 0, off = 0;
    bool have = false;
    auto fetch = [&]() {
        have = e < e_end;
        if (have) {
            const int2 x = __ldg(ent + e);
            const int4 h = __ldg(hd + x.y);
            S = x.x;
            m = h.y;
            len = h.y - h.x;
            off = h.z;
        }
    };
    fetch();
    const bool row_ok = lane < rows;
    for (int s0 = 0; s0 < o.nsteps; s0 += TRI_ROT_WINDOW) {
#pragma unroll
        for (int u = 0; u < TRI_ROT_WINDOW; ++u) {
            const int s = s0 + u;
            if (have && s >= S + len) {
                ++e;
                fetch();
            }
            if (have && s >= S && row_ok) {
                const int j = s - S, i = m - 1 - j;
                const double2 q = __ldg(lg + off + j);
                const double a = tile[i * R + lane], b = tile[(i + 1) * R + lane];
                tile[(i + 1) * R + lane] = fma(q.y, a, q.x * b);
                tile[i * R + lane] = fma(q.x, a, -q.y * b);
            }
        }
        __syncthreads();
    }
    double* Y = scratch + jb.s_off + (size_t)n * n;
    for (int idx = threadIdx.x; idx < n * R; idx += blockDim.x) {
        const int c = idx / R, r = idx % R;
        if (r < rows) Y[(size_t)(rj.r0 + r) * n + (n - 1 - c)] = tile[idx];
    }
}

// Sorted eigenvalues of every block to wout (one CTA per block).
__global__ void tri_wout_kernel(TriJob const* __restrict__ jobs, double const* __restrict__ sorted,
                                int64_t const* __restrict__ soff, double* __restrict__ wout) {
    pdl_wait();
    const TriJob jb = jobs[blockIdx.x];
    const int64_t o = soff[blockIdx.x];
    for (int i = threadIdx.x; i < jb.n; i += blockDim.x) wout[jb.w_off + i] = sorted[o + i];
}

// CTAs per block in the reduction: 16-32 columns each, at most 16 (a
// non-portable cluster size, opted into at launch)
int cluster_for(int n) {
    if (n >= 256) return 16;
    if (n >= 128) return 8;
    if (n >= 64) return 4;
    if (n >= 32) return 2;
    return 1;
}
}  // namespace

struct TriPending {
    std::vector<EigItem> items;   // ordered by cluster size, largest first
    std::vector<int> ids;         // the caller's id of each item
    std::vector<TriJob> jobs;
    DevBufPtr buf;                // jobs table | aux (d, e, tau, v, p, partials)
    size_t o_aux = 0;
    int nmax = 0;
    std::vector<std::vector<QlSweep>> sweeps;   // QL sweeps and rotations per block
    std::vector<std::vector<QlRot>> rots;
    std::vector<std::vector<int32_t>> order;    // eigenvalue positions, descending (ties by position)
    std::vector<int> status;
};
void TriPendingFree::operator()(TriPending* p) const { delete p; }

namespace {
// Persistent host threads for the per-block host stages (the QL recurrence,
// the rotation schedules). One caller at a time uses them; a caller that
// finds them busy runs its blocks itself. Spawning threads per bond split
// cost about 0.5 ms each time.
class HostPool {
public:
    static HostPool& get() {
        static HostPool p;
        return p;
    }
    // Runs f(b) for every b < n on the pool and the calling thread; false if
    // the pool is busy (nothing ran).
    bool run(int n, std::function<void(int)> const& f) {
        // (a forked child has none of the parent's threads)
        if (getpid() != pid_) return false;
        std::unique_lock<std::mutex> busy(use_, std::try_to_lock);
        if (!busy.owns_lock() || threads_.empty()) return false;
        {
            std::lock_guard<std::mutex> g(mu_);
            job_ = &f;
            n_ = n;
            next_.store(0);
            pending_ = (int)threads_.size();
            ++gen_;
        }
        cv_.notify_all();
        work();
        std::unique_lock<std::mutex> g(mu_);
        done_.wait(g, [&] { return pending_ == 0; });
        job_ = nullptr;
        return true;
    }
    ~HostPool() {
        {
            std::lock_guard<std::mutex> g(mu_);
            stop_ = true;
        }
        cv_.notify_all();
        for (auto& t : threads_) t.join();
    }

private:
    HostPool() : pid_(getpid()) {
        const unsigned hc = std::thread::hardware_concurrency();
        const int nt = std::max(0, std::min(15, (int)hc - 1));
        for (int t = 0; t < nt; ++t) threads_.emplace_back([this] { loop(); });
    }
    void work() {
        for (int b; (b = next_.fetch_add(1)) < n_;) (*job_)(b);
    }
    void loop() {
        uint64_t seen = 0;
        for (;;) {
            {
                std::unique_lock<std::mutex> g(mu_);
                cv_.wait(g, [&] { return stop_ || gen_ != seen; });
                if (stop_) return;
                seen = gen_;
            }
            work();
            std::lock_guard<std::mutex> g(mu_);
            if (--pending_ == 0) done_.notify_all();
        }
    }
    std::vector<std::thread> threads_;
    std::mutex use_, mu_;
    std::condition_variable cv_, done_;
    std::function<void(int)> const* job_ = nullptr;
    std::atomic<int> next_{0};
    int n_ = 0, pending_ = 0;
    uint64_t gen_ = 0;
    bool stop_ = false;
    pid_t pid_;
};

// Runs f(b) for b < n on the calling thread, or on the host pool as well when
// the work is large and the caller is not a solver-pool fiber (whose workers
// already run one solve each).
template <typename F>
void for_blocks(int n, double work, F const& f) {
    if (n > 1 && !fiber_active() && work > 2e5) {
        std::function<void(int)> fn = [&](int b) { f(b); };
        if (HostPool::get().run(n, fn)) return;
    }
    for (int b = 0; b < n; ++b) f(b);
}
size_t a16(size_t x) { return (x + 15) / 16 * 16; }
}  // namespace

TriPendingPtr tri_eigh_begin(Ctx& ctx, std::vector<EigItem> const& items_in, std::vector<int> const& ids_in,
                             double const* src, double* wout, double* scratch, int* bad) {
    *bad = 0;
    TriPendingPtr P(new TriPending);
    if (items_in.empty()) return P;
    // items ordered by cluster size (largest first), so that each size is one launch
    std::vector<int> ord(items_in.size());
    std::iota(ord.begin(), ord.end(), 0);
    std::stable_sort(ord.begin(), ord.end(),
                     [&](int x, int y) { return cluster_for(items_in[x].n) > cluster_for(items_in[y].n); });
    for (int i : ord) {
        P->items.push_back(items_in[i]);
        P->ids.push_back(ids_in[i]);
    }
    auto const& items = P->items;
    const int nj = (int)items.size();
    for (auto const& it : items) P->nmax = std::max(P->nmax, it.n);
    ITG_REQUIRE(P->nmax <= TRI_MAX_N, "tri_eigh: block larger than the tridiagonal path supports");
    P->jobs.resize(nj);
    int64_t aux_tot = 0;
    for (int b = 0; b < nj; ++b) {
        TriJob& j = P->jobs[b];
        j = TriJob{};
        j.a_off = items[b].a_off;
        j.v_off = items[b].v_off;
        j.w_off = items[b].w_off;
        j.s_off = items[b].s_off;
        j.aux_off = aux_tot;
        aux_tot += tri_aux_doubles(items[b].n);
        j.n = items[b].n;
        j.keep = 0;
    }
    const size_t up = a16(sizeof(TriJob) * nj);
    P->o_aux = up;
    P->buf = dev_alloc(up + sizeof(double) * aux_tot, ctx.stream);
    ctx.ensure_stage(up);
    std::memcpy(ctx.stage, P->jobs.data(), sizeof(TriJob) * nj);
    char* db = P->buf->as<char>();
    ITG_CHECK_CUDA(cudaMemcpyAsync(db, ctx.stage, up, cudaMemcpyHostToDevice, ctx.stream));
    TriJob const* d_jobs = reinterpret_cast<TriJob const*>(db);
    double* d_aux = reinterpret_cast<double*>(db + P->o_aux);
    const bool timing = std::getenv("ITG_EIG_TIME") != nullptr;
    auto t0 = std::chrono::steady_clock::now();

    // 1. reduction: one launch per cluster size; the launches are independent,
    //    so they run side by side on the context's side streams
    {
        const size_t smem = sizeof(double) * 2 * (size_t)P->nmax;
        grow_smem_attr((void const*)tri_reduce_kernel, smem);
        static const bool cluster16 = [] {
            ITG_CHECK_CUDA(cudaFuncSetAttribute(tri_reduce_kernel, cudaFuncAttributeNonPortableClusterSizeAllowed, 1));
            return true;
        }();
        (void)cluster16;
        int ngroups = 0;
        for (int b = 0; b < nj;) {
            int e = b;
            while (e < nj && cluster_for(items[e].n) == cluster_for(items[b].n)) ++e;
            ++ngroups;
            b = e;
        }
        const bool fan = ngroups > 1;
        if (fan) ctx.fork();
        int g = 0, b = 0;
        while (b < nj) {
            const int C = cluster_for(items[b].n);
            int e = b;
            while (e < nj && cluster_for(items[e].n) == C) ++e;
            cudaLaunchConfig_t cfg = {};
            cfg.gridDim = dim3((unsigned)((e - b) * C));
            cfg.blockDim = dim3(TRI_THREADS);
            cfg.dynamicSmemBytes = smem;
            cfg.stream = fan ? ctx.side_stream(g % Ctx::NSIDE) : ctx.stream;
            cudaLaunchAttribute attr[1];
            attr[0].id = cudaLaunchAttributeClusterDimension;
            attr[0].val.clusterDim.x = (unsigned)C;
            attr[0].val.clusterDim.y = 1;
            attr[0].val.clusterDim.z = 1;
            cfg.attrs = attr;
            cfg.numAttrs = 1;
            ITG_CHECK_CUDA(cudaLaunchKernelEx(&cfg, tri_reduce_kernel, d_jobs + b, src, scratch, d_aux));
            ctx.kernel_launches++;
            b = e;
            ++g;
        }
        if (fan) ctx.join(std::min(ngroups, (int)Ctx::NSIDE));
    }
    // 2. (d, e) of every block to the host; QL there
    const size_t aux_bytes = sizeof(double) * aux_tot;
    ctx.ensure_pin(aux_bytes);
    ITG_CHECK_CUDA(cudaMemcpyAsync(ctx.pin, d_aux, aux_bytes, cudaMemcpyDeviceToHost, ctx.stream));
    ctx.sync();
    auto t1 = std::chrono::steady_clock::now();
    std::vector<double> de(static_cast<double*>(ctx.pin), static_cast<double*>(ctx.pin) + aux_tot);
    P->sweeps.resize(nj);
    P->rots.resize(nj);
    P->order.resize(nj);
    P->status.assign(nj, 0);
    std::vector<std::vector<double>> sorted(nj);
    double work = 0;
    for (auto const& it : items) work += (double)it.n * it.n;
    for_blocks(nj, work, [&](int b) {
        const int n = items[b].n;
        double* d = de.data() + P->jobs[b].aux_off;
        P->status[b] = tridiag_ql(n, d, d + n, P->sweeps[b], P->rots[b]);
        auto& o = P->order[b];
        o.resize(n);
        std::iota(o.begin(), o.end(), 0);
        std::stable_sort(o.begin(), o.end(), [&](int x, int y) { return d[x] > d[y]; });
        sorted[b].resize(n);
        for (int i = 0; i < n; ++i) sorted[b][i] = d[o[i]];
    });
    for (int b = 0; b < nj; ++b) *bad += (P->status[b] != 0);
    auto t2 = std::chrono::steady_clock::now();
    // 3. sorted eigenvalues to wout
    {
        int64_t tot = 0;
        std::vector<int64_t> soff(nj);
        for (int b = 0; b < nj; ++b) { soff[b] = tot; tot += items[b].n; }
        const size_t o_s = a16(sizeof(int64_t) * nj), bytes = o_s + sizeof(double) * tot;
        ctx.ensure_stage(bytes);
        char* st = static_cast<char*>(ctx.stage);
        std::memcpy(st, soff.data(), sizeof(int64_t) * nj);
        for (int b = 0; b < nj; ++b)
            std::memcpy(st + o_s + sizeof(double) * soff[b], sorted[b].data(), sizeof(double) * items[b].n);
        DevBuf wb(bytes, ctx.stream);
        ITG_CHECK_CUDA(cudaMemcpyAsync(wb.p, st, bytes, cudaMemcpyHostToDevice, ctx.stream));
        launch_pdl(ctx, nj, 128, 0, tri_wout_kernel, d_jobs, reinterpret_cast<double const*>(wb.as<char>() + o_s),
                                                     wb.as<int64_t>(), wout);
        ITG_CHECK_CUDA(cudaGetLastError());
        ctx.kernel_launches++;
    }
    if (timing) {
        std::fprintf(stderr, "itg tri begin (ms): reduce+copy %.3f host ql %.3f; n:",
                     std::chrono::duration<double, std::milli>(t1 - t0).count(),
                     std::chrono::duration<double, std::milli>(t2 - t1).count());
        for (int b = 0; b < nj; ++b) std::fprintf(stderr, " %d", items[b].n);
        std::fprintf(stderr, "\n");
    }
    return P;
}

void tri_eigh_finish(Ctx& ctx, TriPending& P, std::vector<int> const& keep, double* vout, double* scratch) {
    const int nj = (int)P.items.size();
    if (nj == 0) return;
    auto const& items = P.items;
    int kmax = 0;
    for (int b = 0; b < nj; ++b) {
        const int k = P.status[b] == 0 ? std::max(0, std::min(keep.at(P.ids[b]), items[b].n)) : 0;
        P.jobs[b].keep = k;
        kmax = std::max(kmax, k);
    }
    if (kmax == 0) return;
    const bool timing = std::getenv("ITG_EIG_TIME") != nullptr;
    auto t0 = std::chrono::steady_clock::now();
    // rows per tile of the rotation pass (lane = row): a full warp, fewer when
    // shared memory runs out
    int R = 32;
    while (R > 1 && sizeof(double) * (size_t)R * P.nmax > TRI_SMEM_LIMIT) R /= 2;
    // host: the reversed rotation sequence in mirrored columns, its lockstep
    // schedule, and the kept eigenvalues' positions
    std::vector<std::vector<QlSweep>> msw(nj);
    std::vector<std::vector<QlRot>> mrot(nj);
    std::vector<std::vector<int32_t>> woff(nj);
    std::vector<std::vector<QlStart>> ent(nj);
    std::vector<int> steps(nj, 0);
    double work = 0;
    for (int b = 0; b < nj; ++b) work += (double)P.rots[b].size() * (P.jobs[b].keep > 0);
    for_blocks(nj, work * 8, [&](int b) {
        const int n = items[b].n;
        if (P.jobs[b].keep == 0) return;
        auto const& sw = P.sweeps[b];
        auto const& rt = P.rots[b];
        msw[b].reserve(sw.size());
        mrot[b].reserve(rt.size());
        for (int t = (int)sw.size() - 1; t >= 0; --t) {
            const int l = sw[t].l, m = sw[t].m, len = m - l;
            msw[b].push_back(QlSweep{n - 1 - m, n - 1 - l, (int32_t)mrot[b].size(), 0});
            for (int j = 0; j < len; ++j) mrot[b].push_back(rt[sw[t].off + (len - 1 - j)]);
        }
        steps[b] = ql_schedule(n, msw[b], TRI_ROT_WARPS, TRI_ROT_WINDOW, woff[b], ent[b]);
    });
    // blob: QlOut table | sweeps | rotations | schedules | kept positions
    std::vector<QlOut> qo(nj);
    size_t n_sw = 0, n_rot = 0, n_sched = 0, n_sel = 0;
    for (int b = 0; b < nj; ++b) {
        n_sw += msw[b].size();
        n_rot += mrot[b].size();
        n_sched += 2 * ((TRI_ROT_WARPS + 2) / 2) + 2 * ent[b].size();
        n_sel += P.jobs[b].keep;
    }
    const size_t b_hdr = a16(sizeof(QlOut) * nj), b_rot = a16(b_hdr + sizeof(QlSweep) * n_sw);
    const size_t b_sched = a16(b_rot + sizeof(QlRot) * n_rot), b_sel = a16(b_sched + sizeof(int32_t) * n_sched);
    const size_t blob_bytes = a16(b_sel + sizeof(int32_t) * n_sel);
    if (ctx.stage_bytes < blob_bytes) ctx.ensure_stage(blob_bytes + blob_bytes / 2);
    char* st = static_cast<char*>(ctx.stage);
    {
        size_t o_sw = b_hdr, o_rot = b_rot, o_sc = b_sched, o_sel = b_sel;
        for (int b = 0; b < nj; ++b) {
            qo[b] = QlOut{};
            if (P.jobs[b].keep == 0) continue;
            qo[b].hdr_off = (int64_t)o_sw;
            qo[b].rot_off = (int64_t)o_rot;
            qo[b].sched_off = (int64_t)o_sc;
            qo[b].sel_off = (int64_t)o_sel;
            qo[b].nsweeps = (int32_t)msw[b].size();
            qo[b].nsteps = steps[b];
            std::memcpy(st + o_sw, msw[b].data(), sizeof(QlSweep) * msw[b].size());
            o_sw += sizeof(QlSweep) * msw[b].size();
            std::memcpy(st + o_rot, mrot[b].data(), sizeof(QlRot) * mrot[b].size());
            o_rot += sizeof(QlRot) * mrot[b].size();
            std::vector<int32_t> sc(woff[b]);
            sc.resize(2 * ((TRI_ROT_WARPS + 2) / 2), 0);
            for (auto const& x : ent[b]) { sc.push_back(x.step); sc.push_back(x.sweep); }
            std::memcpy(st + o_sc, sc.data(), sizeof(int32_t) * sc.size());
            o_sc += sizeof(int32_t) * sc.size();
            std::memcpy(st + o_sel, P.order[b].data(), sizeof(int32_t) * P.jobs[b].keep);
            o_sel += sizeof(int32_t) * P.jobs[b].keep;
        }
        std::memcpy(st, qo.data(), sizeof(QlOut) * nj);
    }
    DevBuf blob(blob_bytes, ctx.stream);
    ITG_CHECK_CUDA(cudaMemcpyAsync(blob.p, st, blob_bytes, cudaMemcpyHostToDevice, ctx.stream));
    // the jobs table again (now with the kept counts) and the tile lists, staged
    // once the blob's copy has read the stage
    std::vector<RowJob> rjobs;
    std::vector<ColJob> cjobs;
    for (int b = 0; b < nj; ++b) {
        for (int r0 = 0; r0 < P.jobs[b].keep; r0 += R) rjobs.push_back(RowJob{b, r0});
        for (int c0 = 0; c0 < P.jobs[b].keep; c0 += TRI_APPLYQ_WARPS) cjobs.push_back(ColJob{b, c0});
    }
    const size_t jbytes = sizeof(TriJob) * nj, o_rj = a16(jbytes), o_cj = a16(o_rj + sizeof(RowJob) * rjobs.size());
    const size_t tbytes = o_cj + sizeof(ColJob) * cjobs.size();
    ctx.sync();
    ctx.ensure_stage(tbytes);
    st = static_cast<char*>(ctx.stage);
    std::memcpy(st, P.jobs.data(), jbytes);
    std::memcpy(st + o_rj, rjobs.data(), sizeof(RowJob) * rjobs.size());
    std::memcpy(st + o_cj, cjobs.data(), sizeof(ColJob) * cjobs.size());
    char* db = P.buf->as<char>();
    ITG_CHECK_CUDA(cudaMemcpyAsync(db, st, jbytes, cudaMemcpyHostToDevice, ctx.stream));
    DevBuf tabs(tbytes - o_rj + 16, ctx.stream);
    ITG_CHECK_CUDA(cudaMemcpyAsync(tabs.p, st + o_rj, tbytes - o_rj, cudaMemcpyHostToDevice, ctx.stream));
    TriJob const* d_jobs = reinterpret_cast<TriJob const*>(db);
    double const* d_aux = reinterpret_cast<double const*>(db + P.o_aux);
    RowJob const* d_rj = reinterpret_cast<RowJob const*>(tabs.as<char>());
    ColJob const* d_cj = reinterpret_cast<ColJob const*>(tabs.as<char>() + (o_cj - o_rj));
    auto t1 = std::chrono::steady_clock::now();
    // 1. kept eigenvectors of the tridiagonal matrices (reversed rotations on unit vectors)
    {
        const size_t smem = sizeof(double) * (size_t)R * P.nmax;
        grow_smem_attr((void const*)tri_rot_kernel, smem);
        launch_pdl(ctx, (int)rjobs.size(), TRI_ROT_WARPS * 32, smem, tri_rot_kernel, 
            d_rj, d_jobs, scratch, reinterpret_cast<QlOut const*>(blob.as<char>()), blob.as<char>(), R);
        ITG_CHECK_CUDA(cudaGetLastError());
        ctx.kernel_launches++;
    }
    if (timing) ctx.sync();
    auto t1b = std::chrono::steady_clock::now();
    // 2. back to the block's basis: the Householder reflectors applied to each kept column
    {
        const size_t smem = sizeof(double) * TRI_APPLYQ_WARPS * (size_t)P.nmax;
        grow_smem_attr((void const*)tri_applyq_kernel, smem);
        launch_pdl(ctx, (int)cjobs.size(), TRI_APPLYQ_WARPS * 32, smem, tri_applyq_kernel, d_cj, d_jobs, scratch, d_aux,
                                                                                        vout, P.nmax);
        ITG_CHECK_CUDA(cudaGetLastError());
        ctx.kernel_launches++;
    }
    ctx.sync();   // the stage and the blob are released
    if (timing) {
        auto t2 = std::chrono::steady_clock::now();
        size_t kept = 0, tot = 0;
        for (int b = 0; b < nj; ++b) { kept += P.jobs[b].keep; tot += items[b].n; }
        std::fprintf(stderr, "itg tri finish (ms): host %.3f device %.3f (rotations %.3f); kept %zu of %zu\n",
                     std::chrono::duration<double, std::milli>(t1 - t0).count(),
                     std::chrono::duration<double, std::milli>(t2 - t1).count(),
                     std::chrono::duration<double, std::milli>(t1b - t1).count(), kept, tot);
    }
}

}  // namespace itg
