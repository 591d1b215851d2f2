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
//   2. tri_formq_kernel: Q = H_0 H_1 ... H_{n-3} formed column by column (one warp
//      per column, columns independent, spread over the whole GPU).
//   3. the implicit QL recurrence on (d, e) (tridiag_ql.cpp): a chain of
//      dependent scalar FP64 operations, ~n^2 rotations per block with a square
//      root and two divisions each. On this part an SM issues ~2 FP64 FMAs per
//      clock, so one thread's dependent FP64 chain advances by one operation
//      every few tens of cycles (measured: ~1.7 us per rotation on the SM); the
//      host core runs it in nanoseconds per operation. It only records the plane
//      rotations, while the device forms Q;
//   4. tri_rot_kernel: the recorded rotations applied to the rows of Q (rows
//      transform independently: a tile of rows per CTA, in shared memory; the
//      CTA's eight warps apply rotations of eight sweeps at once, on a
//      lockstep schedule from the host that keeps them on disjoint columns);
//   5. tri_out_kernel: eigenvalues sorted descending, eigenvector columns moved
//      with them.
// The FP64 work is ~n^3 FMA for the reduction, ~2n^3/3 for Q and ~n^2 rotations
// x n rows for the accumulation, against ~4n^3 per Jacobi sweep; every O(n^3)
// stage spreads one block over many SMs.
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
#include <thread>

namespace cg = cooperative_groups;

namespace itg {

namespace {
constexpr int TRI_THREADS = 256;
constexpr int TRI_FORMQ_WARPS = 4;
constexpr int TRI_ROT_WARPS = 8;         // sweeps applied at once to one row tile
constexpr int TRI_ROT_WINDOW = 4;        // lockstep steps between barriers
constexpr size_t TRI_SMEM_LIMIT = 200 * 1024;

struct TriJob {
    int64_t a_off;     // input block (n x n, column-major) in src
    int64_t v_off;     // eigenvectors (columns, eigenvalues descending) in vout
    int64_t w_off;     // eigenvalues (descending) in wout
    int64_t s_off;     // 2 n^2 doubles: reduced matrix + reflectors, then Q
    int64_t aux_off;   // tri_aux_doubles(n) doubles in aux: d, e, tau, v, p, partial sums
    int32_t n, pad;
};
struct ColJob { int32_t job, c0; };
struct RowJob { int32_t job, r0; };

__host__ __device__ inline int64_t tri_aux_doubles(int n) { return 5 * (int64_t)n + 16; }

__device__ __forceinline__ double warp_sum(double v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
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
    double ss = 0.0;
    for (int i = k + 2 + threadIdx.x; i < n; i += blockDim.x) ss = fma(col[i], col[i], ss);
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

__global__ void __launch_bounds__(TRI_THREADS) tri_reduce_kernel(TriJob const* __restrict__ jobs,
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
            for (int j = j0 + warp * C; j < n; j += nw * C) {
                double const* col = A + (size_t)j * n;
                double acc = 0.0;
                for (int i = k + 1 + lane; i < n; i += 32) acc = fma(col[i], vs[i], acc);
                const double pj = tk * warp_sum(acc);
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

// Q e_j = H_0 (H_1 (... H_{n-3} e_j)); H_k acts on rows k+1..n-1, so only
// reflectors k < j touch column j.
__global__ void __launch_bounds__(TRI_FORMQ_WARPS * 32) tri_formq_kernel(ColJob const* __restrict__ cjobs,
                                                                         TriJob const* __restrict__ jobs,
                                                                         double* __restrict__ scratch,
                                                                         double const* __restrict__ aux, int nmax) {
    extern __shared__ double sm[];
    const ColJob cj = cjobs[blockIdx.x];
    const TriJob jb = jobs[cj.job];
    const int n = jb.n;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int j = cj.c0 + warp;
    if (j >= n) return;
    double const* R = scratch + jb.s_off;               // reflectors below the subdiagonal
    double* Q = scratch + jb.s_off + (size_t)n * n;
    double const* tau = aux + jb.aux_off + 2 * (size_t)n;
    double* y = sm + (size_t)warp * nmax;
    for (int i = lane; i < n; i += 32) y[i] = (i == j) ? 1.0 : 0.0;
    __syncwarp();
    for (int k = min(j - 1, n - 3); k >= 0; --k) {
        const double t = tau[k];
        if (t == 0.0) continue;
        double const* v = R + (size_t)k * n;
        double acc = 0.0;
        for (int i = k + 2 + lane; i < n; i += 32) acc = fma(v[i], y[i], acc);
        const double dt = t * (warp_sum(acc) + y[k + 1]);
        __syncwarp();
        if (lane == 0) y[k + 1] -= dt;
        for (int i = k + 2 + lane; i < n; i += 32) y[i] = fma(-dt, v[i], y[i]);
        __syncwarp();
    }
    for (int i = lane; i < n; i += 32) Q[(size_t)j * n + i] = y[i];
}

// What the host's QL pass hands back per block (offsets into the uploaded blob).
struct QlOut {
    int64_t eig_off;   // eigenvalues (unsorted, doubles)
    int64_t hdr_off;   // sweeps (QlSweep = int4: l, m, rotation offset, 0)
    int64_t rot_off;   // rotations (QlRot = double2: c, s)
    int64_t sched_off; // TRI_ROT_WARPS + 1 entry offsets, then entries (QlStart = int2: start step, sweep)
    int32_t nsweeps, status, nsteps, pad;
};

// The recorded rotations applied to rows r0..r0+R-1 of Q (the tile lives in
// shared memory as tile[col * R + row], lane = row). The CTA's warps apply
// rotations of different QL sweeps at once, in lockstep: at step s a warp
// applies rotation s - S of its current sweep (started at step S), with a
// barrier every TRI_ROT_WINDOW steps; the host's schedule keeps the sweeps
// far enough apart that the warps of one window touch disjoint columns, so
// each column sees its rotations in the recorded order.
// Rotation i of a sweep: (z_i, z_{i+1}) <- (c z_i - s z_{i+1}, s z_i + c z_{i+1}).
__global__ void __launch_bounds__(TRI_ROT_WARPS * 32) tri_rot_kernel(RowJob const* __restrict__ rjobs,
                                                                     TriJob const* __restrict__ jobs,
                                                                     double* __restrict__ scratch,
                                                                     QlOut const* __restrict__ qo,
                                                                     char const* __restrict__ blob, int R) {
    extern __shared__ double tile[];
    const RowJob rj = rjobs[blockIdx.x];
    const TriJob jb = jobs[rj.job];
    const QlOut o = qo[rj.job];
    if (o.status != 0) return;
    const int n = jb.n;
    const int rows = min(R, n - rj.r0);
    double* Q = scratch + jb.s_off + (size_t)n * n;
    for (int idx = threadIdx.x; idx < n * R; idx += blockDim.x) {
        const int c = idx / R, r = idx % R;
        if (r < rows) tile[idx] = Q[(size_t)c * n + rj.r0 + r];
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
    // TRI_ROT_WINDOW steps between barriers: the schedule puts every rotation in
    // a later window than the other warps' earlier rotations on its columns
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
    for (int idx = threadIdx.x; idx < n * R; idx += blockDim.x) {
        const int c = idx / R, rr = idx % R;
        if (rr < rows) Q[(size_t)c * n + rj.r0 + rr] = tile[idx];
    }
}

// Eigenvalues descending (ties by position) with their columns; one warp per column.
__global__ void tri_out_kernel(ColJob const* __restrict__ cjobs, TriJob const* __restrict__ jobs,
                               double const* __restrict__ scratch, QlOut const* __restrict__ qo,
                               char const* __restrict__ blob, double* __restrict__ vout, double* __restrict__ wout) {
    const ColJob cj = cjobs[blockIdx.x];
    const TriJob jb = jobs[cj.job];
    const QlOut o = qo[cj.job];
    if (o.status != 0) return;
    const int n = jb.n;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int j = cj.c0 + warp;
    if (j >= n) return;
    double const* d = reinterpret_cast<double const*>(blob + o.eig_off);
    const double dj = d[j];
    int cnt = 0;
    for (int i = lane; i < n; i += 32) {
        const double di = d[i];
        cnt += (di > dj || (di == dj && i < j)) ? 1 : 0;
    }
    for (int o2 = 16; o2 > 0; o2 >>= 1) cnt += __shfl_xor_sync(0xffffffffu, cnt, o2);
    double const* Q = scratch + jb.s_off + (size_t)n * n;
    if (lane == 0) wout[jb.w_off + cnt] = dj;
    for (int i = lane; i < n; i += 32) vout[jb.v_off + (size_t)cnt * n + i] = Q[(size_t)j * n + i];
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

int tri_eigh(Ctx& ctx, std::vector<EigItem> const& items_in, double const* src, double* vout, double* wout,
             double* scratch) {
    if (items_in.empty()) return 0;
    // jobs ordered by cluster size (largest first), so that each size is one launch
    std::vector<EigItem> items(items_in);
    std::stable_sort(items.begin(), items.end(),
                     [](EigItem const& a, EigItem const& b) { return cluster_for(a.n) > cluster_for(b.n); });
    const int nj = (int)items.size();
    int nmax = 0;
    for (auto const& it : items) nmax = std::max(nmax, it.n);
    ITG_REQUIRE(nmax <= TRI_MAX_N, "tri_eigh: block larger than the tridiagonal path supports");
    // rows per tile of the rotation pass (lane = row): a full warp, fewer when
    // shared memory runs out
    int R = 32;
    if (char const* env = std::getenv("ITG_TRI_ROWS")) R = std::max(1, std::min(32, std::atoi(env)));
    while (R > 1 && sizeof(double) * (size_t)R * nmax > TRI_SMEM_LIMIT) R /= 2;
    std::vector<TriJob> jobs(nj);
    std::vector<ColJob> cjobs;
    std::vector<RowJob> rjobs;
    int64_t aux_tot = 0;
    for (int b = 0; b < nj; ++b) {
        auto const& it = items[b];
        TriJob& j = jobs[b];
        j = TriJob{};
        j.a_off = it.a_off;
        j.v_off = it.v_off;
        j.w_off = it.w_off;
        j.s_off = it.s_off;
        j.aux_off = aux_tot;
        aux_tot += tri_aux_doubles(it.n);
        j.n = it.n;
        for (int c0 = 0; c0 < it.n; c0 += TRI_FORMQ_WARPS) cjobs.push_back(ColJob{b, c0});
        for (int r0 = 0; r0 < it.n; r0 += R) rjobs.push_back(RowJob{b, r0});
    }
    auto a16 = [](size_t x) { return (x + 15) / 16 * 16; };
    const size_t o_jobs = 0, o_cj = a16(sizeof(TriJob) * nj), o_rj = a16(o_cj + sizeof(ColJob) * cjobs.size());
    const size_t up = a16(o_rj + sizeof(RowJob) * rjobs.size());
    const size_t o_aux = up;
    const size_t total = o_aux + sizeof(double) * aux_tot;
    DevBuf buf(total, ctx.stream);
    ctx.ensure_stage(up);
    char* st = static_cast<char*>(ctx.stage);
    std::memcpy(st + o_jobs, jobs.data(), sizeof(TriJob) * nj);
    std::memcpy(st + o_cj, cjobs.data(), sizeof(ColJob) * cjobs.size());
    std::memcpy(st + o_rj, rjobs.data(), sizeof(RowJob) * rjobs.size());
    char* db = buf.as<char>();
    ITG_CHECK_CUDA(cudaMemcpyAsync(db, st, up, cudaMemcpyHostToDevice, ctx.stream));
    TriJob const* d_jobs = reinterpret_cast<TriJob const*>(db + o_jobs);
    ColJob const* d_cj = reinterpret_cast<ColJob const*>(db + o_cj);
    RowJob const* d_rj = reinterpret_cast<RowJob const*>(db + o_rj);
    double* d_aux = reinterpret_cast<double*>(db + o_aux);

    // diagnostics (ITG_EIG_TIME): device time of the reduction and of Q, host
    // time of the QL pass, device time of the rotations and the output
    const bool timing = std::getenv("ITG_EIG_TIME") != nullptr;
    cudaEvent_t ev[5] = {};
    if (timing) {
        for (auto& x : ev) ITG_CHECK_CUDA(cudaEventCreate(&x));
        ITG_CHECK_CUDA(cudaEventRecord(ev[0], ctx.stream));
    }
    // 1. reduction: one launch per run of jobs with the same cluster size
    {
        const size_t smem = sizeof(double) * 2 * (size_t)nmax;
        if (smem > 48 * 1024)
            ITG_CHECK_CUDA(cudaFuncSetAttribute(tri_reduce_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                (int)smem));
        ITG_CHECK_CUDA(cudaFuncSetAttribute(tri_reduce_kernel, cudaFuncAttributeNonPortableClusterSizeAllowed, 1));
        // one launch per cluster size; the launches are independent, so they
        // run side by side on the context's side streams
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
    // (d, e) of every block to the host; Q is formed on the device meanwhile
    const size_t aux_bytes = sizeof(double) * aux_tot;
    ctx.ensure_pin(aux_bytes);
    ITG_CHECK_CUDA(cudaMemcpyAsync(ctx.pin, d_aux, aux_bytes, cudaMemcpyDeviceToHost, ctx.stream));
    cudaEvent_t de_ready;
    ITG_CHECK_CUDA(cudaEventCreateWithFlags(&de_ready, cudaEventDisableTiming));
    ITG_CHECK_CUDA(cudaEventRecord(de_ready, ctx.stream));
    if (timing) ITG_CHECK_CUDA(cudaEventRecord(ev[1], ctx.stream));
    {
        const size_t smem = sizeof(double) * TRI_FORMQ_WARPS * (size_t)nmax;
        if (smem > 48 * 1024)
            ITG_CHECK_CUDA(cudaFuncSetAttribute(tri_formq_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                (int)smem));
        tri_formq_kernel<<<(int)cjobs.size(), TRI_FORMQ_WARPS * 32, smem, ctx.stream>>>(d_cj, d_jobs, scratch, d_aux,
                                                                                       nmax);
        ITG_CHECK_CUDA(cudaGetLastError());
        ctx.kernel_launches++;
    }
    if (timing) ITG_CHECK_CUDA(cudaEventRecord(ev[2], ctx.stream));
    // 2. QL recurrences on the host, as soon as (d, e) arrived
    if (fiber_active()) fiber_wait_event(de_ready);
    else ITG_CHECK_CUDA(cudaEventSynchronize(de_ready));
    cudaEventDestroy(de_ready);
    auto th0 = std::chrono::steady_clock::now();
    std::vector<double> de(static_cast<double*>(ctx.pin), static_cast<double*>(ctx.pin) + aux_tot);
    std::vector<QlOut> qo(nj);
    std::vector<QlSweep> sweeps;
    std::vector<QlRot> rots;
    std::vector<std::vector<double>> eigs(nj);
    // blocks are independent: outside the solver pool (whose workers already
    // run one solve each) large passes use a few host threads
    std::vector<std::vector<QlSweep>> bsw(nj);
    std::vector<std::vector<QlRot>> brot(nj);
    std::vector<std::vector<int32_t>> bwoff(nj);
    std::vector<std::vector<QlStart>> bent(nj);
    std::vector<int> bst(nj, 0), bsteps(nj, 0);
    auto run_block = [&](int b) {
        const int n = items[b].n;
        double* d = de.data() + jobs[b].aux_off;
        bst[b] = tridiag_ql(n, d, d + n, bsw[b], brot[b]);
        eigs[b].assign(d, d + n);
        if (bst[b] == 0) bsteps[b] = ql_schedule(n, bsw[b], TRI_ROT_WARPS, TRI_ROT_WINDOW, bwoff[b], bent[b]);
        else bwoff[b].assign(TRI_ROT_WARPS + 1, 0);
    };
    double work = 0;
    for (auto const& it : items) work += (double)it.n * it.n;
    const int nthreads = (!fiber_active() && work > 2e5) ? std::min<int>(nj, 8) : 1;
    if (nthreads > 1) {
        std::atomic<int> next{0};
        std::vector<std::thread> pool;
        for (int t = 0; t < nthreads; ++t)
            pool.emplace_back([&] {
                for (int b; (b = next.fetch_add(1)) < nj;) run_block(b);
            });
        for (auto& t : pool) t.join();
    } else {
        for (int b = 0; b < nj; ++b) run_block(b);
    }
    int bad = 0;
    std::vector<int32_t> sched;   // per block: woff (padded to 8 bytes), then entries as int pairs
    for (int b = 0; b < nj; ++b) {
        qo[b].status = bst[b];
        bad += (bst[b] != 0);
        qo[b].nsweeps = (int32_t)bsw[b].size();
        qo[b].nsteps = bsteps[b];
        qo[b].pad = 0;
        qo[b].hdr_off = (int64_t)sweeps.size();   // element offsets for now
        qo[b].rot_off = (int64_t)rots.size();
        qo[b].sched_off = (int64_t)sched.size();
        sweeps.insert(sweeps.end(), bsw[b].begin(), bsw[b].end());
        rots.insert(rots.end(), brot[b].begin(), brot[b].end());
        sched.insert(sched.end(), bwoff[b].begin(), bwoff[b].end());
        for (int k = TRI_ROT_WARPS + 1; k < 2 * ((TRI_ROT_WARPS + 2) / 2); ++k) sched.push_back(0);
        for (auto const& x : bent[b]) {
            sched.push_back(x.step);
            sched.push_back(x.sweep);
        }
    }
    auto th1 = std::chrono::steady_clock::now();
    // blob: QlOut table | eigenvalues | sweeps | rotations
    int64_t eig_tot = 0;
    for (int b = 0; b < nj; ++b) eig_tot += items[b].n;
    const size_t b_qo = 0, b_eig = a16(sizeof(QlOut) * nj), b_hdr = a16(b_eig + sizeof(double) * eig_tot);
    const size_t b_rot = a16(b_hdr + sizeof(QlSweep) * sweeps.size());
    const size_t b_sched = a16(b_rot + sizeof(QlRot) * rots.size());
    const size_t blob_bytes = a16(b_sched + sizeof(int32_t) * sched.size());
    {
        int64_t eo = 0;
        for (int b = 0; b < nj; ++b) {
            qo[b].eig_off = (int64_t)(b_eig + sizeof(double) * eo);
            qo[b].hdr_off = (int64_t)(b_hdr + sizeof(QlSweep) * qo[b].hdr_off);
            qo[b].rot_off = (int64_t)(b_rot + sizeof(QlRot) * qo[b].rot_off);
            qo[b].sched_off = (int64_t)(b_sched + sizeof(int32_t) * qo[b].sched_off);
            eo += items[b].n;
        }
    }
    if (ctx.stage_bytes < blob_bytes) ctx.ensure_stage(blob_bytes + blob_bytes / 2);
    st = static_cast<char*>(ctx.stage);
    std::memcpy(st + b_qo, qo.data(), sizeof(QlOut) * nj);
    {
        int64_t eo = 0;
        for (int b = 0; b < nj; ++b) {
            std::memcpy(st + b_eig + sizeof(double) * eo, eigs[b].data(), sizeof(double) * items[b].n);
            eo += items[b].n;
        }
    }
    if (!sweeps.empty()) std::memcpy(st + b_hdr, sweeps.data(), sizeof(QlSweep) * sweeps.size());
    if (!rots.empty()) std::memcpy(st + b_rot, rots.data(), sizeof(QlRot) * rots.size());
    if (!sched.empty()) std::memcpy(st + b_sched, sched.data(), sizeof(int32_t) * sched.size());
    DevBuf blob(blob_bytes, ctx.stream);
    ITG_CHECK_CUDA(cudaMemcpyAsync(blob.p, st, blob_bytes, cudaMemcpyHostToDevice, ctx.stream));
    QlOut const* d_qo = reinterpret_cast<QlOut const*>(blob.as<char>() + b_qo);
    if (timing) ITG_CHECK_CUDA(cudaEventRecord(ev[3], ctx.stream));
    // 3. rotations applied to Q's rows
    {
        const size_t smem = sizeof(double) * (size_t)R * nmax;
        if (smem > 48 * 1024)
            ITG_CHECK_CUDA(cudaFuncSetAttribute(tri_rot_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        tri_rot_kernel<<<(int)rjobs.size(), TRI_ROT_WARPS * 32, smem, ctx.stream>>>(d_rj, d_jobs, scratch, d_qo,
                                                                                   blob.as<char>(), R);
        ITG_CHECK_CUDA(cudaGetLastError());
        ctx.kernel_launches++;
    }
    // 4. sorted output
    tri_out_kernel<<<(int)cjobs.size(), TRI_FORMQ_WARPS * 32, 0, ctx.stream>>>(d_cj, d_jobs, scratch, d_qo,
                                                                              blob.as<char>(), vout, wout);
    ITG_CHECK_CUDA(cudaGetLastError());
    ctx.kernel_launches++;
    if (timing) ITG_CHECK_CUDA(cudaEventRecord(ev[4], ctx.stream));
    // the staging buffer holds the blob until its copy has run
    ctx.sync();
    if (timing) {
        float ms[4];
        for (int i = 0; i < 4; ++i) ITG_CHECK_CUDA(cudaEventElapsedTime(&ms[i], ev[i], ev[i + 1]));
        std::fprintf(stderr,
                     "itg tri stages (ms): reduce %.3f formq %.3f wait+ql+upload %.3f rot+out %.3f; host ql %.3f; "
                     "rotations %zu; n:",
                     ms[0], ms[1], ms[2], ms[3], std::chrono::duration<double, std::milli>(th1 - th0).count(),
                     rots.size());
        for (int b = 0; b < nj; ++b) std::fprintf(stderr, " %d", items[b].n);
        std::fprintf(stderr, "\n");
        for (auto& x : ev) cudaEventDestroy(x);
    }
    return bad;
}

}  // namespace itg
