// Memory-bound helpers of the DMRG hot path on sm_103a:
//   * vector kernels for Davidson (axpy/axpby/scale, batched dot products, norm)
//     -- PlusEQ / dnrm2 / ddot at itensor/itdata/qdense.cc:303-311,409-417,506-664;
//   * block gather with separable offset tables -- the permute-copies of
//     QCombiner combine/uncombine (itensor/itdata/qcombiner.cc:125-300) and of
//     transform (itensor/tensor/ten_impl.h:107-160);
//   * batched symmetric eigensolver (cyclic Jacobi, FP64, one CTA per QN block)
//     -- blockwise dsyev of diag_hermitian (itensor/hermitian.cc:180-260,
//     itensor/tensor/algs.cc:34-41).
#include "ops.h"
#include <cmath>
#include <algorithm>
#include <cstring>

namespace itg {

// ------------------------------------------------------------------ vector kernels
__global__ void fill_kernel(double* x, int64_t n, double v) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) x[i] = v;
}
__global__ void scale_kernel(double* x, int64_t n, double a) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) x[i] *= a;
}
// y = a x + b y. With b == 0, y is not read: it may be fresh pool memory whose
// bits (old digit panels, integers) need not be finite doubles, and 0 * NaN = NaN.
__global__ void axpby_kernel(double* y, double const* x, int64_t n, double a, double b) {
    if (b == 0.0) {
        for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
            y[i] = a * x[i];
        return;
    }
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        y[i] = fma(a, x[i], b * y[i]);
}
__global__ void axpy_kernel(double* y, double const* x, int64_t n, double a) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        y[i] = fma(a, x[i], y[i]);
}

static int grid_for(Ctx& ctx, int64_t n) {
    int64_t g = (n + 255) / 256;
    return (int)std::max<int64_t>(1, std::min<int64_t>(g, (int64_t)ctx.sm_count * 8));
}

void launch_fill(Ctx& ctx, double* x, int64_t n, double v) {
    if (n <= 0) return;
    fill_kernel<<<grid_for(ctx, n), 256, 0, ctx.stream>>>(x, n, v);
    ITG_CHECK_CUDA(cudaGetLastError());
    ctx.kernel_launches++;
}
void launch_scale(Ctx& ctx, double* x, int64_t n, double a) {
    if (n <= 0) return;
    scale_kernel<<<grid_for(ctx, n), 256, 0, ctx.stream>>>(x, n, a);
    ITG_CHECK_CUDA(cudaGetLastError());
    ctx.kernel_launches++;
}
void launch_axpy(Ctx& ctx, double* y, double const* x, int64_t n, double a) {
    if (n <= 0) return;
    axpy_kernel<<<grid_for(ctx, n), 256, 0, ctx.stream>>>(y, x, n, a);
    ITG_CHECK_CUDA(cudaGetLastError());
    ctx.kernel_launches++;
}
void launch_axpby(Ctx& ctx, double* y, double const* x, int64_t n, double a, double b) {
    if (n <= 0) return;
    axpby_kernel<<<grid_for(ctx, n), 256, 0, ctx.stream>>>(y, x, n, a, b);
    ITG_CHECK_CUDA(cudaGetLastError());
    ctx.kernel_launches++;
}

// Dot products of x with nv vectors, two-level: per-CTA partial sums in a
// fixed order, then one CTA reduces the partials (deterministic result).
constexpr int DOT_CTAS = 256;
__global__ void dots_partial_kernel(double const* const* V, int nv, double const* x, int64_t n, double* part) {
    __shared__ double sh[32];
    for (int v = 0; v < nv; ++v) {
        double const* a = V[v];
        double s = 0;
        for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
            s = fma(a[i], x[i], s);
        for (int o = 16; o; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
        if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = s;
        __syncthreads();
        if (threadIdx.x < 32) {
            double t = threadIdx.x < (blockDim.x >> 5) ? sh[threadIdx.x] : 0.0;
            for (int o = 16; o; o >>= 1) t += __shfl_down_sync(0xffffffffu, t, o);
            if (threadIdx.x == 0) part[(size_t)v * gridDim.x + blockIdx.x] = t;
        }
        __syncthreads();
    }
}
__global__ void dots_final_kernel(double const* part, int nparts, int nv, double* out) {
    __shared__ double sh[32];
    for (int v = 0; v < nv; ++v) {
        double s = 0;
        for (int i = threadIdx.x; i < nparts; i += blockDim.x) s += part[(size_t)v * nparts + i];
        for (int o = 16; o; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
        if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = s;
        __syncthreads();
        if (threadIdx.x < 32) {
            double t = threadIdx.x < (blockDim.x >> 5) ? sh[threadIdx.x] : 0.0;
            for (int o = 16; o; o >>= 1) t += __shfl_down_sync(0xffffffffu, t, o);
            if (threadIdx.x == 0) out[v] = t;
        }
        __syncthreads();
    }
}

void dots(Ctx& ctx, double const* const* V, int nv, double const* x, int64_t n, double* out) {
    if (nv <= 0) return;
    // pointer list + partials + results in one pool allocation; result via mapped memory
    size_t o_ptr = 0, o_part = ((sizeof(void*) * nv + 15) / 16) * 16;
    size_t bytes = o_part + sizeof(double) * (size_t)DOT_CTAS * nv;
    DevBuf scratch(bytes, ctx.stream);
    ctx.ensure_stage(sizeof(void*) * nv);
    std::memcpy(ctx.stage, V, sizeof(void*) * nv);
    ITG_CHECK_CUDA(cudaMemcpyAsync(scratch.as<char>() + o_ptr, ctx.stage, sizeof(void*) * nv, cudaMemcpyHostToDevice, ctx.stream));
    ctx.ensure_pin(sizeof(double) * nv);
    int nb = (int)std::max<int64_t>(1, std::min<int64_t>(DOT_CTAS, (n + 255) / 256));
    dots_partial_kernel<<<nb, 256, 0, ctx.stream>>>(reinterpret_cast<double const* const*>(scratch.as<char>() + o_ptr), nv, x, n,
                                                    reinterpret_cast<double*>(scratch.as<char>() + o_part));
    dots_final_kernel<<<1, 256, 0, ctx.stream>>>(reinterpret_cast<double const*>(scratch.as<char>() + o_part), nb, nv,
                                                 static_cast<double*>(ctx.pin_dev));
    ITG_CHECK_CUDA(cudaGetLastError());
    ctx.kernel_launches += 2;
    ctx.sync();
    std::memcpy(out, ctx.pin, sizeof(double) * nv);
}

double dot(Ctx& ctx, double const* a, double const* b, int64_t n) {
    double r = 0;
    double const* V[1] = {a};
    dots(ctx, V, 1, b, n, &r);
    return r;
}

double norm(Ctx& ctx, double const* a, int64_t n) {
    double r = dot(ctx, a, a, n);
    return std::sqrt(std::max(r, 0.0));
}

// ------------------------------------------------------------------ gather
// dst[doff + d1[i] + d2[j]] = src[soff + s1[i] + s2[j]], i < n1 (fastest), j < n2
__global__ void gather_kernel(GatherItem const* __restrict__ items, int32_t const* __restrict__ tab,
                              double const* __restrict__ src, double* __restrict__ dst) {
    const GatherItem it = items[blockIdx.x];
    const int64_t n = (int64_t)it.n1 * it.n2;
    for (int64_t e = threadIdx.x; e < n; e += blockDim.x) {
        int i = (int)(e % it.n1), j = (int)(e / it.n1);
        dst[it.doff + tab[it.td1 + i] + tab[it.td2 + j]] = src[it.soff + tab[it.ts1 + i] + tab[it.ts2 + j]];
    }
}

void GatherPlan::upload(Ctx& ctx) {
    size_t o_items = 0, o_tab = ((sizeof(GatherItem) * std::max<size_t>(1, items.size()) + 15) / 16) * 16;
    size_t bytes = o_tab + sizeof(int32_t) * std::max<size_t>(1, tab.size());
    ctx.ensure_stage(bytes);
    char* st = static_cast<char*>(ctx.stage);
    if (!items.empty()) std::memcpy(st + o_items, items.data(), sizeof(GatherItem) * items.size());
    if (!tab.empty()) std::memcpy(st + o_tab, tab.data(), sizeof(int32_t) * tab.size());
    dev = dev_alloc(bytes, ctx.stream);
    ITG_CHECK_CUDA(cudaMemcpyAsync(dev->as<char>(), st, bytes, cudaMemcpyHostToDevice, ctx.stream));
    ctx.sync();
    d_items = reinterpret_cast<GatherItem*>(dev->as<char>() + o_items);
    d_tab = reinterpret_cast<int32_t*>(dev->as<char>() + o_tab);
    nitems = (int)items.size();
}

void launch_gather(Ctx& ctx, GatherPlan const& g, double const* src, double* dst) {
    if (g.nitems == 0) return;
    gather_kernel<<<g.nitems, 256, 0, ctx.stream>>>(g.d_items, g.d_tab, src, dst);
    ITG_CHECK_CUDA(cudaGetLastError());
    ctx.kernel_launches++;
}

// ------------------------------------------------------------------ batched Jacobi eigensolver
// Cyclic two-sided Jacobi with tournament ordering: each round applies n/2
// disjoint rotations in parallel (columns, then rows), n-1 rounds per sweep.
// Rotation (c,s) from the symmetric Schur decomposition of the 2x2 pivot
// (Golub & Van Loan, Matrix Computations, sec. 8.5). A rotation is skipped
// when |a_pq| <= max(1e-15 sqrt(|a_pp a_qq|), 1e-20 ||A||_F) (the relative
// test of Demmel & Veselic plus an absolute floor far below any truncation
// threshold); the matrix is converged when a sweep skips every pair. The sweep
// loop is capped (no unbounded wait); a capped matrix still counts as
// converged when its largest off-diagonal entry is below 1e-13 ||A||_F.
constexpr int EIG_MAX_SWEEPS = 60;
constexpr int EIG_THREADS = 256;

__global__ void __launch_bounds__(EIG_THREADS) jacobi_kernel(EigItem const* __restrict__ items, double const* __restrict__ src,
                                                             double* __restrict__ vout, double* __restrict__ wout,
                                                             double* __restrict__ scratch, int* __restrict__ status) {
    extern __shared__ unsigned char eig_smem[];
    const EigItem it = items[blockIdx.x];
    const int n = it.n;
    const int np = n + (n & 1);  // even number of slots, slot n is a dummy when n is odd
    const int half = np / 2;
    int* slot = reinterpret_cast<int*>(eig_smem);           // np
    double* cs = reinterpret_cast<double*>(eig_smem + ((np * sizeof(int) + 15) / 16) * 16);  // 2*half
    int* pq = reinterpret_cast<int*>(cs + 2 * half);        // 2*half
    __shared__ int rotated;
    __shared__ double red[32];
    double* A = scratch + it.s_off;
    double* V = A + (size_t)n * n;
    const int tid = threadIdx.x;
    // load A, V = I, Frobenius norm
    double loc = 0;
    for (int e = tid; e < n * n; e += blockDim.x) {
        double x = src[it.a_off + e];
        A[e] = x;
        V[e] = (e % n == e / n) ? 1.0 : 0.0;
        loc = fma(x, x, loc);
    }
    for (int o = 16; o; o >>= 1) loc += __shfl_down_sync(0xffffffffu, loc, o);
    if ((tid & 31) == 0) red[tid >> 5] = loc;
    __syncthreads();
    if (tid == 0) {
        double s = 0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) s += red[w];
        red[0] = sqrt(s);
    }
    for (int i = tid; i < np; i += blockDim.x) slot[i] = i;
    __syncthreads();
    const double normA = red[0];
    const double abs_floor = 1e-20 * normA;
    int sweeps = 0;
    bool converged = (n <= 1);
    while (!converged && sweeps < EIG_MAX_SWEEPS) {
        if (tid == 0) rotated = 0;
        __syncthreads();
        for (int round = 0; round < np - 1; ++round) {
            for (int k = tid; k < half; k += blockDim.x) {
                int p = slot[k], q = slot[np - 1 - k];
                if (p > q) { int t = p; p = q; q = t; }
                double c = 1.0, s = 0.0;
                if (q < n) {
                    double apq = A[(size_t)q * n + p];
                    double app = A[(size_t)p * n + p], aqq = A[(size_t)q * n + q];
                    if (fabs(apq) > fmax(1e-15 * sqrt(fabs(app * aqq)), abs_floor)) {
                        double tau = (aqq - app) / (2.0 * apq);
                        double t = (tau >= 0 ? 1.0 : -1.0) / (fabs(tau) + sqrt(1.0 + tau * tau));
                        c = 1.0 / sqrt(1.0 + t * t);
                        s = t * c;
                        rotated = 1;
                    }
                }
                cs[2 * k] = c; cs[2 * k + 1] = s;
                pq[2 * k] = p; pq[2 * k + 1] = q;
            }
            __syncthreads();
            // columns p, q of A and V
            for (int e = tid; e < half * n; e += blockDim.x) {
                int k = e / n, i = e % n;
                double s = cs[2 * k + 1];
                if (s == 0.0) continue;
                double c = cs[2 * k];
                int p = pq[2 * k], q = pq[2 * k + 1];
                double ap = A[(size_t)p * n + i], aq = A[(size_t)q * n + i];
                A[(size_t)p * n + i] = c * ap - s * aq;
                A[(size_t)q * n + i] = s * ap + c * aq;
                double vp = V[(size_t)p * n + i], vq = V[(size_t)q * n + i];
                V[(size_t)p * n + i] = c * vp - s * vq;
                V[(size_t)q * n + i] = s * vp + c * vq;
            }
            __syncthreads();
            // rows p, q of A
            for (int e = tid; e < half * n; e += blockDim.x) {
                int k = e / n, j = e % n;
                double s = cs[2 * k + 1];
                if (s == 0.0) continue;
                double c = cs[2 * k];
                int p = pq[2 * k], q = pq[2 * k + 1];
                double ap = A[(size_t)j * n + p], aq = A[(size_t)j * n + q];
                A[(size_t)j * n + p] = c * ap - s * aq;
                A[(size_t)j * n + q] = s * ap + c * aq;
            }
            __syncthreads();
            // tournament rotation of slots 1..np-1
            if (tid == 0 && np > 2) {
                int last = slot[np - 1];
                for (int i = np - 1; i > 1; --i) slot[i] = slot[i - 1];
                slot[1] = last;
            }
            __syncthreads();
        }
        ++sweeps;
        converged = (rotated == 0);
        __syncthreads();
    }
    // eigenvalues descending (ties by position), eigenvector columns follow
    for (int i = tid; i < n; i += blockDim.x) {
        double di = A[(size_t)i * n + i];
        int r = 0;
        for (int j = 0; j < n; ++j) {
            double dj = A[(size_t)j * n + j];
            r += (dj > di) || (dj == di && j < i);
        }
        wout[it.w_off + r] = di;
        slot[i] = r;  // slot[] reused as the rank table (np >= n)
    }
    __syncthreads();
    for (int e = tid; e < n * n; e += blockDim.x) {
        int col = e / n, row = e % n;
        vout[it.v_off + (size_t)slot[col] * n + row] = V[e];
    }
    if (!converged) {
        // sweep cap reached: accept when the remaining coupling is negligible
        double mx = 0;
        for (int e = tid; e < n * n; e += blockDim.x)
            if (e % n != e / n) mx = fmax(mx, fabs(A[e]));
        for (int o = 16; o; o >>= 1) mx = fmax(mx, __shfl_down_sync(0xffffffffu, mx, o));
        __syncthreads();
        if ((tid & 31) == 0) red[tid >> 5] = mx;
        __syncthreads();
        if (tid == 0) {
            double m = 0;
            for (int w = 0; w < (int)(blockDim.x >> 5); ++w) m = fmax(m, red[w]);
            status[blockIdx.x] = (m <= 1e-13 * normA) ? 0 : 1;
        }
    } else if (tid == 0) {
        status[blockIdx.x] = 0;
    }
}

int batched_eigh(Ctx& ctx, std::vector<EigItem> const& items, double const* src, double* vout, double* wout,
                 double* scratch) {
    if (items.empty()) return 0;
    int nmax = 0;
    for (auto const& it : items) nmax = std::max(nmax, it.n);
    const int np = nmax + (nmax & 1);
    size_t smem = ((np * sizeof(int) + 15) / 16) * 16 + sizeof(double) * np + sizeof(int) * np + 64;
    if (smem > 48 * 1024) {
        ITG_CHECK_CUDA(cudaFuncSetAttribute(jacobi_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    }
    size_t o_items = 0, o_stat = ((sizeof(EigItem) * items.size() + 15) / 16) * 16;
    DevBuf buf(o_stat + sizeof(int) * items.size(), ctx.stream);
    ctx.ensure_stage(sizeof(EigItem) * items.size());
    std::memcpy(ctx.stage, items.data(), sizeof(EigItem) * items.size());
    ITG_CHECK_CUDA(cudaMemcpyAsync(buf.as<char>() + o_items, ctx.stage, sizeof(EigItem) * items.size(),
                                   cudaMemcpyHostToDevice, ctx.stream));
    int* d_stat = reinterpret_cast<int*>(buf.as<char>() + o_stat);
    jacobi_kernel<<<(int)items.size(), EIG_THREADS, smem, ctx.stream>>>(reinterpret_cast<EigItem*>(buf.as<char>() + o_items), src,
                                                                         vout, wout, scratch, d_stat);
    ITG_CHECK_CUDA(cudaGetLastError());
    ctx.kernel_launches++;
    std::vector<int> st(items.size());
    ctx.d2h(st.data(), d_stat, sizeof(int) * items.size());
    int bad = 0;
    for (int s : st) bad += s;
    return bad;
}


}  // namespace itg

namespace itg {
// Deterministic pseudo-random fill in [0,1) (splitmix64 of the element index
// and a seed); used when Davidson must replace a dependent vector.
__global__ void random_kernel(double* x, int64_t n, uint64_t seed) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        uint64_t z = seed + 0x9e3779b97f4a7c15ull * (uint64_t)(i + 1);
        z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
        z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
        z ^= z >> 31;
        x[i] = (double)(z >> 11) * (1.0 / 9007199254740992.0);
    }
}
void launch_random(Ctx& ctx, double* x, int64_t n, uint64_t seed) {
    if (n <= 0) return;
    random_kernel<<<grid_for(ctx, n), 256, 0, ctx.stream>>>(x, n, seed);
    ITG_CHECK_CUDA(cudaGetLastError());
    ctx.kernel_launches++;
}
}  // namespace itg
