// Batched singular value decomposition of QN blocks (FP64), for the SVD route
// of the bond split: svdImpl's QN branch, itensor/svd.cc:169-222, which calls
// SVDRef per block (itensor/tensor/algs.cc:586-631).
//
// One-sided Jacobi (Hestenes): the columns of X (rows >= cols) are rotated in
// pairs until mutually orthogonal; then sigma_j = |x_j|, U_j = x_j / sigma_j
// and V accumulates the rotations, so X = U diag(sigma) V^T. One CTA per
// block, one warp per column pair of a round (tournament order), the three dot
// products of a pair reduced with shuffles. A pair is skipped when
// |x_p . x_q| <= max(1e-15 |x_p| |x_q|, 1e-17 |X|_F^2): the absolute floor
// stops tiny columns from chasing the rounding noise of large ones, and a
// coupling that small moves no squared singular value by more than 1e-17 |X|_F^2.
// The block is converged when a sweep skips every pair; sweeps are capped, and
// a capped block still counts as converged when its largest coupling in the
// last sweep is <= 1e-13 |X|_F^2.
#include "ops.h"
#include <algorithm>
#include <cstring>

namespace itg {

constexpr int SVD_MAX_SWEEPS = 60;
constexpr int SVD_THREADS = 256;

__global__ void __launch_bounds__(SVD_THREADS) jacobi_svd_kernel(SvdItem const* __restrict__ items,
                                                                 double const* __restrict__ src,
                                                                 double* __restrict__ uout, double* __restrict__ sout,
                                                                 double* __restrict__ vout, double* __restrict__ scratch,
                                                                 int* __restrict__ status) {
    extern __shared__ int svd_slot[];
    __shared__ int rotated;
    __shared__ double red[32];
    const SvdItem it = items[blockIdx.x];
    const int m = it.rows, n = it.cols;           // X is m x n with m >= n (column-major)
    const int np = n + (n & 1), half = np / 2;
    double* X = scratch + it.s_off;               // m x n working copy
    double* V = X + (size_t)m * n;                // n x n
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nw = blockDim.x >> 5;
    // load (optionally transposed), V = I, Frobenius norm^2
    double loc = 0;
    for (int e = tid; e < m * n; e += blockDim.x) {
        const int i = e % m, j = e / m;
        const double x = it.transpose ? src[it.a_off + j + (int64_t)i * it.ld] : src[it.a_off + i + (int64_t)j * it.ld];
        X[e] = x;
        loc = fma(x, x, loc);
    }
    for (int e = tid; e < n * n; e += blockDim.x) V[e] = (e % n == e / n) ? 1.0 : 0.0;
    for (int o = 16; o; o >>= 1) loc += __shfl_down_sync(0xffffffffu, loc, o);
    if (lane == 0) red[warp] = loc;
    for (int i = tid; i < np; i += blockDim.x) svd_slot[i] = i;
    __syncthreads();
    double norm2 = 0;
    for (int w = 0; w < nw; ++w) norm2 += red[w];
    const double abs_floor = 1e-17 * norm2;
    __shared__ unsigned long long maxg_bits;  // max |g| of the sweep (non-negative doubles order as integers)
    bool converged = (n <= 1);
    int sweeps = 0;
    while (!converged && sweeps < SVD_MAX_SWEEPS) {
        if (tid == 0) { rotated = 0; maxg_bits = 0ull; }
        __syncthreads();
        for (int round = 0; round < np - 1; ++round) {
            for (int k = warp; k < half; k += nw) {
                int p = svd_slot[k], q = svd_slot[np - 1 - k];
                if (p > q) { int t = p; p = q; q = t; }
                if (q >= n) continue;  // dummy slot
                double* xp = X + (size_t)p * m;
                double* xq = X + (size_t)q * m;
                double a = 0, b = 0, g = 0;
                for (int i = lane; i < m; i += 32) {
                    const double u = xp[i], w = xq[i];
                    a = fma(u, u, a);
                    b = fma(w, w, b);
                    g = fma(u, w, g);
                }
                for (int o = 16; o; o >>= 1) {
                    a += __shfl_xor_sync(0xffffffffu, a, o);
                    b += __shfl_xor_sync(0xffffffffu, b, o);
                    g += __shfl_xor_sync(0xffffffffu, g, o);
                }
                if (fabs(g) <= fmax(1e-15 * sqrt(a * b), abs_floor)) continue;
                if (lane == 0) atomicMax(&maxg_bits, (unsigned long long)__double_as_longlong(fabs(g)));
                const double zeta = (b - a) / (2.0 * g);
                const double t = (zeta >= 0 ? 1.0 : -1.0) / (fabs(zeta) + sqrt(1.0 + zeta * zeta));
                const double c = 1.0 / sqrt(1.0 + t * t), s = c * t;
                for (int i = lane; i < m; i += 32) {
                    const double u = xp[i], w = xq[i];
                    xp[i] = c * u - s * w;
                    xq[i] = s * u + c * w;
                }
                double* vp = V + (size_t)p * n;
                double* vq = V + (size_t)q * n;
                for (int i = lane; i < n; i += 32) {
                    const double u = vp[i], w = vq[i];
                    vp[i] = c * u - s * w;
                    vq[i] = s * u + c * w;
                }
                if (lane == 0) rotated = 1;
            }
            __syncthreads();
            if (tid == 0 && np > 2) {
                const int last = svd_slot[np - 1];
                for (int i = np - 1; i > 1; --i) svd_slot[i] = svd_slot[i - 1];
                svd_slot[1] = last;
            }
            __syncthreads();
        }
        ++sweeps;
        converged = (rotated == 0);
        const double maxg = __longlong_as_double((long long)maxg_bits);
        __syncthreads();
        if (!converged && sweeps == SVD_MAX_SWEEPS && maxg <= 1e-13 * norm2) converged = true;
    }
    // singular values = column norms; order descending (ties by column)
    double* sig = V + (size_t)n * n;  // n scratch doubles after V
    for (int j = warp; j < n; j += nw) {
        double a = 0;
        const double* xj = X + (size_t)j * m;
        for (int i = lane; i < m; i += 32) a = fma(xj[i], xj[i], a);
        for (int o = 16; o; o >>= 1) a += __shfl_xor_sync(0xffffffffu, a, o);
        if (lane == 0) sig[j] = sqrt(a);
    }
    __syncthreads();
    for (int j = tid; j < n; j += blockDim.x) {
        const double sj = sig[j];
        int r = 0;
        for (int k = 0; k < n; ++k) r += (sig[k] > sj) || (sig[k] == sj && k < j);
        svd_slot[j] = r;
        sout[it.s_out + r] = sj;
    }
    __syncthreads();
    // left vectors (normalised columns of X) and right vectors (columns of V), in rank order
    for (int e = tid; e < m * n; e += blockDim.x) {
        const int i = e % m, j = e / m;
        const double sj = sig[j];
        uout[it.u_off + (size_t)svd_slot[j] * m + i] = sj > 0 ? X[e] / sj : 0.0;
    }
    for (int e = tid; e < n * n; e += blockDim.x) {
        const int i = e % n, j = e / n;
        vout[it.v_off + (size_t)svd_slot[j] * n + i] = V[e];
    }
    if (tid == 0) status[blockIdx.x] = converged ? 0 : 1;
}

int batched_svd(Ctx& ctx, std::vector<SvdItem> const& items, double const* src, double* uout, double* sout,
                double* vout, double* scratch) {
    if (items.empty()) return 0;
    int nmax = 0;
    for (auto const& it : items) nmax = std::max(nmax, it.cols);
    const size_t smem = sizeof(int) * (nmax + 2);
    if (smem > 48 * 1024)
        ITG_CHECK_CUDA(cudaFuncSetAttribute(jacobi_svd_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    const size_t o_stat = ((sizeof(SvdItem) * items.size() + 15) / 16) * 16;
    DevBuf buf(o_stat + sizeof(int) * items.size(), ctx.stream);
    ctx.ensure_stage(sizeof(SvdItem) * items.size());
    std::memcpy(ctx.stage, items.data(), sizeof(SvdItem) * items.size());
    ITG_CHECK_CUDA(cudaMemcpyAsync(buf.p, ctx.stage, sizeof(SvdItem) * items.size(), cudaMemcpyHostToDevice, ctx.stream));
    int* d_stat = reinterpret_cast<int*>(buf.as<char>() + o_stat);
    jacobi_svd_kernel<<<(int)items.size(), SVD_THREADS, smem, ctx.stream>>>(buf.as<SvdItem>(), src, uout, sout, vout,
                                                                           scratch, d_stat);
    ITG_CHECK_CUDA(cudaGetLastError());
    ctx.kernel_launches++;
    std::vector<int> st(items.size());
    ctx.d2h(st.data(), d_stat, sizeof(int) * items.size());
    int bad = 0;
    for (int s : st) bad += s;
    return bad;
}

}  // namespace itg
