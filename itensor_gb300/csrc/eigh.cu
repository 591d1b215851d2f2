// Batched symmetric eigensolver for the QN blocks of the density matrix:
// blockwise dsyev of diag_hermitian (itensor/hermitian.cc:180-260,
// itensor/tensor/algs.cc:34-41), eigenvalues descending.
//
// Cyclic two-sided Jacobi (Golub & Van Loan, Matrix Computations, sec. 8.5),
// one CTA per block. A sweep is n-1 rounds of the round-robin ("circle")
// schedule: in round r slot n'-1 meets r and slot (r+k) meets (r-k) mod (n'-1),
// n' = n rounded up to even (slot n is a dummy when n is odd), so the n'/2
// rotations of a round touch disjoint index pairs. A round is two steps:
//   1. every pair's rotation (c, s, t) from its 2x2 pivot;
//   2. A <- J^T A J as independent 2x2 block updates R_k^T A[k,l] R_l over
//      block pairs k <= l (the mirror block written from the same values, so
//      A stays exactly symmetric and only half the blocks are computed), and
//      V <- V J on column pairs.
// FP64 issue slots (~2 FMA per clock per SM on this part) bound the kernel, so
// block pairs whose two rotations are both the identity are skipped.
// A rotation is skipped when |a_pq| <= max(1e-15 sqrt(|a_pp a_qq|), 1e-17 ||A||_F):
// the relative test of Demmel & Veselic, plus an absolute floor at which a
// rotation moves no eigenvalue by more than 1e-17 ||A||_F. The matrix is
// converged when a sweep skips every pair. Sweeps are capped; a capped matrix
// still counts as converged when its largest off-diagonal entry is below
// 1e-13 ||A||_F. The matrix and vectors live in shared memory when they fit
// (n up to ~118 for both, ~166 for the matrix alone), else in global scratch.
#include "ops.h"
#include <algorithm>
#include <cstring>

namespace itg {

constexpr int EIG_MAX_SWEEPS = 60;
constexpr int EIG_THREADS = 256;

struct JacobiShared {
    double* cst;   // 3 per pair: c, s, t
    int* pq;       // 2 per pair
    int* rotated;
};

// Pair k of round r of the circle schedule over np slots (np even).
__device__ __forceinline__ void round_pair(int r, int k, int np, int& p, int& q) {
    const int m = np - 1;
    int a, b;
    if (k == 0) {
        a = m;
        b = r;
    } else {
        a = r + k;
        if (a >= m) a -= m;
        b = r - k;
        if (b < 0) b += m;
    }
    p = min(a, b);
    q = max(a, b);
}

// Runs sweeps on the symmetric n x n matrix A (element (i,j) at A[j*lda+i]) and
// accumulates the rotations into V (n x n, element (i,j) at V[j*ldv+i]).
// Returns true when a sweep skipped every pair.
__device__ bool jacobi_run(double* A, int lda, double* V, int ldv, int n, int np, double abs_floor,
                           JacobiShared sh) {
    const int tid = threadIdx.x, nt = blockDim.x;
    const int half = np / 2;
    for (int sweep = 0; sweep < EIG_MAX_SWEEPS; ++sweep) {
        if (tid == 0) *sh.rotated = 0;
        __syncthreads();
        for (int r = 0; r < np - 1; ++r) {
            // 1. rotations of the round
            for (int k = tid; k < half; k += nt) {
                int p, q;
                round_pair(r, k, np, p, q);
                double c = 1.0, s = 0.0, t = 0.0;
                if (q < n) {
                    const double apq = A[(size_t)q * lda + p];
                    const double app = A[(size_t)p * lda + p], aqq = A[(size_t)q * lda + q];
                    if (fabs(apq) > fmax(1e-15 * sqrt(fabs(app * aqq)), abs_floor)) {
                        const double tau = (aqq - app) / (2.0 * apq);
                        t = (tau >= 0 ? 1.0 : -1.0) / (fabs(tau) + sqrt(1.0 + tau * tau));
                        c = 1.0 / sqrt(1.0 + t * t);
                        s = t * c;
                        *sh.rotated = 1;
                    }
                }
                sh.cst[3 * k] = c;
                sh.cst[3 * k + 1] = s;
                sh.cst[3 * k + 2] = t;
                sh.pq[2 * k] = p;
                sh.pq[2 * k + 1] = q;
            }
            __syncthreads();
            // 2a. A <- J^T A J, block pairs k <= l
            for (int e = tid; e < half * half; e += nt) {
                const int k = e % half, l = e / half;
                if (k > l) continue;
                const double sk = sh.cst[3 * k + 1], sl = sh.cst[3 * l + 1];
                if (sk == 0.0 && sl == 0.0) continue;
                const int p = sh.pq[2 * k], q = sh.pq[2 * k + 1];
                if (k == l) {
                    // pivot block: diagonalised exactly
                    const double t = sh.cst[3 * k + 2];
                    const double apq = A[(size_t)q * lda + p];
                    A[(size_t)p * lda + p] -= t * apq;
                    A[(size_t)q * lda + q] += t * apq;
                    A[(size_t)q * lda + p] = 0.0;
                    A[(size_t)p * lda + q] = 0.0;
                    continue;
                }
                const double ck = sh.cst[3 * k], cl = sh.cst[3 * l];
                const int u = sh.pq[2 * l], w = sh.pq[2 * l + 1];
                const bool qk = q < n, wl = w < n;  // dummy slots hold no row / column
                // block rows (p, q), columns (u, w); x = A(p,u), y = A(p,w), z = A(q,u), v = A(q,w)
                const double x = A[(size_t)u * lda + p];
                const double y = wl ? A[(size_t)w * lda + p] : 0.0;
                const double z = qk ? A[(size_t)u * lda + q] : 0.0;
                const double v = (qk && wl) ? A[(size_t)w * lda + q] : 0.0;
                // columns (u, w) by (cl, sl), then rows (p, q) by (ck, sk)
                const double x1 = cl * x - sl * y, y1 = sl * x + cl * y;
                const double z1 = cl * z - sl * v, v1 = sl * z + cl * v;
                const double x2 = ck * x1 - sk * z1, z2 = sk * x1 + ck * z1;
                const double y2 = ck * y1 - sk * v1, v2 = sk * y1 + ck * v1;
                A[(size_t)u * lda + p] = x2;
                A[(size_t)p * lda + u] = x2;
                if (wl) { A[(size_t)w * lda + p] = y2; A[(size_t)p * lda + w] = y2; }
                if (qk) { A[(size_t)u * lda + q] = z2; A[(size_t)q * lda + u] = z2; }
                if (qk && wl) { A[(size_t)w * lda + q] = v2; A[(size_t)q * lda + w] = v2; }
            }
            // 2b. V <- V J on column pairs (rows contiguous)
            for (int e = tid; e < half * n; e += nt) {
                const int i = e % n, k = e / n;
                const double s = sh.cst[3 * k + 1];
                if (s == 0.0) continue;
                const double c = sh.cst[3 * k];
                const int p = sh.pq[2 * k], q = sh.pq[2 * k + 1];
                const double a = V[(size_t)p * ldv + i], b = V[(size_t)q * ldv + i];
                V[(size_t)p * ldv + i] = c * a - s * b;
                V[(size_t)q * ldv + i] = s * a + c * b;
            }
            __syncthreads();
        }
        const bool done = (*sh.rotated == 0);
        __syncthreads();
        if (done) return true;
    }
    return false;
}

template <bool SMEM_A, bool SMEM_V>
__global__ void __launch_bounds__(EIG_THREADS) jacobi_kernel(EigItem const* __restrict__ items, double const* __restrict__ src,
                                                             double* __restrict__ vout, double* __restrict__ wout,
                                                             double* __restrict__ scratch, int* __restrict__ status) {
    extern __shared__ __align__(16) unsigned char eig_smem[];
    __shared__ int rotated;
    __shared__ double red[32];
    const EigItem it = items[blockIdx.x];
    const int n = it.n;
    const int np = n + (n & 1);
    const int half = np / 2;
    const int tid = threadIdx.x;
    // shared layout: cst (3 half doubles) | [A (np x (np+1))] | [V (n x n)] | pq (2 half ints) | rank (n ints)
    double* cst = reinterpret_cast<double*>(eig_smem);
    double* sp = cst + 3 * half;
    double* A;
    int lda;
    if (SMEM_A) { A = sp; lda = np + 1; sp += (size_t)np * lda; }
    else { A = scratch + it.s_off; lda = n; }
    double* V;
    if (SMEM_V) { V = sp; sp += (size_t)n * n; }
    else { V = scratch + it.s_off + (size_t)n * n; }
    int* pq = reinterpret_cast<int*>(sp);
    int* rank = pq + 2 * half;
    // load A, V = I, Frobenius norm
    double loc = 0;
    for (int e = tid; e < n * n; e += blockDim.x) {
        const int i = e % n, j = e / n;
        const double x = src[it.a_off + e];
        A[(size_t)j * lda + i] = x;
        V[e] = (i == j) ? 1.0 : 0.0;
        loc = fma(x, x, loc);
    }
    for (int o = 16; o; o >>= 1) loc += __shfl_down_sync(0xffffffffu, loc, o);
    if ((tid & 31) == 0) red[tid >> 5] = loc;
    __syncthreads();
    double norm2 = 0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) norm2 += red[w];
    const double normA = sqrt(norm2);
    __syncthreads();
    bool converged = (n <= 1);
    if (!converged) converged = jacobi_run(A, lda, V, n, n, np, 1e-17 * normA, JacobiShared{cst, pq, &rotated});
    // eigenvalues descending (ties by position); eigenvector columns follow
    for (int i = tid; i < n; i += blockDim.x) {
        const double di = A[(size_t)i * lda + i];
        int r = 0;
        for (int j = 0; j < n; ++j) {
            const double dj = A[(size_t)j * lda + j];
            r += (dj > di) || (dj == di && j < i);
        }
        wout[it.w_off + r] = di;
        rank[i] = r;
    }
    __syncthreads();
    for (int e = tid; e < n * n; e += blockDim.x) {
        const int col = e / n, row = e % n;
        vout[it.v_off + (size_t)rank[col] * n + row] = V[e];
    }
    if (!converged) {
        // sweep cap reached: accept when the remaining coupling is negligible
        double mx = 0;
        for (int e = tid; e < n * n; e += blockDim.x) {
            const int i = e % n, j = e / n;
            if (i != j) mx = fmax(mx, fabs(A[(size_t)j * lda + i]));
        }
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

namespace {
constexpr size_t EIG_SMEM_LIMIT = 227 * 1024;

size_t eig_smem_bytes(int n, bool sa, bool sv) {
    const int np = n + (n & 1), half = np / 2;
    size_t b = sizeof(double) * 3 * half;
    if (sa) b += sizeof(double) * (size_t)np * (np + 1);
    if (sv) b += sizeof(double) * (size_t)n * n;
    b += sizeof(int) * (2 * half + n);
    return b;
}

template <bool SA, bool SV>
void launch_eig(Ctx& ctx, int nitems, size_t smem, EigItem const* d_items, double const* src, double* vout, double* wout,
                double* scratch, int* d_stat) {
    if (smem > 48 * 1024)
        ITG_CHECK_CUDA(cudaFuncSetAttribute(jacobi_kernel<SA, SV>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    jacobi_kernel<SA, SV><<<nitems, EIG_THREADS, smem, ctx.stream>>>(d_items, src, vout, wout, scratch, d_stat);
    ITG_CHECK_CUDA(cudaGetLastError());
    ctx.kernel_launches++;
}
}  // namespace

int batched_eigh(Ctx& ctx, std::vector<EigItem> const& items, double const* src, double* vout, double* wout,
                 double* scratch) {
    if (items.empty()) return 0;
    int nmax = 0;
    for (auto const& it : items) nmax = std::max(nmax, it.n);
    const bool sa = eig_smem_bytes(nmax, true, false) <= EIG_SMEM_LIMIT;
    const bool sv = sa && eig_smem_bytes(nmax, true, true) <= EIG_SMEM_LIMIT;
    const size_t smem = eig_smem_bytes(nmax, sa, sv);
    size_t o_items = 0, o_stat = ((sizeof(EigItem) * items.size() + 15) / 16) * 16;
    DevBuf buf(o_stat + sizeof(int) * items.size(), ctx.stream);
    ctx.ensure_stage(sizeof(EigItem) * items.size());
    std::memcpy(ctx.stage, items.data(), sizeof(EigItem) * items.size());
    ITG_CHECK_CUDA(cudaMemcpyAsync(buf.as<char>() + o_items, ctx.stage, sizeof(EigItem) * items.size(),
                                   cudaMemcpyHostToDevice, ctx.stream));
    EigItem const* d_items = reinterpret_cast<EigItem const*>(buf.as<char>() + o_items);
    int* d_stat = reinterpret_cast<int*>(buf.as<char>() + o_stat);
    const int ni = (int)items.size();
    if (sa && sv) launch_eig<true, true>(ctx, ni, smem, d_items, src, vout, wout, scratch, d_stat);
    else if (sa) launch_eig<true, false>(ctx, ni, smem, d_items, src, vout, wout, scratch, d_stat);
    else launch_eig<false, false>(ctx, ni, smem, d_items, src, vout, wout, scratch, d_stat);
    std::vector<int> st(items.size());
    ctx.d2h(st.data(), d_stat, sizeof(int) * items.size());
    int bad = 0;
    for (int s : st) bad += s;
    return bad;
}

}  // namespace itg
