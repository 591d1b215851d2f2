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
//      A stays exactly symmetric and only half the blocks are computed).
// FP64 issue slots (~2 FMA per clock per SM on this part) bound the kernel, so
// block pairs whose two rotations are both the identity are skipped, and the
// eigenvectors are not accumulated inside the CTA: every round's (c, s) is
// logged, and a second kernel applies the logged rotations to the rows of
// V = I, a few rows per CTA over many SMs (rows transform independently;
// the rotations of one round touch disjoint columns). Blocks too large for
// the log fall back to accumulating V in the CTA.
// A rotation is skipped when |a_pq| <= max(1e-15 sqrt(|a_pp a_qq|), 2^-52 ||A||_F):
// the relative test of Demmel & Veselic with an absolute floor at the
// backward-error level of a dense symmetric eigensolver (LAPACK's dsyev is
// accurate to O(eps ||A||) in absolute terms). The matrix is converged when a
// sweep skips every pair. Sweeps are capped; a capped matrix still counts as
// converged when its largest off-diagonal entry is below 1e-13 ||A||_F.
#include "ops.h"
#include "eigh_tri.h"
#include <algorithm>
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>

namespace itg {

constexpr int EIG_MAX_SWEEPS = 30;
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

// Rotation (c, s, t) that annihilates a_pq, or false when the pair is
// skipped (|a_pq| <= max(1e-15 sqrt(|a_pp a_qq|), abs_floor)). t is the root
// of smaller magnitude of a_pq t^2 + (a_qq - a_pp) t - a_pq = 0 (Golub & Van
// Loan 8.4.2), c = 1/sqrt(1 + t^2), s = t c.
//
// fast: the dependent chain of one rotation holds no FP64 division or square
// root (each a long sequence of dependent FP64 instructions, and FP64 issues
// at about two per clock per SM here). The operands are scaled by a power of
// two (exact) so that |a_pq| lies in [1, 2); t is seeded in FP32 and refined
// by two Newton steps on the quadratic in FP64 with a fixed FP32 inverse
// slope (relative error ~2^-22, then ~2^-44, then rounding); 1/sqrt(1 + t^2)
// is seeded by the FP32 reciprocal square root and refined by two Newton
// steps y <- y + y (1 - x y^2) / 2. The skip test compares squares in the
// scaled units. Off: the textbook formulas with IEEE division and square root.
__device__ __forceinline__ bool jacobi_pivot(double app, double aqq, double apq, double abs_floor, bool fast,
                                             double& c, double& s, double& t) {
    if (!(fabs(apq) > abs_floor)) return false;
    const int ex = ((__double2hiint(apq) >> 20) & 0x7ff) - 1023;
    if (fast && ex > -1000 && ex < 1000) {
        const double sc = __hiloint2double((1023 - ex) << 20, 0);  // 2^-ex, exact
        const double as = apq * sc, ds = (aqq - app) * sc;
        if (!(as * as > 1e-30 * fabs((app * sc) * (aqq * sc)))) return false;
        const float asf = (float)as, dsf = (float)ds;
        const float tauf = dsf / (2.0f * asf);
        const float t0 = copysignf(1.0f, tauf) / (fabsf(tauf) + sqrtf(fmaf(tauf, tauf, 1.0f)));
        const double r = (double)(1.0f / fmaf(2.0f * asf, t0, dsf));
        double tt = (double)t0;
        double g = fma(fma(as, tt, ds), tt, -as);
        tt = fma(-g, r, tt);
        g = fma(fma(as, tt, ds), tt, -as);
        tt = fma(-g, r, tt);
        const double x = fma(tt, tt, 1.0);
        double y = (double)rsqrtf((float)x);
        double e = fma(-x * y, y, 1.0);
        y = fma(0.5 * y, e, y);
        e = fma(-x * y, y, 1.0);
        y = fma(0.5 * y, e, y);
        t = tt;
        c = y;
        s = tt * y;
        return true;
    }
    if (!(fabs(apq) > 1e-15 * sqrt(fabs(app * aqq)))) return false;
    const double tau = (aqq - app) / (2.0 * apq);
    t = (tau >= 0 ? 1.0 : -1.0) / (fabs(tau) + sqrt(1.0 + tau * tau));
    c = 1.0 / sqrt(1.0 + t * t);
    s = t * c;
    return true;
}

// Runs sweeps on the symmetric n x n matrix A (element (i,j) at A[j*lda+i]).
// Rotations are accumulated into V (element (i,j) at V[j*ldv+i]) when V is
// given, and logged as (c, s) per pair and round when rlog is given. Returns
// the number of sweeps run; *converged tells whether the last one skipped
// every pair.
__device__ int jacobi_run(double* A, int lda, double* V, int ldv, double2* rlog, int n, int np, double abs_floor,
                          bool fast, JacobiShared sh, bool* converged) {
    const int tid = threadIdx.x, nt = blockDim.x;
    const int half = np / 2;
    *converged = false;
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
                    if (jacobi_pivot(app, aqq, apq, abs_floor, fast, c, s, t)) *sh.rotated = 1;
                }
                sh.cst[3 * k] = c;
                sh.cst[3 * k + 1] = s;
                sh.cst[3 * k + 2] = t;
                sh.pq[2 * k] = p;
                sh.pq[2 * k + 1] = q;
                if (rlog) rlog[((size_t)sweep * (np - 1) + r) * half + k] = make_double2(c, s);
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
            // 2b. V <- V J on column pairs (rows contiguous), when accumulated here
            if (V) {
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
            }
            __syncthreads();
        }
        const bool done = (*sh.rotated == 0);
        __syncthreads();
        if (done) {
            *converged = true;
            return sweep + 1;
        }
    }
    return EIG_MAX_SWEEPS;
}

// One block on the device: EigItem plus the offset of its rotation log
// (double2 units; -1 when V is accumulated in the CTA) and of its eigenvalue
// ranks in this launch's rank array.
struct EigJob {
    int64_t a_off, v_off, w_off, s_off, r_off;
    int32_t n, k_off;
};

template <bool SMEM_A, bool SMEM_V>
__global__ void __launch_bounds__(EIG_THREADS) jacobi_kernel(EigJob const* __restrict__ jobs, double const* __restrict__ src,
                                                             double* __restrict__ vout, double* __restrict__ wout,
                                                             double* __restrict__ scratch, double2* __restrict__ rlog,
                                                             int* __restrict__ ranks, int* __restrict__ sweeps_out,
                                                             int* __restrict__ status, int fast) {
    pdl_wait();
    extern __shared__ __align__(16) unsigned char eig_smem[];
    __shared__ int rotated;
    __shared__ double red[32];
    const EigJob it = jobs[blockIdx.x];
    const int n = it.n;
    const int np = n + (n & 1);
    const int half = np / 2;
    const int tid = threadIdx.x;
    const bool logv = it.r_off >= 0;
    // shared layout: cst (3 half doubles) | [A (np x (np+1))] | [V (n x n)] | pq (2 half ints) | rank (n ints)
    double* cst = reinterpret_cast<double*>(eig_smem);
    double* sp = cst + 3 * half;
    double* A;
    int lda;
    if (SMEM_A) { A = sp; lda = np + 1; sp += (size_t)np * lda; }
    else { A = scratch + it.s_off; lda = n; }
    double* V = nullptr;
    if (!logv) {
        if (SMEM_V) { V = sp; sp += (size_t)n * n; }
        else { V = scratch + it.s_off + (size_t)n * n; }
    }
    int* pq = reinterpret_cast<int*>(sp);
    int* rank = pq + 2 * half;
    // load A (and V = I), Frobenius norm
    double loc = 0;
    for (int e = tid; e < n * n; e += blockDim.x) {
        const int i = e % n, j = e / n;
        const double x = src[it.a_off + e];
        A[(size_t)j * lda + i] = x;
        if (V) V[e] = (i == j) ? 1.0 : 0.0;
        loc = fma(x, x, loc);
    }
    for (int o = 16; o; o >>= 1) loc += __shfl_down_sync(0xffffffffu, loc, o);
    if ((tid & 31) == 0) red[tid >> 5] = loc;
    __syncthreads();
    double norm2 = 0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) norm2 += red[w];
    const double normA = sqrt(norm2);
    __syncthreads();
    bool converged = true;
    int nsw = 0;
    if (n > 1)
        nsw = jacobi_run(A, lda, V, n, logv ? rlog + it.r_off : nullptr, n, np, 0x1p-52 * normA, fast != 0,
                         JacobiShared{cst, pq, &rotated}, &converged);
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
        if (logv) ranks[it.k_off + i] = r;
    }
    __syncthreads();
    if (V) {
        for (int e = tid; e < n * n; e += blockDim.x) {
            const int col = e / n, row = e % n;
            vout[it.v_off + (size_t)rank[col] * n + row] = V[e];
        }
    }
    if (tid == 0) sweeps_out[blockIdx.x] = nsw;
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

// Rows [row0, row0 + rows) of one block's eigenvector matrix: V = I, then
// every logged rotation in order (column pairs of a round are disjoint, so a
// round is one parallel step), then written to vout in eigenvalue order.
struct VJob {
    int64_t v_off, r_off, k_off;
    int32_t n, row0, rows, blk;
};

__global__ void __launch_bounds__(EIG_THREADS) vapply_kernel(VJob const* __restrict__ jobs, double2 const* __restrict__ rlog,
                                                             int const* __restrict__ ranks, int const* __restrict__ sweeps,
                                                             double* __restrict__ vout) {
    pdl_wait();
    extern __shared__ __align__(16) unsigned char va_smem[];
    double* vr = reinterpret_cast<double*>(va_smem);  // rows x n, row-major
    const VJob j = jobs[blockIdx.x];
    const int n = j.n, np = n + (n & 1), half = np / 2, R = j.rows;
    const int tid = threadIdx.x, nt = blockDim.x;
    for (int e = tid; e < R * n; e += nt) {
        const int r = e / n, col = e % n;
        vr[e] = (j.row0 + r == col) ? 1.0 : 0.0;
    }
    __syncthreads();
    const int nsw = min(max(sweeps[j.blk], 0), EIG_MAX_SWEEPS);  // the log holds at most this many
    for (int sw = 0; sw < nsw; ++sw) {
        for (int rd = 0; rd < np - 1; ++rd) {
            const double2* lg = rlog + j.r_off + ((size_t)sw * (np - 1) + rd) * half;
            for (int e = tid; e < R * half; e += nt) {
                const int rr = e / half, k = e % half;
                const double2 cs = lg[k];
                if (cs.y == 0.0) continue;
                int p, q;
                round_pair(rd, k, np, p, q);
                if (q >= n) continue;
                double* row = vr + (size_t)rr * n;
                const double a = row[p], b = row[q];
                row[p] = cs.x * a - cs.y * b;
                row[q] = cs.y * a + cs.x * b;
            }
            __syncthreads();
        }
    }
    for (int e = tid; e < R * n; e += nt) {
        const int r = e / n, col = e % n;
        vout[j.v_off + (size_t)ranks[j.k_off + col] * n + j.row0 + r] = vr[e];
    }
}

// Blocks of at most 16 rows (most density-matrix blocks of a chain): the
// same cyclic Jacobi, laid out for the FP64 pipe of this part. One FP64 warp
// instruction holds its SMSP's FP64 pipe for about 64 cycles whatever the
// number of active lanes (measured: a dependent DFMA, DADD, DSETP or F2F
// costs ~64 cycles from one warp; four warps on four SMSPs ~76 each), so a
// round costs FP64 instructions per warp, not flops:
//  - the rotation of each pair (lanes 0..7 of warp 0) is the critical path;
//    its skip tests are integer compares of the bit patterns (|a_pq| against
//    the absolute floor exactly; the relative test 1e-30 a_pp a_qq < a_pq^2
//    on the exponent-and-top-mantissa words, a log2 approximation within
//    0.09), and its FP32 seeds are converted with integer operations, so it
//    holds 17 FP64 instructions (one subtraction, two Newton steps for t,
//    two for 1/sqrt(1 + t^2), s = t c). The seed comes from the unscaled
//    operands: every Newton iterate equals the power-of-two scaled form's
//    while |a_pq| and |a_qq - a_pp| stay inside FP32's range (checked; else
//    the IEEE formulas);
//  - the 2x2 block updates: one lane per output element of the off-diagonal
//    blocks k < l (warps 0-3, 4 lanes per block in one warp, operands read
//    before a __syncwarp and written after it), row and column coefficients
//    chosen by integer selects so the lanes of a warp take one path (6 FP64
//    instructions), the diagonal blocks on warp 4;
//  - V <- V J of round g on warps 5-7 (SMSPs 1-3) while warp 0 (SMSP 0)
//    computes the rotations of round g + 1 (rotations double-buffered).
// Results agree with jacobi_kernel to rounding (same rotations, same update
// formulas; a pair whose coupling sits within the log approximation of the
// relative threshold can be skipped by one and rotated by the other).
constexpr int JS_THREADS = 256;
constexpr int JS_MAXN = 16;
constexpr long long JS_ABS_MASK = 0x7fffffffffffffffLL;
constexpr long long JS_REL_LOG = 104501084LL;  // 99.66 * 2^20: -log2(1e-30) in units of (bits >> 32)

__device__ __forceinline__ long long js_log2fix(double x) { return (__double_as_longlong(x) & JS_ABS_MASK) >> 32; }

// double -> float by truncation (a seed), signed zero below FP32's normal range
__device__ __forceinline__ float js_d2f(double x) {
    const long long b = __double_as_longlong(x);
    const unsigned hi = (unsigned)(b >> 32), lo = (unsigned)b;
    const int e = (int)((hi >> 20) & 0x7ff) - 1023 + 127;
    const unsigned sign = hi & 0x80000000u;
    if (e <= 0) return __uint_as_float(sign);
    return __uint_as_float(sign | ((unsigned)e << 23) | ((hi & 0xfffffu) << 3) | (lo >> 29));
}

// float -> double, exact for normal floats (denormals give signed zero)
__device__ __forceinline__ double js_f2d(float f) {
    const unsigned u = __float_as_uint(f);
    const unsigned e = (u >> 23) & 0xffu;
    const unsigned long long sign = (unsigned long long)(u & 0x80000000u) << 32;
    if (e == 0) return __longlong_as_double((long long)sign);
    return __longlong_as_double(
        (long long)(sign | ((unsigned long long)(e + 896u) << 52) | ((unsigned long long)(u & 0x7fffffu) << 29)));
}

__device__ __forceinline__ double js_neg(double x) { return __longlong_as_double(__double_as_longlong(x) ^ (1LL << 63)); }

// jacobi_pivot with integer skip tests and unscaled seeds (see above)
__device__ __forceinline__ bool js_pivot(double app, double aqq, double apq, long long floor_bits, double& c, double& s,
                                         double& t) {
    const long long b = __double_as_longlong(apq) & JS_ABS_MASK;
    if (b <= floor_bits) return false;
    if (2 * (b >> 32) <= js_log2fix(app) + js_log2fix(aqq) - JS_REL_LOG) return false;
    const double d = aqq - app;
    const int epq = (int)(b >> 52) - 1023;
    const int ed = (int)((__double_as_longlong(d) & JS_ABS_MASK) >> 52) - 1023;
    if (epq > -120 && epq < 120 && ed < 120) {
        const float asf = js_d2f(apq), dsf = js_d2f(d);
        const float tauf = __fdividef(dsf, 2.0f * asf);
        const float t0 = copysignf(__fdividef(1.0f, fabsf(tauf) + sqrtf(fmaf(tauf, tauf, 1.0f))), tauf);
        const double r = js_f2d(__fdividef(1.0f, fmaf(2.0f * asf, t0, dsf)));
        double tt = js_f2d(t0);
        double g = fma(fma(apq, tt, d), tt, -apq);
        tt = fma(-g, r, tt);
        g = fma(fma(apq, tt, d), tt, -apq);
        tt = fma(-g, r, tt);
        const double x = fma(tt, tt, 1.0);
        double y = js_f2d(rsqrtf(js_d2f(x)));
        double e = fma(-x * y, y, 1.0);
        y = fma(0.5 * y, e, y);
        e = fma(-x * y, y, 1.0);
        y = fma(0.5 * y, e, y);
        t = tt;
        c = y;
        s = tt * y;
        return true;
    }
    const double tau = d / (2.0 * apq);
    t = (tau >= 0 ? 1.0 : -1.0) / (fabs(tau) + sqrt(1.0 + tau * tau));
    c = 1.0 / sqrt(1.0 + t * t);
    s = t * c;
    return true;
}

__global__ void __launch_bounds__(JS_THREADS) jacobi_small_kernel(EigJob const* __restrict__ jobs,
                                                                  double const* __restrict__ src, double* __restrict__ vout,
                                                                  double* __restrict__ wout, int* __restrict__ sweeps_out,
                                                                  int* __restrict__ status) {
    pdl_wait();
    __shared__ double A[JS_MAXN * (JS_MAXN + 1)];
    __shared__ double V[JS_MAXN * JS_MAXN];
    __shared__ double cst[2][3 * JS_MAXN / 2];
    __shared__ int pq[2][JS_MAXN];
    __shared__ int rf[2][JS_MAXN / 2];
    __shared__ int rank[JS_MAXN];
    __shared__ int rot_sweep;
    __shared__ double red[JS_THREADS / 32];
    const EigJob it = jobs[blockIdx.x];
    const int n = it.n, np = n + (n & 1), half = np / 2, lda = np + 1;
    const int tid = threadIdx.x, warp = tid >> 5;
    double loc = 0;
    for (int e = tid; e < n * n; e += JS_THREADS) {
        const int i = e % n, j = e / n;
        const double x = src[it.a_off + e];
        A[j * lda + i] = x;
        V[e] = (i == j) ? 1.0 : 0.0;
        loc = fma(x, x, loc);
    }
    if (tid == 0) rot_sweep = 0;
    for (int o = 16; o; o >>= 1) loc += __shfl_down_sync(0xffffffffu, loc, o);
    if ((tid & 31) == 0) red[warp] = loc;
    __syncthreads();
    double norm2 = 0;
    for (int w = 0; w < JS_THREADS / 32; ++w) norm2 += red[w];
    const double normA = sqrt(norm2);
    const long long floor_bits = __double_as_longlong(0x1p-52 * normA);
    // this thread's update work: kind 1 = element (ei, ej) of off-diagonal
    // block (bk, bl); kind 2 = diagonal entry ei of block bk
    const int noff = half * (half - 1) / 2;
    int kind = 0, bk = 0, bl = 0, ei = 0, ej = 0;
    if (tid < 4 * noff) {
        int b = tid >> 2, k = 0;
        while (b >= half - 1 - k) {
            b -= half - 1 - k;
            ++k;
        }
        kind = 1;
        bk = k;
        bl = k + 1 + b;
        ei = (tid >> 1) & 1;
        ej = tid & 1;
    } else if (tid >= 128 && tid - 128 < 2 * half) {
        kind = 2;
        bk = (tid - 128) >> 1;
        ei = (tid - 128) & 1;
    }
    // V items (pair, row) on warps 5-7
    const int vi0 = tid - 160, nvi = half * n;
    auto v_update = [&](int buf) {
        for (int e = vi0; e < nvi; e += 96) {
            const int k = e / n, i = e % n;
            if (!rf[buf][k]) continue;
            const double c = cst[buf][3 * k], s = cst[buf][3 * k + 1];
            const int p = pq[buf][2 * k], q = pq[buf][2 * k + 1];
            const double a = V[p * n + i], b = V[q * n + i];
            V[p * n + i] = c * a - s * b;
            V[q * n + i] = s * a + c * b;
        }
    };
    // rot_sweep holds the last sweep (1-based) that rotated; it only grows, so
    // a thread reading it late in the next sweep still sees "not converged"
    bool converged = (n <= 1);
    int nsw = 0, g = 0;
    for (int sweep = 0; sweep < EIG_MAX_SWEEPS && !converged; ++sweep) {
        for (int r = 0; r < np - 1; ++r, ++g) {
            const int bf = g & 1;
            if (tid < half) {
                const int k = tid;
                int p, q;
                round_pair(r, k, np, p, q);
                double c = 1.0, s = 0.0, t = 0.0;
                bool rot = false;
                if (q < n) rot = js_pivot(A[p * lda + p], A[q * lda + q], A[q * lda + p], floor_bits, c, s, t);
                if (rot) rot_sweep = sweep + 1;
                cst[bf][3 * k] = c;
                cst[bf][3 * k + 1] = s;
                cst[bf][3 * k + 2] = t;
                pq[bf][2 * k] = p;
                pq[bf][2 * k + 1] = q;
                rf[bf][k] = rot;
            } else if (vi0 >= 0 && g > 0) {
                v_update(bf ^ 1);
            }
            __syncthreads();
            if (kind == 1) {
                const int fk = rf[bf][bk], fl = rf[bf][bl];
                const int p = pq[bf][2 * bk], q = pq[bf][2 * bk + 1], u = pq[bf][2 * bl], w = pq[bf][2 * bl + 1];
                const bool qk = q < n, wl = w < n;  // dummy slots hold no row / column
                const int oi = ei ? q : p, oj = ej ? w : u;
                double out = 0;
                if (fk | fl) {
                    const double ck = cst[bf][3 * bk], sk = cst[bf][3 * bk + 1];
                    const double cl = cst[bf][3 * bl], sl = cst[bf][3 * bl + 1];
                    const double x = A[u * lda + p];
                    const double y = wl ? A[w * lda + p] : 0.0;
                    const double z = qk ? A[u * lda + q] : 0.0;
                    const double v = (qk && wl) ? A[w * lda + q] : 0.0;
                    // column oj by (cl, sl), then row oi by (ck, sk)
                    const double m0 = ej ? sl : cl, m1 = ej ? cl : js_neg(sl);
                    const double r0 = ei ? sk : ck, r1 = ei ? ck : js_neg(sk);
                    const double a0 = fma(m0, x, m1 * y), a1 = fma(m0, z, m1 * v);
                    out = fma(r0, a0, r1 * a1);
                }
                __syncwarp();
                if ((fk | fl) && (ei == 0 || qk) && (ej == 0 || wl)) {
                    A[oj * lda + oi] = out;
                    A[oi * lda + oj] = out;
                }
            } else if (kind == 2) {
                // pivot block: diagonalised exactly
                const int fk = rf[bf][bk];
                const int p = pq[bf][2 * bk], q = pq[bf][2 * bk + 1];
                double apq = 0, d = 0;
                if (fk) {
                    apq = A[q * lda + p];
                    d = ei ? A[q * lda + q] : A[p * lda + p];
                }
                __syncwarp();
                if (fk) {
                    const double t = cst[bf][3 * bk + 2];
                    if (ei == 0) {
                        A[p * lda + p] = d - t * apq;
                        A[q * lda + p] = 0.0;
                        A[p * lda + q] = 0.0;
                    } else {
                        A[q * lda + q] = d + t * apq;
                    }
                }
            } else if (tid < 160) {
                __syncwarp();
            }
            __syncthreads();
        }
        nsw = sweep + 1;
        converged = rot_sweep < sweep + 1;
    }
    if (g > 0 && vi0 >= 0) v_update((g - 1) & 1);
    __syncthreads();
    // eigenvalues descending (ties by position); eigenvector columns follow
    for (int i = tid; i < n; i += JS_THREADS) {
        const double di = A[i * lda + i];
        int rr = 0;
        for (int j = 0; j < n; ++j) {
            const double dj = A[j * lda + j];
            rr += (dj > di) || (dj == di && j < i);
        }
        wout[it.w_off + rr] = di;
        rank[i] = rr;
    }
    __syncthreads();
    for (int e = tid; e < n * n; e += JS_THREADS) {
        const int col = e / n, row = e % n;
        vout[it.v_off + (size_t)rank[col] * n + row] = V[e];
    }
    if (tid == 0) sweeps_out[blockIdx.x] = nsw;
    if (!converged) {
        // sweep cap reached: accept when the remaining coupling is negligible
        double mx = 0;
        for (int e = tid; e < n * n; e += JS_THREADS) {
            const int i = e % n, j = e / n;
            if (i != j) mx = fmax(mx, fabs(A[j * lda + i]));
        }
        for (int o = 16; o; o >>= 1) mx = fmax(mx, __shfl_down_sync(0xffffffffu, mx, o));
        __syncthreads();
        if ((tid & 31) == 0) red[warp] = mx;
        __syncthreads();
        if (tid == 0) {
            double m = 0;
            for (int w = 0; w < JS_THREADS / 32; ++w) m = fmax(m, red[w]);
            status[blockIdx.x] = (m <= 1e-13 * normA) ? 0 : 1;
        }
    } else if (tid == 0) {
        status[blockIdx.x] = 0;
    }
}

namespace {
constexpr size_t EIG_SMEM_LIMIT = 227 * 1024;
constexpr size_t EIG_LOG_LIMIT = size_t(512) << 20;   // bytes of rotation log per launch
constexpr int EIG_LOG_MIN_N = 32;                     // smaller blocks accumulate V in the CTA

size_t eig_smem_bytes(int n, bool sa, bool sv) {
    const int np = n + (n & 1), half = np / 2;
    size_t b = sizeof(double) * 3 * half;
    if (sa) b += sizeof(double) * (size_t)np * (np + 1);
    if (sv) b += sizeof(double) * (size_t)n * n;
    b += sizeof(int) * (2 * half + n);
    return b;
}

template <bool SA, bool SV>
void launch_eig(Ctx& ctx, int njobs, size_t smem, EigJob const* d_jobs, double const* src, double* vout, double* wout,
                double* scratch, double2* rlog, int* ranks, int* sweeps, int* d_stat) {
    grow_smem_attr((void const*)jacobi_kernel<SA, SV>, smem);
    // ITG_EIG_IEEE_ROT: rotations by IEEE division and square root (diagnostics)
    static const int fast = std::getenv("ITG_EIG_IEEE_ROT") ? 0 : 1;
    launch_pdl(ctx, njobs, EIG_THREADS, smem, jacobi_kernel<SA, SV>, d_jobs, src, vout, wout, scratch, rlog, ranks, sweeps,
                                                                    d_stat, fast);
    ITG_CHECK_CUDA(cudaGetLastError());
    ctx.kernel_launches++;
}
}  // namespace

// Returns the number of blocks known not to have converged. A solve that runs
// alone does not wait for the statuses here: they are copied to
// ctx.defer_host and *pending is set to their count (eigh_collect reads them
// after the eigenvalue read's wait). Inside a solver-pool fiber the wait
// stays here: measured on the 256-chain batch, deferring it cost 10% of the
// pool's throughput (26.4-27.0 against 29.1-30.1 solves/s, alternating
// runs), while a lone solve gains from it. Either way the results are the same.
static int jacobi_eigh(Ctx& ctx, std::vector<EigItem> const& items, double const* src, double* vout, double* wout,
                       double* scratch, int* pending) {
    *pending = 0;
    if (items.empty()) return 0;
    const int nb = (int)items.size();
    int nmax = 0;
    int64_t ntot = 0;
    size_t log_elems = 0;
    for (auto const& it : items) {
        nmax = std::max(nmax, it.n);
        ntot += it.n;
        const int np = it.n + (it.n & 1);
        log_elems += (size_t)EIG_MAX_SWEEPS * std::max(np - 1, 0) * (np / 2);
    }
    const bool logv = nmax >= EIG_LOG_MIN_N && log_elems * sizeof(double2) <= EIG_LOG_LIMIT;
    // device jobs; eigenvector rows split so that the rotation pass spreads over the SMs
    std::vector<EigJob> jobs(nb);
    std::vector<VJob> vjobs;
    int rows = 16;
    if (logv) {
        while (rows > 1) {
            int64_t cnt = 0;
            for (auto const& it : items) cnt += (it.n + rows - 1) / rows;
            if (cnt >= 2 * (int64_t)ctx.sm_count && (size_t)rows * nmax * sizeof(double) <= EIG_SMEM_LIMIT) break;
            rows /= 2;
        }
        while (rows > 1 && (size_t)rows * nmax * sizeof(double) > EIG_SMEM_LIMIT) rows /= 2;
    }
    size_t roff = 0;
    int32_t koff = 0;  // ranks of this launch's items, packed in item order
    for (int b = 0; b < nb; ++b) {
        auto const& it = items[b];
        const int np = it.n + (it.n & 1);
        jobs[b] = EigJob{it.a_off, it.v_off, it.w_off, it.s_off, logv ? (int64_t)roff : -1, it.n, koff};
        if (logv) {
            for (int r0 = 0; r0 < it.n; r0 += rows)
                vjobs.push_back(VJob{it.v_off, (int64_t)roff, (int64_t)koff, it.n, r0, std::min(rows, it.n - r0), b});
            roff += (size_t)EIG_MAX_SWEEPS * std::max(np - 1, 0) * (np / 2);
        }
        koff += it.n;
    }
    const bool sa = eig_smem_bytes(nmax, true, false) <= EIG_SMEM_LIMIT;
    const bool sv = !logv && sa && eig_smem_bytes(nmax, true, true) <= EIG_SMEM_LIMIT;
    const size_t smem = eig_smem_bytes(nmax, sa, sv);
    // one upload: jobs | vjobs; one device buffer: records | status | sweeps | ranks | log
    auto a16 = [](size_t x) { return (x + 15) / 16 * 16; };
    const size_t o_jobs = 0, o_vj = a16(sizeof(EigJob) * nb), up = a16(o_vj + sizeof(VJob) * vjobs.size());
    const size_t o_stat = up, o_sw = a16(o_stat + sizeof(int) * nb), o_rank = a16(o_sw + sizeof(int) * nb);
    const size_t o_log = a16(o_rank + sizeof(int) * (size_t)ntot);
    const size_t total = o_log + (logv ? sizeof(double2) * log_elems : 0);
    DevBuf buf(total, ctx.stream);
    // through the staging ring: this function returns without waiting for the
    // stream, and the tridiagonal path refills the context's pinned buffer
    char* st = ctx.stage_ring(up);
    std::memcpy(st + o_jobs, jobs.data(), sizeof(EigJob) * nb);
    if (!vjobs.empty()) std::memcpy(st + o_vj, vjobs.data(), sizeof(VJob) * vjobs.size());
    ctx.ring_copy(buf.p, st, up);
    char* db = buf.as<char>();
    int* d_stat = reinterpret_cast<int*>(db + o_stat);
    int* d_sw = reinterpret_cast<int*>(db + o_sw);
    int* d_rank = reinterpret_cast<int*>(db + o_rank);
    double2* d_log = logv ? reinterpret_cast<double2*>(db + o_log) : nullptr;
    EigJob const* d_jobs = reinterpret_cast<EigJob const*>(db + o_jobs);
    static const bool ieee_rot = std::getenv("ITG_EIG_IEEE_ROT") != nullptr;
    if (!logv && nmax <= JS_MAXN && !ieee_rot) {
        launch_pdl(ctx, nb, JS_THREADS, 0, jacobi_small_kernel, d_jobs, src, vout, wout, d_sw, d_stat);
        ITG_CHECK_CUDA(cudaGetLastError());
        ctx.kernel_launches++;
    } else if (sa && sv) launch_eig<true, true>(ctx, nb, smem, d_jobs, src, vout, wout, scratch, d_log, d_rank, d_sw, d_stat);
    else if (sa) launch_eig<true, false>(ctx, nb, smem, d_jobs, src, vout, wout, scratch, d_log, d_rank, d_sw, d_stat);
    else launch_eig<false, false>(ctx, nb, smem, d_jobs, src, vout, wout, scratch, d_log, d_rank, d_sw, d_stat);
    if (logv && !vjobs.empty()) {
        const size_t vsm = sizeof(double) * (size_t)rows * nmax;
        grow_smem_attr((void const*)vapply_kernel, vsm);
        launch_pdl(ctx, (int)vjobs.size(), EIG_THREADS, vsm, vapply_kernel, 
            reinterpret_cast<VJob const*>(db + o_vj), d_log, d_rank, d_sw, vout);
        ITG_CHECK_CUDA(cudaGetLastError());
        ctx.kernel_launches++;
    }
    if (!std::getenv("ITG_EIG_LOG") && !fiber_active()) {
        void* hs = ctx.ensure_defer(sizeof(int) * nb);
        ITG_CHECK_CUDA(cudaMemcpyAsync(hs, d_stat, sizeof(int) * nb, cudaMemcpyDeviceToHost, ctx.stream));
        *pending = nb;
        return 0;
    }
    std::vector<int> stv(nb);
    ctx.d2h(stv.data(), d_stat, sizeof(int) * nb);
    int bad = 0;
    for (int s : stv) bad += s;
    if (std::getenv("ITG_EIG_LOG")) {
        std::vector<int> swv(nb);
        ctx.d2h(swv.data(), d_sw, sizeof(int) * nb);
        std::fprintf(stderr, "itg eigh:");
        for (int b = 0; b < nb; ++b) std::fprintf(stderr, " %d/%d", items[b].n, swv[b]);
        std::fprintf(stderr, "\n");
    }
    return bad;
}

// Small blocks: one-CTA Jacobi; large ones: the tridiagonal path (eigh_tri.cu).
EighPending batched_eigh_begin(Ctx& ctx, std::vector<EigItem> const& items, double const* src, double* vout,
                               double* wout, double* scratch) {
    int tmin = TRI_MIN_N_DEFAULT;
    if (char const* env = std::getenv("ITG_EIG_TRI_MIN")) tmin = std::max(1, std::atoi(env));
    std::vector<EigItem> small, large;
    std::vector<int> large_ids;
    for (int i = 0; i < (int)items.size(); ++i) {
        auto const& it = items[i];
        if (it.n >= tmin && it.n <= TRI_MAX_N) {
            large.push_back(it);
            large_ids.push_back(i);
        } else {
            small.push_back(it);
        }
    }
    const bool timing = std::getenv("ITG_EIG_TIME") != nullptr;  // diagnostics: wall time of each path
    auto now = [&] { ctx.sync(); return std::chrono::steady_clock::now(); };
    auto t0 = timing ? now() : std::chrono::steady_clock::time_point{};
    // Jacobi first: its uploads go through the staging ring (no wait), the
    // tridiagonal path's through the context's pinned buffer, which it waits
    // for before it returns
    EighPending p;
    p.bad = jacobi_eigh(ctx, small, src, vout, wout, scratch, &p.jac_pending);
    auto t1 = timing ? now() : t0;
    int bad_tri = 0;
    p.tri = tri_eigh_begin(ctx, large, large_ids, src, wout, scratch, &bad_tri);
    p.bad += bad_tri;
    if (timing) {
        auto t2 = now();
        int nl = 0, ns = 0;
        for (auto const& it : large) nl = std::max(nl, it.n);
        for (auto const& it : small) ns = std::max(ns, it.n);
        std::fprintf(stderr, "itg eigh-time: tri %zu blocks nmax %d %.3f ms | jacobi %zu blocks nmax %d %.3f ms\n",
                     large.size(), nl, std::chrono::duration<double, std::milli>(t2 - t1).count(), small.size(), ns,
                     std::chrono::duration<double, std::milli>(t1 - t0).count());
    }
    return p;
}

int eigh_collect(Ctx& ctx, EighPending& p) {
    if (p.jac_pending) {
        int const* st = static_cast<int const*>(ctx.defer_host);
        for (int i = 0; i < p.jac_pending; ++i) p.bad += st[i];
        p.jac_pending = 0;
    }
    return p.bad;
}

void batched_eigh_finish(Ctx& ctx, EighPending& p, std::vector<int> const& keep, double* vout, double* scratch) {
    if (p.tri) tri_eigh_finish(ctx, *p.tri, keep, vout, scratch);
}

int batched_eigh(Ctx& ctx, std::vector<EigItem> const& items, double const* src, double* vout, double* wout,
                 double* scratch) {
    EighPending p = batched_eigh_begin(ctx, items, src, vout, wout, scratch);
    if (p.jac_pending) ctx.sync();
    if (eigh_collect(ctx, p)) return p.bad;
    std::vector<int> all(items.size());
    for (size_t i = 0; i < items.size(); ++i) all[i] = items[i].n;
    batched_eigh_finish(ctx, p, all, vout, scratch);
    return 0;
}

}  // namespace itg
