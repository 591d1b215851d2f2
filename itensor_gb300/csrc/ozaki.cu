// Split-precision block GEMM (after Ozaki et al., error-free splitting of
// matrix products) on the BF16 tensor pipe of sm_103a.
//
// Every operand block is seen as a rows x K matrix (A: rows = m, B: rows = n).
// Each row gets a power-of-two scale e with |x| < 2^e, and each entry becomes
// the signed fixed-point integer X = round(x 2^(7S - e)) cut into S balanced
// base-128 digits: d_1..d_{S-1} in [-64, 63], d_0 in [-128, 128], all exact
// in BF16. Balanced digits carry signs independent of the entry's sign, so
// the digit products left out below average to zero rather than shrinking
// every product. Digit products are exact in FP32 and so are their sums while
// |sum| < 2^24. Digit pairs (s,t) with s+t < S are accumulated per diagonal
// D = s+t with mma.sync m16n8k16 (FP32 accumulate), folded exactly into one
// int64 per output (sum_D acc_D 2^(7(S-1-D))) every KCHUNK k (a diagonal holds
// at most S digit products of |d| <= 128 per k, so KCHUNK * S * 128^2 <= 2^24
// keeps every partial sum an exact FP32 integer: 128 k for S = 5, 6; 256 for
// S <= 4), and scaled into the FP64 output once
// per block pair (one fold is below 2^57 in magnitude, so the int64 sum of a
// pair cannot overflow while the pair's K <= 64 * KCHUNK; plans with a longer
// pair run the FP64 kernel, see plan_uses_split). Accuracy ~2^(-7S)
// of the row/column maxima. Slicing and
// folding are integer work: FP64 issue slots on this part are ~1/60 of FP32.
//
// prep: one CTA per item of whole rows (~2048 elements), one warp per row,
//       writes the row exponents and the S digit planes, k-contiguous, K
//       padded to 16.
// gemm: output tiles of 32 x 32 (4 warps of 16 x 16) or 64 x 32 (8 warps),
//       one CTA per tile or persistent CTAs over the tile list; the variant
//       is chosen per plan by autotune_ozaki. Digit panels are staged with
//       cp.async into a two-stage shared-memory ring and read with ldmatrix.
#include "engine.h"
#include <cuda_bf16.h>
#include <algorithm>
#include <cstdio>
#include <cstdlib>

namespace itg {

__device__ __forceinline__ int exp_field(double x) {
    return (int)((__double_as_longlong(x) >> 52) & 0x7FF);
}

// The S balanced digits of x against the row exponent field emax, written to
// dst[s * plane] (BF16-exact integers).
template <int S>
__device__ __forceinline__ void oz_digits(double x, int emax, __nv_bfloat16* dst, int64_t plane) {
    long long bits = __double_as_longlong(x);
    int ef = (int)((bits >> 52) & 0x7FF);
    unsigned long long Xf = 0;
    if (ef != 0) {
        unsigned long long mant = (bits & ((1ull << 52) - 1)) | (1ull << 52);
        int sh = ef - 1075 + 7 * S - (emax - 1022);  // <= 7S - 53 < 0 for S <= 7
        // rounded to nearest, not truncated: truncation shrinks every entry's
        // magnitude and the bias adds up coherently in the products
        if (sh >= 0) Xf = mant << sh;
        else if (sh > -64) Xf = (mant >> (-sh)) + ((mant >> (-sh - 1)) & 1ull);
    }
    // balanced digits: d_1..d_{S-1} in [-64, 63], d_0 in [-128, 128] (BF16-exact).
    // Their signs are independent of the entry's sign, so the digit products
    // left out (s + t >= S) average to zero instead of always shrinking |x y|.
    long long X = bits < 0 ? -(long long)Xf : (long long)Xf;
    int dig[S];
#pragma unroll
    for (int s = S - 1; s >= 1; --s) {
        const long long d = ((X + 64) & 127) - 64;
        dig[s] = (int)d;
        X = (X - d) >> 7;
    }
    dig[0] = (int)X;
#pragma unroll
    for (int s = 0; s < S; ++s) dst[s * plane] = __float2bfloat16_rn((float)dig[s]);
}

// Rows of up to 32 * OZ_PREP_REGS entries: one warp per row, the row read once
// into registers, the exponent a warp max, the digits written k-contiguous
// (items of OZ_PREP_ITEM_ROWS rows, all rows in flight at once). Longer rows:
// items of a few rows whose rows x K entries are spread over the whole CTA.
template <int S>
__global__ void __launch_bounds__(256) ozaki_prep_kernel(const PrepItem* __restrict__ items, const OpBlockRec* __restrict__ ops,
                                                         const int32_t* __restrict__ tab, const double* __restrict__ A,
                                                         const double* __restrict__ B, __nv_bfloat16* __restrict__ panels,
                                                         int64_t plane, int32_t* __restrict__ exps) {
    const PrepItem pi = items[blockIdx.x];
    const OpBlockRec ob = ops[pi.op];
    const double* __restrict__ base = (pi.which ? B : A) + ob.src;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    if (ob.Kp > 32 * OZ_PREP_REGS) {
        // long rows: the item's rows x K entries spread over the CTA (a few rows per item)
        __shared__ int rexp[OZ_PREP_LONG_ROWS];
        __shared__ int32_t trow[OZ_PREP_LONG_ROWS];
        const int rows = pi.r1 - pi.r0;
        const int n = rows * ob.K;
        for (int r = threadIdx.x; r < rows; r += blockDim.x) {
            rexp[r] = 0;
            trow[r] = tab_at(tab, ob.trow, pi.r0 + r);
        }
        __syncthreads();
        for (int e = threadIdx.x; e < n; e += blockDim.x) {
            const int r = e % rows, k = e / rows;
            atomicMax(&rexp[r], exp_field(base[trow[r] + tab_at(tab, ob.tcol, k)]));
        }
        __syncthreads();
        for (int r = threadIdx.x; r < rows; r += blockDim.x) exps[ob.exp + pi.r0 + r] = rexp[r] - 1022;
        const int np = rows * ob.Kp;
        __nv_bfloat16* pan = panels + ob.panel + (int64_t)pi.r0 * ob.Kp;
        for (int e = threadIdx.x; e < np; e += blockDim.x) {
            const int k = e % ob.Kp, r = e / ob.Kp;
            oz_digits<S>(k < ob.K ? base[trow[r] + tab_at(tab, ob.tcol, k)] : 0.0, rexp[r], pan + e, plane);
        }
        return;
    }
    for (int r = pi.r0 + warp; r < pi.r1; r += nw) {
        const int32_t ro = tab_at(tab, ob.trow, r);
        double xr[OZ_PREP_REGS];
        int emax = 0;
#pragma unroll
        for (int j = 0; j < OZ_PREP_REGS; ++j) {
            const int k = lane + 32 * j;
            xr[j] = k < ob.K ? base[ro + tab_at(tab, ob.tcol, k)] : 0.0;
            emax = max(emax, exp_field(xr[j]));
        }
        for (int k = lane + 32 * OZ_PREP_REGS; k < ob.K; k += 32)
            emax = max(emax, exp_field(base[ro + tab_at(tab, ob.tcol, k)]));
        emax = __reduce_max_sync(0xffffffffu, emax);
        if (lane == 0) exps[ob.exp + r] = emax - 1022;  // |x| < 2^(E-1022)
        __nv_bfloat16* pan = panels + ob.panel + (int64_t)r * ob.Kp;
#pragma unroll
        for (int j = 0; j < OZ_PREP_REGS; ++j) {
            const int k = lane + 32 * j;
            if (k < ob.Kp) oz_digits<S>(xr[j], emax, pan + k, plane);
        }
        for (int k = lane + 32 * OZ_PREP_REGS; k < ob.Kp; k += 32)
            oz_digits<S>(k < ob.K ? base[ro + tab_at(tab, ob.tcol, k)] : 0.0, emax, pan + k, plane);
    }
}

// v * 2^e as FP64, built with integer instructions (round to nearest, ties to
// even): the FP64 unit issues ~1/60 of the FP32 rate on this part. Values stay
// in the normal range here (|v| < 2^63, e >= -1100 with nonzero v well above).
__device__ __forceinline__ double scaled_i64(long long v, int e) {
    if (v == 0) return 0.0;
    const unsigned long long sign = v < 0 ? (1ull << 63) : 0ull;
    unsigned long long u = v < 0 ? (unsigned long long)(-v) : (unsigned long long)v;
    int msb = 63 - __clzll(u);
    unsigned long long mant;
    if (msb > 52) {
        const int sh = msb - 52;
        mant = u >> sh;
        const unsigned long long rem = u & ((1ull << sh) - 1), half = 1ull << (sh - 1);
        if (rem > half || (rem == half && (mant & 1ull))) ++mant;
        if (mant >> 53) { mant >>= 1; ++msb; }
    } else {
        mant = u << (52 - msb);
    }
    const long long ex = (long long)msb + e + 1023;
    if (ex <= 0) return 0.0;  // below the normal range: negligible against the tile's scale
    return __longlong_as_double((long long)(sign | ((unsigned long long)ex << 52) | (mant & ((1ull << 52) - 1))));
}

__device__ __forceinline__ void cp_async16(void* smem, const void* gmem, bool valid) {
    const unsigned saddr = (unsigned)__cvta_generic_to_shared(smem);
    const int bytes = valid ? 16 : 0;  // 0: zero-fill, nothing read
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(saddr), "l"(gmem), "r"(bytes));
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N)); }

__device__ __forceinline__ void ldmatrix_x4(uint32_t (&r)[4], const void* smem) {
    const unsigned a = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];\n"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
                 : "r"(a));
}

// One output tile of TM = 16 WM rows x 32 columns, WM x 2 warps of 16 x 16
// (2 mma n-tiles each). Panels are staged with cp.async into a two-stage ring
// and read with ldmatrix; per pair the S(S+1)/2 digit products go to S FP32
// diagonal accumulators, folded into int64 every KCHUNK k, and the pair's int64
// sum is scaled into the FP64 output (integer instructions) and added.
template <int S, int WM>
__device__ __forceinline__ void oz_tile(ItemRec const& it, const PairRec* __restrict__ pairs,
                                        const CBlockRec* __restrict__ cblk, const OpBlockRec* __restrict__ ops,
                                        const int32_t* __restrict__ tab, const __nv_bfloat16* __restrict__ panels,
                                        int64_t plane, const int32_t* __restrict__ exps, double* __restrict__ C,
                                        unsigned char* smem) {
    constexpr int TM = 16 * WM, TN = 32, TK = 16, LD = TK + 8;  // row stride 48 B: 16-B aligned, no ldmatrix conflicts
    constexpr int NT = 64 * WM;
    constexpr int KCHUNK = (S <= 4) ? 256 : 128;
    static_assert((long long)KCHUNK * S * 128 * 128 <= (1LL << 24), "digit sums must stay exact in FP32");
    typedef __nv_bfloat16 TileA[S][TM][LD];
    typedef __nv_bfloat16 TileB[S][TN][LD];
    TileA* As = reinterpret_cast<TileA*>(smem);                      // [2]
    TileB* Bs = reinterpret_cast<TileB*>(smem + 2 * sizeof(TileA));  // [2]
    int* ea = reinterpret_cast<int*>(smem + 2 * sizeof(TileA) + 2 * sizeof(TileB));
    int* eb = ea + TM;
    const CBlockRec cb = cblk[it.c];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int wm = (warp % WM) * 16, wn = (warp / WM) * 16;
    const int g = lane >> 2, tg = lane & 3;
    // ldmatrix lane addresses (see the m16n8k16 fragment layouts)
    const int a_row = wm + (lane & 15), a_col = (lane >> 4) * 8;
    const int b_row = wn + (lane & 7) + ((lane >> 4) << 3), b_col = ((lane >> 3) & 1) * 8;
    double out[2][4];
#pragma unroll
    for (int j = 0; j < 2; ++j)
#pragma unroll
        for (int q = 0; q < 4; ++q) out[j][q] = 0.0;
    for (int p = it.p0; p < it.p1; ++p) {
        const PairRec pr = pairs[p];
        const OpBlockRec oa = ops[pr.ia], ob = ops[pr.ib];
        const __nv_bfloat16* pa = panels + oa.panel;
        const __nv_bfloat16* pb = panels + ob.panel;
        // stage k-step k0 into ring slot `buf`: S planes x rows x 2 halves, for A and B
        auto stage = [&](int k0, int buf) {
            for (int e = tid; e < 2 * S * (TM + TN); e += NT) {
                const int half = e & 1, r2 = e >> 1;
                if (r2 < S * TM) {
                    const int row = r2 % TM, s = r2 / TM;
                    const bool ok = it.m0 + row < cb.M;
                    const __nv_bfloat16* src = ok ? pa + s * plane + (int64_t)(it.m0 + row) * oa.Kp + k0 + half * 8 : pa;
                    cp_async16(&As[buf][s][row][half * 8], src, ok);
                } else {
                    const int row = (r2 - S * TM) % TN, s = (r2 - S * TM) / TN;
                    const bool ok = it.n0 + row < cb.N;
                    const __nv_bfloat16* src = ok ? pb + s * plane + (int64_t)(it.n0 + row) * ob.Kp + k0 + half * 8 : pb;
                    cp_async16(&Bs[buf][s][row][half * 8], src, ok);
                }
            }
            cp_async_commit();
        };
        for (int r = tid; r < TM + TN; r += NT) {
            if (r < TM) ea[r] = (it.m0 + r < cb.M) ? exps[oa.exp + it.m0 + r] : 0;
            else eb[r - TM] = (it.n0 + r - TM < cb.N) ? exps[ob.exp + it.n0 + r - TM] : 0;
        }
        long long tot[2][4];
        float acc[S][2][4];
#pragma unroll
        for (int j = 0; j < 2; ++j)
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                tot[j][q] = 0;
#pragma unroll
                for (int d = 0; d < S; ++d) acc[d][j][q] = 0.f;
            }
        const int nk = (pr.K + TK - 1) / TK;
        int kacc = 0;
        stage(0, 0);
        for (int kk = 0; kk < nk; ++kk) {
            const int buf = kk & 1;
            if (kk + 1 < nk) {
                stage((kk + 1) * TK, buf ^ 1);
                cp_async_wait<1>();
            } else {
                cp_async_wait<0>();
            }
            __syncthreads();
            uint32_t bfr[S][4];
#pragma unroll
            for (int t = 0; t < S; ++t) ldmatrix_x4(bfr[t], &Bs[buf][t][b_row][b_col]);
#pragma unroll
            for (int s = 0; s < S; ++s) {
                uint32_t af[4];
                ldmatrix_x4(af, &As[buf][s][a_row][a_col]);
#pragma unroll
                for (int t = 0; t + s < S; ++t)
#pragma unroll
                    for (int j = 0; j < 2; ++j) {
                        float* c = acc[s + t][j];
                        // register-only: not volatile, so the compiler may interleave independent MMAs
                        asm("mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, "
                            "{%8,%9}, {%0,%1,%2,%3};\n"
                            : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
                            : "r"(af[0]), "r"(af[1]), "r"(af[2]), "r"(af[3]), "r"(bfr[t][2 * j]),
                              "r"(bfr[t][2 * j + 1]));
                    }
            }
            __syncthreads();  // ring slot `buf` is refilled by the next stage()
            kacc += TK;
            if (kacc >= KCHUNK || kk + 1 == nk) {
#pragma unroll
                for (int j = 0; j < 2; ++j)
#pragma unroll
                    for (int q = 0; q < 4; ++q) {
                        long long v = 0;
#pragma unroll
                        for (int d = 0; d < S; ++d) {
                            // |acc| < 2^24: a 32-bit conversion is exact (64-bit ones issue on the FP64 pipe)
                            v += (long long)__float2int_rn(acc[d][j][q]) << (7 * (S - 1 - d));
                            acc[d][j][q] = 0.f;
                        }
                        tot[j][q] += v;
                    }
                kacc = 0;
            }
        }
        // value = tot * 2^(e_row + e_col - 7 S - 7): one FP64 scale per output and pair
#pragma unroll
        for (int j = 0; j < 2; ++j)
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const int r = wm + g + (q >= 2 ? 8 : 0);
                const int cc = wn + j * 8 + tg * 2 + (q & 1);
                const double v = scaled_i64(tot[j][q], ea[r] + eb[cc] - 7 * S - 7);
                out[j][q] = (p == it.p0) ? v : out[j][q] + v;
            }
        __syncthreads();  // ea/eb are rewritten by the next pair
    }
#pragma unroll
    for (int j = 0; j < 2; ++j)
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const int m = it.m0 + wm + g + (q >= 2 ? 8 : 0);
            const int n = it.n0 + wn + j * 8 + tg * 2 + (q & 1);
            if (m < cb.M && n < cb.N) C[cb.coff + tab_at(tab, cb.tcm, m) + tab_at(tab, cb.tcn, n)] = out[j][q];
        }
}

template <int S, int WM>
constexpr size_t oz_smem_bytes() {
    return sizeof(__nv_bfloat16) * 2 * S * (16 * WM + 32) * (16 + 8) + sizeof(int) * (16 * WM + 32);
}

// PERSIST: a grid of (SMs x resident CTAs) walks the cost-ordered tile list
// with a fixed stride; otherwise one CTA per tile. Either way every output
// element is computed by one thread in the same order, so all variants give
// bit-identical results.
template <int S, int WM, bool PERSIST>
__global__ void __launch_bounds__(64 * WM, (WM == 2 ? 4 : 2))
gemm_ozaki_kernel(const ItemRec* __restrict__ items, int nitems, const PairRec* __restrict__ pairs,
                  const CBlockRec* __restrict__ cblk, const OpBlockRec* __restrict__ ops, const int32_t* __restrict__ tab,
                  const __nv_bfloat16* __restrict__ panels, int64_t plane, const int32_t* __restrict__ exps,
                  double* __restrict__ C) {
    extern __shared__ __align__(16) unsigned char oz_smem[];
    if (PERSIST) {
        for (int i = blockIdx.x; i < nitems; i += gridDim.x)
            oz_tile<S, WM>(items[i], pairs, cblk, ops, tab, panels, plane, exps, C, oz_smem);
    } else {
        oz_tile<S, WM>(items[blockIdx.x], pairs, cblk, ops, tab, panels, plane, exps, C, oz_smem);
    }
}

// ---------------------------------------------------------------- tensor-core (tcgen05) variant
//
// The same digit products on the 5th-generation tensor cores: one CTA (one
// warpgroup) per output tile of 128 rows (TMEM lanes) x TN columns. Per k-step
// of 16 the S digit planes of both operands' tiles are staged with cp.async
// into shared memory in the no-swizzle K-major core-matrix layout (8 rows x
// 16 bytes per core matrix; neighbours along k 128 B apart, along the rows
// 256 B apart), two stages in a ring. One thread issues the S(S+1)/2
// tcgen05.mma (kind::f16, BF16 in, FP32 accumulate) of the step, each into the
// TMEM columns of its diagonal D = s + t, and commits them to the stage's
// mbarrier; the stage is refilled once that barrier has flipped. Every KCHUNK k
// (and at each pair's end) the warps read the S diagonals back with
// tcgen05.ld (thread t holds row t), fold them exactly into int64 and, per
// pair, scale into the FP64 result as the mma.sync variants do: the results
// are bit-identical to theirs. Every wait on an mbarrier is bounded (clock64);
// a wait that gives up sets the context's status word, waits (bounded) for the
// MMAs in flight, frees TMEM and returns without writing the tile.

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

__device__ __forceinline__ bool mbar_try_wait(uint32_t bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    return ok != 0;
}

// Waits for the completion of the barrier phase with this parity, at most
// `limit` SM clocks; false when it gave up.
__device__ __forceinline__ bool mbar_wait_bounded(uint32_t bar, uint32_t parity, long long limit) {
    const long long t0 = clock64();
    while (!mbar_try_wait(bar, parity))
        if (clock64() - t0 > limit) return false;
    return true;
}

// Shared-memory matrix descriptor of tcgen05.mma: start address, leading
// (k-direction) and stride (row-direction) byte offsets of the core matrices,
// descriptor version 1, no swizzle.
__device__ __forceinline__ uint64_t tc_sdesc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
    return (uint64_t)((saddr & 0x3FFFFu) >> 4) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
           ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}

// Instruction descriptor of kind::f16: FP32 accumulator, BF16 A and B, both
// K-major, M x N.
__host__ __device__ constexpr uint32_t tc_idesc_bf16(int M, int N) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void tc_mma(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc, uint32_t acc) {
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.u32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(acc));
}

__device__ __forceinline__ void tc_commit(uint32_t bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar) : "memory");
}

// 32 consecutive TMEM columns of this warp's 32 lanes (thread = lane = row)
__device__ __forceinline__ void tc_ld32(uint32_t taddr, uint32_t (&r)[32]) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
        "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
          "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
          "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

template <int S, int TN>
struct TcShape {
    static constexpr int TM = TC_TILE_M, KS = 16;
    static constexpr int A_PLANE = TM * KS * 2;   // bytes of one digit plane of the row tile
    static constexpr int B_PLANE = TN * KS * 2;   // of the column tile
    static constexpr int STAGE = S * (A_PLANE + B_PLANE);
    static constexpr int KCHUNK = (S <= 4) ? 256 : 128;
    static constexpr int CHUNK_STEPS = KCHUNK / KS;
    static constexpr uint32_t TMEM_COLS = (S * TN <= 128) ? 128 : (S * TN <= 256 ? 256 : 512);
    static constexpr int OUT = 8 * TN * TM;          // FP64 partial results, [column][row]
    static constexpr int TAIL = 64 + 4 * TN;        // barriers, TMEM address, column exponents
    // at least 80 KB, so that at most two CTAs share an SM (their TMEM then always fits)
    static constexpr size_t SMEM =
        (2 * STAGE + OUT + TAIL) > 80 * 1024 ? (size_t)(2 * STAGE + OUT + TAIL) : (size_t)80 * 1024;
};

template <int S, int TN>
__global__ void __launch_bounds__(128, 1)
gemm_ozaki_tc_kernel(const TcItem* __restrict__ items, const PairRec* __restrict__ pairs,
                     const CBlockRec* __restrict__ cblk, const OpBlockRec* __restrict__ ops,
                     const int32_t* __restrict__ tab, const __nv_bfloat16* __restrict__ panels, int64_t plane,
                     const int32_t* __restrict__ exps, double* __restrict__ C, int* __restrict__ status,
                     long long wait_limit, int stuck_test) {
    using SH = TcShape<S, TN>;
    static_assert(S * TN <= 512, "diagonal accumulators must fit in TMEM");
    static_assert((long long)SH::KCHUNK * S * 128 * 128 <= (1LL << 24), "digit sums must stay exact in FP32");
    extern __shared__ __align__(128) unsigned char tc_smem[];
    unsigned char* stage0 = tc_smem;
    double* outs = reinterpret_cast<double*>(tc_smem + 2 * SH::STAGE);  // outs[j * TM + row]
    uint64_t* mbar = reinterpret_cast<uint64_t*>(tc_smem + 2 * SH::STAGE + SH::OUT);
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(tc_smem + 2 * SH::STAGE + SH::OUT + 16);
    int* ecol = reinterpret_cast<int*>(tc_smem + 2 * SH::STAGE + SH::OUT + 64);
    const int tid = threadIdx.x, warp = tid >> 5;
    const TcItem it = items[blockIdx.x];
    const CBlockRec cb = cblk[it.c];
    const uint32_t bar0 = smem_u32(&mbar[0]), bar1 = smem_u32(&mbar[1]);
    // a barrier nothing arrives at: with stuck_test the first fold waits on it
    // until the wait limit runs out (the test of the timeout path)
    const uint32_t bar_stuck = smem_u32(tmem_slot + 2);
    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar0));
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar1));
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar_stuck));
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                     "r"(SH::TMEM_COLS));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tmem_slot;
    const uint32_t tmem_warp = tmem + ((uint32_t)(warp * 32) << 16);
    const int Mrows = it.swap ? cb.N : cb.M, Ncols = it.swap ? cb.M : cb.N;
    constexpr uint32_t IDESC = tc_idesc_bf16(SH::TM, TN);
    uint32_t ncommit[2] = {0u, 0u};
    long long tot[TN];
    bool fail = false;
    const int row = it.r0 + tid;
    for (int p = it.p0; p < it.p1 && !fail; ++p) {
        const PairRec pr = pairs[p];
        const OpBlockRec orow = ops[it.swap ? pr.ib : pr.ia];
        const OpBlockRec ocol = ops[it.swap ? pr.ia : pr.ib];
        const __nv_bfloat16* prow = panels + orow.panel;
        const __nv_bfloat16* pcol = panels + ocol.panel;
        const int Kp = orow.Kp;
        const int nk = Kp / SH::KS;
        const int erow = row < Mrows ? exps[orow.exp + row] : 0;
        __syncthreads();  // the previous pair's readers of ecol are done
        for (int j = tid; j < TN; j += 128) ecol[j] = (it.c0 + j < Ncols) ? exps[ocol.exp + it.c0 + j] : 0;
#pragma unroll
        for (int j = 0; j < TN; ++j) tot[j] = 0;
        // stage k-step kk into ring slot buf: 16-byte chunks (8 k of one row) into core matrices
        auto load = [&](int kk, int buf) {
            unsigned char* sb = stage0 + buf * SH::STAGE;
            const int k0 = kk * SH::KS;
#pragma unroll 1
            for (int e = tid; e < S * (SH::TM + TN) * 2; e += 128) {
                const int kg = e & 1, r2 = e >> 1;
                if (r2 < S * SH::TM) {
                    const int s = r2 / SH::TM, r = r2 % SH::TM;
                    const bool ok = it.r0 + r < Mrows;
                    const __nv_bfloat16* src = ok ? prow + s * plane + (int64_t)(it.r0 + r) * Kp + k0 + kg * 8 : prow;
                    cp_async16(sb + s * SH::A_PLANE + ((r >> 3) * 2 + kg) * 128 + (r & 7) * 16, src, ok);
                } else {
                    const int r3 = r2 - S * SH::TM;
                    const int s = r3 / TN, r = r3 % TN;
                    const bool ok = it.c0 + r < Ncols;
                    const __nv_bfloat16* src = ok ? pcol + s * plane + (int64_t)(it.c0 + r) * Kp + k0 + kg * 8 : pcol;
                    cp_async16(sb + S * SH::A_PLANE + s * SH::B_PLANE + ((r >> 3) * 2 + kg) * 128 + (r & 7) * 16, src,
                               ok);
                }
            }
            cp_async_commit();
        };
        load(0, 0);
        for (int kk = 0; kk < nk; ++kk) {
            const int buf = kk & 1;
            if (kk + 1 < nk) {
                // ring slot buf^1 was last read by the MMAs of step kk-1 (or an earlier pair's)
                if (ncommit[buf ^ 1] > 0) {
                    const bool ok = mbar_wait_bounded(buf ? bar0 : bar1, (ncommit[buf ^ 1] - 1) & 1, wait_limit);
                    if (__syncthreads_or(!ok)) { fail = true; break; }
                }
                load(kk + 1, buf ^ 1);
                cp_async_wait<1>();
            } else {
                cp_async_wait<0>();
            }
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");  // cp.async data -> the MMA's reads
            __syncthreads();
            tc_fence_after();
            if (tid == 0) {
                const bool first = (kk % SH::CHUNK_STEPS) == 0;
                const uint32_t sa = smem_u32(stage0 + buf * SH::STAGE), sbb = sa + S * SH::A_PLANE;
#pragma unroll 1
                for (int s = 0; s < S; ++s)
#pragma unroll 1
                    for (int t = 0; s + t < S; ++t)
                        tc_mma(tmem + (uint32_t)((s + t) * TN), tc_sdesc(sa + s * SH::A_PLANE, 128, 256),
                               tc_sdesc(sbb + t * SH::B_PLANE, 128, 256), IDESC, (first && s == 0) ? 0u : 1u);
                tc_commit(buf ? bar1 : bar0);
            }
            ncommit[buf]++;
            if ((kk + 1) % SH::CHUNK_STEPS == 0 || kk + 1 == nk) {
                const bool ok = stuck_test ? mbar_wait_bounded(bar_stuck, 0, wait_limit)
                                           : mbar_wait_bounded(buf ? bar1 : bar0, (ncommit[buf] - 1) & 1, wait_limit);
                if (__syncthreads_or(!ok)) { fail = true; break; }
                tc_fence_after();
#pragma unroll
                for (int d = 0; d < S; ++d)
#pragma unroll
                    for (int c0 = 0; c0 < TN; c0 += 32) {
                        uint32_t r[32];
                        tc_ld32(tmem_warp + (uint32_t)(d * TN + c0), r);
#pragma unroll
                        for (int j = 0; j < 32; ++j)
                            // |acc| < 2^24: the 32-bit conversion is exact
                            tot[c0 + j] += (long long)__float2int_rn(__uint_as_float(r[j])) << (7 * (S - 1 - d));
                    }
                tc_fence_before();
                __syncthreads();  // every warp has read TMEM before the next MMAs overwrite it
            }
        }
        if (fail) break;
#pragma unroll
        for (int j = 0; j < TN; ++j) {
            const double v = scaled_i64(tot[j], erow + ecol[j] - 7 * S - 7);
            outs[j * SH::TM + tid] = (p == it.p0) ? v : outs[j * SH::TM + tid] + v;
        }
    }
    if (fail) {
        if (tid == 0) atomicExch(status, 1);
        cp_async_wait<0>();
        // the MMAs in flight finish before TMEM is released (bounded again)
        if (ncommit[0] > 0) mbar_wait_bounded(bar0, (ncommit[0] - 1) & 1, wait_limit);
        if (ncommit[1] > 0) mbar_wait_bounded(bar1, (ncommit[1] - 1) & 1, wait_limit);
    } else if (row < Mrows) {
#pragma unroll
        for (int j = 0; j < TN; ++j) {
            const int col = it.c0 + j;
            if (col < Ncols) {
                const int m = it.swap ? col : row, n = it.swap ? row : col;
                C[cb.coff + tab_at(tab, cb.tcm, m) + tab_at(tab, cb.tcn, n)] = outs[j * SH::TM + tid];
            }
        }
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(SH::TMEM_COLS));
}

namespace {
// Resident CTAs per SM of a variant (queried once per process).
template <int S, int WM, bool PERSIST>
int oz_resident() {
    static int r = [] {
        int n = 0;
        cudaFuncSetAttribute(gemm_ozaki_kernel<S, WM, PERSIST>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)oz_smem_bytes<S, WM>());
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, gemm_ozaki_kernel<S, WM, PERSIST>, 64 * WM,
                                                      oz_smem_bytes<S, WM>());
        return std::max(1, n);
    }();
    return r;
}

template <int S, int WM, bool PERSIST>
void launch_gemm(Ctx& ctx, Plan const& p, double* C, __nv_bfloat16 const* panels, int64_t plane, int32_t const* exps) {
    const ItemRec* items = WM == 2 ? p.d_items : p.d_items64;
    const int nitems = WM == 2 ? p.nitems : p.nitems64;
    if (nitems == 0) return;
    const int resident = oz_resident<S, WM, PERSIST>();
    const int grid = PERSIST ? std::min(nitems, ctx.sm_count * resident) : nitems;
    gemm_ozaki_kernel<S, WM, PERSIST><<<grid, 64 * WM, oz_smem_bytes<S, WM>(), ctx.stream>>>(
        items, nitems, p.d_pairs, p.d_cblk, p.d_ops, p.d_tab, panels, plane, exps, C);
}

// Clock budget of one mbarrier wait of the tensor-core kernel (about a second
// at full clock; ITG_TC_WAIT_LIMIT overrides it, e.g. to exercise the timeout
// path with a budget the MMAs cannot meet).
long long tc_wait_limit() {
    static const long long lim = [] {
        const char* e = std::getenv("ITG_TC_WAIT_LIMIT");
        return e ? std::max(0LL, std::atoll(e)) : 2000000000LL;
    }();
    return lim;
}

template <int S>
void launch_tc(Ctx& ctx, Plan const& p, double* C, __nv_bfloat16 const* panels, int64_t plane, int32_t const* exps) {
    if (p.nitems_tc == 0) return;
    using SH = TcShape<S, TC_TILE_N>;
    static const bool attr = [] {
        cudaFuncSetAttribute(gemm_ozaki_tc_kernel<S, TC_TILE_N>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)SH::SMEM);
        return true;
    }();
    (void)attr;
    // ITG_TC_TEST_STUCK_WAIT: every tile's first fold waits on a barrier nothing
    // arrives at, so the bounded wait runs out (tests of the ERR_TIMEOUT path)
    static const int stuck = std::getenv("ITG_TC_TEST_STUCK_WAIT") ? 1 : 0;
    gemm_ozaki_tc_kernel<S, TC_TILE_N><<<p.nitems_tc, 128, SH::SMEM, ctx.stream>>>(
        p.d_items_tc, p.d_pairs, p.d_cblk, p.d_ops, p.d_tab, panels, plane, exps, C, ctx.err_dev, tc_wait_limit(),
        stuck);
}

template <int S>
void launch_variant(Ctx& ctx, Plan const& p, int v, double* C, __nv_bfloat16 const* panels, int64_t plane,
                    int32_t const* exps) {
    switch (v) {
        case 4: launch_tc<S>(ctx, p, C, panels, plane, exps); break;
        case 1: launch_gemm<S, 4, false>(ctx, p, C, panels, plane, exps); break;
        case 2: launch_gemm<S, 2, true>(ctx, p, C, panels, plane, exps); break;
        case 3: launch_gemm<S, 4, true>(ctx, p, C, panels, plane, exps); break;
        default: launch_gemm<S, 2, false>(ctx, p, C, panels, plane, exps); break;
    }
}

template <int S>
void launch_s(Ctx& ctx, Plan const& p, double const* A, double const* B, double* C, __nv_bfloat16* panels,
              int64_t plane, int32_t* exps, bool prep_b, int variant) {
    // A items come first: without prep_b only A is sliced (B's panels are already in place)
    const int nprep = prep_b ? p.nprep : p.nprepA;
    if (nprep > 0)
        ozaki_prep_kernel<S><<<nprep, 256, 0, ctx.stream>>>(p.d_prep, p.d_ops, p.d_tab, A, B, panels, plane, exps);
    launch_variant<S>(ctx, p, variant, C, panels, plane, exps);
}
}  // namespace

void launch_ozaki(Ctx& ctx, Plan const& p, double const* A, double const* B, double* C, int S,
                  __nv_bfloat16* panels, int32_t* exps, bool prep_b) {
    const int64_t plane = (p.panel_elems + 15) / 16 * 16;
    const int v = ctx.gemm_variant >= 0 ? ctx.gemm_variant : std::max(0, p.oz_variant.load(std::memory_order_relaxed));
    switch (S) {
        case 3: launch_s<3>(ctx, p, A, B, C, panels, plane, exps, prep_b, v); break;
        case 4: launch_s<4>(ctx, p, A, B, C, panels, plane, exps, prep_b, v); break;
        case 5: launch_s<5>(ctx, p, A, B, C, panels, plane, exps, prep_b, v); break;
        default: launch_s<6>(ctx, p, A, B, C, panels, plane, exps, prep_b, v); break;
    }
    ITG_CHECK_CUDA(cudaGetLastError());
}

// Tile-shape autotuner: slices both operands once, then times every variant
// (32 x 32 or 64 x 32 tiles; one CTA per tile or persistent CTAs) on the
// plan's own data with CUDA events and keeps the fastest in the plan. The
// variants give bit-identical results, so tuning changes only the time.
int autotune_ozaki(Ctx& ctx, Plan const& p, double const* A, double const* B, double* C, int S,
                   __nv_bfloat16* panels, int32_t* exps) {
    const int64_t plane = (p.panel_elems + 15) / 16 * 16;
    auto prep = [&] {
        if (p.nprep == 0) return;
        switch (S) {
            case 3: ozaki_prep_kernel<3><<<p.nprep, 256, 0, ctx.stream>>>(p.d_prep, p.d_ops, p.d_tab, A, B, panels, plane, exps); break;
            case 4: ozaki_prep_kernel<4><<<p.nprep, 256, 0, ctx.stream>>>(p.d_prep, p.d_ops, p.d_tab, A, B, panels, plane, exps); break;
            case 5: ozaki_prep_kernel<5><<<p.nprep, 256, 0, ctx.stream>>>(p.d_prep, p.d_ops, p.d_tab, A, B, panels, plane, exps); break;
            default: ozaki_prep_kernel<6><<<p.nprep, 256, 0, ctx.stream>>>(p.d_prep, p.d_ops, p.d_tab, A, B, panels, plane, exps); break;
        }
    };
    auto run = [&](int v) {
        switch (S) {
            case 3: launch_variant<3>(ctx, p, v, C, panels, plane, exps); break;
            case 4: launch_variant<4>(ctx, p, v, C, panels, plane, exps); break;
            case 5: launch_variant<5>(ctx, p, v, C, panels, plane, exps); break;
            default: launch_variant<6>(ctx, p, v, C, panels, plane, exps); break;
        }
    };
    prep();
    constexpr int NV = 4, REPS = 3;
    cudaEvent_t ev[NV][2];
    for (int v = 0; v < NV; ++v)
        for (int k = 0; k < 2; ++k) ITG_CHECK_CUDA(cudaEventCreate(&ev[v][k]));
    for (int v = 0; v < NV; ++v) {
        run(v);  // warm
        ITG_CHECK_CUDA(cudaEventRecord(ev[v][0], ctx.stream));
        for (int r = 0; r < REPS; ++r) run(v);
        ITG_CHECK_CUDA(cudaEventRecord(ev[v][1], ctx.stream));
    }
    ITG_CHECK_CUDA(cudaGetLastError());
    ctx.kernel_launches += 1 + NV * (REPS + 1);
    ctx.sync();
    int best = 0;
    float best_ms = 0;
    for (int v = 0; v < NV; ++v) {
        float ms = 0;
        ITG_CHECK_CUDA(cudaEventElapsedTime(&ms, ev[v][0], ev[v][1]));
        if (v == 0 || ms < best_ms) { best = v; best_ms = ms; }
    }
    if (std::getenv("ITG_TUNE_LOG")) {
        std::fprintf(stderr, "itg autotune: %d tiles, %.3g flops:", p.nitems, p.flops);
        for (int v = 0; v < NV; ++v) {
            float ms = 0;
            cudaEventElapsedTime(&ms, ev[v][0], ev[v][1]);
            std::fprintf(stderr, " v%d %.1f us", v, 1e3 * ms / REPS);
        }
        std::fprintf(stderr, " -> v%d\n", best);
    }
    for (int v = 0; v < NV; ++v)
        for (int k = 0; k < 2; ++k) cudaEventDestroy(ev[v][k]);
    p.oz_variant.store(best, std::memory_order_relaxed);
    return best;
}

}  // namespace itg
