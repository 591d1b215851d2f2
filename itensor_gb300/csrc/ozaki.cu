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
//       writes the row exponents and the S digit planes, tiled (see
//       OpBlockRec in engine.h), K padded to 16.
// gemm: mma.sync variants: output tiles of 32 x 32 (4 warps of 16 x 16) or
//       64 x 32 (8 warps), one CTA per tile or persistent CTAs over the tile
//       list; digit panels staged with cp.async into a two-stage shared-memory
//       ring and read with ldmatrix. tcgen05 variant: ozaki_tc.cuh. The
//       variant is chosen per plan by autotune_ozaki.
#include "engine.h"
#include <cuda_bf16.h>
#include <algorithm>
#include <cstdio>
#include <cstdlib>

namespace itg {

__device__ __forceinline__ int exp_field(double x) {
    return (int)((__double_as_longlong(x) >> 52) & 0x7FF);
}

// The S balanced digits of x against the row exponent field emax (BF16-exact
// integers): d_1..d_{S-1} in [-64, 63], d_0 in [-128, 128].
template <int S>
__device__ __forceinline__ void oz_digit_vals(double x, int emax, int (&dig)[S]) {
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
    // balanced digits: their signs are independent of the entry's sign, so the
    // digit products left out (s + t >= S) average to zero instead of always
    // shrinking |x y|
    long long X = bits < 0 ? -(long long)Xf : (long long)Xf;
#pragma unroll
    for (int s = S - 1; s >= 1; --s) {
        const long long d = ((X + 64) & 127) - 64;
        dig[s] = (int)d;
        X = (X - d) >> 7;
    }
    dig[0] = (int)X;
}

// One CTA (8 warps) per item of up to 8 rows: one row group of the tiled
// panel, whole rows so that the row exponents are complete. First warp w
// finds row w's exponent (lanes stride over k, then a shuffle max). Then the
// warps share out the k-steps: per k-step of 16 the row group's 128 entries
// of the tiled panel (two 8 x 8 core matrices) are one contiguous run per
// digit plane; lane l computes entries 4l..4l+3 (row (l/2) mod 8, k = 8 (l/16)
// + 4 (l mod 2) ..+3) and writes their digits as one 8-byte store per plane,
// so a warp writes 256 contiguous bytes per plane. Rows past the block's end
// get zero digits.
// The column offsets of a chunk of PREP_KCHUNK contracted positions are looked
// up once per CTA into shared memory (a table lookup can take an integer
// division), then read by both passes.
constexpr int PREP_KCHUNK = 1024;

template <int S>
__device__ __forceinline__ void prep_item(PrepItem const& pi, const OpBlockRec* __restrict__ ops,
                                          const int32_t* __restrict__ tab, const double* __restrict__ A,
                                          const double* __restrict__ B, __nv_bfloat16* __restrict__ panels,
                                          int64_t plane, int32_t* __restrict__ exps) {
    __shared__ int rexp[8];
    __shared__ int32_t coff[PREP_KCHUNK];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const OpBlockRec ob = ops[pi.op];
    const double* __restrict__ base = (pi.which ? B : A) + ob.src;
    auto load_offsets = [&](int kc) {
        const int kn = min(PREP_KCHUNK, ob.K - kc);
        __syncthreads();  // the previous chunk's readers are done
        for (int j = threadIdx.x; j < kn; j += blockDim.x) coff[j] = tab_at(tab, ob.tcol, kc + j);
        __syncthreads();
        return kn;
    };
    // row exponents: warp w takes row r0 + w
    {
        const int r = pi.r0 + warp;
        const int32_t ro = r < pi.r1 ? tab_at(tab, ob.trow, r) : 0;
        int emax = 0;
        for (int kc = 0; kc < ob.K; kc += PREP_KCHUNK) {
            const int kn = load_offsets(kc);
            if (r < pi.r1)
                for (int j = lane; j < kn; j += 32) emax = max(emax, exp_field(base[ro + coff[j]]));
        }
        emax = __reduce_max_sync(0xffffffffu, emax);
        if (lane == 0) {
            rexp[warp] = emax;
            if (r < pi.r1) exps[ob.exp + r] = emax - 1022;  // |x| < 2^(E-1022)
        }
    }
    __syncthreads();
    // digits, one 128-entry run per k-step and plane
    const int row = (lane >> 1) & 7, kq = (lane >> 4) * 8 + (lane & 1) * 4;
    const int er = rexp[row];
    const int rr = pi.r0 + row;
    const bool rrv = rr < pi.r1;
    const int32_t ro = rrv ? tab_at(tab, ob.trow, rr) : 0;
    const int nrg = panel_row_groups(ob.rows);
    __nv_bfloat16* dst0 = panels + ob.panel + (int64_t)(pi.r0 >> 3) * 128 + lane * 4;
    int kc = 0;  // first position of the chunk of offsets in shared memory
    for (int kb = 0; kb < ob.Kp; kb += PREP_KCHUNK) {
        // k-steps of this chunk: [kb, kb + PREP_KCHUNK) (a multiple of 16)
        if (kb < ob.K) {
            kc = kb;
            load_offsets(kc);
        }
        const int ks_end = min(ob.Kp, kb + PREP_KCHUNK) / 16;
        for (int ks = kb / 16 + warp; ks < ks_end; ks += 8) {
            int dig[4][S];
#pragma unroll
            for (int i = 0; i < 4; ++i) {
                const int k = ks * 16 + kq + i;
                oz_digit_vals<S>((rrv && k < ob.K) ? base[ro + coff[k - kc]] : 0.0, er, dig[i]);
            }
            __nv_bfloat16* dst = dst0 + (int64_t)ks * nrg * 128;
#pragma unroll
            for (int s = 0; s < S; ++s) {
                __nv_bfloat162 lo = __floats2bfloat162_rn((float)dig[0][s], (float)dig[1][s]);
                __nv_bfloat162 hi = __floats2bfloat162_rn((float)dig[2][s], (float)dig[3][s]);
                uint2 v;
                v.x = *reinterpret_cast<uint32_t*>(&lo);
                v.y = *reinterpret_cast<uint32_t*>(&hi);
                *reinterpret_cast<uint2*>(dst + s * plane) = v;
            }
        }
    }
}

template <int S>
__global__ void __launch_bounds__(256) ozaki_prep_kernel(const PrepItem* __restrict__ items, int nitems,
                                                         const OpBlockRec* __restrict__ ops,
                                                         const int32_t* __restrict__ tab, const double* __restrict__ A,
                                                         const double* __restrict__ B, __nv_bfloat16* __restrict__ panels,
                                                         int64_t plane, int32_t* __restrict__ exps) {
    pdl_wait();
    prep_item<S>(items[blockIdx.x], ops, tab, A, B, panels, plane, exps);
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
                    const __nv_bfloat16* src =
                        ok ? pa + s * plane + panel_off(it.m0 + row, k0 + half * 8, panel_row_groups(oa.rows)) : pa;
                    cp_async16(&As[buf][s][row][half * 8], src, ok);
                } else {
                    const int row = (r2 - S * TM) % TN, s = (r2 - S * TM) / TN;
                    const bool ok = it.n0 + row < cb.N;
                    const __nv_bfloat16* src =
                        ok ? pb + s * plane + panel_off(it.n0 + row, k0 + half * 8, panel_row_groups(ob.rows)) : pb;
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
    pdl_wait();
    extern __shared__ __align__(16) unsigned char oz_smem[];
    if (PERSIST) {
        for (int i = blockIdx.x; i < nitems; i += gridDim.x)
            oz_tile<S, WM>(items[i], pairs, cblk, ops, tab, panels, plane, exps, C, oz_smem);
    } else {
        oz_tile<S, WM>(items[blockIdx.x], pairs, cblk, ops, tab, panels, plane, exps, C, oz_smem);
    }
}

// ---------------------------------------------------------------- grouped launches
// Split-precision contractions of several independent solves in one launch
// (the solver pool's cross-solve grouping): the grid covers the prep items,
// or the 32 x 32 output tiles, of every contraction in the group; a CTA finds
// its contraction by binary search over the prefix positions and runs the
// same per-item code as a lone launch, so every output is bit-identical to it.
__device__ __forceinline__ int group_of(const GroupRef* __restrict__ refs, int nrefs, int b, bool tiles) {
    int lo = 0, hi = nrefs - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) / 2;
        if ((tiles ? refs[mid].tile_start : refs[mid].prep_start) <= b) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

template <int S>
__global__ void __launch_bounds__(256) ozaki_prep_group_kernel(const GroupRef* __restrict__ refs, int nrefs) {
    const GroupRef& g = refs[group_of(refs, nrefs, blockIdx.x, false)];
    prep_item<S>(g.prep[blockIdx.x - g.prep_start], g.ops, g.tab, g.A, g.B, g.panels, g.plane, g.exps);
}

template <int S>
__global__ void __launch_bounds__(128, 4) gemm_ozaki_group_kernel(const GroupRef* __restrict__ refs, int nrefs) {
    extern __shared__ __align__(16) unsigned char oz_smem[];
    const GroupRef& g = refs[group_of(refs, nrefs, blockIdx.x, true)];
    oz_tile<S, 2>(g.items[blockIdx.x - g.tile_start], g.pairs, g.cblk, g.ops, g.tab, g.panels, g.plane, g.exps, g.C,
                  oz_smem);
}

void launch_ozaki_group(cudaStream_t stream, GroupRef const* refs, int nrefs, int total_prep, int total_tiles, int S) {
    auto go = [&](auto prep, auto gemm, size_t smem) {
        if (total_prep > 0) prep<<<total_prep, 256, 0, stream>>>(refs, nrefs);
        if (total_tiles > 0) {
            static const bool attr = [&] {
                cudaFuncSetAttribute(gemm, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
                return true;
            }();
            (void)attr;
            gemm<<<total_tiles, 128, smem, stream>>>(refs, nrefs);
        }
    };
    switch (S) {
        case 3: go(ozaki_prep_group_kernel<3>, gemm_ozaki_group_kernel<3>, oz_smem_bytes<3, 2>()); break;
        case 4: go(ozaki_prep_group_kernel<4>, gemm_ozaki_group_kernel<4>, oz_smem_bytes<4, 2>()); break;
        case 5: go(ozaki_prep_group_kernel<5>, gemm_ozaki_group_kernel<5>, oz_smem_bytes<5, 2>()); break;
        default: go(ozaki_prep_group_kernel<6>, gemm_ozaki_group_kernel<6>, oz_smem_bytes<6, 2>()); break;
    }
    ITG_CHECK_CUDA(cudaGetLastError());
}

// ---------------------------------------------------------------- tensor-core (tcgen05) variant
#include "ozaki_tc.cuh"

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
    launch_pdl(ctx, grid, 64 * WM, oz_smem_bytes<S, WM>(), gemm_ozaki_kernel<S, WM, PERSIST>,
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
    // ITG_TC_TEST_STUCK_WAIT: the epilogue's first wait is on a barrier nothing
    // arrives at, so the bounded wait runs out (tests of the ERR_TIMEOUT path)
    static const int stuck = std::getenv("ITG_TC_TEST_STUCK_WAIT") ? 1 : 0;
    const int grid = std::min(p.nitems_tc, ctx.sm_count);  // persistent: one CTA per SM
    launch_pdl(ctx, grid, SH::THREADS, SH::SMEM, gemm_ozaki_tc_kernel<S, TC_TILE_N>, p.d_items_tc, p.nitems_tc,
               p.d_pairs_tc, p.d_tab, panels, plane, exps, C, ctx.err_dev, tc_wait_limit(), stuck);
}

template <int S>
void launch_variant(Ctx& ctx, Plan const& p, int v, double* C, __nv_bfloat16 const* panels, int64_t plane,
                    int32_t const* exps) {
    if (v == 1 || v == 3 || v == 4) ensure_variant_tables(ctx, p);  // 64-row or tcgen05 tiles
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
        launch_pdl(ctx, nprep, 256, 0, ozaki_prep_kernel<S>, p.d_prep, nprep, p.d_ops, p.d_tab, A, B, panels, plane, exps);
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
            case 3: ozaki_prep_kernel<3><<<p.nprep, 256, 0, ctx.stream>>>(p.d_prep, p.nprep, p.d_ops, p.d_tab, A, B, panels, plane, exps); break;
            case 4: ozaki_prep_kernel<4><<<p.nprep, 256, 0, ctx.stream>>>(p.d_prep, p.nprep, p.d_ops, p.d_tab, A, B, panels, plane, exps); break;
            case 5: ozaki_prep_kernel<5><<<p.nprep, 256, 0, ctx.stream>>>(p.d_prep, p.nprep, p.d_ops, p.d_tab, A, B, panels, plane, exps); break;
            default: ozaki_prep_kernel<6><<<p.nprep, 256, 0, ctx.stream>>>(p.d_prep, p.nprep, p.d_ops, p.d_tab, A, B, panels, plane, exps); break;
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
    constexpr int NV = 5, REPS = 3;  // 4: the tensor-core (tcgen05) kernel
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
