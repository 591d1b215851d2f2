// Block-sparse contraction on sm_103a: device planner + grouped block GEMMs.
//
// Planner (one CTA): reproduces getContractedOffsets (itensor/itdata/qutil.h:93-242)
// bit-exactly. A blocks are ranked by their uncontracted coordinates, B blocks by
// theirs; candidate pairs are enumerated in (B-group, A, B) order, which is already
// the reversed-lexicographic order of the output block, so matching, compaction,
// deduplication and the offset prefix sum are three block-wide scans -- no sort
// of the pair list is needed.
//
// GEMMs: every output tile walks the pairs feeding its block. Operands are read
// through per-block offset tables (offset(m,k) = T_m[m] + T_k[k]), so arbitrary
// index permutations cost nothing extra and no permuted copy is ever formed.
#include "engine.h"
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cuda_bf16.h>
#include <algorithm>
#include <cstring>
#include <numeric>
#include <unordered_set>

namespace itg {

// ------------------------------------------------------------------ block scan
__device__ __forceinline__ int block_excl_scan(int v, int* total, int* sh_warp) {
    int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) sh_warp[warp] = x;
    __syncthreads();
    int nw = blockDim.x >> 5;
    if (warp == 0) {
        int w = lane < nw ? sh_warp[lane] : 0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            int y = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w += y;
        }
        if (lane < nw) sh_warp[lane] = w;  // inclusive warp prefix
    }
    __syncthreads();
    int before = warp ? sh_warp[warp - 1] : 0;
    *total = sh_warp[nw - 1];
    __syncthreads();
    return before + x - v;
}

struct PlanArgs {
    int nA, nB, rA, rB, ncon, nau, nbu;
    const int32_t* Acoords;
    const int32_t* Bcoords;
    const int32_t* pos;     // [acon(ncon) | bcon(ncon) | aunc(nau) | bunc(nbu)]
    const int32_t* bits;    // bit widths: [con(ncon) | aunc(nau) | bunc(nbu)]
    const int32_t* cdims;   // C natural-order sector dims, concatenated
    const int32_t* cdstart; // start of each C index in cdims
    // scratch (device)
    uint64_t* keyA; uint64_t* keyB; uint64_t* conA; uint64_t* conB;
    int32_t* sortA; int32_t* sortB; int32_t* gstart; uint64_t* pkey;
    // outputs (host-mapped)
    int32_t* out_counts;    // [npairs, nC, overflow]
    int32_t* pair_a; int32_t* pair_b; int32_t* pair_c;
    int32_t* c_coords;      // nC * (nau+nbu)
    int64_t* c_off;         // nC + 1 (last = total size)
    int cap_pairs, cap_c;
};

__device__ uint64_t pack_key(const int32_t* c, const int32_t* pos, const int32_t* bits, int n) {
    uint64_t k = 0;
    int sh = 0;
    for (int i = 0; i < n; ++i) {
        k |= (uint64_t)(uint32_t)c[pos[i]] << sh;
        sh += bits[i];
    }
    return k;
}

__global__ void __launch_bounds__(1024) plan_kernel(PlanArgs a) {
    __shared__ int sh_warp[32];
    __shared__ int sh_ngroups;
    const int tid = threadIdx.x, nt = blockDim.x;
    const int32_t* acon = a.pos;
    const int32_t* bcon = a.pos + a.ncon;
    const int32_t* aunc = a.pos + 2 * a.ncon;
    const int32_t* bunc = aunc + a.nau;
    const int32_t* bcon_bits = a.bits;
    const int32_t* aunc_bits = a.bits + a.ncon;
    const int32_t* bunc_bits = aunc_bits + a.nau;
    int bitsA = 0;
    for (int i = 0; i < a.nau; ++i) bitsA += aunc_bits[i];
    // 1. keys
    for (int i = tid; i < a.nA; i += nt) {
        const int32_t* c = a.Acoords + (size_t)i * a.rA;
        a.keyA[i] = pack_key(c, aunc, aunc_bits, a.nau);
        a.conA[i] = pack_key(c, acon, bcon_bits, a.ncon);
    }
    for (int j = tid; j < a.nB; j += nt) {
        const int32_t* c = a.Bcoords + (size_t)j * a.rB;
        a.keyB[j] = pack_key(c, bunc, bunc_bits, a.nbu);
        a.conB[j] = pack_key(c, bcon, bcon_bits, a.ncon);
    }
    __syncthreads();
    // 2. rank sorts (stable by original position)
    for (int i = tid; i < a.nA; i += nt) {
        uint64_t k = a.keyA[i];
        int r = 0;
        for (int j = 0; j < a.nA; ++j) {
            uint64_t kj = a.keyA[j];
            r += (kj < k) || (kj == k && j < i);
        }
        a.sortA[r] = i;
    }
    for (int i = tid; i < a.nB; i += nt) {
        uint64_t k = a.keyB[i];
        int r = 0;
        for (int j = 0; j < a.nB; ++j) {
            uint64_t kj = a.keyB[j];
            r += (kj < k) || (kj == k && j < i);
        }
        a.sortB[r] = i;
    }
    __syncthreads();
    // 3. groups of equal B keys among sorted B
    int base = 0;
    for (int s0 = 0; s0 < a.nB; s0 += nt) {
        int s = s0 + tid;
        int f = 0;
        if (s < a.nB) f = (s == 0) || (a.keyB[a.sortB[s]] != a.keyB[a.sortB[s - 1]]);
        int tot;
        int ex = block_excl_scan(f, &tot, sh_warp);
        if (f) a.gstart[base + ex] = s;
        base += tot;
    }
    if (tid == 0) { a.gstart[base] = a.nB; sh_ngroups = base; }
    __syncthreads();
    const int ng = sh_ngroups;
    // 4. candidates in (group, sorted A, B in group) order; compact the matches
    const long long total = (long long)a.nA * a.nB;
    int np = 0;
    bool overflow = false;
    for (long long t0 = 0; t0 < total; t0 += nt) {
        long long t = t0 + tid;
        int f = 0, ia = -1, jb = -1;
        if (t < total) {
            int lo = 0, hi = ng - 1;  // last group g with nA*gstart[g] <= t
            while (lo < hi) {
                int mid = (lo + hi + 1) >> 1;
                if ((long long)a.nA * a.gstart[mid] <= t) lo = mid;
                else hi = mid - 1;
            }
            int g = lo;
            int gs = a.gstart[g], sz = a.gstart[g + 1] - gs;
            long long local = t - (long long)a.nA * gs;
            ia = a.sortA[local / sz];
            jb = a.sortB[gs + (int)(local % sz)];
            f = a.conA[ia] == a.conB[jb];
        }
        int tot;
        int ex = block_excl_scan(f, &tot, sh_warp);
        if (f) {
            int p = np + ex;
            if (p < a.cap_pairs) {
                a.pair_a[p] = ia;
                a.pair_b[p] = jb;
                a.pkey[p] = a.keyA[ia] | (a.keyB[jb] << bitsA);
            }
        }
        np += tot;
    }
    if (np > a.cap_pairs) overflow = true;
    __syncthreads();
    // 5. output blocks: boundaries of equal keys, coordinates and sizes
    int nc = 0;
    const int rC = a.nau + a.nbu;
    if (!overflow) {
        for (int p0 = 0; p0 < np; p0 += nt) {
            int p = p0 + tid;
            int f = 0;
            if (p < np) f = (p == 0) || (a.pkey[p] != a.pkey[p - 1]);
            int tot;
            int ex = block_excl_scan(f, &tot, sh_warp);
            __syncthreads();
            if (p < np) {
                // C index of this pair: blocks before it = nc + (inclusive count) - 1
                a.pair_c[p] = nc + ex + f - 1;
            }
            if (f && nc + ex < a.cap_c) {
                int c = nc + ex;
                const int32_t* ca = a.Acoords + (size_t)a.pair_a[p] * a.rA;
                const int32_t* cb = a.Bcoords + (size_t)a.pair_b[p] * a.rB;
                int64_t size = 1;
                for (int i = 0; i < a.nau; ++i) {
                    int s = ca[aunc[i]];
                    a.c_coords[(size_t)c * rC + i] = s;
                    size *= a.cdims[a.cdstart[i] + s];
                }
                for (int i = 0; i < a.nbu; ++i) {
                    int s = cb[bunc[i]];
                    a.c_coords[(size_t)c * rC + a.nau + i] = s;
                    size *= a.cdims[a.cdstart[a.nau + i] + s];
                }
                a.c_off[c] = size;
            }
            nc += tot;
        }
        // fix pair_c of pairs whose block started in an earlier chunk: pair_c from
        // the scan above is exact because nc carries across chunks.
    }
    if (nc > a.cap_c) overflow = true;
    __syncthreads();
    // 6. offsets = exclusive prefix sum of block sizes (serial over chunks, 64-bit)
    if (!overflow) {
        __shared__ long long sh_carry;
        if (tid == 0) sh_carry = 0;
        __syncthreads();
        for (int c0 = 0; c0 < nc; c0 += nt) {
            int c = c0 + tid;
            long long v = (c < nc) ? a.c_off[c] : 0;
            // 64-bit inclusive scan via warp shuffles + shared warp sums
            long long x = v;
            int lane = tid & 31, warp = tid >> 5;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                long long y = __shfl_up_sync(0xffffffffu, x, o);
                if (lane >= o) x += y;
            }
            __shared__ long long sw[32];
            if (lane == 31) sw[warp] = x;
            __syncthreads();
            if (warp == 0) {
                long long w = lane < (nt >> 5) ? sw[lane] : 0;
#pragma unroll
                for (int o = 1; o < 32; o <<= 1) {
                    long long y = __shfl_up_sync(0xffffffffu, w, o);
                    if (lane >= o) w += y;
                }
                sw[lane] = w;
            }
            __syncthreads();
            long long incl = x + (warp ? sw[warp - 1] : 0);
            long long carry = sh_carry;
            __syncthreads();
            if (c < nc) a.c_off[c] = carry + incl - v;
            if (tid == nt - 1) sh_carry = carry + incl;
            __syncthreads();
        }
        if (tid == 0) a.c_off[nc] = sh_carry;
    }
    if (tid == 0) {
        a.out_counts[0] = np;
        a.out_counts[1] = nc;
        a.out_counts[2] = overflow ? 1 : 0;
    }
}

// ------------------------------------------------------------------ FP64 block GEMM
// One CTA per 32x32 output tile; 256 threads, 2x2 outputs each. Warps own
// output columns, so warps whose columns lie outside a narrow block skip the
// FMA loop entirely (FP64 issue slots are the bound on this part).
__device__ __forceinline__ void f64_tile(ItemRec const& it, const PairRec* __restrict__ pairs,
                                         const CBlockRec* __restrict__ cblk, const int32_t* __restrict__ tab,
                                         const double* __restrict__ A, const double* __restrict__ B,
                                         double* __restrict__ C) {
    constexpr int T = GEMM_TILE, TK = 16;
    __shared__ double As[TK][T + 1];
    __shared__ double Bs[TK][T + 1];
    __shared__ int32_t rowA[T], colB[T], kA[TK], kB[TK];   // this tile's offsets
    const CBlockRec cb = cblk[it.c];
    const int tid = threadIdx.x;
    const int tx = tid & 15, ty = tid >> 4;     // rows tx*2+{0,1}, cols ty*2+{0,1}
    const int warp_col0 = (tid >> 5) * 4;       // first column touched by this warp
    const bool warp_active = it.n0 + warp_col0 < cb.N;
    double acc00 = 0, acc01 = 0, acc10 = 0, acc11 = 0;
    for (int p = it.p0; p < it.p1; ++p) {
        const PairRec pr = pairs[p];
        if (tid < T) {
            const int m = it.m0 + tid, n = it.n0 + tid;
            rowA[tid] = m < cb.M ? tab_at(tab, pr.tam, m) : 0;
            colB[tid] = n < cb.N ? tab_at(tab, pr.tbn, n) : 0;
        }
        for (int k0 = 0; k0 < pr.K; k0 += TK) {
            if (tid >= 64 && tid < 64 + TK) {
                const int k = k0 + tid - 64;
                kA[tid - 64] = k < pr.K ? tab_at(tab, pr.tak, k) : 0;
                kB[tid - 64] = k < pr.K ? tab_at(tab, pr.tbk, k) : 0;
            }
            __syncthreads();
            for (int e = tid; e < TK * T; e += 256) {
                int i = e % T, kk = e / T;
                int m = it.m0 + i, k = k0 + kk;
                As[kk][i] = (m < cb.M && k < pr.K) ? A[pr.aoff + rowA[i] + kA[kk]] : 0.0;
                int n = it.n0 + i;
                Bs[kk][i] = (n < cb.N && k < pr.K) ? B[pr.boff + kB[kk] + colB[i]] : 0.0;
            }
            __syncthreads();
            if (warp_active) {
                const int kmax = min(TK, pr.K - k0);
                for (int kk = 0; kk < kmax; ++kk) {
                    double a0 = As[kk][tx * 2], a1 = As[kk][tx * 2 + 1];
                    double b0 = Bs[kk][ty * 2], b1 = Bs[kk][ty * 2 + 1];
                    acc00 = fma(a0, b0, acc00);
                    acc01 = fma(a0, b1, acc01);
                    acc10 = fma(a1, b0, acc10);
                    acc11 = fma(a1, b1, acc11);
                }
            }
            __syncthreads();
        }
    }
    const int m = it.m0 + tx * 2, n = it.n0 + ty * 2;
    double accs[2][2] = {{acc00, acc01}, {acc10, acc11}};
#pragma unroll
    for (int r = 0; r < 2; ++r)
#pragma unroll
        for (int s = 0; s < 2; ++s)
            if (m + r < cb.M && n + s < cb.N) C[cb.coff + tab_at(tab, cb.tcm, m + r) + tab_at(tab, cb.tcn, n + s)] = accs[r][s];
}

__global__ void __launch_bounds__(256) gemm_f64_kernel(const ItemRec* __restrict__ items,
                                                       const PairRec* __restrict__ pairs,
                                                       const CBlockRec* __restrict__ cblk,
                                                       const int32_t* __restrict__ tab,
                                                       const double* __restrict__ A,
                                                       const double* __restrict__ B,
                                                       double* __restrict__ C) {
    pdl_wait();
    f64_tile(items[blockIdx.x], pairs, cblk, tab, A, B, C);
}

// FP64 contractions of several independent solves in one launch (the solver
// pool's cross-solve grouping): a CTA finds its contraction by binary search
// over the tile prefix positions and runs the lone launch's tile code.
__global__ void __launch_bounds__(256) gemm_f64_group_kernel(const GroupRef* __restrict__ refs, int nrefs) {
    int lo = 0, hi = nrefs - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) / 2;
        if (refs[mid].tile_start <= (int)blockIdx.x) lo = mid;
        else hi = mid - 1;
    }
    const GroupRef& g = refs[lo];
    f64_tile(g.items[blockIdx.x - g.tile_start], g.pairs, g.cblk, g.tab, g.A, g.B, g.C);
}

void launch_f64_group(cudaStream_t stream, GroupRef const* refs, int nrefs, int total_tiles) {
    if (total_tiles > 0) gemm_f64_group_kernel<<<total_tiles, 256, 0, stream>>>(refs, nrefs);
    ITG_CHECK_CUDA(cudaGetLastError());
}

// ------------------------------------------------------------------ skinny FP64 block GEMM
// b != 0 (either sign of zero excluded) tested on the bit pattern: an FP64
// compare issues on the FP64 pipe, which bounds these kernels.
__device__ __forceinline__ bool nonzero_bits(double b) {
    return (__double_as_longlong(b) & 0x7FFFFFFFFFFFFFFFll) != 0;
}

// For contractions whose output blocks are at most SKINNY_N columns wide (the
// MPO-tensor steps of the H_eff apply: N = (s', w') <= 3, K = (s, w) <= 3).
// One thread per output row keeps all N sums in registers; the B block
// (K x N) is staged in shared memory. Tiles are 256 * R rows of one block.
constexpr int SKINNY_N = 8, SKINNY_THREADS = 256, SKINNY_K = 64;

// NN = exact output width of the block (1..SKINNY_N). Rows m0 + t + j*256,
// j < R, per thread; R (1, 2 or 4) is chosen per plan so that small
// contractions still spread over the SMs (FP64 issue slots bound this step:
// about two FP64 FMA per clock per SM). Zero entries of the staged B block are
// skipped with a branch that is uniform over the CTA (MPO-tensor blocks are
// mostly zeros).
template <int NN, int R>
__device__ __forceinline__ void skinny_item(ItemRec const& it, CBlockRec const& cb, const PairRec* __restrict__ pairs,
                                            const int32_t* __restrict__ tab, const double* __restrict__ A,
                                            const double* __restrict__ B, double* __restrict__ C,
                                            double (*Bs)[SKINNY_N]) {
    double acc[R][NN];
#pragma unroll
    for (int j = 0; j < R; ++j)
#pragma unroll
        for (int n = 0; n < NN; ++n) acc[j][n] = 0.0;
    int mrow[R];
#pragma unroll
    for (int j = 0; j < R; ++j) mrow[j] = it.m0 + threadIdx.x + j * SKINNY_THREADS;
    // row sets whose whole warp lies past the block's end skip their FMAs (a
    // warp-uniform branch: FP64 issue slots bound this kernel)
    bool wlive[R];
#pragma unroll
    for (int j = 0; j < R; ++j) wlive[j] = it.m0 + (int)(threadIdx.x & ~31u) + j * SKINNY_THREADS < cb.M;
    for (int p = it.p0; p < it.p1; ++p) {
        const PairRec pr = pairs[p];
        int arow[R];
#pragma unroll
        for (int j = 0; j < R; ++j) arow[j] = mrow[j] < cb.M ? tab_at(tab, pr.tam, mrow[j]) : -1;
        for (int k0 = 0; k0 < pr.K; k0 += SKINNY_K) {
            const int kn = min(SKINNY_K, pr.K - k0);
            __syncthreads();
            for (int e = threadIdx.x; e < kn * NN; e += blockDim.x) {
                int k = e / NN, n = e % NN;
                Bs[k][n] = B[pr.boff + tab_at(tab, pr.tbk, k0 + k) + tab_at(tab, pr.tbn, n)];
            }
            __syncthreads();
            for (int k = 0; k < kn; ++k) {
                const int ko = tab_at(tab, pr.tak, k0 + k);
                double a[R];
#pragma unroll
                for (int j = 0; j < R; ++j) a[j] = arow[j] >= 0 ? A[pr.aoff + arow[j] + ko] : 0.0;
#pragma unroll
                for (int n = 0; n < NN; ++n) {
                    const double b = Bs[k][n];
                    if (nonzero_bits(b)) {
#pragma unroll
                        for (int j = 0; j < R; ++j)
                            if (wlive[j]) acc[j][n] = fma(a[j], b, acc[j][n]);
                    }
                }
            }
        }
    }
#pragma unroll
    for (int j = 0; j < R; ++j) {
        if (mrow[j] < cb.M) {
            const int64_t crow = cb.coff + tab_at(tab, cb.tcm, mrow[j]);
#pragma unroll
            for (int n = 0; n < NN; ++n) C[crow + tab_at(tab, cb.tcn, n)] = acc[j][n];
        }
    }
}

// Barrier-free form for plans whose pairs all have K <= SKINNY_K: every thread
// reads the (tiny, L1-resident) B entries itself, the same addresses across
// the CTA, instead of staging each pair's block behind two barriers. Same FMA
// order per output as skinny_item.
template <int NN, int R>
__device__ __forceinline__ void skinny_item_direct(ItemRec const& it, CBlockRec const& cb,
                                                   const PairRec* __restrict__ pairs, const int32_t* __restrict__ tab,
                                                   const double* __restrict__ A, const double* __restrict__ B,
                                                   double* __restrict__ C) {
    double acc[R][NN];
#pragma unroll
    for (int j = 0; j < R; ++j)
#pragma unroll
        for (int n = 0; n < NN; ++n) acc[j][n] = 0.0;
    int mrow[R];
#pragma unroll
    for (int j = 0; j < R; ++j) mrow[j] = it.m0 + threadIdx.x + j * SKINNY_THREADS;
    // row sets whose whole warp lies past the block's end skip their FMAs (a
    // warp-uniform branch: FP64 issue slots bound this kernel)
    bool wlive[R];
#pragma unroll
    for (int j = 0; j < R; ++j) wlive[j] = it.m0 + (int)(threadIdx.x & ~31u) + j * SKINNY_THREADS < cb.M;
    int bcol[NN];
    for (int p = it.p0; p < it.p1; ++p) {
        const PairRec pr = pairs[p];
        int arow[R];
#pragma unroll
        for (int j = 0; j < R; ++j) arow[j] = mrow[j] < cb.M ? tab_at(tab, pr.tam, mrow[j]) : -1;
#pragma unroll
        for (int n = 0; n < NN; ++n) bcol[n] = tab_at(tab, pr.tbn, n);
        for (int k = 0; k < pr.K; ++k) {
            const int ko = tab_at(tab, pr.tak, k);
            const int64_t bk = pr.boff + tab_at(tab, pr.tbk, k);
            double a[R];
#pragma unroll
            for (int j = 0; j < R; ++j) a[j] = arow[j] >= 0 ? A[pr.aoff + arow[j] + ko] : 0.0;
#pragma unroll
            for (int n = 0; n < NN; ++n) {
                const double b = __ldg(B + bk + bcol[n]);
                if (nonzero_bits(b)) {
#pragma unroll
                    for (int j = 0; j < R; ++j)
                            if (wlive[j]) acc[j][n] = fma(a[j], b, acc[j][n]);
                }
            }
        }
    }
#pragma unroll
    for (int j = 0; j < R; ++j) {
        if (mrow[j] < cb.M) {
            const int64_t crow = cb.coff + tab_at(tab, cb.tcm, mrow[j]);
#pragma unroll
            for (int n = 0; n < NN; ++n) C[crow + tab_at(tab, cb.tcn, n)] = acc[j][n];
        }
    }
}

template <int R>
__global__ void __launch_bounds__(SKINNY_THREADS) gemm_f64_skinny_direct_kernel(const ItemRec* __restrict__ items,
                                                                                const PairRec* __restrict__ pairs,
                                                                                const CBlockRec* __restrict__ cblk,
                                                                                const int32_t* __restrict__ tab,
                                                                                const double* __restrict__ A,
                                                                                const double* __restrict__ B,
                                                                                double* __restrict__ C) {
    pdl_wait();
    const ItemRec it = items[blockIdx.x];
    const CBlockRec cb = cblk[it.c];
    switch (cb.N) {
        case 1: skinny_item_direct<1, R>(it, cb, pairs, tab, A, B, C); break;
        case 2: skinny_item_direct<2, R>(it, cb, pairs, tab, A, B, C); break;
        case 3: skinny_item_direct<3, R>(it, cb, pairs, tab, A, B, C); break;
        case 4: skinny_item_direct<4, R>(it, cb, pairs, tab, A, B, C); break;
        case 5: skinny_item_direct<5, R>(it, cb, pairs, tab, A, B, C); break;
        case 6: skinny_item_direct<6, R>(it, cb, pairs, tab, A, B, C); break;
        case 7: skinny_item_direct<7, R>(it, cb, pairs, tab, A, B, C); break;
        default: skinny_item_direct<8, R>(it, cb, pairs, tab, A, B, C); break;
    }
}

template <int R>
__global__ void __launch_bounds__(SKINNY_THREADS) gemm_f64_skinny_kernel(const ItemRec* __restrict__ items,
                                                                         const PairRec* __restrict__ pairs,
                                                                         const CBlockRec* __restrict__ cblk,
                                                                         const int32_t* __restrict__ tab,
                                                                         const double* __restrict__ A,
                                                                         const double* __restrict__ B,
                                                                         double* __restrict__ C) {
    pdl_wait();
    __shared__ double Bs[SKINNY_K][SKINNY_N];
    const ItemRec it = items[blockIdx.x];
    const CBlockRec cb = cblk[it.c];
    switch (cb.N) {
        case 1: skinny_item<1, R>(it, cb, pairs, tab, A, B, C, Bs); break;
        case 2: skinny_item<2, R>(it, cb, pairs, tab, A, B, C, Bs); break;
        case 3: skinny_item<3, R>(it, cb, pairs, tab, A, B, C, Bs); break;
        case 4: skinny_item<4, R>(it, cb, pairs, tab, A, B, C, Bs); break;
        case 5: skinny_item<5, R>(it, cb, pairs, tab, A, B, C, Bs); break;
        case 6: skinny_item<6, R>(it, cb, pairs, tab, A, B, C, Bs); break;
        case 7: skinny_item<7, R>(it, cb, pairs, tab, A, B, C, Bs); break;
        default: skinny_item<8, R>(it, cb, pairs, tab, A, B, C, Bs); break;
    }
}

// For skinny plans with few rows in all (too few 256-row tiles to fill the
// SMs): a CTA takes 32 rows of one output block, and its eight warps take
// every eighth block pair each (lane = row), so a thread's chain of dependent
// loads covers an eighth of the pairs. The eight partial sums of an output are
// added in warp order (deterministic).
constexpr int WIDE_ROWS = 32, WIDE_WARPS = SKINNY_THREADS / 32;

template <int NN>
__device__ __forceinline__ void skinny_item_wide(ItemRec const& it, CBlockRec const& cb,
                                                 const PairRec* __restrict__ pairs, const int32_t* __restrict__ tab,
                                                 const double* __restrict__ A, const double* __restrict__ B,
                                                 double* __restrict__ C, double (*part)[WIDE_ROWS][SKINNY_N]) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int m = it.m0 + lane;
    double acc[NN];
#pragma unroll
    for (int n = 0; n < NN; ++n) acc[n] = 0.0;
    if (m < cb.M) {
        for (int p = it.p0 + warp; p < it.p1; p += WIDE_WARPS) {
            const PairRec pr = pairs[p];
            const int arow = tab_at(tab, pr.tam, m);
            int bcol[NN];
#pragma unroll
            for (int n = 0; n < NN; ++n) bcol[n] = tab_at(tab, pr.tbn, n);
            for (int k = 0; k < pr.K; ++k) {
                const int ko = tab_at(tab, pr.tak, k);
                const int64_t bk = pr.boff + tab_at(tab, pr.tbk, k);
                const double a = A[pr.aoff + arow + ko];
#pragma unroll
                for (int n = 0; n < NN; ++n) {
                    const double b = __ldg(B + bk + bcol[n]);
                    if (nonzero_bits(b)) acc[n] = fma(a, b, acc[n]);
                }
            }
        }
    }
#pragma unroll
    for (int n = 0; n < NN; ++n) part[warp][lane][n] = acc[n];
    __syncthreads();
    // thread t sums output (row t % 32, column t / 32) over the warps in order
    const int row = threadIdx.x % WIDE_ROWS, n = threadIdx.x / WIDE_ROWS;
    if (n < NN && it.m0 + row < cb.M) {
        double v = part[0][row][n];
        for (int w = 1; w < WIDE_WARPS; ++w) v += part[w][row][n];
        C[cb.coff + tab_at(tab, cb.tcm, it.m0 + row) + tab_at(tab, cb.tcn, n)] = v;
    }
}

__global__ void __launch_bounds__(SKINNY_THREADS) gemm_f64_skinny_wide_kernel(const ItemRec* __restrict__ items,
                                                                              const PairRec* __restrict__ pairs,
                                                                              const CBlockRec* __restrict__ cblk,
                                                                              const int32_t* __restrict__ tab,
                                                                              const double* __restrict__ A,
                                                                              const double* __restrict__ B,
                                                                              double* __restrict__ C) {
    pdl_wait();
    __shared__ double part[WIDE_WARPS][WIDE_ROWS][SKINNY_N];
    const ItemRec it = items[blockIdx.x];
    const CBlockRec cb = cblk[it.c];
    switch (cb.N) {
        case 1: skinny_item_wide<1>(it, cb, pairs, tab, A, B, C, part); break;
        case 2: skinny_item_wide<2>(it, cb, pairs, tab, A, B, C, part); break;
        case 3: skinny_item_wide<3>(it, cb, pairs, tab, A, B, C, part); break;
        case 4: skinny_item_wide<4>(it, cb, pairs, tab, A, B, C, part); break;
        case 5: skinny_item_wide<5>(it, cb, pairs, tab, A, B, C, part); break;
        case 6: skinny_item_wide<6>(it, cb, pairs, tab, A, B, C, part); break;
        case 7: skinny_item_wide<7>(it, cb, pairs, tab, A, B, C, part); break;
        default: skinny_item_wide<8>(it, cb, pairs, tab, A, B, C, part); break;
    }
}

// Launches the skinny kernel with the plan's rows per thread.
static void launch_skinny(Ctx& ctx, Plan const& p, double const* A, double const* B, double* C) {
    if (p.skinny_wide) {
        launch_pdl(ctx, p.nitems, SKINNY_THREADS, 0, gemm_f64_skinny_wide_kernel, p.d_items, p.d_pairs, p.d_cblk,
                                                                                 p.d_tab, A, B, C);
        return;
    }
    if (p.max_pair_K <= SKINNY_K) {
        switch (p.skinny_r) {
            case 1:
                launch_pdl(ctx, p.nitems, SKINNY_THREADS, 0, gemm_f64_skinny_direct_kernel<1>, p.d_items, p.d_pairs, p.d_cblk,
                                                                                               p.d_tab, A, B, C);
                break;
            case 2:
                launch_pdl(ctx, p.nitems, SKINNY_THREADS, 0, gemm_f64_skinny_direct_kernel<2>, p.d_items, p.d_pairs, p.d_cblk,
                                                                                               p.d_tab, A, B, C);
                break;
            default:
                launch_pdl(ctx, p.nitems, SKINNY_THREADS, 0, gemm_f64_skinny_direct_kernel<4>, p.d_items, p.d_pairs, p.d_cblk,
                                                                                               p.d_tab, A, B, C);
                break;
        }
        return;
    }
    switch (p.skinny_r) {
        case 1:
            launch_pdl(ctx, p.nitems, SKINNY_THREADS, 0, gemm_f64_skinny_kernel<1>, p.d_items, p.d_pairs, p.d_cblk, p.d_tab, A, B, C);
            break;
        case 2:
            launch_pdl(ctx, p.nitems, SKINNY_THREADS, 0, gemm_f64_skinny_kernel<2>, p.d_items, p.d_pairs, p.d_cblk, p.d_tab, A, B, C);
            break;
        default:
            launch_pdl(ctx, p.nitems, SKINNY_THREADS, 0, gemm_f64_skinny_kernel<4>, p.d_items, p.d_pairs, p.d_cblk, p.d_tab, A, B, C);
            break;
    }
}

// The split-precision (Ozaki BF16) kernels live in ozaki.cu.

// ------------------------------------------------------------------ host side
namespace {
// live streams and their contexts' block caches: many readers, rare writers
std::shared_mutex g_streams_mu;
std::unordered_map<cudaStream_t, std::shared_ptr<BlockCache>>& live_streams() {
    static std::unordered_map<cudaStream_t, std::shared_ptr<BlockCache>> v;
    return v;
}
}  // namespace
void stream_register(cudaStream_t s, std::shared_ptr<BlockCache> cache) {
    std::unique_lock<std::shared_mutex> g(g_streams_mu);
    live_streams()[s] = std::move(cache);
}
void stream_unregister(cudaStream_t s) {
    std::unique_lock<std::shared_mutex> g(g_streams_mu);
    live_streams().erase(s);
}
bool stream_alive(cudaStream_t s) {
    std::shared_lock<std::shared_mutex> g(g_streams_mu);
    return live_streams().count(s) != 0;
}
std::shared_ptr<BlockCache> stream_cache(cudaStream_t s) {
    std::shared_lock<std::shared_mutex> g(g_streams_mu);
    auto it = live_streams().find(s);
    return it == live_streams().end() ? nullptr : it->second;
}
bool& cache_bypass() {
    thread_local bool bypass = false;
    return bypass;
}

double split_min_flops() {
    static const double v = [] {
        const char* e = std::getenv("ITG_SPLIT_MIN_FLOPS");
        return e ? std::max(0.0, std::atof(e)) : 1e7;
    }();
    return v;
}

Ctx::Ctx(int dev) : device(dev) {
    ITG_CHECK_CUDA(cudaSetDevice(dev));
    ITG_CHECK_CUDA(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
    cache = std::make_shared<BlockCache>(stream);
    stream_register(stream, cache);
    int sms = 0;
    ITG_CHECK_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    sm_count = sms;
    cudaMemPool_t pool;
    ITG_CHECK_CUDA(cudaDeviceGetDefaultMemPool(&pool, dev));
    uint64_t thr = UINT64_MAX;  // keep freed blocks cached in the pool
    ITG_CHECK_CUDA(cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr));
    ITG_CHECK_CUDA(cudaEventCreateWithFlags(&sync_event, cudaEventDisableTiming));
    // one pinned allocation: the status word, then the first deferred-read area
    // (pinning host memory takes the driver's lock; solver-pool contexts are
    // created while other solves launch)
    ITG_CHECK_CUDA(cudaHostAlloc(reinterpret_cast<void**>(&err_host), 64 + DEFER0, cudaHostAllocMapped));
    ITG_CHECK_CUDA(cudaHostGetDevicePointer(reinterpret_cast<void**>(&err_dev), err_host, 0));
    err_host[0] = 0;
    defer_host = reinterpret_cast<char*>(err_host) + 64;
    defer_bytes = DEFER0;
}

cudaStream_t Ctx::side_stream(int i) {
    if (!side[i]) {
        ITG_CHECK_CUDA(cudaStreamCreateWithFlags(&side[i], cudaStreamNonBlocking));
        ITG_CHECK_CUDA(cudaEventCreateWithFlags(&side_done[i], cudaEventDisableTiming));
    }
    return side[i];
}

void Ctx::fork() {
    if (!fork_event) ITG_CHECK_CUDA(cudaEventCreateWithFlags(&fork_event, cudaEventDisableTiming));
    ITG_CHECK_CUDA(cudaEventRecord(fork_event, stream));
    for (int i = 0; i < NSIDE; ++i) ITG_CHECK_CUDA(cudaStreamWaitEvent(side_stream(i), fork_event, 0));
}

void Ctx::join(int nused) {
    for (int i = 0; i < nused; ++i) {
        ITG_CHECK_CUDA(cudaEventRecord(side_done[i], side[i]));
        ITG_CHECK_CUDA(cudaStreamWaitEvent(stream, side_done[i], 0));
    }
}

Ctx::~Ctx() {
    if (stream) cudaStreamSynchronize(stream);
    for (int i = 0; i < NSIDE; ++i) {
        if (side[i]) { cudaStreamSynchronize(side[i]); cudaStreamDestroy(side[i]); }
        if (side_done[i]) cudaEventDestroy(side_done[i]);
    }
    if (fork_event) cudaEventDestroy(fork_event);
    for (auto& r : prof) { cudaEventDestroy(r.start); cudaEventDestroy(r.stop); }
    plans.reset();
    split_scratch.reset();
    reduce_buf.reset();
    scal_dev.reset();
    if (scal_host) cudaFreeHost(scal_host);
    if (sync_event) cudaEventDestroy(sync_event);
    if (err_host) cudaFreeHost(err_host);
    if (pin) cudaFreeHost(pin);
    if (stage) cudaFreeHost(stage);
    if (ring) cudaFreeHost(ring);
    if (defer_own) cudaFreeHost(defer_host);
    for (int i = 0; i < 2; ++i)
        if (ring_ev[i]) cudaEventDestroy(ring_ev[i]);
    if (std::getenv("ITG_WAIT_LOG"))
        std::fprintf(stderr, "itg context: %llu host waits, %llu kernel launches\n", (unsigned long long)host_waits,
                     (unsigned long long)kernel_launches);
    if (stream) {
        stream_unregister(stream);
        if (cache) cache->release();  // while the stream lives
        cudaStreamDestroy(stream);
    }
}

void Ctx::ensure_pin(size_t bytes) {
    if (pin_bytes >= bytes) return;
    sync();
    if (pin) cudaFreeHost(pin);
    pin = nullptr;
    // geometric growth: pinning host memory costs milliseconds per call
    size_t nb = std::max<size_t>({bytes, size_t(1) << 20, pin_bytes + pin_bytes / 2});
    ITG_CHECK_CUDA(cudaHostAlloc(&pin, nb, cudaHostAllocMapped));
    ITG_CHECK_CUDA(cudaHostGetDevicePointer(&pin_dev, pin, 0));
    pin_bytes = nb;
}

void Ctx::sync() {
    ++host_waits;
    if (fiber_active()) {
        ITG_CHECK_CUDA(cudaEventRecord(sync_event, stream));
        fiber_wait_event(sync_event);
    } else {
        ITG_CHECK_CUDA(cudaStreamSynchronize(stream));
    }
    if (err_host && *reinterpret_cast<volatile int*>(err_host)) {
        const int code = err_host[0];
        err_host[0] = 0;
        throw Error(ERR_TIMEOUT, "a kernel's bounded wait gave up (tensor-core MMA completion, code " +
                                     std::to_string(code) + "); its output is not valid");
    }
}

void Ctx::wait_event(cudaEvent_t ev) {
    ++host_waits;
    if (fiber_active()) fiber_wait_event(ev);
    else ITG_CHECK_CUDA(cudaEventSynchronize(ev));
}

char* Ctx::stage_ring(size_t n) {
    n = (n + 255) / 256 * 256;
    if (n > ring_half) {
        // grow: the copies from the old ring must have run
        sync();
        if (ring) cudaFreeHost(ring);
        ring = nullptr;
        ring_half = std::max<size_t>({n, size_t(256) << 10, 2 * ring_half});
        ITG_CHECK_CUDA(cudaHostAlloc(reinterpret_cast<void**>(&ring), 2 * ring_half, cudaHostAllocMapped));
        ITG_CHECK_CUDA(cudaHostGetDevicePointer(reinterpret_cast<void**>(&ring_dev), ring, 0));
        for (int i = 0; i < 2; ++i) {
            if (!ring_ev[i]) ITG_CHECK_CUDA(cudaEventCreateWithFlags(&ring_ev[i], cudaEventDisableTiming));
            ring_pending[i] = false;
        }
        ring_off = 0;
        ring_cur = 0;
    }
    if (ring_off + n > ring_half) {
        // every copy from this half has been enqueued: mark its end, go to the other half
        ITG_CHECK_CUDA(cudaEventRecord(ring_ev[ring_cur], stream));
        ring_pending[ring_cur] = true;
        ring_cur ^= 1;
        ring_off = 0;
        if (ring_pending[ring_cur]) {
            wait_event(ring_ev[ring_cur]);
            ring_pending[ring_cur] = false;
        }
    }
    char* p = ring + (size_t)ring_cur * ring_half + ring_off;
    ring_off += n;
    return p;
}

void Ctx::upload(void* dst, void const* src, size_t n) {
    if (!n) return;
    char* p = stage_ring(n);
    std::memcpy(p, src, n);
    ring_copy(dst, p, n);
}

__global__ void ring_copy_kernel(char* __restrict__ dst, char const* __restrict__ src, size_t n) {
    pdl_wait();
    const size_t i0 = blockIdx.x * (size_t)blockDim.x + threadIdx.x, step = (size_t)gridDim.x * blockDim.x;
    if (((reinterpret_cast<uintptr_t>(dst) | reinterpret_cast<uintptr_t>(src) | n) & 15) == 0) {
        for (size_t i = i0; i < n / 16; i += step) reinterpret_cast<int4*>(dst)[i] = reinterpret_cast<int4 const*>(src)[i];
    } else {
        for (size_t i = i0; i < n; i += step) dst[i] = src[i];
    }
}

void Ctx::ring_copy(void* dst, char const* st, size_t n) {
    if (!n) return;
    ITG_REQUIRE(ring && st >= ring && st + n <= ring + 2 * ring_half, "ring_copy: source outside the staging ring");
    const char* src = ring_dev + (st - ring);
    const size_t units = (n + 15) / 16;
    const int grid = (int)std::max<size_t>(1, std::min<size_t>((units + 255) / 256, (size_t)2 * sm_count));
    launch_pdl(*this, grid, 256, 0, ring_copy_kernel, static_cast<char*>(dst), src, n);
    kernel_launches++;
}

void Ctx::d2h(void* dst, void const* src, size_t bytes) {
    if (!bytes) return;
    ensure_pin(bytes);
    ITG_CHECK_CUDA(cudaMemcpyAsync(pin, src, bytes, cudaMemcpyDeviceToHost, stream));
    sync();
    std::memcpy(dst, pin, bytes);
}

void* Ctx::split_buffer(size_t bytes) {
    if (!split_scratch || split_scratch->bytes < bytes)
        split_scratch = dev_alloc(std::max<size_t>(bytes, split_scratch ? split_scratch->bytes * 3 / 2 : 0), stream);
    return split_scratch->p;
}

std::shared_ptr<MemAccount>& current_account() {
    thread_local std::shared_ptr<MemAccount> acct;
    return acct;
}

std::shared_ptr<BlockCache>& current_cache() {
    thread_local std::shared_ptr<BlockCache> cache;
    return cache;
}

AllocCounters& alloc_counters() {
    static AllocCounters c;
    return c;
}

void BlockCache::trim(size_t keep) {
    std::lock_guard<std::mutex> g(mu);
    if (held <= keep) return;
    const bool alive = stream_alive(stream);
    while (held > keep && !free.empty()) {
        auto it = std::prev(free.end());
        if (alive) cudaFreeAsync(it->second, stream);
        else cudaFree(it->second);
        alloc_counters().driver_frees.fetch_add(1, std::memory_order_relaxed);
        held -= it->first;
        free.erase(it);
    }
}

void* Ctx::ensure_defer(size_t bytes) {
    if (defer_bytes < bytes) {
        sync();
        if (defer_own) cudaFreeHost(defer_host);
        defer_host = nullptr;
        defer_own = true;
        const size_t nb = std::max<size_t>({bytes, size_t(4) << 10, 2 * defer_bytes});
        ITG_CHECK_CUDA(cudaHostAlloc(&defer_host, nb, cudaHostAllocDefault));
        defer_bytes = nb;
    }
    return defer_host;
}

void Ctx::ensure_stage(size_t bytes) {
    if (stage_bytes >= bytes) return;
    sync();
    if (stage) cudaFreeHost(stage);
    stage = nullptr;
    size_t nb = std::max<size_t>({bytes, size_t(1) << 20, stage_bytes + stage_bytes / 2});
    ITG_CHECK_CUDA(cudaHostAlloc(&stage, nb, cudaHostAllocDefault));
    stage_bytes = nb;
}

Match match_indices(std::vector<Index> const& A, std::vector<Index> const& B) {
    Match m;
    std::vector<char> bused(B.size(), 0);
    std::vector<char> acon(A.size(), 0);
    for (size_t i = 0; i < A.size(); ++i)
        for (size_t j = 0; j < B.size(); ++j)
            if (!bused[j] && A[i].same(B[j])) {
                // one index seen twice must have one sector structure (the reference's
                // Index carries its sectors, so equal indices cannot disagree)
                if (A[i].sec != B[j].sec)
                    ITG_REQUIRE(A[i].sec->dim == B[j].sec->dim,
                                "contract: a contracted index has different sector sizes on the two operands");
                m.a_con.push_back((int)i);
                m.b_con.push_back((int)j);
                bused[j] = 1;
                acon[i] = 1;
                break;
            }
    for (size_t i = 0; i < A.size(); ++i) if (!acon[i]) m.a_unc.push_back((int)i);
    for (size_t j = 0; j < B.size(); ++j) if (!bused[j]) m.b_unc.push_back((int)j);
    return m;
}

namespace {

template <typename T> void put(std::string& s, T const& v) { s.append(reinterpret_cast<char const*>(&v), sizeof(T)); }
template <typename T> void putv(std::string& s, std::vector<T> const& v) {
    put(s, (uint64_t)v.size());
    if (!v.empty()) s.append(reinterpret_cast<char const*>(v.data()), v.size() * sizeof(T));
}
void put_layout_structure(std::string& s, Layout const& L) {
    put(s, (int32_t)L.rank());
    for (auto const& I : L.inds) putv(s, I.sec->dim);
    putv(s, L.coords);
}

int bits_for(int n) {
    int b = 0;
    while ((1 << b) < n) ++b;
    return b;
}

// Appends the offset table of a fused index with these dims and strides
// (first dim fastest) in the two-level form read by tab_at.
void enum_offsets(std::vector<int32_t>& tab, std::vector<int> const& dims, std::vector<int64_t> const& strides) {
    const int n = (int)dims.size();
    int64_t P = 1, s = 1;
    int j = 0;
    if (n > 0) {
        s = strides[0];
        P = dims[0];
        j = 1;
        while (j < n && strides[j] == s * P) P *= dims[j++];
    }
    tab.push_back((int32_t)P);
    tab.push_back((int32_t)s);
    int64_t total = 1;
    for (int k = j; k < n; ++k) total *= dims[k];
    std::vector<int> dig(n, 0);
    int64_t off = 0;
    for (int64_t t = 0; t < total; ++t) {
        tab.push_back((int32_t)off);
        for (int k = j; k < n; ++k) {
            off += strides[k];
            if (++dig[k] < dims[k]) break;
            off -= strides[k] * dims[k];
            dig[k] = 0;
        }
    }
}

std::vector<int64_t> block_strides(Layout const& L, int b) {
    std::vector<int64_t> st(L.rank());
    int64_t s = 1;
    for (int k = 0; k < L.rank(); ++k) { st[k] = s; s *= L.inds[k].bdim(L.block(b)[k]); }
    return st;
}

size_t align16(size_t x) { return (x + 15) & ~size_t(15); }

}  // namespace

void ensure_variant_tables(Ctx& ctx, Plan const& p) {
    if (p.skinny || p.variants_ready.load(std::memory_order_acquire)) return;
    std::lock_guard<std::mutex> g(p.vmu);
    if (p.variants_ready.load(std::memory_order_relaxed)) return;
    ITG_REQUIRE(p.vsrc, "plan: no source for the variant tile tables");
    Plan::VariantSource const& v = *p.vsrc;
    const int ncb = (int)v.cblk.size();
    // 64-row tiles, most expensive first (stable, as the 32-row list)
    std::vector<ItemRec> items64;
    {
        std::vector<ItemRec> raw;
        std::vector<double> cost;
        for (int c = 0; c < ncb; ++c)
            for (int m0 = 0; m0 < v.cblk[c].M; m0 += 64)
                for (int n0 = 0; n0 < v.cblk[c].N; n0 += GEMM_TILE) {
                    raw.push_back(ItemRec{c, m0, n0, v.cp0[c], v.cp1[c]});
                    cost.push_back(v.cost[c]);
                }
        std::vector<int> o(raw.size());
        std::iota(o.begin(), o.end(), 0);
        std::stable_sort(o.begin(), o.end(), [&](int x, int y) { return cost[x] > cost[y]; });
        for (int i : o) items64.push_back(raw[i]);
    }
    // tensor-core tiles: 128 rows along each block's longer side, TC_TILE_N
    // columns along the other; the pairs seen from each block's rows and columns
    std::vector<TcTile> items_tc;
    std::vector<TcPair> pairs_tc(v.pia.size());
    {
        std::vector<TcTile> raw;
        std::vector<double> cost;
        for (int c = 0; c < ncb; ++c) {
            CBlockRec const& cb = v.cblk[c];
            const int swap = cb.N > cb.M ? 1 : 0;
            const int R = swap ? cb.N : cb.M, W = swap ? cb.M : cb.N;
            for (int q = v.cp0[c]; q < v.cp1[c]; ++q) {
                OpBlockRec const& orow = v.ops[swap ? v.pib[q] : v.pia[q]];
                OpBlockRec const& ocol = v.ops[swap ? v.pia[q] : v.pib[q]];
                pairs_tc[q] = TcPair{orow.panel, ocol.panel, orow.exp, ocol.exp, panel_row_groups(orow.rows),
                                     panel_row_groups(ocol.rows), orow.Kp / 16, 0};
            }
            for (int r0 = 0; r0 < R; r0 += TC_TILE_M)
                for (int c0 = 0; c0 < W; c0 += TC_TILE_N) {
                    raw.push_back(TcTile{cb.coff, swap ? cb.tcn : cb.tcm, swap ? cb.tcm : cb.tcn, R, W, r0, c0,
                                         v.cp0[c], v.cp1[c], swap, 0});
                    cost.push_back(v.cost[c]);
                }
        }
        std::vector<int> o(raw.size());
        std::iota(o.begin(), o.end(), 0);
        std::stable_sort(o.begin(), o.end(), [&](int x, int y) { return cost[x] > cost[y]; });
        for (int i : o) items_tc.push_back(raw[i]);
    }
    const size_t t_i64 = 0, t_itc = align16(sizeof(ItemRec) * items64.size());
    const size_t t_ptc = align16(t_itc + sizeof(TcTile) * items_tc.size());
    const size_t bytes = align16(t_ptc + sizeof(TcPair) * std::max<size_t>(1, pairs_tc.size()));
    // like the plan's own tables: the plan's memory, not the calling solve's
    std::shared_ptr<MemAccount> saved = std::move(current_account());
    current_account().reset();
    DevBufPtr dev = dev_alloc(bytes, ctx.stream);
    current_account() = std::move(saved);
    char* st = ctx.stage_ring(bytes);
    if (!items64.empty()) std::memcpy(st + t_i64, items64.data(), sizeof(ItemRec) * items64.size());
    if (!items_tc.empty()) std::memcpy(st + t_itc, items_tc.data(), sizeof(TcTile) * items_tc.size());
    if (!pairs_tc.empty()) std::memcpy(st + t_ptc, pairs_tc.data(), sizeof(TcPair) * pairs_tc.size());
    ctx.ring_copy(dev->p, st, bytes);
    ctx.sync();  // resident before any stream launches with them
    char* db = dev->as<char>();
    p.d_items64 = reinterpret_cast<ItemRec*>(db + t_i64);
    p.nitems64 = (int)items64.size();
    p.d_items_tc = reinterpret_cast<TcTile*>(db + t_itc);
    p.d_pairs_tc = reinterpret_cast<TcPair*>(db + t_ptc);
    p.nitems_tc = (int)items_tc.size();
    p.dev_variants = std::move(dev);
    p.vsrc.reset();
    p.variants_ready.store(true, std::memory_order_release);
}

// Contractions with at most this many candidate block pairs are planned on
// the host (plan_host); larger ones by plan_kernel. ITG_HOST_PLAN_PAIRS moves
// the threshold (0: every plan on the device).
static long long host_plan_pairs() {
    const char* e = std::getenv("ITG_HOST_PLAN_PAIRS");
    return e ? std::max(0LL, std::atoll(e)) : (1LL << 16);
}

// Host form of plan_kernel: the same keys, the same stable orders, the same
// pairs in the same sequence (B-key groups, A in key order, B within the
// group), hence the same output blocks, offsets and pair-to-block map.
static void plan_host(Layout const& A, Layout const& B, Match const& mt, std::vector<int32_t> const& bits,
                      std::vector<int32_t> const& cdims, std::vector<int32_t> const& cdstart, std::vector<int32_t>& pa,
                      std::vector<int32_t>& pb, std::vector<int32_t>& pc, std::vector<int32_t>& ccoords,
                      std::vector<int64_t>& coff, int64_t& csize) {
    const int nA = A.nblocks(), nB = B.nblocks(), rA = A.rank(), rB = B.rank();
    const int ncon = (int)mt.a_con.size(), nau = (int)mt.a_unc.size(), nbu = (int)mt.b_unc.size();
    auto pack = [&](int32_t const* c, std::vector<int> const& pos, int b0) {
        uint64_t k = 0;
        int sh = 0;
        for (size_t i = 0; i < pos.size(); ++i) {
            k |= (uint64_t)(uint32_t)c[pos[i]] << sh;
            sh += bits[b0 + i];
        }
        return k;
    };
    int bitsA = 0;
    for (int i = 0; i < nau; ++i) bitsA += bits[ncon + i];
    std::vector<uint64_t> keyA(nA), conA(nA), keyB(nB), conB(nB);
    for (int i = 0; i < nA; ++i) {
        int32_t const* c = A.coords.data() + (size_t)i * rA;
        keyA[i] = pack(c, mt.a_unc, ncon);
        conA[i] = pack(c, mt.a_con, 0);
    }
    for (int j = 0; j < nB; ++j) {
        int32_t const* c = B.coords.data() + (size_t)j * rB;
        keyB[j] = pack(c, mt.b_unc, ncon + nau);
        conB[j] = pack(c, mt.b_con, 0);
    }
    std::vector<int32_t> sA(nA), sB(nB);
    std::iota(sA.begin(), sA.end(), 0);
    std::iota(sB.begin(), sB.end(), 0);
    std::stable_sort(sA.begin(), sA.end(), [&](int x, int y) { return keyA[x] < keyA[y]; });
    std::stable_sort(sB.begin(), sB.end(), [&](int x, int y) { return keyB[x] < keyB[y]; });
    const int rC = nau + nbu;
    pa.clear(); pb.clear(); pc.clear(); ccoords.clear(); coff.clear();
    uint64_t last = 0;
    for (int g0 = 0; g0 < nB;) {
        int g1 = g0 + 1;
        while (g1 < nB && keyB[sB[g1]] == keyB[sB[g0]]) ++g1;
        for (int r = 0; r < nA; ++r) {
            const int ia = sA[r];
            for (int t = g0; t < g1; ++t) {
                const int jb = sB[t];
                if (conA[ia] != conB[jb]) continue;
                const uint64_t pk = keyA[ia] | (keyB[jb] << bitsA);
                if (pa.empty() || pk != last) {
                    // a new output block: coordinates and size from this pair
                    int32_t const* ca = A.coords.data() + (size_t)ia * rA;
                    int32_t const* cb = B.coords.data() + (size_t)jb * rB;
                    int64_t size = 1;
                    for (int i = 0; i < nau; ++i) {
                        const int sct = ca[mt.a_unc[i]];
                        ccoords.push_back(sct);
                        size *= cdims[cdstart[i] + sct];
                    }
                    for (int i = 0; i < nbu; ++i) {
                        const int sct = cb[mt.b_unc[i]];
                        ccoords.push_back(sct);
                        size *= cdims[cdstart[nau + i] + sct];
                    }
                    coff.push_back(size);
                    last = pk;
                }
                pa.push_back(ia);
                pb.push_back(jb);
                pc.push_back((int32_t)coff.size() - 1);
            }
        }
        g0 = g1;
    }
    (void)rC;
    int64_t tot = 0;
    for (auto& o : coff) {
        const int64_t sz = o;
        o = tot;
        tot += sz;
    }
    csize = tot;
}

std::shared_ptr<Plan> get_plan(Ctx& ctx, Layout const& A, Layout const& B, Match const& mt,
                               std::shared_ptr<Layout> target) {
    const int nau = (int)mt.a_unc.size(), nbu = (int)mt.b_unc.size(), ncon = (int)mt.a_con.size();
    const int rC = nau + nbu;
    // natural output index order: A's uncontracted, then B's (contractIS)
    std::vector<Index> cinds;
    for (int i : mt.a_unc) cinds.push_back(A.inds[i]);
    for (int j : mt.b_unc) cinds.push_back(B.inds[j]);
    std::vector<int> perm(rC);  // natural C position -> target position
    if (target) {
        ITG_REQUIRE(target->rank() == rC, "contract: target layout has rank " + std::to_string(target->rank()) +
                                              ", the product has rank " + std::to_string(rC));
        for (int k = 0; k < rC; ++k) {
            perm[k] = target->find_index(cinds[k]);
            ITG_REQUIRE(perm[k] >= 0, "contract: target layout lacks an output index");
        }
    } else {
        std::iota(perm.begin(), perm.end(), 0);
    }
    std::string key;
    key.reserve(256 + 4 * (A.coords.size() + B.coords.size()));
    put_layout_structure(key, A);
    put_layout_structure(key, B);
    putv(key, mt.a_con); putv(key, mt.b_con); putv(key, mt.a_unc); putv(key, mt.b_unc);
    put(key, (int32_t)(target ? 1 : 0));
    if (target) { put_layout_structure(key, *target); putv(key, perm); }
    if (auto hit = ctx.plans->find(key)) { ctx.plan_hits++; return hit; }
    // Plan tables belong to the context's plan cache, not to the solve that
    // builds them: they are not charged to its memory account. They come from
    // the context's block cache like its other buffers and are read only by
    // launches on its stream (which also orders their upload and their free).
    struct Uncharged {
        std::shared_ptr<MemAccount> saved;
        Uncharged() : saved(std::move(current_account())) { current_account().reset(); }
        ~Uncharged() { current_account() = std::move(saved); }
    } uncharged;

    const int nA = A.nblocks(), nB = B.nblocks(), rA = A.rank(), rB = B.rank();
    // ---- device planner inputs
    std::vector<int32_t> pos, bits, cdims, cdstart;
    for (int i : mt.a_con) pos.push_back(i);
    for (int j : mt.b_con) pos.push_back(j);
    for (int i : mt.a_unc) pos.push_back(i);
    for (int j : mt.b_unc) pos.push_back(j);
    int bcon = 0, bunc = 0;
    for (int q = 0; q < ncon; ++q) { int b = bits_for(A.inds[mt.a_con[q]].nblock()); bits.push_back(b); bcon += b; }
    for (int i : mt.a_unc) { int b = bits_for(A.inds[i].nblock()); bits.push_back(b); bunc += b; }
    for (int j : mt.b_unc) { int b = bits_for(B.inds[j].nblock()); bits.push_back(b); bunc += b; }
    if (bcon > 64 || bunc > 64) throw Error(ERR_RANGE, "contract: block coordinates need more than 64 key bits");
    for (auto const& I : cinds) {
        cdstart.push_back((int32_t)cdims.size());
        for (int d : I.sec->dim) cdims.push_back(d);
    }
    const long long cap_ll = std::max<long long>(1, (long long)nA * nB);
    if (cap_ll > (1ll << 26)) throw Error(ERR_RANGE, "contract: too many candidate block pairs");
    const int cap = (int)cap_ll;

    auto plan = std::make_shared<Plan>();
    // diagnostics (ITG_PLAN_TIME): planner kernel (with its copies) and host table time per plan
    static const bool plan_timing = std::getenv("ITG_PLAN_TIME") != nullptr;
    auto pt0 = std::chrono::steady_clock::now();
    if (nA > 0 && nB > 0) {
        std::vector<int32_t> pa, pb, pc;
        auto natural = std::make_shared<Layout>();
        natural->inds = cinds;
        int np = 0, nc = 0;
        auto pt1 = pt0;
        if (cap <= host_plan_pairs()) {
            // few candidate pairs: the same planner on the host, no launch and no wait
            plan_host(A, B, mt, bits, cdims, cdstart, pa, pb, pc, natural->coords, natural->offs, natural->size);
            np = (int)pa.size();
            nc = (int)natural->offs.size();
            if (rC == 0) natural->finish();
            pt1 = std::chrono::steady_clock::now();
        } else {
            // inputs -> device (one staged copy)
            size_t o_ac = 0, o_bc = align16(o_ac + sizeof(int32_t) * std::max<size_t>(1, A.coords.size()));
            size_t o_pos = align16(o_bc + sizeof(int32_t) * std::max<size_t>(1, B.coords.size()));
            size_t o_bits = align16(o_pos + sizeof(int32_t) * std::max<size_t>(1, pos.size()));
            size_t o_cd = align16(o_bits + sizeof(int32_t) * std::max<size_t>(1, bits.size()));
            size_t o_cs = align16(o_cd + sizeof(int32_t) * std::max<size_t>(1, cdims.size()));
            size_t in_bytes = align16(o_cs + sizeof(int32_t) * std::max<size_t>(1, cdstart.size()));
            ctx.ensure_stage(in_bytes);
            char* st = static_cast<char*>(ctx.stage);
            auto cp = [&](size_t o, auto const& v) { if (!v.empty()) std::memcpy(st + o, v.data(), v.size() * sizeof(v[0])); };
            cp(o_ac, A.coords); cp(o_bc, B.coords); cp(o_pos, pos); cp(o_bits, bits); cp(o_cd, cdims); cp(o_cs, cdstart);
            size_t o_keyA = align16(in_bytes), o_keyB = align16(o_keyA + 8 * (size_t)nA);
            size_t o_conA = align16(o_keyB + 8 * (size_t)nB), o_conB = align16(o_conA + 8 * (size_t)nA);
            size_t o_sA = align16(o_conB + 8 * (size_t)nB), o_sB = align16(o_sA + 4 * (size_t)nA);
            size_t o_gs = align16(o_sB + 4 * (size_t)nB), o_pk = align16(o_gs + 4 * (size_t)(nB + 1));
            size_t dev_bytes = align16(o_pk + 8 * (size_t)cap);
            DevBuf scratch(dev_bytes, ctx.stream);
            char* dv = scratch.as<char>();
            ITG_CHECK_CUDA(cudaMemcpyAsync(dv, st, in_bytes, cudaMemcpyHostToDevice, ctx.stream));
            // outputs in host-mapped memory
            size_t p_cnt = 0, p_pa = 16, p_pb = align16(p_pa + 4 * (size_t)cap), p_pc = align16(p_pb + 4 * (size_t)cap);
            size_t p_cc = align16(p_pc + 4 * (size_t)cap), p_co = align16(p_cc + 4 * (size_t)cap * std::max(rC, 1));
            size_t out_bytes = align16(p_co + 8 * ((size_t)cap + 1));
            ctx.ensure_pin(out_bytes);
            char* hp = static_cast<char*>(ctx.pin);
            char* dp = static_cast<char*>(ctx.pin_dev);
            PlanArgs a;
            a.nA = nA; a.nB = nB; a.rA = rA; a.rB = rB; a.ncon = ncon; a.nau = nau; a.nbu = nbu;
            a.Acoords = reinterpret_cast<const int32_t*>(dv + o_ac);
            a.Bcoords = reinterpret_cast<const int32_t*>(dv + o_bc);
            a.pos = reinterpret_cast<const int32_t*>(dv + o_pos);
            a.bits = reinterpret_cast<const int32_t*>(dv + o_bits);
            a.cdims = reinterpret_cast<const int32_t*>(dv + o_cd);
            a.cdstart = reinterpret_cast<const int32_t*>(dv + o_cs);
            a.keyA = reinterpret_cast<uint64_t*>(dv + o_keyA); a.keyB = reinterpret_cast<uint64_t*>(dv + o_keyB);
            a.conA = reinterpret_cast<uint64_t*>(dv + o_conA); a.conB = reinterpret_cast<uint64_t*>(dv + o_conB);
            a.sortA = reinterpret_cast<int32_t*>(dv + o_sA); a.sortB = reinterpret_cast<int32_t*>(dv + o_sB);
            a.gstart = reinterpret_cast<int32_t*>(dv + o_gs); a.pkey = reinterpret_cast<uint64_t*>(dv + o_pk);
            a.out_counts = reinterpret_cast<int32_t*>(dp + p_cnt);
            a.pair_a = reinterpret_cast<int32_t*>(dp + p_pa); a.pair_b = reinterpret_cast<int32_t*>(dp + p_pb);
            a.pair_c = reinterpret_cast<int32_t*>(dp + p_pc);
            a.c_coords = reinterpret_cast<int32_t*>(dp + p_cc);
            a.c_off = reinterpret_cast<int64_t*>(dp + p_co);
            a.cap_pairs = cap; a.cap_c = cap;
            plan_kernel<<<1, 1024, 0, ctx.stream>>>(a);
            ITG_CHECK_CUDA(cudaGetLastError());
            ctx.kernel_launches++;
            ctx.sync();
            int32_t const* cnt = reinterpret_cast<int32_t const*>(hp + p_cnt);
            if (cnt[2]) throw Error(ERR_INTERNAL, "contract planner: capacity overflow");
            np = cnt[0];
            nc = cnt[1];
            pt1 = std::chrono::steady_clock::now();
            pa.assign(reinterpret_cast<int32_t*>(hp + p_pa), reinterpret_cast<int32_t*>(hp + p_pa) + np);
            pb.assign(reinterpret_cast<int32_t*>(hp + p_pb), reinterpret_cast<int32_t*>(hp + p_pb) + np);
            pc.assign(reinterpret_cast<int32_t*>(hp + p_pc), reinterpret_cast<int32_t*>(hp + p_pc) + np);
            if (rC > 0) {
                natural->coords.assign(reinterpret_cast<int32_t*>(hp + p_cc), reinterpret_cast<int32_t*>(hp + p_cc) + (size_t)nc * rC);
                natural->offs.assign(reinterpret_cast<int64_t*>(hp + p_co), reinterpret_cast<int64_t*>(hp + p_co) + nc);
                natural->size = reinterpret_cast<int64_t*>(hp + p_co)[nc];
            } else {
                natural->finish();  // one scalar block
            }
        }
        plan->C = target ? target : natural;
        // ---- map natural blocks to target blocks
        const Layout& CL = *plan->C;
        std::vector<int> nat2t(std::max(nc, 1), 0);
        if (rC > 0) {
            std::vector<int32_t> tc(rC);
            for (int c = 0; c < nc; ++c) {
                for (int k = 0; k < rC; ++k) tc[perm[k]] = natural->coords[(size_t)c * rC + k];
                int tb = CL.find_block(tc.data());
                ITG_REQUIRE(tb >= 0, "contract: target layout lacks a produced block");
                nat2t[c] = tb;
            }
        }
        const auto pq_map = std::chrono::steady_clock::now();
        // ---- tables
        std::vector<int32_t> tab;
        std::vector<int> tamA(nA, -1), takA(nA, -1), tbkB(nB, -1), tbnB(nB, -1);
        auto ensureA = [&](int ab) {
            if (tamA[ab] >= 0) return;
            auto st_ = block_strides(A, ab);
            std::vector<int> dm, dk; std::vector<int64_t> sm, sk;
            for (int i : mt.a_unc) { dm.push_back(A.inds[i].bdim(A.block(ab)[i])); sm.push_back(st_[i]); }
            for (int i : mt.a_con) { dk.push_back(A.inds[i].bdim(A.block(ab)[i])); sk.push_back(st_[i]); }
            tamA[ab] = (int)tab.size(); enum_offsets(tab, dm, sm);
            takA[ab] = (int)tab.size(); enum_offsets(tab, dk, sk);
        };
        auto ensureB = [&](int bb) {
            if (tbkB[bb] >= 0) return;
            auto st_ = block_strides(B, bb);
            std::vector<int> dk, dn; std::vector<int64_t> sk, sn;
            for (int j : mt.b_con) { dk.push_back(B.inds[j].bdim(B.block(bb)[j])); sk.push_back(st_[j]); }
            for (int j : mt.b_unc) { dn.push_back(B.inds[j].bdim(B.block(bb)[j])); sn.push_back(st_[j]); }
            tbkB[bb] = (int)tab.size(); enum_offsets(tab, dk, sk);
            tbnB[bb] = (int)tab.size(); enum_offsets(tab, dn, sn);
        };
        const int ncb = CL.nblocks();
        std::vector<CBlockRec> cblk(ncb);
        for (int c = 0; c < ncb; ++c) {
            auto st_ = rC ? block_strides(CL, c) : std::vector<int64_t>();
            std::vector<int> dm, dn; std::vector<int64_t> sm, sn;
            for (int q = 0; q < nau; ++q) { int tpos = perm[q]; dm.push_back(CL.inds[tpos].bdim(CL.block(c)[tpos])); sm.push_back(st_[tpos]); }
            for (int q = 0; q < nbu; ++q) { int tpos = perm[nau + q]; dn.push_back(CL.inds[tpos].bdim(CL.block(c)[tpos])); sn.push_back(st_[tpos]); }
            CBlockRec r;
            r.coff = CL.offs[c];
            r.M = 1; for (int d : dm) r.M *= d;
            r.N = 1; for (int d : dn) r.N *= d;
            r.tcm = (int)tab.size(); enum_offsets(tab, dm, sm);
            r.tcn = (int)tab.size(); enum_offsets(tab, dn, sn);
            cblk[c] = r;
        }
        // pairs grouped by target block (stable)
        std::vector<std::vector<int>> bypc(ncb);
        for (int p = 0; p < np; ++p) bypc[rC ? nat2t[pc[p]] : 0].push_back(p);
        std::vector<PairRec> pairs;
        pairs.reserve(np);
        std::vector<int> cp0(ncb), cp1(ncb);
        std::vector<double> cK(ncb, 0.0);
        double flops = 0; int64_t bytes_ab = 0; int maxK = 0; double sumK = 0;
        for (int c = 0; c < ncb; ++c) {
            cp0[c] = (int)pairs.size();
            int ksum = 0;
            for (int p : bypc[c]) {
                ensureA(pa[p]); ensureB(pb[p]);
                PairRec r;
                r.aoff = A.offs[pa[p]]; r.boff = B.offs[pb[p]];
                r.tam = tamA[pa[p]]; r.tak = takA[pa[p]]; r.tbk = tbkB[pb[p]]; r.tbn = tbnB[pb[p]];
                int K = 1;
                for (int i : mt.a_con) K *= A.inds[i].bdim(A.block(pa[p])[i]);
                r.K = K; r.pad = 0;
                plan->max_pair_K = std::max(plan->max_pair_K, K);
                pairs.push_back(r);
                ksum += K;
                flops += 2.0 * cblk[c].M * (double)cblk[c].N * K;
                bytes_ab += (int64_t)cblk[c].M * K + (int64_t)K * cblk[c].N;
            }
            cp1[c] = (int)pairs.size();
            cK[c] = ksum;
            maxK = std::max(maxK, ksum);
            sumK += ksum;
        }
        const auto pq_pairs = std::chrono::steady_clock::now();
        // narrow outputs (N <= SKINNY_N) make a skinny plan: row tiles, FP64 only
        int maxN = 0;
        for (int c = 0; c < ncb; ++c) maxN = std::max(maxN, cblk[c].N);
        plan->skinny = (maxN <= SKINNY_N);
        // operand panels for the split-precision path: every A and B block in use
        // (a skinny plan never takes that path and builds none)
        std::vector<OpBlockRec> ops;
        std::vector<int> ia_of(nA, -1), ib_of(nB, -1);
        int64_t panel = 0, expo = 0;
        int max_rows = 1;
        auto add_op = [&](int64_t src, int rows, int K, int trow, int tcol) {
            OpBlockRec o;
            o.src = src; o.rows = rows; o.K = K; o.Kp = (K + 15) / 16 * 16;
            o.trow = trow; o.tcol = tcol;
            o.panel = panel; o.exp = (int32_t)expo;
            panel += (int64_t)panel_row_groups(rows) * 8 * o.Kp;  // tiled: whole row groups, 128-element units
            expo += rows;
            max_rows = std::max(max_rows, rows);
            ops.push_back(o);
            return (int)ops.size() - 1;
        };
        auto rows_of = [&](Layout const& Lx, int b, std::vector<int> const& pos) {
            int r = 1;
            for (int i : pos) r *= Lx.inds[i].bdim(Lx.block(b)[i]);
            return r;
        };
        for (int ab = 0; ab < nA; ++ab)
            if (!plan->skinny && tamA[ab] >= 0)
                ia_of[ab] = add_op(A.offs[ab], rows_of(A, ab, mt.a_unc), rows_of(A, ab, mt.a_con), tamA[ab], takA[ab]);
        const int nopsA = (int)ops.size();
        for (int bb = 0; bb < nB; ++bb)
            if (!plan->skinny && tbkB[bb] >= 0)
                ib_of[bb] = add_op(B.offs[bb], rows_of(B, bb, mt.b_unc), rows_of(B, bb, mt.b_con), tbnB[bb], tbkB[bb]);
        const int nopsB = (int)ops.size() - nopsA;
        // prep items: one row group of the tiled panel (8 rows, whole rows so the
        // row exponents are complete) each, one warp per item; A's items first
        std::vector<PrepItem> prep;
        {
            size_t np8 = 0;
            for (auto const& op8 : ops) np8 += (size_t)(op8.rows + 7) / 8;
            prep.reserve(np8);
        }
        for (int o = 0; o < (int)ops.size(); ++o) {
            const int rows = ops[o].rows;
            for (int r0 = 0; r0 < rows; r0 += 8)
                prep.push_back(PrepItem{o, r0, std::min(rows, r0 + 8), o < nopsA ? 0 : 1});
        }
        {
            int q = 0;
            for (int c = 0; c < ncb; ++c)
                for (int p : bypc[c]) { pairs[q].ia = ia_of[pa[p]]; pairs[q].ib = ib_of[pb[p]]; ++q; }
        }
        const auto pq_ops = std::chrono::steady_clock::now();
        // tiles, most expensive first; a skinny plan gets row tiles
        std::vector<ItemRec> items;
        std::vector<double> cost;
        if (plan->skinny) {
            // rows per thread: the largest of 4, 2, 1 that still gives two items per SM
            plan->skinny_r = 4;
            while (plan->skinny_r > 1) {
                int64_t n_items = 0;
                for (int c = 0; c < ncb; ++c) n_items += (cblk[c].M + SKINNY_THREADS * plan->skinny_r - 1) / (SKINNY_THREADS * plan->skinny_r);
                if (n_items >= 2 * (int64_t)ctx.sm_count) break;
                plan->skinny_r /= 2;
            }
            if (plan->skinny_r == 1 && plan->max_pair_K <= SKINNY_K && !std::getenv("ITG_SKINNY_NO_WIDE")) {
                int64_t n_items = 0;
                for (int c = 0; c < ncb; ++c) n_items += (cblk[c].M + SKINNY_THREADS - 1) / SKINNY_THREADS;
                plan->skinny_wide = n_items < 2 * (int64_t)ctx.sm_count;
            }
        }
        const int tm = plan->skinny_wide ? WIDE_ROWS : plan->skinny ? SKINNY_THREADS * plan->skinny_r : GEMM_TILE;
        const int tn = plan->skinny ? SKINNY_N : GEMM_TILE;
        for (int c = 0; c < ncb; ++c)
            for (int m0 = 0; m0 < cblk[c].M; m0 += tm)
                for (int n0 = 0; n0 < cblk[c].N; n0 += tn) {
                    items.push_back(ItemRec{c, m0, n0, cp0[c], cp1[c]});
                    cost.push_back(cK[c] + 1.0);
                }
        std::vector<int> ord(items.size());
        std::iota(ord.begin(), ord.end(), 0);
        std::stable_sort(ord.begin(), ord.end(), [&](int x, int y) { return cost[x] > cost[y]; });
        std::vector<ItemRec> sitems(items.size());
        for (size_t i = 0; i < ord.size(); ++i) sitems[i] = items[ord[i]];
        const auto pq_items = std::chrono::steady_clock::now();
        // the other split-precision tile shapes are built on first use from this
        if (!plan->skinny) {
            auto vs = std::make_shared<Plan::VariantSource>();
            vs->cblk = cblk;
            vs->cp0 = cp0;
            vs->cp1 = cp1;
            vs->cost.resize(ncb);
            for (int c = 0; c < ncb; ++c) vs->cost[c] = cK[c] + 1.0;
            vs->pia.resize(pairs.size());
            vs->pib.resize(pairs.size());
            for (size_t q = 0; q < pairs.size(); ++q) { vs->pia[q] = pairs[q].ia; vs->pib[q] = pairs[q].ib; }
            vs->ops = ops;
            plan->vsrc = std::move(vs);
        }
        const auto pq_vsrc = std::chrono::steady_clock::now();
        // upload
        size_t t_items = 0, t_pairs = align16(sizeof(ItemRec) * sitems.size());
        size_t t_cblk = align16(t_pairs + sizeof(PairRec) * pairs.size());
        size_t t_ops = align16(t_cblk + sizeof(CBlockRec) * cblk.size());
        size_t t_prep = align16(t_ops + sizeof(OpBlockRec) * ops.size());
        size_t t_tab = align16(t_prep + sizeof(PrepItem) * prep.size());
        size_t tbytes = align16(t_tab + sizeof(int32_t) * std::max<size_t>(1, tab.size()));
        char* st = ctx.stage_ring(tbytes);
        if (!sitems.empty()) std::memcpy(st + t_items, sitems.data(), sizeof(ItemRec) * sitems.size());
        if (!pairs.empty()) std::memcpy(st + t_pairs, pairs.data(), sizeof(PairRec) * pairs.size());
        if (!cblk.empty()) std::memcpy(st + t_cblk, cblk.data(), sizeof(CBlockRec) * cblk.size());
        if (!ops.empty()) std::memcpy(st + t_ops, ops.data(), sizeof(OpBlockRec) * ops.size());
        if (!prep.empty()) std::memcpy(st + t_prep, prep.data(), sizeof(PrepItem) * prep.size());
        plan->nprep = (int)prep.size();
        plan->nprepA = 0;
        for (auto const& it : prep) plan->nprepA += (it.which == 0);
        if (!tab.empty()) std::memcpy(st + t_tab, tab.data(), sizeof(int32_t) * tab.size());
        plan->nopsA = nopsA;
        plan->nopsB = nopsB;
        plan->panel_elems = panel;
        plan->exp_elems = expo;
        plan->max_rows = max_rows;
        plan->dev = dev_alloc(tbytes, ctx.stream);
        char* db = plan->dev->as<char>();
        ctx.ring_copy(db, st, tbytes);
        plan->d_items = reinterpret_cast<ItemRec*>(db + t_items);
        plan->d_pairs = reinterpret_cast<PairRec*>(db + t_pairs);
        plan->d_cblk = reinterpret_cast<CBlockRec*>(db + t_cblk);
        plan->d_ops = reinterpret_cast<OpBlockRec*>(db + t_ops);
        plan->d_prep = reinterpret_cast<PrepItem*>(db + t_prep);
        plan->d_tab = reinterpret_cast<int32_t*>(db + t_tab);
        plan->nitems = (int)sitems.size();
        plan->npairs = np;
        plan->ncblk = ncb;
        plan->flops = flops;
        plan->bytes_ab = bytes_ab;
        plan->maxK = maxK;
        plan->avgK = ncb ? sumK / ncb : 0;
        if (plan_timing) {
            auto pt2 = std::chrono::steady_clock::now();
            auto ms = [](auto a, auto b) { return std::chrono::duration<double, std::milli>(b - a).count(); };
            std::fprintf(stderr,
                         "itg plan: nA %d nB %d pairs %d C %d device %.3f ms host %.3f ms (block map %.3f, offset "
                         "tables and pairs %.3f, operand panels %.3f, tiles %.3f, variant source %.3f, upload %.3f)\n",
                         nA, nB, np, nc, ms(pt0, pt1), ms(pt1, pt2), ms(pt1, pq_map), ms(pq_map, pq_pairs),
                         ms(pq_pairs, pq_ops), ms(pq_ops, pq_items), ms(pq_items, pq_vsrc), ms(pq_vsrc, pt2));
        }
    } else {
        // an empty operand: the output has no blocks (or is the scalar 0)
        auto natural = std::make_shared<Layout>();
        natural->inds = cinds;
        natural->finish();
        if (rC > 0) { natural->offs.clear(); natural->size = 0; }
        plan->C = target ? target : natural;
        // zero-fill every block of the output layout
        const Layout& CL = *plan->C;
        std::vector<CBlockRec> cblk;
        std::vector<int32_t> tab;
        std::vector<ItemRec> items;
        for (int c = 0; c < CL.nblocks(); ++c) {
            CBlockRec r;
            r.coff = CL.offs[c];
            r.M = (int)CL.block_size(c); r.N = 1;
            r.tcm = (int)tab.size(); enum_offsets(tab, {r.M}, {1});
            r.tcn = (int)tab.size(); enum_offsets(tab, {}, {});
            cblk.push_back(r);
            for (int m0 = 0; m0 < r.M; m0 += GEMM_TILE) items.push_back(ItemRec{c, m0, 0, 0, 0});
        }
        size_t t_items = 0, t_cblk = align16(sizeof(ItemRec) * std::max<size_t>(1, items.size()));
        size_t t_tab = align16(t_cblk + sizeof(CBlockRec) * std::max<size_t>(1, cblk.size()));
        size_t tbytes = align16(t_tab + sizeof(int32_t) * std::max<size_t>(1, tab.size()));
        char* st = ctx.stage_ring(tbytes);
        if (!items.empty()) std::memcpy(st + t_items, items.data(), sizeof(ItemRec) * items.size());
        if (!cblk.empty()) std::memcpy(st + t_cblk, cblk.data(), sizeof(CBlockRec) * cblk.size());
        if (!tab.empty()) std::memcpy(st + t_tab, tab.data(), sizeof(int32_t) * tab.size());
        plan->dev = dev_alloc(tbytes, ctx.stream);
        char* db = plan->dev->as<char>();
        ctx.ring_copy(db, st, tbytes);
        plan->d_items = reinterpret_cast<ItemRec*>(db + t_items);
        plan->d_pairs = nullptr;
        plan->d_cblk = reinterpret_cast<CBlockRec*>(db + t_cblk);
        plan->d_tab = reinterpret_cast<int32_t*>(db + t_tab);
        plan->nitems = (int)items.size();
    }
    plan->scalar = (rC == 0);
    ctx.plans_built++;
    return ctx.plans->insert(std::move(key), plan);
}

void exec_plan(Ctx& ctx, Plan const& p, double const* A, double const* B, double* C, int prec) {
    if (p.nitems == 0) return;
    if (prec < 0) prec = ctx.precision;
    ProfRec pr{};
    if (ctx.profiling) {
        ITG_CHECK_CUDA(cudaEventCreate(&pr.start));
        ITG_CHECK_CUDA(cudaEventCreate(&pr.stop));
        ITG_CHECK_CUDA(cudaEventRecord(pr.start, ctx.stream));
        pr.flops = p.flops;
        pr.nitems = p.nitems;
        pr.kind = p.skinny ? 2 : plan_uses_split(p, prec) ? 1 : 0;
    }
    // narrow, small-K contractions (the MPO-tensor steps) are bandwidth-shaped: FP64 is exact there
    if (p.skinny && (prec == PREC_F64 || prec == PREC_OZAKI_BF16)) {
        launch_skinny(ctx, p, A, B, C);
    } else if (plan_uses_split(p, prec)) {
        const int S = ctx.ozaki_slices;
        const int64_t plane = (p.panel_elems + 15) / 16 * 16;
        __nv_bfloat16* panels = static_cast<__nv_bfloat16*>(ctx.split_buffer(split_scratch_bytes(p, S)));
        int32_t* exps = reinterpret_cast<int32_t*>(panels + plane * S);
        if (ctx.gemm_variant < 0 && p.oz_variant.load(std::memory_order_relaxed) < 0 && p.flops >= AUTOTUNE_MIN_FLOPS &&
            p.split_uses.fetch_add(1, std::memory_order_relaxed) + 1 >= AUTOTUNE_MIN_USES)
            autotune_ozaki(ctx, p, A, B, C, S, panels, exps);
        // in a solver-pool fiber that groups launches: one launch with the other solves' contractions
        if (ctx.profiling || !fiber_group_contract(ctx, p, A, B, C, S, panels, exps, true)) {
            launch_ozaki(ctx, p, A, B, C, S, panels, exps);
            ctx.kernel_launches += 1;
        } else {
            ctx.kernel_launches -= 1;  // flush() counted the group's two launches
        }
    } else if (prec == PREC_F64 || prec == PREC_OZAKI_BF16) {
        // in a solver-pool fiber that groups launches: one launch with the other solves' contractions
        if (ctx.profiling || !fiber_group_contract(ctx, p, A, B, C, 0, nullptr, nullptr, false))
            launch_pdl(ctx, p.nitems, 256, 0, gemm_f64_kernel, p.d_items, p.d_pairs, p.d_cblk, p.d_tab, A, B, C);
        else
            ctx.kernel_launches -= 1;  // flush() counted the group's launch
    } else {
        throw Error(ERR_ARG, "contract: unsupported precision mode");
    }
    ITG_CHECK_CUDA(cudaGetLastError());
    ctx.kernel_launches++;
    ctx.flops_done += p.flops;
    if (ctx.profiling) {
        ITG_CHECK_CUDA(cudaEventRecord(pr.stop, ctx.stream));
        ctx.prof.push_back(pr);
    }
}

void exec_plan_f64_only(Ctx& ctx, Plan const& p, double const* A, double const* B, double* C) {
    if (p.nitems == 0) return;
    if (p.skinny)
        launch_skinny(ctx, p, A, B, C);
    else
        launch_pdl(ctx, p.nitems, 256, 0, gemm_f64_kernel, p.d_items, p.d_pairs, p.d_cblk, p.d_tab, A, B, C);
    ITG_CHECK_CUDA(cudaGetLastError());
    ctx.kernel_launches++;
    ctx.flops_done += p.flops;
}

Tensor contract(Ctx& ctx, Tensor const& A, Tensor const& B, int prec, std::shared_ptr<Layout> target) {
    ITG_REQUIRE(A.valid() && B.valid(), "contract: null tensor");
    Match mt = match_indices(A.inds(), B.inds());
    auto plan = get_plan(ctx, *A.lay, *B.lay, mt, target);
    // plans are shared by every contraction of the same block structure: the
    // output carries this contraction's own indices (or the caller's target)
    std::shared_ptr<Layout> CL = target;
    if (!CL) {
        CL = std::make_shared<Layout>(*plan->C);
        CL->inds.clear();
        for (int i : mt.a_unc) CL->inds.push_back(A.inds()[i]);
        for (int j : mt.b_unc) CL->inds.push_back(B.inds()[j]);
    }
    Tensor C(CL, ctx.stream);
    exec_plan(ctx, *plan, A.data(), B.data(), C.data(), prec);
    if (plan->scalar) {
        double v = 0;
        ctx.d2h(&v, C.data(), sizeof(double));
        C.scalar = v;
    }
    return C;
}

}  // namespace itg
