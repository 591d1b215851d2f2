// Tensor-core (tcgen05) variant of the split-precision block GEMM; included
// by ozaki.cu (it shares that file's digit format, scaled_i64 and tab_at).
//
// The same digit products as the mma.sync variants, on the 5th-generation
// tensor cores. A persistent CTA per SM walks the cost-ordered tile list; a
// tile is 128 rows (TMEM lanes) along an output block's longer side times
// TN columns along the other. Warp roles (320 threads):
//   warp 8  producer: per k-step of 16, one bulk copy (cp.async.bulk, the TMA
//           engine) per digit plane and operand from the tiled panels into a
//           ring of NST shared-memory stages, completing on the stage's
//           `full` mbarrier (transaction count);
//   warp 9  MMA issuer (one thread): the S(S+1)/2 tcgen05.mma (kind::f16,
//           BF16 in, FP32 accumulate) of the step, each into the TMEM
//           columns of its diagonal D = s + t, then tcgen05.commit to the
//           stage's `empty` mbarrier; after the last step of a KCHUNK (or of
//           the pair) a commit to the accumulator set's `tfull` mbarrier.
//           Two accumulator sets alternate, so the MMAs of the next chunk run
//           while the epilogue reads the last one;
//   warps 0-7 epilogue, two warpgroups each holding half of the columns:
//           tcgen05.ld of the S diagonals (thread = row), exact fold into
//           int64, `tempty` arrival, and per pair the scaling into FP64
//           partial sums in shared memory; per tile the store to C, by rows
//           or by columns, whichever runs along C's fastest index.
// The operand tiles arrive exactly in the no-swizzle K-major core-matrix
// layout the MMA reads (the panels are tiled that way), so each is one copy.
// Rows or columns past a block's end bring in other data (or the scratch's
// padding) and only feed outputs that are never stored.
// Results are bit-identical to the mma.sync variants. Every mbarrier wait is
// bounded (clock64) and also gives up when another role has: the kernel then
// sets the context's status word, lets the copies and MMAs in flight finish
// (bounded), frees TMEM and returns without storing the tile.

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

// Waits for the completion of the barrier phase with this parity, for at most
// `limit` SM clocks and only while *abort stays 0; false when it gave up.
__device__ __forceinline__ bool mbar_wait_bounded(uint32_t bar, uint32_t parity, long long limit,
                                                  volatile int* abort) {
    const long long t0 = clock64();
    while (!mbar_try_wait(bar, parity))
        if (*abort || clock64() - t0 > limit) return false;
    return true;
}

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count));
}
__device__ __forceinline__ void mbar_arrive(uint32_t bar) {
    asm volatile("{\n\t.reg .b64 st;\n\tmbarrier.arrive.shared::cta.b64 st, [%0];\n\t}" ::"r"(bar) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
    asm volatile("{\n\t.reg .b64 st;\n\tmbarrier.arrive.expect_tx.shared::cta.b64 st, [%0], %1;\n\t}" ::"r"(bar),
                 "r"(bytes)
                 : "memory");
}
// bulk copy global -> shared (16-byte aligned, size a multiple of 16), completing on bar
__device__ __forceinline__ void bulk_g2s(uint32_t dst, const void* src, uint32_t bytes, uint32_t bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
                 "l"(src), "r"(bytes), "r"(bar)
                 : "memory");
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

// 16 consecutive TMEM columns of this warp's 32 lanes, without waiting (tc_wait_ld)
__device__ __forceinline__ void tc_ld16(uint32_t taddr, uint32_t (&r)[16]) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
}
__device__ __forceinline__ void tc_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

// barrier among the eight epilogue warps only (the producer and MMA warps run on)
__device__ __forceinline__ void epi_sync() { asm volatile("bar.sync 1, 256;" ::: "memory"); }

template <int S, int TN>
struct TcShape {
    static constexpr int TM = TC_TILE_M, KS = 16;
    static constexpr int A_PLANE = TM * KS * 2;   // bytes of one digit plane of the row tile
    static constexpr int B_PLANE = TN * KS * 2;   // of the column tile
    static constexpr int STAGE = S * (A_PLANE + B_PLANE);
    static constexpr int NST = 4;                 // shared-memory stages in the ring
    static constexpr int KCHUNK = (S <= 4) ? 256 : 128;
    static constexpr int CHUNK_STEPS = KCHUNK / KS;
    static constexpr int ACC = S * TN;            // TMEM columns of one accumulator set
    static constexpr uint32_t TMEM_COLS = (2 * ACC <= 128) ? 128 : (2 * ACC <= 256 ? 256 : 512);
    static constexpr int LDO = TN + 1;            // row stride of the FP64 partial results (doubles)
    static constexpr int OUT = 8 * TM * LDO;      // FP64 partial results, [row][column]
    // full[NST], empty[NST], tfull[2], tempty[2], drain, stuck; TMEM address, abort, flags
    static constexpr int BAR_OFF = NST * STAGE + OUT;
    static constexpr int NBAR = 2 * NST + 6;
    static constexpr int MISC_OFF = BAR_OFF + 8 * NBAR;
    static constexpr int ECOL_OFF = MISC_OFF + 16;          // column exponents of the pair
    static constexpr int COFF_OFF = ECOL_OFF + 4 * TN;      // C offsets along the tile's columns
    static constexpr int ROFF_OFF = COFF_OFF + 4 * TN;      // C offsets along the tile's rows
    static constexpr size_t SMEM = (size_t)ROFF_OFF + 4 * TM;
    static constexpr int EPI_WARPS = 8;           // two warpgroups, each half of the columns
    static constexpr int PRODUCER = 8, ISSUER = 9;   // warp numbers
    static constexpr int THREADS = 320;
};

template <int S, int TN>
__global__ void __launch_bounds__(320, 1)
gemm_ozaki_tc_kernel(const TcTile* __restrict__ tiles, int ntiles, const TcPair* __restrict__ tpairs,
                     const int32_t* __restrict__ tab, const __nv_bfloat16* __restrict__ panels, int64_t plane,
                     const int32_t* __restrict__ exps, double* __restrict__ C, int* __restrict__ status,
                     long long wait_limit, int stuck_test) {
    pdl_wait();
    using SH = TcShape<S, TN>;
    static_assert(2 * S * TN <= 512, "two accumulator sets must fit in TMEM");
    static_assert(TN % 32 == 0, "the column-wise store gives each lane one column per 32");
    static_assert((long long)SH::KCHUNK * S * 128 * 128 <= (1LL << 24), "digit sums must stay exact in FP32");
    extern __shared__ __align__(128) unsigned char tc_smem[];
    const uint32_t sbase = smem_u32(tc_smem);
    double* outs = reinterpret_cast<double*>(tc_smem + SH::NST * SH::STAGE);
    const uint32_t bars = sbase + SH::BAR_OFF;
    auto full = [&](int i) { return bars + 8u * i; };
    auto empty = [&](int i) { return bars + 8u * (SH::NST + i); };
    auto tfull = [&](int b) { return bars + 8u * (2 * SH::NST + b); };
    auto tempty = [&](int b) { return bars + 8u * (2 * SH::NST + 2 + b); };
    const uint32_t drain = bars + 8u * (2 * SH::NST + 4);
    const uint32_t stuck = bars + 8u * (2 * SH::NST + 5);  // nothing arrives here
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(tc_smem + SH::MISC_OFF);
    volatile int* abort = reinterpret_cast<volatile int*>(tc_smem + SH::MISC_OFF + 4);
    volatile int* epi_ok = reinterpret_cast<volatile int*>(tc_smem + SH::MISC_OFF + 8);
    int* ecol = reinterpret_cast<int*>(tc_smem + SH::ECOL_OFF);
    int* coff = reinterpret_cast<int*>(tc_smem + SH::COFF_OFF);
    int* roff = reinterpret_cast<int*>(tc_smem + SH::ROFF_OFF);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    if (tid == 0) {
        for (int i = 0; i < SH::NST; ++i) {
            mbar_init(full(i), 1);
            mbar_init(empty(i), 1);
        }
        for (int b = 0; b < 2; ++b) {
            mbar_init(tfull(b), 1);
            mbar_init(tempty(b), 32 * SH::EPI_WARPS);
        }
        mbar_init(drain, 1);
        mbar_init(stuck, 1);
        *abort = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == SH::ISSUER) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                     "r"(SH::TMEM_COLS));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tmem_slot;
    auto fail = [&]() {
        if (atomicExch((int*)abort, 1) == 0) atomicExch(status, 1);
    };

    if (warp == SH::PRODUCER) {
        // ---------------- producer
        if (lane == 0) {
            int stage = 0;
            uint32_t phase = 0;
            uint32_t filled[SH::NST] = {};
            for (int ti = blockIdx.x; ti < ntiles && !*abort; ti += gridDim.x) {
                const TcTile T = tiles[ti];
                const int rg0 = T.r0 >> 3, cg0 = T.c0 >> 3;
                for (int p = T.p0; p < T.p1 && !*abort; ++p) {
                    const TcPair P = tpairs[p];
                    for (int ks = 0; ks < P.nk; ++ks) {
                        if (!mbar_wait_bounded(empty(stage), phase ^ 1u, wait_limit, abort)) { fail(); break; }
                        mbar_expect_tx(full(stage), SH::STAGE);
                        const uint32_t dst = sbase + stage * SH::STAGE;
                        const __nv_bfloat16* a0 = panels + P.rpanel + ((int64_t)ks * P.nrg_r + rg0) * 128;
                        const __nv_bfloat16* b0 = panels + P.cpanel + ((int64_t)ks * P.nrg_c + cg0) * 128;
#pragma unroll 1
                        for (int s = 0; s < S; ++s) {
                            bulk_g2s(dst + s * SH::A_PLANE, a0 + s * plane, SH::A_PLANE, full(stage));
                            bulk_g2s(dst + S * SH::A_PLANE + s * SH::B_PLANE, b0 + s * plane, SH::B_PLANE, full(stage));
                        }
                        filled[stage] = phase + 1;
                        if (++stage == SH::NST) { stage = 0; phase ^= 1u; }
                    }
                }
            }
            // copies in flight land before the CTA ends (after an abort none is consumed)
            for (int i = 0; i < SH::NST; ++i)
                if (filled[i]) {
                    int zero = 0;
                    mbar_wait_bounded(full(i), (filled[i] - 1) & 1u, wait_limit, (volatile int*)&zero);
                }
        }
        __syncwarp();
    } else if (warp == SH::ISSUER) {
        // ---------------- MMA issuer
        if (lane == 0) {
            constexpr uint32_t IDESC = tc_idesc_bf16(SH::TM, TN);
            int stage = 0;
            uint32_t phase = 0, unit = 0;
            bool issued = false;
            for (int ti = blockIdx.x; ti < ntiles && !*abort; ti += gridDim.x) {
                const TcTile T = tiles[ti];
                for (int p = T.p0; p < T.p1 && !*abort; ++p) {
                    const int nk = tpairs[p].nk;
                    bool ok = true;
                    for (int ks = 0; ks < nk && ok; ++ks) {
                        const uint32_t b = unit & 1u;
                        const bool first = (ks % SH::CHUNK_STEPS) == 0;
                        if (first && unit >= 2) {
                            // the epilogue has read this accumulator set's previous use
                            if (!(ok = mbar_wait_bounded(tempty(b), ((unit >> 1) - 1) & 1u, wait_limit, abort))) break;
                        }
                        if (!(ok = mbar_wait_bounded(full(stage), phase, wait_limit, abort))) break;
                        tc_fence_after();
                        const uint32_t sa = sbase + stage * SH::STAGE, sbb = sa + S * SH::A_PLANE;
                        const uint32_t acc = tmem + b * SH::ACC;
#pragma unroll 1
                        for (int s = 0; s < S; ++s)
#pragma unroll 1
                            for (int t = 0; s + t < S; ++t)
                                tc_mma(acc + (uint32_t)((s + t) * TN), tc_sdesc(sa + s * SH::A_PLANE, 128, 256),
                                       tc_sdesc(sbb + t * SH::B_PLANE, 128, 256), IDESC, (first && s == 0) ? 0u : 1u);
                        tc_commit(empty(stage));
                        issued = true;
                        if ((ks + 1) % SH::CHUNK_STEPS == 0 || ks + 1 == nk) {
                            tc_commit(tfull(b));
                            ++unit;
                        }
                        if (++stage == SH::NST) { stage = 0; phase ^= 1u; }
                    }
                    if (!ok) { fail(); break; }
                }
            }
            // every MMA this thread issued has completed before TMEM is released
            if (issued) {
                tc_commit(drain);
                int zero = 0;
                mbar_wait_bounded(drain, 0, wait_limit, (volatile int*)&zero);
            }
        }
        __syncwarp();
    } else {
        // ---------------- epilogue (warps 0-7): thread tid holds tile row tid % 128 and the
        // columns of its warpgroup's half, [g HALF, (g + 1) HALF)
        constexpr int HALF = TN / 2;
        const int g = warp >> 2, trow = tid & 127;
        const uint32_t tmem_warp = tmem + ((uint32_t)((warp & 3) * 32) << 16) + (uint32_t)(g * HALF);
        uint32_t unit = 0;
        bool live = true;
        TcTile T = blockIdx.x < ntiles ? tiles[blockIdx.x] : TcTile{};
        for (int ti = blockIdx.x; ti < ntiles && live; ti += gridDim.x) {
            const TcTile cur = T;
            if (ti + (int)gridDim.x < ntiles) T = tiles[ti + gridDim.x];  // the next tile's record, early
            const int row = cur.r0 + trow;
            const bool row_ok = row < cur.rows;
            epi_sync();  // the previous tile's readers of coff / roff / ecol / outs are done
            // C offsets along the tile's rows and columns, while the MMAs run
            if (g == 0) roff[trow] = row_ok ? tab_at(tab, cur.rtab, row) : 0;
            else if (trow < TN) coff[trow] = (cur.c0 + trow < cur.cols) ? tab_at(tab, cur.ctab, cur.c0 + trow) : 0;
            for (int p = cur.p0; p < cur.p1 && live; ++p) {
                const TcPair P = tpairs[p];
                const int nchunks = (P.nk + SH::CHUNK_STEPS - 1) / SH::CHUNK_STEPS;
                const int erow = row_ok ? exps[P.rexp + row] : 0;
                if (p > cur.p0) epi_sync();  // the previous pair's readers of ecol are done
                if (tid < TN) ecol[tid] = (cur.c0 + tid < cur.cols) ? exps[P.cexp + cur.c0 + tid] : 0;
                long long tot[HALF];
#pragma unroll
                for (int j = 0; j < HALF; ++j) tot[j] = 0;
                for (int ch = 0; ch < nchunks; ++ch) {
                    const uint32_t b = unit & 1u;
                    // one thread waits, the named barrier hands the outcome (and the ordering) to all
                    // (two flag slots: a slot is rewritten only two barriers after it was read)
                    if (tid == 0) {
                        const bool ok = stuck_test ? mbar_wait_bounded(stuck, 0, wait_limit, abort)
                                                   : mbar_wait_bounded(tfull(b), (unit >> 1) & 1u, wait_limit, abort);
                        if (!ok) fail();
                        epi_ok[unit & 1u] = ok ? 1 : 0;
                    }
                    epi_sync();
                    if (!epi_ok[unit & 1u]) { live = false; break; }
                    tc_fence_after();
                    {
                        // all S diagonals of this thread's columns, one wait for the lot
                        uint32_t r[S][HALF];
#pragma unroll
                        for (int d = 0; d < S; ++d) tc_ld16(tmem_warp + b * SH::ACC + (uint32_t)(d * TN), r[d]);
                        tc_wait_ld();
#pragma unroll
                        for (int d = 0; d < S; ++d)
#pragma unroll
                            for (int j = 0; j < HALF; ++j)
                                // |acc| < 2^24: the 32-bit conversion is exact
                                tot[j] += (long long)__float2int_rn(__uint_as_float(r[d][j])) << (7 * (S - 1 - d));
                    }
                    tc_fence_before();
                    mbar_arrive(tempty(b));
                    ++unit;
                }
                if (!live) break;
                epi_sync();  // ecol written
#pragma unroll
                for (int j = 0; j < HALF; ++j) {
                    const int jj = g * HALF + j;
                    const double v = scaled_i64(tot[j], erow + ecol[jj] - 7 * S - 7);
                    double* o = outs + trow * SH::LDO + jj;
                    *o = (p == cur.p0) ? v : *o + v;
                }
            }
            if (!live) break;
            epi_sync();  // every row's results and the offsets are in shared memory
            if (!cur.swap) {
                // tile rows run along C's first (fastest) output index: thread = row
                if (row_ok) {
                    double* base = C + cur.coff + roff[trow];
#pragma unroll 4
                    for (int j = 0; j < HALF; ++j) {
                        const int jj = g * HALF + j;
                        if (cur.c0 + jj < cur.cols) base[coff[jj]] = outs[trow * SH::LDO + jj];
                    }
                }
            } else {
                // tile columns run along C's fastest index: lane = column, one warp per row
                for (int rr = warp; rr < SH::TM && cur.r0 + rr < cur.rows; rr += SH::EPI_WARPS) {
                    double* base = C + cur.coff + roff[rr];
#pragma unroll
                    for (int c = lane; c < TN; c += 32)
                        if (cur.c0 + c < cur.cols) base[coff[c]] = outs[rr * SH::LDO + c];
                }
            }
        }
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (warp == SH::ISSUER) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(SH::TMEM_COLS));
}
