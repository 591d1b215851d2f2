// Contraction engine and per-context state.
//
// A contraction C = A*B of block-sparse tensors runs in two phases:
//   plan  -- block-pair matching, output-block set and offsets, computed on
//            the device (planner kernel), then the GEMM work tables;
//            cached by block structure so repeated applies (Davidson) reuse it;
//   exec  -- one grouped launch over all output tiles: every output tile walks
//            the block pairs that feed its block, so each output element is
//            written once (no atomics, deterministic order).
// Reference: doTask(Contract,QDense,QDense) itensor/itdata/qdense.cc:671-743,
// getContractedOffsets itensor/itdata/qutil.h:93-242,
// loopContractedBlocks itensor/itdata/qutil.h:244-371,
// contract(CProps,...) itensor/tensor/contract.cc:733-824.
#pragma once
#include "tensor.h"
#include <atomic>
#include <utility>
#include <mutex>
#include <shared_mutex>

namespace itg {

struct PairRec {          // one (A block, B block) product feeding an output block
    int64_t aoff, boff;   // element offsets of the two blocks
    int32_t tam, tak;     // table positions: A offsets along m and along k
    int32_t tbk, tbn;     // table positions: B offsets along k and along n
    int32_t K;            // contracted extent
    int32_t ia, ib;       // operand-panel records of the two blocks (split-precision path)
    int32_t pad;
};
// One operand block seen as a rows x K matrix (rows = A's m or B's n), for the
// split-precision path: K padded to Kp (multiple of 16), one power-of-two
// exponent per row, and per digit plane a tiled panel: k-steps of 16
// outermost, then groups of 8 rows, then the two 8-k halves of the step, each
// an 8 rows x 8 k core matrix (16 bytes per row). One k-step of 8g rows is
// then one contiguous run of g x 256 bytes laid out exactly as the tensor
// cores read a K-major operand without swizzle (core matrices 128 B apart
// along k, 256 B apart along the rows), so it moves with one bulk copy.
struct OpBlockRec {
    int64_t src;          // element offset of the block in the operand
    int64_t panel;        // bf16 element offset of digit plane 0 in the panel buffer
    int32_t rows, K, Kp;
    int32_t trow, tcol;   // table positions: offsets along rows and along k
    int32_t exp;          // position of the row exponents in the exponent buffer
};
#ifdef __CUDACC__
#define ITG_HD __host__ __device__ __forceinline__
#else
#define ITG_HD inline
#endif
ITG_HD int panel_row_groups(int rows) { return (rows + 7) >> 3; }
// element offset of digit (row r, k) in a block's tiled panel of nrg row groups
ITG_HD int64_t panel_off(int r, int k, int nrg) {
    return ((int64_t)(k >> 4) * nrg + (r >> 3)) * 128 + ((k >> 3) & 1) * 64 + (r & 7) * 8 + (k & 7);
}
struct PrepItem {         // rows [r0, r1) of operand block `op`; which = 0 (A) or 1 (B)
    int32_t op, r0, r1, which;
};
struct CBlockRec {        // output block
    int64_t coff;
    int32_t tcm, tcn;     // table positions: C offsets along m and along n
    int32_t M, N;
};
struct ItemRec {          // one output tile (TILE x TILE) of one output block
    int32_t c, m0, n0, p0, p1;
};
// One output tile of the tensor-core (tcgen05) split-precision kernel: 128
// rows along the block's longer side (swap = 0: C's m, A's rows; swap = 1: C's
// n, B's rows) times TC_TILE_N columns along the other side. Everything a tile
// needs is in the record (no chain of dependent loads per tile).
struct TcTile {
    int64_t coff;          // C block offset
    int32_t rtab, ctab;    // table positions of C's offsets along the tile's rows and columns
    int32_t rows, cols;    // the block's extent along the tile's rows and columns
    int32_t r0, c0;        // first row and column of the tile
    int32_t p0, p1;        // the block's pairs in the tensor-core pair list
    int32_t swap, pad;
};
// A block pair seen from the tile's rows and columns: the digit panels and
// row exponents of the row-side and column-side operand blocks.
struct TcPair {
    int64_t rpanel, cpanel;  // panel offsets (elements) of both blocks
    int32_t rexp, cexp;      // their row exponents' offsets
    int32_t nrg_r, nrg_c;    // their row groups of 8
    int32_t nk, pad;         // k-steps of 16
};
constexpr int TC_TILE_M = 128;
constexpr int TC_TILE_N = 32;

// Offset tables ("table positions" above): the element offsets of a block's
// rows (or columns, or contracted positions) in enumeration order, stored as
// tab[pos] = P, tab[pos+1] = s, then hi[0..]: entry m = (m mod P) * s + hi[m / P].
// P covers the leading dimensions that are contiguous in units of s, so a
// block whose fused dimensions are all contiguous has a single hi entry and a
// table of three integers instead of one per element.
#ifdef __CUDACC__
__device__ __forceinline__ int32_t tab_at(const int32_t* __restrict__ tab, int32_t pos, int32_t m) {
    const int32_t P = __ldg(tab + pos), s = __ldg(tab + pos + 1);
    if (m < P) return m * s + __ldg(tab + pos + 2);
    const int32_t q = m / P;
    return (m - q * P) * s + __ldg(tab + pos + 2 + q);
}
#endif

constexpr int GEMM_TILE = 32;

struct Plan {
    std::shared_ptr<Layout> C;       // output layout
    DevBufPtr dev;                   // packed device tables
    ItemRec* d_items = nullptr;
    PairRec* d_pairs = nullptr;
    CBlockRec* d_cblk = nullptr;
    int32_t* d_tab = nullptr;
    int nitems = 0, npairs = 0, ncblk = 0;
    double flops = 0;                // sum over block pairs of 2*M*N*K
    int64_t bytes_ab = 0;            // elements of A and B blocks touched
    int maxK = 0;                    // largest summed K of one output block
    int max_pair_K = 0;              // largest K of one block pair
    double avgK = 0;
    bool scalar = false;             // rank-0 result
    bool skinny = false;             // every output block is <= 8 columns wide (row tiles)
    int skinny_r = 4;                // rows per thread of the skinny kernel (row tile = 256 * skinny_r)
    bool skinny_wide = false;        // few rows: 32-row tiles, the block pairs spread over a CTA's warps
    // split-precision operand panels (A blocks, then B blocks)
    OpBlockRec* d_ops = nullptr;
    PrepItem* d_prep = nullptr;
    int nprep = 0, nprepA = 0;      // prep items: A operand first, then B
    int nopsA = 0, nopsB = 0;
    int64_t panel_elems = 0;         // bf16 elements per digit plane set (all blocks)
    int64_t exp_elems = 0;
    int max_rows = 0;
    // Tables of the other split-GEMM tile shapes, built on their first use
    // (autotuning or a forced variant; ensure_variant_tables) from what the
    // planner keeps here: most plans only ever run the 32 x 32 tiles.
    struct VariantSource {
        std::vector<CBlockRec> cblk;
        std::vector<int> cp0, cp1;           // pair range of each output block
        std::vector<double> cost;            // tile order key of each output block
        std::vector<int> pia, pib;           // operand blocks of each pair
        std::vector<OpBlockRec> ops;
    };
    mutable std::shared_ptr<VariantSource> vsrc;
    mutable DevBufPtr dev_variants;
    mutable std::mutex vmu;
    mutable std::atomic<bool> variants_ready{false};
    // 64-row tiles of the same output blocks (the 64 x 32 split-precision variant)
    mutable ItemRec* d_items64 = nullptr;
    mutable int nitems64 = 0;
    // 128 x TC_TILE_N tiles of the tensor-core (tcgen05) variant and its view of the pairs
    mutable TcTile* d_items_tc = nullptr;
    mutable TcPair* d_pairs_tc = nullptr;
    mutable int nitems_tc = 0;
    // split-precision GEMM variant picked by the autotuner (-1: not tuned, run variant 0)
    mutable std::atomic<int> oz_variant{-1};
    // split-precision executions so far (a plan is tuned only once it is reused)
    mutable std::atomic<int> split_uses{0};
};
struct Ctx;
// Builds and uploads the 64-row and tcgen05 tile tables of a plan if they are
// not there yet (waits for the upload, so any stream may then use them).
void ensure_variant_tables(Ctx& ctx, Plan const& p);

// Plans keyed by block structure. One cache may serve several contexts (the
// solver pool shares one across its slots): lookups and inserts are locked,
// builds are not (two contexts may build the same plan; the second insert is
// dropped). A plan's tables are immutable once inserted.
// Plans by block structure, shared by a context or by all slots of a solver
// pool. Split into shards by key hash, each with its own lock, so the pool's
// threads rarely touch the same lock word.
struct PlanCache {
    static constexpr int NSHARD = 32;
    struct alignas(128) Shard {
        std::shared_mutex mu;   // lookups (the common case) share the lock
        std::unordered_map<std::string, std::shared_ptr<Plan>> map;
    };
    Shard shard[NSHARD];
    size_t limit = 32768;       // plans in all shards together
    // the shard from the key's length and a sample of its bytes (keys run to
    // tens of kilobytes; the map hashes the whole key once more itself)
    Shard& of(std::string const& key) {
        uint64_t h = key.size() * 0x9E3779B97F4A7C15ull;
        const size_t step = key.size() / 16 + 1;
        for (size_t i = 0; i < key.size(); i += step) h = (h ^ (unsigned char)key[i]) * 0x100000001B3ull;
        return shard[(h >> 7) % NSHARD];
    }
    std::shared_ptr<Plan> find(std::string const& key) {
        Shard& s = of(key);
        std::shared_lock<std::shared_mutex> g(s.mu);
        auto it = s.map.find(key);
        return it == s.map.end() ? nullptr : it->second;
    }
    std::shared_ptr<Plan> insert(std::string key, std::shared_ptr<Plan> p) {
        Shard& s = of(key);
        std::unique_lock<std::shared_mutex> g(s.mu);
        if (s.map.size() >= limit / NSHARD) s.map.clear();
        return s.map.emplace(std::move(key), std::move(p)).first->second;
    }
    size_t size() {
        size_t n = 0;
        for (auto& s : shard) {
            std::shared_lock<std::shared_mutex> g(s.mu);
            n += s.map.size();
        }
        return n;
    }
    void clear() {
        for (auto& s : shard) {
            std::unique_lock<std::shared_mutex> g(s.mu);
            s.map.clear();
        }
    }
};

struct ProfRec {          // one timed GEMM launch (profiling mode)
    cudaEvent_t start, stop;
    double flops;
    int kind;             // 0 FP64, 1 Ozaki BF16
    int nitems;
};

struct Ctx {
    int device = 0;
    bool profiling = false;
    std::vector<ProfRec> prof;
    cudaStream_t stream = nullptr;
    std::string last_error;
    // host-mapped pinned buffer the planner kernel writes its result into
    void* pin = nullptr;
    void* pin_dev = nullptr;
    size_t pin_bytes = 0;
    // pinned staging buffer for host->device table uploads
    void* stage = nullptr;
    size_t stage_bytes = 0;
    // Pinned staging ring for uploads that do not wait for the stream: two
    // halves, a half reused only after the copies enqueued from it completed.
    char* ring = nullptr;
    char* ring_dev = nullptr;  // the ring's device address (mapped, page-locked)
    size_t ring_half = 0, ring_off = 0;
    int ring_cur = 0;
    cudaEvent_t ring_ev[2] = {};
    bool ring_pending[2] = {};
    std::shared_ptr<PlanCache> plans = std::make_shared<PlanCache>();
    // split-precision digit panels of exec_plan: one growing buffer per context
    // (launches on this stream are ordered, so every exec reuses it)
    DevBufPtr split_scratch;
    // event used by sync() when the calling thread multiplexes solves
    cudaEvent_t sync_event = nullptr;
    // status word in host-mapped memory: a kernel whose bounded wait gave up
    // sets it (and returns); sync() turns it into ERR_TIMEOUT
    int* err_host = nullptr;
    int* err_dev = nullptr;
    // freed buffers of this stream, reused by its next allocations
    std::shared_ptr<BlockCache> cache;
    // partial sums + completion counter of the fused reductions (ops.cu)
    DevBufPtr reduce_buf;
    void ensure_reduce();
    // Scalar slots of the device-resident reductions (Davidson): each result
    // is written to device memory, where later kernels read it as a
    // coefficient, and to a host-mapped mirror the host reads after a sync().
    static constexpr int NSCALAR = 128;
    double* scal_host = nullptr;   // host view of the mapped mirror
    double* scal_map = nullptr;    // device view of the mapped mirror
    DevBufPtr scal_dev;            // device copy (read by kernels)
    void ensure_scalars();
    // side streams for independent launches inside one operation (created on
    // first use; work forked to them is joined back before the operation
    // returns, and uses only buffers allocated on `stream` before the fork)
    static constexpr int NSIDE = 4;
    cudaStream_t side[NSIDE] = {};
    cudaEvent_t side_done[NSIDE] = {};
    cudaEvent_t fork_event = nullptr;
    cudaStream_t side_stream(int i);
    void fork();                 // side streams wait for the work enqueued on `stream` so far
    void join(int nused);        // `stream` waits for side streams 0..nused-1
    // pinned host area for device -> host copies enqueued now and read after a
    // later sync(), so that two reads share one wait (the eigensolver's
    // convergence status rides on the eigenvalue read of the bond split)
    static constexpr size_t DEFER0 = 16 << 10;  // carved from the status word's allocation
    void* defer_host = nullptr;
    size_t defer_bytes = 0;
    bool defer_own = false;  // grown past DEFER0: an allocation of its own
    void* ensure_defer(size_t bytes);
    // Davidson: the last call stopped on its convergence test before its last
    // iteration, so the next call waits for each residual before enqueuing
    // the next vector (a timing hint only: results are the same either way)
    bool dav_stopped_early = false;
    // counters
    uint64_t host_waits = 0;
    uint64_t kernel_launches = 0;
    uint64_t plans_built = 0, plan_hits = 0;
    double flops_done = 0;
    int precision = PREC_F64;
    int ozaki_slices = 6;
    int gemm_variant = -1;           // split-precision GEMM variant override (-1: autotuned per plan)
    int sm_count = 152;
    // set while heff_program captures its launches into a graph: launch_pdl
    // then launches without the programmatic-dependency attribute
    bool capturing = false;

    explicit Ctx(int dev);
    ~Ctx();
    void ensure_pin(size_t bytes);
    void ensure_stage(size_t bytes);
    // n bytes of the staging ring, valid until the copies enqueued from them
    // on `stream` have run (the caller enqueues them before its next take)
    char* stage_ring(size_t n);
    // host -> device copy through the ring, without waiting
    void upload(void* dst, void const* src, size_t n);
    // dst <- n bytes staged at st (a stage_ring pointer), by a copy kernel that
    // reads the ring through its device address (launched like the other small
    // kernels, so a table upload does not break their launch overlap)
    void ring_copy(void* dst, char const* st, size_t n);
    // waits for an event recorded on this context's streams (yields in a fiber)
    void wait_event(cudaEvent_t ev);
    // Waits for the stream. Inside a solver-pool fiber the wait yields to the
    // thread's other solves until the stream's work is done.
    void sync();
    // Device -> host copy through the pinned buffer, waiting as sync() does.
    void d2h(void* dst, void const* src, size_t bytes);
    // Split-precision scratch of at least `bytes` (grown on this stream).
    void* split_buffer(size_t bytes);
};

// Labels: which A index matches which B index (ITensor computeLabels semantics).
struct Match {
    std::vector<int> a_con, b_con;   // contracted positions, in A's order
    std::vector<int> a_unc, b_unc;   // uncontracted positions
};
Match match_indices(std::vector<Index> const& A, std::vector<Index> const& B);

// Builds (or fetches from the cache) the plan for C = A*B. If `target` is
// given, C is produced in that layout (any index order, any superset of the
// produced blocks; blocks with no contributing pair are written as zeros).
std::shared_ptr<Plan> get_plan(Ctx& ctx, Layout const& A, Layout const& B, Match const& mt,
                               std::shared_ptr<Layout> target = nullptr);
// Runs a plan: C = A*B with the given arithmetic.
void exec_plan(Ctx& ctx, Plan const& p, double const* A, double const* B, double* C, int prec);

// ITensor operator*: contracts every index common to A and B.
Tensor contract(Ctx& ctx, Tensor const& A, Tensor const& B, int prec = -1,
                std::shared_ptr<Layout> target = nullptr);

// FP64 kernels of a plan (skinny or tiled), no scratch, no allocation (contract.cu).
void exec_plan_f64_only(Ctx& ctx, Plan const& p, double const* A, double const* B, double* C);
// Split-precision exec with the fixed device scratch array instead of pool
// memory (noalloc.cu); allocates nothing.
void exec_plan_noalloc(Ctx& ctx, Plan const& p, double const* A, double const* B, double* C, int S);

// Split-precision prep + GEMM launches for a plan (ozaki.cu); panels/exps are
// the plan's scratch (S digit planes of the padded panel size, row exponents).
void launch_ozaki(Ctx& ctx, Plan const& p, double const* A, double const* B, double* C, int S, __nv_bfloat16* panels,
                  int32_t* exps, bool prep_b = true);
// One split-precision contraction of a grouped launch (launch_ozaki_group):
// its plan tables, operands, digit-panel scratch and output, and where its
// prep items and output tiles start in the group's grids.
struct GroupRef {
    const PrepItem* prep;
    const OpBlockRec* ops;
    const int32_t* tab;
    const ItemRec* items;
    const PairRec* pairs;
    const CBlockRec* cblk;
    const double* A;
    const double* B;
    double* C;
    __nv_bfloat16* panels;
    int32_t* exps;
    int64_t plane;
    int32_t prep_start, tile_start;
};
// The same for FP64 contractions (gemm_f64_kernel tiles; contract.cu).
void launch_f64_group(cudaStream_t stream, GroupRef const* refs, int nrefs, int total_tiles);
// Prep and GEMM of every contraction in refs (device memory, prefix
// positions filled in) as one launch each, on `stream` (ozaki.cu).
void launch_ozaki_group(cudaStream_t stream, GroupRef const* refs, int nrefs, int total_prep, int total_tiles, int S);
// Inside a solver-pool fiber whose scheduler groups launches: hands the
// contraction (split precision with S slices, or FP64 tiles when S == 0) to
// the thread's next grouped launch and yields until it is enqueued (the
// context's stream then waits for it); returns false when grouping is off,
// and the caller launches it alone (fiber.cpp).
bool fiber_group_contract(Ctx& ctx, Plan const& p, double const* A, double const* B, double* C, int S,
                          __nv_bfloat16* panels, int32_t* exps, bool prep_b);
// The tensor-core variant of the split-precision GEMM (ozaki_tc.cu): digit
// panels staged into shared memory, tcgen05.mma with the diagonal sums in
// tensor memory. Panels and exponents must be in place (the prep has run).
void launch_ozaki_tc(Ctx& ctx, Plan const& p, double* C, int S, __nv_bfloat16 const* panels, int64_t plane,
                     int32_t const* exps);
// Times every split-precision GEMM variant of the plan on these operands and
// stores the fastest in p.oz_variant (ozaki.cu); C is overwritten.
int autotune_ozaki(Ctx& ctx, Plan const& p, double const* A, double const* B, double* C, int S,
                   __nv_bfloat16* panels, int32_t* exps);
// Plans with at least this many algorithmic flops are tuned: a prepared H_eff
// program tunes on its first run, exec_plan once a plan has run
// AUTOTUNE_MIN_USES times (tuning costs about sixteen executions, which a
// plan used for one Davidson call never pays back).
constexpr double AUTOTUNE_MIN_FLOPS = 2e7;
constexpr int AUTOTUNE_MIN_USES = 32;
// Whether exec_plan runs this plan with the split-precision kernels.
// (The int64 digit sums of one block pair are exact up to K = 8192.)
constexpr int SPLIT_MAX_PAIR_K = 8192;
// Below this many algorithmic flops a contraction runs the FP64 kernel even in
// the split precision: slicing both operands costs more than the FP64 GEMM it
// would replace (measured crossover ~1e7 flops on GB300). ITG_SPLIT_MIN_FLOPS
// overrides it (0: every eligible contraction takes the split kernels).
double split_min_flops();
inline bool plan_uses_split(Plan const& p, int prec) {
    return !p.skinny && prec == PREC_OZAKI_BF16 && p.avgK >= 8.0 && p.npairs > 0 && p.max_pair_K <= SPLIT_MAX_PAIR_K &&
           p.flops >= split_min_flops();
}
// Bytes of split-precision scratch (digit planes + row exponents) a plan needs.
// The tensor-core kernel copies whole 128-row (or TC_TILE_N-row) k-steps: the
// rows past a block's end come from whatever follows it (they only feed
// output rows that are never stored), and at the very end of the scratch
// they come from this padding.
constexpr size_t SPLIT_SCRATCH_PAD = 2 * TC_TILE_M * 16 * sizeof(__nv_bfloat16);
inline size_t split_scratch_bytes(Plan const& p, int S) {
    const int64_t plane = (p.panel_elems + 15) / 16 * 16;
    return sizeof(__nv_bfloat16) * (size_t)plane * S + sizeof(int32_t) * (size_t)(p.exp_elems + 4) +
           SPLIT_SCRATCH_PAD;
}

// TFLOP/s of [FP64 FFMA, FP32 FFMA, FP64 mma.sync, TF32 mma.sync, BF16 mma.sync] (peaks.cu)
void measure_peaks(Ctx& ctx, double* tflops);

// ---- kernels launched from other translation units (ops.cu)
void launch_fill(Ctx& ctx, double* x, int64_t n, double v);
void launch_scale(Ctx& ctx, double* x, int64_t n, double a);
// dst = src (n doubles, device memory), as a kernel on the context's stream
void launch_copy(Ctx& ctx, double* dst, double const* src, int64_t n);
void launch_axpy(Ctx& ctx, double* y, double const* x, int64_t n, double a);          // y += a x
void launch_axpby(Ctx& ctx, double* y, double const* x, int64_t n, double a, double b); // y = a x + b y
// dot products of x with each of nv vectors V[k] (device pointers); result to host
void dots(Ctx& ctx, double const* const* V, int nv, double const* x, int64_t n, double* out);
double dot(Ctx& ctx, double const* a, double const* b, int64_t n);
double norm(Ctx& ctx, double const* a, int64_t n);
// Up to MAX device vectors with coefficients, passed to kernels by value. A
// coefficient is c[k], or c[k] times scalar slot cs[k] of the context when
// cs[k] >= 0 (a value an earlier kernel left on the device).
struct VecList {
    static constexpr int MAX = 24;
    double const* p[MAX];
    double c[MAX];
    int cs[MAX];
    int n = 0;
    void add(double const* x, double a, int slot = -1) { p[n] = x; c[n] = a; cs[n] = slot; ++n; }
};
// y = a0 y + sum_k c_k X_k in one launch (y is not read when a0 == 0); returns
// |y|^2 when want_norm (then waits for the stream), else 0.
double combo(Ctx& ctx, double* y, double a0, VecList const& X, int64_t n, bool want_norm);
// The same without waiting: |y|^2 goes to scalar slot norm_slot (none if < 0).
void combo_async(Ctx& ctx, double* y, double a0, VecList const& X, int64_t n, int norm_slot);
// Dot products of x with each vector of V into scalar slots slot, slot+1, ...
// (no wait; coefficients of V are ignored).
void dots_async(Ctx& ctx, VecList const& V, double const* x, int64_t n, int slot);
// x *= 1 / sqrt(max(s, 0)), s = scalar slot norm_slot (no wait).
void scale_rnorm(Ctx& ctx, double* x, int64_t n, int norm_slot);
// x /= |x| when |x| > min_norm, without waiting: |x|^2 in the last scalar
// slot (Ctx::NSCALAR - 1, which Davidson does not use), then one scaling
// kernel that reads it.
void normalize_async(Ctx& ctx, double* x, int64_t n, double min_norm);
// General block permute / gather: dst[dst_off[e]] = src[src_off[e]] described per
// block by offset tables (see ops.cu). Used for combiner, uncombine and
// layout changes.
struct GatherPlan;
void launch_gather(Ctx& ctx, GatherPlan const& g, double const* src, double* dst);


#ifdef __CUDACC__
// Programmatic dependent launch. A kernel launched by launch_pdl may begin
// while the previous kernel on its stream is still running, so its launch
// latency hides behind that kernel (back to back on this part: an empty kernel
// 2.06 -> 1.39 us per launch, a small dot-product kernel 4.10 -> 1.8 us).
// Such a kernel calls pdl_wait() before it touches global memory:
// griddepcontrol.wait returns once the previous grid has completed and its
// writes are visible, so stream order holds; in a kernel launched without the
// attribute it returns at once.
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

template <typename... KArgs, typename... Args>
inline void launch_pdl(Ctx& ctx, dim3 grid, dim3 block, size_t smem, void (*kernel)(KArgs...), Args&&... args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = ctx.stream;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    // not under graph capture: a graph replay already starts its kernels back
    // to back (measured: the m = 1024 apply's replay time did not change with
    // the attribute captured)
    cfg.numAttrs = ctx.capturing ? 0 : 1;
    ITG_CHECK_CUDA(cudaLaunchKernelEx(&cfg, kernel, std::forward<Args>(args)...));
}
#endif

}  // namespace itg
