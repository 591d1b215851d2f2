/*
 * itg.h -- C-ABI of the GB300 (sm_103a) device path for ITensor's two-site DMRG
 * inner loop: block-sparse QN contraction, effective-Hamiltonian apply,
 * Davidson, density-matrix bond split and the DMRG sweep driver.
 *
 * Conventions (shared with ITensor's QDense storage, itensor/itdata/qdense.h:34-187):
 *   - a block is named by one sector number per index (0-based); blocks are
 *     dense, column-major (first index fastest), ordered by reversed-
 *     lexicographic coordinates and packed back to back;
 *   - an index is (id, prime level, arrow, QN sectors); two indices contract
 *     when id and prime level agree;
 *   - a QN holds 4 integer slots; slot k is reduced modulo qn_mod[k] when
 *     |qn_mod[k]| > 1 (Z_n), is a plain integer when |qn_mod[k]| == 1, and is
 *     unused when qn_mod[k] == 0. Negative moduli mark fermionic U(1) numbers
 *     (bookkeeping only, as in itensor/qn.h:36-60).
 *
 * Every function returns an int status (ITG_OK = 0); no C++ exception crosses
 * the boundary. itg_last_error() gives the message of the last failure on a
 * context. A context owns one CUDA stream; calls on one context must not be
 * made from two host threads at once. Device pointers passed in are never
 * freed by the library.
 */
#ifndef ITG_H
#define ITG_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
    ITG_OK = 0,
    ITG_ERR_ARG = 1,       /* malformed arguments or block metadata */
    ITG_ERR_CUDA = 2,      /* CUDA runtime error */
    ITG_ERR_OOM = 3,       /* device allocation failed */
    ITG_ERR_NOCONV = 4,    /* eigensolver hit its sweep cap */
    ITG_ERR_TIMEOUT = 5,   /* a bounded device-side wait gave up */
    ITG_ERR_INTERNAL = 6,
    ITG_ERR_RANGE = 7      /* size beyond a stated maximum */
};

enum {
    ITG_PREC_F64 = 0,        /* plain FP64 -- the drop-in path */
    ITG_PREC_OZAKI_BF16 = 1  /* FP64 operands as exact BF16 integer slices, FP32-exact accumulation */
};

typedef struct itg_ctx itg_ctx;
typedef struct itg_tensor itg_tensor;
typedef struct itg_plan itg_plan;
typedef struct itg_dmrg_result itg_dmrg_result;

typedef struct {
    uint64_t id;
    int32_t plev;
    int32_t dir;            /* +1 Out, -1 In */
    int32_t nsect;
    const int32_t* qn;      /* nsect * 4 values */
    const int32_t* qn_mod;  /* 4 moduli */
    const int32_t* dims;    /* nsect sector sizes */
} itg_index_desc;

/* ---------------------------------------------------------------- context */
int itg_create(int device, itg_ctx** out);
void itg_destroy(itg_ctx* ctx);
const char* itg_last_error(itg_ctx* ctx);
int itg_synchronize(itg_ctx* ctx);
/* Default arithmetic of the block GEMMs; ozaki_slices in 3..6. */
int itg_set_precision(itg_ctx* ctx, int mode, int ozaki_slices);
/* Tile shape of the split-precision block GEMM: -1 (default) lets the
 * autotuner time every variant on a plan's first large use and keep the
 * fastest; 0..3 forces the mma.sync kernel with 32x32 tiles, 64x32 tiles,
 * persistent 32x32, persistent 64x32; 4 the tcgen05 kernel (128 x 32 tiles,
 * TMEM accumulators). All variants give bit-identical results. */
int itg_set_gemm_variant(itg_ctx* ctx, int variant);
int itg_stats(itg_ctx* ctx, uint64_t* kernel_launches, double* gemm_flops, uint64_t* plans_built,
              uint64_t* plan_hits);
int itg_reset_stats(itg_ctx* ctx);
/* The CUDA stream (cudaStream_t) all work of this context is ordered on. */
void* itg_stream(itg_ctx* ctx);
/* Per-launch timing of the block-GEMM launches (CUDA events on the context
 * stream) between begin and end: n launches (capacity *n on input), their
 * durations in ms, algorithmic flops (sum of 2MNK) and arithmetic kind
 * (0 FP64, 1 Ozaki BF16). */
/* Issue-rate microbenchmarks (register-only loops, ~0.3 s): TFLOP/s of
 * [FP64 FFMA, FP32 FFMA, FP64 mma.sync, TF32 mma.sync, BF16 mma.sync]. */
int itg_measure_peaks(itg_ctx* ctx, double* tflops5);
int itg_profile_begin(itg_ctx* ctx);
int itg_profile_end(itg_ctx* ctx, int32_t* n, float* ms, double* flops, int32_t* kind);

/* ---------------------------------------------------------------- tensors
 * Replaces QDense<Real> storage (itensor/itdata/qdense.h:34-60): `coords` are
 * the blocks in storage order (nblocks x rank), data packed in that order.
 * data_is_device != 0: `data` is a device pointer (copied on the context stream). */
int itg_tensor_create(itg_ctx* ctx, int32_t rank, const itg_index_desc* inds, int32_t nblocks, const int32_t* coords,
                      const double* data, int data_is_device, itg_tensor** out);
void itg_tensor_free(itg_tensor* t);
int itg_tensor_layout(const itg_tensor* t, int32_t* rank, int32_t* nblocks, int64_t* size);
/* Index k: nsect first (call with qn/dims NULL), then the sector data. */
int itg_tensor_index(const itg_tensor* t, int32_t k, uint64_t* id, int32_t* plev, int32_t* dir, int32_t* nsect,
                     int32_t* qn, int32_t* qn_mod, int32_t* dims);
int itg_tensor_blocks(const itg_tensor* t, int32_t* coords, int64_t* offsets);
int itg_tensor_read(itg_ctx* ctx, const itg_tensor* t, double* host);
double* itg_tensor_device_ptr(const itg_tensor* t);
/* Value of a rank-0 tensor (a full contraction). */
int itg_tensor_scalar(const itg_tensor* t, double* value);

/* ---------------------------------------------------------------- contraction
 * ITensor operator* for QN tensors: doTask(Contract,QDense,QDense),
 * itensor/itdata/qdense.cc:671-743 (block matching getContractedOffsets,
 * itensor/itdata/qutil.h:93-242). Output indices: A's uncontracted then B's
 * (contractIS, itensor/indexset_impl.h:77-127); output blocks: exactly those
 * produced by a matching block pair, sorted, packed. */
int itg_contract(itg_ctx* ctx, const itg_tensor* A, const itg_tensor* B, int precision, itg_tensor** C);

/* Raw boundary for a QDense caller that keeps its own storage: layouts as
 * sector sizes + block coordinates, contraction labels in the reference's
 * Lind/Rind convention (negative = contracted, equal negative labels pair up;
 * computeLabels itensor/tensor/contract.h:155-216). Data pointers are device
 * memory laid out as the layouts say. */
typedef struct {
    int32_t rank;
    const int32_t* nsect;      /* rank */
    const int32_t* sect_dims;  /* sum(nsect) sector sizes, index by index */
    int32_t nblocks;
    const int32_t* coords;     /* nblocks x rank, storage order */
} itg_layout_desc;
int itg_contract_plan(itg_ctx* ctx, const itg_layout_desc* A, const int32_t* labelsA, const itg_layout_desc* B,
                      const int32_t* labelsB, itg_plan** plan);
int itg_plan_output(const itg_plan* plan, int32_t* rank, int32_t* nblocks, int64_t* size);
int itg_plan_output_blocks(const itg_plan* plan, int32_t* coords, int64_t* offsets);
int itg_plan_flops(const itg_plan* plan, double* flops);
int itg_contract_exec(itg_ctx* ctx, const itg_plan* plan, const double* A, const double* B, double* C, int precision);
/* A plan's device tables belong to the context that built it and are freed on
 * its stream: free a plan only after the work of every context that ran it. */
void itg_plan_free(itg_plan* plan);

/* No counterpart in the reference: an allocation-free variant of
 * itg_contract_exec with the split-precision arithmetic (slices 3..6).
 * For callers that cannot let a library allocate device memory during a call
 * (another framework's allocator owns the device pool, a real-time loop cannot
 * take an allocation's implicit synchronisation, a sandbox forbids cudaMalloc
 * after start-up). The plan (built earlier by itg_contract_plan) and the
 * operands are the caller's; the digit-panel scratch lives in one fixed
 * device array of ITG_NOALLOC_SCRATCH_BYTES per device, held until exit.
 * A plan needing more scratch is rejected with ITG_ERR_RANGE. The first call
 * from each CUDA context on a device (the primary context, or one the caller
 * made current) looks up the array's address there (cudaGetSymbolAddress) and
 * should come before any stream capture. Calls share the array: calls that
 * overlap on the GPU race. Nothing in the array needs to start at zero. */
#define ITG_NOALLOC_SCRATCH_BYTES (16u << 20)
int itg_contract_exec_noalloc(itg_ctx* ctx, const itg_plan* plan, const double* A, const double* B, double* C,
                              int slices);

/* ---------------------------------------------------------------- H_eff
 * LocalOp::product, itensor/mps/localop.h:324-365: out = noPrime(((phi*L)*W1)*W2*R)
 * (L or R may be NULL at the chain ends). The output has the block structure
 * the reference produces. */
int itg_heff_apply(itg_ctx* ctx, const itg_tensor* L, const itg_tensor* W1, const itg_tensor* W2, const itg_tensor* R,
                   const itg_tensor* phi, int precision, itg_tensor** out);

/* Prepared H_eff for repeated applies with one (L, W1, W2, R) and one phi
 * block structure: plans resolved once, intermediates preallocated, and with
 * use_graph != 0 the launches replayed as one CUDA graph. out_size receives
 * the number of output elements (the output has the structure itg_heff_apply
 * returns). itg_heff_run reads phi and writes the result through the given
 * pointers; host != 0 means they are host memory (the copies are part of the
 * call, which then returns after the result is written). */
typedef struct itg_heff itg_heff;
int itg_heff_create(itg_ctx* ctx, const itg_tensor* L, const itg_tensor* W1, const itg_tensor* W2, const itg_tensor* R,
                    const itg_tensor* phi, int precision, int use_graph, itg_heff** out, int64_t* out_size,
                    double* flops);
int itg_heff_run(itg_ctx* ctx, itg_heff* h, const double* phi, double* out, int host);
void itg_heff_free(itg_heff* h);

/* davidson (block size 1), itensor/iterativesolvers.h:99-451. Returns the
 * lowest Ritz value and the normalised Ritz vector (on every block of phi's
 * divergence). */
int itg_davidson(itg_ctx* ctx, const itg_tensor* L, const itg_tensor* W1, const itg_tensor* W2, const itg_tensor* R,
                 const itg_tensor* phi, int32_t maxiter, double errgoal, int precision, double* energy,
                 itg_tensor** phi_out);

/* ---------------------------------------------------------------- bond split
 * denmatDecomp, itensor/decomp.h:316-418, with diag_hermitian's QN branch
 * (itensor/hermitian.cc:180-426) and truncate (itensor/decomp.cc:305-463).
 * A and B give the index split (their data is not read). eigs receives the
 * kept density-matrix eigenvalues (capacity *neigs on input, count on output). */
int itg_denmat_decomp(itg_ctx* ctx, const itg_tensor* AA, const itg_tensor* A, const itg_tensor* B, int fromleft,
                      double cutoff, int32_t maxdim, int32_t mindim, int respect_degenerate, int normalize,
                      int precision, itg_tensor** A_out, itg_tensor** B_out, double* truncerr, double* eigs,
                      int32_t* neigs);

/* denmatDecomp with the noise term: rho += noise * deltaRho (LocalOp::deltaRho,
 * itensor/mps/localop.h:375-406) and rho /= trace(rho) (itensor/decomp.h:386-394)
 * when noise > 0. L/W1 (fromleft) or R/W2 (from the right) are the local
 * operator's environment and MPO tensors; L or R may be null at the chain's
 * ends. With noise == 0 this is itg_denmat_decomp. */
int itg_denmat_decomp_noise(itg_ctx* ctx, const itg_tensor* AA, const itg_tensor* A, const itg_tensor* B, int fromleft,
                            const itg_tensor* L, const itg_tensor* W1, const itg_tensor* W2, const itg_tensor* R,
                            double noise, double cutoff, int32_t maxdim, int32_t mindim, int respect_degenerate,
                            int normalize, int precision, itg_tensor** A_out, itg_tensor** B_out, double* truncerr,
                            double* eigs, int32_t* neigs);

/* SVD route of the bond split: svd (itensor/decomp.cc:121-248) with svdImpl's
 * QN branch (itensor/svd.cc:169-401), as MPS::svdBond uses it with UseSVD or
 * cutoff < 1e-12 (itensor/mps/mps_impl.h:50-65). A's indices that B lacks go to
 * U; the singular values (normalised when normalize != 0) are pushed into B
 * (fromleft) or A. eigs receives the kept squared singular values. */
int itg_svd_split(itg_ctx* ctx, const itg_tensor* AA, const itg_tensor* A, const itg_tensor* B, int fromleft,
                  double cutoff, int32_t maxdim, int32_t mindim, int respect_degenerate, int normalize, int precision,
                  itg_tensor** A_out, itg_tensor** B_out, double* truncerr, double* eigs, int32_t* neigs);

/* truncate, itensor/decomp.cc:305-463 (host function, same decisions and
 * values as the reference). P sorted descending; Pout capacity n. */
int itg_truncate(const double* P, int32_t n, int32_t maxdim, int32_t mindim, double cutoff, int absolute_cutoff,
                 int rel_cutoff, int respect_degenerate, double* Pout, int32_t* m, double* truncerr,
                 double* docut_lower, double* docut_upper, int32_t* ndegen);

/* ---------------------------------------------------------------- DMRG driver
 * dmrg(H, psi0, sweeps) with DMRGWorker (itensor/mps/dmrg.h:336-467). The MPO
 * and the initial product state are built from the model description:
 * type 0: S=1/2 chain, H = sum Jz SzSz + J/2 (S+S- + S-S+) (+ J2 on next neighbours), Sz QN, Neel start;
 * type 1: transverse-field Ising, H = -sum SxSx - h sum Sz, parity QN, all-up start;
 * type 2: Hubbard on an Lx x Ly square lattice snaked column by column,
 *         H = -t sum hops + U sum n_up n_dn, (Nf, Sz) QN, Neel start at half filling. */
typedef struct {
    int32_t type;
    int32_t N;
    double J, Jz, J2, h, t, U;
    int32_t Lx, Ly, yperiodic;
} itg_model_desc;

typedef struct {
    int32_t maxdim, mindim;
    double cutoff;
    int32_t niter;
    double noise;    /* >= 0: density-matrix noise term (LocalOp::deltaRho, itensor/mps/localop.h:375-406) */
    int32_t use_svd; /* 1: SVD bond split (noise ignored); 0: SVD only when noise == 0 and cutoff < 1e-12,
                        else density matrix */
} itg_sweep_desc;

int itg_dmrg_run(itg_ctx* ctx, const itg_model_desc* model, const itg_sweep_desc* sweeps, int32_t nsweeps,
                 int precision, itg_dmrg_result** out);
/* Sums of MPOs: dmrg(psi, {H1, H2, ...}, sweeps) with LocalMPOSet
 * (itensor/mps/dmrg.h:181-230, itensor/mps/localmposet.h): H is the sum of the
 * models' Hamiltonians (same site type and length; one MPO each, on shared site
 * indices), the product state from models[0]. With noise, the density
 * matrix gets the sum of every MPO's noise term (itensor/mps/localmposet.h:166-176). */
int itg_dmrg_run_sum(itg_ctx* ctx, const itg_model_desc* models, int32_t nmodels, const itg_sweep_desc* sweeps,
                     int32_t nsweeps, int precision, itg_dmrg_result** out);
/* Excited states: dmrg(H, psis, psi0, sweeps, {"Weight", weight}) of
 * itensor/mps/dmrg.h:245-266 with LocalMPO_MPS (itensor/mps/localmpo_mps.h),
 * chained. State 0 is the ground state from the model's default product
 * state on sweeps[0]; state k >= 1 minimises H + weight * sum_{j<k} |psi_j><psi_j|
 * from the same product state on sweeps[k]. out receives nstates results
 * (each freed with itg_dmrg_free). */
int itg_dmrg_run_states(itg_ctx* ctx, const itg_model_desc* model, int32_t nstates, const itg_sweep_desc* const* sweeps,
                        const int32_t* nsweeps, double weight, int precision, itg_dmrg_result** out);
/* dmrg() on the caller's own MPO and initial MPS, device tensors built with
 * itg_tensor_create (or loaded with itg_mps_file_load): the overloads
 *   dmrg(H, psi0, sweeps)                  itensor/mps/dmrg.h:67-76      nmpo 1, nprev 0
 *   dmrg(std::vector<MPO>{H1,...}, psi0, ..) itensor/mps/dmrg.h:181-230  nmpo > 1 (LocalMPOSet)
 *   dmrg(H, std::vector<MPS>{...}, psi0, .., {"Weight", w})  itensor/mps/dmrg.h:245-266  nprev > 0
 * W holds nmpo x nsites tensors (MPO k's site j at W[k*nsites + j-1]); an MPO
 * tensor carries the site index of psi0[j] unprimed and primed and shares one
 * link with each neighbour (any index order). prev holds nprev x nsites
 * tensors of earlier states on the same sites. The final MPS stays in the
 * result (itg_dmrg_mps); after the last right-to-left half-sweep its
 * orthogonality centre is site 1 (leftLim 0, rightLim 2). New links keep the
 * tags of the links they replace (MPS::svdBond, itensor/mps/mps_impl.h:81-84).
 * Also itg_dmrg_run, _sum and _states keep their final MPS. */
int itg_dmrg_run_mpo(itg_ctx* ctx, int32_t nsites, int32_t nmpo, const itg_tensor* const* W,
                     const itg_tensor* const* psi0, int32_t nprev, const itg_tensor* const* prev, double weight,
                     const itg_sweep_desc* sweeps, int32_t nsweeps, int precision, itg_dmrg_result** out);
/* Site tensor j (1..N) of the final MPS of a result (a new handle on the same
 * device data; free it with itg_tensor_free). */
int itg_dmrg_mps(const itg_dmrg_result* r, int32_t j, itg_tensor** out);
int itg_dmrg_energy(const itg_dmrg_result* r, double* energy);
int itg_dmrg_nbonds(const itg_dmrg_result* r, int32_t* nbonds);
int itg_dmrg_bonds(const itg_dmrg_result* r, int32_t* sweep, int32_t* halfsweep, int32_t* bond, double* energy,
                   double* truncerr, int32_t* dim);
/* Final link index b (1..N-1): sectors (4 QN values each) and sizes. */
int itg_dmrg_link(const itg_dmrg_result* r, int32_t b, int32_t* dir, int32_t* nsect, int32_t* qn, int32_t* dims);
int itg_dmrg_timing(const itg_dmrg_result* r, int32_t* nsweeps, double* sweep_seconds, int32_t* heff_applies);
/* Wall seconds spent in [environments + two-site tensor, Davidson, bond split], summed over all bond steps. */
int itg_dmrg_phases(const itg_dmrg_result* r, double* seconds3);
void itg_dmrg_free(itg_dmrg_result* r);

/* ---------------------------------------------------------------- checkpoints
 * MPS and MPO files in the reference's plain binary layout: what
 * writeToFile(path, psi) and readFromFile(path, psi) read and write
 * (itensor/util/readwrite.h:337-370; MPS::write/read itensor/mps/mps.cc:353-378,
 * ITensor::write/read itensor/itensor.cc:769-803, QDense write/read
 * itensor/itdata/qdense.h:236-248). An MPO file has the same layout. Site
 * tensors must hold QN block-sparse real storage (QDense<Real>).
 * A file object is a host copy: read -> write gives the same bytes.
 * itg_mps_file_load uploads site tensors 1..N (sites receives N handles);
 * QN slot k of the loaded indices holds the quantum number whose name
 * itg_mps_file_info returns k-th (qn_names: 4 x 8 chars, zero padded; names
 * in the reference's order). itg_mps_file_store downloads site tensors and
 * writes QN slot k under the k-th name of the comma-separated qn_names
 * ("Sz", "Nf,Sz", ...); index tags are carried as the tensors hold them. */
typedef struct itg_mps_file itg_mps_file;
int itg_mps_file_read(const char* path, itg_mps_file** out);
int itg_mps_file_write(const itg_mps_file* f, const char* path);
int itg_mps_file_info(const itg_mps_file* f, int32_t* nsites, int32_t* leftlim, int32_t* rightlim, int32_t* nqn,
                      char* qn_names);
int itg_mps_file_load(itg_ctx* ctx, const itg_mps_file* f, itg_tensor** sites);
int itg_mps_file_store(itg_ctx* ctx, int32_t nsites, const itg_tensor* const* sites, int32_t leftlim, int32_t rightlim,
                       const char* qn_names, itg_mps_file** out);
void itg_mps_file_free(itg_mps_file* f);

/* ---------------------------------------------------------------- solver pool
 * Many independent ground-state solves (dmrg() as above, one per request) on
 * one GPU, with continuous batching. Replaces a host loop that calls dmrg()
 * once per Hamiltonian (sample/dmrg.cc:30-65: MPO, MPS(InitState), Sweeps,
 * dmrg(H, psi0, sweeps)), one request after the other.
 *
 * A request carries a model, a sweep schedule, a precision and an arrival
 * time (seconds after itg_pool_start; <= 0 means at once). It is admitted
 * once it has arrived, a slot is free and its device-memory estimate
 * (itg_pool_estimate) fits in what the budget has left; first come, first
 * served. `workers` host threads each hold `slots_per_worker` slots; a slot
 * is a stream of its own, and a worker switches between its solves whenever
 * one waits for its stream, so every admitted solve has work on the GPU.
 * Results are identical to a lone itg_dmrg_run with the same arguments.
 * Requests may be submitted before or after itg_pool_start, from any thread.
 * Errors of the pool calls are read with itg_last_error(NULL). */
typedef struct itg_pool itg_pool;
int itg_pool_create(int device, int32_t workers, int32_t slots_per_worker, double budget_bytes, itg_pool** out);
int itg_pool_submit(itg_pool* p, const itg_model_desc* model, const itg_sweep_desc* sweeps, int32_t nsweeps,
                    int precision, double arrival_s, int64_t* id);
/* A request on the caller's MPO and initial MPS (as itg_dmrg_run_mpo with one
 * MPO): the tensors are copied to host memory during the call (ctx is the
 * context they were made on), so they may be freed afterwards. keep_mps != 0:
 * the result keeps the final MPS (read with itg_pool_result + itg_dmrg_mps;
 * device memory held until the result and the pool are freed). */
int itg_pool_submit_mpo(itg_pool* p, itg_ctx* ctx, int32_t nsites, const itg_tensor* const* W,
                        const itg_tensor* const* psi0, const itg_sweep_desc* sweeps, int32_t nsweeps, int precision,
                        double arrival_s, int keep_mps, int64_t* id);
/* No counterpart in the reference (it has no batched mode; the nearest is the
 * per-output-block loop of itensor/itdata/qutil.h:330-348). Cross-solve
 * grouping, off by default, set before itg_pool_start: the block GEMMs (FP64,
 * or split precision: prep and GEMM) that a worker's solves reach while all
 * of them wait run as one grouped launch covering every solve's blocks,
 * instead of one launch each. Results are identical either way.
 * itg_pool_grouping_stats counts the grouped launches and the contractions
 * they carried. */
int itg_pool_set_grouping(itg_pool* p, int on);
int itg_pool_grouping_stats(itg_pool* p, int64_t* grouped_launches, int64_t* grouped_contractions);
/* No counterpart in the reference. Calibrated admission, set before
 * itg_pool_start (off with min_solves 0, the default): once min_solves
 * requests of a model family (model type, local and MPO bond dimensions,
 * precision) have finished, that family's requests are admitted by
 * estimate x safety x the largest measured peak/estimate ratio of the family
 * (at least 16 MiB, at most the estimate; safety >= 1). A request admitted
 * below its estimate that runs out of device memory is queued again, first in
 * line, by its full estimate. itg_pool_record_admission gives the bytes a
 * request was admitted by and whether it was re-run; itg_pool_calibration_stats
 * counts calibrated admissions and re-runs. */
int itg_pool_set_calibration(itg_pool* p, int32_t min_solves, double safety);
int itg_pool_calibration_stats(itg_pool* p, int64_t* calibrated_admissions, int64_t* retried);
int itg_pool_record_admission(itg_pool* p, int64_t id, double* admitted_bytes, int32_t* retries);
int itg_pool_start(itg_pool* p);
int itg_pool_drain(itg_pool* p);   /* waits until every submitted request has finished */
/* status: -1 queued, -2 running, 0 done, else the request's error code (message in itg_pool_error).
 * Times are seconds after itg_pool_start; latency = t_done - t_arrive. */
int itg_pool_record(itg_pool* p, int64_t id, int32_t* status, double* energy, double* t_arrive, double* t_admit,
                    double* t_done, double* est_bytes, double* peak_bytes, int32_t* worker);
int itg_pool_error(itg_pool* p, int64_t id, char* buf, int32_t buflen);
/* Full result of a finished request, read with the itg_dmrg_* accessors; free with itg_dmrg_free. */
int itg_pool_result(itg_pool* p, int64_t id, itg_dmrg_result** out);
int itg_pool_stats(itg_pool* p, int64_t* submitted, int64_t* done, int64_t* failed, double* peak_reserved_bytes,
                   int32_t* peak_running, double* elapsed_s);
int itg_pool_estimate(const itg_model_desc* model, const itg_sweep_desc* sweeps, int32_t nsweeps, int precision,
                      double* bytes);
/* The same estimate for an MPO request: nsites sites of local dimension
 * site_dim, MPO bond dimension mpo_bond_dim. */
int itg_pool_estimate_mpo(int32_t nsites, int32_t site_dim, int32_t mpo_bond_dim, const itg_sweep_desc* sweeps,
                          int32_t nsweeps, int precision, double* bytes);
void itg_pool_destroy(itg_pool* p);

#ifdef __cplusplus
}
#endif
#endif
