// extern "C" boundary (include/itg.h): converts between the flat C
// descriptions and the host data model, and turns exceptions into status codes.
#include "../../include/itg.h"
#include "pool.h"
#include "mps_io.h"
#include <cstring>

using namespace itg;

struct itg_ctx {
    Ctx ctx;
    explicit itg_ctx(int dev) : ctx(dev) {}
};
struct itg_tensor {
    Tensor t;
};
struct itg_plan {
    std::shared_ptr<Plan> p;
    std::shared_ptr<Layout> C;
};
struct itg_dmrg_result {
    DmrgResult r;
};
struct itg_heff {
    std::shared_ptr<HeffProgram> p;
};

namespace {
thread_local std::string g_error;

template <typename F>
int guard(itg_ctx* c, F&& f) {
    try {
        f();
        return ITG_OK;
    } catch (Error const& e) {
        (c ? c->ctx.last_error : g_error) = e.what();
        return e.code;
    } catch (std::exception const& e) {
        (c ? c->ctx.last_error : g_error) = e.what();
        return ITG_ERR_INTERNAL;
    }
}

Index index_from(itg_index_desc const& d) {
    ITG_REQUIRE(d.nsect > 0 && d.dims && d.qn_mod, "index: missing sectors");
    ITG_REQUIRE(d.dir == 1 || d.dir == -1, "index: dir must be +1 or -1");
    std::vector<QN> qs(d.nsect);
    std::vector<int32_t> dims(d.dims, d.dims + d.nsect);
    for (int s = 0; s < d.nsect; ++s) {
        ITG_REQUIRE(dims[s] > 0, "index: sector size must be positive");
        for (int k = 0; k < QN_SLOTS; ++k) {
            qs[s].mod[k] = d.qn_mod[k];
            qs[s].v[k] = QN::reduce(d.qn ? d.qn[s * QN_SLOTS + k] : 0, d.qn_mod[k]);
        }
    }
    ITG_REQUIRE(d.id != 0, "index: id must be nonzero");
    return Index(qs, dims, d.dir, d.id, d.plev);
}

Tensor const* opt(itg_tensor const* t) { return t ? &t->t : nullptr; }

ModelSpec model_from(itg_model_desc const& d) {
    ModelSpec m;
    m.type = d.type; m.N = d.N;
    m.J = d.J; m.Jz = d.Jz; m.J2 = d.J2; m.h = d.h; m.t = d.t; m.U = d.U;
    m.Lx = d.Lx; m.Ly = d.Ly; m.yperiodic = d.yperiodic;
    return m;
}

std::vector<Tensor> tensors_from(itg_tensor const* const* t, int n, char const* what) {
    ITG_REQUIRE(t, std::string("dmrg: null ") + what + " array");
    std::vector<Tensor> v;
    for (int j = 0; j < n; ++j) {
        ITG_REQUIRE(t[j], std::string("dmrg: null ") + what + " tensor");
        v.push_back(t[j]->t);
    }
    return v;
}

std::vector<SweepSpec> sweeps_from(itg_sweep_desc const* sweeps, int n) {
    ITG_REQUIRE(sweeps && n > 0, "dmrg: empty sweep schedule");
    std::vector<SweepSpec> sw(n);
    for (int s = 0; s < n; ++s) {
        ITG_REQUIRE(sweeps[s].noise >= 0.0, "dmrg: the noise must be non-negative");
        ITG_REQUIRE(sweeps[s].maxdim >= 1 && sweeps[s].niter >= 1, "dmrg: maxdim and niter must be positive");
        sw[s].maxdim = sweeps[s].maxdim;
        sw[s].mindim = sweeps[s].mindim;
        sw[s].cutoff = sweeps[s].cutoff;
        sw[s].niter = sweeps[s].niter;
        sw[s].noise = sweeps[s].noise;
        sw[s].use_svd = sweeps[s].use_svd != 0;
    }
    return sw;
}
}  // namespace

struct itg_pool {
    SolverPool pool;
    itg_pool(int dev, int w, int s, int64_t budget) : pool(dev, w, s, budget) {}
};

extern "C" {

int itg_create(int device, itg_ctx** out) {
    return guard(nullptr, [&] {
        ITG_REQUIRE(out, "itg_create: null out");
        *out = new itg_ctx(device);
    });
}

void itg_destroy(itg_ctx* c) { delete c; }

const char* itg_last_error(itg_ctx* c) { return c ? c->ctx.last_error.c_str() : g_error.c_str(); }

int itg_synchronize(itg_ctx* c) { return guard(c, [&] { c->ctx.sync(); }); }

int itg_set_precision(itg_ctx* c, int mode, int slices) {
    return guard(c, [&] {
        ITG_REQUIRE(mode == PREC_F64 || mode == PREC_OZAKI_BF16, "precision: unknown mode");
        ITG_REQUIRE(slices >= 3 && slices <= 6, "precision: ozaki_slices must be 3..6");
        c->ctx.precision = mode;
        c->ctx.ozaki_slices = slices;
    });
}

int itg_set_gemm_variant(itg_ctx* c, int variant) {
    return guard(c, [&] {
        ITG_REQUIRE(variant >= -1 && variant <= 4, "gemm variant must be -1..4");
        c->ctx.gemm_variant = variant;
    });
}

int itg_stats(itg_ctx* c, uint64_t* launches, double* flops, uint64_t* built, uint64_t* hits) {
    return guard(c, [&] {
        if (launches) *launches = c->ctx.kernel_launches;
        if (flops) *flops = c->ctx.flops_done;
        if (built) *built = c->ctx.plans_built;
        if (hits) *hits = c->ctx.plan_hits;
    });
}

int itg_reset_stats(itg_ctx* c) {
    return guard(c, [&] {
        c->ctx.kernel_launches = 0;
        c->ctx.flops_done = 0;
        c->ctx.plans_built = 0;
        c->ctx.plan_hits = 0;
    });
}

void* itg_stream(itg_ctx* c) { return c ? (void*)c->ctx.stream : nullptr; }

int itg_measure_peaks(itg_ctx* c, double* tflops5) {
    return guard(c, [&] {
        ITG_REQUIRE(tflops5, "measure_peaks: null output");
        measure_peaks(c->ctx, tflops5);
    });
}

int itg_profile_begin(itg_ctx* c) {
    return guard(c, [&] {
        for (auto& r : c->ctx.prof) { cudaEventDestroy(r.start); cudaEventDestroy(r.stop); }
        c->ctx.prof.clear();
        c->ctx.profiling = true;
    });
}

int itg_profile_end(itg_ctx* c, int32_t* n, float* ms, double* flops, int32_t* kind) {
    return guard(c, [&] {
        ITG_REQUIRE(n, "profile_end: null count");
        c->ctx.sync();
        int cap = *n;
        *n = (int32_t)c->ctx.prof.size();
        for (int i = 0; i < (int)c->ctx.prof.size(); ++i) {
            auto& r = c->ctx.prof[i];
            if (i < cap) {
                float t = 0;
                ITG_CHECK_CUDA(cudaEventElapsedTime(&t, r.start, r.stop));
                if (ms) ms[i] = t;
                if (flops) flops[i] = r.flops;
                if (kind) kind[i] = r.kind;
            }
            cudaEventDestroy(r.start);
            cudaEventDestroy(r.stop);
        }
        c->ctx.prof.clear();
        c->ctx.profiling = false;
    });
}

int itg_tensor_create(itg_ctx* c, int32_t rank, const itg_index_desc* inds, int32_t nblocks, const int32_t* coords,
                      const double* data, int data_is_device, itg_tensor** out) {
    return guard(c, [&] {
        ITG_REQUIRE(out && rank >= 0 && nblocks >= 0, "tensor_create: bad arguments");
        std::vector<Index> is;
        for (int k = 0; k < rank; ++k) is.push_back(index_from(inds[k]));
        auto L = std::make_shared<Layout>();
        L->inds = is;
        if (rank > 0) {
            L->coords.assign(coords, coords + (size_t)nblocks * rank);
            for (int b = 0; b < nblocks; ++b)
                for (int k = 0; k < rank; ++k)
                    ITG_REQUIRE(L->coords[(size_t)b * rank + k] >= 0 && L->coords[(size_t)b * rank + k] < is[k].nblock(),
                                "tensor_create: block coordinate out of range");
            for (int b = 1; b < nblocks; ++b)
                ITG_REQUIRE(coords_less(L->block(b - 1), L->block(b), rank),
                            "tensor_create: blocks not in storage order (or a block listed twice)");
            // one divergence per tensor: every stored block has the same flux (QDense,
            // itensor/itdata/qdense.cc:134-171)
            for (int b = 1; b < nblocks; ++b)
                ITG_REQUIRE(L->flux(L->block(b)) == L->flux(L->block(0)),
                            "tensor_create: blocks of different flux (no single divergence)");
        }
        L->finish();
        Tensor t(L, c->ctx.stream);
        if (L->size > 0 && data) {
            if (data_is_device) {
                ITG_CHECK_CUDA(cudaMemcpyAsync(t.data(), data, sizeof(double) * L->size, cudaMemcpyDeviceToDevice, c->ctx.stream));
            } else {
                t = upload_tensor(c->ctx, L, data);
            }
        } else if (L->size > 0) {
            launch_fill(c->ctx, t.data(), L->size, 0.0);
        }
        *out = new itg_tensor{t};
    });
}

void itg_tensor_free(itg_tensor* t) { delete t; }

int itg_tensor_layout(const itg_tensor* t, int32_t* rank, int32_t* nblocks, int64_t* size) {
    return guard(nullptr, [&] {
        ITG_REQUIRE(t, "tensor_layout: null tensor");
        if (rank) *rank = t->t.rank();
        if (nblocks) *nblocks = t->t.lay->nblocks();
        if (size) *size = t->t.lay->size;
    });
}

int itg_tensor_index(const itg_tensor* t, int32_t k, uint64_t* id, int32_t* plev, int32_t* dir, int32_t* nsect,
                     int32_t* qn, int32_t* qn_mod, int32_t* dims) {
    return guard(nullptr, [&] {
        ITG_REQUIRE(t && k >= 0 && k < t->t.rank(), "tensor_index: bad index position");
        Index const& I = t->t.inds()[k];
        if (id) *id = I.id;
        if (plev) *plev = I.plev;
        if (dir) *dir = I.dir;
        if (nsect) *nsect = I.nblock();
        for (int s = 0; s < I.nblock(); ++s) {
            if (qn) for (int q = 0; q < QN_SLOTS; ++q) qn[s * QN_SLOTS + q] = I.qn(s).v[q];
            if (dims) dims[s] = I.bdim(s);
        }
        if (qn_mod) {
            for (int q = 0; q < QN_SLOTS; ++q) {
                int32_t m = 0;
                for (int s = 0; s < I.nblock(); ++s) if (I.qn(s).mod[q]) m = I.qn(s).mod[q];
                qn_mod[q] = m;
            }
        }
    });
}

int itg_tensor_blocks(const itg_tensor* t, int32_t* coords, int64_t* offsets) {
    return guard(nullptr, [&] {
        ITG_REQUIRE(t, "tensor_blocks: null tensor");
        Layout const& L = *t->t.lay;
        if (coords && !L.coords.empty()) std::memcpy(coords, L.coords.data(), sizeof(int32_t) * L.coords.size());
        if (offsets) std::memcpy(offsets, L.offs.data(), sizeof(int64_t) * L.offs.size());
    });
}

int itg_tensor_read(itg_ctx* c, const itg_tensor* t, double* host) {
    return guard(c, [&] {
        ITG_REQUIRE(t && host, "tensor_read: null argument");
        auto h = download(c->ctx, t->t);
        if (!h.empty()) std::memcpy(host, h.data(), sizeof(double) * h.size());
    });
}

double* itg_tensor_device_ptr(const itg_tensor* t) { return t ? t->t.data() : nullptr; }

int itg_tensor_scalar(const itg_tensor* t, double* v) {
    return guard(nullptr, [&] {
        ITG_REQUIRE(t && v && t->t.rank() == 0, "tensor_scalar: not a rank-0 tensor");
        *v = t->t.scalar;
    });
}

int itg_contract(itg_ctx* c, const itg_tensor* A, const itg_tensor* B, int precision, itg_tensor** C) {
    return guard(c, [&] {
        ITG_REQUIRE(A && B && C, "contract: null argument");
        *C = new itg_tensor{contract(c->ctx, A->t, B->t, precision)};
    });
}

int itg_contract_plan(itg_ctx* c, const itg_layout_desc* A, const int32_t* labelsA, const itg_layout_desc* B,
                      const int32_t* labelsB, itg_plan** plan) {
    return guard(c, [&] {
        ITG_REQUIRE(A && B && plan && labelsA && labelsB, "contract_plan: null argument");
        // anonymous indices: the id encodes the label, so equal negative labels contract
        auto build = [&](itg_layout_desc const* d, int32_t const* labels, int side) {
            Layout L;
            int off = 0;
            for (int k = 0; k < d->rank; ++k) {
                std::vector<int32_t> dims(d->sect_dims + off, d->sect_dims + off + d->nsect[k]);
                off += d->nsect[k];
                std::vector<QN> qs(dims.size());
                uint64_t id = labels[k] < 0 ? (uint64_t)(1000000 - labels[k]) : (uint64_t)(2000000 + 1000 * side + k);
                L.inds.push_back(Index(qs, dims, 1, id, 0));
            }
            L.coords.assign(d->coords, d->coords + (size_t)d->nblocks * d->rank);
            for (int b = 1; b < d->nblocks; ++b)
                ITG_REQUIRE(coords_less(L.block(b - 1), L.block(b), d->rank), "contract_plan: blocks not in storage order");
            L.finish();
            return L;
        };
        Layout LA = build(A, labelsA, 0), LB = build(B, labelsB, 1);
        Match mt = match_indices(LA.inds, LB.inds);
        auto p = get_plan(c->ctx, LA, LB, mt);
        c->ctx.sync();  // the tables are resident before the plan is handed out (any stream may run it)
        *plan = new itg_plan{p, p->C};
    });
}

int itg_plan_output(const itg_plan* p, int32_t* rank, int32_t* nblocks, int64_t* size) {
    return guard(nullptr, [&] {
        ITG_REQUIRE(p, "plan_output: null plan");
        if (rank) *rank = p->C->rank();
        if (nblocks) *nblocks = p->C->nblocks();
        if (size) *size = p->C->size;
    });
}

int itg_plan_output_blocks(const itg_plan* p, int32_t* coords, int64_t* offsets) {
    return guard(nullptr, [&] {
        ITG_REQUIRE(p, "plan_output_blocks: null plan");
        if (coords && !p->C->coords.empty()) std::memcpy(coords, p->C->coords.data(), sizeof(int32_t) * p->C->coords.size());
        if (offsets) std::memcpy(offsets, p->C->offs.data(), sizeof(int64_t) * p->C->offs.size());
    });
}

int itg_plan_flops(const itg_plan* p, double* flops) {
    return guard(nullptr, [&] {
        ITG_REQUIRE(p && flops, "plan_flops: null argument");
        *flops = p->p->flops;
    });
}

int itg_contract_exec(itg_ctx* c, const itg_plan* p, const double* A, const double* B, double* C, int precision) {
    return guard(c, [&] {
        ITG_REQUIRE(p, "contract_exec: null plan");
        exec_plan(c->ctx, *p->p, A, B, C, precision);
    });
}

void itg_plan_free(itg_plan* p) { delete p; }

int itg_contract_exec_noalloc(itg_ctx* c, const itg_plan* p, const double* A, const double* B, double* C, int slices) {
    return guard(c, [&] {
        ITG_REQUIRE(c && p && A && B && C, "contract_exec_noalloc: null argument");
        exec_plan_noalloc(c->ctx, *p->p, A, B, C, slices);
    });
}

int itg_heff_apply(itg_ctx* c, const itg_tensor* L, const itg_tensor* W1, const itg_tensor* W2, const itg_tensor* R,
                   const itg_tensor* phi, int precision, itg_tensor** out) {
    return guard(c, [&] {
        ITG_REQUIRE(W1 && W2 && phi && out, "heff_apply: null argument");
        LocalOp op{opt(L), &W1->t, &W2->t, opt(R)};
        *out = new itg_tensor{heff_product(c->ctx, op, phi->t, precision, false)};
    });
}

int itg_heff_create(itg_ctx* c, const itg_tensor* L, const itg_tensor* W1, const itg_tensor* W2, const itg_tensor* R,
                    const itg_tensor* phi, int precision, int use_graph, itg_heff** out, int64_t* out_size,
                    double* flops) {
    return guard(c, [&] {
        ITG_REQUIRE(W1 && W2 && phi && out, "heff_create: null argument");
        LocalOp op{opt(L), &W1->t, &W2->t, opt(R)};
        auto p = heff_prepare(c->ctx, op, phi->t.lay, precision, false, use_graph != 0, true);
        *out = new itg_heff{p};
        if (out_size) *out_size = p->out_size;
        if (flops) *flops = p->flops;
    });
}

int itg_heff_run(itg_ctx* c, itg_heff* h, const double* phi, double* out, int host) {
    return guard(c, [&] {
        ITG_REQUIRE(h && phi && out, "heff_run: null argument");
        h->p->run(c->ctx, phi, out, host != 0);
    });
}

void itg_heff_free(itg_heff* h) { delete h; }

int itg_davidson(itg_ctx* c, const itg_tensor* L, const itg_tensor* W1, const itg_tensor* W2, const itg_tensor* R,
                 const itg_tensor* phi, int32_t maxiter, double errgoal, int precision, double* energy,
                 itg_tensor** phi_out) {
    return guard(c, [&] {
        ITG_REQUIRE(W1 && W2 && phi && energy && phi_out, "davidson: null argument");
        LocalOp op{opt(L), &W1->t, &W2->t, opt(R)};
        // canonical layout: every block of phi's divergence
        auto full = std::make_shared<Layout>(allowed_layout(phi->t.inds(), tensor_div(phi->t)));
        Tensor v(full, c->ctx.stream);
        launch_fill(c->ctx, v.data(), full->size, 0.0);
        // scatter phi's blocks into the canonical layout
        GatherPlan g;
        Layout const& PL = *phi->t.lay;
        for (int b = 0; b < PL.nblocks(); ++b) {
            int fb = full->find_block(PL.block(b));
            ITG_REQUIRE(fb >= 0, "davidson: phi has a block outside its divergence");
            GatherItem it;
            it.soff = PL.offs[b];
            it.doff = full->offs[fb];
            it.n1 = (int32_t)PL.block_size(b);
            it.n2 = 1;
            std::vector<int32_t> lin(it.n1);
            for (int i = 0; i < it.n1; ++i) lin[i] = i;
            it.ts1 = it.td1 = g.add_table(lin);
            it.ts2 = it.td2 = g.add_table({0});
            g.items.push_back(it);
        }
        g.upload(c->ctx);
        launch_gather(c->ctx, g, phi->t.data(), v.data());
        *energy = davidson(c->ctx, op, v, maxiter, errgoal, 1, precision);
        *phi_out = new itg_tensor{v};
    });
}

int itg_denmat_decomp(itg_ctx* c, const itg_tensor* AA, const itg_tensor* A, const itg_tensor* B, int fromleft,
                      double cutoff, int32_t maxdim, int32_t mindim, int respect_degenerate, int normalize,
                      int precision, itg_tensor** A_out, itg_tensor** B_out, double* truncerr, double* eigs,
                      int32_t* neigs) {
    return itg_denmat_decomp_noise(c, AA, A, B, fromleft, nullptr, nullptr, nullptr, nullptr, 0.0, cutoff, maxdim,
                                   mindim, respect_degenerate, normalize, precision, A_out, B_out, truncerr, eigs,
                                   neigs);
}

int itg_denmat_decomp_noise(itg_ctx* c, const itg_tensor* AA, const itg_tensor* A, const itg_tensor* B, int fromleft,
                            const itg_tensor* L, const itg_tensor* W1, const itg_tensor* W2, const itg_tensor* R,
                            double noise, double cutoff, int32_t maxdim, int32_t mindim, int respect_degenerate,
                            int normalize, int precision, itg_tensor** A_out, itg_tensor** B_out, double* truncerr,
                            double* eigs, int32_t* neigs) {
    return guard(c, [&] {
        ITG_REQUIRE(AA && A && B && A_out && B_out, "denmat_decomp: null argument");
        ITG_REQUIRE(noise >= 0.0, "denmat_decomp: the noise must be non-negative");
        ITG_REQUIRE(noise == 0.0 || (fromleft ? W1 : W2), "denmat_decomp: the noise term needs the MPO tensor");
        SplitArgs sa;
        sa.cutoff = cutoff;
        sa.maxdim = maxdim;
        sa.mindim = mindim;
        sa.respect_degenerate = respect_degenerate != 0;
        sa.normalize = normalize != 0;
        LocalOp op;
        op.L = opt(L);
        op.W1 = opt(W1);
        op.W2 = opt(W2);
        op.R = opt(R);
        SplitResult r = denmat_decomp(c->ctx, AA->t, A->t, B->t, fromleft != 0, sa, precision,
                                      noise > 0 ? &op : nullptr, noise);
        *A_out = new itg_tensor{r.A};
        *B_out = new itg_tensor{r.B};
        if (truncerr) *truncerr = r.truncerr;
        if (neigs) {
            int cap = *neigs;
            *neigs = (int32_t)r.probs.size();
            if (eigs) for (int i = 0; i < std::min<int>(cap, (int)r.probs.size()); ++i) eigs[i] = r.probs[i];
        }
    });
}

int itg_svd_split(itg_ctx* c, const itg_tensor* AA, const itg_tensor* A, const itg_tensor* B, int fromleft,
                  double cutoff, int32_t maxdim, int32_t mindim, int respect_degenerate, int normalize, int precision,
                  itg_tensor** A_out, itg_tensor** B_out, double* truncerr, double* eigs, int32_t* neigs) {
    return guard(c, [&] {
        ITG_REQUIRE(AA && A && B && A_out && B_out, "svd_split: null argument");
        SplitArgs sa;
        sa.cutoff = cutoff;
        sa.maxdim = maxdim;
        sa.mindim = mindim;
        sa.respect_degenerate = respect_degenerate != 0;
        sa.normalize = normalize != 0;
        SplitResult r = svd_split(c->ctx, AA->t, A->t, B->t, fromleft != 0, sa, precision);
        *A_out = new itg_tensor{r.A};
        *B_out = new itg_tensor{r.B};
        if (truncerr) *truncerr = r.truncerr;
        if (neigs) {
            int cap = *neigs;
            *neigs = (int32_t)r.probs.size();
            if (eigs) for (int i = 0; i < std::min<int>(cap, (int)r.probs.size()); ++i) eigs[i] = r.probs[i];
        }
    });
}

int itg_truncate(const double* P, int32_t n, int32_t maxdim, int32_t mindim, double cutoff, int absolute_cutoff,
                 int rel_cutoff, int respect_degenerate, double* Pout, int32_t* m, double* truncerr,
                 double* docut_lower, double* docut_upper, int32_t* ndegen) {
    return guard(nullptr, [&] {
        ITG_REQUIRE(P && n > 0, "truncate: empty spectrum");
        TruncResult r = truncate(std::vector<double>(P, P + n), maxdim, mindim, cutoff, absolute_cutoff != 0,
                                 rel_cutoff != 0, respect_degenerate != 0);
        if (Pout) std::memcpy(Pout, r.P.data(), sizeof(double) * r.P.size());
        if (m) *m = (int32_t)r.P.size();
        if (truncerr) *truncerr = r.truncerr;
        if (docut_lower) *docut_lower = r.docut_lower;
        if (docut_upper) *docut_upper = r.docut_upper;
        if (ndegen) *ndegen = r.ndegen;
    });
}

int itg_dmrg_run(itg_ctx* c, const itg_model_desc* model, const itg_sweep_desc* sweeps, int32_t nsweeps,
                 int precision, itg_dmrg_result** out) {
    return guard(c, [&] {
        ITG_REQUIRE(model && sweeps && nsweeps > 0 && out, "dmrg_run: bad arguments");
        ModelSpec m = model_from(*model);
        Hamiltonian H = make_hamiltonian(m);
        ITG_REQUIRE(H.N >= 2, "dmrg_run: need at least two sites");
        MPO mpo = build_mpo(c->ctx, H);
        auto psi = product_mps(c->ctx, mpo, H.st, default_state(m));
        std::vector<SweepSpec> sw = sweeps_from(sweeps, nsweeps);
        auto* res = new itg_dmrg_result;
        try {
            res->r = dmrg(c->ctx, mpo, psi, sw, precision);
        } catch (...) {
            delete res;
            throw;
        }
        *out = res;
    });
}

int itg_dmrg_run_sum(itg_ctx* c, const itg_model_desc* models, int32_t nmodels, const itg_sweep_desc* sweeps,
                     int32_t nsweeps, int precision, itg_dmrg_result** out) {
    return guard(c, [&] {
        ITG_REQUIRE(models && nmodels >= 1 && sweeps && nsweeps > 0 && out, "dmrg_run_sum: bad arguments");
        ModelSpec m0 = model_from(models[0]);
        Hamiltonian H0 = make_hamiltonian(m0);
        ITG_REQUIRE(H0.N >= 2, "dmrg_run_sum: need at least two sites");
        MPO mpo = build_mpo(c->ctx, H0);
        std::vector<MPO> more;
        for (int k = 1; k < nmodels; ++k) {
            ModelSpec mk = model_from(models[k]);
            ITG_REQUIRE(mk.type == m0.type, "dmrg_run_sum: the models must share their site type");
            Hamiltonian Hk = make_hamiltonian(mk);
            ITG_REQUIRE(Hk.N == H0.N, "dmrg_run_sum: the models must have the same number of sites");
            more.push_back(build_mpo(c->ctx, Hk, &mpo.sites));
        }
        auto psi = product_mps(c->ctx, mpo, H0.st, default_state(m0));
        std::vector<SweepSpec> sw = sweeps_from(sweeps, nsweeps);
        auto* res = new itg_dmrg_result;
        try {
            res->r = dmrg(c->ctx, mpo, psi, sw, precision, nullptr, 1.0, more.empty() ? nullptr : &more);
        } catch (...) {
            delete res;
            throw;
        }
        *out = res;
    });
}

int itg_dmrg_run_states(itg_ctx* c, const itg_model_desc* model, int32_t nstates, const itg_sweep_desc* const* sweeps,
                        const int32_t* nsweeps, double weight, int precision, itg_dmrg_result** out) {
    return guard(c, [&] {
        ITG_REQUIRE(model && nstates >= 1 && sweeps && nsweeps && out, "dmrg_run_states: bad arguments");
        ITG_REQUIRE(weight > 0, "dmrg_run_states: the weight must be positive");
        ModelSpec m = model_from(*model);
        Hamiltonian H = make_hamiltonian(m);
        ITG_REQUIRE(H.N >= 2, "dmrg_run_states: need at least two sites");
        MPO mpo = build_mpo(c->ctx, H);
        std::vector<std::vector<Tensor>> prev;
        std::vector<itg_dmrg_result*> made;
        try {
            for (int k = 0; k < nstates; ++k) {
                auto psi = product_mps(c->ctx, mpo, H.st, default_state(m));
                std::vector<SweepSpec> sw = sweeps_from(sweeps[k], nsweeps[k]);
                auto* res = new itg_dmrg_result;
                made.push_back(res);
                res->r = dmrg(c->ctx, mpo, psi, sw, precision, k ? &prev : nullptr, weight);
                prev.push_back(res->r.psi);
            }
        } catch (...) {
            for (auto* r : made) delete r;
            throw;
        }
        for (int k = 0; k < nstates; ++k) out[k] = made[k];
    });
}

int itg_dmrg_run_mpo(itg_ctx* c, int32_t nsites, int32_t nmpo, const itg_tensor* const* W, const itg_tensor* const* psi0,
                     int32_t nprev, const itg_tensor* const* prev, double weight, const itg_sweep_desc* sweeps,
                     int32_t nsweeps, int precision, itg_dmrg_result** out) {
    return guard(c, [&] {
        ITG_REQUIRE(c && out && nsites >= 2 && nmpo >= 1 && nprev >= 0, "dmrg_run_mpo: bad arguments");
        ITG_REQUIRE(nprev == 0 || weight > 0, "dmrg_run_mpo: the weight must be positive");
        std::vector<Tensor> start = tensors_from(psi0, nsites, "MPS");
        MPO H = mpo_from_tensors(tensors_from(W, nsites, "MPO"), start);
        std::vector<MPO> more;
        for (int k = 1; k < nmpo; ++k)
            more.push_back(mpo_from_tensors(tensors_from(W + (size_t)k * nsites, nsites, "MPO"), start, &H.sites));
        std::vector<std::vector<Tensor>> prevs;
        for (int k = 0; k < nprev; ++k) {
            ITG_REQUIRE(prev, "dmrg_run_mpo: null array of earlier states");
            prevs.push_back(tensors_from(prev + (size_t)k * nsites, nsites, "earlier-state"));
        }
        std::vector<SweepSpec> sw = sweeps_from(sweeps, nsweeps);
        auto* res = new itg_dmrg_result;
        try {
            res->r = dmrg(c->ctx, H, start, sw, precision, prevs.empty() ? nullptr : &prevs, weight,
                          more.empty() ? nullptr : &more);
        } catch (...) {
            delete res;
            throw;
        }
        *out = res;
    });
}

int itg_dmrg_mps(const itg_dmrg_result* r, int32_t j, itg_tensor** out) {
    return guard(nullptr, [&] {
        ITG_REQUIRE(r && out, "dmrg_mps: null argument");
        ITG_REQUIRE(!r->r.psi.empty(), "dmrg_mps: this result holds no MPS");
        ITG_REQUIRE(j >= 1 && j <= (int)r->r.psi.size(), "dmrg_mps: site out of range");
        *out = new itg_tensor{r->r.psi[j - 1]};
    });
}

struct itg_mps_file {
    MpsFile f;
};

int itg_mps_file_read(const char* path, itg_mps_file** out) {
    return guard(nullptr, [&] {
        ITG_REQUIRE(path && out, "mps_file_read: null argument");
        auto* f = new itg_mps_file{read_mps_file(path)};
        *out = f;
    });
}

int itg_mps_file_write(const itg_mps_file* f, const char* path) {
    return guard(nullptr, [&] {
        ITG_REQUIRE(f && path, "mps_file_write: null argument");
        write_mps_file(f->f, path);
    });
}

int itg_mps_file_info(const itg_mps_file* f, int32_t* nsites, int32_t* leftlim, int32_t* rightlim, int32_t* nqn,
                      char* qn_names) {
    return guard(nullptr, [&] {
        ITG_REQUIRE(f, "mps_file_info: null file");
        if (nsites) *nsites = f->f.N;
        if (leftlim) *leftlim = f->f.leftlim;
        if (rightlim) *rightlim = f->f.rightlim;
        if (nqn) *nqn = (int32_t)f->f.qn_names.size();
        if (qn_names) {
            std::memset(qn_names, 0, 4 * 8);
            for (size_t k = 0; k < f->f.qn_names.size(); ++k) std::memcpy(qn_names + 8 * k, f->f.qn_names[k].data(), 7);
        }
    });
}

int itg_mps_file_load(itg_ctx* c, const itg_mps_file* f, itg_tensor** sites) {
    return guard(c, [&] {
        ITG_REQUIRE(c && f && sites, "mps_file_load: null argument");
        std::vector<Tensor> ts = load_mps(c->ctx, f->f);
        for (size_t j = 0; j < ts.size(); ++j) sites[j] = new itg_tensor{ts[j]};
    });
}

int itg_mps_file_store(itg_ctx* c, int32_t nsites, const itg_tensor* const* sites, int32_t leftlim, int32_t rightlim,
                       const char* qn_names, itg_mps_file** out) {
    return guard(c, [&] {
        ITG_REQUIRE(c && out && nsites >= 1, "mps_file_store: bad arguments");
        std::vector<std::array<char, 7>> names;
        std::string s = qn_names ? qn_names : "";
        size_t p = 0;
        while (p < s.size()) {
            size_t q = s.find(',', p);
            if (q == std::string::npos) q = s.size();
            std::string n = s.substr(p, q - p);
            ITG_REQUIRE(!n.empty() && n.size() <= 7, "mps_file_store: QN names hold 1 to 7 characters");
            std::array<char, 7> a{};
            std::memcpy(a.data(), n.data(), n.size());
            names.push_back(a);
            p = q + 1;
        }
        auto* f = new itg_mps_file{store_mps(c->ctx, tensors_from(sites, nsites, "MPS"), leftlim, rightlim, names)};
        *out = f;
    });
}

void itg_mps_file_free(itg_mps_file* f) { delete f; }

int itg_dmrg_energy(const itg_dmrg_result* r, double* e) {
    return guard(nullptr, [&] { ITG_REQUIRE(r && e, "null"); *e = r->r.energy; });
}
int itg_dmrg_nbonds(const itg_dmrg_result* r, int32_t* n) {
    return guard(nullptr, [&] { ITG_REQUIRE(r && n, "null"); *n = (int32_t)r->r.bonds.size(); });
}
int itg_dmrg_bonds(const itg_dmrg_result* r, int32_t* sweep, int32_t* ha, int32_t* bond, double* energy,
                   double* truncerr, int32_t* dim) {
    return guard(nullptr, [&] {
        ITG_REQUIRE(r, "null");
        for (size_t i = 0; i < r->r.bonds.size(); ++i) {
            auto const& b = r->r.bonds[i];
            if (sweep) sweep[i] = b.sweep;
            if (ha) ha[i] = b.halfsweep;
            if (bond) bond[i] = b.bond;
            if (energy) energy[i] = b.energy;
            if (truncerr) truncerr[i] = b.truncerr;
            if (dim) dim[i] = (int32_t)b.dim;
        }
    });
}
int itg_dmrg_link(const itg_dmrg_result* r, int32_t b, int32_t* dir, int32_t* nsect, int32_t* qn, int32_t* dims) {
    return guard(nullptr, [&] {
        ITG_REQUIRE(r && b >= 1 && b <= (int)r->r.links.size(), "dmrg_link: bond out of range");
        Index const& I = r->r.links[b - 1];
        if (dir) *dir = I.dir;
        if (nsect) *nsect = I.nblock();
        for (int s = 0; s < I.nblock(); ++s) {
            if (qn) for (int q = 0; q < QN_SLOTS; ++q) qn[s * QN_SLOTS + q] = I.qn(s).v[q];
            if (dims) dims[s] = I.bdim(s);
        }
    });
}
int itg_dmrg_timing(const itg_dmrg_result* r, int32_t* nsweeps, double* secs, int32_t* applies) {
    return guard(nullptr, [&] {
        ITG_REQUIRE(r, "null");
        if (nsweeps) *nsweeps = (int32_t)r->r.sweep_seconds.size();
        if (secs) for (size_t i = 0; i < r->r.sweep_seconds.size(); ++i) secs[i] = r->r.sweep_seconds[i];
        if (applies) *applies = r->r.heff_applies;
    });
}
int itg_dmrg_phases(const itg_dmrg_result* r, double* s) {
    return guard(nullptr, [&] {
        ITG_REQUIRE(r && s, "null");
        for (int k = 0; k < 3; ++k) s[k] = r->r.phase_seconds[k];
    });
}
void itg_dmrg_free(itg_dmrg_result* r) { delete r; }

int itg_pool_create(int device, int32_t workers, int32_t slots_per_worker, double budget_bytes, itg_pool** out) {
    return guard(nullptr, [&] {
        ITG_REQUIRE(out, "pool_create: null out");
        int n = 0;
        ITG_CHECK_CUDA(cudaGetDeviceCount(&n));
        ITG_REQUIRE(device >= 0 && device < n, "pool_create: no such device");
        *out = new itg_pool(device, workers, slots_per_worker, (int64_t)budget_bytes);
    });
}

int itg_pool_submit(itg_pool* p, const itg_model_desc* model, const itg_sweep_desc* sweeps, int32_t nsweeps,
                    int precision, double arrival_s, int64_t* id) {
    return guard(nullptr, [&] {
        ITG_REQUIRE(p && model && id, "pool_submit: bad arguments");
        ITG_REQUIRE(precision == PREC_F64 || precision == PREC_OZAKI_BF16, "pool_submit: unsupported precision");
        SolveRequest r;
        r.model = model_from(*model);
        r.sweeps = sweeps_from(sweeps, nsweeps);
        r.prec = precision;
        r.arrival = arrival_s;
        *id = p->pool.submit(std::move(r));
    });
}

int itg_pool_submit_mpo(itg_pool* p, itg_ctx* c, int32_t nsites, const itg_tensor* const* W,
                        const itg_tensor* const* psi0, const itg_sweep_desc* sweeps, int32_t nsweeps, int precision,
                        double arrival_s, int keep_mps, int64_t* id) {
    return guard(nullptr, [&] {
        ITG_REQUIRE(p && c && id && nsites >= 2, "pool_submit_mpo: bad arguments");
        ITG_REQUIRE(precision == PREC_F64 || precision == PREC_OZAKI_BF16, "pool_submit_mpo: unsupported precision");
        std::vector<Tensor> w = tensors_from(W, nsites, "MPO"), s = tensors_from(psi0, nsites, "MPS");
        mpo_from_tensors(w, s);  // checks the structure now, so a bad request fails here
        auto in = std::make_shared<MpoInput>();
        for (auto const& t : w) in->W.push_back(HostTensor{t.lay, download(c->ctx, t)});
        for (auto const& t : s) in->psi0.push_back(HostTensor{t.lay, download(c->ctx, t)});
        SolveRequest r;
        r.mpo = in;
        r.keep_mps = keep_mps != 0;
        r.sweeps = sweeps_from(sweeps, nsweeps);
        r.prec = precision;
        r.arrival = arrival_s;
        *id = p->pool.submit(std::move(r));
    });
}

int itg_pool_set_grouping(itg_pool* p, int on) {
    return guard(nullptr, [&] {
        ITG_REQUIRE(p, "null pool");
        p->pool.set_grouping(on != 0);
    });
}

int itg_pool_grouping_stats(itg_pool* p, int64_t* grouped_launches, int64_t* grouped_contractions) {
    return guard(nullptr, [&] {
        ITG_REQUIRE(p, "null pool");
        PoolStats s = p->pool.stats();
        if (grouped_launches) *grouped_launches = s.grouped_launches;
        if (grouped_contractions) *grouped_contractions = s.grouped_contractions;
    });
}

int itg_pool_set_calibration(itg_pool* p, int32_t min_solves, double safety) {
    return guard(nullptr, [&] {
        ITG_REQUIRE(p, "null pool");
        p->pool.set_calibration(min_solves, safety);
    });
}

int itg_pool_calibration_stats(itg_pool* p, int64_t* calibrated_admissions, int64_t* retried) {
    return guard(nullptr, [&] {
        ITG_REQUIRE(p, "null pool");
        PoolStats s = p->pool.stats();
        if (calibrated_admissions) *calibrated_admissions = s.calibrated;
        if (retried) *retried = s.retried;
    });
}

int itg_pool_record_admission(itg_pool* p, int64_t id, double* admitted_bytes, int32_t* retries) {
    return guard(nullptr, [&] {
        ITG_REQUIRE(p, "null pool");
        SolveRecord r = p->pool.record(id);
        if (admitted_bytes) *admitted_bytes = (double)r.adm_bytes;
        if (retries) *retries = r.retries;
    });
}

int itg_pool_start(itg_pool* p) {
    return guard(nullptr, [&] { ITG_REQUIRE(p, "null pool"); p->pool.start(); });
}

int itg_pool_drain(itg_pool* p) {
    return guard(nullptr, [&] { ITG_REQUIRE(p, "null pool"); p->pool.drain(); });
}

int itg_pool_record(itg_pool* p, int64_t id, int32_t* status, double* energy, double* t_arrive, double* t_admit,
                    double* t_done, double* est_bytes, double* peak_bytes, int32_t* worker) {
    return guard(nullptr, [&] {
        ITG_REQUIRE(p, "null pool");
        SolveRecord r = p->pool.record(id);
        if (status) *status = r.status;
        if (energy) *energy = r.result.energy;
        if (t_arrive) *t_arrive = r.t_arrive;
        if (t_admit) *t_admit = r.t_admit;
        if (t_done) *t_done = r.t_done;
        if (est_bytes) *est_bytes = (double)r.est_bytes;
        if (peak_bytes) *peak_bytes = (double)r.peak_bytes;
        if (worker) *worker = r.worker;
    });
}

int itg_pool_error(itg_pool* p, int64_t id, char* buf, int32_t buflen) {
    return guard(nullptr, [&] {
        ITG_REQUIRE(p && buf && buflen > 0, "pool_error: bad arguments");
        SolveRecord r = p->pool.record(id);
        std::snprintf(buf, (size_t)buflen, "%s", r.error.c_str());
    });
}

int itg_pool_result(itg_pool* p, int64_t id, itg_dmrg_result** out) {
    return guard(nullptr, [&] {
        ITG_REQUIRE(p && out, "pool_result: bad arguments");
        SolveRecord r = p->pool.record(id);
        ITG_REQUIRE(r.status == 0, "pool_result: request " + std::to_string(id) + " has not finished successfully");
        auto* res = new itg_dmrg_result;
        res->r = std::move(r.result);
        *out = res;
    });
}

int itg_pool_stats(itg_pool* p, int64_t* submitted, int64_t* done, int64_t* failed, double* peak_reserved_bytes,
                   int32_t* peak_running, double* elapsed_s) {
    return guard(nullptr, [&] {
        ITG_REQUIRE(p, "null pool");
        PoolStats s = p->pool.stats();
        if (submitted) *submitted = s.submitted;
        if (done) *done = s.done;
        if (failed) *failed = s.failed;
        if (peak_reserved_bytes) *peak_reserved_bytes = (double)s.peak_reserved_bytes;
        if (peak_running) *peak_running = s.peak_running;
        if (elapsed_s) *elapsed_s = s.elapsed;
    });
}

int itg_pool_estimate(const itg_model_desc* model, const itg_sweep_desc* sweeps, int32_t nsweeps, int precision,
                      double* bytes) {
    return guard(nullptr, [&] {
        ITG_REQUIRE(model && bytes, "pool_estimate: bad arguments");
        *bytes = (double)solve_footprint_estimate(model_from(*model), sweeps_from(sweeps, nsweeps), precision);
    });
}

int itg_pool_estimate_mpo(int32_t nsites, int32_t site_dim, int32_t mpo_bond_dim, const itg_sweep_desc* sweeps,
                          int32_t nsweeps, int precision, double* bytes) {
    return guard(nullptr, [&] {
        ITG_REQUIRE(bytes && nsites >= 2 && site_dim >= 1 && mpo_bond_dim >= 1, "pool_estimate_mpo: bad arguments");
        *bytes = (double)solve_footprint_estimate(nsites, site_dim, mpo_bond_dim, sweeps_from(sweeps, nsweeps),
                                                  precision);
    });
}

void itg_pool_destroy(itg_pool* p) { delete p; }

}  // extern "C"
