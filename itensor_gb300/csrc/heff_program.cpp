// Prepared effective-Hamiltonian apply (LocalOp::product,
// itensor/mps/localop.h:324-365) for repeated use with one operator: the four
// contraction plans are resolved once, the intermediates are preallocated,
// and the launches can be replayed as one CUDA graph, so an apply costs no
// host-side planning.
#include "algo.h"

namespace itg {

HeffProgram::~HeffProgram() {
    if (graph) cudaGraphExecDestroy(graph);
}

std::shared_ptr<HeffProgram> heff_prepare(Ctx& ctx, LocalOp const& op, std::shared_ptr<Layout> phi_layout, int prec,
                                          bool into_phi_layout, bool use_graph, bool fuse_mpo) {
    ITG_REQUIRE(op.W1 && op.W2 && phi_layout, "heff_prepare: missing operand");
    auto P = std::make_shared<HeffProgram>();
    P->prec = prec < 0 ? ctx.precision : prec;
    P->use_graph = use_graph;
    P->slices = ctx.ozaki_slices;
    std::vector<Tensor const*> chain;
    if (!op.L) {
        if (op.R) chain.push_back(op.R);
        chain.push_back(op.W2);
        chain.push_back(op.W1);
    } else {
        chain.push_back(op.L);
        chain.push_back(op.W1);
        chain.push_back(op.W2);
        if (op.R) chain.push_back(op.R);
    }
    std::shared_ptr<Layout> target;
    if (into_phi_layout) {
        target = std::make_shared<Layout>(*phi_layout);
        target->inds = prime_all(phi_layout->inds);
    }
    P->in_size = phi_layout->size;
    P->in = dev_alloc(sizeof(double) * std::max<int64_t>(1, P->in_size), ctx.stream);

    // The layouts the reference's chain produces, step by step (plans only,
    // nothing runs): ((phi L) W1) W2 R. Their flops are the algorithmic work.
    std::vector<std::shared_ptr<Layout>> ref_out;
    std::vector<double> ref_flops;
    std::vector<std::shared_ptr<Plan>> ref_plans;  // reused below when the chain runs as it is
    {
        std::shared_ptr<Layout> cur = phi_layout;
        for (size_t s = 0; s < chain.size(); ++s) {
            const bool last = (s + 1 == chain.size());
            Match mt = match_indices(cur->inds, chain[s]->inds());
            auto plan = get_plan(ctx, *cur, *chain[s]->lay, mt, last ? target : nullptr);
            auto outL = std::make_shared<Layout>(*plan->C);
            if (!(last && target)) {
                outL->inds.clear();
                for (int i : mt.a_unc) outL->inds.push_back(cur->inds[i]);
                for (int j : mt.b_unc) outL->inds.push_back(chain[s]->inds()[j]);
            }
            P->flops += plan->flops;
            ref_flops.push_back(plan->flops);
            ref_plans.push_back(plan);
            ref_out.push_back(outL);
            cur = outL;
        }
    }
    // The two MPO tensors are contracted with each other once (W1 W2, or W2 W1
    // from the right end), so an apply runs one MPO-tensor step instead of two
    // and one intermediate less goes through memory. That step writes the
    // layout the reference's second MPO step produces (same index order, same
    // blocks), so everything after it is unchanged. The fused step sums over
    // both sites' indices and the outer MPO link at once, so its flops are about
    // d/2 times those of the two steps it replaces (d the site dimension): it
    // is taken only where it costs no more flops than they do (spin-1/2 models;
    // not the Hubbard model's d = 4).
    // Site dimensions above 2 are ruled out before any plan is built (the
    // check below needs two extra plans); the caller turns fusion on
    // (fuse_mpo: the prepared programs of the C-ABI).
    int dsite = 0;
    for (auto const& I : op.W1->inds())
        if (phi_layout->find_index(I) >= 0) dsite = std::max(dsite, (int)I.dim());
    Tensor Wf;
    size_t wpos = 0;
    for (size_t s = 0; fuse_mpo && dsite <= 2 && s + 1 < chain.size(); ++s)
        if ((chain[s] == op.W1 && chain[s + 1] == op.W2) || (chain[s] == op.W2 && chain[s + 1] == op.W1)) wpos = s + 1;
    if (wpos > 0) {
        Wf = contract(ctx, *chain[wpos - 1], *chain[wpos], PREC_F64);
        std::shared_ptr<Layout> in = wpos >= 2 ? ref_out[wpos - 2] : phi_layout;
        Match mf = match_indices(in->inds, Wf.inds());
        const bool last = (wpos + 1 == chain.size());
        auto pf = get_plan(ctx, *in, *Wf.lay, mf, (last && target) ? target : ref_out[wpos]);
        if (pf->flops <= 1.05 * (ref_flops[wpos - 1] + ref_flops[wpos])) {
            chain.erase(chain.begin() + (long)wpos);
            chain[wpos - 1] = &Wf;
            ref_out.erase(ref_out.begin() + (long)(wpos - 1));  // the fused step writes the second step's layout
        } else {
            wpos = 0;
        }
    }
    std::shared_ptr<Layout> cur = phi_layout;
    for (size_t s = 0; s < chain.size(); ++s) {
        const bool last = (s + 1 == chain.size());
        Match mt = match_indices(cur->inds, chain[s]->inds());
        const bool fused = wpos > 0 && s == wpos - 1;
        // unfused, step s is the reference chain's step s: its plan is already resolved
        auto plan = wpos == 0 ? ref_plans[s]
                              : get_plan(ctx, *cur, *chain[s]->lay, mt,
                                         (last && target) ? target : (fused ? ref_out[s] : nullptr));
        std::shared_ptr<Layout> outL;
        if (last && target) {
            outL = target;
        } else if (fused) {
            outL = ref_out[s];
        } else {
            outL = std::make_shared<Layout>(*plan->C);
            outL->inds.clear();
            for (int i : mt.a_unc) outL->inds.push_back(cur->inds[i]);
            for (int j : mt.b_unc) outL->inds.push_back(chain[s]->inds()[j]);
        }
        HeffProgram::Step st;
        st.plan = plan;
        st.operand = *chain[s];
        st.operand_left = false;
        st.in_buf = (s == 0) ? -1 : (int)P->inter.size() - 1;
        st.split = plan_uses_split(*plan, P->prec);
        if (st.split) st.scratch = dev_alloc(split_scratch_bytes(*plan, P->slices), ctx.stream);
        if (last) {
            st.out_buf = -2;
            P->out_size = outL->size;
            P->out = dev_alloc(sizeof(double) * std::max<int64_t>(1, P->out_size), ctx.stream);
        } else {
            P->inter.push_back(dev_alloc(sizeof(double) * std::max<int64_t>(1, outL->size), ctx.stream));
            st.out_buf = (int)P->inter.size() - 1;
        }
        P->steps.push_back(st);
        cur = outL;
    }
    if (into_phi_layout) {
        P->out_layout = phi_layout;
    } else {
        P->out_layout = std::make_shared<Layout>(*cur);
        P->out_layout->inds = noprime_all(cur->inds);
    }
    return P;
}

void HeffProgram::launch_steps(Ctx& ctx) {
    for (auto& st : steps) {
        double const* a = st.in_buf == -1 ? in->as<double>() : inter[st.in_buf]->as<double>();
        double* c = st.out_buf == -2 ? out->as<double>() : inter[st.out_buf]->as<double>();
        if (st.split) {
            // the operand (L, W or R) is fixed for the program's life: slice it once
            Plan const& p = *st.plan;
            const int64_t plane = (p.panel_elems + 15) / 16 * 16;
            __nv_bfloat16* panels = st.scratch->as<__nv_bfloat16>();
            int32_t* exps = reinterpret_cast<int32_t*>(panels + plane * slices);
            ProfRec pr{};
            if (ctx.profiling) {
                ITG_CHECK_CUDA(cudaEventCreate(&pr.start));
                ITG_CHECK_CUDA(cudaEventCreate(&pr.stop));
                ITG_CHECK_CUDA(cudaEventRecord(pr.start, ctx.stream));
                pr.flops = p.flops;
                pr.kind = 1;
                pr.nitems = p.nitems;
            }
            // first run (never inside a graph capture): pick the GEMM tile shape on this data
            // (a graph-replayed program is built to be run many times; otherwise the plan must be reused first)
            if (!st.operand_sliced && ctx.gemm_variant < 0 && p.oz_variant.load(std::memory_order_relaxed) < 0 &&
                p.flops >= AUTOTUNE_MIN_FLOPS &&
                (use_graph || p.split_uses.fetch_add(1, std::memory_order_relaxed) + 1 >= AUTOTUNE_MIN_USES))
                autotune_ozaki(ctx, p, a, st.operand.data(), c, slices, panels, exps);
            // in a solver-pool fiber that groups launches: one launch with the other solves' contractions
            const bool grouped = !use_graph && !ctx.profiling &&
                                 fiber_group_contract(ctx, p, a, st.operand.data(), c, slices, panels, exps,
                                                   !st.operand_sliced);
            if (!grouped) launch_ozaki(ctx, p, a, st.operand.data(), c, slices, panels, exps, !st.operand_sliced);
            if (ctx.profiling) {
                ITG_CHECK_CUDA(cudaEventRecord(pr.stop, ctx.stream));
                ctx.prof.push_back(pr);
            }
            if (!grouped) ctx.kernel_launches += (!st.operand_sliced || p.nprepA > 0) ? 2 : 1;
            ctx.flops_done += p.flops;
            st.operand_sliced = true;
        } else {
            exec_plan(ctx, *st.plan, a, st.operand.data(), c, prec);
        }
    }
}

// The device address of a page-locked host buffer (null for pageable memory,
// which only a copy-engine transfer may read).
static void* pinned_device_ptr(void const* p) {
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        (void)cudaGetLastError();
        return nullptr;
    }
    return a.type == cudaMemoryTypeHost ? a.devicePointer : nullptr;
}

void HeffProgram::run(Ctx& ctx, double const* in_ptr, double* out_ptr, bool host) {
    // Host buffers that are page-locked are read and written by the copy
    // kernel through their device addresses (no copy-engine transfer between
    // the kernels); pageable ones go through cudaMemcpyAsync.
    void* in_dev = host && in_size > 0 ? pinned_device_ptr(in_ptr) : nullptr;
    void* out_dev = host && out_size > 0 ? pinned_device_ptr(out_ptr) : nullptr;
    if (in_size > 0) {
        if (!host)
            launch_copy(ctx, static_cast<double*>(in->p), in_ptr, in_size);
        else if (in_dev)
            launch_copy(ctx, static_cast<double*>(in->p), static_cast<double const*>(in_dev), in_size);
        else
            ITG_CHECK_CUDA(cudaMemcpyAsync(in->p, in_ptr, sizeof(double) * in_size, cudaMemcpyHostToDevice, ctx.stream));
    }
    if (use_graph) {
        if (!graph) {
            launch_steps(ctx);  // first run outside capture: allocates the split-precision scratch
            const bool prof = ctx.profiling;
            ctx.profiling = false;
            const uint64_t l0 = ctx.kernel_launches;
            const double f0 = ctx.flops_done;
            cudaGraph_t g;
            ITG_CHECK_CUDA(cudaStreamBeginCapture(ctx.stream, cudaStreamCaptureModeThreadLocal));
            ctx.capturing = true;
            try {
                launch_steps(ctx);
            } catch (...) {
                ctx.capturing = false;
                throw;
            }
            ctx.capturing = false;
            ITG_CHECK_CUDA(cudaStreamEndCapture(ctx.stream, &g));
            launches_per_run = (int)(ctx.kernel_launches - l0);
            ctx.kernel_launches = l0;
            ctx.flops_done = f0;
            ctx.profiling = prof;
            ITG_CHECK_CUDA(cudaGraphInstantiate(&graph, g, 0));
            cudaGraphDestroy(g);
        }
        ITG_CHECK_CUDA(cudaGraphLaunch(graph, ctx.stream));
        ctx.kernel_launches += launches_per_run;
        ctx.flops_done += flops;
    } else {
        launch_steps(ctx);
    }
    if (out_size > 0) {
        if (!host)
            launch_copy(ctx, out_ptr, static_cast<double const*>(out->p), out_size);
        else if (out_dev)
            launch_copy(ctx, static_cast<double*>(out_dev), static_cast<double const*>(out->p), out_size);
        else
            ITG_CHECK_CUDA(cudaMemcpyAsync(out_ptr, out->p, sizeof(double) * out_size, cudaMemcpyDeviceToHost, ctx.stream));
    }
    if (host) ctx.sync();
}

}  // namespace itg
