// Two-site DMRG sweep loop on the device path: DMRGWorker
// (itensor/mps/dmrg.h:336-467), sweepnext (itensor/mps/sweeps.h:489-503),
// LocalMPO environments (itensor/mps/localmpo.h:443-618).
#include "algo.h"
#include <chrono>

namespace itg {

namespace {
struct Environments {
    std::vector<Tensor> const* W;
    std::vector<Tensor> PH;   // PH[k]: sites 1..k (left) or k..N (right)
    int N, LHlim, RHlim;
    Environments(std::vector<Tensor> const& w) : W(&w), PH(w.size() + 2), N((int)w.size()), LHlim(0), RHlim((int)w.size() + 1) {}

    Tensor grow(Ctx& ctx, Tensor const* E, Tensor const& A, Tensor const& Wn, int prec) {
        Tensor T = E ? contract(ctx, *E, A, prec) : A;
        T = contract(ctx, T, Wn, prec);
        Tensor Ad = relabel(A, prime_all(dag_all(A.inds())));
        return contract(ctx, T, Ad, prec);
    }
    void makeL(Ctx& ctx, std::vector<Tensor> const& psi, int k, int prec) {
        while (LHlim < k) {
            int ll = LHlim;
            PH[ll + 1] = grow(ctx, PH[ll].valid() ? &PH[ll] : nullptr, psi[ll], (*W)[ll], prec);
            LHlim = ll + 1;
        }
    }
    void makeR(Ctx& ctx, std::vector<Tensor> const& psi, int k, int prec) {
        while (RHlim > k) {
            int rl = RHlim;
            PH[rl - 1] = grow(ctx, PH[rl].valid() ? &PH[rl] : nullptr, psi[rl - 2], (*W)[rl - 2], prec);
            RHlim = rl - 1;
        }
    }
    LocalOp position(Ctx& ctx, int b, std::vector<Tensor> const& psi, int prec) {
        makeL(ctx, psi, b - 1, prec);
        makeR(ctx, psi, b + 2, prec);
        LHlim = b - 1;
        RHlim = b + 2;
        LocalOp op;
        op.L = (b - 1 >= 1) ? &PH[b - 1] : nullptr;
        op.R = (b + 2 <= N) ? &PH[b + 2] : nullptr;
        op.W1 = &(*W)[b - 1];
        op.W2 = &(*W)[b];
        return op;
    }
};
// LocalMPO built from an earlier state psi_j (itensor/mps/localmpo.h:340-349,
// makeL/makeR :543-594, product :389-421): environments of <psi_j|psi> with
// dag(prime(psi_j(k), "Link")), and at bond b the projector
// P_j = dag(L_j psi_j(b)' psi_j(b+1)' R_j) in the layout of phi.
struct MpsEnvironments {
    std::vector<Tensor> const* P;
    std::vector<Index> const* sites;
    std::vector<Tensor> PH;
    int N, LHlim, RHlim;
    MpsEnvironments(std::vector<Tensor> const& p, std::vector<Index> const& s)
        : P(&p), sites(&s), PH(p.size() + 2), N((int)p.size()), LHlim(0), RHlim((int)p.size() + 1) {}

    // dag(prime(psi_j(k), "Link")): every index of the site tensor but the site primed
    Tensor dagp(int k) const {
        Tensor const& A = (*P)[k - 1];
        std::vector<Index> inds = dag_all(A.inds());
        for (auto& I : inds)
            if (!I.same((*sites)[k - 1])) I = I.prime();
        return relabel(A, inds);
    }
    void makeL(Ctx& ctx, std::vector<Tensor> const& psi, int k, int prec) {
        while (LHlim < k) {
            int ll = LHlim;
            Tensor E = PH[ll].valid() ? contract(ctx, PH[ll], psi[ll], prec) : psi[ll];
            PH[ll + 1] = contract(ctx, E, dagp(ll + 1), prec);
            LHlim = ll + 1;
        }
    }
    void makeR(Ctx& ctx, std::vector<Tensor> const& psi, int k, int prec) {
        while (RHlim > k) {
            int rl = RHlim;
            Tensor E = PH[rl].valid() ? contract(ctx, PH[rl], psi[rl - 2], prec) : psi[rl - 2];
            PH[rl - 1] = contract(ctx, E, dagp(rl - 1), prec);
            RHlim = rl - 1;
        }
    }
    Tensor projector(Ctx& ctx, int b, std::vector<Tensor> const& psi, std::shared_ptr<Layout> phi_layout, int prec) {
        makeL(ctx, psi, b - 1, prec);
        makeR(ctx, psi, b + 2, prec);
        LHlim = b - 1;
        RHlim = b + 2;
        Tensor o = (b - 1 >= 1) ? contract(ctx, PH[b - 1], dagp(b), prec) : dagp(b);
        Tensor r = (b + 2 <= N) ? contract(ctx, PH[b + 2], dagp(b + 1), prec) : dagp(b + 1);
        // dag(othr) has phi's indices (same ids and primes, arrows flipped): for real
        // data it is the same numbers, written straight into phi's layout
        return contract(ctx, o, r, prec, phi_layout);
    }
};

// T with the tags of index `link` replaced (same data, same block structure)
Tensor with_link_tags(Tensor const& T, Index const& link, std::array<char, TAG_BYTES> const& tags) {
    std::vector<Index> inds = T.inds();
    for (auto& I : inds)
        if (I.id == link.id) I.tags = tags;
    return relabel(T, inds);
}
}  // namespace

MPO mpo_from_tensors(std::vector<Tensor> const& W, std::vector<Tensor> const& psi0, std::vector<Index> const* sites) {
    const int N = (int)W.size();
    ITG_REQUIRE(N >= 2 && (int)psi0.size() == N, "dmrg: the MPO and the MPS need the same length, at least 2");
    MPO H;
    H.W = W;
    for (int j = 0; j < N; ++j) {
        ITG_REQUIRE(W[j].valid() && psi0[j].valid(), "dmrg: null MPO or MPS tensor");
        Index site;
        bool found = false;
        for (auto const& I : psi0[j].inds()) {
            if (I.plev != 0) continue;
            bool in_w = false, primed = false;
            for (auto const& J : W[j].inds()) {
                if (J.id == I.id && J.plev == 0) in_w = true;
                if (J.id == I.id && J.plev == 1) primed = true;
            }
            if (in_w && primed) { site = I; found = true; break; }
        }
        ITG_REQUIRE(found, "dmrg: MPO tensor " + std::to_string(j + 1) +
                               " does not act on a site index of MPS tensor " + std::to_string(j + 1));
        if (sites) ITG_REQUIRE(site.same((*sites)[j]), "dmrg: the MPOs of a sum act on different site indices");
        H.sites.push_back(site);
        if (j + 1 < N) {
            Match mt = match_indices(W[j].inds(), W[j + 1].inds());
            ITG_REQUIRE(mt.a_con.size() == 1, "dmrg: neighbouring MPO tensors must share exactly one link");
            H.bond_dim = std::max<int>(H.bond_dim, (int)W[j].inds()[mt.a_con[0]].dim());
            Match pm = match_indices(psi0[j].inds(), psi0[j + 1].inds());
            ITG_REQUIRE(pm.a_con.size() == 1, "dmrg: neighbouring MPS tensors must share exactly one link");
        }
    }
    return H;
}

DmrgResult dmrg(Ctx& ctx, MPO const& H, std::vector<Tensor> psi, std::vector<SweepSpec> const& sweeps, int prec,
                std::vector<std::vector<Tensor>> const* prev, double weight, std::vector<MPO> const* more) {
    const int N = (int)psi.size();
    ITG_REQUIRE(N >= 2 && (int)H.W.size() == N, "dmrg: MPO and MPS lengths differ");
    Environments env(H.W);
    std::vector<Environments> menv;
    if (more)
        for (auto const& M : *more) {
            ITG_REQUIRE((int)M.W.size() == N, "dmrg: an MPO of the sum has another length");
            menv.emplace_back(M.W);
        }
    std::vector<LocalOp> mops(menv.size());
    std::vector<MpsEnvironments> penv;
    if (prev)
        for (auto const& p : *prev) {
            ITG_REQUIRE((int)p.size() == N, "dmrg: an earlier state has another length");
            penv.emplace_back(p, H.sites);
        }
    std::vector<Tensor> proj(penv.size());
    DmrgResult res;
    double energy = 0;
    for (size_t sw = 0; sw < sweeps.size(); ++sw) {
        auto t0 = std::chrono::steady_clock::now();
        SweepSpec const& s = sweeps[sw];
        for (int b = 1, ha = 1; ha <= 2;) {
          try {
            using clk = std::chrono::steady_clock;
            auto tp0 = clk::now();
            LocalOp op = env.position(ctx, b, psi, prec);
            // phi on every block of its divergence, so H_eff and Davidson work on flat vectors
            Tensor const& A = psi[b - 1];
            Tensor const& B = psi[b];
            Match mt = match_indices(A.inds(), B.inds());
            std::vector<Index> pinds;
            for (int i : mt.a_unc) pinds.push_back(A.inds()[i]);
            for (int j : mt.b_unc) pinds.push_back(B.inds()[j]);
            auto full = std::make_shared<Layout>(allowed_layout(pinds, tensor_div(A) + tensor_div(B)));
            Tensor phi = contract(ctx, A, B, prec, full);
            if (!menv.empty()) {
                for (size_t k = 0; k < menv.size(); ++k) mops[k] = menv[k].position(ctx, b, psi, prec);
                op.terms = &mops;
            }
            if (!penv.empty()) {
                for (size_t j = 0; j < penv.size(); ++j) proj[j] = penv[j].projector(ctx, b, psi, full, PREC_F64);
                op.proj = &proj;
                op.proj_weight = weight;
            }
            auto tp1 = clk::now();
            energy = davidson(ctx, op, phi, s.niter, 1e-14, 1, prec, &res.heff_applies);
            auto tp2 = clk::now();
            SplitArgs sa;
            sa.cutoff = s.cutoff;
            sa.maxdim = s.maxdim;
            sa.mindim = s.mindim;
            sa.respect_degenerate = true;
            sa.normalize = true;
            // MPS::svdBond: SVD when UseSVD or (noise == 0 and cutoff < 1e-12), else density matrix
            // with the noise term (the SVD route ignores noise, as the reference does)
            const bool svd_route = s.use_svd || (s.noise == 0 && s.cutoff < 1e-12);
            SplitResult sr = svd_route ? svd_split(ctx, phi, A, B, ha == 1, sa, prec)
                                       : denmat_decomp(ctx, phi, A, B, ha == 1, sa, prec, &op, s.noise);
            // the new link keeps the old link's tags (MPS::svdBond, itensor/mps/mps_impl.h:81-84)
            if (!mt.a_con.empty()) {
                auto const& tags = A.inds()[mt.a_con[0]].tags;
                if (tags != std::array<char, TAG_BYTES>{}) {
                    sr.A = with_link_tags(sr.A, sr.link, tags);
                    sr.B = with_link_tags(sr.B, sr.link, tags);
                    sr.link.tags = tags;
                }
            }
            psi[b - 1] = sr.A;
            psi[b] = sr.B;
            auto tp3 = clk::now();
            res.phase_seconds[0] += std::chrono::duration<double>(tp1 - tp0).count();
            res.phase_seconds[1] += std::chrono::duration<double>(tp2 - tp1).count();
            res.phase_seconds[2] += std::chrono::duration<double>(tp3 - tp2).count();
            res.bonds.push_back(BondRecord{(int)sw + 1, ha, b, energy, sr.truncerr, (long)sr.link.dim()});
          } catch (Error const& e) {
            throw Error(e.code, std::string(e.what()) + " [sweep " + std::to_string(sw + 1) + ", half-sweep " +
                                    std::to_string(ha) + ", bond " + std::to_string(b) + "]");
          }
            // sweepnext: b = 1..N-1, then N-1..1
            const int inc = (ha == 1) ? 1 : -1;
            b += inc;
            if (b == (ha == 1 ? N : 0)) { b -= inc; ++ha; }
        }
        ctx.sync();
        res.sweep_seconds.push_back(std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count());
    }
    res.energy = energy;
    for (int b = 0; b + 1 < N; ++b) {
        Match mt = match_indices(psi[b].inds(), psi[b + 1].inds());
        ITG_REQUIRE(!mt.a_con.empty(), "dmrg: neighbouring tensors share no link");
        res.links.push_back(psi[b].inds()[mt.a_con[0]]);
    }
    res.psi = std::move(psi);
    return res;
}

}  // namespace itg
