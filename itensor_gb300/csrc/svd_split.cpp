// SVD route of the bond split (MPS::svdBond with UseSVD or cutoff < 1e-12):
// svd (itensor/decomp.cc:121-248) -> svdImpl's QN branch (itensor/svd.cc:169-401).
// The fused matrix AAc(vi, ui) is decomposed block by block on the device
// (one-sided Jacobi, svd.cu); the truncation decisions run on the host with the
// reference's truncate and per-block keep rule (on s^2).
#include "algo.h"
#include <algorithm>
#include <cmath>
#include <cstring>
#include <numeric>

namespace itg {

SplitResult svd_split(Ctx& ctx, Tensor const& AA, Tensor const& A, Tensor const& B, bool fromleft,
                      SplitArgs const& args, int prec) {
    std::vector<Index> Uinds, Vinds;
    for (auto const& I : AA.inds()) {
        if (A.lay->find_index(I) >= 0 && B.lay->find_index(I) < 0) Uinds.push_back(I);
        else Vinds.push_back(I);
    }
    ITG_REQUIRE(!Uinds.empty() && !Vinds.empty(), "svd_split: empty index group");
    Combiner cu = make_combiner(Uinds), cv = make_combiner(Vinds);
    Tensor AAc = combine(ctx, combine(ctx, AA, cu), cv);  // indices (vi, ui)
    Layout const& L = *AAc.lay;
    const Index ui = cu.ci, vi = cv.ci;
    const int nb = L.nblocks();
    std::vector<SvdItem> items(nb);
    std::vector<int> bu(nb), bv(nb), du(nb), dv(nb), k(nb);
    int64_t uo = 0, so = 0, vo = 0, sc = 0;
    for (int b = 0; b < nb; ++b) {
        bv[b] = L.block(b)[0];
        bu[b] = L.block(b)[1];
        dv[b] = vi.bdim(bv[b]);
        du[b] = ui.bdim(bu[b]);
        SvdItem it;
        it.a_off = L.offs[b];
        it.ld = dv[b];  // the stored block is dv x du, column-major
        if (dv[b] >= du[b]) { it.rows = dv[b]; it.cols = du[b]; it.transpose = 0; }  // X = block = M^T
        else { it.rows = du[b]; it.cols = dv[b]; it.transpose = 1; }                  // X = block^T = M
        k[b] = it.cols;
        it.u_off = uo; uo += (int64_t)it.rows * it.cols;
        it.v_off = vo; vo += (int64_t)it.cols * it.cols;
        it.s_out = so; so += it.cols;
        it.s_off = sc; sc += (int64_t)it.rows * it.cols + (int64_t)it.cols * it.cols + it.cols;
        items[b] = it;
    }
    // both factor sets in one buffer: [left factors of X | right factors of X]
    for (auto& it : items) it.v_off += uo;
    DevBuf fac(sizeof(double) * std::max<int64_t>(uo + vo, 1), ctx.stream);
    DevBuf sbuf(sizeof(double) * std::max<int64_t>(so, 1), ctx.stream);
    DevBuf scr(sizeof(double) * std::max<int64_t>(sc, 1), ctx.stream);
    if (batched_svd(ctx, items, AAc.data(), fac.as<double>(), sbuf.as<double>(), fac.as<double>(), scr.as<double>()))
        throw Error(ERR_NOCONV, "svd_split: singular value decomposition hit its sweep cap");
    std::vector<double> s(std::max<int64_t>(so, 1));
    if (so) {
        ctx.d2h(s.data(), sbuf.p, sizeof(double) * so);
    }
    std::vector<double> probs;
    for (int64_t i = 0; i < so; ++i) probs.push_back(s[i] * s[i]);
    std::sort(probs.begin(), probs.end(), std::greater<double>());
    ITG_REQUIRE(!probs.empty(), "svd_split: tensor has no blocks");
    const long maxdim = args.maxdim > 0 ? args.maxdim : (long)probs.size();
    TruncResult tr = truncate(probs, maxdim, args.mindim, args.cutoff, false, true, args.respect_degenerate);
    const long m = (long)tr.P.size();
    int ndegen = tr.ndegen;
    std::vector<int> keep(nb, 0);
    long total_m = 0;
    for (int b = 0; b < nb; ++b) {
        double const* d = s.data() + items[b].s_out;
        int this_m = 0;
        while (this_m < k[b] && total_m < m && d[this_m] * d[this_m] > tr.docut_upper) { ++this_m; ++total_m; }
        while (ndegen > 0 && this_m < k[b] && total_m < m && d[this_m] * d[this_m] > tr.docut_lower) {
            ++this_m; ++total_m; --ndegen;
        }
        keep[b] = this_m;
    }
    std::vector<QN> lq, rq;
    std::vector<int32_t> kd;
    for (int b = 0; b < nb; ++b)
        if (keep[b] > 0) { lq.push_back(ui.qn(bu[b])); rq.push_back(vi.qn(bv[b])); kd.push_back(keep[b]); }
    ITG_REQUIRE(!kd.empty(), "svd_split: nothing kept");
    Index Lidx(lq, kd, ui.dir), Ridx(rq, kd, vi.dir);
    // U(ui, dag L), V(vi, dag R), D(L, R)
    std::vector<int32_t> uc, vc, dc;
    std::vector<int> kb;  // kept block numbers in order
    for (int b = 0, n = 0; b < nb; ++b)
        if (keep[b] > 0) {
            uc.insert(uc.end(), {bu[b], n});
            vc.insert(vc.end(), {bv[b], n});
            dc.insert(dc.end(), {n, n});
            kb.push_back(b);
            ++n;
        }
    auto UL = std::make_shared<Layout>(make_layout({ui, Lidx.dag()}, uc));
    auto VL = std::make_shared<Layout>(make_layout({vi, Ridx.dag()}, vc));
    auto DL = std::make_shared<Layout>(make_layout({Lidx, Ridx}, dc));
    Tensor U(UL, ctx.stream), V(VL, ctx.stream);
    // first keep columns of the block factors: contiguous column-major prefixes
    GatherPlan gu, gv;
    for (size_t n = 0; n < kb.size(); ++n) {
        const int b = kb[n];
        const SvdItem& it = items[b];
        const bool tr_ = it.transpose != 0;
        // left factor of M (u-space): V_x (no transpose) or U_x (transpose); right factor: the other
        const int64_t usrc = tr_ ? it.u_off : it.v_off;
        const int64_t vsrc = tr_ ? it.v_off : it.u_off;
        auto add = [&](GatherPlan& g, Layout const& TL, int32_t c0, int64_t src, int rows) {
            int32_t cc[2] = {c0, (int32_t)n};
            const int tb = TL.find_block(cc);
            GatherItem gi;
            gi.soff = src;
            gi.doff = TL.offs[tb];
            gi.n1 = rows * keep[b];
            gi.n2 = 1;
            std::vector<int32_t> lin(gi.n1);
            std::iota(lin.begin(), lin.end(), 0);
            gi.ts1 = gi.td1 = g.add_table(lin);
            gi.ts2 = gi.td2 = g.add_table({0});
            g.items.push_back(gi);
        };
        add(gu, *UL, bu[b], usrc, du[b]);
        add(gv, *VL, bv[b], vsrc, dv[b]);
    }
    gu.upload(ctx);
    launch_gather(ctx, gu, fac.as<double>(), U.data());
    gv.upload(ctx);
    launch_gather(ctx, gv, fac.as<double>(), V.data());
    // D on the host: diagonal blocks of the kept singular values
    std::vector<double> dh(DL->size, 0.0);
    double dn2 = 0;
    for (size_t n = 0; n < kb.size(); ++n) {
        const int b = kb[n];
        int32_t cc[2] = {(int32_t)n, (int32_t)n};
        const int db = DL->find_block(cc);
        for (int i = 0; i < keep[b]; ++i) {
            const double v = s[items[b].s_out + i];
            dh[DL->offs[db] + i + (int64_t)keep[b] * i] = v;
            dn2 += v * v;
        }
    }
    if (args.normalize && dn2 > 0)
        for (auto& x : dh) x /= std::sqrt(dn2);
    Tensor D = upload_tensor(ctx, DL, dh.data());
    Tensor Uo = uncombine(ctx, U, cu);
    Tensor Vo = uncombine(ctx, V, cv);
    SplitResult res;
    res.probs = tr.P;
    res.truncerr = tr.truncerr;
    res.link = Lidx;
    if (fromleft) { res.A = Uo; res.B = contract(ctx, Vo, D, prec); }
    else { res.A = contract(ctx, Uo, D, prec); res.B = Vo; }
    return res;
}

}  // namespace itg
