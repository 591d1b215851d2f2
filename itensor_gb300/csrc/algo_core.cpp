// Tensor helpers, truncation, combiner, H_eff product, Davidson and the
// density-matrix bond split. All tensor arithmetic runs on the device; the
// host keeps block metadata, the (niter+2)-sized Rayleigh-Ritz matrix and the
// truncation decisions.
#include "algo.h"
#include "eigh_tri.h"
#include <algorithm>
#include <cmath>
#include <cstring>
#include <limits>
#include <numeric>

namespace itg {

void launch_random(Ctx& ctx, double* x, int64_t n, uint64_t seed);

// ---------------------------------------------------------------- tensors
Tensor upload_tensor(Ctx& ctx, std::shared_ptr<Layout> lay, double const* host) {
    Tensor t(lay, ctx.stream);
    if (lay->size > 0) {
        ctx.ensure_stage(sizeof(double) * lay->size);
        std::memcpy(ctx.stage, host, sizeof(double) * lay->size);
        ITG_CHECK_CUDA(cudaMemcpyAsync(t.data(), ctx.stage, sizeof(double) * lay->size, cudaMemcpyHostToDevice, ctx.stream));
        ctx.sync();
    }
    return t;
}

std::vector<double> download(Ctx& ctx, Tensor const& t) {
    std::vector<double> h(std::max<int64_t>(t.lay->size, 0));
    if (!h.empty()) {
        ctx.d2h(h.data(), t.data(), sizeof(double) * h.size());
    }
    return h;
}

QN tensor_div(Tensor const& t) {
    if (t.lay->nblocks() == 0 || t.rank() == 0) return QN();
    return t.lay->flux(t.lay->block(0));
}

std::vector<Index> prime_all(std::vector<Index> inds, int inc) {
    for (auto& I : inds) I = I.prime(inc);
    return inds;
}
std::vector<Index> dag_all(std::vector<Index> inds) {
    for (auto& I : inds) I = I.dag();
    return inds;
}
std::vector<Index> noprime_all(std::vector<Index> inds) {
    for (auto& I : inds) I = I.noprime();
    return inds;
}

Tensor copy_tensor(Ctx& ctx, Tensor const& t) {
    Tensor r(t.lay, ctx.stream);
    launch_copy(ctx, r.data(), t.data(), t.lay->size);
    r.scalar = t.scalar;
    return r;
}

double tensor_norm(Ctx& ctx, Tensor const& t) { return norm(ctx, t.data(), t.lay->size); }

// ---------------------------------------------------------------- truncate
TruncResult truncate(std::vector<double> P, long maxdim, long mindim, double cutoff, bool absoluteCutoff,
                     bool doRelCutoff, bool respectDegenerate) {
    TruncResult r;
    const double eps = std::numeric_limits<double>::epsilon();
    long origm = (long)P.size();
    long n = origm - 1;
    if (origm == 0) return r;
    if (P[0] == 0.0) {
        P.resize(1);
        r.P = P; r.truncerr = 0; r.docut_lower = -eps; r.docut_upper = eps; r.ndegen = 1;
        return r;
    }
    if (origm == 1) {
        double dc = 1e-3 * P[0];
        r.P = P; r.truncerr = 0; r.docut_lower = P[0] - dc; r.docut_upper = P[0] + dc; r.ndegen = 1;
        return r;
    }
    const double P0 = P[0];
    for (auto& x : P) x /= P0;
    if (absoluteCutoff || !doRelCutoff) cutoff /= P0;
    for (long zn = n; zn >= 0; --zn) {
        if (P[zn] >= 0) break;
        P[zn] = 0;
    }
    double truncerr = 0;
    while (n >= maxdim) { truncerr += P[n]; --n; }
    if (absoluteCutoff) {
        for (; P[n] <= cutoff && n >= mindim; --n) truncerr += P[n];
    } else {
        double scale = 1.0;
        if (doRelCutoff) {
            scale = 0;
            for (double x : P) scale += x;
            if (scale == 0.0) scale = 1.0;
        }
        while (truncerr + P[n] <= cutoff * scale && n >= mindim) { truncerr += P[n]; --n; }
        truncerr = (scale == 0 ? 0 : truncerr / scale);
    }
    if (n < 0) n = 0;
    long m = n + 1;
    double degen_cutoff = 1e-3 * P[n];
    if (P[n] == 0.0) degen_cutoff = eps;
    double lo = P[n] - degen_cutoff, up = P[n] + degen_cutoff;
    int ndegen_below = 1;
    if (n > 0)
        while ((n - ndegen_below >= 0) && (std::abs(P[n - ndegen_below] - P[n]) < degen_cutoff)) ++ndegen_below;
    int ndegen_above = 0;
    if (n + 1 < origm)
        while ((n + 1 + ndegen_above < origm) && (std::abs(P[n + 1 + ndegen_above] - P[n]) < degen_cutoff)) ++ndegen_above;
    if (respectDegenerate && (ndegen_below + ndegen_above > 1)) {
        if (maxdim < m + ndegen_above) {
            m -= ndegen_below;
            ndegen_above += ndegen_below;
            ndegen_below = 0;
        } else {
            m += ndegen_above;
            ndegen_below += ndegen_above;
            ndegen_above = 0;
        }
    }
    P.resize(m);
    for (auto& x : P) x *= P0;
    r.P = P;
    r.truncerr = truncerr * P0;
    r.docut_lower = lo * P0;
    r.docut_upper = up * P0;
    r.ndegen = ndegen_below;
    return r;
}

// ---------------------------------------------------------------- combiner
Combiner make_combiner(std::vector<Index> const& inds) {
    Combiner C;
    C.inds = inds;
    int cdir = 1;
    bool allin = !inds.empty();
    for (auto const& I : inds) if (I.dir != -1) { allin = false; break; }
    if (allin) cdir = -1;
    const int r = (int)inds.size();
    std::vector<QN> qs;
    std::vector<int32_t> ms;
    std::vector<int32_t> c(r, 0);
    while (true) {  // first fused index fastest
        QN q;
        int32_t m = 1;
        for (int k = 0; k < r; ++k) {
            q = q + inds[k].qn(c[k]).times(inds[k].dir * cdir);
            m *= inds[k].bdim(c[k]);
        }
        size_t n = 0;
        for (; n < qs.size(); ++n) if (qs[n] == q) break;
        if (n < qs.size()) {
            C.ranges[c] = {(int32_t)n, ms[n], m};
            ms[n] += m;
        } else {
            C.ranges[c] = {(int32_t)qs.size(), 0, m};
            qs.push_back(q);
            ms.push_back(m);
        }
        int k = 0;
        while (k < r) {
            if (++c[k] < inds[k].nblock()) break;
            c[k] = 0;
            ++k;
        }
        if (k == r) break;
    }
    C.ci = Index(qs, ms, cdir);
    return C;
}

namespace {
std::vector<int64_t> strides_of(Layout const& L, int b) {
    std::vector<int64_t> st(L.rank());
    int64_t s = 1;
    for (int k = 0; k < L.rank(); ++k) { st[k] = s; s *= L.inds[k].bdim(L.block(b)[k]); }
    return st;
}
std::vector<int32_t> offsets_for(std::vector<int> const& dims, std::vector<int64_t> const& strides, int64_t base = 0) {
    int n = (int)dims.size();
    int64_t total = 1;
    for (int d : dims) total *= d;
    std::vector<int32_t> out;
    out.reserve(total);
    std::vector<int> dig(n, 0);
    int64_t off = base;
    for (int64_t t = 0; t < total; ++t) {
        out.push_back((int32_t)off);
        for (int k = 0; k < n; ++k) {
            off += strides[k];
            if (++dig[k] < dims[k]) break;
            off -= strides[k] * dims[k];
            dig[k] = 0;
        }
    }
    return out;
}
}  // namespace

Tensor combine(Ctx& ctx, Tensor const& T, Combiner const& C) {
    Layout const& L = *T.lay;
    std::vector<int> pos;
    for (auto const& I : C.inds) {
        int p = L.find_index(I);
        ITG_REQUIRE(p >= 0, "combine: tensor lacks a fused index");
        pos.push_back(p);
    }
    std::vector<int> rest;
    for (int k = 0; k < L.rank(); ++k)
        if (std::find(pos.begin(), pos.end(), k) == pos.end()) rest.push_back(k);
    std::vector<Index> oinds{C.ci};
    for (int k : rest) oinds.push_back(L.inds[k]);
    const int ro = (int)oinds.size();
    std::vector<int32_t> ocoords;
    std::vector<std::array<int32_t, 3>> rng(L.nblocks());
    for (int b = 0; b < L.nblocks(); ++b) {
        std::vector<int32_t> sub;
        for (int p : pos) sub.push_back(L.block(b)[p]);
        rng[b] = C.ranges.at(sub);
        ocoords.push_back(rng[b][0]);
        for (int k : rest) ocoords.push_back(L.block(b)[k]);
    }
    auto O = std::make_shared<Layout>(make_layout(oinds, ocoords));
    Tensor out(O, ctx.stream);
    launch_fill(ctx, out.data(), O->size, 0.0);
    GatherPlan g;
    std::vector<int32_t> oc(ro);
    for (int b = 0; b < L.nblocks(); ++b) {
        auto st = strides_of(L, b);
        oc[0] = rng[b][0];
        for (size_t q = 0; q < rest.size(); ++q) oc[q + 1] = L.block(b)[rest[q]];
        int ob = O->find_block(oc.data());
        auto ost = strides_of(*O, ob);
        std::vector<int> d1, d2;
        std::vector<int64_t> s1, s2, o2;
        for (int p : pos) { d1.push_back(L.inds[p].bdim(L.block(b)[p])); s1.push_back(st[p]); }
        for (size_t q = 0; q < rest.size(); ++q) { d2.push_back(L.inds[rest[q]].bdim(L.block(b)[rest[q]])); s2.push_back(st[rest[q]]); o2.push_back(ost[q + 1]); }
        GatherItem it;
        it.soff = L.offs[b];
        it.doff = O->offs[ob] + rng[b][1];
        it.n1 = 1; for (int d : d1) it.n1 *= d;
        it.n2 = 1; for (int d : d2) it.n2 *= d;
        it.ts1 = g.add_table(offsets_for(d1, s1));
        it.ts2 = g.add_table(offsets_for(d2, s2));
        std::vector<int32_t> lin(it.n1);
        std::iota(lin.begin(), lin.end(), 0);
        it.td1 = g.add_table(lin);
        it.td2 = g.add_table(offsets_for(d2, o2));
        if (it.n1 > 0 && it.n2 > 0) g.items.push_back(it);
    }
    g.upload(ctx);
    launch_gather(ctx, g, T.data(), out.data());
    return out;
}

Tensor uncombine(Ctx& ctx, Tensor const& T, Combiner const& C) {
    Layout const& L = *T.lay;
    const int jc = L.find_index(C.ci);
    ITG_REQUIRE(jc >= 0, "uncombine: tensor lacks the fused index");
    const int nc = (int)C.inds.size();
    std::vector<Index> oinds(L.inds.begin(), L.inds.begin() + jc);
    oinds.insert(oinds.end(), C.inds.begin(), C.inds.end());
    oinds.insert(oinds.end(), L.inds.begin() + jc + 1, L.inds.end());
    struct Piece { int b; std::vector<int32_t> sub; int32_t start, ext; };
    std::vector<Piece> pieces;
    std::vector<int32_t> ocoords;
    for (int b = 0; b < L.nblocks(); ++b) {
        int n = L.block(b)[jc];
        for (auto const& kv : C.ranges) {
            if (kv.second[0] != n) continue;
            pieces.push_back(Piece{b, kv.first, kv.second[1], kv.second[2]});
            for (int k = 0; k < jc; ++k) ocoords.push_back(L.block(b)[k]);
            for (int s : kv.first) ocoords.push_back(s);
            for (int k = jc + 1; k < L.rank(); ++k) ocoords.push_back(L.block(b)[k]);
        }
    }
    auto O = std::make_shared<Layout>(make_layout(oinds, ocoords));
    Tensor out(O, ctx.stream);
    GatherPlan g;
    std::vector<int32_t> oc(O->rank());
    for (auto const& pc : pieces) {
        auto st = strides_of(L, pc.b);
        int q = 0;
        for (int k = 0; k < jc; ++k) oc[q++] = L.block(pc.b)[k];
        for (int s : pc.sub) oc[q++] = s;
        for (int k = jc + 1; k < L.rank(); ++k) oc[q++] = L.block(pc.b)[k];
        int ob = O->find_block(oc.data());
        auto ost = strides_of(*O, ob);
        // 1: the fused digits (rows start..start+ext of index jc); 2: all other indices
        std::vector<int> d1, d2;
        std::vector<int64_t> o1, s2, o2;
        for (int k = 0; k < nc; ++k) { d1.push_back(C.inds[k].bdim(pc.sub[k])); o1.push_back(ost[jc + k]); }
        for (int k = 0; k < L.rank(); ++k) {
            if (k == jc) continue;
            int ok = k < jc ? k : k + nc - 1;
            d2.push_back(L.inds[k].bdim(L.block(pc.b)[k]));
            s2.push_back(st[k]);
            o2.push_back(ost[ok]);
        }
        GatherItem it;
        it.soff = L.offs[pc.b];
        it.doff = O->offs[ob];
        it.n1 = pc.ext;
        it.n2 = 1; for (int d : d2) it.n2 *= d;
        std::vector<int32_t> srow(pc.ext);
        for (int i = 0; i < pc.ext; ++i) srow[i] = (int32_t)((pc.start + i) * st[jc]);
        it.ts1 = g.add_table(srow);
        it.ts2 = g.add_table(offsets_for(d2, s2));
        it.td1 = g.add_table(offsets_for(d1, o1));
        it.td2 = g.add_table(offsets_for(d2, o2));
        if (it.n1 > 0 && it.n2 > 0) g.items.push_back(it);
    }
    g.upload(ctx);
    launch_gather(ctx, g, T.data(), out.data());
    return out;
}

// ---------------------------------------------------------------- H_eff
Tensor heff_product(Ctx& ctx, LocalOp const& op, Tensor const& phi, int prec, bool into_phi_layout) {
    // the last contraction writes straight into phi's layout (all indices primed)
    std::shared_ptr<Layout> target;
    if (into_phi_layout) {
        target = std::make_shared<Layout>(*phi.lay);
        target->inds = prime_all(phi.lay->inds);
    }
    Tensor p;
    if (!op.L) {
        p = phi;
        if (op.R) p = contract(ctx, p, *op.R, prec);
        p = contract(ctx, p, *op.W2, prec);
        p = contract(ctx, p, *op.W1, prec, target);
    } else {
        p = contract(ctx, phi, *op.L, prec);
        p = contract(ctx, p, *op.W1, prec);
        if (op.R) {
            p = contract(ctx, p, *op.W2, prec);
            p = contract(ctx, p, *op.R, prec, target);
        } else {
            p = contract(ctx, p, *op.W2, prec, target);
        }
    }
    if (into_phi_layout) return relabel(p, phi.lay->inds);
    return relabel(p, noprime_all(p.inds()));
}

// ---------------------------------------------------------------- small symmetric eigensolver (host)
// Cyclic Jacobi for the (niter+2)-sized Rayleigh-Ritz matrix; eigenvalues
// ascending, eigenvectors in the columns of U (n x n, column-major).
static void small_eigh(int n, std::vector<double> M, std::vector<double>& w, std::vector<double>& U) {
    U.assign((size_t)n * n, 0.0);
    for (int i = 0; i < n; ++i) U[(size_t)i * n + i] = 1.0;
    auto a = [&](int i, int j) -> double& { return M[(size_t)j * n + i]; };
    for (int sweep = 0; sweep < 100; ++sweep) {
        double off = 0;
        for (int p = 0; p < n; ++p) for (int q = p + 1; q < n; ++q) off += a(p, q) * a(p, q);
        if (off < 1e-300) break;
        for (int p = 0; p < n; ++p)
            for (int q = p + 1; q < n; ++q) {
                double apq = a(p, q);
                if (std::abs(apq) < 1e-300) continue;
                double tau = (a(q, q) - a(p, p)) / (2 * apq);
                double t = (tau >= 0 ? 1.0 : -1.0) / (std::abs(tau) + std::sqrt(1 + tau * tau));
                double c = 1 / std::sqrt(1 + t * t), s = t * c;
                for (int k = 0; k < n; ++k) {
                    double kp = a(k, p), kq = a(k, q);
                    a(k, p) = c * kp - s * kq;
                    a(k, q) = s * kp + c * kq;
                }
                for (int k = 0; k < n; ++k) {
                    double pk = a(p, k), qk = a(q, k);
                    a(p, k) = c * pk - s * qk;
                    a(q, k) = s * pk + c * qk;
                }
                for (int k = 0; k < n; ++k) {
                    double up = U[(size_t)p * n + k], uq = U[(size_t)q * n + k];
                    U[(size_t)p * n + k] = c * up - s * uq;
                    U[(size_t)q * n + k] = s * up + c * uq;
                }
            }
    }
    std::vector<int> ord(n);
    std::iota(ord.begin(), ord.end(), 0);
    std::stable_sort(ord.begin(), ord.end(), [&](int x, int y) { return a(x, x) < a(y, y); });
    w.resize(n);
    std::vector<double> U2((size_t)n * n);
    for (int k = 0; k < n; ++k) {
        w[k] = a(ord[k], ord[k]);
        for (int i = 0; i < n; ++i) U2[(size_t)k * n + i] = U[(size_t)ord[k] * n + i];
    }
    U.swap(U2);
}

static int64_t dense_size(Tensor const& t) {
    int64_t s = 1;
    for (auto const& I : t.inds()) s *= I.dim();
    return s;
}

// Scalar slots of one Davidson call (Ctx::NSCALAR slots per context).
namespace {
enum DavSlot : int { S_NRM = 0, S_E0 = 1, S_Q = 2, S_G = 3, S_VQ = 8, S_M = 40, S_PZ = 72 };
static_assert(S_PZ + VecList::MAX <= Ctx::NSCALAR, "davidson: scalar slots");
}

// The reductions stay on the device: dot products and norms land in scalar
// slots that the next kernels read as coefficients, and the host reads them
// only where the reference's control flow branches on them. Each iteration
// runs ahead of its convergence test (Gram-Schmidt, the next apply and the
// projected matrix's new column are enqueued before the host reads the
// residual), so a call with niter 2 waits for its stream twice: after
// iteration 0 (<phi|H|phi>, the residual, the Gram-Schmidt norm, the new
// column) and after iteration 1 (the same). After a call that stopped on its
// residual, the next one waits for each residual first (four waits), so
// converged sweeps do not pay for extensions they drop. The arithmetic is that of the
// host-driven form (the same kernels, coefficients formed by the same
// products), so the results are bit-identical to it; work run ahead of a
// stop is dropped.
double davidson(Ctx& ctx, LocalOp const& op, Tensor& phi, int maxiter, double errgoal, int miniter, int prec,
                int* applies) {
    const double approx0 = 1e-12;
    const int64_t n = phi.lay->size;
    int napply = 0;
    ctx.ensure_scalars();
    double const* scal = ctx.scal_host;
    Tensor phi_in = phi;
    // |phi|^2 to the device; phi scaled there. A zero phi shows at the first
    // wait and takes the reference's re-randomising start instead.
    {
        VecList L;
        L.add(phi.data(), 0.0);
        dots_async(ctx, L, phi.data(), n, S_NRM);
    }
    phi = copy_tensor(ctx, phi);
    scale_rnorm(ctx, phi.data(), n, S_NRM);
    const int64_t maxsize = dense_size(phi);
    const int actual_maxiter = (int)std::min<int64_t>(maxiter, maxsize - 1);
    const int msz = actual_maxiter + 2;
    ITG_REQUIRE(msz + 1 <= VecList::MAX, "davidson: at most " + std::to_string(VecList::MAX - 3) + " iterations");
    std::vector<Tensor> V(msz), AV(msz);
    std::vector<double> M((size_t)msz * msz, std::numeric_limits<double>::quiet_NaN());
    auto Mat = [&](int i, int j) -> double& { return M[(size_t)j * msz + i]; };
    // one prepared program for every apply of this call (plans resolved once)
    // unfused MPO steps: the same arithmetic whether the solve runs alone or in
    // a solver pool (where the fusion's two extra plans cost more host time than
    // the launch they save), so a solve's result does not depend on where it runs
    auto prog = heff_prepare(ctx, op, phi.lay, prec, true, false, false);
    const int nproj = op.proj ? (int)op.proj->size() : 0;
    ITG_REQUIRE(nproj <= VecList::MAX, "davidson: too many projected states");
    std::vector<double const*> pptr(nproj);
    for (int j = 0; j < nproj; ++j) {
        ITG_REQUIRE((*op.proj)[j].lay->size == n, "davidson: projector not in phi's layout");
        pptr[j] = (*op.proj)[j].data();
    }
    // the other MPOs of a sum, each its own prepared program, added to y
    std::vector<std::shared_ptr<HeffProgram>> more;
    if (op.terms)
        for (auto const& t : *op.terms) more.push_back(heff_prepare(ctx, t, phi.lay, prec, true, false));
    Tensor tmp;
    if (!more.empty()) tmp = Tensor(phi.lay, ctx.stream);
    auto apply = [&](Tensor const& x) {
        Tensor y(phi.lay, ctx.stream);
        prog->run(ctx, x.data(), y.data());
        for (auto const& p : more) {
            p->run(ctx, x.data(), tmp.data());
            VecList X;
            X.add(tmp.data(), 1.0);
            combo_async(ctx, y.data(), 1.0, X, n, -1);
        }
        if (nproj) {
            // y += w sum_j P_j (P_j . x), the dot products left on the device
            VecList P, X;
            for (int j = 0; j < nproj; ++j) P.add(pptr[j], 0.0);
            dots_async(ctx, P, x.data(), n, S_PZ);
            for (int j = 0; j < nproj; ++j) X.add(pptr[j], op.proj_weight, S_PZ + j);
            combo_async(ctx, y.data(), 1.0, X, n, -1);
        }
        ++napply;
        return y;
    };
    // Gram-Schmidt of q against V[0..ni-1] and normalisation, on the device
    auto gs_device = [&](Tensor& q, int ni) {
        VecList Lv, Lg;
        for (int k = 0; k < ni; ++k) Lv.add(V[k].data(), 0.0);
        dots_async(ctx, Lv, q.data(), n, S_VQ);
        for (int k = 0; k < ni; ++k) Lg.add(V[k].data(), -1.0, S_VQ + k);
        combo_async(ctx, q.data(), 1.0, Lg, n, S_G);
        scale_rnorm(ctx, q.data(), n, S_G);
    };
    V[0] = phi;
    AV[0] = apply(V[0]);
    {
        VecList L;
        L.add(V[0].data(), 0.0);
        dots_async(ctx, L, AV[0].data(), n, S_E0);
    }
    double initEn = 0, last_lambda = 1000.0, lambda = 0;
    const bool run_ahead = !ctx.dav_stopped_early;
    bool stopped_early = false;
    Tensor phi_t = phi;
    std::vector<double> D, U;
    int ii = 0;
    for (ii = 0; ii <= actual_maxiter; ++ii) {
        const int ni = ii + 1;
        Tensor q(phi.lay, ctx.stream);
        if (ii == 0) {
            // q = H V0 - lambda V0 and |q|^2, lambda = <V0|H|V0> from its slot
            VecList L;
            L.add(AV[0].data(), 1.0);
            L.add(V[0].data(), -1.0, S_E0);
            combo_async(ctx, q.data(), 0.0, L, n, S_Q);
        } else {
            std::vector<double> Msub((size_t)(ii + 1) * (ii + 1));
            for (int j = 0; j <= ii; ++j) for (int i = 0; i <= ii; ++i) Msub[(size_t)j * (ii + 1) + i] = Mat(i, j);
            small_eigh(ii + 1, Msub, D, U);
            lambda = D[0];
            const double sgn = U[0] < 0 ? -1.0 : 1.0;  // fix sign: U(0,t) >= 0
            Tensor pt(phi.lay, ctx.stream);
            // Ritz vector pt = sum_k u_k V_k and residual q = sum_k u_k H V_k - lambda pt
            VecList Lp, Lq;
            for (int k = 0; k <= ii; ++k) {
                Lp.add(V[k].data(), sgn * U[k]);
                Lq.add(AV[k].data(), sgn * U[k]);
            }
            Lq.add(pt.data(), -lambda);
            combo_async(ctx, pt.data(), 0.0, Lp, n, -1);
            phi_t = pt;
            // the last iteration stops whatever the residual: it is not needed
            if (ii == actual_maxiter) break;
            combo_async(ctx, q.data(), 0.0, Lq, n, S_Q);
        }
        // one Gram-Schmidt pass on the device, the next vector applied and its
        // column of the projected matrix formed
        auto extend = [&] {
            gs_device(q, ni);
            V[ni] = q;
            AV[ni] = apply(V[ni]);
            VecList Lv;
            for (int k = 0; k <= ni; ++k) Lv.add(V[k].data(), 0.0);
            dots_async(ctx, Lv, AV[ni].data(), n, S_M);
        };
        // Ahead of the host's look at the residual, unless the last call
        // stopped on its residual (then this one likely does too): one wait
        // returns the residual and the extension. When the residual ends the
        // iteration the extension is dropped (the results are those of the
        // stop before it).
        const bool ahead = run_ahead && ii < actual_maxiter;
        if (ahead) extend();
        ctx.sync();
        if (ii == 0) {
            if (!(scal[S_NRM] > 0.0)) {
                // zero starting vector: the reference's random restart
                // (itensor/iterativesolvers.h), which needs the host in the loop
                phi = phi_in;
                double nrm = tensor_norm(ctx, phi);
                int guard = 0;
                while (nrm == 0.0 && guard++ < 4) {
                    launch_random(ctx, phi.data(), n, 0x5eed + guard);
                    nrm = tensor_norm(ctx, phi);
                }
                ITG_REQUIRE(nrm > 0, "davidson: zero initial vector");
                return davidson(ctx, op, phi, maxiter, errgoal, miniter, prec, applies);
            }
            initEn = scal[S_E0];
            lambda = initEn;
            Mat(0, 0) = lambda;
        }
        const double qnorm = std::sqrt(std::max(scal[S_Q], 0.0));
        const bool converged = (qnorm < errgoal && std::abs(lambda - last_lambda) < errgoal) ||
                               qnorm < std::max(approx0, errgoal * 1e-3);
        last_lambda = lambda;
        if (qnorm < 1e-20 || (converged && ii >= miniter) || ii == actual_maxiter) {
            if (ahead) --napply;  // the apply made ahead is not part of the result
            stopped_early = ii < actual_maxiter;
            break;
        }
        if (!ahead) {
            extend();
            ctx.sync();
        }
        double qnrm = std::sqrt(std::max(scal[S_G], 0.0));
        if (qnrm < 1e-10) {
            // q depended on V: the pass above divided by a tiny norm. Redo it
            // the reference's way from there (re-randomise; rare)
            --napply;
            int pass = 1, tot_pass = 1;
            bool done = false;
            for (;;) {
                if (qnrm < 1e-10) {
                    launch_random(ctx, q.data(), n, 0x9e3779b9ull * (ni + 7 * tot_pass));
                    qnrm = norm(ctx, q.data(), n);
                    --pass;
                    if (ni >= maxsize || tot_pass > 3) { done = true; break; }
                }
                launch_scale(ctx, q.data(), n, 1.0 / qnrm);
                ++pass;
                if (pass > 1) break;
                ++tot_pass;
                std::vector<double const*> vp(ni);
                for (int k = 0; k < ni; ++k) vp[k] = V[k].data();
                std::vector<double> Vq(ni);
                dots(ctx, vp.data(), ni, q.data(), n, Vq.data());
                VecList Lg;
                for (int k = 0; k < ni; ++k) Lg.add(V[k].data(), -Vq[k]);
                qnrm = std::sqrt(std::max(combo(ctx, q.data(), 1.0, Lg, n, true), 0.0));
            }
            if (done) break;
            V[ni] = q;
            AV[ni] = apply(V[ni]);
            VecList Lv;
            for (int k = 0; k <= ni; ++k) Lv.add(V[k].data(), 0.0);
            dots_async(ctx, Lv, AV[ni].data(), n, S_M);
            ctx.sync();
        }
        for (int k = 0; k <= ni; ++k) { Mat(k, ni) = scal[S_M + k]; Mat(ni, k) = scal[S_M + k]; }
    }
    phi = phi_t;
    ctx.dav_stopped_early = stopped_early;
    if (applies) *applies += napply;
    return lambda;
}

// ---------------------------------------------------------------- density-matrix bond split
Tensor delta_rho(Ctx& ctx, LocalOp const& op, Tensor const& AA, Combiner const& cmb, bool fromleft) {
    Tensor const* env = fromleft ? op.L : op.R;
    Tensor const* W = fromleft ? op.W1 : op.W2;
    ITG_REQUIRE(W, "delta_rho: missing MPO tensor");
    Tensor X = env ? contract(ctx, AA, *env, PREC_F64) : AA;
    X = contract(ctx, X, *W, PREC_F64);
    X = relabel(X, noprime_all(X.inds()));
    Tensor Xc = combine(ctx, X, cmb);
    std::vector<Index> dinds = dag_all(Xc.inds());
    dinds[0] = dinds[0].prime();
    return contract(ctx, Xc, relabel(Xc, dinds), PREC_F64);
}

// rho + noise * sum_k (D_k + D_k^T)/2 on the union of the block structures,
// divided by its trace (itensor/decomp.h:386-394; ITensor's += keeps every
// block of either operand).
static Tensor noisy_rho(Ctx& ctx, Tensor const& rho, std::vector<Tensor> const& Ds, double noise) {
    Layout const& RL = *rho.lay;
    std::vector<int32_t> coords(RL.coords);
    for (auto const& D : Ds) coords.insert(coords.end(), D.lay->coords.begin(), D.lay->coords.end());
    auto UL = std::make_shared<Layout>(make_layout(rho.inds(), coords));
    Tensor out(UL, ctx.stream);
    std::vector<std::vector<NoiseBlock>> passes(Ds.size(), std::vector<NoiseBlock>(UL->nblocks()));
    std::vector<double const*> ds;
    for (size_t k = 0; k < Ds.size(); ++k) {
        Layout const& DL = *Ds[k].lay;
        ds.push_back(Ds[k].data());
        for (int b = 0; b < UL->nblocks(); ++b) {
            int32_t const* c = UL->block(b);
            ITG_REQUIRE(c[0] == c[1], "noisy_rho: density matrix block off the diagonal");
            const int rb = RL.find_block(c), db = DL.find_block(c);
            NoiseBlock& nb = passes[k][b];
            nb.out_off = UL->offs[b];
            // pass 0 reads rho (or nothing where rho has no block); later passes read out
            nb.rho_off = k == 0 ? (rb >= 0 ? RL.offs[rb] : -1) : UL->offs[b];
            nb.d_off = db >= 0 ? DL.offs[db] : -1;
            nb.n = (int32_t)rho.inds()[0].bdim(c[0]);
            nb.pad = 0;
        }
    }
    launch_noisy_rho(ctx, passes, rho.data(), ds, out.data(), UL->size, noise);
    return out;
}

SplitResult denmat_decomp(Ctx& ctx, Tensor const& AA, Tensor const& A, Tensor const& B, bool fromleft,
                          SplitArgs const& args, int prec, LocalOp const* op, double noise) {
    Tensor const& to_orth = fromleft ? A : B;
    Tensor const& newoc = fromleft ? B : A;
    std::vector<Index> cinds;
    for (auto const& I : to_orth.inds()) if (newoc.lay->find_index(I) < 0) cinds.push_back(I);
    Combiner cmb = make_combiner(cinds);
    Tensor AAc = combine(ctx, AA, cmb);
    const Index ci = cmb.ci;
    // rho = AAc * dag(prime(AAc, ci)), indices (ci, ci')
    std::vector<Index> dinds = dag_all(AAc.inds());
    dinds[0] = dinds[0].prime();
    Tensor rho = contract(ctx, AAc, relabel(AAc, dinds), PREC_F64);
    if (noise > 0 && op) {
        // LocalMPOSet::deltaRho sums the terms of every MPO (itensor/mps/localmposet.h:166-176)
        std::vector<Tensor> Ds{delta_rho(ctx, *op, AA, cmb, fromleft)};
        if (op->terms)
            for (auto const& t : *op->terms) Ds.push_back(delta_rho(ctx, t, AA, cmb, fromleft));
        rho = noisy_rho(ctx, rho, Ds, noise);
    }
    Layout const& RL = *rho.lay;
    // one eigenproblem per diagonal block, in storage order
    const int nb = RL.nblocks();
    std::vector<EigItem> items(nb);
    std::vector<int> bsec(nb), bn(nb);
    int64_t vtot = 0, wtot = 0, stot = 0;
    for (int b = 0; b < nb; ++b) {
        int sec = RL.block(b)[0];
        int n = ci.bdim(sec);
        bsec[b] = sec; bn[b] = n;
        items[b].a_off = RL.offs[b];
        items[b].n = n;
        items[b].v_off = vtot; vtot += (int64_t)n * n;
        items[b].w_off = wtot; wtot += n;
        items[b].s_off = stot; stot += 2 * (int64_t)n * n;
        items[b].pad = 0;
    }
    DevBuf vbuf(sizeof(double) * std::max<int64_t>(vtot, 1), ctx.stream);
    DevBuf wbuf(sizeof(double) * std::max<int64_t>(wtot, 1), ctx.stream);
    DevBuf sbuf(sizeof(double) * std::max<int64_t>(stot, 1), ctx.stream);
    // eigenvalues first; the eigenvectors of the large blocks only for the kept states
    EighPending eig = batched_eigh_begin(ctx, items, rho.data(), vbuf.as<double>(), wbuf.as<double>(),
                                         sbuf.as<double>());
    std::vector<double> w(std::max<int64_t>(wtot, 1));
    // one wait: the eigenvalues, and the convergence statuses enqueued before them
    if (wtot) ctx.d2h(w.data(), wbuf.as<double>(), sizeof(double) * wtot);
    else if (eig.jac_pending) ctx.sync();
    if (eigh_collect(ctx, eig)) throw Error(ERR_NOCONV, "denmat_decomp: eigensolver hit its sweep cap");
    std::vector<double> alleig(w.begin(), w.begin() + wtot);
    std::sort(alleig.begin(), alleig.end(), std::greater<double>());
    const long maxdim = args.maxdim > 0 ? args.maxdim : (long)ci.dim();
    TruncResult tr = truncate(alleig, maxdim, args.mindim, args.cutoff, false, true, args.respect_degenerate);
    const long m = (long)tr.P.size();
    int ndegen = tr.ndegen;
    std::vector<int> keep(nb, 0);
    long total_m = 0;
    for (int b = 0; b < nb; ++b) {
        double const* d = w.data() + items[b].w_off;
        int this_m = 0;
        while (this_m < bn[b] && total_m < m && d[this_m] > tr.docut_upper) { ++this_m; ++total_m; }
        while (ndegen > 0 && this_m < bn[b] && total_m < m && d[this_m] > tr.docut_lower) {
            ++this_m; ++total_m; --ndegen;
        }
        keep[b] = this_m;
    }
    batched_eigh_finish(ctx, eig, keep, vbuf.as<double>(), sbuf.as<double>());
    std::vector<QN> dq;
    std::vector<int32_t> dd;
    for (int b = 0; b < nb; ++b) if (keep[b] > 0) { dq.push_back(ci.qn(bsec[b])); dd.push_back(keep[b]); }
    bool empty = dq.empty();
    if (empty) {
        ITG_REQUIRE(nb > 0, "denmat_decomp: no blocks");
        dq.push_back(ci.qn(bsec[0]));
        dd.push_back(1);
    }
    Index dind(dq, dd, -ci.dir);
    // U(dag(ci), dag(d)): block (sec, n) = first keep columns of that block's eigenvectors
    std::vector<int32_t> ucoords;
    {
        int nn = 0;
        for (int b = 0; b < nb; ++b)
            if (keep[b] > 0) { ucoords.push_back(bsec[b]); ucoords.push_back(nn++); }
    }
    auto UL = std::make_shared<Layout>(make_layout({ci.dag(), dind.dag()}, empty ? std::vector<int32_t>{} : ucoords));
    Tensor U(UL, ctx.stream);
    if (!empty) {
        GatherPlan g;
        int nn = 0;
        for (int b = 0; b < nb; ++b) {
            if (keep[b] == 0) continue;
            int32_t c[2] = {bsec[b], nn++};
            int ub = UL->find_block(c);
            GatherItem it;
            it.soff = items[b].v_off;
            it.doff = UL->offs[ub];
            it.n1 = bn[b] * keep[b];
            it.n2 = 1;
            std::vector<int32_t> lin(it.n1);
            std::iota(lin.begin(), lin.end(), 0);
            it.ts1 = g.add_table(lin);
            it.td1 = it.ts1;
            it.ts2 = g.add_table({0});
            it.td2 = it.ts2;
            g.items.push_back(it);
        }
        g.upload(ctx);
        launch_gather(ctx, g, vbuf.as<double>(), U.data());
    }
    // to_orth = cmb^dag * dag(U): indices (cinds..., d); newoc = U * AAc: (dag(d), rest...)
    Tensor Ud = relabel(U, dag_all(U.inds()));
    Tensor new_orth = uncombine(ctx, Ud, cmb);
    Tensor new_oc = contract(ctx, U, AAc, prec);
    // new_oc /= |new_oc| when |new_oc| > 1e-16, on the device (no wait)
    if (args.normalize) normalize_async(ctx, new_oc.data(), new_oc.lay->size, 1e-16);
    SplitResult res;
    res.probs = tr.P;
    res.truncerr = tr.truncerr;
    res.link = dind;
    if (fromleft) { res.A = new_orth; res.B = new_oc; }
    else { res.A = new_oc; res.B = new_orth; }
    return res;
}

}  // namespace itg
