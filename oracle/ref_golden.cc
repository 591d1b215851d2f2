// Golden-fixture generator. Links the ITensor C++ reference (built from its own
// sources by oracle/Makefile.ref) and writes JSON fixtures holding both the
// inputs and the reference outputs of each hot-path operation:
//   contract   doTask(Contract,QDense,QDense)   itensor/itdata/qdense.cc:671-743
//   heff       LocalOp::product                 itensor/mps/localop.h:324-365
//   davidson   davidson                         itensor/iterativesolvers.h:99-451
//   truncate   truncate                         itensor/decomp.cc:305-463
//   denmat     denmatDecomp / diag_hermitian    itensor/decomp.h:316-418, itensor/hermitian.cc:180-426
//   svd        svd (QN)                          itensor/decomp.cc:121-248, itensor/svd.cc:169-422
//   dmrg       dmrg() with a recording observer itensor/mps/dmrg.h:336-467
// Test infrastructure only; run by tests/golden/make_golden.py in a container
// that has the reference sources.
#include "itensor/all.h"
#include "itensor/itdata/qdense.h"
#include "Heisenberg.h"
#include <cstdio>
#include <fstream>
#include <sstream>
#include <string>
#include <cmath>
#include <cstdint>
#include <chrono>
#include <cstdlib>

using namespace itensor;

// ---------------------------------------------------------------- RNG
// splitmix64 -> uniform [0,1) -> Box-Muller normal. The fixture stores the
// values themselves, so nothing downstream needs to reproduce this stream.
struct Rng {
    uint64_t s;
    explicit Rng(uint64_t seed) : s(seed) {}
    uint64_t next() {
        uint64_t z = (s += 0x9e3779b97f4a7c15ULL);
        z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
        z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
        return z ^ (z >> 31);
    }
    double uni() { return (next() >> 11) * (1.0 / 9007199254740992.0); }
    double normal() {
        double u1 = uni(), u2 = uni();
        if (u1 < 1e-300) u1 = 1e-300;
        return std::sqrt(-2.0 * std::log(u1)) * std::cos(6.283185307179586 * u2);
    }
};

// ---------------------------------------------------------------- JSON helpers
static std::string num(double x) {
    char b[40];
    std::snprintf(b, sizeof b, "%.17g", x);
    return b;
}

static std::string jqn(QN const& q) {
    std::ostringstream o;
    o << "[";
    bool first = true;
    for (size_t n = 0; n < QNSize(); ++n) {
        auto const& v = q.num(n);
        if (v.mod() == 0) continue;
        if (!first) o << ",";
        first = false;
        o << "[\"" << std::string(v.name()) << "\"," << v.val() << "," << v.mod() << "]";
    }
    o << "]";
    return o.str();
}

static std::string jindex(Index const& I) {
    std::ostringstream o;
    o << "{\"id\":\"" << id(I) << "\",\"plev\":" << primeLevel(I) << ",\"dir\":" << int(I.dir())
      << ",\"tags\":\"" << tags(I) << "\",\"sectors\":[";
    for (long b = 1; b <= I.nblock(); ++b) {
        if (b > 1) o << ",";
        o << "[" << jqn(I.qn(b)) << "," << I.blocksize0(b - 1) << "]";
    }
    o << "]}";
    return o.str();
}

static QDenseReal const* qdense_of(ITensor const& T) {
    auto* w = dynamic_cast<ITWrap<QDenseReal> const*>(&*T.store());
    return w ? &w->d : nullptr;
}
static QDenseReal* qdense_of_mut(ITensor& T) {
    auto* w = dynamic_cast<ITWrap<QDenseReal>*>(T.store().get());
    return w ? &w->d : nullptr;
}

// Block-sparse tensor: indices, block coordinates (0-based sector numbers),
// element offsets and the data, with the ITensor scale folded in.
static std::string jtensor(ITensor T) {
    std::ostringstream o;
    o << "{\"inds\":[";
    for (long j = 0; j < order(T); ++j) {
        if (j) o << ",";
        o << jindex(inds(T)[j]);
    }
    o << "]";
    if (!T) { o << ",\"blocks\":[],\"offsets\":[],\"data\":[]}"; return o.str(); }
    T.scaleTo(1.0);
    auto* d = qdense_of(T);
    if (!d) {
        // rank-0 result or non-QDense storage: report the single value
        o << ",\"scalar\":" << num(elt(T)) << "}";
        return o.str();
    }
    o << ",\"blocks\":[";
    for (size_t b = 0; b < d->offsets.size(); ++b) {
        if (b) o << ",";
        o << "[";
        auto const& blk = d->offsets[b].block;
        for (size_t k = 0; k < blk.size(); ++k) { if (k) o << ","; o << blk[k]; }
        o << "]";
    }
    o << "],\"offsets\":[";
    for (size_t b = 0; b < d->offsets.size(); ++b) { if (b) o << ","; o << d->offsets[b].offset; }
    o << "],\"data\":[";
    for (size_t i = 0; i < d->store.size(); ++i) { if (i) o << ","; o << num(d->store[i]); }
    o << "]}";
    return o.str();
}

static void fill_normal(ITensor& T, Rng& r) {
    auto* d = qdense_of_mut(T);
    if (!d) { std::fprintf(stderr, "fill_normal: not QDense\n"); std::exit(1); }
    for (auto& x : d->store) x = r.normal();
}

// QN tensor holding only the listed blocks (block-deficient), N(0,1) entries.
static ITensor deficient(IndexSet const& is, QN const& div, Rng& r, double keep_frac) {
    ITensor full(div, is);
    auto* d = qdense_of(full);
    Blocks keep;
    for (auto const& bo : d->offsets)
        if (r.uni() < keep_frac) keep.push_back(bo.block);
    if (keep.empty()) keep.push_back(d->offsets.front().block);
    auto T = ITensor(is, QDenseReal(is, keep));
    fill_normal(T, r);
    return T;
}

static ITensor randqn(QN const& div, IndexSet const& is, Rng& r) {
    ITensor T(div, is);
    fill_normal(T, r);
    return T;
}

static void write_file(std::string const& path, std::string const& body) {
    std::ofstream f(path);
    f << body << "\n";
    std::printf("wrote %s (%zu bytes)\n", path.c_str(), body.size());
}

// ---------------------------------------------------------------- index builders
static QN sz(int v) { return QN({"Sz", v}); }
static QN nfsz(int n, int s) { return QN({"Nf", n, -1}, {"Sz", s}); }
static QN par(int p) { return QN({"Parity", p, 2}); }

static Index mkidx(std::vector<std::pair<QN, long>> secs, Arrow dir, std::string const& tags) {
    Index::qnstorage st;
    for (auto& s : secs) st.emplace_back(s.first, s.second);
    return Index(std::move(st), dir, TagSet(tags));
}

// Sz link of total dimension m over 2K+1 sectors q=2(k-K), Gaussian sizes
// floor(m*g_k/sum g) with g_k = exp(-(k-K)^2/(2 sigma^2)), remainder to the
// centre sector (the synthetic bond layout of the isolated H_eff workload).
static Index gauss_link(long m, int K, double sigma, Arrow dir, std::string const& tags) {
    std::vector<double> g(2 * K + 1);
    double tot = 0;
    for (int k = 0; k <= 2 * K; ++k) { g[k] = std::exp(-(k - K) * (k - K) / (2 * sigma * sigma)); tot += g[k]; }
    std::vector<long> sizes(2 * K + 1);
    long used = 0;
    for (int k = 0; k <= 2 * K; ++k) { sizes[k] = (long)std::floor(m * g[k] / tot); used += sizes[k]; }
    sizes[K] += m - used;
    std::vector<std::pair<QN, long>> secs;
    for (int k = 0; k <= 2 * K; ++k) if (sizes[k] > 0) secs.push_back({sz(2 * (k - K)), sizes[k]});
    return mkidx(secs, dir, tags);
}

static ITensor with_blocks(IndexSet const& is, Blocks const& blocks, Rng& r) {
    auto T = ITensor(is, QDenseReal(is, blocks));
    fill_normal(T, r);
    return T;
}

static std::string jcase(std::string const& name, ITensor const& A, ITensor const& B) {
    auto C = A * B;
    std::ostringstream o;
    o << "{\"name\":\"" << name << "\",\"A\":" << jtensor(A) << ",\"B\":" << jtensor(B)
      << ",\"C\":" << jtensor(C) << "}";
    return o.str();
}

static void gen_contract(std::string const& dir) {
    Rng r(1234);
    std::vector<std::string> cases;
    // matrix x matrix, mixed arrows
    {
        auto i = mkidx({{sz(-2), 2}, {sz(0), 3}, {sz(2), 1}, {sz(4), 2}}, Out, "i");
        auto j = mkidx({{sz(-2), 3}, {sz(0), 2}, {sz(2), 2}}, Out, "j");
        auto k = mkidx({{sz(0), 4}, {sz(2), 3}, {sz(-2), 1}}, Out, "k");
        auto A = randqn(sz(0), IndexSet(i, dag(j)), r);
        auto B = randqn(sz(0), IndexSet(j, dag(k)), r);
        cases.push_back(jcase("mat", A, B));
    }
    // rank-3 x rank-3, two contracted indices in swapped order, nonzero divergence
    {
        auto a = mkidx({{sz(-1), 2}, {sz(1), 3}}, Out, "a");
        auto b = mkidx({{sz(-2), 2}, {sz(0), 1}, {sz(2), 3}}, Out, "b");
        auto c = mkidx({{sz(-1), 3}, {sz(1), 2}}, In, "c");
        auto d = mkidx({{sz(0), 2}, {sz(2), 2}, {sz(-2), 3}}, Out, "d");
        auto A = randqn(sz(2), IndexSet(a, b, c), r);
        auto B = randqn(sz(1), IndexSet(dag(c), d, dag(b)), r);
        cases.push_back(jcase("perm2", A, B));
    }
    // psi(l,s1,s2,r) * L(l,w,l') : the first step of the H_eff apply
    {
        auto l = gauss_link(24, 3, 1.5, Out, "l");
        auto rr = gauss_link(20, 3, 1.5, Out, "r");
        auto s1 = mkidx({{sz(1), 1}, {sz(-1), 1}}, Out, "s1");
        auto s2 = mkidx({{sz(1), 1}, {sz(-1), 1}}, Out, "s2");
        auto w = mkidx({{sz(0), 3}, {sz(-2), 1}, {sz(2), 1}}, Out, "w");
        auto psi = randqn(sz(0), IndexSet(dag(l), s1, s2, rr), r);
        auto L = randqn(sz(0), IndexSet(l, w, dag(prime(l))), r);
        cases.push_back(jcase("psiL", psi, L));
        cases.push_back(jcase("Lpsi", L, psi));
    }
    // block-deficient operands: only the produced output blocks exist
    {
        auto i = mkidx({{sz(-2), 2}, {sz(0), 3}, {sz(2), 2}}, Out, "i");
        auto j = mkidx({{sz(-2), 2}, {sz(0), 2}, {sz(2), 3}}, Out, "j");
        auto k = mkidx({{sz(-2), 1}, {sz(0), 2}, {sz(2), 2}}, Out, "k");
        auto m = mkidx({{sz(0), 2}, {sz(2), 1}, {sz(-2), 2}}, Out, "m");
        auto A = deficient(IndexSet(i, dag(j), k), sz(0), r, 0.5);
        auto B = deficient(IndexSet(j, m, dag(k)), sz(0), r, 0.5);
        cases.push_back(jcase("deficient", A, B));
    }
    // no pair of blocks matches: the result has no blocks
    {
        auto i = mkidx({{sz(0), 2}, {sz(2), 2}}, Out, "i");
        auto j = mkidx({{sz(0), 3}, {sz(2), 2}}, Out, "j");
        auto k = mkidx({{sz(0), 2}, {sz(2), 3}}, Out, "k");
        Blocks ba; { Block b(2); b[0] = 0; b[1] = 0; ba.push_back(b); }
        Blocks bb; { Block b(2); b[0] = 1; b[1] = 1; bb.push_back(b); }
        auto A = with_blocks(IndexSet(i, dag(j)), ba, r);
        auto B = with_blocks(IndexSet(j, dag(k)), bb, r);
        cases.push_back(jcase("empty", A, B));
    }
    // outer product (no contracted index)
    {
        auto i = mkidx({{sz(-1), 2}, {sz(1), 1}}, Out, "i");
        auto j = mkidx({{sz(-1), 1}, {sz(1), 2}}, Out, "j");
        auto k = mkidx({{sz(0), 2}, {sz(2), 1}}, Out, "k");
        auto A = randqn(sz(0), IndexSet(i, dag(j)), r);
        auto B = randqn(sz(2), IndexSet(k), r);
        cases.push_back(jcase("outer", A, B));
    }
    // U(1)xU(1) (Nf,Sz) electron-like sectors
    {
        auto s = mkidx({{nfsz(0, 0), 1}, {nfsz(1, 1), 1}, {nfsz(1, -1), 1}, {nfsz(2, 0), 1}}, Out, "site");
        auto l = mkidx({{nfsz(0, 0), 2}, {nfsz(1, 1), 3}, {nfsz(1, -1), 3}, {nfsz(2, 0), 2}, {nfsz(2, 2), 1}}, Out, "l");
        auto rl = mkidx({{nfsz(1, 1), 2}, {nfsz(1, -1), 2}, {nfsz(2, 0), 4}, {nfsz(3, 1), 2}, {nfsz(3, -1), 2}}, Out, "r");
        auto A = randqn(QN(), IndexSet(dag(l), s, rl), r);
        auto B = randqn(QN(), IndexSet(dag(rl), s.prime(), mkidx({{nfsz(2, 0), 2}, {nfsz(3, 1), 2}, {nfsz(3, -1), 1}, {nfsz(4, 0), 2}}, Out, "x")), r);
        cases.push_back(jcase("u1u1", A, B));
    }
    // Z2 parity sectors
    {
        auto a = mkidx({{par(0), 3}, {par(1), 2}}, Out, "a");
        auto b = mkidx({{par(0), 2}, {par(1), 3}}, Out, "b");
        auto c = mkidx({{par(1), 2}, {par(0), 2}}, Out, "c");
        auto A = randqn(par(1), IndexSet(a, dag(b)), r);
        auto B = randqn(par(1), IndexSet(b, c), r);
        cases.push_back(jcase("z2", A, B));
    }
    // full contraction to a scalar
    {
        auto a = mkidx({{sz(-1), 2}, {sz(1), 3}}, Out, "a");
        auto b = mkidx({{sz(-1), 3}, {sz(1), 2}}, In, "b");
        auto A = randqn(sz(0), IndexSet(a, b), r);
        cases.push_back(jcase("scalar", dag(A), A));
    }
    // larger H_eff-like step (W contraction: bandwidth-shaped, K <= 3)
    {
        auto l = gauss_link(40, 4, 2.0, Out, "l");
        auto s1 = mkidx({{sz(1), 1}, {sz(-1), 1}}, Out, "s1");
        auto s2 = mkidx({{sz(1), 1}, {sz(-1), 1}}, Out, "s2");
        auto rr = gauss_link(36, 4, 2.0, Out, "r");
        auto w = mkidx({{sz(0), 3}, {sz(-2), 1}, {sz(2), 1}}, Out, "w");
        auto w2 = mkidx({{sz(0), 3}, {sz(-2), 1}, {sz(2), 1}}, Out, "w2");
        auto T1 = randqn(sz(0), IndexSet(s1, s2, rr, w, dag(prime(l))), r);
        auto W = randqn(sz(0), IndexSet(dag(s1), prime(s1), dag(w), w2), r);
        cases.push_back(jcase("T1W", T1, W));
    }
    std::ostringstream o;
    o << "{\"kind\":\"contract\",\"cases\":[";
    for (size_t n = 0; n < cases.size(); ++n) { if (n) o << ",\n"; o << cases[n]; }
    o << "]}";
    write_file(dir + "/contract.json", o.str());
}

// ---------------------------------------------------------------- H_eff + davidson
static MPS neel_mps(SpinHalf const& sites, int N) {
    auto st = InitState(sites);
    for (int i = 1; i <= N; ++i) st.set(i, i % 2 == 1 ? "Up" : "Dn");
    return MPS(st);
}

static void gen_heff(std::string const& dir) {
    std::ostringstream o;
    o << "{\"kind\":\"heff\",\"cases\":[";
    // (1) real environments at bond b of a Heisenberg chain partly optimised by DMRG
    {
        int N = 12, b = 5;
        auto sites = SpinHalf(N);
        auto H = MPO(Heisenberg(sites));
        auto psi = neel_mps(sites, N);
        auto sw = Sweeps(2);
        sw.maxdim() = 8, 16;
        sw.cutoff() = 1e-10;
        sw.niter() = 2;
        dmrg(psi, H, sw, {"Quiet", true, "Silent", true});
        psi.position(b);
        LocalMPO PH(H);
        PH.position(b, psi);
        auto phi = psi(b) * psi(b + 1);
        ITensor phip;
        PH.product(phi, phip);
        auto phi2 = phi;
        auto en = davidson(PH, phi2, {"MaxIter", 2, "DebugLevel", -1});
        auto phi9 = phi;
        auto en9 = davidson(PH, phi9, {"MaxIter", 9, "DebugLevel", -1});
        o << "{\"name\":\"heis12_b5\",\"L\":" << jtensor(PH.L()) << ",\"W1\":" << jtensor(H(b))
          << ",\"W2\":" << jtensor(H(b + 1)) << ",\"R\":" << jtensor(PH.R()) << ",\"phi\":" << jtensor(phi)
          << ",\"Hphi\":" << jtensor(phip) << ",\"davidson_niter2\":{\"energy\":" << num(en)
          << ",\"phi\":" << jtensor(phi2) << "},\"davidson_niter9\":{\"energy\":" << num(en9)
          << ",\"phi\":" << jtensor(phi9) << "}},\n";
    }
    // (2) reference unit test: 4-site Heisenberg, davidson at b=2, MaxIter=9
    {
        int N = 4;
        auto sites = SpinHalf(N);
        auto H = MPO(Heisenberg(sites));
        auto psi = neel_mps(sites, N);
        LocalMPO PH(H);
        psi.position(2);
        PH.position(2, psi);
        auto phi = psi(2) * psi(3);
        auto phi9 = phi;
        auto en9 = davidson(PH, phi9, {"MaxIter", 9, "DebugLevel", -1});
        o << "{\"name\":\"heis4_b2\",\"L\":" << jtensor(PH.L()) << ",\"W1\":" << jtensor(H(2))
          << ",\"W2\":" << jtensor(H(3)) << ",\"R\":" << jtensor(PH.R()) << ",\"phi\":" << jtensor(phi)
          << ",\"davidson_niter9\":{\"energy\":" << num(en9) << ",\"phi\":" << jtensor(phi9) << "}},\n";
    }
    // (3) synthetic N(0,1) environments on Gaussian Sz links (the isolated-apply layout, small m)
    {
        Rng r(777);
        int N = 12, b = 5;
        auto sites = SpinHalf(N);
        auto H = MPO(Heisenberg(sites));
        auto W1 = H(b), W2 = H(b + 1);
        auto s1 = sites(b), s2 = sites(b + 1);
        auto wl = commonIndex(H(b - 1), H(b));
        auto wr = commonIndex(H(b + 1), H(b + 2));
        auto l = gauss_link(48, 3, 1.5, Out, "l");
        auto rr = gauss_link(40, 3, 1.5, Out, "r");
        auto psi = randqn(QN(), IndexSet(dag(l), s1, s2, rr), r);
        auto L = randqn(QN(), IndexSet(l, wl, dag(prime(l))), r);
        auto R = randqn(QN(), IndexSet(dag(rr), dag(wr), prime(rr)), r);
        LocalOp op(W1, W2, L, R);
        ITensor phip;
        op.product(psi, phip);
        o << "{\"name\":\"gauss48\",\"L\":" << jtensor(L) << ",\"W1\":" << jtensor(W1) << ",\"W2\":"
          << jtensor(W2) << ",\"R\":" << jtensor(R) << ",\"phi\":" << jtensor(psi) << ",\"Hphi\":"
          << jtensor(phip) << "}";
    }
    o << "]}";
    write_file(dir + "/heff.json", o.str());
}

// ---------------------------------------------------------------- truncate
static void gen_truncate(std::string const& dir) {
    struct TC { std::vector<double> P; long maxdim, mindim; double cutoff; bool absc, rel, resp; };
    std::vector<TC> tcs = {
        {{1, 0.5, 0.25, 1e-3, 1e-6, 1e-12}, 10, 1, 1e-10, false, true, true},
        {{1, 0.3, 0.3, 0.3, 0.1}, 3, 1, 1e-10, false, true, true},
        {{1, 0.3, 0.3, 0.3, 0.1}, 3, 1, 1e-10, false, true, false},
        {{1, 0.3, 0.3, 0.3, 0.1}, 4, 1, 1e-10, false, true, true},
        {{1, 0.3, 0.3, 0.3, 0.1}, 2, 1, 1e-10, false, true, true},
        {{0, 0, 0}, 5, 1, 1e-10, false, true, true},
        {{0.7}, 5, 1, 1e-10, false, true, true},
        {{1, 0.5, -1e-17, -1e-16}, 10, 1, 1e-10, false, true, true},
        {{1, 0.2, 0.1, 0.05, 0.01}, 10, 3, 0.5, false, true, true},
        {{1, 0.2, 0.1, 0.05, 0.01}, 10, 1, 0.02, true, true, true},
        {{2, 0.4, 0.2, 0.1, 0.02}, 10, 1, 0.02, false, false, true},
        {{1, 1e-11, 1e-11, 1e-11, 5e-12}, 10, 1, 1e-10, false, true, true},
        {{1, 0.25, 0.25, 0.2502, 0.2499, 0.1, 0.1, 1e-9}, 4, 1, 1e-10, false, true, true},
        {{1, 0.25, 0.25, 0.2502, 0.2499, 0.1, 0.1, 1e-9}, 6, 1, 1e-10, false, true, true},
        {{1, 0.25, 0.25, 0.2502, 0.2499, 0.1, 0.1, 1e-9}, 7, 1, 1e-10, false, true, true},
        {{1, 0.25, 0.25, 0.2502, 0.2499, 0.1, 0.1, 1e-9}, 8, 1, 1e-8, false, true, true},
    };
    Rng r(99);
    for (int n = 0; n < 24; ++n) {
        TC t;
        int len = 5 + (int)(r.uni() * 40);
        for (int k = 0; k < len; ++k) t.P.push_back(std::pow(10.0, -14.0 * r.uni()));
        if (n % 3 == 0) for (int k = 1; k + 1 < len; k += 3) t.P[k + 1] = t.P[k];
        std::sort(t.P.begin(), t.P.end(), std::greater<double>());
        t.maxdim = 2 + (long)(r.uni() * len);
        t.mindim = 1 + (n % 4);
        t.cutoff = std::pow(10.0, -12.0 + 10.0 * r.uni());
        t.absc = (n % 7 == 3);
        t.rel = (n % 5 != 4);
        t.resp = (n % 2 == 0);
        tcs.push_back(t);
    }
    std::ostringstream o;
    o << "{\"kind\":\"truncate\",\"cases\":[";
    for (size_t n = 0; n < tcs.size(); ++n) {
        auto& t = tcs[n];
        auto P = Vector(t.P.size());
        for (size_t k = 0; k < t.P.size(); ++k) P(k) = t.P[k];
        auto [te, lo, up, nd] = truncate(P, t.maxdim, t.mindim, t.cutoff, t.absc, t.rel, {"RespectDegenerate", t.resp});
        if (n) o << ",\n";
        o << "{\"P\":[";
        for (size_t k = 0; k < t.P.size(); ++k) { if (k) o << ","; o << num(t.P[k]); }
        o << "],\"maxdim\":" << t.maxdim << ",\"mindim\":" << t.mindim << ",\"cutoff\":" << num(t.cutoff)
          << ",\"absoluteCutoff\":" << (t.absc ? "true" : "false") << ",\"doRelCutoff\":" << (t.rel ? "true" : "false")
          << ",\"respectDegenerate\":" << (t.resp ? "true" : "false") << ",\"truncerr\":" << num(te)
          << ",\"docut_lower\":" << num(lo) << ",\"docut_upper\":" << num(up) << ",\"ndegen\":" << nd
          << ",\"Pout\":[";
        for (long k = 0; k < (long)P.size(); ++k) { if (k) o << ","; o << num(P(k)); }
        o << "]}";
    }
    o << "]}";
    write_file(dir + "/truncate.json", o.str());
}

// ---------------------------------------------------------------- bond split
static std::string jspec(Spectrum const& s) {
    std::ostringstream o;
    o << "{\"truncerr\":" << num(s.truncerr()) << ",\"eigs\":[";
    auto const& e = s.eigsKept();
    for (long k = 0; k < (long)e.size(); ++k) { if (k) o << ","; o << num(e(k)); }
    o << "]}";
    return o.str();
}

static void gen_bondsplit(std::string const& dir) {
    Rng r(4242);
    std::ostringstream o;
    o << "{\"kind\":\"bondsplit\",\"cases\":[";
    struct BC { std::string name; int ml, mr; double cutoff; long maxdim, mindim; bool fromleft, usesvd; };
    std::vector<BC> bcs = {
        {"dm_left_cut", 24, 20, 1e-10, 100, 1, true, false},
        {"dm_right_cut", 24, 20, 1e-10, 100, 1, false, false},
        {"dm_left_maxdim", 24, 20, 1e-10, 9, 1, true, false},
        {"dm_left_bigcut", 30, 30, 1e-3, 200, 2, true, false},
        {"svd_left", 24, 20, 1e-14, 100, 1, true, true},
        {"svd_right_maxdim", 24, 20, 1e-14, 11, 1, false, true},
    };
    auto s1 = mkidx({{sz(1), 1}, {sz(-1), 1}}, Out, "s1");
    auto s2 = mkidx({{sz(1), 1}, {sz(-1), 1}}, Out, "s2");
    for (size_t n = 0; n < bcs.size(); ++n) {
        auto& c = bcs[n];
        auto l = gauss_link(c.ml, 3, 1.5, Out, "l");
        auto rr = gauss_link(c.mr, 3, 1.5, Out, "r");
        auto mid = gauss_link(8, 2, 1.0, Out, "mid");
        auto AA = randqn(QN(), IndexSet(dag(l), s1, s2, rr), r);
        auto A = ITensor(QN(), IndexSet(dag(l), s1, mid));
        auto B = ITensor(QN(), IndexSet(dag(mid), s2, rr));
        Args args = {"Cutoff", c.cutoff, "MaxDim", (int)c.maxdim, "MinDim", (int)c.mindim,
                     "RespectDegenerate", true};
        Spectrum spec;
        ITensor Aout = A, Bout = B;
        if (c.usesvd) {
            ITensor D;
            spec = svd(AA, Aout, D, Bout, args);
            if (c.fromleft) Bout *= D; else Aout *= D;
        } else {
            spec = denmatDecomp(AA, Aout, Bout, c.fromleft ? Fromleft : Fromright, LocalMPO(), args);
        }
        auto link = commonIndex(Aout, Bout);
        if (n) o << ",\n";
        o << "{\"name\":\"" << c.name << "\",\"cutoff\":" << num(c.cutoff) << ",\"maxdim\":" << c.maxdim
          << ",\"mindim\":" << c.mindim << ",\"fromleft\":" << (c.fromleft ? "true" : "false")
          << ",\"usesvd\":" << (c.usesvd ? "true" : "false") << ",\"AA\":" << jtensor(AA)
          << ",\"A\":" << jtensor(A) << ",\"B\":" << jtensor(B) << ",\"spec\":" << jspec(spec)
          << ",\"link\":" << jindex(link) << ",\"Aout\":" << jtensor(Aout) << ",\"Bout\":" << jtensor(Bout)
          << ",\"AB\":" << jtensor(Aout * Bout) << "}";
    }
    o << "]}";
    write_file(dir + "/bondsplit.json", o.str());
}

// ---------------------------------------------------------------- DMRG
struct Recorder : public DMRGObserver {
    std::ostringstream rec;
    bool first = true;
    explicit Recorder(MPS const& psi) : DMRGObserver(psi, {"EnergyErrgoal", -1.0}) {}
    void measure(Args const& args) override {
        int b = args.getInt("AtBond"), ha = args.getInt("HalfSweep"), sw = args.getInt("Sweep");
        if (!first) rec << ",";
        first = false;
        rec << "[" << sw << "," << ha << "," << b << "," << num(args.getReal("Energy")) << ","
            << num(args.getReal("Truncerr")) << "," << spectrum().numEigsKept() << "]";
    }
};

template <typename SitesT>
static std::string run_dmrg(std::string const& name, SitesT const& sites, MPO const& H, MPS const& psi0,
                            Sweeps const& sw, std::string const& model) {
    Recorder obs(psi0);
    auto [E, psi] = dmrg(H, psi0, sw, obs, {"Quiet", true, "Silent", true});
    std::ostringstream o;
    o << "{\"name\":\"" << name << "\",\"model\":" << model << ",\"N\":" << length(psi) << ",\"sweeps\":[";
    for (int s = 1; s <= sw.nsweep(); ++s) {
        if (s > 1) o << ",";
        o << "{\"maxdim\":" << sw.maxdim(s) << ",\"mindim\":" << sw.mindim(s) << ",\"cutoff\":" << num(sw.cutoff(s))
          << ",\"niter\":" << sw.niter(s) << ",\"noise\":" << num(sw.noise(s)) << "}";
    }
    o << "],\"energy\":" << num(E) << ",\"bonds\":[" << obs.rec.str() << "],\"links\":[";
    for (int b = 1; b < length(psi); ++b) { if (b > 1) o << ","; o << jindex(linkIndex(psi, b)); }
    o << "],\"sites\":[";
    for (int j = 1; j <= length(psi); ++j) { if (j > 1) o << ","; o << jindex(sites(j)); }
    o << "]}";
    std::printf("  %s: E=%.15f maxlink=%ld\n", name.c_str(), E, maxLinkDim(psi));
    return o.str();
}

// Excited-state DMRG (itensor/mps/dmrg.h:245-266, LocalMPO_MPS of
// itensor/mps/localmpo_mps.h): the ground state from `sw0`, then the state
// that minimises H + weight |psi0><psi0| from psi_start on `sw`; records the
// second run like run_dmrg, plus the ground run's energy and the overlap.
template <typename SitesT>
static std::string run_dmrg_excited(std::string const& name, SitesT const& sites, MPO const& H, MPS const& psi_start,
                                    Sweeps const& sw0, Sweeps const& sw, double weight, std::string const& model) {
    auto [E0, psi0] = dmrg(H, psi_start, sw0, {"Quiet", true, "Silent", true});
    Recorder obs(psi_start);
    auto [E, psi] = dmrg(H, std::vector<MPS>{psi0}, psi_start, sw, obs,
                         {"Quiet", true, "Silent", true, "Weight", weight});
    auto sweeps_json = [](Sweeps const& w) {
        std::ostringstream o;
        o << "[";
        for (int s = 1; s <= w.nsweep(); ++s) {
            if (s > 1) o << ",";
            o << "{\"maxdim\":" << w.maxdim(s) << ",\"mindim\":" << w.mindim(s) << ",\"cutoff\":" << num(w.cutoff(s))
              << ",\"niter\":" << w.niter(s) << ",\"noise\":" << num(w.noise(s)) << "}";
        }
        o << "]";
        return o.str();
    };
    std::ostringstream o;
    o << "{\"name\":\"" << name << "\",\"model\":" << model << ",\"N\":" << length(psi)
      << ",\"ground_sweeps\":" << sweeps_json(sw0) << ",\"ground_energy\":" << num(E0) << ",\"weight\":" << num(weight)
      << ",\"sweeps\":" << sweeps_json(sw) << ",\"energy\":" << num(E)
      << ",\"overlap_with_ground\":" << num(inner(psi0, psi)) << ",\"bonds\":[" << obs.rec.str() << "],\"links\":[";
    for (int b = 1; b < length(psi); ++b) { if (b > 1) o << ","; o << jindex(linkIndex(psi, b)); }
    o << "],\"sites\":[";
    for (int j = 1; j <= length(psi); ++j) { if (j > 1) o << ","; o << jindex(sites(j)); }
    o << "]}";
    std::printf("  %s: E0=%.15f E1=%.15f <0|1>=%.3e\n", name.c_str(), E0, E, inner(psi0, psi));
    return o.str();
}

// dmrg with a sum of MPOs (itensor/mps/dmrg.h:209-230, LocalMPOSet of
// itensor/mps/localmposet.h), recorded like run_dmrg.
template <typename SitesT>
static std::string run_dmrg_set(std::string const& name, SitesT const& sites, std::vector<MPO> const& Hs,
                                MPS const& psi0, Sweeps const& sw, std::string const& model) {
    Recorder obs(psi0);
    auto [E, psi] = dmrg(Hs, psi0, sw, obs, {"Quiet", true, "Silent", true});
    std::ostringstream o;
    o << "{\"name\":\"" << name << "\",\"model\":" << model << ",\"N\":" << length(psi) << ",\"sweeps\":[";
    for (int s = 1; s <= sw.nsweep(); ++s) {
        if (s > 1) o << ",";
        o << "{\"maxdim\":" << sw.maxdim(s) << ",\"mindim\":" << sw.mindim(s) << ",\"cutoff\":" << num(sw.cutoff(s))
          << ",\"niter\":" << sw.niter(s) << ",\"noise\":" << num(sw.noise(s)) << "}";
    }
    o << "],\"energy\":" << num(E) << ",\"bonds\":[" << obs.rec.str() << "],\"links\":[";
    for (int b = 1; b < length(psi); ++b) { if (b > 1) o << ","; o << jindex(linkIndex(psi, b)); }
    o << "]}";
    std::printf("  %s: E=%.15f maxlink=%ld\n", name.c_str(), E, maxLinkDim(psi));
    return o.str();
}

static Sweeps mksweeps(std::vector<int> maxdims, double cutoff, int niter = 2) {
    auto sw = Sweeps((int)maxdims.size());
    for (int s = 1; s <= (int)maxdims.size(); ++s) {
        sw.setmaxdim(s, maxdims[s - 1]);
        sw.setcutoff(s, cutoff);
        sw.setniter(s, niter);
        sw.setnoise(s, 0.0);
        sw.setmindim(s, 1);
    }
    return sw;
}

static void gen_dmrg(std::string const& dir) {
    std::vector<std::string> cs;
    {   // Heisenberg N=20, Sz QN, Neel, 5 sweeps maxdim 10,20,100,100,200, cutoff 1e-10, niter 2
        int N = 20;
        auto sites = SpinHalf(N);
        MPO H = Heisenberg(sites);
        cs.push_back(run_dmrg("heis20", sites, H, neel_mps(sites, N), mksweeps({10, 20, 100, 100, 200}, 1e-10),
                              "{\"type\":\"heisenberg\",\"J\":1.0,\"Jz\":1.0}"));
        // the same with the noise schedule of sample/dmrg.cc (1e-7, 1e-8, then 0)
        auto swn = mksweeps({10, 20, 100, 100, 200}, 1e-10);
        swn.setnoise(1, 1e-7);
        swn.setnoise(2, 1e-8);
        cs.push_back(run_dmrg("heis20_noise", sites, H, neel_mps(sites, N), swn,
                              "{\"type\":\"heisenberg\",\"J\":1.0,\"Jz\":1.0}"));
    }
    {   // first excited state of the Heisenberg chain N=12 (Sz = 0 triplet member), weight 20
        int N = 12;
        auto sites = SpinHalf(N);
        MPO H = Heisenberg(sites);
        cs.push_back(run_dmrg_excited("heis12_excited", sites, H, neel_mps(sites, N), mksweeps({10, 20, 40, 40, 40}, 1e-10),
                                      mksweeps({10, 20, 40, 40, 40, 40}, 1e-10), 20.0,
                                      "{\"type\":\"heisenberg\",\"J\":1.0,\"Jz\":1.0}"));
    }
    {   // XXZ N=16, Delta=0.5
        int N = 16; double D = 0.5;
        auto sites = SpinHalf(N);
        auto ampo = AutoMPO(sites);
        for (int j = 1; j < N; ++j) {
            ampo += 0.5, "S+", j, "S-", j + 1;
            ampo += 0.5, "S-", j, "S+", j + 1;
            ampo += D, "Sz", j, "Sz", j + 1;
        }
        auto H = toMPO(ampo);
        cs.push_back(run_dmrg("xxz16", sites, H, neel_mps(sites, N), mksweeps({10, 20, 40, 40}, 1e-10),
                              "{\"type\":\"xxz\",\"J\":1.0,\"Jz\":0.5}"));
    }
    {   // J1-J2 N=16, J2=0.3
        int N = 16; double J2 = 0.3;
        auto sites = SpinHalf(N);
        auto ampo = AutoMPO(sites);
        for (int j = 1; j < N; ++j) {
            ampo += 0.5, "S+", j, "S-", j + 1;
            ampo += 0.5, "S-", j, "S+", j + 1;
            ampo += "Sz", j, "Sz", j + 1;
        }
        for (int j = 1; j < N - 1; ++j) {
            ampo += 0.5 * J2, "S+", j, "S-", j + 2;
            ampo += 0.5 * J2, "S-", j, "S+", j + 2;
            ampo += J2, "Sz", j, "Sz", j + 2;
        }
        auto H = toMPO(ampo);
        cs.push_back(run_dmrg("j1j2_16", sites, H, neel_mps(sites, N), mksweeps({10, 20, 40, 60}, 1e-10),
                              "{\"type\":\"j1j2\",\"J2\":0.3}"));
        // the same Hamiltonian as a sum of two MPOs: nearest and next-nearest neighbours
        auto a1 = AutoMPO(sites), a2 = AutoMPO(sites);
        for (int j = 1; j < N; ++j) {
            a1 += 0.5, "S+", j, "S-", j + 1;
            a1 += 0.5, "S-", j, "S+", j + 1;
            a1 += "Sz", j, "Sz", j + 1;
        }
        for (int j = 1; j < N - 1; ++j) {
            a2 += 0.5 * J2, "S+", j, "S-", j + 2;
            a2 += 0.5 * J2, "S-", j, "S+", j + 2;
            a2 += J2, "Sz", j, "Sz", j + 2;
        }
        cs.push_back(run_dmrg_set("j1j2_16_set", sites, std::vector<MPO>{toMPO(a1), toMPO(a2)}, neel_mps(sites, N),
                                  mksweeps({10, 20, 40, 60}, 1e-10), "{\"type\":\"j1j2\",\"J2\":0.3}"));
    }
    {   // transverse-field Ising N=16 with parity QN: H = -sum Sx Sx - h sum Sz, all Up
        int N = 16; double h = 0.5;
        auto sites = SpinHalf(N, {"ConserveSz", false, "ConserveParity", true});
        auto ampo = AutoMPO(sites);
        for (int j = 1; j < N; ++j) { ampo += -1.0, "Sx", j, "Sx", j + 1; ampo += -h, "Sz", j; }
        ampo += -h, "Sz", N;
        auto H = toMPO(ampo);
        auto st = InitState(sites, "Up");
        cs.push_back(run_dmrg("tfi16", sites, H, MPS(st), mksweeps({10, 20, 30, 30}, 1e-10),
                              "{\"type\":\"tfi\",\"h\":0.5}"));
    }
    {   // Hubbard chain N=8, t=1, U=4, half filling, U(1)xU(1)
        int N = 8; double t = 1.0, U = 4.0;
        auto sites = Electron(N);
        auto ampo = AutoMPO(sites);
        for (int j = 1; j < N; ++j) {
            ampo += -t, "Cdagup", j, "Cup", j + 1;
            ampo += -t, "Cdagup", j + 1, "Cup", j;
            ampo += -t, "Cdagdn", j, "Cdn", j + 1;
            ampo += -t, "Cdagdn", j + 1, "Cdn", j;
        }
        for (int j = 1; j <= N; ++j) ampo += U, "Nupdn", j;
        auto H = toMPO(ampo);
        auto st = InitState(sites);
        for (int j = 1; j <= N; ++j) st.set(j, j % 2 == 1 ? "Up" : "Dn");
        cs.push_back(run_dmrg("hubbard8", sites, H, MPS(st), mksweeps({20, 40, 80, 80}, 1e-10),
                              "{\"type\":\"hubbard\",\"t\":1.0,\"U\":4.0,\"Lx\":8,\"Ly\":1}"));
    }
    {   // Hubbard 4x2 ladder snake (squareLattice Nx=4, Ny=2), t=1, U=4, half filling
        int Nx = 4, Ny = 2, N = Nx * Ny; double t = 1.0, U = 4.0;
        auto sites = Electron(N);
        auto ampo = AutoMPO(sites);
        auto lattice = squareLattice(Nx, Ny, {"YPeriodic", false});
        for (auto j : lattice) {
            ampo += -t, "Cdagup", j.s1, "Cup", j.s2;
            ampo += -t, "Cdagup", j.s2, "Cup", j.s1;
            ampo += -t, "Cdagdn", j.s1, "Cdn", j.s2;
            ampo += -t, "Cdagdn", j.s2, "Cdn", j.s1;
        }
        for (int j = 1; j <= N; ++j) ampo += U, "Nupdn", j;
        auto H = toMPO(ampo);
        auto st = InitState(sites);
        for (int j = 1; j <= N; ++j) st.set(j, j % 2 == 1 ? "Up" : "Dn");
        cs.push_back(run_dmrg("hubbard4x2", sites, H, MPS(st), mksweeps({20, 40, 80, 80}, 1e-10),
                              "{\"type\":\"hubbard\",\"t\":1.0,\"U\":4.0,\"Lx\":4,\"Ly\":2,\"yperiodic\":false}"));
    }
    std::ostringstream o;
    o << "{\"kind\":\"dmrg\",\"cases\":[";
    for (size_t n = 0; n < cs.size(); ++n) { if (n) o << ",\n"; o << cs[n]; }
    o << "]}";
    write_file(dir + "/dmrg.json", o.str());
}

// ---------------------------------------------------------------- benchmark configurations
// The isolated H_eff apply in the benchmark's layout (Gaussian Sz link over
// 2K+1 = 31 sectors, sigma = 6, N(0,1) blocks, Heisenberg bulk MPO tensors),
// at bond dimension m (the benchmark runs m = 1024; the fixture is smaller).
static void gen_heff_config(std::string const& dir, long m) {
    Rng r(20241204);
    int N = 12, b = 5;
    auto sites = SpinHalf(N);
    auto H = MPO(Heisenberg(sites));
    auto W1 = H(b), W2 = H(b + 1);
    auto s1 = sites(b), s2 = sites(b + 1);
    auto wl = commonIndex(H(b - 1), H(b));
    auto wr = commonIndex(H(b + 1), H(b + 2));
    auto l = gauss_link(m, 15, 6.0, Out, "l");
    auto rr = gauss_link(m, 15, 6.0, Out, "r");
    auto psi = randqn(QN(), IndexSet(dag(l), s1, s2, rr), r);
    auto L = randqn(QN(), IndexSet(l, wl, dag(prime(l))), r);
    auto R = randqn(QN(), IndexSet(dag(rr), dag(wr), prime(rr)), r);
    LocalOp op(W1, W2, L, R);
    ITensor phip;
    op.product(psi, phip);
    std::ostringstream o;
    o << "{\"kind\":\"heff\",\"cases\":[{\"name\":\"gauss31_m" << m << "\",\"m\":" << m << ",\"L\":" << jtensor(L)
      << ",\"W1\":" << jtensor(W1) << ",\"W2\":" << jtensor(W2) << ",\"R\":" << jtensor(R) << ",\"phi\":"
      << jtensor(psi) << ",\"Hphi\":" << jtensor(phip) << "}]}";
    write_file(dir + "/heff_config.json", o.str());
}

// Hubbard model on the 4 x 16 cylinder (squareLattice Nx=16, Ny=4, periodic in
// y, as sample/hubbard_2d.cc:17-46), t=1, U=4, half filling, Neel start; the
// sweep table's maxdims up to `maxdim`, cutoff 1e-9, niter 2, noise 0 (so that
// every bond step is reproducible; the sample's noise splits multiplets).
static void gen_cylinder(std::string const& dir, int maxdim) {
    int Nx = 16, Ny = 4, N = Nx * Ny;
    double t = 1.0, U = 4.0;
    auto sites = Electron(N);
    auto ampo = AutoMPO(sites);
    auto lattice = squareLattice(Nx, Ny, {"YPeriodic", true});
    for (auto j : lattice) {
        ampo += -t, "Cdagup", j.s1, "Cup", j.s2;
        ampo += -t, "Cdagup", j.s2, "Cup", j.s1;
        ampo += -t, "Cdagdn", j.s1, "Cdn", j.s2;
        ampo += -t, "Cdagdn", j.s2, "Cdn", j.s1;
    }
    for (int j = 1; j <= N; ++j) ampo += U, "Nupdn", j;
    auto H = toMPO(ampo);
    auto st = InitState(sites);
    for (int j = 1; j <= N; ++j) st.set(j, j % 2 == 1 ? "Up" : "Dn");
    std::vector<int> mds;
    for (int d : {20, 60, 100, 100, 200, 400, 800, 2000, 3000}) if (d < maxdim) mds.push_back(d);
    mds.push_back(maxdim);
    auto sw = mksweeps(mds, 1e-9);
    auto t0 = std::chrono::steady_clock::now();
    auto rec = run_dmrg("hubbard_cylinder_4x16", sites, H, MPS(st), sw,
                        "{\"type\":\"hubbard\",\"t\":1.0,\"U\":4.0,\"Lx\":16,\"Ly\":4,\"yperiodic\":true}");
    double secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    std::printf("  cylinder up to maxdim %d: %.1f s\n", maxdim, secs);
    write_file(dir + "/cylinder.json", "{\"kind\":\"dmrg\",\"seconds\":" + num(secs) + ",\"cases\":[" + rec + "]}");
}

// dmrg() on the caller's own MPO and initial MPS: the reference's MPO tensors
// (sample/Heisenberg.h for the chain, toMPO for the Hubbard ladder) and
// MPS(InitState) tensors, with the run they give.
template <typename SitesT>
static std::string mpo_case(std::string const& name, SitesT const& sites, MPO const& H, MPS const& psi0,
                            Sweeps const& sw, std::string const& model) {
    int N = length(psi0);
    std::ostringstream o;
    o << "{\"W\":[";
    for (int j = 1; j <= N; ++j) { if (j > 1) o << ","; o << jtensor(H(j)); }
    o << "],\"psi0\":[";
    for (int j = 1; j <= N; ++j) { if (j > 1) o << ","; o << jtensor(psi0(j)); }
    o << "],\"run\":" << run_dmrg(name, sites, H, psi0, sw, model) << "}";
    return o.str();
}

static void gen_mpo_io(std::string const& dir) {
    std::vector<std::string> cs;
    {
        int N = 20;
        auto sites = SpinHalf(N);
        MPO H = Heisenberg(sites);
        cs.push_back(mpo_case("heis20", sites, H, neel_mps(sites, N), mksweeps({10, 20, 100, 100, 200}, 1e-10),
                              "{\"type\":\"heisenberg\",\"J\":1.0,\"Jz\":1.0}"));
    }
    {
        int Nx = 4, Ny = 2, N = Nx * Ny;
        auto sites = Electron(N);
        auto ampo = AutoMPO(sites);
        for (auto j : squareLattice(Nx, Ny, {"YPeriodic", false})) {
            ampo += -1.0, "Cdagup", j.s1, "Cup", j.s2;
            ampo += -1.0, "Cdagup", j.s2, "Cup", j.s1;
            ampo += -1.0, "Cdagdn", j.s1, "Cdn", j.s2;
            ampo += -1.0, "Cdagdn", j.s2, "Cdn", j.s1;
        }
        for (int j = 1; j <= N; ++j) ampo += 4.0, "Nupdn", j;
        auto H = toMPO(ampo);
        auto st = InitState(sites);
        for (int j = 1; j <= N; ++j) st.set(j, j % 2 == 1 ? "Up" : "Dn");
        cs.push_back(mpo_case("hubbard4x2", sites, H, MPS(st), mksweeps({20, 40, 80, 80}, 1e-10),
                              "{\"type\":\"hubbard\",\"t\":1.0,\"U\":4.0,\"Lx\":4,\"Ly\":2,\"yperiodic\":false}"));
    }
    std::ostringstream o;
    o << "{\"kind\":\"mpo_io\",\"cases\":[";
    for (size_t n = 0; n < cs.size(); ++n) { if (n) o << ",\n"; o << cs[n]; }
    o << "]}";
    write_file(dir + "/mpo_io.json", o.str());
}

// Checkpoints in the reference's binary layout (MPS::write, itensor/mps/mps.cc:365-378,
// ITensor::write itensor/itensor.cc:769-784, QDense write itensor/itdata/qdense.h:236-241,
// writeToFile itensor/util/readwrite.h:363-370): the MPO and the MPS after the
// first sweeps, the record of the run continued from that MPS, and the final MPS.
template <typename SitesT>
static std::string checkpoint_case(std::string const& dir, std::string const& name, SitesT const& sites, MPO const& H,
                                   MPS const& psi0, Sweeps const& sw_first, Sweeps const& sw_rest,
                                   std::string const& model) {
    auto [E1, psi1] = dmrg(H, psi0, sw_first, {"Quiet", true, "Silent", true});
    writeToFile(dir + "/" + name + ".mpo", H);
    writeToFile(dir + "/" + name + "_start.mps", psi1);
    Recorder obs(psi1);
    auto [E2, psi2] = dmrg(H, psi1, sw_rest, obs, {"Quiet", true, "Silent", true});
    writeToFile(dir + "/" + name + "_final.mps", psi2);
    std::ostringstream o;
    o << "{\"name\":\"" << name << "\",\"model\":" << model << ",\"N\":" << length(psi2) << ",\"mpo\":\"" << name
      << ".mpo\",\"start\":\"" << name << "_start.mps\",\"final\":\"" << name << "_final.mps\",\"start_energy\":"
      << num(E1) << ",\"start_lims\":[" << psi1.leftLim() << "," << psi1.rightLim() << "],\"final_lims\":["
      << psi2.leftLim() << "," << psi2.rightLim() << "],\"sweeps\":[";
    for (int s = 1; s <= sw_rest.nsweep(); ++s) {
        if (s > 1) o << ",";
        o << "{\"maxdim\":" << sw_rest.maxdim(s) << ",\"mindim\":" << sw_rest.mindim(s) << ",\"cutoff\":"
          << num(sw_rest.cutoff(s)) << ",\"niter\":" << sw_rest.niter(s) << ",\"noise\":" << num(sw_rest.noise(s))
          << "}";
    }
    o << "],\"energy\":" << num(E2) << ",\"bonds\":[" << obs.rec.str() << "],\"start_links\":[";
    for (int b = 1; b < length(psi1); ++b) { if (b > 1) o << ","; o << jindex(linkIndex(psi1, b)); }
    o << "],\"links\":[";
    for (int b = 1; b < length(psi2); ++b) { if (b > 1) o << ","; o << jindex(linkIndex(psi2, b)); }
    o << "],\"sites\":[";
    for (int j = 1; j <= length(psi2); ++j) { if (j > 1) o << ","; o << jindex(sites(j)); }
    o << "]}";
    std::printf("  %s: E(start)=%.15f E(final)=%.15f\n", name.c_str(), E1, E2);
    return o.str();
}

static void gen_checkpoint(std::string const& dir) {
    std::vector<std::string> cs;
    {
        int N = 12;
        auto sites = SpinHalf(N);
        MPO H = Heisenberg(sites);
        cs.push_back(checkpoint_case(dir, "heis12", sites, H, neel_mps(sites, N), mksweeps({8, 16}, 1e-10),
                                     mksweeps({32, 32}, 1e-10), "{\"type\":\"heisenberg\",\"J\":1.0,\"Jz\":1.0}"));
    }
    {
        int Nx = 4, Ny = 2, N = Nx * Ny;
        auto sites = Electron(N);
        auto ampo = AutoMPO(sites);
        for (auto j : squareLattice(Nx, Ny, {"YPeriodic", false})) {
            ampo += -1.0, "Cdagup", j.s1, "Cup", j.s2;
            ampo += -1.0, "Cdagup", j.s2, "Cup", j.s1;
            ampo += -1.0, "Cdagdn", j.s1, "Cdn", j.s2;
            ampo += -1.0, "Cdagdn", j.s2, "Cdn", j.s1;
        }
        for (int j = 1; j <= N; ++j) ampo += 4.0, "Nupdn", j;
        auto H = toMPO(ampo);
        auto st = InitState(sites);
        for (int j = 1; j <= N; ++j) st.set(j, j % 2 == 1 ? "Up" : "Dn");
        cs.push_back(checkpoint_case(dir, "hubbard4x2", sites, H, MPS(st), mksweeps({10, 20}, 1e-10),
                                     mksweeps({40, 40}, 1e-10),
                                     "{\"type\":\"hubbard\",\"t\":1.0,\"U\":4.0,\"Lx\":4,\"Ly\":2,\"yperiodic\":false}"));
    }
    std::ostringstream o;
    o << "{\"kind\":\"checkpoint\",\"cases\":[";
    for (size_t n = 0; n < cs.size(); ++n) { if (n) o << ",\n"; o << cs[n]; }
    o << "]}";
    write_file(dir + "/checkpoint.json", o.str());
}

// Reads an MPS (or MPO) file with the reference's readFromFile and writes it
// back with writeToFile: a file the reference can read gives the same bytes.
static int rewrite_mps(std::string const& in, std::string const& out) {
    MPS psi;
    readFromFile(in, psi);
    writeToFile(out, psi);
    return 0;
}

int main(int argc, char** argv) {
    std::string dir = argc > 1 ? argv[1] : "tests/golden";
    std::string what = argc > 2 ? argv[2] : "all";
    if (dir == "--rewrite" && argc > 3) return rewrite_mps(argv[2], argv[3]);
    if (what == "cylinder") { gen_cylinder(dir, argc > 3 ? std::atoi(argv[3]) : 200); return 0; }
    if (what == "all" || what == "configs") gen_heff_config(dir, 256);
    if (what == "all" || what == "mpo_io") gen_mpo_io(dir);
    if (what == "all" || what == "checkpoint") gen_checkpoint(dir);
    if (what == "all" || what == "contract") gen_contract(dir);
    if (what == "all" || what == "heff") gen_heff(dir);
    if (what == "all" || what == "truncate") gen_truncate(dir);
    if (what == "all" || what == "bondsplit") gen_bondsplit(dir);
    if (what == "all" || what == "dmrg") gen_dmrg(dir);
    return 0;
}
