// Site types, model Hamiltonians, MPO construction and product-state MPS.
// Host-side setup executed once per solve (the reference builds these with
// SiteSet / AutoMPO, itensor/mps/sites/spinhalf.h:39-56,
// itensor/mps/sites/electron.h:41-60, sample/Heisenberg.h:55-116).
//
// The MPO is an upper-triangular finite-state machine: link state 0 =
// "done", 1 = "not started", then one channel per (left operator, distance).
// A term c A_i B_j (i<j) leaves "not started" with A at site i, travels through
// channel (A, k) carrying the identity (or the fermion string F), and ends
// with c B at site j. Any exact MPO of H yields the same effective
// Hamiltonian on the two-site space, so sweeps agree with the reference.
#include "algo.h"
#include <algorithm>
#include <cmath>

namespace itg {

static QN qn1(int slot, int v, int mod) {
    QN q;
    q.v[slot] = QN::reduce(v, mod);
    q.mod[slot] = mod;
    return q;
}

SiteType spin_half(int conserve) {
    SiteType st;
    st.name = "S=1/2";
    if (conserve == 1) st.qn = {qn1(0, 1, 1), qn1(0, -1, 1)};
    else if (conserve == 2) st.qn = {qn1(0, 1, 2), qn1(0, 0, 2)};
    else st.qn = {QN(), QN()};
    // column-major 2x2: element (i,j) at i + 2j; basis Up, Dn
    st.ops["Id"] = {1, 0, 0, 1};
    st.ops["Sz"] = {0.5, 0, 0, -0.5};
    st.ops["S+"] = {0, 0, 1, 0};   // |Up><Dn|
    st.ops["S-"] = {0, 1, 0, 0};   // |Dn><Up|
    st.ops["Sx"] = {0, 0.5, 0.5, 0};
    st.labels = {"Up", "Dn"};
    return st;
}

static std::vector<double> matmul(std::vector<double> const& a, std::vector<double> const& b, int d) {
    std::vector<double> c((size_t)d * d, 0.0);
    for (int i = 0; i < d; ++i)
        for (int j = 0; j < d; ++j) {
            double s = 0;
            for (int k = 0; k < d; ++k) s += a[i + d * k] * b[k + d * j];
            c[i + d * j] = s;
        }
    return c;
}
static std::vector<double> transpose(std::vector<double> const& a, int d) {
    std::vector<double> t((size_t)d * d);
    for (int i = 0; i < d; ++i) for (int j = 0; j < d; ++j) t[j + d * i] = a[i + d * j];
    return t;
}

SiteType electron() {
    SiteType st;
    st.name = "Electron";
    // slot 0: Nf (fermionic U(1)), slot 1: Sz; basis Emp, Up, Dn, UpDn with |UpDn> = c+_up c+_dn |0>
    auto q = [](int nf, int sz) { QN a = qn1(0, nf, -1); a.v[1] = sz; a.mod[1] = 1; return a; };
    st.qn = {q(0, 0), q(1, 1), q(1, -1), q(2, 0)};
    const int d = 4;
    std::vector<double> adu(16, 0), add(16, 0), F(16, 0), I(16, 0);
    adu[1 + d * 0] = 1; adu[3 + d * 2] = 1;   // a+_up
    add[2 + d * 0] = 1; add[3 + d * 1] = -1;  // a+_dn passes the up mode
    F[0] = 1; F[1 + d] = -1; F[2 + 2 * d] = -1; F[3 + 3 * d] = 1;
    for (int i = 0; i < d; ++i) I[i + d * i] = 1;
    auto au = transpose(adu, d), ad = transpose(add, d);
    auto nu = matmul(adu, au, d), nd = matmul(add, ad, d);
    st.ops["Id"] = I;
    st.ops["F"] = F;
    st.ops["Adagup"] = adu; st.ops["Aup"] = au;
    st.ops["Adagdn"] = add; st.ops["Adn"] = ad;
    st.ops["Nup"] = nu; st.ops["Ndn"] = nd;
    st.ops["Nupdn"] = matmul(nu, nd, d);
    st.ops["AdagupF"] = matmul(adu, F, d);
    st.ops["FAup"] = matmul(F, au, d);
    st.ops["AdagdnF"] = matmul(add, F, d);
    st.ops["FAdn"] = matmul(F, ad, d);
    st.fermionic = {"AdagupF", "FAup", "AdagdnF", "FAdn"};
    st.labels = {"Emp", "Up", "Dn", "UpDn"};
    return st;
}

// Bond list of a square lattice numbered column by column (n = (x-1) Ly + y),
// the order of squareLattice (itensor/mps/lattice/square.h:9-37).
static std::vector<std::pair<int, int>> square_bonds(int Nx, int Ny, bool yperiodic) {
    yperiodic = yperiodic && Ny > 2;
    std::vector<std::pair<int, int>> b;
    for (int n = 1; n <= Nx * Ny; ++n) {
        int x = (n - 1) / Ny + 1, y = (n - 1) % Ny + 1;
        if (x < Nx) b.push_back({n, n + Ny});
        if (Ny > 1) {
            if (y < Ny) b.push_back({n, n + 1});
            if (yperiodic && y == 1) b.push_back({n, n + Ny - 1});
        }
    }
    return b;
}

Hamiltonian make_hamiltonian(ModelSpec const& m) {
    Hamiltonian H;
    if (m.type == 0) {
        H.st = spin_half(1);
        H.N = m.N;
        for (int j = 1; j < m.N; ++j) {
            H.two.push_back({m.Jz, "Sz", j, "Sz", j + 1});
            H.two.push_back({0.5 * m.J, "S+", j, "S-", j + 1});
            H.two.push_back({0.5 * m.J, "S-", j, "S+", j + 1});
        }
        if (m.J2 != 0.0)
            for (int j = 1; j + 2 <= m.N; ++j) {
                H.two.push_back({m.J2, "Sz", j, "Sz", j + 2});
                H.two.push_back({0.5 * m.J2, "S+", j, "S-", j + 2});
                H.two.push_back({0.5 * m.J2, "S-", j, "S+", j + 2});
            }
    } else if (m.type == 1) {
        H.st = spin_half(2);
        H.N = m.N;
        for (int j = 1; j < m.N; ++j) H.two.push_back({-1.0, "Sx", j, "Sx", j + 1});
        for (int j = 1; j <= m.N; ++j) H.one.push_back({-m.h, "Sz", j});
    } else if (m.type == 2) {
        H.st = electron();
        H.N = m.Lx * m.Ly;
        for (auto [i, j] : square_bonds(m.Lx, m.Ly, m.yperiodic != 0)) {
            int a = std::min(i, j), b = std::max(i, j);
            H.two.push_back({-m.t, "AdagupF", a, "Aup", b});
            H.two.push_back({-m.t, "FAup", a, "Adagup", b});
            H.two.push_back({-m.t, "AdagdnF", a, "Adn", b});
            H.two.push_back({-m.t, "FAdn", a, "Adagdn", b});
        }
        for (int j = 1; j <= H.N; ++j) H.one.push_back({m.U, "Nupdn", j});
    } else {
        throw Error(ERR_ARG, "unknown model type");
    }
    // terms with a zero coefficient carry no MPO channel (a model may set J = 0
    // to hold only the next-nearest terms of a sum of MPOs)
    H.two.erase(std::remove_if(H.two.begin(), H.two.end(), [](Term2 const& t) { return t.c == 0.0; }), H.two.end());
    H.one.erase(std::remove_if(H.one.begin(), H.one.end(), [](Term1 const& t) { return t.c == 0.0; }), H.one.end());
    return H;
}

std::vector<int> default_state(ModelSpec const& m) {
    // Neel product state (spin: Up=0, Dn=1; electron: Up=1, Dn=2); all Up for the Ising chain
    int N = m.type == 2 ? m.Lx * m.Ly : m.N;
    std::vector<int> s(N);
    for (int j = 0; j < N; ++j) {
        if (m.type == 1) s[j] = 0;
        else if (m.type == 2) s[j] = (j % 2 == 0) ? 1 : 2;
        else s[j] = (j % 2 == 0) ? 0 : 1;
    }
    return s;
}

static QN op_flux(SiteType const& st, std::vector<double> const& O) {
    int d = st.d();
    for (int j = 0; j < d; ++j)
        for (int i = 0; i < d; ++i)
            if (O[i + d * j] != 0.0) return st.qn[i] - st.qn[j];
    return QN();
}

// Coefficient carried by the starting operator a at site i: the common
// coefficient of every two-site term starting there, else 1 (the ending
// operator carries the rest). For the nearest-neighbour Heisenberg chain this
// is the gauge of sample/Heisenberg.h:79-90 (J/2 and Jz on the left operator),
// which the density-matrix noise term (a sum over MPO link channels,
// itensor/mps/localop.h:375-406) depends on.
static double left_coef(Hamiltonian const& H, std::string const& a, int i) {
    double c0 = 0.0;
    bool any = false;
    for (auto const& t : H.two) {
        if (t.a != a || t.i != i) continue;
        if (!any) { c0 = t.c; any = true; }
        else if (t.c != c0) return 1.0;
    }
    return (any && c0 != 0.0) ? c0 : 1.0;
}

int mpo_bond_dim(Hamiltonian const& H) {
    std::vector<std::string> lefts;
    int rng = 1;
    for (auto const& t : H.two) {
        if (std::find(lefts.begin(), lefts.end(), t.a) == lefts.end()) lefts.push_back(t.a);
        rng = std::max(rng, t.j - t.i);
    }
    return 2 + (int)lefts.size() * rng;
}

MPO build_mpo(Ctx& ctx, Hamiltonian const& H, std::vector<Index> const* sites) {
    SiteType const& st = H.st;
    const int N = H.N, d = st.d();
    std::vector<std::string> lefts;
    int rng = 1;
    for (auto const& t : H.two) {
        if (std::find(lefts.begin(), lefts.end(), t.a) == lefts.end()) lefts.push_back(t.a);
        rng = std::max(rng, t.j - t.i);
    }
    // states: done, start, then (a, k)
    const int D = 2 + (int)lefts.size() * rng;
    auto chan = [&](int ai, int k) { return 2 + ai * rng + (k - 1); };
    std::vector<QN> sq(D);
    for (size_t ai = 0; ai < lefts.size(); ++ai) {
        QN f = op_flux(st, st.ops.at(lefts[ai]));
        for (int k = 1; k <= rng; ++k) sq[chan((int)ai, k)] = -f;
    }
    std::vector<QN> secq;
    std::vector<int32_t> secd;
    std::vector<int> sec_of(D), off_in(D);
    for (int s = 0; s < D; ++s) {
        size_t n = 0;
        for (; n < secq.size(); ++n) if (secq[n] == sq[s]) break;
        if (n == secq.size()) { secq.push_back(sq[s]); secd.push_back(0); }
        sec_of[s] = (int)n;
        off_in[s] = secd[n]++;
    }
    MPO mpo;
    mpo.bond_dim = D;
    std::vector<Index> links;
    for (int l = 0; l <= N; ++l) links.push_back(Index(secq, secd, 1));
    if (sites) {
        ITG_REQUIRE((int)sites->size() == N, "build_mpo: site list of another length");
        mpo.sites = *sites;
    } else {
        for (int n = 0; n < N; ++n) mpo.sites.push_back(Index(st.qn, std::vector<int32_t>(d, 1), 1));
    }
    for (int n = 1; n <= N; ++n) {
        // dense W[s_in, s_out, row, col]
        std::vector<double> W((size_t)d * d * D * D, 0.0);
        auto put = [&](int r, int c, std::string const& O, double coef) {
            auto const& M = st.ops.at(O);
            for (int si = 0; si < d; ++si)
                for (int so = 0; so < d; ++so)
                    W[si + d * (so + d * (r + (size_t)D * c))] += coef * M[so + d * si];
        };
        put(0, 0, "Id", 1.0);
        put(1, 1, "Id", 1.0);
        for (auto const& t : H.one) if (t.i == n) put(1, 0, t.op, t.c);
        for (size_t ai = 0; ai < lefts.size(); ++ai) {
            bool ferm = std::find(st.fermionic.begin(), st.fermionic.end(), lefts[ai]) != st.fermionic.end();
            bool starts = false;
            for (auto const& t : H.two) if (t.a == lefts[ai] && t.i == n) starts = true;
            if (starts) put(1, chan((int)ai, 1), lefts[ai], left_coef(H, lefts[ai], n));
            for (int k = 1; k < rng; ++k) {
                bool pass = false;
                for (auto const& t : H.two) if (t.a == lefts[ai] && t.i == n - k && t.j > n) pass = true;
                if (pass) put(chan((int)ai, k), chan((int)ai, k + 1), ferm ? "F" : "Id", 1.0);
            }
        }
        for (auto const& t : H.two)
            if (t.j == n) {
                int ai = (int)(std::find(lefts.begin(), lefts.end(), t.a) - lefts.begin());
                put(chan(ai, t.j - t.i), 0, t.b, t.c / left_coef(H, t.a, t.i));
            }
        // QN blocks of (dag(s), s', dag(row link), col link); first/last project the boundary
        const bool first = (n == 1), last = (n == N);
        std::vector<Index> inds{mpo.sites[n - 1].dag(), mpo.sites[n - 1].prime()};
        if (!first) inds.push_back(links[n - 1].dag());
        if (!last) inds.push_back(links[n]);
        Layout all = allowed_layout(inds, QN());
        std::vector<int32_t> coords;
        std::vector<std::vector<double>> bdata;
        const int r = (int)inds.size();
        for (int b = 0; b < all.nblocks(); ++b) {
            int32_t const* c = all.block(b);
            int si = c[0], so = c[1];
            int rsec = first ? -1 : c[2];
            int csec = last ? -1 : c[first ? 2 : 3];
            std::vector<int> rows, cols;
            for (int s = 0; s < D; ++s) {
                if (first ? s == 1 : sec_of[s] == rsec) rows.push_back(s);
                if (last ? s == 0 : sec_of[s] == csec) cols.push_back(s);
            }
            std::vector<double> blk(rows.size() * cols.size(), 0.0);
            bool nz = false;
            for (size_t ir = 0; ir < rows.size(); ++ir)
                for (size_t ic = 0; ic < cols.size(); ++ic) {
                    double v = W[si + d * (so + d * (rows[ir] + (size_t)D * cols[ic]))];
                    if (v != 0.0) {
                        nz = true;
                        size_t ri = first ? 0 : off_in[rows[ir]];
                        size_t cidx = last ? 0 : off_in[cols[ic]];
                        size_t nrow = first ? 1 : links[n - 1].bdim(rsec);
                        blk[ri + nrow * cidx] = v;
                    }
                }
            if (!nz) continue;
            coords.insert(coords.end(), c, c + r);
            // reorder the (row, col) dense block into the block's column-major layout
            size_t nrow = first ? 1 : links[n - 1].bdim(rsec);
            size_t ncol = last ? 1 : links[n].bdim(csec);
            std::vector<double> out(nrow * ncol, 0.0);
            for (size_t ir = 0; ir < rows.size(); ++ir)
                for (size_t ic = 0; ic < cols.size(); ++ic) {
                    size_t ri = first ? 0 : off_in[rows[ir]];
                    size_t cidx = last ? 0 : off_in[cols[ic]];
                    out[ri + nrow * cidx] = blk[ri + nrow * cidx];
                }
            bdata.push_back(out);
        }
        auto L = std::make_shared<Layout>(make_layout(inds, coords));
        std::vector<double> host(L->size, 0.0);
        // coords were produced in storage order already (allowed_layout order)
        for (int b = 0; b < L->nblocks(); ++b) std::copy(bdata[b].begin(), bdata[b].end(), host.begin() + L->offs[b]);
        mpo.W.push_back(upload_tensor(ctx, L, host.data()));
    }
    return mpo;
}

std::vector<Tensor> product_mps(Ctx& ctx, MPO const& H, SiteType const& st, std::vector<int> const& states) {
    const int N = (int)states.size();
    std::vector<QN> qa(N + 1);
    QN tot;
    for (int s : states) tot = tot + st.qn[s];
    qa[0] = tot;
    for (int i = 1; i <= N; ++i) qa[i] = qa[i - 1] - st.qn[states[i - 1]];
    std::vector<Index> links(N + 1);
    for (int i = 1; i < N; ++i) links[i] = Index({qa[i]}, {1}, 1);
    std::vector<Tensor> psi;
    for (int i = 1; i <= N; ++i) {
        std::vector<Index> inds;
        std::vector<int32_t> c;
        if (i > 1) { inds.push_back(links[i - 1].dag()); c.push_back(0); }
        inds.push_back(H.sites[i - 1]);
        c.push_back(states[i - 1]);
        if (i < N) { inds.push_back(links[i]); c.push_back(0); }
        auto L = std::make_shared<Layout>(make_layout(inds, c));
        double one = 1.0;
        psi.push_back(upload_tensor(ctx, L, &one));
    }
    return psi;
}

}  // namespace itg
