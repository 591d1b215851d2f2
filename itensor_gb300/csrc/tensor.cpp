// Block-structure helpers for the host data model (see tensor.h).
#include "tensor.h"
#include <atomic>
#include <numeric>

namespace itg {

uint64_t new_index_id() {
    static std::atomic<uint64_t> next{0x1000};
    return next.fetch_add(1);
}

bool coords_less(int32_t const* a, int32_t const* b, int rank) {
    for (int k = rank - 1; k >= 0; --k) {
        if (a[k] != b[k]) return a[k] < b[k];
    }
    return false;
}

int Layout::find_block(int32_t const* c) const {
    int lo = 0, hi = nblocks();
    int r = rank();
    while (lo < hi) {
        int mid = (lo + hi) / 2;
        if (coords_less(block(mid), c, r)) lo = mid + 1;
        else hi = mid;
    }
    if (lo < nblocks() && !coords_less(c, block(lo), r)) return lo;
    return -1;
}

Layout allowed_layout(std::vector<Index> const& inds, QN const& div) {
    Layout L;
    L.inds = inds;
    int r = (int)inds.size();
    if (r == 0) { L.finish(); return L; }
    std::vector<int32_t> c(r, 0);
    // iterate with the first index fastest: this is already reversed-lexicographic order
    while (true) {
        if (L.flux(c.data()) == div) L.coords.insert(L.coords.end(), c.begin(), c.end());
        int k = 0;
        while (k < r) {
            if (++c[k] < inds[k].nblock()) break;
            c[k] = 0;
            ++k;
        }
        if (k == r) break;
    }
    L.finish();
    return L;
}

Layout make_layout(std::vector<Index> const& inds, std::vector<int32_t> coords) {
    Layout L;
    L.inds = inds;
    int r = (int)inds.size();
    if (r == 0) { L.finish(); return L; }
    int nb = (int)(coords.size() / r);
    std::vector<int> ord(nb);
    std::iota(ord.begin(), ord.end(), 0);
    std::sort(ord.begin(), ord.end(), [&](int a, int b) { return coords_less(&coords[(size_t)a * r], &coords[(size_t)b * r], r); });
    L.coords.reserve(coords.size());
    for (int i = 0; i < nb; ++i) {
        int32_t const* c = &coords[(size_t)ord[i] * r];
        if (i > 0 && !coords_less(&L.coords[L.coords.size() - r], c, r)) continue;  // drop duplicates
        L.coords.insert(L.coords.end(), c, c + r);
    }
    L.finish();
    return L;
}

Tensor relabel(Tensor const& t, std::vector<Index> inds) {
    Tensor r = t;
    auto L = std::make_shared<Layout>(*t.lay);
    L->inds = std::move(inds);
    r.lay = L;
    return r;
}

}  // namespace itg
