// Implicit QL for the symmetric tridiagonal eigenproblem: the tql2 procedure
// of Bowdler, Martin, Reinsch & Wilkinson (Handbook for Automatic Computation,
// vol. II, contribution II/3), the same family of iterations as LAPACK's dsteqr
// that the reference reaches through dsyev (itensor/tensor/algs.cc:34-41).
// Only the rotations are recorded here; the device applies them to the
// Householder basis Q (eigh_tri.cu). The recurrence is a chain of dependent
// scalar FP64 operations with a square root and two divisions per rotation;
// it runs on the host core, where such a chain costs a few nanoseconds per
// operation, while every O(n^3) stage runs on the GPU.
#include "tridiag_ql.h"
#include <algorithm>
#include <cmath>

namespace itg {

int tridiag_ql(int n, double* d, double* e, std::vector<QlSweep>& sweeps, std::vector<QlRot>& rots) {
    if (n <= 0) return 0;
    const size_t base = rots.size();
    const double eps = 2.220446049250313e-16;
    e[n - 1] = 0.0;
    double f = 0.0, tst1 = 0.0;
    for (int l = 0; l < n; ++l) {
        tst1 = std::max(tst1, std::fabs(d[l]) + std::fabs(e[l]));
        int m = l;
        while (m < n - 1 && std::fabs(e[m]) > eps * tst1) ++m;
        if (m > l) {
            int iter = 0;
            do {
                if (++iter > 30) return 1;
                // shift from the leading 2x2 block
                double g = d[l];
                double p = (d[l + 1] - g) / (2.0 * e[l]);
                double r = std::hypot(p, 1.0);
                if (p < 0) r = -r;
                d[l] = e[l] / (p + r);
                d[l + 1] = e[l] * (p + r);
                const double dl1 = d[l + 1];
                double h = g - d[l];
                for (int i = l + 2; i < n; ++i) d[i] -= h;
                f += h;
                // QL sweep from the bottom of the unreduced block
                p = d[m];
                double c = 1.0, c2 = 1.0, c3 = 1.0, s = 0.0, s2 = 0.0;
                const double el1 = e[l + 1];
                sweeps.push_back(QlSweep{l, m, (int32_t)(rots.size() - base), 0});
                for (int i = m - 1; i >= l; --i) {
                    c3 = c2;
                    c2 = c;
                    s2 = s;
                    const double ei = e[i], di = d[i];
                    g = c * ei;
                    h = c * p;
                    r = std::sqrt(p * p + ei * ei);
                    if (!(r > 1e-150 && r < 1e150)) r = std::hypot(p, ei);
                    e[i + 1] = s * r;
                    s = ei / r;
                    c = p / r;
                    p = c * di - s * g;
                    d[i + 1] = h + s * (c * g + s * di);
                    rots.push_back(QlRot{c, s});
                }
                p = -s * s2 * c3 * el1 * e[l] / dl1;
                e[l] = s * p;
                d[l] = c * p;
            } while (std::fabs(e[l]) > eps * tst1);
        }
        d[l] += f;
        e[l] = 0.0;
    }
    return 0;
}

int ql_schedule(int n, std::vector<QlSweep> const& sweeps, int workers, int window, std::vector<int32_t>& woff,
                std::vector<QlStart>& entries) {
    // per column: window of its last rotation and the worker that applied it
    std::vector<int64_t> last_win(std::max(n, 1) + 1, -1);
    std::vector<int> last_worker(std::max(n, 1) + 1, -1);
    std::vector<int64_t> free_at(workers, 0);
    std::vector<std::vector<QlStart>> per(workers);
    int64_t nsteps = 0;
    for (size_t t = 0; t < sweeps.size(); ++t) {
        const int l = sweeps[t].l, m = sweeps[t].m;
        int w = 0;
        for (int k = 1; k < workers; ++k)
            if (free_at[k] < free_at[w]) w = k;
        // rotation i (columns i, i+1) runs at step S + (m - 1 - i); it must fall in
        // a later window than the last rotation on either column by another worker
        // (a worker's own rotations are ordered by its program)
        int64_t S = free_at[w];
        for (int i = l; i < m; ++i)
            for (int c = i; c <= i + 1; ++c)
                if (last_worker[c] >= 0 && last_worker[c] != w)
                    S = std::max(S, (last_win[c] + 1) * window - (m - 1 - i));
        for (int i = m - 1; i >= l; --i) {
            const int64_t win = (S + (m - 1 - i)) / window;
            for (int c = i; c <= i + 1; ++c) {
                last_win[c] = std::max(last_win[c], win);
                last_worker[c] = w;
            }
        }
        free_at[w] = S + (m - l);
        nsteps = std::max(nsteps, free_at[w]);
        per[w].push_back(QlStart{(int32_t)S, (int32_t)t});
    }
    woff.assign(workers + 1, 0);
    entries.clear();
    for (int w = 0; w < workers; ++w) {
        woff[w] = (int32_t)entries.size();
        entries.insert(entries.end(), per[w].begin(), per[w].end());
    }
    woff[workers] = (int32_t)entries.size();
    return (int)((nsteps + window - 1) / window * window);
}

}  // namespace itg
