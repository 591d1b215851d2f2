// Host-side checks of the large-block eigensolver's CPU stages (tridiag_ql.cpp):
//  1. the implicit QL eigenvalues against the tridiagonal's characteristic
//     residual (T - lambda) y = 0 for the accumulated eigenvectors;
//  2. the lockstep schedule (ql_schedule) with windows of 1..8 steps: replaying
//     the recorded rotations window by window, warps in either order, gives the
//     same result as applying them one after another, and no two warps touch
//     the same column inside a window;
//  3. the kept-vector stage: the rotations in reverse order on unit vectors, in
//     mirrored columns, give the columns of the full rotation product.
// Built and run by tests/test_native_cpu.py; prints one line and exits 0 on success.
#include "tridiag_ql.h"
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <map>
#include <numeric>
#include <random>

using namespace itg;

namespace {
// rotation at column i applied to rows of Z (Z[r * n + c]): the device kernel's formula
void rotate_rows(std::vector<double>& Z, int rows, int n, int i, QlRot q) {
    for (int r = 0; r < rows; ++r) {
        const double a = Z[(size_t)r * n + i], b = Z[(size_t)r * n + i + 1];
        Z[(size_t)r * n + i + 1] = q.s * a + q.c * b;
        Z[(size_t)r * n + i] = q.c * a - q.s * b;
    }
}

// window-by-window replay of a schedule; returns the number of column conflicts
int replay(std::vector<double>& Z, int rows, int n, std::vector<QlSweep> const& sw, std::vector<QlRot> const& rot,
           std::vector<int32_t> const& woff, std::vector<QlStart> const& ent, int W, int K, int nsteps, bool reverse) {
    int conflicts = 0;
    std::vector<int> ptr(W);
    for (int w = 0; w < W; ++w) ptr[w] = woff[w];
    for (int s0 = 0; s0 < nsteps; s0 += K) {
        std::map<int, int> owner;
        for (int ww = 0; ww < W; ++ww) {
            const int w = reverse ? W - 1 - ww : ww;
            for (int u = 0; u < K; ++u) {
                const int s = s0 + u;
                if (ptr[w] < woff[w + 1]) {
                    auto x = ent[ptr[w]];
                    if (s >= x.step + (sw[x.sweep].m - sw[x.sweep].l)) ++ptr[w];
                }
                if (ptr[w] < woff[w + 1]) {
                    auto x = ent[ptr[w]];
                    auto const& h = sw[x.sweep];
                    if (s >= x.step) {
                        const int j = s - x.step, i = h.m - 1 - j;
                        for (int c = i; c <= i + 1; ++c) {
                            auto it = owner.find(c);
                            if (it != owner.end() && it->second != w) ++conflicts;
                            owner[c] = w;
                        }
                        rotate_rows(Z, rows, n, i, rot[h.off + j]);
                    }
                }
            }
        }
    }
    return conflicts;
}
}  // namespace

int main() {
    std::mt19937 rng(2024);
    std::normal_distribution<double> N01;
    double worst_res = 0, worst_sched = 0, worst_kept = 0;
    int conflicts = 0, failures = 0;
    for (int trial = 0; trial < 40; ++trial) {
        const int n = 2 + (int)(rng() % 160);
        std::vector<double> d(n), e(n);
        for (int i = 0; i < n; ++i) {
            d[i] = N01(rng) * std::exp(-0.05 * i);
            e[i] = N01(rng) * std::exp(-0.04 * i);
        }
        if (trial % 4 == 0)
            for (int i = 0; i < n; i += 9) e[i] = 0;  // split into unreduced blocks
        const std::vector<double> d0 = d, e0 = e;
        std::vector<QlSweep> sw;
        std::vector<QlRot> rot;
        if (tridiag_ql(n, d.data(), e.data(), sw, rot)) { ++failures; continue; }
        // 1. eigenvectors (columns of I G, sequential) against T
        std::vector<double> Z((size_t)n * n, 0.0);
        for (int i = 0; i < n; ++i) Z[(size_t)i * n + i] = 1.0;
        for (auto const& h : sw)
            for (int i = h.m - 1, j = 0; i >= h.l; --i, ++j) rotate_rows(Z, n, n, i, rot[h.off + j]);
        for (int j = 0; j < n; ++j)
            for (int c = 0; c < n; ++c) {
                double ty = d0[c] * Z[(size_t)c * n + j];
                if (c > 0) ty += e0[c - 1] * Z[(size_t)(c - 1) * n + j];
                if (c + 1 < n) ty += e0[c] * Z[(size_t)(c + 1) * n + j];
                worst_res = std::max(worst_res, std::fabs(ty - d[j] * Z[(size_t)c * n + j]));
            }
        // 2. lockstep schedules
        for (int W : {8, 16, 32})
        for (int K : {1, 4, 8}) {
            std::vector<int32_t> woff;
            std::vector<QlStart> ent;
            const int nsteps = ql_schedule(n, sw, W, K, woff, ent);
            for (bool rev : {false, true}) {
                std::vector<double> Y((size_t)n * n, 0.0);
                for (int i = 0; i < n; ++i) Y[(size_t)i * n + i] = 1.0;
                conflicts += replay(Y, n, n, sw, rot, woff, ent, W, K, nsteps, rev);
                for (size_t q = 0; q < Y.size(); ++q) worst_sched = std::max(worst_sched, std::fabs(Y[q] - Z[q]));
            }
        }
        // 3. kept vectors: reversed rotations on unit vectors in mirrored columns
        std::vector<int> ord(n);
        std::iota(ord.begin(), ord.end(), 0);
        std::stable_sort(ord.begin(), ord.end(), [&](int x, int y) { return d[x] > d[y]; });
        const int k = 1 + (int)(rng() % n);
        std::vector<QlSweep> msw;
        std::vector<QlRot> mrot;
        for (int t = (int)sw.size() - 1; t >= 0; --t) {
            const int l = sw[t].l, m = sw[t].m, len = m - l;
            msw.push_back(QlSweep{n - 1 - m, n - 1 - l, (int32_t)mrot.size(), 0});
            for (int j = 0; j < len; ++j) mrot.push_back(rot[sw[t].off + (len - 1 - j)]);
        }
        std::vector<int32_t> woff;
        std::vector<QlStart> ent;
        const int nsteps = ql_schedule(n, msw, 8, 4, woff, ent);
        std::vector<double> T((size_t)k * n, 0.0);
        for (int r = 0; r < k; ++r) T[(size_t)r * n + (n - 1 - ord[r])] = 1.0;
        conflicts += replay(T, k, n, msw, mrot, woff, ent, 8, 4, nsteps, false);
        for (int r = 0; r < k; ++r)
            for (int c = 0; c < n; ++c)
                worst_kept = std::max(worst_kept, std::fabs(T[(size_t)r * n + (n - 1 - c)] - Z[(size_t)c * n + ord[r]]));
    }
    std::printf("residual %.2e schedule %.2e kept %.2e conflicts %d failures %d\n", worst_res, worst_sched, worst_kept,
                conflicts, failures);
    return (worst_res < 1e-12 && worst_sched == 0.0 && worst_kept < 1e-13 && conflicts == 0 && failures == 0) ? 0 : 1;
}
