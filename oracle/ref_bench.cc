// CPU baseline: times the ITensor C++ reference (built from its own sources by
// oracle/Makefile.ref, linked to a LAPACK/BLAS) on the benchmark's workloads.
// Test and baseline infrastructure only; nothing in the product links it.
//
//   ref_bench heff <dir> <seconds>   LocalOp::product (itensor/mps/localop.h:324-365)
//                                    on psi, L, W1, W2, R read with readFromFile
//                                    from <dir>/{psi,L,W1,W2,R}.itensor, repeated
//                                    for about <seconds>
//   ref_bench dmrg <reps>            dmrg() of the N=20 Heisenberg chain (Sz QN,
//                                    sample/Heisenberg.h MPO, Neel start, 5 sweeps
//                                    maxdim 10,20,100,100,200, cutoff 1e-10, niter 2)
// Prints one JSON line. Threads: OMP_NUM_THREADS (the reference parallelises
// over output blocks, itensor/itdata/qutil.h:330-348); BLAS runs one thread.
#include "itensor/all.h"
#include "Heisenberg.h"
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <string>

using namespace itensor;
using clk = std::chrono::steady_clock;

static double secs(clk::time_point a) { return std::chrono::duration<double>(clk::now() - a).count(); }

static int bench_heff(std::string const& dir, double budget) {
    ITensor psi, L, W1, W2, R;
    readFromFile(dir + "/psi.itensor", psi);
    readFromFile(dir + "/L.itensor", L);
    readFromFile(dir + "/W1.itensor", W1);
    readFromFile(dir + "/W2.itensor", W2);
    readFromFile(dir + "/R.itensor", R);
    LocalOp op(W1, W2, L, R);
    ITensor out;
    op.product(psi, out);  // warm
    auto t0 = clk::now();
    op.product(psi, out);
    double one = secs(t0);
    long n = std::max<long>(1, (long)(budget / std::max(one, 1e-4)));
    t0 = clk::now();
    for (long i = 0; i < n; ++i) op.product(psi, out);
    double el = secs(t0);
    std::printf("{\"n\":%ld,\"sec\":%.9g,\"norm\":%.17g}\n", n, el, norm(out));
    return 0;
}

static int bench_dmrg(int reps) {
    int N = 20;
    auto sites = SpinHalf(N);
    MPO H = Heisenberg(sites);
    auto st = InitState(sites);
    for (int i = 1; i <= N; ++i) st.set(i, i % 2 == 1 ? "Up" : "Dn");
    auto sw = Sweeps(5);
    sw.maxdim() = 10, 20, 100, 100, 200;
    sw.cutoff() = 1e-10;
    sw.niter() = 2;
    sw.noise() = 0.0;
    double best = 1e30, E = 0;
    for (int r = 0; r < reps; ++r) {
        auto t0 = clk::now();
        auto [en, psi] = dmrg(H, MPS(st), sw, {"Quiet", true, "Silent", true});
        best = std::min(best, secs(t0));
        E = en;
    }
    std::printf("{\"reps\":%d,\"best_sec\":%.9g,\"energy\":%.17g}\n", reps, best, E);
    return 0;
}

int main(int argc, char** argv) {
    std::string what = argc > 1 ? argv[1] : "";
    if (what == "heff" && argc > 3) return bench_heff(argv[2], std::atof(argv[3]));
    if (what == "dmrg") return bench_dmrg(argc > 2 ? std::atoi(argv[2]) : 3);
    std::fprintf(stderr, "usage: ref_bench heff <dir> <seconds> | ref_bench dmrg [reps]\n");
    return 2;
}
