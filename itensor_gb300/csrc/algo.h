// Host-side algorithms of the two-site DMRG inner loop, driving the device
// kernels. Each function follows the reference routine named beside it.
#pragma once
#include "ops.h"
#include <map>

namespace itg {

// ---------------------------------------------------------------- tensors
Tensor upload_tensor(Ctx& ctx, std::shared_ptr<Layout> lay, double const* host);
std::vector<double> download(Ctx& ctx, Tensor const& t);
QN tensor_div(Tensor const& t);
std::vector<Index> prime_all(std::vector<Index> inds, int inc = 1);
std::vector<Index> dag_all(std::vector<Index> inds);
std::vector<Index> noprime_all(std::vector<Index> inds);
Tensor copy_tensor(Ctx& ctx, Tensor const& t);
double tensor_norm(Ctx& ctx, Tensor const& t);

// ---------------------------------------------------------------- truncate
// itensor/decomp.cc:305-463 (bit-for-bit the same decisions and values)
struct TruncResult {
    std::vector<double> P;
    double truncerr = 0, docut_lower = 0, docut_upper = 0;
    int ndegen = 0;
};
TruncResult truncate(std::vector<double> P, long maxdim, long mindim, double cutoff, bool absoluteCutoff,
                     bool doRelCutoff, bool respectDegenerate);

// ---------------------------------------------------------------- combiner
// combiner / QCombiner (itensor/itensor.cc:1469-1560, itensor/itdata/qcombiner.cc:125-300)
struct Combiner {
    std::vector<Index> inds;
    Index ci;
    // sector tuple (one per fused index) -> (sector of ci, start, extent)
    std::map<std::vector<int32_t>, std::array<int32_t, 3>> ranges;
};
Combiner make_combiner(std::vector<Index> const& inds);
Tensor combine(Ctx& ctx, Tensor const& T, Combiner const& C);     // inds: [ci] + rest
Tensor uncombine(Ctx& ctx, Tensor const& T, Combiner const& C);   // ci replaced in place

// ---------------------------------------------------------------- H_eff and Davidson
// LocalOp::product (itensor/mps/localop.h:324-365); L or R may be null.
struct LocalOp {
    Tensor const* L = nullptr;
    Tensor const* W1 = nullptr;
    Tensor const* W2 = nullptr;
    Tensor const* R = nullptr;
    // Excited states (LocalMPO_MPS, itensor/mps/localmpo_mps.h:137-150): the
    // apply adds proj_weight * sum_j P_j (P_j . phi), P_j stored in phi's layout.
    std::vector<Tensor> const* proj = nullptr;
    double proj_weight = 0.0;
    // Sums of MPOs (LocalMPOSet, itensor/mps/localmposet.h:140-152): the local
    // operators of the other MPOs, whose products are added to this one's.
    std::vector<LocalOp> const* terms = nullptr;
};
// H_eff * phi written in phi's layout (phi must hold every block of its divergence).
// into_phi_layout=false returns the reference's own output structure instead.
Tensor heff_product(Ctx& ctx, LocalOp const& op, Tensor const& phi, int prec, bool into_phi_layout = true);
// A prepared H_eff apply for a fixed (L, W1, W2, R, phi layout): plans resolved
// once, intermediates preallocated, launches optionally replayed as one CUDA
// graph. run() reads phi from `in` and writes H_eff phi to `out` (device
// pointers, or host pointers when host=true: copies are part of the run).
struct HeffProgram {
    struct Step {
        std::shared_ptr<Plan> plan;
        Tensor operand;        // L, W1, W2 or R
        bool operand_left;     // operand is the left factor of the contraction
        int in_buf, out_buf;   // -1 = program input, -2 = program output, else intermediate
        bool split = false;    // split-precision kernels; scratch holds the digit panels
        DevBufPtr scratch;
        bool operand_sliced = false;  // the fixed operand's panels are in place
    };
    int slices = 6;
    std::vector<Step> steps;
    std::vector<DevBufPtr> inter;
    DevBufPtr in, out;
    int64_t in_size = 0, out_size = 0;
    std::shared_ptr<Layout> out_layout;
    int prec = 0;
    bool use_graph = false;
    cudaGraphExec_t graph = nullptr;
    int launches_per_run = 0;
    double flops = 0;
    ~HeffProgram();
    void run(Ctx& ctx, double const* in_ptr, double* out_ptr, bool host = false);
    void launch_steps(Ctx& ctx);
};
// fuse_mpo: contract the two MPO tensors once and run one MPO step per apply
// (for programs applied many times; it is skipped where it costs more flops)
std::shared_ptr<HeffProgram> heff_prepare(Ctx& ctx, LocalOp const& op, std::shared_ptr<Layout> phi_layout, int prec,
                                          bool into_phi_layout, bool use_graph, bool fuse_mpo = false);

// davidson, block size 1 (itensor/iterativesolvers.h:99-451); phi is replaced by the
// normalised lowest Ritz vector; returns the Ritz value.
double davidson(Ctx& ctx, LocalOp const& op, Tensor& phi, int maxiter, double errgoal, int miniter, int prec,
                int* applies = nullptr);

// ---------------------------------------------------------------- bond split
struct SplitArgs {
    double cutoff = 0;
    long maxdim = 0, mindim = 1;
    bool respect_degenerate = true;
    bool normalize = true;
};
struct SplitResult {
    Tensor A, B;
    std::vector<double> probs;
    double truncerr = 0;
    Index link;
};
// denmatDecomp (itensor/decomp.h:316-418) with diag_hermitian's QN branch
// (itensor/hermitian.cc:180-426) and the DoNormalize step of MPS::svdBond.
// With noise > 0 and op given, rho += noise * deltaRho (LocalOp::deltaRho,
// itensor/mps/localop.h:375-406) and rho is divided by its trace.
SplitResult denmat_decomp(Ctx& ctx, Tensor const& AA, Tensor const& A, Tensor const& B, bool fromleft,
                          SplitArgs const& args, int prec, LocalOp const* op = nullptr, double noise = 0.0);
// The noise term of the density matrix: AA times the environment and MPO
// tensor of the side being orthogonalised, primes removed, combined with cmb
// and squared over every index but cmb.ci: indices (ci, ci'). Not symmetrised.
Tensor delta_rho(Ctx& ctx, LocalOp const& op, Tensor const& AA, Combiner const& cmb, bool fromleft);

// svd route of MPS::svdBond (itensor/mps/mps_impl.h:50-65): svd
// (itensor/decomp.cc:121-248) with svdImpl's QN branch (itensor/svd.cc:169-401);
// A's indices not on B go to U. The singular values (normalised when
// args.normalize) are pushed into B (fromleft) or A. probs = kept s^2.
SplitResult svd_split(Ctx& ctx, Tensor const& AA, Tensor const& A, Tensor const& B, bool fromleft,
                      SplitArgs const& args, int prec);

// ---------------------------------------------------------------- models / MPO / MPS
struct SiteType {
    std::string name;
    std::vector<QN> qn;                                   // per basis state
    std::map<std::string, std::vector<double>> ops;       // d x d, element (i,j) = <i|O|j> at i + d j
    std::vector<std::string> fermionic;                   // left operators of a hop that carry the string
    std::vector<std::string> labels;
    int d() const { return (int)qn.size(); }
};
SiteType spin_half(int conserve);   // 0 none, 1 Sz, 2 parity
SiteType electron();

struct Term2 { double c; std::string a; int i; std::string b; int j; };
struct Term1 { double c; std::string op; int i; };
struct Hamiltonian {
    SiteType st;
    int N = 0;
    std::vector<Term1> one;
    std::vector<Term2> two;
};
// model: 0 Heisenberg/XXZ/J1-J2 (J, Jz, J2), 1 transverse-field Ising (h),
// 2 Hubbard on an Lx x Ly square lattice snaked column by column (t, U, yperiodic)
struct ModelSpec {
    int type = 0;
    int N = 0;
    double J = 1, Jz = 1, J2 = 0, h = 0, t = 1, U = 0;
    int Lx = 0, Ly = 1;
    int yperiodic = 0;
};
Hamiltonian make_hamiltonian(ModelSpec const& m);
// Bond dimension of the MPO build_mpo makes: done, start, and one channel per
// (left operator, distance still to go).
int mpo_bond_dim(Hamiltonian const& H);

struct MPO {
    std::vector<Index> sites;
    std::vector<Tensor> W;      // W_n: (dag(s_n), s_n', dag(link_{n-1}), link_n), ends projected
    int bond_dim = 0;
};
// sites: the site indices to use (another MPO's, for sums of MPOs); new ones if null.
MPO build_mpo(Ctx& ctx, Hamiltonian const& H, std::vector<Index> const* sites = nullptr);
// A caller's MPO tensors with an initial MPS on the same sites (site j: the
// index psi0[j] shares with W[j] at prime level 0, which W[j] also holds
// primed; neighbouring tensors share one link each), as dmrg(H, psi0, sweeps)
// receives them (itensor/mps/dmrg.h:67-76). `sites`: the site indices another
// MPO of a sum already uses (they must agree).
MPO mpo_from_tensors(std::vector<Tensor> const& W, std::vector<Tensor> const& psi0,
                     std::vector<Index> const* sites = nullptr);
// Product state with the link QNs of MPS(InitState) (itensor/mps/mps.cc:558-585).
std::vector<Tensor> product_mps(Ctx& ctx, MPO const& H, SiteType const& st, std::vector<int> const& states);
std::vector<int> default_state(ModelSpec const& m);

// ---------------------------------------------------------------- DMRG
struct SweepSpec {
    long maxdim = 0, mindim = 1;
    double cutoff = 0;
    int niter = 2;
    double noise = 0;
    bool use_svd = false;  // as UseSVD; the SVD route is also taken when cutoff < 1e-12
};
struct BondRecord { int sweep, halfsweep, bond; double energy, truncerr; long dim; };
struct DmrgResult {
    double energy = 0;
    std::vector<Tensor> psi;   // the final MPS
    std::vector<BondRecord> bonds;
    std::vector<Index> links;
    std::vector<double> sweep_seconds;
    int heff_applies = 0;
    // wall seconds in: environments + two-site tensor, Davidson, bond split
    double phase_seconds[3] = {0, 0, 0};
};
// DMRGWorker (itensor/mps/dmrg.h:336-467) with LocalMPO environments
// (itensor/mps/localmpo.h:443-618).
// With `prev`, the state that minimises H + weight sum_j |psi_j><psi_j| (the
// excited-state dmrg of itensor/mps/dmrg.h:245-266, LocalMPO_MPS of
// itensor/mps/localmpo_mps.h): prev holds earlier results' MPS in the same QN sector.
// With `more`, H is the sum of H and the MPOs in `more` (on the same sites):
// dmrg(psi, {H1, H2, ...}, sweeps) with LocalMPOSet (itensor/mps/dmrg.h:181-230).
DmrgResult dmrg(Ctx& ctx, MPO const& H, std::vector<Tensor> psi, std::vector<SweepSpec> const& sweeps, int prec,
                std::vector<std::vector<Tensor>> const* prev = nullptr, double weight = 1.0,
                std::vector<MPO> const* more = nullptr);

}  // namespace itg
