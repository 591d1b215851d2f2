// Large-block path of the batched symmetric eigensolver (eigh_tri.cu), in two
// stages so that a caller that truncates computes only the eigenvectors it keeps.
#pragma once
#include "ops.h"
#include <memory>

namespace itg {

constexpr int TRI_MAX_N = 6000;
// Blocks with n >= this size take the tridiagonal path (ITG_EIG_TRI_MIN overrides).
constexpr int TRI_MIN_N_DEFAULT = 16;

// State between the two stages: the reduced blocks (reflectors in the first
// half of each item's scratch), the QL rotation logs and eigenvalue orders.
struct TriPending;
struct TriPendingFree {
    void operator()(TriPending* p) const;
};
using TriPendingPtr = std::unique_ptr<TriPending, TriPendingFree>;

// Stage 1: every item's eigenvalues, descending, written to wout (2 n^2
// doubles of scratch per item, kept until stage 2). ids[i] names item i in the
// keep vector of stage 2. *bad counts the blocks whose QL did not converge.
TriPendingPtr tri_eigh_begin(Ctx& ctx, std::vector<EigItem> const& items, std::vector<int> const& ids,
                             double const* src, double* wout, double* scratch, int* bad);
// Stage 2: the eigenvectors of the keep[id] largest eigenvalues of each item,
// as the first keep[id] columns of its block in vout (descending order).
void tri_eigh_finish(Ctx& ctx, TriPending& p, std::vector<int> const& keep, double* vout, double* scratch);

// The batched eigensolver in the same two stages: begin diagonalises the small
// blocks completely (one-CTA Jacobi) and gives every block's eigenvalues
// (descending) in wout; finish adds the first keep[i] eigenvectors of each
// large block i (the small blocks already have all of theirs).
struct EighPending {
    TriPendingPtr tri;
    int bad = 0;          // blocks whose iteration did not converge (known so far)
    int jac_pending = 0;  // Jacobi statuses on their way to ctx.defer_host
};
// After a sync() that follows batched_eigh_begin: adds the Jacobi statuses to
// p.bad and returns it.
int eigh_collect(Ctx& ctx, EighPending& p);
EighPending batched_eigh_begin(Ctx& ctx, std::vector<EigItem> const& items, double const* src, double* vout,
                               double* wout, double* scratch);
void batched_eigh_finish(Ctx& ctx, EighPending& p, std::vector<int> const& keep, double* vout, double* scratch);

}  // namespace itg
