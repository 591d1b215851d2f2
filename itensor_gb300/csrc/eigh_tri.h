// Large-block path of the batched symmetric eigensolver (eigh_tri.cu).
#pragma once
#include "ops.h"

namespace itg {

constexpr int TRI_MAX_N = 6000;
// Blocks with n >= this size take the tridiagonal path (ITG_EIG_TRI_MIN overrides).
constexpr int TRI_MIN_N_DEFAULT = 16;

// Same contract as batched_eigh for the given items (eigenvalues descending,
// eigenvectors in columns; 2 n^2 doubles of scratch per item). Returns the
// number of blocks whose QL iteration did not converge.
int tri_eigh(Ctx& ctx, std::vector<EigItem> const& items, double const* src, double* vout, double* wout,
             double* scratch);

}  // namespace itg
