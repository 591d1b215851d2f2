// Host side of the large-block eigensolver: the implicit QL recurrence on the
// tridiagonal matrix (d, e) that the device reduction produced.
#pragma once
#include <cstdint>
#include <vector>

namespace itg {

struct QlSweep { int32_t l, m, off, pad; };   // rotations off.. (m-l of them) act on columns l..m
struct QlRot { double c, s; };

// Eigenvalues of the symmetric tridiagonal matrix with diagonal d[0..n) and
// off-diagonal e[i] = T(i, i+1) (e[n-1] ignored), by implicit QL with
// Wilkinson-type shifts. d is replaced by the eigenvalues (unsorted); every QL
// sweep is appended to `sweeps` with its plane rotations in `rots` (offsets
// relative to the first rotation this call appends). Returns 0, or 1 when an
// eigenvalue needed more than 30 sweeps.
int tridiag_ql(int n, double* d, double* e, std::vector<QlSweep>& sweeps, std::vector<QlRot>& rots);

}  // namespace itg
