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

// Lockstep schedule for applying the recorded sweeps with `workers` workers
// that each apply one rotation per step, with a barrier after every `window`
// steps: every sweep starts at the earliest step at which each of its
// rotations falls in a later window than all rotations of earlier sweeps on
// another worker that share a column (rotations on disjoint column pairs
// commute), on the worker that is free first. Fills the per-worker entry
// lists (start step, sweep index), entries of worker w at
// [woff[w], woff[w+1]), and returns the number of steps (a whole number of windows).
struct QlStart { int32_t step, sweep; };
int ql_schedule(int n, std::vector<QlSweep> const& sweeps, int workers, int window, std::vector<int32_t>& woff,
                std::vector<QlStart>& entries);

}  // namespace itg
