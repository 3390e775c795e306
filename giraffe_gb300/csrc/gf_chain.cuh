// Direct solver for K_AA of Beam_1 chains (elements e = 0..m-1 on nodes
// 2e, 2e+1, 2e+2; node-major DOF numbering), FP64, no pivoting.
//
// K_AA of such a chain is block-tridiagonal over the corner nodes once the
// midside nodes are condensed: a midside node couples only to the two corner
// nodes of its element.  The solve therefore runs as
//   1. condensation   per element: Z_s = A_ss^{-1} [b_s | A_sa | A_sb] and the
//                     Schur contributions to the two corners (parallel over
//                     all elements of all chains);
//   2. corner system  D_k, L_k (coupling to the previous corner), U_k (to the
//                     next) and b_k per free corner;
//   3. cyclic reduction over corner positions, one level per launch: odd
//                     positions are eliminated (Z = D^{-1} [b | L | U]),
//                     even positions absorb them; the last survivor is
//                     solved directly;
//   4. back substitution level by level, then the midside nodes.
// The critical path is O(log m) small dense solves instead of the O(n)
// column recurrence of a banded LU, which on a GPU with slow FP64 latency
// (~64 cycles per dependent FP64 operation) dominates long chains.  The
// solver never reads an assembled K_AA: it takes each element's tangent K_e
// from the element scratch (plus the nodal load stiffness), which is the
// same K_AA term by term.  Equations follow from block
// Gaussian elimination on the assembled matrix; the reference solves the
// same K_AA with PARDISO (reference src/SparseMatrix.cpp:74-166).
#pragma once
#include <cuda_runtime.h>

#include "gf_types.h"

namespace gf {

void launch_chain_solve(const Batch& b, const ChainData& c, cudaStream_t st);

}  // namespace gf
