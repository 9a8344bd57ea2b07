// fsai.cuh -- factorised sparse approximate inverse (FSAI) factor of the PCG's
// factored preconditioner P = G^T G + eps D^{-1} (pcg.cuh: PcgFactor).
//
// Kolotilina and Yeremin's FSAI, in 3x3 blocks and in the
// block-Jacobi-normalised operator Â = C^{-1} A C^{-T} (A(i, i) = C(i) C(i)^T):
// for each vertex i, with P_i = {the kept lower neighbours j < i, then i},
//   Y = Â[P_i, P_i]^{-1} E_i       (E_i: the identity block of i)
//   Y(i) = L L^T                   (3x3 Cholesky of Y's block of i)
//   Ĝ(i, P_i) = L^{-1} Y^T,        so Ĝ(i, i) = L^T
// which makes (Ĝ Â Ĝ^T)(i, i) = I and (Ĝ Â)(i, j) = 0 for j in P_i, j != i.
// G = Ĝ C^{-1}. The reference has no such preconditioner; its PCG uses
// block-Jacobi (crates/ppf-cts-solver/src/cpp/solver/solver.cu:357-400), which
// stays the fallback of every factored solve.
//
// The pattern of row i is its lower neighbours in the operator (fixed
// pattern and contact blocks), Dirichlet vertices left out; rows with more
// than kFsaiMaxLower keep the strongest couplings by |Â(i, j)|_F (ties: the
// earlier in the row's transpose lists). One warp per row builds and solves
// the dense system (at most 48 x 48) in shared memory.
#pragma once

#include "pcg.cuh"
#include "precond.cuh"

namespace ppf {
namespace gpu {

constexpr int kFsaiMaxLower = 15;

// The assembled system as upper CSRs plus transpose lists (the solver's
// fixed pattern, diagonal included, and its contact blocks).
struct FsaiSystem {
    unsigned n;
    const unsigned *f_off, *f_col;
    const float *f_val;
    const unsigned *f_troff;
    const uint2 *f_tr;
    const unsigned *d_off, *d_col;
    const float *d_val;
    const unsigned *d_troff;
    const uint2 *d_tr;
    const unsigned *diag_slot, *dof_mask;
};

// Builds the FSAI factor of the operator A into F (after F.cinv holds C^{-1},
// launch_chol_inv): per-edge G(hi, lo) into F.edge_f / F.edge_d (indexed by
// the upper entries of the fixed and contact CSRs; dyn_cap = the contact
// CSR's capacity), the diagonal blocks into F.diag, then the factor's slot
// arrays through the slots' source maps. A row whose dense system is not
// positive definite keeps Ĝ(i, i) = I and no edges (block-Jacobi for that
// row) and sets STATUS_PRECOND_NONSPD.
void launch_factor_fsai(const PcgOperator &A, const FsaiSystem &S, unsigned nnz_fixed,
                        unsigned dyn_cap, const unsigned *fixed_src, const unsigned *dyn_src,
                        const unsigned *ovf_src, FactorBuffers &F, unsigned *d_status,
                        cudaStream_t q);

} // namespace gpu
} // namespace ppf
