// precond.cuh -- the factored preconditioner P = G^T G + eps D^{-1} of the
// PCG (pcg.cuh: PcgFactor), on the operator's own pattern.
//
// Everything is expressed in the block-Jacobi-normalised operator
//   Â = C^{-1} A C^{-T},  A(i, i) = C(i) C(i)^T  (lower Cholesky factor),
// whose diagonal blocks are the identity. A factor Ĝ (block lower
// triangular, Ĝ(i, i) lower triangular) defines G = Ĝ C^{-1}, so that
// G A G^T = Ĝ Â Ĝ^T and Ĝ = I gives back block-Jacobi.
//
// For an edge between vertices hi > lo, Ĝ(hi, lo) is a function of the
// ordered pair and of Â(hi, lo) only. Both slots of the edge (row hi, column
// lo and row lo, column hi) evaluate it from bit-identical inputs (the stored
// blocks are exact transposes), so y = G r and z = G^T y use the same G.
#pragma once

#include "learned.cuh"
#include "pcg.cuh"
#include "scene.cuh"

namespace ppf {
namespace gpu {

// Parallel value arrays of a factor (PcgFactor) plus the per-vertex C^{-1}.
struct FactorBuffers {
    DevBuf<float> fixed, contact, ovf, diag, cinv;
    PcgFactor view(float eps) const {
        return PcgFactor{fixed.data(), contact.data(), ovf.data(), diag.data(), eps};
    }
};

// C(i)^{-1} (column-major, lower triangular) of every diagonal block; a
// non-positive pivot latches STATUS_PRECOND_NONSPD and falls back to the
// inverse square root of the block's diagonal.
void launch_chol_inv(unsigned n, const float *upper_val, const unsigned *diag_slot, float *cinv,
                     unsigned *d_status, cudaStream_t q);

// The first-order factor Ĝ(i, i) = I, Ĝ(hi, lo) = -alpha Â(hi, lo): with
// alpha = 1/2 it halves the block-Jacobi iteration count on contact-coupled
// cloth systems. Sizes the factor's arrays to the operator.
void launch_factor_first_order(const PcgOperator &A, const unsigned *dof_mask, float alpha,
                               FactorBuffers &F, cudaStream_t q);

// The learned factor: Ĝ from the network's head output Y (n x 80) and its
// bf16 weights w (learned.cuh), on the same slots as the first-order one.
void launch_factor_learned(const PcgOperator &A, const unsigned *dof_mask, const float *Y,
                           const bf16_t *w, FactorBuffers &F, cudaStream_t q);

// Sizes F's value arrays to A's (fixed slots, contact slots, overflow
// entries, vertices).
void reserve_factor(const PcgOperator &A, unsigned fixed_slots, unsigned contact_slots,
                    unsigned ovf_entries, FactorBuffers &F);

} // namespace gpu
} // namespace ppf
