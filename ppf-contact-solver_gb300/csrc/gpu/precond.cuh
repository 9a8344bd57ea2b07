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

// Lower Cholesky factor L of a symmetric 3x3 block: inv = L^{-1}; false when
// a pivot is not positive.
__device__ __forceinline__ bool chol_inv3(const Mat3 &a, Mat3 &inv) {
    const float l00 = sqrtf(a(0, 0));
    const float l10 = a(1, 0) / l00, l20 = a(2, 0) / l00;
    const float d1 = a(1, 1) - l10 * l10;
    const float l11 = sqrtf(d1);
    const float l21 = (a(2, 1) - l20 * l10) / l11;
    const float d2 = a(2, 2) - l20 * l20 - l21 * l21;
    const float l22 = sqrtf(d2);
    if (!(a(0, 0) > 0.0f && d1 > 0.0f && d2 > 0.0f) || !isfinite(l22)) return false;
    const float i00 = 1.0f / l00, i11 = 1.0f / l11, i22 = 1.0f / l22;
    const float i10 = -l10 * i00 * i11;
    const float i21 = -l21 * i11 * i22;
    const float i20 = -(l20 * i00 + l21 * i10) * i22;
    inv = Mat3::zero();
    inv(0, 0) = i00;
    inv(1, 0) = i10;
    inv(1, 1) = i11;
    inv(2, 0) = i20;
    inv(2, 1) = i21;
    inv(2, 2) = i22;
    return true;
}

// Parallel value arrays of a factor (PcgFactor) plus the per-vertex C^{-1};
// edge_f / edge_d: per upper entry of the fixed / contact CSR, G(hi, lo)
// (FSAI only).
struct FactorBuffers {
    DevBuf<bf16_t> fixed, contact, ovf;
    DevBuf<float> diag, cinv, edge_f, edge_d;
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
