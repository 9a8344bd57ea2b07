// precond.cu -- factor arrays of the PCG's factored preconditioner.
#include "../physics/linalg.cuh"
#include "fatal.cuh"
#include "precond.cuh"

namespace ppf {
namespace gpu {

namespace {

constexpr unsigned kT = 256;

__device__ __forceinline__ Mat3 ld_mat3(const float *p) {
    Mat3 m;
#pragma unroll
    for (int e = 0; e < 9; ++e) m.m[e] = __ldg(p + e);
    return m;
}
__device__ __forceinline__ void st_mat3(float *p, const Mat3 &m) {
#pragma unroll
    for (int e = 0; e < 9; ++e) p[e] = m.m[e];
}

__global__ void k_chol_inv(unsigned n, const float *upper_val, const unsigned *diag_slot,
                           float *cinv, unsigned *status) {
    const unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const Mat3 a = ld_mat3(upper_val + 9 * (size_t)__ldg(diag_slot + i));
    Mat3 c;
    if (!chol_inv3(a, c)) {
        atomicOr(status, STATUS_PRECOND_NONSPD);
        c = Mat3::zero();
        for (int k = 0; k < 3; ++k) c(k, k) = 1.0f / sqrtf(fmaxf(fabsf(a(k, k)), 1e-30f));
    }
    st_mat3(cinv + 9 * (size_t)i, c);
}

// Ĝ of the first-order rule.
struct FirstOrderHead {
    float alpha;
    __device__ __forceinline__ Mat3 edge(unsigned, unsigned, const Mat3 &ah) const {
        return (-alpha) * ah;
    }
    __device__ __forceinline__ Mat3 diag(unsigned) const { return Mat3::identity(); }
};

// Ĝ emitted by the learned network (learned.cuh): the edge head evaluated on
// the slot's own Â(hi, lo), the vertex scale d_i from the head's output Y.
struct LearnedHead {
    const float *Y;
    const bf16_t *w;
    __device__ __forceinline__ Mat3 edge(unsigned hi, unsigned lo, const Mat3 &ah) const {
        return (-learned_alpha_of(learned_edge_o(Y, w, hi, lo, ah))) * ah;
    }
    __device__ __forceinline__ Mat3 diag(unsigned i) const {
        return learned_diag_scale(Y, i) * Mat3::identity();
    }
};

// The factor value of one slot of row a holding the operator block B =
// A(a, b): G(a, b) for b < a, G(b, a)^T for b > a, zero on the diagonal, for
// padding and for Dirichlet vertices.
template <class Head>
__device__ __forceinline__ Mat3 slot_value(unsigned a, unsigned b, const Mat3 &B,
                                           const Mat3 &Ca, const unsigned *dof_mask,
                                           const float *cinv, const Head &head) {
    if (b == a || __ldg(dof_mask + b) != 0u) return Mat3::zero();
    const bool lower = b < a;
    const Mat3 Cb = ld_mat3(cinv + 9 * (size_t)b);
    const unsigned hi = lower ? a : b, lo = lower ? b : a;
    const Mat3 Ahl = lower ? B : B.transpose();
    const Mat3 &Chi = lower ? Ca : Cb;
    const Mat3 &Clo = lower ? Cb : Ca;
    const Mat3 ah = (Chi * Ahl) * Clo.transpose();
    const Mat3 G = head.edge(hi, lo, ah) * Clo;
    return lower ? G : G.transpose();
}

// One thread per (slice, lane) of a SELL part: every slot of its row.
template <class Head>
__global__ void k_factor_sell(SellMatrix M, unsigned rows, const unsigned *perm,
                              const unsigned *dof_mask, const float *cinv, Head head,
                              bf16_t *out) {
    const unsigned t = blockIdx.x * blockDim.x + threadIdx.x;
    const unsigned sl = t / kSliceRows, lane = t % kSliceRows;
    if (sl >= M.n_slices) return;
    const bool real = t < rows;
    const unsigned a = real ? (perm ? __ldg(perm + t) : t) : 0u;
    const bool live = real && __ldg(dof_mask + a) == 0u;
    const Mat3 Ca = live ? ld_mat3(cinv + 9 * (size_t)a) : Mat3::zero();
    const unsigned s0 = __ldg(M.slice_off + sl), s1 = __ldg(M.slice_off + sl + 1);
    for (unsigned s = s0; s < s1; ++s) {
        const size_t base = (size_t)s * 9 * kSliceRows + lane;
        Mat3 v = Mat3::zero();
        if (live) {
            const unsigned b = __ldg(M.col + (size_t)s * kSliceRows + lane);
            Mat3 B;
#pragma unroll
            for (int e = 0; e < 9; ++e) B.m[e] = __ldg(M.val + base + e * kSliceRows);
            v = slot_value(a, b, B, Ca, dof_mask, cinv, head);
        }
#pragma unroll
        for (int e = 0; e < 9; ++e) out[base + e * kSliceRows] = __float2bfloat16_rn(v.m[e]);
    }
}

// One warp per overflow row: every entry of it.
template <class Head>
__global__ void k_factor_ovf(OverflowRows O, const unsigned *dof_mask, const float *cinv,
                             Head head, bf16_t *out) {
    const unsigned k = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31u;
    if (k >= O.count) return;
    const unsigned a = __ldg(O.row + k);
    const bool live = __ldg(dof_mask + a) == 0u;
    const Mat3 Ca = live ? ld_mat3(cinv + 9 * (size_t)a) : Mat3::zero();
    const uint2 rg = __ldg(O.range + k);
    for (unsigned e = rg.x + lane; e < rg.x + rg.y; e += 32u) {
        Mat3 v = Mat3::zero();
        if (live) v = slot_value(a, __ldg(O.col + e), ld_mat3(O.val + 9 * (size_t)e), Ca,
                                 dof_mask, cinv, head);
#pragma unroll
        for (int q = 0; q < 9; ++q) out[9 * (size_t)e + q] = __float2bfloat16_rn(v.m[q]);
    }
}

template <class Head>
__global__ void k_factor_diag(unsigned n, const unsigned *dof_mask, const float *cinv, Head head,
                              float *diag) {
    const unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const Mat3 C = ld_mat3(cinv + 9 * (size_t)i);
    const Mat3 g = __ldg(dof_mask + i) ? C : head.diag(i) * C;
    st_mat3(diag + 9 * (size_t)i, g);
}

template <class Head>
void launch_factor(const PcgOperator &A, const unsigned *dof_mask, const Head &head,
                   FactorBuffers &F, cudaStream_t q) {
    const float *cinv = F.cinv.data();
    if (A.fixed.n_slices) {
        k_factor_sell<<<div_up(A.fixed.n_slices * kSliceRows, kT), kT, 0, q>>>(
            A.fixed, A.n, nullptr, dof_mask, cinv, head, F.fixed.data());
        PPF_LAUNCH_CHECK();
    }
    if (A.contact.sell.n_slices) {
        k_factor_sell<<<div_up(A.contact.sell.n_slices * kSliceRows, kT), kT, 0, q>>>(
            A.contact.sell, A.contact.rows, A.contact.perm, dof_mask, cinv, head,
            F.contact.data());
        PPF_LAUNCH_CHECK();
    }
    if (A.ovf.count) {
        k_factor_ovf<<<div_up(A.ovf.count * 32u, kT), kT, 0, q>>>(A.ovf, dof_mask, cinv, head,
                                                                  F.ovf.data());
        PPF_LAUNCH_CHECK();
    }
    k_factor_diag<<<div_up(A.n, kT), kT, 0, q>>>(A.n, dof_mask, cinv, head, F.diag.data());
    PPF_LAUNCH_CHECK();
}

} // namespace

void launch_chol_inv(unsigned n, const float *upper_val, const unsigned *diag_slot, float *cinv,
                     unsigned *d_status, cudaStream_t q) {
    k_chol_inv<<<div_up(n, kT), kT, 0, q>>>(n, upper_val, diag_slot, cinv, d_status);
    PPF_LAUNCH_CHECK();
}

void reserve_factor(const PcgOperator &A, unsigned fixed_slots, unsigned contact_slots,
                    unsigned ovf_entries, FactorBuffers &F) {
    F.fixed.reserve(9 * (size_t)kSliceRows * fixed_slots + 1);
    F.contact.reserve(9 * (size_t)kSliceRows * contact_slots + 1);
    F.ovf.reserve(9 * (size_t)ovf_entries + 1);
    F.diag.reserve(9 * (size_t)A.n);
    F.cinv.reserve(9 * (size_t)A.n);
}

void launch_factor_first_order(const PcgOperator &A, const unsigned *dof_mask, float alpha,
                               FactorBuffers &F, cudaStream_t q) {
    launch_factor(A, dof_mask, FirstOrderHead{alpha}, F, q);
}

void launch_factor_learned(const PcgOperator &A, const unsigned *dof_mask, const float *Y,
                           const bf16_t *w, FactorBuffers &F, cudaStream_t q) {
    launch_factor(A, dof_mask, LearnedHead{Y, w}, F, q);
}

} // namespace gpu
} // namespace ppf
