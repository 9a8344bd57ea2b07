// learned.cuh -- the learned factor of the PCG preconditioner.
//
// A message-passing network over the Newton system's own sparsity (the fixed
// elastic pattern plus the contact blocks) emits the factor of
//   P = G^T G + eps D^{-1},   G = Ĝ C^{-1},   A(i, i) = C(i) C(i)^T,
// on A's pattern (pcg.cuh: PcgFactor), in the block-Jacobi-normalised
// operator Â = C^{-1} A C^{-T}:
//   Ĝ(i, i)   = d_i I,               d_i = exp(clamp(Y[i, 64], -4, 4))
//   Ĝ(hi, lo) = -alpha_e Â(hi, lo),  alpha_e = 2 sigmoid(o_e)
// The reference has no learned preconditioner; its PCG uses block-Jacobi
// (crates/ppf-cts-solver/src/cpp/solver/solver.cu:357-400), which stays the
// fallback of every factored solve.
//
// Network (hidden width 32, bf16 weights, fp32 accumulation on the tensor
// cores: the forward layers as tcgen05.mma tiles with tensor-memory
// accumulators, the backward products as mma.sync m16n8k16 tiles; every
// layer input carries a constant-1 column holding the bias):
//   X0 = [node features, 1]                    n x 16  (k_node_inputs)
//   H0 = bf16(relu(X0 W0^T))                   n x 32
//   Xl = [H, bf16(mean_nbr H), 1, 0..]          n x 80  (k_aggregate)
//   Hl = bf16(relu(Xl Wl^T)),  l = 1..3
//   Xh = [H3, 1, 0..]                          n x 48
//   Y  = Xh Wh^T (fp32)                        n x 80: P1 | P2 | q
//   edge (hi > lo): f = bf16([Â(hi, lo), |Â(hi, lo)|_F, 1, 0..])      16
//                   z = relu(Y[hi, 0:32] + Y[lo, 32:64] + Wf f)
//                   o = wo . [z, 1]
// The edge head is evaluated per slot by the factor kernels (precond.cu) and
// per edge by the trainer, through the one function below, so both slots of
// an edge and the trained and applied factors carry the same bits.
#pragma once

#include <cuda_bf16.h>

#include "common.cuh"

namespace ppf {
namespace gpu {

namespace learned {
constexpr unsigned kHidden = 32;
constexpr unsigned kIn0 = 16, kInL = 80, kInH = 48, kOutH = 80, kInF = 16;
// flat weight blob, row-major [out][in] matrices
constexpr unsigned kOffW0 = 0;                        // 32 x 16
constexpr unsigned kOffW1 = 512;                      // 3 x (32 x 80)
constexpr unsigned kOffWh = kOffW1 + 3 * 32 * kInL;   // 80 x 48
constexpr unsigned kOffWf = kOffWh + kOutH * kInH;    // 32 x 16
constexpr unsigned kOffWo = kOffWf + 32 * kInF;       // 48
constexpr unsigned kWeights = kOffWo + 48;            // 12592
constexpr float kClampQ = 4.0f;
static_assert(kWeights == 12592, "weight blob layout");
} // namespace learned

typedef __nv_bfloat16 bf16_t;

// One part of the system (fixed pattern or contact blocks) as an upper CSR
// with 9 column-major floats per block, plus its transpose list: for vertex
// c, tr[tr_off[c] .. tr_off[c+1]) = (row, slot) of the upper entries (row, c),
// row != c.
struct LearnedPart {
    const unsigned *off, *col;
    const float *val;
    const unsigned *tr_off;
    const uint2 *tr;
    unsigned nnz;
};

struct LearnedGraph {
    unsigned n;
    LearnedPart fixed, contact;
    const unsigned *diag_slot; // slot of A(i, i) in the fixed part
    const unsigned *dof_mask;  // nonzero: Dirichlet vertex (left out)
    const float *mass;
    const float *cinv; // C(i)^{-1}, 9 column-major floats per vertex
};

// Per-vertex arrays of one forward pass.
struct LearnedNodes {
    DevBuf<bf16_t> X0, H, X, Xh; // H: 4 layers x n x 32
    DevBuf<float> deg, Y;
    void reserve(unsigned n);
};

// Runs the vertex part of the network on g: features, the four layers and
// the head, leaving Y (n x 80, fp32) in b.Y. w: the bf16 weight blob.
void learned_forward_nodes(const LearnedGraph &g, const bf16_t *w, LearnedNodes &b,
                           cudaStream_t q);

// Â(hi, lo) = (C_hi A(hi, lo)) C_lo^T with A(hi, lo) = the upper block B^T.
__device__ __forceinline__ Mat3 learned_edge_ahat(const Mat3 &Chi, const Mat3 &Clo,
                                                  const Mat3 &B) {
    return (Chi * B.transpose()) * Clo.transpose();
}

__device__ __forceinline__ float learned_fro(const Mat3 &m) {
    float acc = 0.0f;
#pragma unroll
    for (int e = 0; e < 9; ++e) acc = acc + m.m[e] * m.m[e];
    return sqrtf(acc);
}

// Edge features f (bf16-rounded, as floats): Â(hi, lo) column-major, its
// Frobenius norm, the bias 1.
__device__ __forceinline__ void learned_edge_features(const Mat3 &ah, float (&f)[11]) {
#pragma unroll
    for (int e = 0; e < 9; ++e) f[e] = __bfloat162float(__float2bfloat16_rn(ah.m[e]));
    f[9] = __bfloat162float(__float2bfloat16_rn(learned_fro(ah)));
    f[10] = 1.0f;
}

// z_k (k < 32) of the edge head and its output o.
__device__ __forceinline__ float learned_edge_z(const float *Y, const bf16_t *w, unsigned hi,
                                                unsigned lo, const float (&f)[11], int k) {
    using namespace learned;
    const bf16_t *wf = w + kOffWf + k * kInF;
    float t = 0.0f;
#pragma unroll
    for (int c = 0; c < 11; ++c) t = t + __bfloat162float(wf[c]) * f[c];
    const float a = (__ldg(Y + (size_t)hi * kOutH + k) + __ldg(Y + (size_t)lo * kOutH + 32 + k)) + t;
    return fmaxf(a, 0.0f);
}

__device__ __forceinline__ float learned_edge_o(const float *Y, const bf16_t *w, unsigned hi,
                                                unsigned lo, const Mat3 &ah) {
    using namespace learned;
    float f[11];
    learned_edge_features(ah, f);
    float o = 0.0f;
    for (int k = 0; k < 32; ++k)
        o = o + __bfloat162float(w[kOffWo + k]) * learned_edge_z(Y, w, hi, lo, f, k);
    return o + __bfloat162float(w[kOffWo + 32]);
}

__device__ __forceinline__ float learned_alpha_of(float o) { return 2.0f / (1.0f + expf(-o)); }

__device__ __forceinline__ float learned_diag_scale(const float *Y, unsigned i) {
    const float q = __ldg(Y + (size_t)i * learned::kOutH + 64);
    return expf(fminf(fmaxf(q, -learned::kClampQ), learned::kClampQ));
}

// Trainer entry points (api in learned.cu): samples kept on the device.
int learned_add_sample(unsigned n, const unsigned *f_off, const unsigned *f_col,
                       const float *f_val, const unsigned *c_off, const unsigned *c_col,
                       const float *c_val, const unsigned *dof_mask, const float *mass);
void learned_clear_samples();
// Selects the forward layers' tensor-core path (1: tcgen05, 0: mma.sync; -1
// only reads it); returns the previous one.
int learned_tensor_path(int tc);
// Nonzero once a tcgen05 tile gave up waiting for its accumulator.
unsigned learned_tc_status();
int learned_sample_info(int s, unsigned *n, unsigned *edges, unsigned *n_free);
int learned_forward(int s, const bf16_t *d_w, float *h_alpha, float *h_d);
int learned_loss_grad(int s, const bf16_t *d_w, const float *d_probes, unsigned n_probes,
                      float *d_grad, float *h_loss, cudaStream_t q);

} // namespace gpu
} // namespace ppf
