// fsai.cu -- the FSAI factor of the PCG's factored preconditioner (fsai.cuh).
#include "fatal.cuh"
#include "fsai.cuh"
#include "learned.cuh"

namespace ppf {
namespace gpu {

namespace {

constexpr int kFsaiDim = 3 * (kFsaiMaxLower + 1); // 48
constexpr int kFsaiWarps = 4;                     // rows per block
constexpr unsigned kFsaiCand = 512;               // candidates a row considers
constexpr unsigned kT = 256;

__device__ __forceinline__ Mat3 ld9(const float *p) {
    Mat3 m;
#pragma unroll
    for (int e = 0; e < 9; ++e) m.m[e] = __ldg(p + e);
    return m;
}

__device__ __forceinline__ void st9(float *p, const Mat3 &m) {
#pragma unroll
    for (int e = 0; e < 9; ++e) p[e] = m.m[e];
}

// A(r, c), r < c, from the upper CSRs (zero when the two are not coupled).
__device__ Mat3 upper_block(const FsaiSystem &S, unsigned r, unsigned c) {
    for (unsigned p = __ldg(S.f_off + r), e = __ldg(S.f_off + r + 1); p < e; ++p)
        if (__ldg(S.f_col + p) == c) return ld9(S.f_val + 9 * (size_t)p);
    for (unsigned p = __ldg(S.d_off + r), e = __ldg(S.d_off + r + 1); p < e; ++p)
        if (__ldg(S.d_col + p) == c) return ld9(S.d_val + 9 * (size_t)p);
    return Mat3::zero();
}

// Candidate t of row i: the t-th lower neighbour in the fixed transpose list,
// then in the contact one: (neighbour r, upper entry p, contact part?).
struct Cand {
    unsigned r, p;
    bool contact;
};
__device__ __forceinline__ Cand cand_at(const FsaiSystem &S, unsigned i, unsigned nf,
                                        unsigned t) {
    if (t < nf) {
        const uint2 e = __ldg(S.f_tr + __ldg(S.f_troff + i) + t);
        return Cand{e.x, e.y, false};
    }
    const uint2 e = __ldg(S.d_tr + __ldg(S.d_troff + i) + (t - nf));
    return Cand{e.x, e.y, true};
}

// |Â(i, r)|_F of a candidate, or -1 for a Dirichlet neighbour.
__device__ __forceinline__ float cand_norm(const FsaiSystem &S, const float *cinv, unsigned i,
                                           const Mat3 &Ci, const Cand &c) {
    if (__ldg(S.dof_mask + c.r)) return -1.0f;
    const float *b = (c.contact ? S.d_val : S.f_val) + 9 * (size_t)c.p;
    return learned_fro(learned_edge_ahat(Ci, ld9(cinv + 9 * (size_t)c.r), ld9(b)));
}

// Marks the kept candidates of row i in sel (bits, candidate order): every
// non-Dirichlet candidate when there are at most kFsaiMaxLower, else the
// kFsaiMaxLower strongest (ties: the earlier candidate). Returns how many.
__device__ unsigned select_candidates(const FsaiSystem &S, const float *cinv, unsigned i,
                                      const Mat3 &Ci, unsigned nf, unsigned total,
                                      unsigned *sel, unsigned lane) {
    for (unsigned w = lane; w < kFsaiCand / 32; w += 32) sel[w] = 0u;
    __syncwarp();
    unsigned live = 0;
    for (unsigned t = lane; t < total; t += 32)
        live += cand_norm(S, cinv, i, Ci, cand_at(S, i, nf, t)) >= 0.0f ? 1u : 0u;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) live += __shfl_xor_sync(0xffffffffu, live, o);
    if (live <= (unsigned)kFsaiMaxLower) {
        for (unsigned t = lane; t < total; t += 32)
            if (cand_norm(S, cinv, i, Ci, cand_at(S, i, nf, t)) >= 0.0f)
                atomicOr(sel + t / 32, 1u << (t % 32));
        __syncwarp();
        return live;
    }
    for (int round = 0; round < kFsaiMaxLower; ++round) {
        float best = -1.0f;
        unsigned bt = 0xFFFFFFFFu;
        for (unsigned t = lane; t < total; t += 32) {
            if (sel[t / 32] & (1u << (t % 32))) continue;
            const float v = cand_norm(S, cinv, i, Ci, cand_at(S, i, nf, t));
            if (v > best) {
                best = v;
                bt = t;
            }
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const float ob = __shfl_xor_sync(0xffffffffu, best, o);
            const unsigned ot = __shfl_xor_sync(0xffffffffu, bt, o);
            if (ob > best || (ob == best && ot < bt)) {
                best = ob;
                bt = ot;
            }
        }
        __syncwarp();
        if (lane == 0 && bt != 0xFFFFFFFFu) sel[bt / 32] |= 1u << (bt % 32);
        __syncwarp();
    }
    return kFsaiMaxLower;
}

struct FsaiShared {
    float M[kFsaiDim][kFsaiDim + 1]; // Â[P, P], then its Cholesky factor
    float Y[kFsaiDim][3];            // Â[P, P]^{-1} E_i
    unsigned sel[kFsaiCand / 32];
    unsigned J[kFsaiMaxLower], E[kFsaiMaxLower]; // kept neighbours, their entries
};

// One warp per row i: G(i, j) for its kept lower neighbours into the edge
// arrays (entry | bit 31 for the contact part), G(i, i) into gdiag.
__global__ void __launch_bounds__(32 * kFsaiWarps)
    k_fsai(FsaiSystem S, const float *cinv, float *edge_f, float *edge_d, float *gdiag,
           unsigned *status) {
    __shared__ FsaiShared sh[kFsaiWarps];
    const unsigned lane = threadIdx.x & 31u, wi = threadIdx.x >> 5;
    const unsigned i = blockIdx.x * kFsaiWarps + wi;
    if (i >= S.n) return; // whole warps leave; the kernel has no block barrier
    FsaiShared &W = sh[wi];
    const Mat3 Ci = ld9(cinv + 9 * (size_t)i);
    if (__ldg(S.dof_mask + i)) {
        if (lane == 0) st9(gdiag + 9 * (size_t)i, Ci);
        return;
    }
    const unsigned nf = __ldg(S.f_troff + i + 1) - __ldg(S.f_troff + i);
    const unsigned nd = __ldg(S.d_troff + i + 1) - __ldg(S.d_troff + i);
    const unsigned total = min(nf + nd, kFsaiCand);
    select_candidates(S, cinv, i, Ci, nf, total, W.sel, lane);
    if (lane == 0) {
        unsigned m = 0;
        for (unsigned w = 0; w < (total + 31) / 32; ++w)
            for (unsigned bits = W.sel[w]; bits; bits &= bits - 1) {
                const unsigned t = 32 * w + (unsigned)(__ffs(bits) - 1);
                const Cand c = cand_at(S, i, nf, t);
                if (m < (unsigned)kFsaiMaxLower) {
                    W.J[m] = c.r;
                    W.E[m] = c.p | (c.contact ? kSlotTransposed : 0u);
                    ++m;
                }
            }
        W.sel[0] = m;
    }
    __syncwarp();
    const unsigned m = W.sel[0];
    const unsigned d = 3 * (m + 1);
    // Â[P, P], P = (J[0..m), i): block (a, b) for a <= b, both triangles
    const unsigned pairs = (m + 1) * (m + 2) / 2;
    for (unsigned q = lane; q < pairs; q += 32) {
        unsigned a = 0, rem = q;
        while (rem >= m + 1 - a) {
            rem -= m + 1 - a;
            ++a;
        }
        const unsigned b = a + rem;
        const unsigned va = a < m ? W.J[a] : i, vb = b < m ? W.J[b] : i;
        const Mat3 Ca = ld9(cinv + 9 * (size_t)va), Cb = ld9(cinv + 9 * (size_t)vb);
        Mat3 blk;
        if (a == b) {
            blk = (Ca * ld9(S.f_val + 9 * (size_t)__ldg(S.diag_slot + va))) * Ca.transpose();
        } else if (b == m) {
            // Â(j_a, i) = Â(i, j_a)^T from the row's own entry
            const unsigned e = W.E[a];
            const float *bp = ((e & kSlotTransposed) ? S.d_val : S.f_val) +
                              9 * (size_t)(e & ~kSlotTransposed);
            blk = learned_edge_ahat(Ci, Ca, ld9(bp)).transpose();
        } else {
            const Mat3 U = upper_block(S, min(va, vb), max(va, vb));
            const Mat3 Aab = va < vb ? U : U.transpose();
            blk = (Ca * Aab) * Cb.transpose();
        }
#pragma unroll
        for (int x = 0; x < 3; ++x)
#pragma unroll
            for (int y = 0; y < 3; ++y) {
                W.M[3 * a + x][3 * b + y] = blk(x, y);
                W.M[3 * b + y][3 * a + x] = blk(x, y);
            }
    }
    // Cholesky, lower, in place
    bool ok = true;
    for (unsigned k = 0; k < d; ++k) {
        __syncwarp();
        const float piv = W.M[k][k];
        if (!(piv > 0.0f) || !isfinite(piv)) {
            ok = false;
            break;
        }
        const float lkk = sqrtf(piv);
        __syncwarp();
        if (lane == 0) W.M[k][k] = lkk;
        for (unsigned r = k + 1 + lane; r < d; r += 32) W.M[r][k] = W.M[r][k] / lkk;
        __syncwarp();
        for (unsigned r = k + 1 + lane; r < d; r += 32) {
            const float lrk = W.M[r][k];
            for (unsigned c = k + 1; c <= r; ++c) W.M[r][c] = W.M[r][c] - lrk * W.M[c][k];
        }
    }
    __syncwarp();
    Mat3 Gii = Mat3::identity();
    if (ok) {
        // z = L^{-1} E_i (nonzero in the last three rows only), then L^T y = z
        for (unsigned r = lane; r < d; r += 32)
#pragma unroll
            for (int c = 0; c < 3; ++c) W.Y[r][c] = 0.0f;
        __syncwarp();
        if (lane < 3) {
            const unsigned c = lane, b0 = 3 * m;
            for (unsigned x = 0; x < 3; ++x) {
                float v = x == c ? 1.0f : 0.0f;
                for (unsigned y = 0; y < x; ++y) v = v - W.M[b0 + x][b0 + y] * W.Y[b0 + y][c];
                W.Y[b0 + x][c] = v / W.M[b0 + x][b0 + x];
            }
        }
        for (int k = (int)d - 1; k >= 0; --k) {
            __syncwarp();
            if (lane < 3) W.Y[k][lane] = W.Y[k][lane] / W.M[k][k];
            __syncwarp();
            for (int r = (int)lane; r < k; r += 32)
#pragma unroll
                for (int c = 0; c < 3; ++c) W.Y[r][c] = W.Y[r][c] - W.M[k][r] * W.Y[k][c];
        }
        __syncwarp();
        // Y(i) = L3 L3^T; Ĝ(i, P) = L3^{-1} Y^T
        Mat3 Yii;
#pragma unroll
        for (int x = 0; x < 3; ++x)
#pragma unroll
            for (int y = 0; y < 3; ++y)
                Yii(x, y) = 0.5f * (W.Y[3 * m + x][y] + W.Y[3 * m + y][x]);
        Mat3 L3inv;
        ok = chol_inv3(Yii, L3inv);
        if (ok) {
            Gii = L3inv * Yii;
            for (unsigned a = lane; a < m; a += 32) {
                Mat3 Yat;
#pragma unroll
                for (int x = 0; x < 3; ++x)
#pragma unroll
                    for (int y = 0; y < 3; ++y) Yat(x, y) = W.Y[3 * a + y][x];
                const unsigned va = W.J[a], e = W.E[a];
                const Mat3 G = (L3inv * Yat) * ld9(cinv + 9 * (size_t)va);
                float *dst = ((e & kSlotTransposed) ? edge_d : edge_f) +
                             9 * (size_t)(e & ~kSlotTransposed);
                st9(dst, G);
            }
        }
    }
    if (!ok) {
        Gii = Mat3::identity();
        if (lane == 0) atomicOr(status, STATUS_PRECOND_NONSPD);
    }
    if (lane == 0) st9(gdiag + 9 * (size_t)i, Gii * Ci);
}

// The factor's slot arrays from the per-edge values: a slot whose source bit
// says "transposed" lies in the edge's higher row and holds G(hi, lo); the
// other holds its transpose. Diagonal, padding and Dirichlet slots hold zero.
__global__ void k_fsai_fill_sell(SellMatrix M, unsigned rows, const unsigned *perm,
                                 const unsigned *src, const float *edge, const unsigned *dof,
                                 bf16_t *out) {
    const unsigned t = blockIdx.x * blockDim.x + threadIdx.x;
    const unsigned sl = t / kSliceRows, lane = t % kSliceRows;
    if (sl >= M.n_slices) return;
    const bool real = t < rows;
    const unsigned a = real ? (perm ? __ldg(perm + t) : t) : 0u;
    const bool live = real && __ldg(dof + a) == 0u;
    for (unsigned s = __ldg(M.slice_off + sl), s1 = __ldg(M.slice_off + sl + 1); s < s1; ++s) {
        const size_t idx = (size_t)s * kSliceRows + lane;
        Mat3 v = Mat3::zero();
        const unsigned sv = __ldg(src + idx), b = __ldg(M.col + idx);
        if (live && sv != kSlotPad && b != a && __ldg(dof + b) == 0u) {
            v = ld9(edge + 9 * (size_t)(sv & ~kSlotTransposed));
            if (!(sv & kSlotTransposed)) v = v.transpose();
        }
        bf16_t *d = out + (size_t)s * 9 * kSliceRows + lane;
#pragma unroll
        for (int e = 0; e < 9; ++e) d[e * kSliceRows] = __float2bfloat16_rn(v.m[e]);
    }
}

// One warp per overflow row: its entries, as k_fsai_fill_sell.
__global__ void k_fsai_fill_ovf(OverflowRows O, const unsigned *src, const float *edge,
                                const unsigned *dof, bf16_t *out) {
    const unsigned k = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31u;
    if (k >= O.count) return;
    const unsigned a = __ldg(O.row + k);
    const bool live = __ldg(dof + a) == 0u;
    const uint2 rg = __ldg(O.range + k);
    for (unsigned e = rg.x + lane; e < rg.x + rg.y; e += 32u) {
        Mat3 v = Mat3::zero();
        const unsigned sv = __ldg(src + e), b = __ldg(O.col + e);
        if (live && sv != kSlotPad && b != a && __ldg(dof + b) == 0u) {
            v = ld9(edge + 9 * (size_t)(sv & ~kSlotTransposed));
            if (!(sv & kSlotTransposed)) v = v.transpose();
        }
#pragma unroll
        for (int q = 0; q < 9; ++q) out[9 * (size_t)e + q] = __float2bfloat16_rn(v.m[q]);
    }
}

} // namespace

void launch_factor_fsai(const PcgOperator &A, const FsaiSystem &S, unsigned nnz_fixed,
                        unsigned dyn_cap, const unsigned *fixed_src, const unsigned *dyn_src,
                        const unsigned *ovf_src, FactorBuffers &F, unsigned *d_status,
                        cudaStream_t q) {
    F.edge_f.reserve(9 * (size_t)nnz_fixed + 1);
    F.edge_d.reserve(9 * (size_t)dyn_cap + 1);
    PPF_CUDA(cudaMemsetAsync(F.edge_f.data(), 0, 9 * (size_t)nnz_fixed * sizeof(float), q));
    PPF_CUDA(cudaMemsetAsync(F.edge_d.data(), 0, 9 * (size_t)dyn_cap * sizeof(float), q));
    if (!S.n) return;
    k_fsai<<<div_up(S.n, (unsigned)kFsaiWarps), 32 * kFsaiWarps, 0, q>>>(
        S, F.cinv.data(), F.edge_f.data(), F.edge_d.data(), F.diag.data(), d_status);
    PPF_LAUNCH_CHECK();
    if (A.fixed.n_slices) {
        k_fsai_fill_sell<<<div_up(A.fixed.n_slices * kSliceRows, kT), kT, 0, q>>>(
            A.fixed, A.n, nullptr, fixed_src, F.edge_f.data(), S.dof_mask, F.fixed.data());
        PPF_LAUNCH_CHECK();
    }
    if (A.contact.sell.n_slices) {
        k_fsai_fill_sell<<<div_up(A.contact.sell.n_slices * kSliceRows, kT), kT, 0, q>>>(
            A.contact.sell, A.contact.rows, A.contact.perm, dyn_src, F.edge_d.data(), S.dof_mask,
            F.contact.data());
        PPF_LAUNCH_CHECK();
    }
    if (A.ovf.count) {
        k_fsai_fill_ovf<<<div_up(A.ovf.count * 32u, kT), kT, 0, q>>>(
            A.ovf, ovf_src, F.edge_d.data(), S.dof_mask, F.ovf.data());
        PPF_LAUNCH_CHECK();
    }
}

} // namespace gpu
} // namespace ppf
