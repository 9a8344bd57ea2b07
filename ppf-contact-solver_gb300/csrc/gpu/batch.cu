// batch.cu -- many independent Newton systems solved by block-Jacobi PCG in
// one launch.
//
// Small scenes (a few hundred to ten thousand vertices) leave a whole-GPU
// persistent PCG idle: its grid barriers cost more than the products. Here
// one CTA of 512 threads owns one system and runs the reference's
// block-Jacobi PCG on it (crates/ppf-cts-solver/src/cpp/solver/solver.cu:
// 357-400, 431-571, 1002-1278: x0 = 0, L1 residual against the seeded one,
// checks at iterations 1, 5, 9, ... and at every iteration once below 8 tol,
// the 256 eps curvature verdict) with block barriers only, so every system
// converges on its own schedule and hundreds of uneven systems share one
// launch. Rows are strided over the CTA's threads; sums fold in a fixed
// order, so a system's result does not depend on the others in the launch.
#include <algorithm>
#include <numeric>
#include <vector>

#include "../../../include/ppf_gb300_ext.h"
#include "../physics/eig.cuh"
#include "common.cuh"
#include "fatal.cuh"
#include "precond.cuh"

#include <cooperative_groups.h>

namespace ppf {
namespace gpu {
namespace {

namespace cg = cooperative_groups;

// Threads per CTA of a team. 512: two CTAs share an SM, and a small
// system's iteration is shorter than on 1024 (the 256 uneven drops, one
// launch per system: 578 against 751 ms).
constexpr unsigned kBT = 512;
// Rows of the first size bucket (then doubling).
constexpr unsigned kBucketRows = 1024;
constexpr float kSlack = 256.0f;
constexpr float kEps = 1.19209290e-7f;

struct BatchArgs {
    unsigned base;             // first system of this launch
    const unsigned *order;     // null, or the system of each CTA (largest first)
    const unsigned *row_off;   // systems + 1: vertex rows of each system
    const unsigned *off;       // rows + 1: both-triangle block rows
    const unsigned *col;       // global row of each block's column
    const float *val;          // 9 per block, column-major
    // the same blocks sliced for the products (SELL-32): each system's rows
    // in slices of 32 from its first row, block k of row i at rbase[i] +
    // 32 k; entry e of the 32 blocks at 32 m .. 32 m + 31 at 32 (9 m + e) ..
    // 32 (9 m + e) + 31, so a warp's 32 rows read each entry coalesced
    const unsigned *rbase;     // rows: SELL position of the row's first block
    const unsigned *scol;      // SELL: global row of each block's column
    const float *sval;         // SELL: 9 per block, entry-interleaved
    const float *b;            // 3 per row
    float *x, *r, *z, *p, *Ap; // 3 per row
    float *inv;                // 9 per row: inverse of the diagonal block
    // FSAI factor (null: block-Jacobi): per block slot G(i, j) for j < i and
    // G(j, i)^T for j > i (bf16, SELL positions as sval), per row G(i, i)
    // (fp32); y: 3 per row
    const bf16_t *gval;
    const float *gdiag;
    float *y;
    float eps;
    float tol;
    unsigned max_iter;
    unsigned *iters;
    float *resid;
    int *state;
};

__device__ __forceinline__ Vec3 ld3(const float *v, unsigned i) {
    return vec3(v[3 * i], v[3 * i + 1], v[3 * i + 2]);
}
__device__ __forceinline__ void st3v(float *v, unsigned i, const Vec3 &a) {
    v[3 * i] = a[0];
    v[3 * i + 1] = a[1];
    v[3 * i + 2] = a[2];
}
__device__ __forceinline__ Mat3 ldm(const float *p) {
    Mat3 m;
#pragma unroll
    for (int e = 0; e < 9; ++e) m.m[e] = __ldg(p + e);
    return m;
}
// block q of a SELL-32 value array (entry-interleaved in groups of 32)
__device__ __forceinline__ size_t sell_at(unsigned q, int e) {
    return ((size_t)(q >> 5) * 9 + e) * 32 + (q & 31u);
}
__device__ __forceinline__ Mat3 ldm_sell(const float *v, unsigned q) {
    Mat3 m;
#pragma unroll
    for (int e = 0; e < 9; ++e) m.m[e] = __ldg(v + sell_at(q, e));
    return m;
}
__device__ __forceinline__ Mat3 ldm_sell(const bf16_t *v, unsigned q) {
    Mat3 m;
#pragma unroll
    for (int e = 0; e < 9; ++e) m.m[e] = __bfloat162float(__ldg(v + sell_at(q, e)));
    return m;
}

// The team that solves one system: one CTA (kCluster false; block barriers)
// or a thread-block cluster (kCluster true; cluster barriers and the CTAs'
// partial sums read through distributed shared memory). Rows are strided
// over the team's threads. Sums fold in a fixed order, so every thread of
// the team gets the same bits.
template <bool kCluster> struct Team {
    unsigned rank = 0, size = 1;
    __device__ Team() {
        if (kCluster) {
            cg::cluster_group cl = cg::this_cluster();
            rank = cl.block_rank();
            size = cl.num_blocks();
        }
    }
    __device__ __forceinline__ void sync() const {
        if (kCluster) cg::this_cluster().sync();
        else __syncthreads();
    }
    __device__ __forceinline__ unsigned first(unsigned lo) const {
        return lo + rank * kBT + threadIdx.x;
    }
    __device__ __forceinline__ unsigned stride() const { return size * kBT; }
    // a vector entry another thread of the team may have written: through L2
    // when that thread can sit on another SM
    __device__ __forceinline__ Vec3 ld_shared_vec(const float *v, unsigned i) const {
        if (kCluster) return vec3(__ldcg(v + 3 * i), __ldcg(v + 3 * i + 1), __ldcg(v + 3 * i + 2));
        return vec3(v[3 * i], v[3 * i + 1], v[3 * i + 2]);
    }
    // team-wide (a, b); `part` is a double-buffered per-CTA slot, `k` the
    // buffer (alternating between calls, so one barrier per sum suffices)
    __device__ float2 sum2(float a, float b, float2 *sh, float2 *part, unsigned k) const {
        for (int o = 16; o > 0; o >>= 1) {
            a += __shfl_xor_sync(0xffffffffu, a, o);
            b += __shfl_xor_sync(0xffffffffu, b, o);
        }
        if ((threadIdx.x & 31u) == 0) sh[threadIdx.x >> 5] = make_float2(a, b);
        __syncthreads();
        float2 t = make_float2(0.0f, 0.0f);
        for (unsigned w = 0; w < kBT / 32; ++w) {
            t.x += sh[w].x;
            t.y += sh[w].y;
        }
        if (!kCluster) {
            __syncthreads();
            return t;
        }
        if (threadIdx.x == 0) part[k] = t;
        cg::cluster_group cl = cg::this_cluster();
        cl.sync();
        float2 u = make_float2(0.0f, 0.0f);
        for (unsigned r = 0; r < size; ++r) {
            const float2 v = *cl.map_shared_rank(part + k, r);
            u.x += v.x;
            u.y += v.y;
        }
        return u;
    }
};

// The FSAI preconditioner P = G^T G + eps D^{-1} (the factored preconditioner
// of pcg.cuh, on the batch's full rows) in two passes with a team barrier
// between them: y = G r over the slots left of the diagonal (factor_y), then
// z = G^T y + eps D^{-1} r over the slots right of it (factor_z). Between
// exact passes the update phase carries y by y -= alpha G A p, which needs
// no barrier of its own (A p is final team-wide once p^T A p is summed); the
// exact pass runs every kYRefresh iterations to bound the drift.
constexpr unsigned kYRefresh = 16;

// acc + the sum over row i's slots left of the diagonal (they come first:
// columns sorted) of G(i, j) v_j; the next slot's column loads one slot
// ahead.
template <bool kCluster>
__device__ __forceinline__ Vec3 lower_product(const BatchArgs &g, const Team<kCluster> &team,
                                              unsigned i, const float *v, Vec3 acc) {
    const unsigned len = __ldg(g.off + i + 1) - __ldg(g.off + i), q0 = __ldg(g.rbase + i);
    unsigned j = len ? __ldg(g.scol + q0) : i;
    for (unsigned k = 0; k < len && j < i; ++k) {
        const unsigned q = q0 + 32u * k;
        const unsigned jn = k + 1 < len ? __ldg(g.scol + q + 32u) : i;
        acc += ldm_sell(g.gval, q) * team.ld_shared_vec(v, j);
        j = jn;
    }
    return acc;
}

// y = G r of this thread's rows (every r final).
template <bool kCluster>
__device__ void factor_y(const BatchArgs &g, const Team<kCluster> &team, unsigned i0, unsigned di,
                         unsigned hi) {
    for (unsigned i = i0; i < hi; i += di)
        st3v(g.y, i, lower_product(g, team, i, g.r, ldm(g.gdiag + 9 * (size_t)i) * ld3(g.r, i)));
}

// z = G^T y + eps D^{-1} r of this thread's rows (every y final); writes
// p = z too when set_p; returns their part of r^T z.
template <bool kCluster>
__device__ float factor_z(const BatchArgs &g, const Team<kCluster> &team, unsigned i0, unsigned di,
                          unsigned hi, bool set_p) {
    float a = 0.0f;
    for (unsigned i = i0; i < hi; i += di) {
        const Vec3 ri = ld3(g.r, i);
        Mat3 P;
#pragma unroll
        for (int q = 0; q < 9; ++q) P.m[q] = g.inv[9 * (size_t)i + q];
        Vec3 zi = ldm(g.gdiag + 9 * (size_t)i).transpose() * ld3(g.y, i);
        const unsigned len = __ldg(g.off + i + 1) - __ldg(g.off + i), q0 = __ldg(g.rbase + i);
        unsigned j = len ? __ldg(g.scol + q0) : 0u;
        for (unsigned k = 0; k < len; ++k) {
            const unsigned q = q0 + 32u * k;
            const unsigned jn = k + 1 < len ? __ldg(g.scol + q + 32u) : 0u;
            if (j > i) zi += ldm_sell(g.gval, q) * team.ld_shared_vec(g.y, j);
            j = jn;
        }
        zi += g.eps * (P * ri);
        st3v(g.z, i, zi);
        if (set_p) st3v(g.p, i, zi);
        a += ri.dot(zi);
    }
    return a;
}

// One system per team: team t (CTA, or cluster of CTAs) takes system
// order[t] (base + t without an order).
template <bool kCluster>
__global__ void __launch_bounds__(kBT) k_batch_pcg(BatchArgs g) {
    __shared__ float2 sh[kBT / 32];
    __shared__ float2 part[2];
    const Team<kCluster> team;
    const unsigned t_idx = blockIdx.x / team.size;
    const unsigned s = g.order ? __ldg(g.order + t_idx) : g.base + t_idx;
    const unsigned lo = __ldg(g.row_off + s), hi = __ldg(g.row_off + s + 1);
    const unsigned i0 = team.first(lo), di = team.stride();
    unsigned k = 0;
    // x0 = 0, r = b, block-Jacobi inverse, z = P r, p = z
    float a = 0.0f, e = 0.0f;
    for (unsigned i = i0; i < hi; i += di) {
        Mat3 d = Mat3::identity();
        for (unsigned q = __ldg(g.off + i), q1 = __ldg(g.off + i + 1); q < q1; ++q)
            if (__ldg(g.col + q) == i) d = ldm(g.val + 9 * (size_t)q);
        Mat3 P;
        if (!eig::invert_spd(d, P)) P = Mat3::identity();
#pragma unroll
        for (int q = 0; q < 9; ++q) g.inv[9 * (size_t)i + q] = P.m[q];
        const Vec3 bi = vec3(__ldg(g.b + 3 * i), __ldg(g.b + 3 * i + 1), __ldg(g.b + 3 * i + 2));
        st3v(g.x, i, Vec3::zero());
        st3v(g.r, i, bi);
        if (!g.gval) {
            const Vec3 zi = P * bi;
            st3v(g.z, i, zi);
            st3v(g.p, i, zi);
            a += bi.dot(zi);
        }
        e += fabsf(bi[0]) + fabsf(bi[1]) + fabsf(bi[2]);
    }
    if (g.gval) {
        team.sync();
        factor_y(g, team, i0, di, hi);
        team.sync();
        a = factor_z(g, team, i0, di, hi, true);
    }
    float2 t = team.sum2(a, e, sh, part, k);
    k ^= 1u;
    float rz = t.x;
    const float err0 = t.y;
    if (err0 == 0.0f) {
        if (team.rank == 0 && threadIdx.x == 0) {
            g.iters[s] = 0;
            g.resid[s] = 0.0f;
            g.state[s] = 0;
        }
        team.sync(); // no CTA leaves while another may still read its partials
        return;
    }
    unsigned stride = 4, next_check = 1;
    int broke = 0;
    for (unsigned iter = 1;; ++iter) {
        // A p, p^T A p and its round-off scale
        a = e = 0.0f;
        for (unsigned i = i0; i < hi; i += di) {
            Vec3 acc = Vec3::zero(), ab = Vec3::zero();
            const unsigned len = __ldg(g.off + i + 1) - __ldg(g.off + i), q0 = __ldg(g.rbase + i);
            for (unsigned k = 0; k < len; ++k) {
                const unsigned q = q0 + 32u * k;
                const float *m = g.sval + sell_at(q, 0); // entry e at m + 32 e
                const Vec3 v = team.ld_shared_vec(g.p, __ldg(g.scol + q));
                Vec3 term;
                term[0] = __ldg(m + 0) * v[0] + __ldg(m + 96) * v[1] + __ldg(m + 192) * v[2];
                term[1] = __ldg(m + 32) * v[0] + __ldg(m + 128) * v[1] + __ldg(m + 224) * v[2];
                term[2] = __ldg(m + 64) * v[0] + __ldg(m + 160) * v[1] + __ldg(m + 256) * v[2];
                acc += term;
                ab += term.cwise_abs();
            }
            const Vec3 pi = ld3(g.p, i);
            st3v(g.Ap, i, acc);
            a += pi.dot(acc);
            e += fabsf(pi[0]) * ab[0] + fabsf(pi[1]) * ab[1] + fabsf(pi[2]) * ab[2];
        }
        t = team.sum2(a, e, sh, part, k);
        k ^= 1u;
        const float pAp = t.x, bound = kSlack * kEps * t.y;
        float alpha = 0.0f;
        if (pAp > bound) {
            alpha = rz / pAp;
        } else if (!broke) {
            broke = (pAp < -bound || pAp != pAp) ? 1 : 3;
        }
        // x += alpha p, r -= alpha A p, z = P r (rows of this thread only);
        // with the FSAI factor y -= alpha G A p, or the exact y below
        const bool exact_y = iter % kYRefresh == 0;
        a = e = 0.0f;
        for (unsigned i = i0; i < hi; i += di) {
            Vec3 xi = ld3(g.x, i), ri = ld3(g.r, i);
            const Vec3 pi = ld3(g.p, i), api = ld3(g.Ap, i);
            for (int c = 0; c < 3; ++c) {
                xi[c] += alpha * pi[c];
                ri[c] = ri[c] - alpha * api[c];
            }
            st3v(g.x, i, xi);
            st3v(g.r, i, ri);
            if (!g.gval) {
                Mat3 P;
#pragma unroll
                for (int q = 0; q < 9; ++q) P.m[q] = g.inv[9 * (size_t)i + q];
                const Vec3 zi = P * ri;
                st3v(g.z, i, zi);
                a += ri.dot(zi);
            } else if (!exact_y) {
                const Vec3 gap = lower_product(g, team, i, g.Ap, ldm(g.gdiag + 9 * (size_t)i) * api);
                st3v(g.y, i, ld3(g.y, i) - alpha * gap);
            }
            e += fabsf(ri[0]) + fabsf(ri[1]) + fabsf(ri[2]);
        }
        if (g.gval) {
            team.sync();
            if (exact_y) {
                factor_y(g, team, i0, di, hi);
                team.sync();
            }
            a = factor_z(g, team, i0, di, hi, false);
        }
        t = team.sum2(a, e, sh, part, k);
        k ^= 1u;
        const float rz_new = t.x, err_now = t.y;
        const float beta = rz_new / rz;
        rz = rz_new;
        const bool at_cap = iter >= g.max_iter;
        if (iter == next_check || at_cap) {
            const float reresid = err_now / err0;
            int st = -1;
            if (reresid < g.tol) st = 0;
            else if (broke == 3) st = 1;
            else if (broke == 1) st = 2;
            else if (!isfinite(reresid) || at_cap) st = 2;
            if (st >= 0) {
                if (team.rank == 0 && threadIdx.x == 0) {
                    g.iters[s] = iter;
                    g.resid[s] = reresid;
                    g.state[s] = st;
                }
                team.sync();
                return;
            }
            if (reresid < 8.0f * g.tol) stride = 1;
            next_check = iter + stride;
        }
        // p = z + beta p, then the whole team sees the new p
        for (unsigned i = i0; i < hi; i += di) {
            const Vec3 zi = ld3(g.z, i), pi = ld3(g.p, i);
            st3v(g.p, i, zi + beta * pi);
        }
        team.sync();
    }
}

// ---- FSAI factor of every system (fsai.cuh restated on the batch's full rows) ----
constexpr int kBfMax = 15;                // kept lower neighbours per row
constexpr int kBfDim = 3 * (kBfMax + 1);  // 48
constexpr unsigned kBfWarps = 4;

// The slot of column c in row r (rows sorted by column), or ~0u.
__device__ __forceinline__ unsigned find_slot(const unsigned *off, const unsigned *col,
                                              unsigned r, unsigned c) {
    unsigned lo = __ldg(off + r), hi = __ldg(off + r + 1);
    while (lo < hi) {
        const unsigned mid = (lo + hi) >> 1;
        if (__ldg(col + mid) < c) lo = mid + 1;
        else hi = mid;
    }
    return (lo < __ldg(off + r + 1) && __ldg(col + lo) == c) ? lo : ~0u;
}

// C(i)^{-1} of every row's diagonal block (identity fallback).
__global__ void k_batch_cinv(unsigned rows, const unsigned *off, const unsigned *col,
                             const float *val, float *cinv) {
    const unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= rows) return;
    const unsigned k = find_slot(off, col, i, i);
    Mat3 c = Mat3::identity();
    if (k != ~0u && !chol_inv3(ldm(val + 9 * (size_t)k), c)) c = Mat3::identity();
#pragma unroll
    for (int e = 0; e < 9; ++e) cinv[9 * (size_t)i + e] = c.m[e];
}

struct BfShared {
    float M[kBfDim][kBfDim + 1];
    float Y[kBfDim][3];
    unsigned J[kBfMax], K[kBfMax];
};

// One warp per row i: G(i, j) of its (at most 15 strongest) lower
// neighbours into their slots of row i, G(i, i) into gdiag.
__global__ void __launch_bounds__(32 * kBfWarps)
    k_batch_fsai(unsigned rows, const unsigned *off, const unsigned *col, const float *val,
                 const float *cinv, bf16_t *gval, float *gdiag) {
    __shared__ BfShared sh[kBfWarps];
    const unsigned lane = threadIdx.x & 31u, wi = threadIdx.x >> 5;
    const unsigned i = blockIdx.x * kBfWarps + wi;
    if (i >= rows) return;
    BfShared &W = sh[wi];
    const Mat3 Ci = ldm(cinv + 9 * (size_t)i);
    const unsigned k0 = __ldg(off + i);
    unsigned nl = 0; // lower slots come first (columns sorted)
    while (k0 + nl < __ldg(off + i + 1) && __ldg(col + k0 + nl) < i) ++nl;
    auto norm_of = [&](unsigned t) {
        const unsigned j = __ldg(col + k0 + t);
        const Mat3 ah = (Ci * ldm(val + 9 * (size_t)(k0 + t))) * ldm(cinv + 9 * (size_t)j).transpose();
        float acc = 0.0f;
#pragma unroll
        for (int e = 0; e < 9; ++e) acc = acc + ah.m[e] * ah.m[e];
        return sqrtf(acc);
    };
    // kept: all lower slots, or the 15 strongest (ties: the earlier slot)
    unsigned m = 0;
    if (lane == 0) {
        if (nl <= (unsigned)kBfMax) {
            for (unsigned t = 0; t < nl; ++t) {
                W.J[m] = __ldg(col + k0 + t);
                W.K[m] = k0 + t;
                ++m;
            }
        } else {
            // selection by repeated maxima over the (few) lower slots
            unsigned taken[4] = {0u, 0u, 0u, 0u}; // up to 128 lower slots considered
            const unsigned cap = nl < 128u ? nl : 128u;
            for (int round = 0; round < kBfMax; ++round) {
                float best = -1.0f;
                unsigned bt = ~0u;
                for (unsigned t = 0; t < cap; ++t) {
                    if (taken[t >> 5] & (1u << (t & 31u))) continue;
                    const float v = norm_of(t);
                    if (v > best) {
                        best = v;
                        bt = t;
                    }
                }
                if (bt == ~0u) break;
                taken[bt >> 5] |= 1u << (bt & 31u);
            }
            for (unsigned t = 0; t < cap; ++t)
                if (taken[t >> 5] & (1u << (t & 31u))) {
                    W.J[m] = __ldg(col + k0 + t);
                    W.K[m] = k0 + t;
                    ++m;
                }
        }
    }
    m = __shfl_sync(0xffffffffu, m, 0);
    __syncwarp();
    const unsigned d = 3 * (m + 1);
    const unsigned pairs = (m + 1) * (m + 2) / 2;
    for (unsigned q = lane; q < pairs; q += 32) {
        unsigned a = 0, rem = q;
        while (rem >= m + 1 - a) {
            rem -= m + 1 - a;
            ++a;
        }
        const unsigned b = a + rem;
        const unsigned va = a < m ? W.J[a] : i, vb = b < m ? W.J[b] : i;
        const Mat3 Ca = ldm(cinv + 9 * (size_t)va), Cb = ldm(cinv + 9 * (size_t)vb);
        Mat3 blk = Mat3::zero();
        const unsigned kk = find_slot(off, col, va, vb); // A(va, vb) in row va
        if (kk != ~0u) blk = (Ca * ldm(val + 9 * (size_t)kk)) * Cb.transpose();
#pragma unroll
        for (int x = 0; x < 3; ++x)
#pragma unroll
            for (int y = 0; y < 3; ++y) {
                W.M[3 * a + x][3 * b + y] = blk(x, y);
                W.M[3 * b + y][3 * a + x] = blk(x, y);
            }
    }
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
                const Mat3 G = (L3inv * Yat) * ldm(cinv + 9 * (size_t)W.J[a]);
#pragma unroll
                for (int e = 0; e < 9; ++e) gval[9 * (size_t)W.K[a] + e] = __float2bfloat16_rn(G.m[e]);
            }
        }
    }
    if (!ok) Gii = Mat3::identity();
    if (lane == 0) {
        const Mat3 g = Gii * Ci;
#pragma unroll
        for (int e = 0; e < 9; ++e) gdiag[9 * (size_t)i + e] = g.m[e];
    }
}

// Upper slots (a, b > a) take the transpose of the edge's value, stored in
// row b's slot for column a.
__global__ void k_batch_fsai_mirror(unsigned rows, const unsigned *off, const unsigned *col,
                                    bf16_t *gval) {
    const unsigned a = blockIdx.x * blockDim.x + threadIdx.x;
    if (a >= rows) return;
    for (unsigned k = __ldg(off + a), k1 = __ldg(off + a + 1); k < k1; ++k) {
        const unsigned b = __ldg(col + k);
        if (b <= a) continue;
        const unsigned kk = find_slot(off, col, b, a);
        // the transpose of the edge's bf16 value, bit for bit
#pragma unroll
        for (int x = 0; x < 3; ++x)
#pragma unroll
            for (int y = 0; y < 3; ++y)
                gval[9 * (size_t)k + 3 * x + y] =
                    kk != ~0u ? gval[9 * (size_t)kk + 3 * y + x] : __float2bfloat16_rn(0.0f);
    }
}

// Row i's blocks (CSR slots off[i] ..) to their SELL positions rbase[i] +
// 32 k: columns, and 9 values per block (fp32 operator or bf16 factor).
__global__ void k_batch_sell_cols(unsigned rows, const unsigned *off, const unsigned *rbase,
                                  const unsigned *col, unsigned *scol) {
    const unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= rows) return;
    const unsigned q0 = __ldg(off + i), len = __ldg(off + i + 1) - q0, b = __ldg(rbase + i);
    for (unsigned k = 0; k < len; ++k) scol[b + 32u * k] = __ldg(col + q0 + k);
}
template <class T>
__global__ void k_batch_sell_vals(unsigned rows, const unsigned *off, const unsigned *rbase,
                                  const T *val, T *sval) {
    const unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= rows) return;
    const unsigned q0 = __ldg(off + i), len = __ldg(off + i + 1) - q0, b = __ldg(rbase + i);
    for (unsigned k = 0; k < len; ++k)
#pragma unroll
        for (int e = 0; e < 9; ++e) sval[sell_at(b + 32u * k, e)] = val[9 * (size_t)(q0 + k) + e];
}

// SELL-32 positions of a batch: each system's rows in slices of 32 from its
// first row, a slice as wide as its longest row. Fills rbase (rows) and
// returns the slices' total blocks.
size_t sell_layout(unsigned n, const unsigned *row_off, const unsigned *off,
                   std::vector<unsigned> &rbase) {
    rbase.assign(row_off[n], 0u);
    size_t base = 0;
    for (unsigned s = 0; s < n; ++s)
        for (unsigned lo = row_off[s]; lo < row_off[s + 1]; lo += 32) {
            const unsigned hi = std::min(lo + 32u, row_off[s + 1]);
            unsigned w = 0;
            for (unsigned i = lo; i < hi; ++i) w = std::max(w, off[i + 1] - off[i]);
            for (unsigned i = lo; i < hi; ++i) rbase[i] = (unsigned)std::min<size_t>(base + (i - lo), ~0u);
            base += 32 * (size_t)w;
        }
    return base;
}
// SELL positions must fit the kernels' 32-bit block index
constexpr size_t kSellMaxBlocks = 0xFFFFFFFFull - 64;

template <class T> struct Dev {
    T *d = nullptr;
    explicit Dev(size_t n, const T *h = nullptr) {
        PPF_CUDA(cudaMalloc(&d, (n ? n : 1) * sizeof(T)));
        if (h && n) PPF_CUDA(cudaMemcpy(d, h, n * sizeof(T), cudaMemcpyHostToDevice));
    }
    ~Dev() { cudaFree(d); }
};

// Team size (CTAs) per system-size bucket: rows <= 1024, <= 2048, <= 4096,
// <= 8192, more. Defaults: one CTA up to 2,048 rows, clusters of 8 above;
// ppf_batch_autotune replaces them with measured choices.
constexpr unsigned kBuckets = 5;
unsigned g_team_ctas[kBuckets] = {1, 1, 8, 8, 8};

unsigned bucket_of(unsigned rows) {
    unsigned b = 0;
    for (unsigned lim = kBucketRows; b + 1 < kBuckets && rows > lim; lim *= 2) ++b;
    return b;
}

// One launch of `systems` teams of `ctas` CTAs (ctas == 1: plain CTAs, else
// thread-block clusters). Returns the launch's error instead of throwing, so
// a cluster size the device cannot schedule is just a failed candidate.
cudaError_t launch_teams(const BatchArgs &g, unsigned systems, unsigned ctas, cudaStream_t q) {
    if (!systems) return cudaSuccess;
    if (ctas == 1) {
        k_batch_pcg<false><<<systems, kBT, 0, q>>>(g);
        count_launches();
        return cudaGetLastError();
    }
    static bool non_portable = false;
    if (ctas > 8 && !non_portable) {
        cudaError_t e = cudaFuncSetAttribute(k_batch_pcg<true>,
                                             cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
        if (e != cudaSuccess) return e;
        non_portable = true;
    }
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(systems * ctas);
    cfg.blockDim = dim3(kBT);
    cfg.stream = q;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = ctas;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    count_launches();
    return cudaLaunchKernelEx(&cfg, k_batch_pcg<true>, g);
}

// A batch uploaded to the device, with its work buffers.
struct DeviceBatch {
    unsigned n_sys, rows, blocks;
    size_t sell_blocks;
    Dev<unsigned> row, off, col, it, rbase, scol;
    Dev<float> val, sval, b, x, r, z, p, Ap, inv, res;
    Dev<int> st;
    // rbase: sell_layout's positions (sell_blocks in all)
    DeviceBatch(unsigned n, const unsigned *row_off, const unsigned *h_off,
                const unsigned *h_col, const float *h_val, const float *rhs,
                const std::vector<unsigned> &h_rbase, size_t sell)
        : n_sys(n), rows(row_off[n]), blocks(h_off[row_off[n]]), sell_blocks(sell),
          row(n + 1, row_off), off(rows + 1, h_off), col(blocks, h_col), it(n),
          rbase(rows, h_rbase.data()), scol(sell), val(9 * (size_t)blocks, h_val),
          sval(9 * sell), b(3 * (size_t)rows, rhs), x(3 * (size_t)rows), r(3 * (size_t)rows),
          z(3 * (size_t)rows), p(3 * (size_t)rows), Ap(3 * (size_t)rows),
          inv(9 * (size_t)rows), res(n), st(n) {}
    // the operator's SELL copy (on stream 0)
    void slice() const {
        if (!rows) return;
        k_batch_sell_cols<<<div_up(rows, 256u), 256>>>(rows, off.d, rbase.d, col.d, scol.d);
        PPF_LAUNCH_CHECK();
        k_batch_sell_vals<float><<<div_up(rows, 256u), 256>>>(rows, off.d, rbase.d, val.d, sval.d);
        PPF_LAUNCH_CHECK();
    }
    BatchArgs args(float tol, unsigned max_iter) const {
        BatchArgs g{};
        g.row_off = row.d;
        g.off = off.d;
        g.col = col.d;
        g.val = val.d;
        g.rbase = rbase.d;
        g.scol = scol.d;
        g.sval = sval.d;
        g.b = b.d;
        g.x = x.d;
        g.r = r.d;
        g.z = z.d;
        g.p = p.d;
        g.Ap = Ap.d;
        g.inv = inv.d;
        g.tol = tol;
        g.max_iter = max_iter;
        g.iters = it.d;
        g.resid = res.d;
        g.state = st.d;
        return g;
    }
};

// Runs the systems of `order` (device array: group after group, each group
// largest first) as consecutive groups of (count, team CTAs), one stream per
// group, or one launch per system; returns the device time in ms.
float run_groups(const BatchArgs &g0, const unsigned *d_order,
                 const std::vector<std::pair<unsigned, unsigned>> &groups, bool one_by_one) {
    std::vector<cudaStream_t> qs(groups.size() + 1);
    for (auto &q : qs) PPF_CUDA(cudaStreamCreateWithFlags(&q, cudaStreamNonBlocking));
    cudaEvent_t e0, e1;
    PPF_CUDA(cudaEventCreate(&e0));
    PPF_CUDA(cudaEventCreate(&e1));
    std::vector<cudaEvent_t> done(groups.size());
    for (auto &e : done) PPF_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    PPF_CUDA(cudaDeviceSynchronize());
    PPF_CUDA(cudaEventRecord(e0, qs[0]));
    unsigned first = 0;
    cudaError_t err = cudaSuccess;
    for (size_t k = 0; k < groups.size(); ++k) {
        cudaStream_t q = one_by_one ? qs[0] : qs[k + 1];
        if (!one_by_one) PPF_CUDA(cudaStreamWaitEvent(q, e0, 0));
        BatchArgs g = g0;
        if (one_by_one) {
            for (unsigned j = 0; j < groups[k].first && err == cudaSuccess; ++j) {
                g.order = d_order + first + j;
                err = launch_teams(g, 1, groups[k].second, q);
            }
        } else {
            g.order = d_order + first;
            err = launch_teams(g, groups[k].first, groups[k].second, q);
        }
        first += groups[k].first;
        PPF_CUDA(cudaEventRecord(done[k], q));
        PPF_CUDA(cudaStreamWaitEvent(qs[0], done[k], 0));
    }
    PPF_CUDA(cudaEventRecord(e1, qs[0]));
    PPF_CUDA(cudaEventSynchronize(e1));
    float ms = 0.0f;
    PPF_CUDA(cudaEventElapsedTime(&ms, e0, e1));
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    for (auto &e : done) cudaEventDestroy(e);
    for (auto &q : qs) cudaStreamDestroy(q);
    if (err != cudaSuccess) return -1.0f;
    return ms;
}

} // namespace
} // namespace gpu
} // namespace ppf

namespace {
using namespace ppf::gpu;

bool valid_batch(unsigned n_sys, const unsigned *row_off, const unsigned *off,
                 const unsigned *col, const float *val, const float *rhs) {
    if (!n_sys || !row_off || !off || !col || !val || !rhs) return false;
    for (unsigned s = 0; s < n_sys; ++s)
        if (row_off[s + 1] < row_off[s]) return false;
    const unsigned rows = row_off[n_sys];
    for (unsigned s = 0; s < n_sys; ++s)
        for (unsigned i = row_off[s]; i < row_off[s + 1]; ++i) {
            if (off[i + 1] < off[i]) return false;
            for (unsigned k = off[i]; k < off[i + 1]; ++k)
                if (col[k] < row_off[s] || col[k] >= row_off[s + 1] || col[k] >= rows)
                    return false;
        }
    return true;
}

// Systems grouped by the team size of their bucket, each group largest
// first (by blocks): the order and the (count, CTAs) of each group.
void group_systems(unsigned n_sys, const unsigned *row_off, const unsigned *off,
                   std::vector<unsigned> &order,
                   std::vector<std::pair<unsigned, unsigned>> &groups) {
    order.clear();
    groups.clear();
    const unsigned sizes[] = {1, 2, 4, 8, 16};
    for (unsigned c : sizes) {
        std::vector<unsigned> g;
        for (unsigned s = 0; s < n_sys; ++s)
            if (g_team_ctas[bucket_of(row_off[s + 1] - row_off[s])] == c) g.push_back(s);
        if (g.empty()) continue;
        std::stable_sort(g.begin(), g.end(), [&](unsigned a, unsigned b) {
            return off[row_off[a + 1]] - off[row_off[a]] > off[row_off[b + 1]] - off[row_off[b]];
        });
        order.insert(order.end(), g.begin(), g.end());
        groups.emplace_back((unsigned)g.size(), c);
    }
}
} // namespace

extern "C" int ppf_batch_pcg(unsigned n_sys, const unsigned *row_off, const unsigned *off,
                             const unsigned *col, const float *val, const float *rhs, float tol,
                             unsigned max_iter, int precond, int one_by_one, float *x_out,
                             unsigned *iters_out, float *resid_out, int *state_out,
                             float *ms_out) {
    try {
        if (!valid_batch(n_sys, row_off, off, col, val, rhs)) return -1;
        if (precond != PPF_PRECOND_BLOCK_JACOBI && precond != PPF_PRECOND_FSAI) return -1;
        std::vector<unsigned> rbase;
        const size_t sell = sell_layout(n_sys, row_off, off, rbase);
        if (sell > kSellMaxBlocks) return -1;
        DeviceBatch B(n_sys, row_off, off, col, val, rhs, rbase, sell);
        std::vector<unsigned> order;
        std::vector<std::pair<unsigned, unsigned>> groups;
        group_systems(n_sys, row_off, off, order, groups);
        Dev<unsigned> d_order(n_sys, order.data());
        BatchArgs g = B.args(tol, max_iter);
        const bool fsai = precond == PPF_PRECOND_FSAI;
        Dev<float> cinv(fsai ? 9 * (size_t)B.rows : 1), gdiag(fsai ? 9 * (size_t)B.rows : 1),
            yv(fsai ? 3 * (size_t)B.rows : 1);
        Dev<bf16_t> gval(fsai ? 9 * (size_t)B.blocks : 1);
        Dev<bf16_t> gsell(fsai ? 9 * B.sell_blocks : 1);
        // the SELL copies (and the FSAI factor), timed with the solve
        float build_ms = 0.0f;
        {
            cudaEvent_t b0, b1;
            PPF_CUDA(cudaEventCreate(&b0));
            PPF_CUDA(cudaEventCreate(&b1));
            PPF_CUDA(cudaDeviceSynchronize());
            PPF_CUDA(cudaEventRecord(b0, 0));
            B.slice();
            if (fsai) {
                PPF_CUDA(cudaMemsetAsync(gval.d, 0, 9 * (size_t)B.blocks * sizeof(bf16_t), 0));
                k_batch_cinv<<<div_up(B.rows, 256u), 256>>>(B.rows, B.off.d, B.col.d, B.val.d,
                                                            cinv.d);
                PPF_LAUNCH_CHECK();
                k_batch_fsai<<<div_up(B.rows, kBfWarps), 32 * kBfWarps>>>(
                    B.rows, B.off.d, B.col.d, B.val.d, cinv.d, gval.d, gdiag.d);
                PPF_LAUNCH_CHECK();
                k_batch_fsai_mirror<<<div_up(B.rows, 256u), 256>>>(B.rows, B.off.d, B.col.d,
                                                                    gval.d);
                PPF_LAUNCH_CHECK();
                k_batch_sell_vals<bf16_t><<<div_up(B.rows, 256u), 256>>>(B.rows, B.off.d,
                                                                         B.rbase.d, gval.d,
                                                                         gsell.d);
                PPF_LAUNCH_CHECK();
                g.gval = gsell.d;
                g.gdiag = gdiag.d;
                g.y = yv.d;
                g.eps = 1e-3f;
            }
            PPF_CUDA(cudaEventRecord(b1, 0));
            PPF_CUDA(cudaEventSynchronize(b1));
            PPF_CUDA(cudaEventElapsedTime(&build_ms, b0, b1));
            cudaEventDestroy(b0);
            cudaEventDestroy(b1);
        }
        const float ms = run_groups(g, d_order.d, groups, one_by_one != 0);
        if (ms < 0.0f) return -1;
        if (ms_out) *ms_out = ms + build_ms;
        const unsigned rows = B.rows;
        if (x_out)
            PPF_CUDA(cudaMemcpy(x_out, B.x.d, 3 * (size_t)rows * sizeof(float),
                                cudaMemcpyDeviceToHost));
        if (iters_out)
            PPF_CUDA(cudaMemcpy(iters_out, B.it.d, n_sys * sizeof(unsigned), cudaMemcpyDeviceToHost));
        if (resid_out)
            PPF_CUDA(cudaMemcpy(resid_out, B.res.d, n_sys * sizeof(float), cudaMemcpyDeviceToHost));
        if (state_out)
            PPF_CUDA(cudaMemcpy(state_out, B.st.d, n_sys * sizeof(int), cudaMemcpyDeviceToHost));
        return 0;
    } catch (const ppf::FatalError &) {
        return -1;
    }
}

extern "C" int ppf_batch_team_ctas(unsigned *table, int set) {
    if (!table) return -1;
    if (set) {
        for (unsigned b = 0; b < kBuckets; ++b)
            if (table[b] != 1 && table[b] != 2 && table[b] != 4 && table[b] != 8 &&
                table[b] != 16)
                return -1;
        for (unsigned b = 0; b < kBuckets; ++b) g_team_ctas[b] = table[b];
    } else {
        for (unsigned b = 0; b < kBuckets; ++b) table[b] = g_team_ctas[b];
    }
    return 0;
}

extern "C" int ppf_batch_autotune(unsigned n_sys, const unsigned *row_off, const unsigned *off,
                                  const unsigned *col, const float *val, const float *rhs,
                                  float tol, unsigned max_iter, unsigned *table_out,
                                  float *ms_out) {
    try {
        if (!valid_batch(n_sys, row_off, off, col, val, rhs)) return -1;
        std::vector<unsigned> rbase;
        const size_t sell = sell_layout(n_sys, row_off, off, rbase);
        if (sell > kSellMaxBlocks) return -1;
        DeviceBatch B(n_sys, row_off, off, col, val, rhs, rbase, sell);
        B.slice();
        const BatchArgs g = B.args(tol, max_iter);
        for (unsigned b = 0; b < kBuckets; ++b) {
            // all of the bucket's systems, largest first, in one launch per
            // candidate: the team size that solves the bucket's population
            // fastest (throughput, as the systems share the GPU in a batch)
            std::vector<unsigned> members;
            unsigned largest_rows = 0;
            for (unsigned s = 0; s < n_sys; ++s)
                if (bucket_of(row_off[s + 1] - row_off[s]) == b) {
                    members.push_back(s);
                    largest_rows = std::max(largest_rows, row_off[s + 1] - row_off[s]);
                }
            if (members.empty()) continue;
            std::stable_sort(members.begin(), members.end(), [&](unsigned a, unsigned c) {
                return off[row_off[a + 1]] - off[row_off[a]] > off[row_off[c + 1]] - off[row_off[c]];
            });
            Dev<unsigned> d_order(members.size(), members.data());
            const unsigned count = (unsigned)members.size();
            unsigned pick = g_team_ctas[b];
            float pick_ms = -1.0f;
            for (unsigned c : {1u, 2u, 4u, 8u, 16u}) {
                if (c > 1 && (c / 2) * kBT >= largest_rows) break; // half the team would idle
                float t = -1.0f;
                for (int rep = 0; rep < 3; ++rep) {
                    const float m = run_groups(g, d_order.d, {{count, c}}, false);
                    if (m < 0.0f) {
                        t = -1.0f;
                        break;
                    }
                    t = t < 0.0f ? m : std::min(t, m);
                }
                if (ms_out) ms_out[b * 5 + (c == 1 ? 0 : c == 2 ? 1 : c == 4 ? 2 : c == 8 ? 3 : 4)] = t;
                if (t >= 0.0f && (pick_ms < 0.0f || t < pick_ms)) {
                    pick = c;
                    pick_ms = t;
                }
            }
            g_team_ctas[b] = pick;
        }
        if (table_out)
            for (unsigned b = 0; b < kBuckets; ++b) table_out[b] = g_team_ctas[b];
        return 0;
    } catch (const ppf::FatalError &) {
        return -1;
    }
}
