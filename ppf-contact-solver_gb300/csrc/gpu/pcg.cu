// pcg.cu -- persistent block-Jacobi PCG over the SELL-32 operator.
//
// One cooperative launch per solve. Per iteration k the grid runs two
// phases separated by two grid-wide reductions (the minimum for the standard
// recurrence, which needs p^T A p before alpha and r^T z before beta):
//
//   S: p_k = z + beta p_{k-1} is formed on the fly for every column a row
//      touches (each reader evaluates the same expression, so every copy of
//      p_k(j) has the same bits as the owner's), A p_k is accumulated row by
//      row, the owner stores p_k(i) and (A p)(i); partial p^T A p and the
//      round-off scale sum |p_i| sum |terms|               -> reduce #1
//   U: alpha; x += alpha p; r -= alpha A p; z = P r; partial r^T z, |r|_1
//                                                          -> reduce #2
//
// Forming p on the fly removes the third grid barrier a stored p update
// would need before the next product; p alternates between two buffers so
// the previous direction stays readable while the new one is written.
// z, p and A p are kept as one float4 per vertex, so a neighbour gather is a
// single 16-byte load. Values another block wrote during the launch are read
// with ld.cg (from L2, never a line an SM's L1 kept from an earlier phase);
// a vertex's own values, written by the same thread, are read back directly.
// The operator is read-only inside the launch and goes through the
// non-coherent path.
#include "../physics/eig.cuh"
#include "assemble.cuh"
#include "pcg.cuh"

#include <algorithm>

namespace ppf {
namespace gpu {

namespace {

constexpr unsigned kThreads = 1024; // one block per SM
constexpr unsigned kWarps = kThreads / 32;
constexpr float kCurvatureSlack = 256.0f;
constexpr float kFloatEps = 1.19209290e-7f;
constexpr unsigned long long kBarrierTimeoutNs = 2000000000ull; // 2 s
constexpr unsigned kPad = 0xFFFFFFFFu;
constexpr unsigned kTransposed = 0x80000000u;

__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Grid barrier for a cooperative launch (all blocks co-resident). Waits are
// bounded in wall time; a timeout latches STATUS_PCG_BREAKDOWN in `abort` so
// every block leaves the solve instead of waiting again.
__device__ bool grid_barrier(unsigned *bar, unsigned nblocks, unsigned *abort) {
    __syncthreads();
    __shared__ int s_ok;
    if (threadIdx.x == 0) {
        volatile unsigned *gen = bar + 1;
        volatile unsigned *ab = abort;
        unsigned g = *gen;
        __threadfence();
        unsigned arrived = atomicAdd(bar, 1u);
        int ok = 1;
        if (arrived == nblocks - 1) {
            bar[0] = 0u;
            __threadfence();
            atomicAdd(bar + 1, 1u);
        } else {
            unsigned long long t0 = global_ns();
            while (*gen == g) {
                if (*ab) {
                    ok = 0;
                    break;
                }
                if (global_ns() - t0 > kBarrierTimeoutNs) {
                    atomicOr(abort, STATUS_PCG_BREAKDOWN);
                    ok = 0;
                    break;
                }
                __nanosleep(32);
            }
        }
        __threadfence();
        s_ok = ok && (*ab == 0u);
    }
    __syncthreads();
    return s_ok != 0;
}

// Block sum of two values (fixed order), result on thread 0.
__device__ void block_sum2(float &a, float &b) {
    __shared__ float s[2][kWarps];
    unsigned lane = threadIdx.x & 31u, w = threadIdx.x >> 5;
    for (int off = 16; off > 0; off >>= 1) {
        a += __shfl_down_sync(0xffffffffu, a, off);
        b += __shfl_down_sync(0xffffffffu, b, off);
    }
    if (lane == 0) {
        s[0][w] = a;
        s[1][w] = b;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        float x = 0.0f, y = 0.0f;
        for (unsigned k = 0; k < kWarps; ++k) {
            x += s[0][k];
            y += s[1][k];
        }
        a = x;
        b = y;
    }
    __syncthreads();
}

// Grid-wide sum of two values: block partials to `part`, barrier, then every
// block folds the partials in block order (identical result in every block).
// The callers alternate `part` between two buffers from one reduction to the
// next, so a fast block writing the next partials never overwrites ones
// still being read.
__device__ bool grid_sum2(float &a, float &b, float *part, unsigned *bar, unsigned nb,
                          unsigned *abort) {
    block_sum2(a, b);
    if (threadIdx.x == 0) {
        part[2 * blockIdx.x] = a;
        part[2 * blockIdx.x + 1] = b;
    }
    if (!grid_barrier(bar, nb, abort)) return false;
    __shared__ float s[2];
    if (threadIdx.x < 32) {
        float x = 0.0f, y = 0.0f;
        for (unsigned k = threadIdx.x; k < nb; k += 32) {
            x += __ldcg(part + 2 * k);
            y += __ldcg(part + 2 * k + 1);
        }
        for (int off = 16; off > 0; off >>= 1) {
            x += __shfl_down_sync(0xffffffffu, x, off);
            y += __shfl_down_sync(0xffffffffu, y, off);
        }
        if (threadIdx.x == 0) {
            s[0] = x;
            s[1] = y;
        }
    }
    __syncthreads();
    a = s[0];
    b = s[1];
    return true;
}

__device__ __forceinline__ Vec3 ldcg3(const float *v, unsigned i) {
    return vec3(__ldcg(v + 3 * i), __ldcg(v + 3 * i + 1), __ldcg(v + 3 * i + 2));
}
__device__ __forceinline__ Vec3 ld4(const float4 *v, unsigned i) {
    float4 a = __ldcg(v + i);
    return vec3(a.x, a.y, a.z);
}
__device__ __forceinline__ void st4(float4 *v, unsigned i, const Vec3 &a) {
    v[i] = make_float4(a[0], a[1], a[2], 0.0f);
}
__device__ __forceinline__ void st3(float *v, unsigned i, const Vec3 &a) {
    v[3 * i] = a[0];
    v[3 * i + 1] = a[1];
    v[3 * i + 2] = a[2];
}

// Neighbour value of one slot: v(j) = u(j) + beta w(j) from the float4
// vectors, or x(j) from the AoS input of the initial product.
struct GatherCombined {
    const float4 *u, *w;
    float beta;
    __device__ __forceinline__ Vec3 operator()(unsigned j) const {
        return ld4(u, j) + beta * ld4(w, j);
    }
};
struct GatherPlain {
    const float *x;
    __device__ __forceinline__ Vec3 operator()(unsigned j) const { return ldcg3(x, j); }
};

// One slot's block times its neighbour value.
template <class G>
__device__ __forceinline__ void slot_term(const SellMatrix &M, size_t s, unsigned lane,
                                          unsigned j, const G &gather, Vec3 &acc,
                                          Vec3 &abssum) {
    const float *a = M.val + s * 9 * kSliceRows + lane;
    float m[9];
#pragma unroll
    for (int e = 0; e < 9; ++e) m[e] = __ldg(a + e * kSliceRows);
    const Vec3 v = gather(j);
    // column-major block: t_r = sum_c m[3 c + r] v_c
    Vec3 t;
    t[0] = m[0] * v[0] + m[3] * v[1] + m[6] * v[2];
    t[1] = m[1] * v[0] + m[4] * v[1] + m[7] * v[2];
    t[2] = m[2] * v[0] + m[5] * v[1] + m[8] * v[2];
    acc += t;
    abssum += t.cwise_abs();
}

// Row (32 s + lane) of A v over one SELL matrix. abssum collects the
// component-wise |term| of every block product. Slots are taken four at a
// time (column indices first) so four gathers are in flight per lane; the
// terms are still added in slot order.
template <class G>
__device__ __forceinline__ void sell_row(const SellMatrix &M, unsigned slice, unsigned lane,
                                         const G &gather, Vec3 &acc, Vec3 &abssum) {
    const unsigned s0 = __ldg(M.slice_off + slice), s1 = __ldg(M.slice_off + slice + 1);
    unsigned s = s0;
    for (; s + 4 <= s1; s += 4) {
        unsigned j[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) j[q] = __ldg(M.col + (size_t)(s + q) * kSliceRows + lane);
#pragma unroll
        for (int q = 0; q < 4; ++q) slot_term(M, s + q, lane, j[q], gather, acc, abssum);
    }
    for (; s < s1; ++s) {
        const unsigned j = __ldg(M.col + (size_t)s * kSliceRows + lane);
        slot_term(M, s, lane, j, gather, acc, abssum);
    }
}

__device__ __forceinline__ Mat3 load_inv(const float *inv, unsigned slice, unsigned lane) {
    Mat3 P;
    const float *a = inv + (size_t)slice * 9 * kSliceRows + lane;
#pragma unroll
    for (int e = 0; e < 9; ++e) P.m[e] = __ldg(a + e * kSliceRows);
    return P;
}

struct PcgArgs {
    PcgOperator A;
    float *x, *r;
    float4 *z, *p0, *p1, *Ap;
    float *part; // 2 buffers of 2 floats per block
    unsigned *bar;
    float tol;
    unsigned max_iter;
    PcgResult *res;
};

__global__ void __launch_bounds__(kThreads, 1) k_pcg(PcgArgs g) {
    const PcgOperator &A = g.A;
    const unsigned nb = gridDim.x;
    const unsigned lane = threadIdx.x & 31u;
    const unsigned warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const unsigned nwarps = (gridDim.x * blockDim.x) >> 5;
    const unsigned n_slices = A.fixed.n_slices;
    unsigned *abort = g.bar + 2;
    float *part0 = g.part, *part1 = g.part + 2 * nb;
    float a, b;

    // r = b - A x0, z = P r, p_0 = 0; err0 = |r|_1, rz0 = r^T z
    a = b = 0.0f;
    for (unsigned sl = warp; sl < n_slices; sl += nwarps) {
        const unsigned i = sl * kSliceRows + lane;
        Vec3 acc = Vec3::zero(), ab = Vec3::zero();
        const GatherPlain gx{g.x};
        sell_row(A.fixed, sl, lane, gx, acc, ab);
        sell_row(A.dyn, sl, lane, gx, acc, ab);
        if (i < A.n) {
            Vec3 ri = ldcg3(g.r, i) - acc;
            Vec3 zi = load_inv(A.inv_diag, sl, lane) * ri;
            st3(g.r, i, ri);
            st4(g.z, i, zi);
            st4(g.p0, i, Vec3::zero());
            a += fabsf(ri[0]) + fabsf(ri[1]) + fabsf(ri[2]);
            b += ri.dot(zi);
        }
    }
    if (!grid_sum2(a, b, part0, g.bar, nb, abort)) goto aborted;
    {
        const float err0 = a;
        float rz0 = b;
        if (err0 == 0.0f) {
            if (blockIdx.x == 0 && threadIdx.x == 0)
                *g.res = PcgResult{1u, 0.0f, 0, 0, 0.0f, 0.0f, 0u};
            return;
        }
        float beta = 0.0f;
        unsigned stride = 4, next_check = 1;
        int broke = 0;
        float break_val = 0.0f;
        for (unsigned iter = 1;; ++iter) {
            const float4 *p_prev = (iter & 1u) ? g.p0 : g.p1;
            float4 *p_new = (iter & 1u) ? g.p1 : g.p0;
            // S: A p_k with p_k = z + beta p_{k-1}
            a = b = 0.0f; // p^T A p, sum |p_i| |terms|
            const GatherCombined gp{g.z, p_prev, beta};
            for (unsigned sl = warp; sl < n_slices; sl += nwarps) {
                const unsigned i = sl * kSliceRows + lane;
                Vec3 acc = Vec3::zero(), ab = Vec3::zero();
                sell_row(A.fixed, sl, lane, gp, acc, ab);
                sell_row(A.dyn, sl, lane, gp, acc, ab);
                if (i < A.n) {
                    Vec3 pi = gp(i);
                    st4(p_new, i, pi);
                    st4(g.Ap, i, acc);
                    a += pi.dot(acc);
                    b += fabsf(pi[0]) * ab[0] + fabsf(pi[1]) * ab[1] + fabsf(pi[2]) * ab[2];
                }
            }
            if (!grid_sum2(a, b, part1, g.bar, nb, abort)) goto aborted;
            const float pAp = a, bound = kCurvatureSlack * kFloatEps * b;
            float alpha;
            if (pAp > bound) {
                alpha = rz0 / pAp;
            } else {
                alpha = 0.0f;
                if (!broke) {
                    broke = (pAp < -bound || pAp != pAp) ? 1 : 3;
                    break_val = pAp;
                }
            }
            // U: x += alpha p, r -= alpha A p, z = P r; r^T z, |r|_1
            a = b = 0.0f;
            for (unsigned sl = warp; sl < n_slices; sl += nwarps) {
                const unsigned i = sl * kSliceRows + lane;
                if (i >= A.n) continue;
                Vec3 pi = ld4(p_new, i), api = ld4(g.Ap, i);
                Vec3 xi = ldcg3(g.x, i), ri = ldcg3(g.r, i);
                for (int k = 0; k < 3; ++k) {
                    xi[k] += alpha * pi[k];
                    ri[k] = ri[k] - alpha * api[k];
                }
                Vec3 zi = load_inv(A.inv_diag, sl, lane) * ri;
                st3(g.x, i, xi);
                st3(g.r, i, ri);
                st4(g.z, i, zi);
                a += ri.dot(zi);
                b += fabsf(ri[0]) + fabsf(ri[1]) + fabsf(ri[2]);
            }
            if (!grid_sum2(a, b, part0, g.bar, nb, abort)) goto aborted;
            const float rz_new = a, err_now = b;
            beta = rz_new / rz0;
            rz0 = rz_new;
            const bool at_cap = iter >= g.max_iter;
            if (iter == next_check || at_cap) {
                const float reresid = err_now / err0;
                PcgResult out{iter, reresid, -1, broke, err0, break_val, 0u};
                if (reresid < g.tol) out.state = 0;
                else if (broke == 3) out.state = 1;
                else if (broke == 1) out.state = 2;
                else if (!isfinite(reresid) || at_cap) out.state = 2;
                if (out.state >= 0) {
                    if (blockIdx.x == 0 && threadIdx.x == 0) *g.res = out;
                    return;
                }
                if (reresid < 8.0f * g.tol) stride = 1;
                next_check = iter + stride;
            }
        }
    }
aborted:
    if (blockIdx.x == 0 && threadIdx.x == 0)
        *g.res = PcgResult{0u, 0.0f, 2, 0, 0.0f, 0.0f, STATUS_PCG_BREAKDOWN};
}

__global__ void k_block_jacobi(unsigned n, const float *upper_val, const unsigned *diag_slot,
                               float *inv, unsigned *status) {
    unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    Mat3 m = load_mat3(upper_val + 9 * (size_t)diag_slot[i]);
    Mat3 o;
    if (!eig::invert_spd(m, o)) atomicOr(status, STATUS_PRECOND_NONSPD);
    float *d = inv + (size_t)(i / kSliceRows) * 9 * kSliceRows + (i % kSliceRows);
#pragma unroll
    for (int e = 0; e < 9; ++e) d[e * kSliceRows] = o.m[e];
}

// (slot, lane) -> copy of the source upper block (transposed when flagged).
__global__ void k_sell_pack(unsigned elems, const unsigned *src, const float *upper,
                            float *val) {
    unsigned t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= elems) return;
    unsigned sidx = src[t];
    float m[9];
    if (sidx == kPad) {
#pragma unroll
        for (int e = 0; e < 9; ++e) m[e] = 0.0f;
    } else {
        const float *b = upper + 9 * (size_t)(sidx & ~kTransposed);
        if (sidx & kTransposed) {
#pragma unroll
            for (int r = 0; r < 3; ++r)
#pragma unroll
                for (int c = 0; c < 3; ++c) m[3 * c + r] = b[3 * r + c];
        } else {
#pragma unroll
            for (int e = 0; e < 9; ++e) m[e] = b[e];
        }
    }
    unsigned slot = t / kSliceRows, lane = t % kSliceRows;
    float *d = val + (size_t)slot * 9 * kSliceRows + lane;
#pragma unroll
    for (int e = 0; e < 9; ++e) d[e * kSliceRows] = m[e];
}

// Contact part: per-row block count (upper + transposed), max per slice.
// Blocks that touch a Dirichlet vertex are exactly zero after elimination
// and are left out (a pinned collider vertex can carry thousands of them).
// Launched with whole warps per slice (blockDim a multiple of 32).
__device__ __forceinline__ unsigned dyn_row_count(unsigned i, const unsigned *off,
                                                  const unsigned *col, const unsigned *tr_off,
                                                  const uint2 *tr, const unsigned *mask) {
    if (mask[i]) return 0u;
    unsigned c = 0;
    for (unsigned q = off[i]; q < off[i + 1]; ++q) c += mask[col[q]] ? 0u : 1u;
    for (unsigned q = tr_off[i]; q < tr_off[i + 1]; ++q) c += mask[tr[q].x] ? 0u : 1u;
    return c;
}

__global__ void k_dyn_slice_k(unsigned n, unsigned n_slices, const unsigned *off,
                              const unsigned *col, const unsigned *tr_off, const uint2 *tr,
                              const unsigned *mask, unsigned *slice_k) {
    unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
    unsigned sl = i / kSliceRows;
    if (sl >= n_slices) return;
    unsigned c = i < n ? dyn_row_count(i, off, col, tr_off, tr, mask) : 0u;
    c = __reduce_max_sync(0xffffffffu, c);
    if ((i % kSliceRows) == 0) slice_k[sl] = c;
}

__device__ __forceinline__ void put_slot(unsigned *out_col, float *out_val, unsigned s,
                                         unsigned lane, unsigned j, const float (&m)[9]) {
    out_col[(size_t)s * kSliceRows + lane] = j;
    float *d = out_val + (size_t)s * 9 * kSliceRows + lane;
#pragma unroll
    for (int e = 0; e < 9; ++e) d[e * kSliceRows] = m[e];
}

__global__ void k_dyn_sell_fill(unsigned n, unsigned n_slices, const unsigned *off,
                                const unsigned *col, const float *upper, const unsigned *tr_off,
                                const uint2 *tr, const unsigned *mask,
                                const unsigned *slice_off, unsigned *out_col, float *out_val) {
    unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
    unsigned sl = i / kSliceRows, lane = i % kSliceRows;
    if (sl >= n_slices) return;
    unsigned s = slice_off[sl];
    const unsigned s1 = slice_off[sl + 1];
    if (i < n && !mask[i]) {
        for (unsigned q = off[i]; q < off[i + 1]; ++q) {
            unsigned j = col[q];
            if (mask[j]) continue;
            const float *b = upper + 9 * (size_t)q;
            float m[9];
#pragma unroll
            for (int e = 0; e < 9; ++e) m[e] = b[e];
            put_slot(out_col, out_val, s++, lane, j, m);
        }
        for (unsigned q = tr_off[i]; q < tr_off[i + 1]; ++q) {
            uint2 rp = tr[q];
            if (mask[rp.x]) continue;
            const float *b = upper + 9 * (size_t)rp.y;
            float m[9];
#pragma unroll
            for (int r = 0; r < 3; ++r)
#pragma unroll
                for (int c = 0; c < 3; ++c) m[3 * c + r] = b[3 * r + c];
            put_slot(out_col, out_val, s++, lane, rp.x, m);
        }
    }
    const unsigned self = i < n ? i : n - 1;
    const float zero[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    for (; s < s1; ++s) put_slot(out_col, out_val, s, lane, self, zero);
}

} // namespace

void PcgWorkspace::reserve(unsigned n) {
    z.reserve(n);
    p0.reserve(n);
    p1.reserve(n);
    Ap.reserve(n);
    if (grid == 0) {
        int dev = 0, sms = 0, per_sm = 0;
        PPF_CUDA(cudaGetDevice(&dev));
        PPF_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
        PPF_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_pcg, kThreads, 0));
        if (per_sm < 1) per_sm = 1;
        if (per_sm > 1) per_sm = 1;
        grid = (unsigned)(sms * per_sm);
        threads = kThreads;
    }
    partials.reserve(4 * (size_t)grid + 4);
    barrier.reserve(4);
    result.reserve(1);
}

void sell_build_fixed(unsigned n, const std::vector<unsigned> &off,
                      const std::vector<unsigned> &col, const std::vector<unsigned> &tr_off,
                      const std::vector<uint2> &tr, SellLayout &out) {
    const unsigned n_slices = (n + kSliceRows - 1) / kSliceRows;
    std::vector<unsigned> slice_off(n_slices + 1, 0u);
    for (unsigned sl = 0; sl < n_slices; ++sl) {
        unsigned k = 0;
        for (unsigned l = 0; l < kSliceRows; ++l) {
            unsigned i = sl * kSliceRows + l;
            if (i >= n) break;
            k = std::max(k, (off[i + 1] - off[i]) + (tr_off[i + 1] - tr_off[i]));
        }
        slice_off[sl + 1] = slice_off[sl] + k;
    }
    const unsigned slots = slice_off[n_slices];
    std::vector<unsigned> c((size_t)slots * kSliceRows), src((size_t)slots * kSliceRows);
    for (unsigned sl = 0; sl < n_slices; ++sl)
        for (unsigned l = 0; l < kSliceRows; ++l) {
            unsigned i = sl * kSliceRows + l;
            unsigned self = i < n ? i : n - 1;
            unsigned k = 0;
            auto put = [&](unsigned j, unsigned s) {
                size_t e = (size_t)(slice_off[sl] + k) * kSliceRows + l;
                c[e] = j;
                src[e] = s;
                ++k;
            };
            if (i < n) {
                for (unsigned q = off[i]; q < off[i + 1]; ++q) put(col[q], q);
                for (unsigned q = tr_off[i]; q < tr_off[i + 1]; ++q)
                    put(tr[q].x, tr[q].y | kTransposed);
            }
            while (slice_off[sl] + k < slice_off[sl + 1]) put(self, kPad);
        }
    out.n_slices = n_slices;
    out.slots = slots;
    out.slice_off.reserve(n_slices + 1);
    out.col.reserve((size_t)slots * kSliceRows + 1);
    out.src.reserve((size_t)slots * kSliceRows + 1);
    out.val.reserve((size_t)slots * kSliceRows * 9 + 1);
    PPF_CUDA(cudaMemcpy(out.slice_off.data(), slice_off.data(), slice_off.size() * 4,
                        cudaMemcpyHostToDevice));
    if (slots) {
        PPF_CUDA(cudaMemcpy(out.col.data(), c.data(), c.size() * 4, cudaMemcpyHostToDevice));
        PPF_CUDA(cudaMemcpy(out.src.data(), src.data(), src.size() * 4, cudaMemcpyHostToDevice));
    }
}

void sell_pack_fixed(SellLayout &L, const float *upper_val, cudaStream_t q) {
    unsigned elems = L.slots * kSliceRows;
    if (!elems) return;
    k_sell_pack<<<div_up(elems, 256u), 256, 0, q>>>(elems, L.src.data(), upper_val,
                                                    L.val.data());
    PPF_LAUNCH_CHECK();
}

void sell_build_dyn(unsigned n, const unsigned *off, const unsigned *col, const float *val,
                    const unsigned *tr_off, const uint2 *tr, const unsigned *dof_mask,
                    SellLayout &out, DevBuf<unsigned> &slice_k, DevBuf<unsigned> &scan_tmp,
                    cudaStream_t q) {
    const unsigned n_slices = (n + kSliceRows - 1) / kSliceRows;
    out.n_slices = n_slices;
    out.slice_off.reserve(n_slices + 1);
    slice_k.reserve(n_slices + 1);
    scan_tmp.reserve(scan_tmp_size(n_slices + 1));
    const unsigned threads = n_slices * kSliceRows;
    k_dyn_slice_k<<<div_up(threads, 256u), 256, 0, q>>>(n, n_slices, off, col, tr_off, tr,
                                                        dof_mask, slice_k.data());
    PPF_LAUNCH_CHECK();
    exclusive_scan(slice_k.data(), out.slice_off.data(), n_slices, scan_tmp.data(), q);
    unsigned slots = 0;
    PPF_CUDA(cudaMemcpyAsync(&slots, out.slice_off.data() + n_slices, sizeof(unsigned),
                             cudaMemcpyDeviceToHost, q));
    PPF_CUDA(cudaStreamSynchronize(q));
    out.slots = slots;
    out.col.reserve((size_t)slots * kSliceRows + 1);
    out.val.reserve((size_t)slots * kSliceRows * 9 + 1);
    if (!slots) return;
    k_dyn_sell_fill<<<div_up(threads, 256u), 256, 0, q>>>(n, n_slices, off, col, val, tr_off,
                                                          tr, dof_mask, out.slice_off.data(),
                                                          out.col.data(), out.val.data());
    PPF_LAUNCH_CHECK();
}

void launch_block_jacobi(unsigned n, const float *upper_val, const unsigned *diag_slot,
                         float *inv_diag, unsigned *d_status, cudaStream_t q) {
    if (!n) return;
    k_block_jacobi<<<div_up(n, kThreads), kThreads, 0, q>>>(n, upper_val, diag_slot, inv_diag,
                                                            d_status);
    PPF_LAUNCH_CHECK();
}

void launch_pcg(const PcgOperator &A, float *x, float *r, float tol, unsigned max_iter,
                PcgWorkspace &ws, cudaStream_t q) {
    ws.reserve(A.n);
    PPF_CUDA(cudaMemsetAsync(ws.barrier.data(), 0, 4 * sizeof(unsigned), q));
    PcgArgs g{A,
              x,
              r,
              ws.z.data(),
              ws.p0.data(),
              ws.p1.data(),
              ws.Ap.data(),
              ws.partials.data(),
              ws.barrier.data(),
              tol,
              max_iter,
              ws.result.data()};
    void *args[] = {(void *)&g};
    PPF_CUDA(cudaLaunchCooperativeKernel((const void *)k_pcg, dim3(ws.grid), dim3(ws.threads),
                                         args, 0, q));
    ++g_kernel_launches;
}

} // namespace gpu
} // namespace ppf
