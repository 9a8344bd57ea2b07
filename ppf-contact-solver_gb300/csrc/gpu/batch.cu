// batch.cu -- many independent Newton systems solved by block-Jacobi PCG in
// one launch.
//
// Small scenes (a few hundred to ten thousand vertices) leave a whole-GPU
// persistent PCG idle: its grid barriers cost more than the products. Here
// one CTA of 1024 threads owns one system and runs the reference's
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

#include <cooperative_groups.h>

namespace ppf {
namespace gpu {
namespace {

namespace cg = cooperative_groups;

constexpr unsigned kBT = 1024;
constexpr float kSlack = 256.0f;
constexpr float kEps = 1.19209290e-7f;

struct BatchArgs {
    unsigned base;             // first system of this launch
    const unsigned *order;     // null, or the system of each CTA (largest first)
    const unsigned *row_off;   // systems + 1: vertex rows of each system
    const unsigned *off;       // rows + 1: both-triangle block rows
    const unsigned *col;       // global row of each block's column
    const float *val;          // 9 per block, column-major
    const float *b;            // 3 per row
    float *x, *r, *z, *p, *Ap; // 3 per row
    float *inv;                // 9 per row: inverse of the diagonal block
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
        const Vec3 zi = P * bi;
        st3v(g.x, i, Vec3::zero());
        st3v(g.r, i, bi);
        st3v(g.z, i, zi);
        st3v(g.p, i, zi);
        a += bi.dot(zi);
        e += fabsf(bi[0]) + fabsf(bi[1]) + fabsf(bi[2]);
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
            for (unsigned q = __ldg(g.off + i), q1 = __ldg(g.off + i + 1); q < q1; ++q) {
                const float *m = g.val + 9 * (size_t)q;
                const Vec3 v = team.ld_shared_vec(g.p, __ldg(g.col + q));
                Vec3 term;
                term[0] = __ldg(m + 0) * v[0] + __ldg(m + 3) * v[1] + __ldg(m + 6) * v[2];
                term[1] = __ldg(m + 1) * v[0] + __ldg(m + 4) * v[1] + __ldg(m + 7) * v[2];
                term[2] = __ldg(m + 2) * v[0] + __ldg(m + 5) * v[1] + __ldg(m + 8) * v[2];
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
        // x += alpha p, r -= alpha A p, z = P r (rows of this thread only)
        a = e = 0.0f;
        for (unsigned i = i0; i < hi; i += di) {
            Vec3 xi = ld3(g.x, i), ri = ld3(g.r, i);
            const Vec3 pi = ld3(g.p, i), api = ld3(g.Ap, i);
            for (int c = 0; c < 3; ++c) {
                xi[c] += alpha * pi[c];
                ri[c] = ri[c] - alpha * api[c];
            }
            Mat3 P;
#pragma unroll
            for (int q = 0; q < 9; ++q) P.m[q] = g.inv[9 * (size_t)i + q];
            const Vec3 zi = P * ri;
            st3v(g.x, i, xi);
            st3v(g.r, i, ri);
            st3v(g.z, i, zi);
            a += ri.dot(zi);
            e += fabsf(ri[0]) + fabsf(ri[1]) + fabsf(ri[2]);
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

template <class T> struct Dev {
    T *d = nullptr;
    explicit Dev(size_t n, const T *h = nullptr) {
        PPF_CUDA(cudaMalloc(&d, (n ? n : 1) * sizeof(T)));
        if (h && n) PPF_CUDA(cudaMemcpy(d, h, n * sizeof(T), cudaMemcpyHostToDevice));
    }
    ~Dev() { cudaFree(d); }
};

constexpr unsigned kClusterCtas = 8;     // CTAs of a large system's cluster
constexpr unsigned kLargeRows = 2 * kBT; // systems above this many rows take a cluster

void launch_single(const BatchArgs &g, unsigned systems, cudaStream_t q) {
    if (!systems) return;
    k_batch_pcg<false><<<systems, kBT, 0, q>>>(g);
    PPF_LAUNCH_CHECK();
}

void launch_clusters(const BatchArgs &g, unsigned systems, cudaStream_t q) {
    if (!systems) return;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(systems * kClusterCtas);
    cfg.blockDim = dim3(kBT);
    cfg.stream = q;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = kClusterCtas;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    PPF_CUDA(cudaLaunchKernelEx(&cfg, k_batch_pcg<true>, g));
    ++g_kernel_launches;
}

} // namespace
} // namespace gpu
} // namespace ppf

extern "C" int ppf_batch_pcg(unsigned n_sys, const unsigned *row_off, const unsigned *off,
                             const unsigned *col, const float *val, const float *rhs, float tol,
                             unsigned max_iter, int one_by_one, float *x_out,
                             unsigned *iters_out, float *resid_out, int *state_out,
                             float *ms_out) {
    using namespace ppf::gpu;
    try {
        if (!n_sys || !row_off || !off || !col || !val || !rhs) return -1;
        const unsigned rows = row_off[n_sys];
        const unsigned blocks = off[rows];
        for (unsigned k = 0; k < blocks; ++k)
            if (col[k] >= rows) return -1;
        Dev<unsigned> d_row(n_sys + 1, row_off), d_off(rows + 1, off), d_col(blocks, col);
        Dev<float> d_val(9 * (size_t)blocks, val), d_b(3 * (size_t)rows, rhs);
        Dev<float> x(3 * (size_t)rows), r(3 * (size_t)rows), z(3 * (size_t)rows),
            p(3 * (size_t)rows), Ap(3 * (size_t)rows), inv(9 * (size_t)rows);
        Dev<unsigned> it(n_sys);
        Dev<float> res(n_sys);
        Dev<int> st(n_sys);
        // small systems take one CTA each, large ones a cluster of CTAs; each
        // class largest first (by blocks), so the long solves start first
        std::vector<unsigned> small, large;
        for (unsigned s = 0; s < n_sys; ++s)
            (row_off[s + 1] - row_off[s] > kLargeRows ? large : small).push_back(s);
        auto by_size = [&](unsigned a, unsigned b) {
            return off[row_off[a + 1]] - off[row_off[a]] > off[row_off[b + 1]] - off[row_off[b]];
        };
        std::stable_sort(small.begin(), small.end(), by_size);
        std::stable_sort(large.begin(), large.end(), by_size);
        std::vector<unsigned> order(small);
        order.insert(order.end(), large.begin(), large.end());
        Dev<unsigned> d_order(n_sys, order.data());
        BatchArgs g{0u,   nullptr, d_row.d, d_off.d, d_col.d, d_val.d, d_b.d, x.d, r.d,  z.d,
                    p.d,  Ap.d,    inv.d,   tol,     max_iter, it.d,   res.d, st.d};
        cudaStream_t qs, ql;
        PPF_CUDA(cudaStreamCreateWithFlags(&qs, cudaStreamNonBlocking));
        PPF_CUDA(cudaStreamCreateWithFlags(&ql, cudaStreamNonBlocking));
        cudaEvent_t e0, e1, es, el;
        PPF_CUDA(cudaEventCreate(&e0));
        PPF_CUDA(cudaEventCreate(&e1));
        PPF_CUDA(cudaEventCreateWithFlags(&es, cudaEventDisableTiming));
        PPF_CUDA(cudaEventCreateWithFlags(&el, cudaEventDisableTiming));
        PPF_CUDA(cudaDeviceSynchronize());
        PPF_CUDA(cudaEventRecord(e0, qs));
        PPF_CUDA(cudaStreamWaitEvent(ql, e0, 0));
        if (one_by_one) {
            // one launch per system, each with its own team kind
            for (unsigned k = 0; k < n_sys; ++k) {
                BatchArgs h = g;
                h.order = d_order.d + k;
                if (k < small.size()) launch_single(h, 1, qs);
                else launch_clusters(h, 1, qs);
            }
        } else {
            BatchArgs hs = g, hl = g;
            hs.order = d_order.d;
            hl.order = d_order.d + small.size();
            launch_clusters(hl, (unsigned)large.size(), ql);
            launch_single(hs, (unsigned)small.size(), qs);
        }
        PPF_CUDA(cudaEventRecord(el, ql));
        PPF_CUDA(cudaStreamWaitEvent(qs, el, 0));
        PPF_CUDA(cudaEventRecord(e1, qs));
        PPF_CUDA(cudaEventSynchronize(e1));
        float ms = 0.0f;
        PPF_CUDA(cudaEventElapsedTime(&ms, e0, e1));
        for (cudaEvent_t ev : {e0, e1, es, el}) cudaEventDestroy(ev);
        cudaStreamDestroy(qs);
        cudaStreamDestroy(ql);
        if (ms_out) *ms_out = ms;
        if (x_out)
            PPF_CUDA(cudaMemcpy(x_out, x.d, 3 * (size_t)rows * sizeof(float),
                                cudaMemcpyDeviceToHost));
        if (iters_out)
            PPF_CUDA(cudaMemcpy(iters_out, it.d, n_sys * sizeof(unsigned), cudaMemcpyDeviceToHost));
        if (resid_out)
            PPF_CUDA(cudaMemcpy(resid_out, res.d, n_sys * sizeof(float), cudaMemcpyDeviceToHost));
        if (state_out)
            PPF_CUDA(cudaMemcpy(state_out, st.d, n_sys * sizeof(int), cudaMemcpyDeviceToHost));
        return 0;
    } catch (const ppf::FatalError &) {
        return -1;
    }
}
