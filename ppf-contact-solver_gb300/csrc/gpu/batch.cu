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
#include <vector>

#include "../../../include/ppf_gb300_ext.h"
#include "../physics/eig.cuh"
#include "common.cuh"
#include "fatal.cuh"

namespace ppf {
namespace gpu {
namespace {

constexpr unsigned kBT = 1024;
constexpr float kSlack = 256.0f;
constexpr float kEps = 1.19209290e-7f;

struct BatchArgs {
    unsigned base;             // first system of this launch
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

// Block-wide sums of (a, b): every thread gets the same bits (warp sums,
// then the 32 warp sums added in warp order by every thread).
__device__ __forceinline__ float2 block_sum2(float a, float b, float2 *sh) {
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
    __syncthreads();
    return t;
}

__global__ void __launch_bounds__(kBT) k_batch_pcg(BatchArgs g) {
    __shared__ float2 sh[kBT / 32];
    const unsigned s = g.base + blockIdx.x;
    const unsigned lo = __ldg(g.row_off + s), hi = __ldg(g.row_off + s + 1);
    const unsigned tid = threadIdx.x;
    // x0 = 0, r = b, block-Jacobi inverse, z = P r, p = z
    float a = 0.0f, e = 0.0f;
    for (unsigned i = lo + tid; i < hi; i += kBT) {
        Mat3 d = Mat3::identity();
        for (unsigned k = __ldg(g.off + i), k1 = __ldg(g.off + i + 1); k < k1; ++k)
            if (__ldg(g.col + k) == i) d = ldm(g.val + 9 * (size_t)k);
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
    float2 t = block_sum2(a, e, sh);
    float rz = t.x;
    const float err0 = t.y;
    if (err0 == 0.0f) {
        if (tid == 0) {
            g.iters[s] = 0;
            g.resid[s] = 0.0f;
            g.state[s] = 0;
        }
        return;
    }
    unsigned stride = 4, next_check = 1;
    int broke = 0;
    for (unsigned iter = 1;; ++iter) {
        // A p, p^T A p and its round-off scale
        a = e = 0.0f;
        for (unsigned i = lo + tid; i < hi; i += kBT) {
            Vec3 acc = Vec3::zero(), ab = Vec3::zero();
            for (unsigned k = __ldg(g.off + i), k1 = __ldg(g.off + i + 1); k < k1; ++k) {
                const float *m = g.val + 9 * (size_t)k;
                const Vec3 v = ld3(g.p, __ldg(g.col + k));
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
        t = block_sum2(a, e, sh);
        const float pAp = t.x, bound = kSlack * kEps * t.y;
        float alpha = 0.0f;
        if (pAp > bound) {
            alpha = rz / pAp;
        } else if (!broke) {
            broke = (pAp < -bound || pAp != pAp) ? 1 : 3;
        }
        // x += alpha p, r -= alpha A p, z = P r
        a = e = 0.0f;
        for (unsigned i = lo + tid; i < hi; i += kBT) {
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
        t = block_sum2(a, e, sh);
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
                if (tid == 0) {
                    g.iters[s] = iter;
                    g.resid[s] = reresid;
                    g.state[s] = st;
                }
                return;
            }
            if (reresid < 8.0f * g.tol) stride = 1;
            next_check = iter + stride;
        }
        // p = z + beta p
        for (unsigned i = lo + tid; i < hi; i += kBT) {
            const Vec3 zi = ld3(g.z, i), pi = ld3(g.p, i);
            st3v(g.p, i, zi + beta * pi);
        }
        __syncthreads();
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
        BatchArgs g{0u,   d_row.d, d_off.d, d_col.d, d_val.d, d_b.d, x.d, r.d,   z.d,  p.d,
                    Ap.d, inv.d,   tol,     max_iter, it.d,   res.d, st.d};
        cudaEvent_t e0, e1;
        PPF_CUDA(cudaEventCreate(&e0));
        PPF_CUDA(cudaEventCreate(&e1));
        PPF_CUDA(cudaEventRecord(e0, 0));
        if (one_by_one) {
            for (unsigned s = 0; s < n_sys; ++s) {
                g.base = s;
                k_batch_pcg<<<1, kBT>>>(g);
                PPF_LAUNCH_CHECK();
            }
        } else {
            k_batch_pcg<<<n_sys, kBT>>>(g);
            PPF_LAUNCH_CHECK();
        }
        PPF_CUDA(cudaEventRecord(e1, 0));
        PPF_CUDA(cudaEventSynchronize(e1));
        float ms = 0.0f;
        PPF_CUDA(cudaEventElapsedTime(&ms, e0, e1));
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
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
