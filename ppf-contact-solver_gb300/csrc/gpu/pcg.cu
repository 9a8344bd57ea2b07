// pcg.cu -- persistent block-Jacobi PCG.
#include "../physics/eig.cuh"
#include "pcg.cuh"

namespace ppf {
namespace gpu {

namespace {

constexpr unsigned kThreads = 256;
constexpr unsigned kWarps = kThreads / 32;
constexpr float kCurvatureSlack = 256.0f;
constexpr float kFloatEps = 1.19209290e-7f;
constexpr unsigned long long kBarrierTimeoutNs = 2000000000ull; // 2 s

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
                __nanosleep(64);
            }
        }
        __threadfence();
        s_ok = ok && (*ab == 0u);
    }
    __syncthreads();
    return s_ok != 0;
}

// Block sum of up to three values, result broadcast to every thread.
__device__ void block_sum3(float &a, float &b, float &c) {
    __shared__ float s[3][kWarps];
    unsigned lane = threadIdx.x & 31u, w = threadIdx.x >> 5;
    for (int off = 16; off > 0; off >>= 1) {
        a += __shfl_down_sync(0xffffffffu, a, off);
        b += __shfl_down_sync(0xffffffffu, b, off);
        c += __shfl_down_sync(0xffffffffu, c, off);
    }
    if (lane == 0) {
        s[0][w] = a;
        s[1][w] = b;
        s[2][w] = c;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        float x = 0.0f, y = 0.0f, z = 0.0f;
        for (unsigned k = 0; k < kWarps; ++k) {
            x += s[0][k];
            y += s[1][k];
            z += s[2][k];
        }
        s[0][0] = x;
        s[1][0] = y;
        s[2][0] = z;
    }
    __syncthreads();
    a = s[0][0];
    b = s[1][0];
    c = s[2][0];
    __syncthreads();
}

// Sum of the per-block partials in block order (identical in every block).
__device__ void reduce_partials(const float *part, unsigned nblocks, float &a,
                                float &b, float &c) {
    __shared__ float s[3];
    if (threadIdx.x < 32) {
        float x = 0.0f, y = 0.0f, z = 0.0f;
        for (unsigned k = threadIdx.x; k < nblocks; k += 32) {
            x += __ldcg(part + 3 * k);
            y += __ldcg(part + 3 * k + 1);
            z += __ldcg(part + 3 * k + 2);
        }
        for (int off = 16; off > 0; off >>= 1) {
            x += __shfl_down_sync(0xffffffffu, x, off);
            y += __shfl_down_sync(0xffffffffu, y, off);
            z += __shfl_down_sync(0xffffffffu, z, off);
        }
        if (threadIdx.x == 0) {
            s[0] = x;
            s[1] = y;
            s[2] = z;
        }
    }
    __syncthreads();
    a = s[0];
    b = s[1];
    c = s[2];
    __syncthreads();
}

__device__ __forceinline__ Vec3 ld3(const float *v, unsigned i) {
    return vec3(__ldcg(v + 3 * i), __ldcg(v + 3 * i + 1), __ldcg(v + 3 * i + 2));
}

// Row i of A v, and the component-wise sum of |contribution|.
__device__ __forceinline__ Vec3 spmv_row(const PcgOperator &A, const float *v, unsigned i,
                                         Vec3 &abssum) {
    Vec3 acc = Vec3::zero();
    abssum = Vec3::zero();
    for (unsigned k = A.f_off[i]; k < A.f_off[i + 1]; ++k) {
        Mat3 m = load_mat3(A.f_val + 9 * (size_t)k);
        Vec3 t = m * ld3(v, A.f_col[k]);
        acc += t;
        abssum += t.cwise_abs();
    }
    for (unsigned k = A.f_tr_off[i]; k < A.f_tr_off[i + 1]; ++k) {
        uint2 rs = A.f_tr[k];
        Mat3 m = load_mat3(A.f_val + 9 * (size_t)rs.y);
        Vec3 t = m.transpose() * ld3(v, rs.x);
        acc += t;
        abssum += t.cwise_abs();
    }
    for (unsigned k = A.d_off[i]; k < A.d_off[i + 1]; ++k) {
        Mat3 m = load_mat3(A.d_val + 9 * (size_t)k);
        Vec3 t = m * ld3(v, A.d_col[k]);
        acc += t;
        abssum += t.cwise_abs();
    }
    for (unsigned k = A.d_tr_off[i]; k < A.d_tr_off[i + 1]; ++k) {
        uint2 rs = A.d_tr[k];
        Mat3 m = load_mat3(A.d_val + 9 * (size_t)rs.y);
        Vec3 t = m.transpose() * ld3(v, rs.x);
        acc += t;
        abssum += t.cwise_abs();
    }
    return acc;
}

__global__ void __launch_bounds__(kThreads)
    k_pcg(PcgOperator A, float *x, float *r, float *z, float *p, float *Ap,
          float *part, unsigned *bar, float tol, unsigned max_iter, PcgResult *res) {
    const unsigned nb = gridDim.x;
    const unsigned gt = blockIdx.x * blockDim.x + threadIdx.x;
    const unsigned gs = gridDim.x * blockDim.x;
    unsigned *abort = bar + 2;
    float a, b, c;

    // r = b - A x, err0 = |r|_1
    float err = 0.0f, d0 = 0.0f, d1 = 0.0f;
    for (unsigned i = gt; i < A.n; i += gs) {
        Vec3 ab;
        Vec3 ax = spmv_row(A, x, i, ab);
        for (int k = 0; k < 3; ++k) {
            float v = r[3 * i + k] - ax[k];
            r[3 * i + k] = v;
            err += fabsf(v);
        }
    }
    block_sum3(err, d0, d1);
    if (threadIdx.x == 0) {
        part[3 * blockIdx.x] = err;
        part[3 * blockIdx.x + 1] = 0.0f;
        part[3 * blockIdx.x + 2] = 0.0f;
    }
    if (!grid_barrier(bar, nb, abort)) goto aborted;
    reduce_partials(part, nb, a, b, c);
    {
        const float err0 = a;
        if (err0 == 0.0f) {
            if (gt == 0) *res = PcgResult{1u, 0.0f, 0, 0, 0.0f, 0.0f, 0u};
            return;
        }
        if (!grid_barrier(bar, nb, abort)) goto aborted;
        // z = P r, rz0, p = z
        float rz = 0.0f;
        for (unsigned i = gt; i < A.n; i += gs) {
            Mat3 P = load_mat3(A.inv_diag + 9 * (size_t)i);
            Vec3 ri = ld3(r, i);
            Vec3 zi = P * ri;
            for (int k = 0; k < 3; ++k) {
                z[3 * i + k] = zi[k];
                p[3 * i + k] = zi[k];
                rz += ri[k] * zi[k];
            }
        }
        d0 = d1 = 0.0f;
        block_sum3(rz, d0, d1);
        if (threadIdx.x == 0) {
            part[3 * blockIdx.x] = rz;
            part[3 * blockIdx.x + 1] = 0.0f;
            part[3 * blockIdx.x + 2] = 0.0f;
        }
        if (!grid_barrier(bar, nb, abort)) goto aborted;
        reduce_partials(part, nb, a, b, c);
        float rz0 = a;
        unsigned stride = 4, next_check = 1;
        int broke = 0;
        float break_val = 0.0f;
        for (unsigned iter = 1;; ++iter) {
            if (!grid_barrier(bar, nb, abort)) goto aborted;
            // Ap = A p; pAp; sum |p_i| |terms|
            float pap = 0.0f, absdot = 0.0f, unused = 0.0f;
            for (unsigned i = gt; i < A.n; i += gs) {
                Vec3 abssum;
                Vec3 ap = spmv_row(A, p, i, abssum);
                Vec3 pi = ld3(p, i);
                for (int k = 0; k < 3; ++k) {
                    Ap[3 * i + k] = ap[k];
                    pap += pi[k] * ap[k];
                    absdot += fabsf(pi[k]) * abssum[k];
                }
            }
            block_sum3(pap, absdot, unused);
            if (threadIdx.x == 0) {
                part[3 * blockIdx.x] = pap;
                part[3 * blockIdx.x + 1] = absdot;
                part[3 * blockIdx.x + 2] = 0.0f;
            }
            if (!grid_barrier(bar, nb, abort)) goto aborted;
            reduce_partials(part, nb, a, b, c);
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
            if (!grid_barrier(bar, nb, abort)) goto aborted;
            // x += alpha p, r -= alpha Ap, z = P r, rz1, |r|_1
            float rz1 = 0.0f, er = 0.0f, u2 = 0.0f;
            for (unsigned i = gt; i < A.n; i += gs) {
                Vec3 ri;
                for (int k = 0; k < 3; ++k) {
                    const unsigned j = 3 * i + k;
                    x[j] += alpha * p[j];
                    ri[k] = r[j] - alpha * Ap[j];
                    r[j] = ri[k];
                }
                Mat3 P = load_mat3(A.inv_diag + 9 * (size_t)i);
                Vec3 zi = P * ri;
                for (int k = 0; k < 3; ++k) {
                    z[3 * i + k] = zi[k];
                    rz1 += ri[k] * zi[k];
                    er += fabsf(ri[k]);
                }
            }
            block_sum3(rz1, er, u2);
            if (threadIdx.x == 0) {
                part[3 * blockIdx.x] = rz1;
                part[3 * blockIdx.x + 1] = er;
                part[3 * blockIdx.x + 2] = 0.0f;
            }
            if (!grid_barrier(bar, nb, abort)) goto aborted;
            reduce_partials(part, nb, a, b, c);
            const float rz_new = a, err_now = b;
            const float beta = rz_new / rz0;
            rz0 = rz_new;
            for (unsigned i = gt; i < A.n; i += gs)
                for (int k = 0; k < 3; ++k) {
                    const unsigned j = 3 * i + k;
                    p[j] = z[j] + beta * p[j];
                }
            const bool at_cap = iter >= max_iter;
            if (iter == next_check || at_cap) {
                const float reresid = err_now / err0;
                PcgResult out{iter, reresid, -1, broke, err0, break_val, 0u};
                if (reresid < tol) out.state = 0;
                else if (broke == 3) out.state = 1;
                else if (broke == 1) out.state = 2;
                else if (!isfinite(reresid) || at_cap) out.state = 2;
                if (out.state >= 0) {
                    if (gt == 0) *res = out;
                    return;
                }
                if (reresid < 8.0f * tol) stride = 1;
                next_check = iter + stride;
            }
        }
    }
aborted:
    if (gt == 0) *res = PcgResult{0u, 0.0f, 2, 0, 0.0f, 0.0f, STATUS_PCG_BREAKDOWN};
}

__global__ void k_block_jacobi(PcgOperator A, const unsigned *diag_slot, float *inv,
                               unsigned *status) {
    unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= A.n) return;
    Mat3 m = load_mat3(A.f_val + 9 * (size_t)diag_slot[i]);
    Mat3 o;
    if (!eig::invert_spd(m, o)) atomicOr(status, STATUS_PRECOND_NONSPD);
    store(inv + 9 * (size_t)i, o);
}

__global__ void k_spmv(PcgOperator A, const float *x, float *y) {
    unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= A.n) return;
    Vec3 ab;
    store3(y + 3 * i, spmv_row(A, x, i, ab));
}

} // namespace

void PcgWorkspace::reserve(unsigned n) {
    z.reserve(3 * (size_t)n);
    p.reserve(3 * (size_t)n);
    Ap.reserve(3 * (size_t)n);
    if (grid == 0) {
        int dev = 0, sms = 0, per_sm = 0;
        PPF_CUDA(cudaGetDevice(&dev));
        PPF_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
        PPF_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_pcg, kThreads, 0));
        if (per_sm < 1) per_sm = 1;
        if (per_sm > 4) per_sm = 4;
        grid = (unsigned)(sms * per_sm);
        threads = kThreads;
    }
    partials.reserve(3 * (size_t)grid + 3);
    barrier.reserve(4);
    result.reserve(1);
}

void launch_block_jacobi(const PcgOperator &A, const unsigned *diag_slot, float *inv_diag,
                         unsigned *d_status, cudaStream_t q) {
    if (!A.n) return;
    k_block_jacobi<<<div_up(A.n, kThreads), kThreads, 0, q>>>(A, diag_slot, inv_diag, d_status);
    PPF_LAUNCH_CHECK();
}

void launch_spmv(const PcgOperator &A, const float *x, float *y, cudaStream_t q) {
    if (!A.n) return;
    k_spmv<<<div_up(A.n, kThreads), kThreads, 0, q>>>(A, x, y);
    PPF_LAUNCH_CHECK();
}

void launch_pcg(const PcgOperator &A, float *x, float *r, float tol, unsigned max_iter,
                PcgWorkspace &ws, cudaStream_t q) {
    ws.reserve(A.n);
    PPF_CUDA(cudaMemsetAsync(ws.barrier.data(), 0, 4 * sizeof(unsigned), q));
    float *z = ws.z.data(), *p = ws.p.data(), *Ap = ws.Ap.data(), *part = ws.partials.data();
    unsigned *bar = ws.barrier.data();
    PcgResult *res = ws.result.data();
    void *args[] = {(void *)&A, &x, &r, &z, &p, &Ap, &part, &bar, &tol, &max_iter, &res};
    PPF_CUDA(cudaLaunchCooperativeKernel((const void *)k_pcg, dim3(ws.grid), dim3(ws.threads),
                                         args, 0, q));
    ++g_kernel_launches;
}

} // namespace gpu
} // namespace ppf
