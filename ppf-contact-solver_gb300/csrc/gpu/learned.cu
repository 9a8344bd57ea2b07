// learned.cu -- the learned preconditioner's network: inference and training
// kernels (layout and formulas in learned.cuh).
//
// Dense layers run on the tensor cores as bf16 x bf16 -> fp32 products:
//   rows mode    C[R x N] = A[R x K] B[N x K]^T: the forward layers as
//                tcgen05.mma tiles (k_gemm_rows_tc), the input gradients as
//                mma.sync.m16n8k16 tiles (k_gemm_rows)
//   reduce mode  C[M x N] += A[R x M]^T B[R x N] (weight grads, mma.sync,
//                split over row ranges, one fp32 atomic add per output per
//                block)
// Graph work (features, neighbour means, edge head, probes) is scalar fp32 in
// a fixed order per vertex: each vertex walks its neighbours as fixed upper
// entries, fixed transposed entries, contact upper entries, contact
// transposed entries, skipping Dirichlet vertices, so every sum has one
// order and the forward pass is deterministic.
#include <algorithm>
#include <vector>

#include "fatal.cuh"
#include "learned.cuh"
#include "precond.cuh"

namespace ppf {
namespace gpu {

using namespace learned;

namespace {

constexpr unsigned kT = 256;

__device__ __forceinline__ Mat3 ld_blk(const float *p) {
    Mat3 m;
#pragma unroll
    for (int e = 0; e < 9; ++e) m.m[e] = __ldg(p + e);
    return m;
}

// f(j, block, i_is_lo, part, edge) for every live neighbour j of vertex i.
template <class F>
__device__ __forceinline__ void walk_neighbours(const LearnedGraph &g, unsigned i, F &&f) {
    if (__ldg(g.dof_mask + i)) return;
#pragma unroll 1
    for (int p = 0; p < 2; ++p) {
        const LearnedPart &P = p ? g.contact : g.fixed;
        const unsigned base = p ? g.fixed.nnz : 0u;
        if (!P.off) continue;
        const unsigned k0 = __ldg(P.off + i), k1 = __ldg(P.off + i + 1);
        for (unsigned k = k0; k < k1; ++k) {
            const unsigned j = __ldg(P.col + k);
            if (j == i || __ldg(g.dof_mask + j)) continue;
            f(j, P.val + 9 * (size_t)k, true, p, base + k);
        }
        const unsigned t0 = __ldg(P.tr_off + i), t1 = __ldg(P.tr_off + i + 1);
        for (unsigned t = t0; t < t1; ++t) {
            const uint2 e = __ldg(P.tr + t);
            if (__ldg(g.dof_mask + e.x)) continue;
            f(e.x, P.val + 9 * (size_t)e.y, false, p, base + e.y);
        }
    }
}

__device__ __forceinline__ Mat3 ahat_of(const LearnedGraph &g, unsigned i, unsigned j,
                                        const float *blk, bool i_is_lo) {
    const Mat3 Ci = ld_blk(g.cinv + 9 * (size_t)i), Cj = ld_blk(g.cinv + 9 * (size_t)j);
    const Mat3 B = ld_blk(blk);
    return i_is_lo ? learned_edge_ahat(Cj, Ci, B) : learned_edge_ahat(Ci, Cj, B);
}

// ---- features ------------------------------------------------------------------------
__global__ void k_node_inputs(LearnedGraph g, bf16_t *X0, float *deg) {
    const unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= g.n) return;
    float x[kIn0];
#pragma unroll
    for (int c = 0; c < (int)kIn0; ++c) x[c] = 0.0f;
    float cnt = 0.0f;
    if (!__ldg(g.dof_mask + i)) {
        const Mat3 a = ld_blk(g.fixed.val + 9 * (size_t)__ldg(g.diag_slot + i));
        const float s = ((a(0, 0) + a(1, 1)) + a(2, 2)) / 3.0f;
#pragma unroll
        for (int e = 0; e < 9; ++e) x[e] = a.m[e] / s;
        const float m = __ldg(g.mass + i);
        const float ratio = m > 0.0f ? s / m : 1.0f;
        x[9] = 0.1f * logf(ratio);
        float cc = 0.0f, cf = 0.0f, s1 = 0.0f, s2 = 0.0f;
        walk_neighbours(g, i, [&](unsigned j, const float *blk, bool lo, int p, unsigned) {
            const float nrm = learned_fro(ahat_of(g, i, j, blk, lo));
            s1 = s1 + nrm;
            s2 = s2 + nrm * nrm;
            if (p) cc += 1.0f;
            else cf += 1.0f;
        });
        x[10] = cc / 8.0f;
        x[11] = s1;
        x[12] = s2;
        x[13] = cf / 16.0f;
        cnt = cc + cf;
    }
    x[15] = 1.0f;
#pragma unroll
    for (int c = 0; c < (int)kIn0; ++c) X0[(size_t)i * kIn0 + c] = __float2bfloat16_rn(x[c]);
    deg[i] = cnt;
}

// X = [H, bf16(mean of H over the neighbours), 1, 0..] (80 wide); with
// mean == false, X = [H, 1, 0..] (48 wide). One warp per vertex, lane = unit.
template <bool kMean>
__global__ void k_aggregate(LearnedGraph g, const bf16_t *H, const float *deg, bf16_t *X) {
    const unsigned i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, k = threadIdx.x & 31u;
    if (i >= g.n) return;
    constexpr unsigned W = kMean ? kInL : kInH;
    bf16_t *row = X + (size_t)i * W;
    row[k] = H[(size_t)i * 32 + k];
    unsigned c0 = 32;
    if (kMean) {
        float acc = 0.0f;
        walk_neighbours(g, i, [&](unsigned j, const float *, bool, int, unsigned) {
            acc = acc + __bfloat162float(H[(size_t)j * 32 + k]);
        });
        const float dg = deg[i];
        row[32 + k] = __float2bfloat16_rn(dg > 0.0f ? acc / dg : 0.0f);
        c0 = 64;
    }
    if (k < 16) row[c0 + k] = __float2bfloat16_rn(k == 0 ? 1.0f : 0.0f);
}

// ---- tensor-core dense layers ----------------------------------------------------------
__device__ __forceinline__ uint32_t ld_pair(const bf16_t *p) {
    return *reinterpret_cast<const uint32_t *>(p);
}

__device__ __forceinline__ void mma16816(float (&d)[4], const uint32_t (&a)[4],
                                         const uint32_t (&b)[2]) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 "
        "{%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};\n"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

constexpr unsigned kRowsTile = 64; // rows per block in rows mode (4 warps x 16)

// C[R x N] = A[R x K] B[N x K]^T, A and B dense row-major bf16. Epilogue:
// relu -> bf16 into Cb (ld N), or plain fp32 into Cf (ld N).
template <int K, int N>
__global__ void __launch_bounds__(128) k_gemm_rows(unsigned R, const bf16_t *__restrict__ A,
                                                   const bf16_t *__restrict__ B, float *Cf,
                                                   bf16_t *Cb) {
    static_assert(K % 16 == 0 && N % 8 == 0, "tile shape");
    __shared__ __align__(16) bf16_t sA[kRowsTile][K + 8];
    __shared__ __align__(16) bf16_t sB[N][K + 8];
    const unsigned r0 = blockIdx.x * kRowsTile;
    constexpr int KV = K / 8; // uint4 per row
    for (int t = threadIdx.x; t < N * KV; t += 128) {
        const int n = t / KV, c = (t % KV) * 8;
        *reinterpret_cast<uint4 *>(&sB[n][c]) =
            __ldg(reinterpret_cast<const uint4 *>(B + (size_t)n * K + c));
    }
    for (int t = threadIdx.x; t < (int)kRowsTile * KV; t += 128) {
        const int r = t / KV, c = (t % KV) * 8;
        uint4 v = make_uint4(0u, 0u, 0u, 0u);
        if (r0 + r < R) v = __ldg(reinterpret_cast<const uint4 *>(A + (size_t)(r0 + r) * K + c));
        *reinterpret_cast<uint4 *>(&sA[r][c]) = v;
    }
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, t4 = lane & 3;
    const int rw = warp * 16;
    float acc[N / 8][4];
#pragma unroll
    for (int nt = 0; nt < N / 8; ++nt)
#pragma unroll
        for (int e = 0; e < 4; ++e) acc[nt][e] = 0.0f;
#pragma unroll
    for (int kk = 0; kk < K; kk += 16) {
        uint32_t a[4];
        a[0] = ld_pair(&sA[rw + g][kk + 2 * t4]);
        a[1] = ld_pair(&sA[rw + g + 8][kk + 2 * t4]);
        a[2] = ld_pair(&sA[rw + g][kk + 8 + 2 * t4]);
        a[3] = ld_pair(&sA[rw + g + 8][kk + 8 + 2 * t4]);
#pragma unroll
        for (int nt = 0; nt < N / 8; ++nt) {
            uint32_t b[2];
            b[0] = ld_pair(&sB[nt * 8 + g][kk + 2 * t4]);
            b[1] = ld_pair(&sB[nt * 8 + g][kk + 8 + 2 * t4]);
            mma16816(acc[nt], a, b);
        }
    }
#pragma unroll
    for (int h = 0; h < 2; ++h) {
        const unsigned r = r0 + rw + g + 8 * h;
        if (r >= R) continue;
#pragma unroll
        for (int nt = 0; nt < N / 8; ++nt) {
            const int c = nt * 8 + 2 * t4;
            const float v0 = acc[nt][2 * h], v1 = acc[nt][2 * h + 1];
            if (Cb) {
                __nv_bfloat162 p;
                p.x = __float2bfloat16_rn(fmaxf(v0, 0.0f));
                p.y = __float2bfloat16_rn(fmaxf(v1, 0.0f));
                *reinterpret_cast<__nv_bfloat162 *>(Cb + (size_t)r * N + c) = p;
            } else {
                *reinterpret_cast<float2 *>(Cf + (size_t)r * N + c) = make_float2(v0, v1);
            }
        }
    }
}

// ---- the same row-tile product on the 5th-generation tensor cores ----------------
// Persistent CTAs of 4 warps walk 128-row tiles. Operands sit in shared memory
// in the no-swizzle K-major canonical layout (8 rows x 16 B core matrices;
// A: core matrix (row group g, K chunk c) at c * 2048 + g * 128 bytes, B: at
// c * N * 16 + g * 128). B (the weights) is staged once per CTA; A tiles are
// double-buffered and fetched with cp.async, so the next tile's rows stream
// in while the current tile's epilogue runs. Per tile one elected thread
// issues K / 16 tcgen05.mma (kind::f16, bf16 inputs, M = 128, fp32
// accumulator of N columns in tensor memory, allocated once per CTA) and
// commits them to an mbarrier; each warp reads its 32 accumulator lanes
// (rows) back with tcgen05.ld for the epilogue. The mbarrier waits are
// bounded: on timeout the kernel latches g_tc_status, waits (bounded again),
// frees its tensor memory and returns.
constexpr unsigned kTcRows = 128;
constexpr unsigned kTcCtasPerSm = 4;
__device__ unsigned g_tc_status;

__device__ __forceinline__ uint64_t tc_smem_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
    return (uint64_t)((saddr & 0x3FFFFu) >> 4) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
           ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}

__device__ __forceinline__ bool tc_wait(uint32_t mbar, uint32_t phase, unsigned limit) {
    uint32_t done = 0;
    for (unsigned it = 0; it < limit && !done; ++it)
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
            " selp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(done)
            : "r"(mbar), "r"(phase)
            : "memory");
    return done != 0;
}

template <int N> constexpr uint32_t tc_cols() { return N <= 32 ? 32u : N <= 64 ? 64u : 128u; }

// 16-byte asynchronous copy global -> shared; src_bytes 0 writes zeros.
__device__ __forceinline__ void cp_async16(uint32_t dst, const void *src, uint32_t src_bytes) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(dst), "l"(src),
                 "r"(src_bytes)
                 : "memory");
}

template <int K>
__device__ __forceinline__ void tc_fetch_tile(uint32_t sa, const bf16_t *A, unsigned R,
                                              unsigned r0) {
    constexpr int KV = K / 8;
    for (int t = threadIdx.x; t < (int)kTcRows * KV; t += 128) {
        const int r = t / KV, c = t % KV;
        const bool in = r0 + r < R;
        const bf16_t *src = in ? A + (size_t)(r0 + r) * K + c * 8 : A;
        cp_async16(sa + c * 2048 + r * 16, src, in ? 16u : 0u);
    }
    asm volatile("cp.async.commit_group;\n" ::: "memory");
}

template <int K, int N>
__global__ void __launch_bounds__(128) k_gemm_rows_tc(unsigned R, const bf16_t *__restrict__ A,
                                                      const bf16_t *__restrict__ B, float *Cf,
                                                      bf16_t *Cb) {
    static_assert(K % 16 == 0 && N % 16 == 0 && N >= 16 && N <= 256, "tcgen05 tile shape");
    constexpr uint32_t kCols = tc_cols<N>();
    extern __shared__ __align__(128) uint8_t tc_smem[];
    uint8_t *sB = tc_smem;                          // N * K * 2
    uint8_t *sA = tc_smem + ((N * K * 2 + 127) / 128) * 128; // 2 x kTcRows * K * 2
    __shared__ __align__(8) uint64_t mbar;
    __shared__ uint32_t tmem_slot;
    const unsigned tid = threadIdx.x, warp = tid >> 5;
    const unsigned tiles = (R + kTcRows - 1) / kTcRows;
    const uint32_t mbar_a = (uint32_t)__cvta_generic_to_shared(&mbar);
    const uint32_t sa0 = (uint32_t)__cvta_generic_to_shared(sA);
    const uint32_t sb0 = (uint32_t)__cvta_generic_to_shared(sB);
    if (warp == 0) {
        const uint32_t slot = (uint32_t)__cvta_generic_to_shared(&tmem_slot);
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(slot),
                     "r"(kCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
    }
    if (tid == 0)
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(mbar_a) : "memory");
    constexpr int KV = K / 8;
    for (int t = tid; t < N * KV; t += 128) {
        const int n = t / KV, c = t % KV;
        *reinterpret_cast<uint4 *>(sB + c * N * 16 + n * 16) =
            __ldg(reinterpret_cast<const uint4 *>(B + (size_t)n * K + c * 8));
    }
    if (blockIdx.x < tiles) tc_fetch_tile<K>(sa0, A, R, blockIdx.x * kTcRows);
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    const uint32_t tmem = tmem_slot;
    const uint32_t idesc = (1u << 4)      // accumulator f32
                           | (1u << 7)    // A bf16
                           | (1u << 10)   // B bf16
                           | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(kTcRows >> 4) << 24);
    bool ok = true;
    unsigned i = 0;
    for (unsigned tile = blockIdx.x; tile < tiles && ok; tile += gridDim.x, ++i) {
        const uint32_t sa = sa0 + (i & 1u) * (kTcRows * K * 2);
        // this tile's rows have landed (this thread's copies), and every
        // thread's copies are visible to the tensor core's async proxy
        asm volatile("cp.async.wait_group 0;\n" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
        asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
        __syncthreads();
        asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
        if (tid == 0) {
#pragma unroll
            for (int s = 0; s < K / 16; ++s) {
                const uint64_t ad = tc_smem_desc(sa + s * 2 * 2048, 2048, 128);
                const uint64_t bd = tc_smem_desc(sb0 + s * 2 * N * 16, N * 16, 128);
                const uint32_t acc = s > 0 ? 1u : 0u;
                asm volatile(
                    "{\n .reg .pred p;\n setp.ne.u32 p, %4, 0;\n"
                    " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem),
                    "l"(ad), "l"(bd), "r"(idesc), "r"(acc)
                    : "memory");
            }
            asm volatile(
                "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(
                    mbar_a)
                : "memory");
        }
        // the next tile streams into the other buffer (its last reader, the
        // previous tile's MMAs, completed before that tile's epilogue)
        const unsigned next = tile + gridDim.x;
        if (next < tiles)
            tc_fetch_tile<K>(sa0 + ((i + 1) & 1u) * (kTcRows * K * 2), A, R, next * kTcRows);
        ok = __syncthreads_and(tc_wait(mbar_a, i & 1u, 1u << 22)) != 0;
        if (!ok) break;
        asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
        const unsigned row = tile * kTcRows + warp * 32 + (tid & 31u);
#pragma unroll
        for (int c = 0; c < N / 16; ++c) {
            uint32_t v[16];
            const uint32_t taddr = tmem + ((warp * 32u) << 16) + (uint32_t)(c * 16);
            asm volatile(
                "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,"
                "%12,%13,%14,%15}, [%16];\n"
                : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]),
                  "=r"(v[6]), "=r"(v[7]), "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]),
                  "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15])
                : "r"(taddr));
            asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
            if (row < R) {
                if (Cb) {
                    uint32_t pk[8];
#pragma unroll
                    for (int j = 0; j < 8; ++j) {
                        __nv_bfloat162 p;
                        p.x = __float2bfloat16_rn(fmaxf(__uint_as_float(v[2 * j]), 0.0f));
                        p.y = __float2bfloat16_rn(fmaxf(__uint_as_float(v[2 * j + 1]), 0.0f));
                        pk[j] = *reinterpret_cast<uint32_t *>(&p);
                    }
                    uint4 *dst = reinterpret_cast<uint4 *>(Cb + (size_t)row * N + c * 16);
                    dst[0] = make_uint4(pk[0], pk[1], pk[2], pk[3]);
                    dst[1] = make_uint4(pk[4], pk[5], pk[6], pk[7]);
                } else {
#pragma unroll
                    for (int j = 0; j < 16; j += 4)
                        *reinterpret_cast<float4 *>(Cf + (size_t)row * N + c * 16 + j) =
                            make_float4(__uint_as_float(v[j]), __uint_as_float(v[j + 1]),
                                        __uint_as_float(v[j + 2]), __uint_as_float(v[j + 3]));
                }
            }
        }
    }
    if (!ok) {
        if (tid == 0) atomicOr(&g_tc_status, 1u);
        tc_wait(mbar_a, (i & 1u), 1u << 22);
    }
    asm volatile("cp.async.wait_group 0;\n" ::: "memory");
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem),
                     "r"(kCols)
                     : "memory");
}

template <int K, int N> constexpr size_t tc_smem_bytes() {
    return ((size_t)(N * K * 2 + 127) / 128) * 128 + 2 * (size_t)kTcRows * K * 2;
}

bool g_use_tc = true; // forward row products on tcgen05 (else mma.sync)

constexpr unsigned kReduceRows = 1024; // rows per block in reduce mode
constexpr int kChunk = 32;             // rows staged per step

// C[M x N] += A[R x M]^T B[R x N] over rows [blockIdx.x * kReduceRows, ...).
template <int M, int N>
__global__ void __launch_bounds__(128) k_gemm_reduce(unsigned R, const bf16_t *__restrict__ A,
                                                     const bf16_t *__restrict__ B, float *C) {
    static_assert(M % 16 == 0 && N % 8 == 0, "tile shape");
    __shared__ __align__(16) bf16_t sAt[M][kChunk + 8];
    __shared__ __align__(16) bf16_t sBt[N][kChunk + 8];
    constexpr int kTiles = (M / 16) * (N / 8);
    constexpr int kPerWarp = (kTiles + 3) / 4;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, t4 = lane & 3;
    float acc[kPerWarp][4];
#pragma unroll
    for (int ti = 0; ti < kPerWarp; ++ti)
#pragma unroll
        for (int e = 0; e < 4; ++e) acc[ti][e] = 0.0f;
    const unsigned rb = blockIdx.x * kReduceRows;
    const unsigned re = min(R, rb + kReduceRows);
    for (unsigned r = rb; r < re; r += kChunk) {
        __syncthreads();
        for (int t = threadIdx.x; t < kChunk * (M / 8); t += 128) {
            const int rr = t / (M / 8), c = (t % (M / 8)) * 8;
            uint4 v = make_uint4(0u, 0u, 0u, 0u);
            if (r + rr < re) v = __ldg(reinterpret_cast<const uint4 *>(A + (size_t)(r + rr) * M + c));
            const bf16_t *e = reinterpret_cast<const bf16_t *>(&v);
#pragma unroll
            for (int j = 0; j < 8; ++j) sAt[c + j][rr] = e[j];
        }
        for (int t = threadIdx.x; t < kChunk * (N / 8); t += 128) {
            const int rr = t / (N / 8), c = (t % (N / 8)) * 8;
            uint4 v = make_uint4(0u, 0u, 0u, 0u);
            if (r + rr < re) v = __ldg(reinterpret_cast<const uint4 *>(B + (size_t)(r + rr) * N + c));
            const bf16_t *e = reinterpret_cast<const bf16_t *>(&v);
#pragma unroll
            for (int j = 0; j < 8; ++j) sBt[c + j][rr] = e[j];
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < kChunk; kk += 16) {
#pragma unroll
            for (int ti = 0; ti < kPerWarp; ++ti) {
                const int tile = warp + 4 * ti;
                if (tile >= kTiles) continue;
                const int mt = tile / (N / 8), nt = tile % (N / 8);
                uint32_t a[4], b[2];
                a[0] = ld_pair(&sAt[mt * 16 + g][kk + 2 * t4]);
                a[1] = ld_pair(&sAt[mt * 16 + g + 8][kk + 2 * t4]);
                a[2] = ld_pair(&sAt[mt * 16 + g][kk + 8 + 2 * t4]);
                a[3] = ld_pair(&sAt[mt * 16 + g + 8][kk + 8 + 2 * t4]);
                b[0] = ld_pair(&sBt[nt * 8 + g][kk + 2 * t4]);
                b[1] = ld_pair(&sBt[nt * 8 + g][kk + 8 + 2 * t4]);
                mma16816(acc[ti], a, b);
            }
        }
    }
#pragma unroll
    for (int ti = 0; ti < kPerWarp; ++ti) {
        const int tile = warp + 4 * ti;
        if (tile >= kTiles) continue;
        const int mt = tile / (N / 8), nt = tile % (N / 8);
        const int m = mt * 16 + g, c = nt * 8 + 2 * t4;
        atomicAdd(C + (size_t)m * N + c, acc[ti][0]);
        atomicAdd(C + (size_t)m * N + c + 1, acc[ti][1]);
        atomicAdd(C + (size_t)(m + 8) * N + c, acc[ti][2]);
        atomicAdd(C + (size_t)(m + 8) * N + c + 1, acc[ti][3]);
    }
}

template <int K, int N>
void gemm_rows(unsigned R, const bf16_t *A, const bf16_t *B, float *Cf, bf16_t *Cb,
               cudaStream_t q) {
    if (!R) return;
    k_gemm_rows<K, N><<<div_up(R, kRowsTile), 128, 0, q>>>(R, A, B, Cf, Cb);
    PPF_LAUNCH_CHECK();
}

// The forward layers' products: tcgen05 tiles (N a multiple of 16), or the
// mma.sync tiles when the tensor path is switched off.
template <int K, int N>
void gemm_fwd(unsigned R, const bf16_t *A, const bf16_t *B, float *Cf, bf16_t *Cb,
              cudaStream_t q) {
    if (!R) return;
    if (g_use_tc) {
        constexpr size_t smem = tc_smem_bytes<K, N>();
        static bool configured = false;
        if (!configured) {
            PPF_CUDA(cudaFuncSetAttribute(k_gemm_rows_tc<K, N>,
                                          cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          (int)smem));
            configured = true;
        }
        const unsigned grid = std::min(div_up(R, kTcRows), kNumSMs * kTcCtasPerSm);
        k_gemm_rows_tc<K, N><<<grid, 128, smem, q>>>(R, A, B, Cf, Cb);
        PPF_LAUNCH_CHECK();
    } else {
        gemm_rows<K, N>(R, A, B, Cf, Cb, q);
    }
}

template <int M, int N>
void gemm_reduce(unsigned R, const bf16_t *A, const bf16_t *B, float *C, cudaStream_t q) {
    if (!R) return;
    k_gemm_reduce<M, N><<<div_up(R, kReduceRows), 128, 0, q>>>(R, A, B, C);
    PPF_LAUNCH_CHECK();
}

} // namespace

void LearnedNodes::reserve(unsigned n) {
    X0.reserve((size_t)n * kIn0);
    H.reserve((size_t)4 * n * 32);
    X.reserve((size_t)3 * n * kInL);
    Xh.reserve((size_t)n * kInH);
    deg.reserve(n);
    Y.reserve((size_t)n * kOutH);
}

void learned_forward_nodes(const LearnedGraph &g, const bf16_t *w, LearnedNodes &b,
                           cudaStream_t q) {
    const unsigned n = g.n;
    b.reserve(n);
    k_node_inputs<<<div_up(n, kT), kT, 0, q>>>(g, b.X0.data(), b.deg.data());
    PPF_LAUNCH_CHECK();
    bf16_t *H = b.H.data();
    gemm_fwd<kIn0, 32>(n, b.X0.data(), w + kOffW0, nullptr, H, q);
    for (int l = 0; l < 3; ++l) {
        bf16_t *X = b.X.data() + (size_t)l * n * kInL;
        k_aggregate<true><<<div_up(32u * n, kT), kT, 0, q>>>(g, H + (size_t)l * n * 32,
                                                             b.deg.data(), X);
        PPF_LAUNCH_CHECK();
        gemm_fwd<kInL, 32>(n, X, w + kOffW1 + l * 32 * kInL, nullptr,
                           H + (size_t)(l + 1) * n * 32, q);
    }
    k_aggregate<false><<<div_up(32u * n, kT), kT, 0, q>>>(g, H + (size_t)3 * n * 32,
                                                          b.deg.data(), b.Xh.data());
    PPF_LAUNCH_CHECK();
    gemm_fwd<kInH, kOutH>(n, b.Xh.data(), w + kOffWh, b.Y.data(), nullptr, q);
}

// ---- training ------------------------------------------------------------------------------
namespace {

struct Sample {
    unsigned n = 0, nnz_f = 0, nnz_c = 0, n_free = 0;
    DevBuf<unsigned> f_off, f_col, f_troff, f_row, c_off, c_col, c_troff, c_row, diag_slot, dof;
    DevBuf<uint2> f_tr, c_tr;
    DevBuf<float> f_val, c_val, mass, cinv;
    DevBuf<unsigned> status;
    LearnedGraph graph() const {
        LearnedGraph g;
        g.n = n;
        g.fixed = LearnedPart{f_off.data(), f_col.data(), f_val.data(), f_troff.data(),
                              f_tr.data(), nnz_f};
        g.contact = LearnedPart{c_off.data(), c_col.data(), c_val.data(), c_troff.data(),
                                c_tr.data(), nnz_c};
        g.diag_slot = diag_slot.data();
        g.dof_mask = dof.data();
        g.mass = mass.data();
        g.cinv = cinv.data();
        return g;
    }
};

struct TrainWork {
    LearnedNodes nodes;
    DevBuf<bf16_t> wt;             // transposed W1..W3 (3 x 80 x 32) and Wh (48 x 80)
    DevBuf<float> ah, alpha, go;   // per edge
    DevBuf<float> gz;              // per edge x 32
    DevBuf<bf16_t> gzb, F;         // per edge x 32, x 16
    DevBuf<float> u, v;            // probes x n x 3
    DevBuf<float> gY, gX;          // n x 80
    DevBuf<bf16_t> gYb, gZ;        // n x 80, n x 32
    DevBuf<float> partial, scal;
};

std::vector<Sample *> g_samples;
TrainWork g_work;

template <class T> void upload_vec(DevBuf<T> &b, const std::vector<T> &h) {
    b.reserve(h.size() + 1);
    if (!h.empty())
        PPF_CUDA(cudaMemcpy(b.data(), h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice));
}

void transpose_list(unsigned n, const unsigned *off, const unsigned *col,
                    std::vector<unsigned> &tr_off, std::vector<uint2> &tr,
                    std::vector<unsigned> &row) {
    const unsigned nnz = off[n];
    std::vector<unsigned> cnt(n + 1, 0u);
    row.assign(nnz, 0u);
    for (unsigned i = 0; i < n; ++i)
        for (unsigned k = off[i]; k < off[i + 1]; ++k) {
            row[k] = i;
            if (col[k] != i) cnt[col[k] + 1]++;
        }
    tr_off.assign(n + 1, 0u);
    for (unsigned i = 0; i < n; ++i) tr_off[i + 1] = tr_off[i] + cnt[i + 1];
    tr.assign(tr_off[n], make_uint2(0u, 0u));
    std::vector<unsigned> fill(tr_off.begin(), tr_off.end() - 1);
    for (unsigned i = 0; i < n; ++i)
        for (unsigned k = off[i]; k < off[i + 1]; ++k)
            if (col[k] != i) tr[fill[col[k]]++] = make_uint2(i, k);
}

__global__ void k_transpose_weights(const bf16_t *w, bf16_t *wt) {
    const unsigned t = blockIdx.x * blockDim.x + threadIdx.x;
    // W_l^T: [80][32] from W_l [32][80], l = 0..2; Wh^T: [48][80] from Wh [80][48]
    if (t < 3u * 32u * kInL) {
        const unsigned l = t / (32u * kInL), r = t % (32u * kInL);
        const unsigned o = r / kInL, i = r % kInL;
        wt[l * 32 * kInL + i * 32 + o] = w[kOffW1 + l * 32 * kInL + o * kInL + i];
    } else if (t < 3u * 32u * kInL + kOutH * kInH) {
        const unsigned r = t - 3u * 32u * kInL;
        const unsigned o = r / kInH, i = r % kInH;
        wt[3u * 32u * kInL + i * kOutH + o] = w[kOffWh + o * kInH + i];
    }
}

// Per edge (upper entry): Â(hi, lo), features, alpha (0 when not live).
__global__ void k_edge_forward(LearnedGraph g, const unsigned *f_row, const unsigned *c_row,
                               const float *Y, const bf16_t *w, float *ah_out, bf16_t *F,
                               float *alpha) {
    const unsigned e = blockIdx.x * blockDim.x + threadIdx.x;
    const unsigned E = g.fixed.nnz + g.contact.nnz;
    if (e >= E) return;
    const bool fx = e < g.fixed.nnz;
    const unsigned k = fx ? e : e - g.fixed.nnz;
    const LearnedPart &P = fx ? g.fixed : g.contact;
    const unsigned lo = __ldg((fx ? f_row : c_row) + k), hi = __ldg(P.col + k);
    const bool live = lo != hi && !__ldg(g.dof_mask + lo) && !__ldg(g.dof_mask + hi);
    Mat3 ah = Mat3::zero();
    float a = 0.0f;
    float f[11];
#pragma unroll
    for (int c = 0; c < 11; ++c) f[c] = 0.0f;
    if (live) {
        ah = learned_edge_ahat(ld_blk(g.cinv + 9 * (size_t)hi), ld_blk(g.cinv + 9 * (size_t)lo),
                               ld_blk(P.val + 9 * (size_t)k));
        learned_edge_features(ah, f);
        a = learned_alpha_of(learned_edge_o(Y, w, hi, lo, ah));
    }
#pragma unroll
    for (int c = 0; c < 9; ++c) ah_out[9 * (size_t)e + c] = ah.m[c];
#pragma unroll
    for (int c = 0; c < (int)kInF; ++c)
        F[(size_t)e * kInF + c] = __float2bfloat16_rn(c < 11 ? f[c] : 0.0f);
    alpha[e] = a;
}

__device__ __forceinline__ Vec3 ld_vec(const float *p) { return vec3(p[0], p[1], p[2]); }

__device__ __forceinline__ float probe_w(const float *probes, unsigned n, unsigned w, unsigned i,
                                         int c) {
    return __ldg(probes + ((size_t)w * n + i) * 3 + c);
}

// u = Ĝ^T w for every probe: u_i = d_i w_i + sum over upper entries (i = lo)
// of (-alpha Â(hi, i))^T w_hi.
__global__ void k_probe_u(LearnedGraph g, const float *Y, const float *ah, const float *alpha,
                          const float *probes, unsigned W, float *u) {
    const unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= g.n) return;
    const bool free = !__ldg(g.dof_mask + i);
    const float d = free ? learned_diag_scale(Y, i) : 0.0f;
    for (unsigned w = 0; w < W; ++w) {
        Vec3 acc = vec3(0.0f, 0.0f, 0.0f);
        if (free) {
#pragma unroll
            for (int c = 0; c < 3; ++c) acc[c] = d * probe_w(probes, g.n, w, i, c);
            walk_neighbours(g, i, [&](unsigned j, const float *, bool i_is_lo, int, unsigned e) {
                if (!i_is_lo) return;
                const Mat3 m = ld_blk(ah + 9 * (size_t)e);
                const float a = __ldg(alpha + e);
                Vec3 wj;
#pragma unroll
                for (int c = 0; c < 3; ++c) wj[c] = probe_w(probes, g.n, w, j, c);
                const Vec3 t = m.transpose() * wj;
#pragma unroll
                for (int c = 0; c < 3; ++c) acc[c] = acc[c] - a * t[c];
            });
        }
#pragma unroll
        for (int c = 0; c < 3; ++c) u[((size_t)w * g.n + i) * 3 + c] = acc[c];
    }
}

// v = Â u; per-block partials of sum_w u . v and of sum ln d (free vertices).
__global__ void k_probe_v(LearnedGraph g, const float *Y, const float *ah, const float *u,
                          unsigned W, float *v, float *partial) {
    const unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
    float dot = 0.0f, lnd = 0.0f;
    if (i < g.n) {
        const bool free = !__ldg(g.dof_mask + i);
        Mat3 aii = Mat3::zero();
        if (free) {
            const Mat3 C = ld_blk(g.cinv + 9 * (size_t)i);
            aii = (C * ld_blk(g.fixed.val + 9 * (size_t)__ldg(g.diag_slot + i))) * C.transpose();
            const float q = __ldg(Y + (size_t)i * kOutH + 64);
            lnd = fminf(fmaxf(q, -kClampQ), kClampQ);
        }
        for (unsigned w = 0; w < W; ++w) {
            const float *uw = u + (size_t)w * g.n * 3;
            Vec3 acc = vec3(0.0f, 0.0f, 0.0f);
            if (free) {
                acc = aii * ld_vec(uw + 3 * (size_t)i);
                walk_neighbours(g, i, [&](unsigned j, const float *, bool i_is_lo, int,
                                          unsigned e) {
                    const Mat3 m = ld_blk(ah + 9 * (size_t)e);
                    const Vec3 t = i_is_lo ? m.transpose() * ld_vec(uw + 3 * (size_t)j)
                                           : m * ld_vec(uw + 3 * (size_t)j);
#pragma unroll
                    for (int c = 0; c < 3; ++c) acc[c] = acc[c] + t[c];
                });
            }
            const Vec3 ui = ld_vec(uw + 3 * (size_t)i);
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                v[((size_t)w * g.n + i) * 3 + c] = acc[c];
                dot = dot + ui[c] * acc[c];
            }
        }
    }
    __shared__ float s_dot[kT], s_lnd[kT];
    s_dot[threadIdx.x] = dot;
    s_lnd[threadIdx.x] = lnd;
    __syncthreads();
    for (unsigned s = kT / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) {
            s_dot[threadIdx.x] += s_dot[threadIdx.x + s];
            s_lnd[threadIdx.x] += s_lnd[threadIdx.x + s];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        partial[2 * blockIdx.x] = s_dot[0];
        partial[2 * blockIdx.x + 1] = s_lnd[0];
    }
}

// scal = {T, L, c = 2 / (W T), n_free}, partials folded in block order.
__global__ void k_probe_finish(const float *partial, unsigned blocks, unsigned W,
                               unsigned n_free, float *scal) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    float dot = 0.0f, lnd = 0.0f;
    for (unsigned b = 0; b < blocks; ++b) {
        dot += partial[2 * b];
        lnd += partial[2 * b + 1];
    }
    const float T = dot / (float)W;
    const float nf = (float)n_free;
    scal[0] = T;
    scal[1] = logf(T / (3.0f * nf)) - 2.0f / nf * lnd;
    scal[2] = 2.0f / ((float)W * T);
    scal[3] = nf;
}

// Per edge: d L / d o, then the edge head's backward pass: gz (fp32 and bf16)
// and the gradient of wo.
__global__ void k_edge_backward(LearnedGraph g, const unsigned *f_row, const unsigned *c_row,
                                const float *Y, const bf16_t *w, const float *ah,
                                const float *alpha, const bf16_t *F, const float *probes,
                                const float *v, unsigned W, const float *scal, float *gz,
                                bf16_t *gzb, float *grad) {
    const unsigned e = blockIdx.x * blockDim.x + threadIdx.x;
    const unsigned E = g.fixed.nnz + g.contact.nnz;
    float go = 0.0f;
    float z[32];
#pragma unroll
    for (int k = 0; k < 32; ++k) z[k] = 0.0f;
    if (e < E) {
        const bool fx = e < g.fixed.nnz;
        const unsigned k = fx ? e : e - g.fixed.nnz;
        const LearnedPart &P = fx ? g.fixed : g.contact;
        const unsigned lo = __ldg((fx ? f_row : c_row) + k), hi = __ldg(P.col + k);
        const bool live = lo != hi && !__ldg(g.dof_mask + lo) && !__ldg(g.dof_mask + hi);
        if (live) {
            const Mat3 m = ld_blk(ah + 9 * (size_t)e);
            float s = 0.0f;
            for (unsigned wi = 0; wi < W; ++wi) {
                Vec3 wh;
#pragma unroll
                for (int c = 0; c < 3; ++c) wh[c] = probe_w(probes, g.n, wi, hi, c);
                const Vec3 t = m * ld_vec(v + ((size_t)wi * g.n + lo) * 3);
                s = s + ((wh[0] * t[0] + wh[1] * t[1]) + wh[2] * t[2]);
            }
            const float a = __ldg(alpha + e);
            go = -__ldg(scal + 2) * s * a * (1.0f - 0.5f * a);
            float f[11];
#pragma unroll
            for (int c = 0; c < 11; ++c) f[c] = __bfloat162float(F[(size_t)e * kInF + c]);
#pragma unroll
            for (int kk = 0; kk < 32; ++kk) z[kk] = learned_edge_z(Y, w, hi, lo, f, kk);
        }
#pragma unroll
        for (int kk = 0; kk < 32; ++kk) {
            const float gk = z[kk] > 0.0f ? go * __bfloat162float(w[kOffWo + kk]) : 0.0f;
            gz[(size_t)e * 32 + kk] = gk;
            gzb[(size_t)e * 32 + kk] = __float2bfloat16_rn(gk);
        }
    }
    // grad of wo: sum over edges of go z_k, and of go (bias); warp sums, then atomics
    const unsigned lane = threadIdx.x & 31u;
#pragma unroll
    for (int kk = 0; kk < 33; ++kk) {
        float val = kk < 32 ? go * z[kk] : go;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) val += __shfl_xor_sync(0xffffffffu, val, o);
        if (lane == 0 && val != 0.0f) atomicAdd(grad + kOffWo + kk, val);
    }
}

// gY (fp32 and bf16): per vertex, the edge head's gz summed over its edges
// (as hi into columns 0..31, as lo into 32..63) and d L / d q in column 64.
// One warp per vertex, lane = unit.
__global__ void k_node_grad_y(LearnedGraph g, const float *Y, const float *gz,
                              const float *probes, const float *v, unsigned W, const float *scal,
                              float *gY, bf16_t *gYb) {
    const unsigned i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, k = threadIdx.x & 31u;
    if (i >= g.n) return;
    float ahi = 0.0f, alo = 0.0f;
    walk_neighbours(g, i, [&](unsigned, const float *, bool i_is_lo, int, unsigned e) {
        const float x = gz[(size_t)e * 32 + k];
        if (i_is_lo) alo = alo + x;
        else ahi = ahi + x;
    });
    float *row = gY + (size_t)i * kOutH;
    bf16_t *rowb = gYb + (size_t)i * kOutH;
    row[k] = ahi;
    row[32 + k] = alo;
    rowb[k] = __float2bfloat16_rn(ahi);
    rowb[32 + k] = __float2bfloat16_rn(alo);
    if (k < 16) {
        float gq = 0.0f;
        if (k == 0 && !__ldg(g.dof_mask + i)) {
            const float q = __ldg(Y + (size_t)i * kOutH + 64);
            if (fabsf(q) <= kClampQ) {
                float s = 0.0f;
                for (unsigned wi = 0; wi < W; ++wi)
                    for (int c = 0; c < 3; ++c)
                        s = s + probe_w(probes, g.n, wi, i, c) * v[((size_t)wi * g.n + i) * 3 + c];
                gq = learned_diag_scale(Y, i) * __ldg(scal + 2) * s - 2.0f / __ldg(scal + 3);
            }
        }
        row[64 + k] = gq;
        rowb[64 + k] = __float2bfloat16_rn(gq);
    }
}

// gZ = bf16(gH * [H > 0]) with gH = gX[:, 0:32] (+ the neighbour-mean
// backward: sum over neighbours j of gX[j, 32:64] / deg_j). One warp per
// vertex, lane = unit; gX has row stride ld.
template <bool kMean>
__global__ void k_relu_backward(LearnedGraph g, const float *gX, unsigned ld, const float *deg,
                                const bf16_t *H, bf16_t *gZ) {
    const unsigned i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, k = threadIdx.x & 31u;
    if (i >= g.n) return;
    float gh = gX[(size_t)i * ld + k];
    if (kMean) {
        float acc = 0.0f;
        walk_neighbours(g, i, [&](unsigned j, const float *, bool, int, unsigned) {
            acc = acc + gX[(size_t)j * ld + 32 + k] / deg[j];
        });
        gh = gh + acc;
    }
    const float h = __bfloat162float(H[(size_t)i * 32 + k]);
    gZ[(size_t)i * 32 + k] = __float2bfloat16_rn(h > 0.0f ? gh : 0.0f);
}

Sample *sample_at(int s) {
    if (s < 0 || s >= (int)g_samples.size() || !g_samples[s]) return nullptr;
    return g_samples[s];
}

// Edge-level and vertex-level forward of sample S into g_work.
void forward_all(Sample &S, const bf16_t *w, cudaStream_t q) {
    const LearnedGraph g = S.graph();
    learned_forward_nodes(g, w, g_work.nodes, q);
    const unsigned E = S.nnz_f + S.nnz_c;
    g_work.ah.reserve(9 * (size_t)E + 1);
    g_work.alpha.reserve(E + 1);
    g_work.F.reserve((size_t)E * kInF + 1);
    if (E) {
        k_edge_forward<<<div_up(E, kT), kT, 0, q>>>(g, S.f_row.data(), S.c_row.data(),
                                                    g_work.nodes.Y.data(), w, g_work.ah.data(),
                                                    g_work.F.data(), g_work.alpha.data());
        PPF_LAUNCH_CHECK();
    }
}

} // namespace

int learned_add_sample(unsigned n, const unsigned *f_off, const unsigned *f_col,
                       const float *f_val, const unsigned *c_off, const unsigned *c_col,
                       const float *c_val, const unsigned *dof_mask, const float *mass) {
    if (!n || !f_off || !f_col || !f_val || !dof_mask || !mass) return -1;
    Sample *S = new Sample();
    S->n = n;
    S->nnz_f = f_off[n];
    std::vector<unsigned> zeros(n + 1, 0u);
    const unsigned *co = c_off ? c_off : zeros.data();
    S->nnz_c = co[n];
    if (S->nnz_c && (!c_col || !c_val)) {
        delete S;
        return -1;
    }
    std::vector<unsigned> diag(n, 0xffffffffu);
    for (unsigned i = 0; i < n; ++i)
        for (unsigned k = f_off[i]; k < f_off[i + 1]; ++k)
            if (f_col[k] == i) diag[i] = k;
    for (unsigned i = 0; i < n; ++i)
        if (diag[i] == 0xffffffffu) {
            delete S;
            return -1; // every vertex needs its diagonal block
        }
    std::vector<unsigned> troff, row;
    std::vector<uint2> tr;
    transpose_list(n, f_off, f_col, troff, tr, row);
    upload_vec(S->f_off, std::vector<unsigned>(f_off, f_off + n + 1));
    upload_vec(S->f_col, std::vector<unsigned>(f_col, f_col + S->nnz_f));
    upload_vec(S->f_val, std::vector<float>(f_val, f_val + 9 * (size_t)S->nnz_f));
    upload_vec(S->f_troff, troff);
    upload_vec(S->f_tr, tr);
    upload_vec(S->f_row, row);
    std::vector<unsigned> ccol(S->nnz_c ? c_col : nullptr, S->nnz_c ? c_col + S->nnz_c : nullptr);
    transpose_list(n, co, ccol.data(), troff, tr, row);
    upload_vec(S->c_off, std::vector<unsigned>(co, co + n + 1));
    upload_vec(S->c_col, ccol);
    upload_vec(S->c_val, S->nnz_c ? std::vector<float>(c_val, c_val + 9 * (size_t)S->nnz_c)
                                  : std::vector<float>());
    upload_vec(S->c_troff, troff);
    upload_vec(S->c_tr, tr);
    upload_vec(S->c_row, row);
    upload_vec(S->diag_slot, diag);
    std::vector<unsigned> dof(dof_mask, dof_mask + n);
    S->n_free = 0;
    for (unsigned i = 0; i < n; ++i) S->n_free += dof[i] ? 0u : 1u;
    if (!S->n_free) {
        delete S;
        return -1;
    }
    upload_vec(S->dof, dof);
    upload_vec(S->mass, std::vector<float>(mass, mass + n));
    S->cinv.reserve(9 * (size_t)n);
    S->status.reserve(1);
    PPF_CUDA(cudaMemset(S->status.data(), 0, sizeof(unsigned)));
    launch_chol_inv(n, S->f_val.data(), S->diag_slot.data(), S->cinv.data(), S->status.data(),
                    0);
    PPF_CUDA(cudaDeviceSynchronize());
    g_samples.push_back(S);
    return (int)g_samples.size() - 1;
}

void learned_clear_samples() {
    PPF_CUDA(cudaDeviceSynchronize());
    for (Sample *S : g_samples) {
        if (!S) continue;
        for (DevBuf<unsigned> *b : {&S->f_off, &S->f_col, &S->f_troff, &S->f_row, &S->c_off,
                                    &S->c_col, &S->c_troff, &S->c_row, &S->diag_slot, &S->dof,
                                    &S->status})
            b->release();
        S->f_tr.release();
        S->c_tr.release();
        S->f_val.release();
        S->c_val.release();
        S->mass.release();
        S->cinv.release();
        delete S;
    }
    g_samples.clear();
}

int learned_tensor_path(int tc) {
    const int prev = g_use_tc ? 1 : 0;
    if (tc >= 0) g_use_tc = tc != 0;
    return prev;
}

unsigned learned_tc_status() {
    unsigned v = 0;
    PPF_CUDA(cudaMemcpyFromSymbol(&v, g_tc_status, sizeof(v)));
    return v;
}

int learned_sample_info(int s, unsigned *n, unsigned *edges, unsigned *n_free) {
    Sample *S = sample_at(s);
    if (!S) return -1;
    if (n) *n = S->n;
    if (edges) *edges = S->nnz_f + S->nnz_c;
    if (n_free) *n_free = S->n_free;
    return 0;
}

int learned_forward(int s, const bf16_t *d_w, float *h_alpha, float *h_d) {
    Sample *S = sample_at(s);
    if (!S || !d_w) return -1;
    forward_all(*S, d_w, 0);
    PPF_CUDA(cudaDeviceSynchronize());
    const unsigned E = S->nnz_f + S->nnz_c;
    if (h_alpha && E)
        PPF_CUDA(cudaMemcpy(h_alpha, g_work.alpha.data(), E * sizeof(float),
                            cudaMemcpyDeviceToHost));
    if (h_d) {
        std::vector<float> Y((size_t)S->n * kOutH);
        PPF_CUDA(cudaMemcpy(Y.data(), g_work.nodes.Y.data(), Y.size() * sizeof(float),
                            cudaMemcpyDeviceToHost));
        for (unsigned i = 0; i < S->n; ++i) h_d[i] = Y[(size_t)i * kOutH + 64];
    }
    return 0;
}

int learned_loss_grad(int s, const bf16_t *d_w, const float *d_probes, unsigned W,
                      float *d_grad, float *h_loss, cudaStream_t q) {
    Sample *S = sample_at(s);
    if (!S || !d_w || !d_probes || !d_grad || W == 0) return -1;
    const LearnedGraph g = S->graph();
    const unsigned n = S->n, E = S->nnz_f + S->nnz_c;
    TrainWork &T = g_work;
    forward_all(*S, d_w, q);
    T.wt.reserve(3 * 32 * kInL + kOutH * kInH);
    k_transpose_weights<<<div_up(3u * 32u * kInL + kOutH * kInH, kT), kT, 0, q>>>(d_w,
                                                                                T.wt.data());
    PPF_LAUNCH_CHECK();
    // probes
    T.u.reserve((size_t)W * n * 3);
    T.v.reserve((size_t)W * n * 3);
    const unsigned blocks = div_up(n, kT);
    T.partial.reserve(2 * (size_t)blocks);
    T.scal.reserve(4);
    const float *Y = T.nodes.Y.data();
    k_probe_u<<<blocks, kT, 0, q>>>(g, Y, T.ah.data(), T.alpha.data(), d_probes, W, T.u.data());
    PPF_LAUNCH_CHECK();
    k_probe_v<<<blocks, kT, 0, q>>>(g, Y, T.ah.data(), T.u.data(), W, T.v.data(),
                                    T.partial.data());
    PPF_LAUNCH_CHECK();
    k_probe_finish<<<1, 32, 0, q>>>(T.partial.data(), blocks, W, S->n_free, T.scal.data());
    PPF_LAUNCH_CHECK();
    // backward
    PPF_CUDA(cudaMemsetAsync(d_grad, 0, kWeights * sizeof(float), q));
    T.gz.reserve((size_t)E * 32 + 1);
    T.gzb.reserve((size_t)E * 32 + 1);
    if (E) {
        k_edge_backward<<<div_up(E, kT), kT, 0, q>>>(
            g, S->f_row.data(), S->c_row.data(), Y, d_w, T.ah.data(), T.alpha.data(),
            T.F.data(), d_probes, T.v.data(), W, T.scal.data(), T.gz.data(), T.gzb.data(),
            d_grad);
        PPF_LAUNCH_CHECK();
    }
    T.gY.reserve((size_t)n * kOutH);
    T.gYb.reserve((size_t)n * kOutH);
    T.gX.reserve((size_t)n * kOutH);
    T.gZ.reserve((size_t)n * 32);
    k_node_grad_y<<<div_up(32u * n, kT), kT, 0, q>>>(g, Y, T.gz.data(), d_probes, T.v.data(), W,
                                                     T.scal.data(), T.gY.data(), T.gYb.data());
    PPF_LAUNCH_CHECK();
    gemm_reduce<32, kInF>(E, T.gzb.data(), T.F.data(), d_grad + kOffWf, q);
    gemm_reduce<kOutH, kInH>(n, T.gYb.data(), T.nodes.Xh.data(), d_grad + kOffWh, q);
    const bf16_t *wt = T.wt.data();
    gemm_rows<kOutH, kInH>(n, T.gYb.data(), wt + 3 * 32 * kInL, T.gX.data(), nullptr, q);
    const bf16_t *H = T.nodes.H.data();
    k_relu_backward<false><<<div_up(32u * n, kT), kT, 0, q>>>(
        g, T.gX.data(), kInH, T.nodes.deg.data(), H + (size_t)3 * n * 32, T.gZ.data());
    PPF_LAUNCH_CHECK();
    for (int l = 2; l >= 0; --l) {
        const bf16_t *X = T.nodes.X.data() + (size_t)l * n * kInL;
        gemm_reduce<32, kInL>(n, T.gZ.data(), X, d_grad + kOffW1 + l * 32 * kInL, q);
        gemm_rows<32, kInL>(n, T.gZ.data(), wt + l * 32 * kInL, T.gX.data(), nullptr, q);
        k_relu_backward<true><<<div_up(32u * n, kT), kT, 0, q>>>(
            g, T.gX.data(), kInL, T.nodes.deg.data(), H + (size_t)l * n * 32, T.gZ.data());
        PPF_LAUNCH_CHECK();
    }
    gemm_reduce<32, kIn0>(n, T.gZ.data(), T.nodes.X0.data(), d_grad + kOffW0, q);
    float scal[4];
    PPF_CUDA(cudaMemcpyAsync(scal, T.scal.data(), sizeof(scal), cudaMemcpyDeviceToHost, q));
    PPF_CUDA(cudaStreamSynchronize(q));
    if (h_loss) *h_loss = scal[1];
    return 0;
}

} // namespace gpu
} // namespace ppf
