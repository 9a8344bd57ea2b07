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
// would need before the next product. For that, each vertex's z and p sit
// in one 32-byte record {z, p} that its owner rewrites at the end of the
// update phase; a neighbour gather is one 256-bit load of the record (one L2
// sector), and the owner keeps the p of the current iteration in a separate
// buffer until then. Values another block wrote during the launch are read
// with ld.cg (from L2, never a line an SM's L1 kept from an earlier phase).
// The operator is read-only inside the launch and goes through the
// non-coherent path.
#include "../physics/eig.cuh"
#include "assemble.cuh"
#include "fatal.cuh"
#include "pcg.cuh"

#include <algorithm>

namespace ppf {
namespace gpu {

namespace {

constexpr unsigned kThreads = 1024; // one block per SM (the largest block; a
                                    // one-cluster solve may run smaller ones)
constexpr unsigned kWarps = kThreads / 32;
static_assert(kWarps == 32, "the block fold reads one partial per lane of warp 0");
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

__device__ __forceinline__ unsigned ld_acquire(const unsigned *p) {
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ unsigned ld_relaxed(const unsigned *p) {
    unsigned v;
    asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ unsigned atom_add_acq_rel(unsigned *p, unsigned v) {
    unsigned old;
    asm volatile("atom.acq_rel.gpu.global.add.u32 %0, [%1], %2;"
                 : "=r"(old)
                 : "l"(p), "r"(v)
                 : "memory");
    return old;
}
__device__ __forceinline__ void red_add_release(unsigned *p, unsigned v) {
    asm volatile("red.release.gpu.global.add.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ void st_relaxed(unsigned *p, unsigned v) {
    asm volatile("st.relaxed.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// Grid-wide sum of N values for a cooperative launch (all blocks
// co-resident). Each block folds its threads' values (fixed shuffle order),
// lane 0 of warp 0 stores the block's partials and arrives at the grid
// barrier with acquire-release semantics (ordering the partials before the
// arrival); the last block to arrive resets the counter and releases the
// generation word, the others wait for it with acquire loads. Warp 0 then
// folds every block's partials in block order, so every block obtains the
// same bits. `part` alternates between two buffers from one reduction to the
// next, so a fast block never overwrites partials still being read.
//
// The wait is bounded in wall time: a timeout (or an abort latched by
// another block) sets STATUS_PCG_BREAKDOWN in `abort`, and every block
// leaves the solve instead of waiting again.
// partials a lane folds with its loads in flight together (grids up to
// 32 * kFoldLoads blocks)
constexpr unsigned kFoldLoads = 5;

// Arrival at and wait on the cluster's hardware barrier by every thread,
// release and acquire at cluster scope (orders the partials stored before it
// for the other CTAs' L2 loads after it).
__device__ __forceinline__ void cluster_barrier() {
    asm volatile("barrier.cluster.arrive.release;\n\tbarrier.cluster.wait.acquire;" ::: "memory");
}

// Folds the first n of the N-value partials at p (lane k holds entries k,
// k + 32, ...), the loads in flight together, in a fixed order: every block
// that folds the same partials gets the same bits. Result on lane 0.
template <int N>
__device__ __forceinline__ void fold_partials(const float *p, unsigned n, unsigned lane,
                                              float (&x)[N]) {
#pragma unroll
    for (int q = 0; q < N; ++q) x[q] = 0.0f;
    if (n <= 32u * kFoldLoads) {
        float pv[kFoldLoads][N];
#pragma unroll
        for (unsigned j = 0; j < kFoldLoads; ++j) {
            const unsigned k = lane + 32u * j;
#pragma unroll
            for (int q = 0; q < N; ++q) pv[j][q] = k < n ? __ldcg(p + N * k + q) : 0.0f;
        }
#pragma unroll
        for (unsigned j = 0; j < kFoldLoads; ++j)
            if (lane + 32u * j < n)
#pragma unroll
                for (int q = 0; q < N; ++q) x[q] += pv[j][q];
    } else {
        for (unsigned k = lane; k < n; k += 32)
#pragma unroll
            for (int q = 0; q < N; ++q) x[q] += __ldcg(p + N * k + q);
    }
    for (int off = 16; off > 0; off >>= 1)
#pragma unroll
        for (int q = 0; q < N; ++q) x[q] += __shfl_down_sync(0xffffffffu, x[q], off);
}

// The bounded wait for the generation word to move past g0. Returns 0 when
// it timed out or another block latched an abort.
__device__ __forceinline__ int grid_wait(unsigned *gen, unsigned g0, unsigned *abort) {
    const unsigned long long t0 = global_ns();
    for (unsigned spin = 0; ld_acquire(gen) == g0; ++spin) {
        if ((spin & 63u) == 63u) {
            if (ld_relaxed(abort) || global_ns() - t0 > kBarrierTimeoutNs) {
                atomicOr(abort, STATUS_PCG_BREAKDOWN);
                return 0;
            }
        }
    }
    return 1;
}

// The barrier has two forms, by `cluster` (the launch's cluster size):
//   0          every block's lane 0 arrives at the grid barrier through L2
//              and folds all blocks' partials;
//   gridDim.x  the launch is one cluster (all its CTAs co-scheduled by the
//              hardware): the cluster's barrier, passed by every thread,
//              stands for the grid barrier; there is no wait to bound.
// `part` holds 2 gridDim.x floats: the block partials.
// Loads a caller issues while its block waits at the grid barrier (none by
// default): anything that does not depend on the sum, so its latency hides
// behind the wait.
struct NoPrefetch {
    __device__ __forceinline__ void operator()() const {}
};

template <int N, class Pre = NoPrefetch>
__device__ bool grid_sum(float (&v)[N], float *part, unsigned *bar, unsigned nb,
                         unsigned *abort, unsigned cluster, const Pre &pre = Pre()) {
    __shared__ float s_w[N][kWarps];
    __shared__ float s_res[N];
    __shared__ int s_ok;
    const unsigned lane = threadIdx.x & 31u, w = threadIdx.x >> 5;
    for (int off = 16; off > 0; off >>= 1)
#pragma unroll
        for (int q = 0; q < N; ++q) v[q] += __shfl_down_sync(0xffffffffu, v[q], off);
    if (lane == 0)
#pragma unroll
        for (int q = 0; q < N; ++q) s_w[q][w] = v[q];
    __syncthreads();
    float x[N];
    if (w == 0) {
#pragma unroll
        for (int q = 0; q < N; ++q) x[q] = lane < (blockDim.x >> 5) ? s_w[q][lane] : 0.0f;
        for (int off = 16; off > 0; off >>= 1)
#pragma unroll
            for (int q = 0; q < N; ++q) x[q] += __shfl_down_sync(0xffffffffu, x[q], off);
        if (lane == 0)
#pragma unroll
            for (int q = 0; q < N; ++q) part[N * blockIdx.x + q] = x[q];
    }
    int ok = 1;
    if (cluster == 0) {
        unsigned g0 = 0;
        bool last = false;
        if (w == 0 && lane == 0) {
            g0 = ld_relaxed(bar + 1);
            last = atom_add_acq_rel(bar, 1u) == nb - 1;
            if (last) {
                st_relaxed(bar, 0u);
                red_add_release(bar + 1, 1u);
            }
        }
        pre();
        if (w == 0 && lane == 0) {
            if (!last) ok = grid_wait(bar + 1, g0, abort);
            if (ok && ld_relaxed(abort)) ok = 0;
        }
    } else {
        pre();
        cluster_barrier();
    }
    if (w == 0) {
        ok = __shfl_sync(0xffffffffu, ok, 0);
        if (ok) fold_partials<N>(part, nb, lane, x);
        if (lane == 0) {
#pragma unroll
            for (int q = 0; q < N; ++q) s_res[q] = x[q];
            s_ok = ok;
        }
    }
    __syncthreads();
#pragma unroll
    for (int q = 0; q < N; ++q) v[q] = s_res[q];
    return s_ok != 0;
}

template <class Pre = NoPrefetch>
__device__ bool grid_sum2(float &a, float &b, float *part, unsigned *bar, unsigned nb,
                          unsigned *abort, unsigned cluster, const Pre &pre = Pre()) {
    float v[2] = {a, b};
    const bool ok = grid_sum<2>(v, part, bar, nb, abort, cluster, pre);
    a = v[0];
    b = v[1];
    return ok;
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

// The {z, p} record of vertex j in one 256-bit load from L2.
__device__ __forceinline__ void ld_record(const float *R, unsigned j, Vec3 &z, Vec3 &p) {
    float r[8];
    asm volatile("ld.global.cg.v8.f32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
                 : "=f"(r[0]), "=f"(r[1]), "=f"(r[2]), "=f"(r[3]), "=f"(r[4]), "=f"(r[5]),
                   "=f"(r[6]), "=f"(r[7])
                 : "l"(R + 8 * (size_t)j));
    z = vec3(r[0], r[1], r[2]);
    p = vec3(r[3], r[4], r[5]);
}
__device__ __forceinline__ void st_record(float *R, unsigned i, const Vec3 &z, const Vec3 &p) {
    float4 *d = reinterpret_cast<float4 *>(R + 8 * (size_t)i);
    d[0] = make_float4(z[0], z[1], z[2], p[0]);
    d[1] = make_float4(p[1], p[2], 0.0f, 0.0f);
}

// Neighbour value of one slot: v(j) = z(j) + beta p(j) from the records, or
// x(j) from the AoS input of the initial product.
struct GatherCombined {
    const float *R;
    float beta;
    __device__ __forceinline__ Vec3 operator()(unsigned j) const {
        Vec3 z, p;
        ld_record(R, j, z, p);
        return z + beta * p;
    }
};
struct GatherPlain {
    const float *x;
    __device__ __forceinline__ Vec3 operator()(unsigned j) const { return ldcg3(x, j); }
};
struct GatherY {
    const float4 *Y;
    __device__ __forceinline__ Vec3 operator()(unsigned j) const { return ld4(Y, j); }
};

// A stored value: the operator's are fp32, a factor's bf16.
__device__ __forceinline__ float ld_val(const float *p) { return __ldg(p); }
__device__ __forceinline__ float ld_val(const bf16_t *p) {
    return __bfloat162float(__ushort_as_bfloat16(__ldg(reinterpret_cast<const unsigned short *>(p))));
}

// Which slots a product takes: all of them, only those below the diagonal
// of their row (column < row), or only those above it (column > row).
enum SlotMask : int { kAllSlots = 0, kBelow = 1, kAbove = 2 };

template <int MASK>
__device__ __forceinline__ bool takes(unsigned j, unsigned row) {
    if (MASK == kBelow) return j < row;
    if (MASK == kAbove) return j > row;
    return true;
}

// One slot's block times its neighbour value. `row` is the slot's row
// (0xffffffff for a lane without one, which a masked product then skips).
template <int MASK, class V, class G>
__device__ __forceinline__ void slot_term(const V *val, size_t s, unsigned lane, unsigned j,
                                          unsigned row, const G &gather, Vec3 &acc,
                                          Vec3 &abssum) {
    if (MASK != kAllSlots && (row == 0xFFFFFFFFu || !takes<MASK>(j, row))) return;
    const V *a = val + s * 9 * kSliceRows + lane;
    float m[9];
#pragma unroll
    for (int e = 0; e < 9; ++e) m[e] = ld_val(a + e * kSliceRows);
    const Vec3 v = gather(j);
    // column-major block: t_r = sum_c m[3 c + r] v_c
    Vec3 t;
    t[0] = m[0] * v[0] + m[3] * v[1] + m[6] * v[2];
    t[1] = m[1] * v[0] + m[4] * v[1] + m[7] * v[2];
    t[2] = m[2] * v[0] + m[5] * v[1] + m[8] * v[2];
    acc += t;
    abssum += t.cwise_abs();
}

// Part of row (32 slice + r) of A v over one SELL matrix: the slots of one
// parity (`par` 0: even, 1: odd). Two lanes share a row, so a warp holds 16
// rows and each lane walks half the row; a warp-wide load then touches two
// 64-byte runs, one per parity. abssum collects the component-wise |term| of
// every block product. Slots are taken four at a time (column indices first)
// so four gathers are in flight per lane.
template <int MASK, class V, class G>
__device__ __forceinline__ void sell_half_row(const SellMatrix &M, const V *val, unsigned slice,
                                              unsigned r,
                                              unsigned par, unsigned row, const G &gather,
                                              Vec3 &acc, Vec3 &abssum) {
    unsigned s0 = __ldg(M.slice_off + slice), s1 = __ldg(M.slice_off + slice + 1);
    if (MASK != kAllSlots && M.slice_mid) {
        const unsigned mid = __ldg(M.slice_mid + slice);
        if (MASK == kBelow) s1 = mid;
        else s0 = mid;
    }
    unsigned s = s0 + par;
    for (; s + 6 < s1; s += 8) {
        unsigned j[4];
#pragma unroll
        for (int q = 0; q < 4; ++q)
            j[q] = __ldg(M.col + (size_t)(s + 2 * q) * kSliceRows + r);
#pragma unroll
        for (int q = 0; q < 4; ++q)
            slot_term<MASK>(val, s + 2 * q, r, j[q], row, gather, acc, abssum);
    }
    for (; s < s1; s += 2) {
        const unsigned j = __ldg(M.col + (size_t)s * kSliceRows + r);
        slot_term<MASK>(val, s, r, j, row, gather, acc, abssum);
    }
}

// Row sum of both parities (the two lanes l and l ^ 16 end with the same
// bits: float addition commutes).
__device__ __forceinline__ void join_halves(Vec3 &acc, Vec3 &abssum) {
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        acc[k] += __shfl_xor_sync(0xffffffffu, acc[k], 16);
        abssum[k] += __shfl_xor_sync(0xffffffffu, abssum[k], 16);
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
    const unsigned *task_start; // grid + 1: each block's static range of product
                                // tasks; task_start[grid] starts the common pool
    unsigned *dyn_ctr;          // one zeroed counter per product phase
    unsigned n_ctr;
    float *x, *r;
    float *R;            // 8 floats per vertex: {z, p} records
    float4 *p, *Ap, *Ap_c, *Ap_ovf;
    float4 *Y;   // G r of the factored preconditioner
    float *part; // 2 buffers of 2 floats per block, then 1 float per block
    unsigned *bar;
    unsigned cluster; // the launch's cluster size (0: none; gridDim.x: one cluster)
    float tol;
    unsigned max_iter;
    PcgResult *res;
    const unsigned *run_if; // null, or the solve runs only when *run_if != 0
};

// Overflow row k of the contact part: the whole warp strides its entries and
// folds the partial products in a fixed shuffle order. Result on lane 0.
template <int MASK, class V, class G>
__device__ __forceinline__ void overflow_row(const OverflowRows &O, const V *vals,
                                             unsigned k, unsigned lane, const G &gather,
                                             Vec3 &acc, Vec3 &abssum) {
    const uint2 rg = __ldg(O.range + k);
    const unsigned row = MASK == kAllSlots ? 0u : __ldg(O.row + k);
    for (unsigned e = rg.x + lane; e < rg.x + rg.y; e += 32u) {
        const unsigned j = __ldg(O.col + e);
        if (!takes<MASK>(j, row)) continue;
        const V *a = vals + 9 * (size_t)e;
        float m[9];
#pragma unroll
        for (int q = 0; q < 9; ++q) m[q] = ld_val(a + q);
        const Vec3 v = gather(j);
        Vec3 t;
        t[0] = m[0] * v[0] + m[3] * v[1] + m[6] * v[2];
        t[1] = m[1] * v[0] + m[4] * v[1] + m[7] * v[2];
        t[2] = m[2] * v[0] + m[5] * v[1] + m[8] * v[2];
        acc += t;
        abssum += t.cwise_abs();
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1)
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            acc[c] += __shfl_down_sync(0xffffffffu, acc[c], off);
            abssum[c] += __shfl_down_sync(0xffffffffu, abssum[c], off);
        }
}

constexpr unsigned kNoTask = 0xFFFFFFFFu;
// Share of the product work (in sixteenths of its cost) split statically
// among the blocks; the rest, the last tasks in order (fixed half slices,
// short and even), goes to whichever warps finish first.
constexpr unsigned kStaticSixteenths = 12; // the default (PcgWorkspace::static_sixteenths)

// The product tasks of one phase: first the block's static range, handed to
// its warps one at a time through a shared counter, then tasks of the common
// pool [dyn0, total) through the phase's global counter. Each product phase
// of a solve has its own counter (zeroed before the launch).
struct BlockTasks {
    unsigned *next;       // shared: [0] the static range's next task, [1] set
                          // once the common pool ran dry for this block
    unsigned begin, end;  // this block's static range
    unsigned dyn0, total; // the common pool
    unsigned *ctrs;       // one per phase
    unsigned n_ctrs;
    unsigned phase = 0;
    unsigned *ctr = nullptr;
    // Starts a product phase (every thread of the block calls it).
    __device__ __forceinline__ void start() {
        ctr = phase < n_ctrs ? ctrs + phase : nullptr;
        ++phase;
        if (threadIdx.x == 0) {
            next[0] = begin;
            next[1] = 0u;
        }
        __syncthreads();
    }
    // The block's warps stop asking the pool's global counter once one of
    // them found it empty, so an empty pool costs about one atomic per block
    // rather than one per warp.
    __device__ __forceinline__ unsigned take(unsigned lane) const {
        unsigned t = 0;
        if (lane == 0u) {
            t = atomicAdd(next, 1u);
            if (t >= end) {
                t = kNoTask;
                volatile unsigned *drained = next + 1;
                if (ctr && !*drained) {
                    const unsigned d = atomicAdd(ctr, 1u);
                    if (d < total - dyn0) t = dyn0 + d;
                    else *drained = 1u;
                }
            }
        }
        return __shfl_sync(0xffffffffu, t, 0);
    }
};

constexpr unsigned kNoIndex = 0xFFFFFFFEu; // row_product: look the contact row up

// (A v)(i): the row's fixed part, plus its contact and overflow parts, if any.
// `c` is the row's contact position when the caller already loaded it.
__device__ __forceinline__ Vec3 row_product(const PcgArgs &g, unsigned i,
                                            unsigned c = kNoIndex) {
    Vec3 ap = ld4(g.Ap, i);
    if (c == kNoIndex) c = __ldg(g.A.contact.index + i);
    if (c != 0xFFFFFFFFu) {
        ap += ld4(g.Ap_c, c);
        const unsigned k = __ldg(g.A.ovf.index + i);
        if (k != 0xFFFFFFFFu) ap += ld4(g.Ap_ovf, k);
    }
    return ap;
}

// The product task list of one solve: overflow rows [0, t1), contact half
// slices [t1, t2), fixed half slices [t2, total). The contact row and
// overflow row counts are read from the device when the layout carries
// them, so a solve launched before they are known (a captured iteration)
// partitions the same list.
struct TaskSpace {
    unsigned t1, t2, total, c_rows;
    __device__ __forceinline__ explicit TaskSpace(const PcgOperator &A) {
        unsigned rows = A.contact.rows, n_ovf = A.ovf.count;
        if (A.contact.sizes) {
            rows = __ldg(A.contact.sizes);
            n_ovf = __ldg(A.contact.sizes + 1);
        }
        c_rows = rows;
        t1 = n_ovf;
        t2 = t1 + 2 * ((rows + kSliceRows - 1) / kSliceRows);
        total = t2 + 2 * A.fixed.n_slices;
    }
};

// One product task of warp `lane`s: the fixed part of a half slice, the
// contact part of a half slice of sorted contact rows, or an overflow row.
// The epilogue gets (row, A-part, |terms|) on the lanes that own a result.
// `vals` are the value arrays the slots are read from: the operator's own
// (fixed, contact, overflow) or a factor's parallel ones.
template <int MASK, class V, class G, class E>
__device__ __forceinline__ void product_task(const PcgArgs &g, const TaskSpace &ts,
                                             const V *const vals[3], unsigned task,
                                             unsigned lane, const G &gather, E &&epilogue) {
    const PcgOperator &A = g.A;
    // task order: overflow rows, contact half slices, fixed half slices (the
    // long and uneven items first, so the common pool at the end of the
    // order holds short, even ones)
    const unsigned t1 = ts.t1, t2 = ts.t2;
    const unsigned par = lane >> 4;
    Vec3 acc = Vec3::zero(), ab = Vec3::zero();
    if (task >= t1) {
        const bool fixed = task >= t2;
        const unsigned u = fixed ? task - t2 : task - t1;
        const unsigned sl = u >> 1, r = (u & 1u) * 16u + (lane & 15u);
        const unsigned q = sl * kSliceRows + r;
        const SellMatrix &M = fixed ? A.fixed : A.contact.sell;
        const V *val = vals[fixed ? 0 : 1];
        unsigned row = 0xFFFFFFFFu;
        if (MASK != kAllSlots) {
            if (fixed) row = q < A.n ? q : 0xFFFFFFFFu;
            else row = q < ts.c_rows ? __ldg(A.contact.perm + q) : 0xFFFFFFFFu;
        }
        sell_half_row<MASK>(M, val, sl, r, par, row, gather, acc, ab);
        join_halves(acc, ab);
        if (par == 0u) {
            if (fixed) {
                if (q < A.n) epilogue(q, 0u, q, acc, ab);
            } else if (q < ts.c_rows) {
                epilogue(__ldg(A.contact.perm + q), 1u, q, acc, ab);
            }
        }
    } else {
        const unsigned k = task;
        overflow_row<MASK>(A.ovf, vals[2], k, lane, gather, acc, ab);
        if (lane == 0u) epilogue(__ldg(A.ovf.row + k), 2u, k, acc, ab);
    }
}

__global__ void __launch_bounds__(kThreads, 1) k_pcg(PcgArgs g) {
    // a conditional solve that is not needed leaves everything as it is
    if (g.run_if && *g.run_if == 0u) return;
    const PcgOperator &A = g.A;
    const unsigned nb = gridDim.x;
    const unsigned lane = threadIdx.x & 31u;
    const unsigned warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const unsigned nwarps = (gridDim.x * blockDim.x) >> 5;
    const unsigned n_slices = A.fixed.n_slices;
    unsigned *abort = g.bar + 2;
    float *part0 = g.part, *part1 = g.part + 2 * nb;
    float a, b;

    // work items of the products: half slices (16 rows, two lanes per row),
    // then one warp per overflow row of the contact part

    __shared__ unsigned s_next[2];
    const TaskSpace ts(A);
    BlockTasks bt{s_next, g.task_start[blockIdx.x], g.task_start[blockIdx.x + 1],
                  g.task_start[gridDim.x], ts.total, g.dyn_ctr, g.n_ctr};
    // A x0 (slice part to Ap, overflow part to Ap_ovf) ...
    bt.start();
    {
        const GatherPlain gx{g.x};
        float4 *dst[3] = {g.Ap, g.Ap_c, g.Ap_ovf};
        const float *const vals[3] = {A.fixed.val, A.contact.sell.val, A.ovf.val};
        for (unsigned task = bt.take(lane); task != kNoTask; task = bt.take(lane))
            product_task<kAllSlots>(g, ts, vals, task, lane, gx,
                         [&](unsigned, unsigned part, unsigned slot, const Vec3 &acc, const Vec3 &) {
                             st4(dst[part], slot, acc);
                         });
    }
    a = b = 0.0f;
    if (!grid_sum2(a, b, part1, g.bar, nb, abort, g.cluster)) goto aborted;
    // ... then r = b - A x0, z = P r, p_0 = 0; err0 = |r|_1, rz0 = r^T z
    a = b = 0.0f;
    for (unsigned sl = warp; sl < n_slices; sl += nwarps) {
        const unsigned i = sl * kSliceRows + lane;
        if (i >= A.n) continue;
        Vec3 ri = ldcg3(g.r, i) - row_product(g, i);
        Vec3 zi = load_inv(A.inv_diag, sl, lane) * ri;
        st3(g.r, i, ri);
        st_record(g.R, i, zi, Vec3::zero());
        a += fabsf(ri[0]) + fabsf(ri[1]) + fabsf(ri[2]);
        b += ri.dot(zi);
    }
    if (!grid_sum2(a, b, part0, g.bar, nb, abort, g.cluster)) goto aborted;
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
            // S: A p_k with p_k = z + beta p_{k-1}
            a = b = 0.0f; // p^T A p, sum |p_i| |terms|
            const GatherCombined gp{g.R, beta};
            bt.start();
            float4 *dst[3] = {g.Ap, g.Ap_c, g.Ap_ovf};
            const float *const vals[3] = {A.fixed.val, A.contact.sell.val, A.ovf.val};
            for (unsigned task = bt.take(lane); task != kNoTask; task = bt.take(lane))
                product_task<kAllSlots>(g, ts, vals, task, lane, gp,
                             [&](unsigned row, unsigned part, unsigned slot, const Vec3 &acc,
                                 const Vec3 &ab) {
                                 const Vec3 pi = gp(row);
                                 if (part == 0u) st4(g.p, row, pi);
                                 st4(dst[part], slot, acc);
                                 a += pi.dot(acc);
                                 b += fabsf(pi[0]) * ab[0] + fabsf(pi[1]) * ab[1] +
                                      fabsf(pi[2]) * ab[2];
                             });
            // the update phase's first slice: what it reads that no other
            // warp writes in this phase, loaded while the block waits
            const unsigned i0 = warp * kSliceRows + lane;
            const bool has0 = warp < n_slices && i0 < A.n;
            Vec3 x0v = Vec3::zero(), r0v = Vec3::zero();
            unsigned c0 = 0xFFFFFFFFu;
            const auto pre = [&]() {
                if (has0) {
                    x0v = ldcg3(g.x, i0);
                    r0v = ldcg3(g.r, i0);
                    c0 = __ldg(A.contact.index + i0);
                }
            };
            if (!grid_sum2(a, b, part1, g.bar, nb, abort, g.cluster, pre)) goto aborted;
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
                const bool first = sl == warp;
                Vec3 pi = ld4(g.p, i), api = row_product(g, i, first ? c0 : kNoIndex);
                Vec3 xi = first ? x0v : ldcg3(g.x, i), ri = first ? r0v : ldcg3(g.r, i);
                for (int k = 0; k < 3; ++k) {
                    xi[k] += alpha * pi[k];
                    ri[k] = ri[k] - alpha * api[k];
                }
                Vec3 zi = load_inv(A.inv_diag, sl, lane) * ri;
                st3(g.x, i, xi);
                st3(g.r, i, ri);
                st_record(g.R, i, zi, pi);
                a += ri.dot(zi);
                b += fabsf(ri[0]) + fabsf(ri[1]) + fabsf(ri[2]);
            }
            if (!grid_sum2(a, b, part0, g.bar, nb, abort, g.cluster)) goto aborted;
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

// The factored preconditioner's two products (P = G^T G + eps D^{-1}):
//   factor_y: y = G r (slots below the diagonal plus the diagonal blocks) into
//             Y, which the caller zeroed; then a grid barrier
//   factor_z: z = G^T y + eps D^{-1} r (slots above the diagonal plus the
//             transposed diagonal blocks), added into the records' z, which
//             the caller zeroed; then the grid-wide r^T z
// Each row's parts (fixed, contact, overflow) are added with atomics; r^T z
// is linear in them, so its partial sums need no complete z. Both return
// false when the grid barrier aborted.
__device__ bool factor_y(const PcgArgs &g, BlockTasks &bt, unsigned lane, float *part,
                         unsigned *abort) {
    const PcgOperator &A = g.A;
    const TaskSpace ts(A);
    const bf16_t *const vals[3] = {A.factor.fixed, A.factor.contact, A.factor.ovf};
    bt.start();
    {
        const GatherPlain gr{g.r};
        for (unsigned task = bt.take(lane); task != kNoTask; task = bt.take(lane))
            product_task<kBelow>(g, ts, vals, task, lane, gr,
                                 [&](unsigned row, unsigned part, unsigned, Vec3 acc, const Vec3 &) {
                                     if (part == 0u)
                                         acc += load_mat3(A.factor.diag + 9 * (size_t)row) *
                                                ldcg3(g.r, row);
                                     float *y = reinterpret_cast<float *>(g.Y + row);
                                     atomicAdd(y, acc[0]);
                                     atomicAdd(y + 1, acc[1]);
                                     atomicAdd(y + 2, acc[2]);
                                 });
    }
    float a = 0.0f, b = 0.0f;
    return grid_sum2(a, b, part, g.bar, gridDim.x, abort, g.cluster);
}

__device__ bool factor_z(const PcgArgs &g, BlockTasks &bt, unsigned lane, float *part,
                         unsigned *abort, float &rz) {
    const PcgOperator &A = g.A;
    const TaskSpace ts(A);
    const bf16_t *const vals[3] = {A.factor.fixed, A.factor.contact, A.factor.ovf};
    bt.start();
    float a = 0.0f;
    {
        const GatherY gy{g.Y};
        for (unsigned task = bt.take(lane); task != kNoTask; task = bt.take(lane))
            product_task<kAbove>(g, ts, vals, task, lane, gy,
                                 [&](unsigned row, unsigned part, unsigned, Vec3 acc, const Vec3 &) {
                                     const Vec3 ri = ldcg3(g.r, row);
                                     if (part == 0u) {
                                         acc += load_mat3(A.factor.diag + 9 * (size_t)row)
                                                    .transpose() *
                                                gy(row);
                                         acc += A.factor.eps *
                                                (load_inv(A.inv_diag, row / kSliceRows,
                                                          row % kSliceRows) *
                                                 ri);
                                     }
                                     float *z = g.R + 8 * (size_t)row;
                                     atomicAdd(z, acc[0]);
                                     atomicAdd(z + 1, acc[1]);
                                     atomicAdd(z + 2, acc[2]);
                                     a += ri.dot(acc);
                                 });
    }
    float b = 0.0f;
    if (!grid_sum2(a, b, part, g.bar, gridDim.x, abort, g.cluster)) return false;
    rz = a;
    return true;
}

// (A v)(j) of every column a product gathers: the sum of the row's parts
// that the product phase stored (complete after its grid barrier).
struct GatherAp {
    const PcgArgs *g;
    __device__ __forceinline__ Vec3 operator()(unsigned j) const { return row_product(*g, j); }
};

// Y -= alpha G (A p): the update of y = G r that follows r -= alpha A p, run
// inside the update phase (A p is complete after the product phase's
// barrier), so y needs no barrier of its own. No barrier here.
__device__ void factor_y_update(const PcgArgs &g, BlockTasks &bt, unsigned lane, float alpha) {
    const PcgOperator &A = g.A;
    const TaskSpace ts(A);
    const bf16_t *const vals[3] = {A.factor.fixed, A.factor.contact, A.factor.ovf};
    bt.start();
    const GatherAp gap{&g};
    for (unsigned task = bt.take(lane); task != kNoTask; task = bt.take(lane))
        product_task<kBelow>(g, ts, vals, task, lane, gap,
                             [&](unsigned row, unsigned part, unsigned, Vec3 acc, const Vec3 &) {
                                 if (part == 0u)
                                     acc += load_mat3(A.factor.diag + 9 * (size_t)row) *
                                            row_product(g, row);
                                 float *y = reinterpret_cast<float *>(g.Y + row);
                                 atomicAdd(y, -alpha * acc[0]);
                                 atomicAdd(y + 1, -alpha * acc[1]);
                                 atomicAdd(y + 2, -alpha * acc[2]);
                             });
}

// y = G r is recomputed from r every this many iterations (otherwise it
// follows r's recurrence), which bounds the rounding the recurrence gathers.
constexpr unsigned kYRefresh = 16;

// PCG with the factored preconditioner: the recurrence, verdicts and checks
// of k_pcg, with z = P r after each update: y = G r follows r's recurrence
// inside the update phase (recomputed from r every kYRefresh iterations),
// then z = G^T y + eps D^{-1} r, so an iteration takes three grid barriers
// (four on a refresh).
__global__ void __launch_bounds__(kThreads, 1) k_pcg_factor(PcgArgs g) {
    const PcgOperator &A = g.A;
    const unsigned nb = gridDim.x;
    const unsigned lane = threadIdx.x & 31u;
    const unsigned warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const unsigned nwarps = (gridDim.x * blockDim.x) >> 5;
    const unsigned n_slices = A.fixed.n_slices;
    unsigned *abort = g.bar + 2;
    float *part0 = g.part, *part1 = g.part + 2 * nb;
    float a, b;

    __shared__ unsigned s_next[2];
    const TaskSpace ts(A);
    BlockTasks bt{s_next, g.task_start[blockIdx.x], g.task_start[blockIdx.x + 1],
                  g.task_start[gridDim.x], ts.total, g.dyn_ctr, g.n_ctr};
    const float *const avals[3] = {A.fixed.val, A.contact.sell.val, A.ovf.val};
    // A x0
    bt.start();
    {
        const GatherPlain gx{g.x};
        float4 *dst[3] = {g.Ap, g.Ap_c, g.Ap_ovf};
        for (unsigned task = bt.take(lane); task != kNoTask; task = bt.take(lane))
            product_task<kAllSlots>(g, ts, avals, task, lane, gx,
                                    [&](unsigned, unsigned part, unsigned slot, const Vec3 &acc,
                                        const Vec3 &) { st4(dst[part], slot, acc); });
    }
    a = b = 0.0f;
    if (!grid_sum2(a, b, part1, g.bar, nb, abort, g.cluster)) goto aborted;
    // r = b - A x0, err0 = |r|_1; records {0, 0}, Y = 0
    a = b = 0.0f;
    for (unsigned sl = warp; sl < n_slices; sl += nwarps) {
        const unsigned i = sl * kSliceRows + lane;
        if (i >= A.n) continue;
        Vec3 ri = ldcg3(g.r, i) - row_product(g, i);
        st3(g.r, i, ri);
        st_record(g.R, i, Vec3::zero(), Vec3::zero());
        st4(g.Y, i, Vec3::zero());
        a += fabsf(ri[0]) + fabsf(ri[1]) + fabsf(ri[2]);
    }
    if (!grid_sum2(a, b, part0, g.bar, nb, abort, g.cluster)) goto aborted;
    {
        const float err0 = a;
        if (err0 == 0.0f) {
            if (blockIdx.x == 0 && threadIdx.x == 0)
                *g.res = PcgResult{1u, 0.0f, 0, 0, 0.0f, 0.0f, 0u};
            return;
        }
        float rz0;
        if (!factor_y(g, bt, lane, part1, abort)) goto aborted;
        if (!factor_z(g, bt, lane, part0, abort, rz0)) goto aborted;
        float beta = 0.0f;
        unsigned stride = 4, next_check = 1;
        int broke = 0;
        float break_val = 0.0f;
        for (unsigned iter = 1;; ++iter) {
            // S: A p_k with p_k = z + beta p_{k-1}
            a = b = 0.0f;
            const GatherCombined gp{g.R, beta};
            bt.start();
            float4 *dst[3] = {g.Ap, g.Ap_c, g.Ap_ovf};
            for (unsigned task = bt.take(lane); task != kNoTask; task = bt.take(lane))
                product_task<kAllSlots>(g, ts, avals, task, lane, gp,
                                        [&](unsigned row, unsigned part, unsigned slot,
                                            const Vec3 &acc, const Vec3 &ab) {
                                            const Vec3 pi = gp(row);
                                            if (part == 0u) st4(g.p, row, pi);
                                            st4(dst[part], slot, acc);
                                            a += pi.dot(acc);
                                            b += fabsf(pi[0]) * ab[0] + fabsf(pi[1]) * ab[1] +
                                                 fabsf(pi[2]) * ab[2];
                                        });
            // the update phase's first slice: x, r and the contact position,
            // which no other warp writes, loaded while the block waits
            const unsigned i0 = warp * kSliceRows + lane;
            const bool has0 = warp < n_slices && i0 < A.n;
            Vec3 x0v = Vec3::zero(), r0v = Vec3::zero();
            unsigned c0 = 0xFFFFFFFFu;
            const auto pre = [&]() {
                if (has0) {
                    x0v = ldcg3(g.x, i0);
                    r0v = ldcg3(g.r, i0);
                    c0 = __ldg(A.contact.index + i0);
                }
            };
            if (!grid_sum2(a, b, part1, g.bar, nb, abort, g.cluster, pre)) goto aborted;
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
            // U: x += alpha p, r -= alpha A p; records {0, p}; |r|_1; and
            // y -= alpha G A p, or, every kYRefresh iterations, Y = 0 for
            // y = G r from scratch after the barrier
            const bool refresh = iter % kYRefresh == 0;
            a = b = 0.0f;
            for (unsigned sl = warp; sl < n_slices; sl += nwarps) {
                const unsigned i = sl * kSliceRows + lane;
                if (i >= A.n) continue;
                const bool first = sl == warp;
                Vec3 pi = ld4(g.p, i), api = row_product(g, i, first ? c0 : kNoIndex);
                Vec3 xi = first ? x0v : ldcg3(g.x, i), ri = first ? r0v : ldcg3(g.r, i);
                for (int k = 0; k < 3; ++k) {
                    xi[k] += alpha * pi[k];
                    ri[k] = ri[k] - alpha * api[k];
                }
                st3(g.x, i, xi);
                st3(g.r, i, ri);
                st_record(g.R, i, Vec3::zero(), pi);
                if (refresh) st4(g.Y, i, Vec3::zero());
                b += fabsf(ri[0]) + fabsf(ri[1]) + fabsf(ri[2]);
            }
            if (!refresh) factor_y_update(g, bt, lane, alpha);
            if (!grid_sum2(a, b, part0, g.bar, nb, abort, g.cluster)) goto aborted;
            const float err_now = b;
            float rz_new;
            if (refresh && !factor_y(g, bt, lane, part1, abort)) goto aborted;
            if (!factor_z(g, bt, lane, part0, abort, rz_new)) goto aborted;
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

constexpr unsigned kSchwarzDim = 3 * kSchwarzMaxMembers;
// floats of a warp's shared region: r, y, z, p of the aggregate and its
// staged packed factor (rounded up to 16 bytes)
constexpr unsigned kSchwarzTri = (kSchwarzDim * (kSchwarzDim + 1) / 2 + 3) & ~3u;
constexpr unsigned kSchwarzWarpFloats = 4 * kSchwarzDim + kSchwarzTri;

// One Schwarz aggregate, by one warp: the update of its member rows
// (`init`: r = r - A x0 and p = 0; otherwise x += alpha p, r -= alpha A p),
// with the coarse level the aggregate's residual sum rc, then
// z = G^T (G r) on the aggregate, and the members' {z, p} records.
// Adds r^T z to `a` and |r|_1 to `b`. `seg` is the warp's shared region
// (kSchwarzWarpFloats, 16-byte aligned); the packed factor is staged there
// with 16-byte loads and both triangular products read it from there.
// Copies aggregate ag's packed factor into the warp's shared segment.
__device__ __forceinline__ void schwarz_stage(const PcgArgs &g, unsigned ag, unsigned lane,
                                              float *seg) {
    const SchwarzView &S = g.A.schwarz;
    const unsigned m = __ldg(S.agg_off + ag + 1) - __ldg(S.agg_off + ag), d = 3u * m;
    const float4 *G4 = reinterpret_cast<const float4 *>(S.ainv + __ldg(S.ainv_off + ag));
    float4 *s4 = reinterpret_cast<float4 *>(seg + 4 * kSchwarzDim);
    const unsigned n4 = (d * (d + 1u) / 2u + 3u) / 4u;
    for (unsigned e = lane; e < n4; e += 32u) s4[e] = __ldg(G4 + e);
}

// `staged`: the aggregate's factor is already in the segment (the caller
// staged it while its block waited at the grid barrier).
__device__ __forceinline__ void schwarz_segment(const PcgArgs &g, unsigned ag, unsigned lane,
                                                bool init, float alpha, float *seg, float &a,
                                                float &b, bool staged = false) {
    const SchwarzView &S = g.A.schwarz;
    constexpr unsigned D = kSchwarzDim;
    float *sr = seg, *sy = seg + D, *sz = seg + 2 * D, *sp = seg + 3 * D;
    float *sG = seg + 4 * D;
    const unsigned base = __ldg(S.agg_off + ag), m = __ldg(S.agg_off + ag + 1) - base;
    const unsigned d = 3u * m;
    for (unsigned k = lane; k < m; k += 32u) {
        const unsigned i = __ldg(S.members + base + k);
        Vec3 ri = ldcg3(g.r, i), pi = Vec3::zero();
        const Vec3 api = row_product(g, i);
        if (init) {
            ri = ri - api;
        } else {
            pi = ld4(g.p, i);
            Vec3 xi = ldcg3(g.x, i);
            for (int c = 0; c < 3; ++c) {
                xi[c] += alpha * pi[c];
                ri[c] = ri[c] - alpha * api[c];
            }
            st3(g.x, i, xi);
        }
        st3(g.r, i, ri);
        for (int c = 0; c < 3; ++c) {
            sr[3 * k + c] = ri[c];
            sp[3 * k + c] = pi[c];
        }
        b += fabsf(ri[0]) + fabsf(ri[1]) + fabsf(ri[2]);
    }
    __syncwarp();
    if (S.n_dom && lane < 3u) { // C r: the aggregate's residual sum, members in order
        float sum = 0.0f;
        for (unsigned k = 0; k < m; ++k) sum += sr[3 * k + lane];
        sy[lane] = sum;
    }
    __syncwarp();
    if (S.n_dom && lane == 0) S.rc[ag] = make_float4(sy[0], sy[1], sy[2], 0.0f);
    __syncwarp();
    if (!staged) schwarz_stage(g, ag, lane, seg);
    __syncwarp();
    for (unsigned p = lane; p < d; p += 32u) { // y = G r
        const float *row = sG + p * (p + 1u) / 2u;
        float acc = 0.0f;
        for (unsigned q = 0; q <= p; ++q) acc += row[q] * sr[q];
        sy[p] = acc;
    }
    __syncwarp();
    for (unsigned p = lane; p < d; p += 32u) { // z = G^T y
        float acc = 0.0f;
        for (unsigned q = p; q < d; ++q) acc += sG[q * (q + 1u) / 2u + p] * sy[q];
        sz[p] = acc;
    }
    __syncwarp();
    for (unsigned k = lane; k < m; k += 32u) {
        const unsigned i = __ldg(S.members + base + k);
        const Vec3 zi = vec3(sz[3 * k], sz[3 * k + 1], sz[3 * k + 2]);
        const Vec3 ri = vec3(sr[3 * k], sr[3 * k + 1], sr[3 * k + 2]);
        st_record(g.R, i, zi, vec3(sp[3 * k], sp[3 * k + 1], sp[3 * k + 2]));
        a += ri.dot(zi);
    }
    __syncwarp();
}

// One coarse domain, by one warp: rc of its nodes (written by the fine
// phase), e = G1^T (G1 rc) with the domain's staged packed factor, then
// z_i += w e(node of i) in the records of every member vertex of every node
// (each vertex is reached by exactly one warp). Adds w rc . e, the coarse
// part of r^T z, to `a`.
__device__ __forceinline__ void schwarz_coarse(const PcgArgs &g, unsigned dm, unsigned lane,
                                               float *seg, float &a) {
    const SchwarzView &S = g.A.schwarz;
    constexpr unsigned D = kSchwarzDim;
    float *sr = seg, *sy = seg + D, *sz = seg + 2 * D;
    float *sG = seg + 4 * D;
    const unsigned base = __ldg(S.dom_off + dm), m = __ldg(S.dom_off + dm + 1) - base;
    const unsigned d = 3u * m;
    for (unsigned k = lane; k < m; k += 32u) {
        const float4 v = __ldcg(S.rc + __ldg(S.dom_members + base + k));
        sr[3 * k] = v.x;
        sr[3 * k + 1] = v.y;
        sr[3 * k + 2] = v.z;
    }
    {
        const float4 *G4 = reinterpret_cast<const float4 *>(S.ainv1 + __ldg(S.ainv1_off + dm));
        float4 *s4 = reinterpret_cast<float4 *>(sG);
        const unsigned n4 = (d * (d + 1u) / 2u + 3u) / 4u;
        for (unsigned e = lane; e < n4; e += 32u) s4[e] = __ldg(G4 + e);
    }
    __syncwarp();
    for (unsigned p = lane; p < d; p += 32u) { // y = G1 rc
        const float *row = sG + p * (p + 1u) / 2u;
        float acc = 0.0f;
        for (unsigned q = 0; q <= p; ++q) acc += row[q] * sr[q];
        sy[p] = acc;
    }
    __syncwarp();
    for (unsigned p = lane; p < d; p += 32u) { // e = G1^T y, weighted
        float acc = 0.0f;
        for (unsigned q = p; q < d; ++q) acc += sG[q * (q + 1u) / 2u + p] * sy[q];
        sz[p] = S.weight * acc;
        a += sr[p] * sz[p];
    }
    __syncwarp();
    // prolongation: two nodes per pass, 16 lanes over each node's members
    const unsigned half = lane >> 4, t = lane & 15u;
    for (unsigned k0 = 0; k0 < m; k0 += 2u) {
        const unsigned k = k0 + half;
        if (k < m) {
            const unsigned node = __ldg(S.dom_members + base + k);
            const unsigned mb = __ldg(S.agg_off + node), mm = __ldg(S.agg_off + node + 1) - mb;
            for (unsigned u = t; u < mm; u += 16u) {
                float4 *rec = reinterpret_cast<float4 *>(g.R + 8 * (size_t)__ldg(S.members + mb + u));
                float4 v = __ldcg(rec);
                v.x += sz[3 * k];
                v.y += sz[3 * k + 1];
                v.z += sz[3 * k + 2];
                *rec = v;
            }
        }
    }
    __syncwarp();
}

// PCG with the aggregate-Schwarz preconditioner: the recurrence, verdicts and
// checks of k_pcg, with the update phase walking aggregates instead of
// slices. With the coarse level, the update phase also restricts r into rc,
// and after its reduction a coarse phase (one warp per domain) adds the
// coarse correction to z and its part of r^T z, reduced by a third grid
// barrier. A non-positive (or non-finite) r^T z ends the solve as failed with
// break cause 2, the reference's cue to solve again with block-Jacobi
// (solver/solver.cu:1627-1676).
__global__ void __launch_bounds__(kThreads, 1) k_pcg_schwarz(PcgArgs g) {
    const PcgOperator &A = g.A;
    const unsigned nb = gridDim.x;
    const unsigned lane = threadIdx.x & 31u, wib = threadIdx.x >> 5;
    const unsigned warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const unsigned nwarps = (gridDim.x * blockDim.x) >> 5;
    const unsigned n_agg = A.schwarz.n_agg, n_dom = A.schwarz.n_dom;
    unsigned *abort = g.bar + 2;
    float *part0 = g.part, *part1 = g.part + 2 * nb, *part2 = g.part + 4 * nb;
    float a, b;
    extern __shared__ float4 s_dyn4[];
    float *seg = reinterpret_cast<float *>(s_dyn4) + (size_t)wib * kSchwarzWarpFloats;

    __shared__ unsigned s_next[2];
    const TaskSpace ts(A);
    BlockTasks bt{s_next, g.task_start[blockIdx.x], g.task_start[blockIdx.x + 1],
                  g.task_start[gridDim.x], ts.total, g.dyn_ctr, g.n_ctr};
    const float *const avals[3] = {A.fixed.val, A.contact.sell.val, A.ovf.val};
    bt.start();
    {
        const GatherPlain gx{g.x};
        float4 *dst[3] = {g.Ap, g.Ap_c, g.Ap_ovf};
        for (unsigned task = bt.take(lane); task != kNoTask; task = bt.take(lane))
            product_task<kAllSlots>(g, ts, avals, task, lane, gx,
                                    [&](unsigned, unsigned part, unsigned slot, const Vec3 &acc,
                                        const Vec3 &) { st4(dst[part], slot, acc); });
    }
    a = b = 0.0f;
    if (!grid_sum2(a, b, part1, g.bar, nb, abort, g.cluster)) goto aborted;
    // r = b - A x0, z = P r, p_0 = 0; rz0, err0
    a = b = 0.0f;
    for (unsigned ag = warp; ag < n_agg; ag += nwarps)
        schwarz_segment(g, ag, lane, true, 0.0f, seg, a, b);
    if (!grid_sum2(a, b, part0, g.bar, nb, abort, g.cluster)) goto aborted;
    if (n_dom) { // coarse correction, then its part of r^T z
        float c[1] = {0.0f};
        for (unsigned dm = warp; dm < n_dom; dm += nwarps) schwarz_coarse(g, dm, lane, seg, c[0]);
        if (!grid_sum<1>(c, part2, g.bar, nb, abort, g.cluster)) goto aborted;
        a += c[0];
    }
    {
        const float err0 = b;
        float rz0 = a;
        if (err0 == 0.0f) {
            if (blockIdx.x == 0 && threadIdx.x == 0)
                *g.res = PcgResult{1u, 0.0f, 0, 0, 0.0f, 0.0f, 0u};
            return;
        }
        if (!(rz0 > 0.0f)) {
            if (blockIdx.x == 0 && threadIdx.x == 0)
                *g.res = PcgResult{1u, 1.0f, 2, 2, err0, rz0, 0u};
            return;
        }
        float beta = 0.0f;
        unsigned stride = 4, next_check = 1;
        int broke = 0;
        float break_val = 0.0f;
        for (unsigned iter = 1;; ++iter) {
            // S: A p_k with p_k = z + beta p_{k-1}
            a = b = 0.0f;
            const GatherCombined gp{g.R, beta};
            bt.start();
            float4 *dst[3] = {g.Ap, g.Ap_c, g.Ap_ovf};
            for (unsigned task = bt.take(lane); task != kNoTask; task = bt.take(lane))
                product_task<kAllSlots>(g, ts, avals, task, lane, gp,
                                        [&](unsigned row, unsigned part, unsigned slot,
                                            const Vec3 &acc, const Vec3 &ab) {
                                            const Vec3 pi = gp(row);
                                            if (part == 0u) st4(g.p, row, pi);
                                            st4(dst[part], slot, acc);
                                            a += pi.dot(acc);
                                            b += fabsf(pi[0]) * ab[0] + fabsf(pi[1]) * ab[1] +
                                                 fabsf(pi[2]) * ab[2];
                                        });
            // the warp's first aggregate's factor staged while the block
            // waits (warp 0 of each block, which waits for it, excepted)
            const bool staged0 = wib != 0u && warp < n_agg;
            const auto pre = [&]() {
                if (staged0) schwarz_stage(g, warp, lane, seg);
            };
            if (!grid_sum2(a, b, part1, g.bar, nb, abort, g.cluster, pre)) goto aborted;
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
            // U: per aggregate, x += alpha p, r -= alpha A p, z = P r
            a = b = 0.0f;
            for (unsigned ag = warp; ag < n_agg; ag += nwarps)
                schwarz_segment(g, ag, lane, false, alpha, seg, a, b, staged0 && ag == warp);
            if (!grid_sum2(a, b, part0, g.bar, nb, abort, g.cluster)) goto aborted;
            if (n_dom) {
                float c[1] = {0.0f};
                for (unsigned dm = warp; dm < n_dom; dm += nwarps)
                    schwarz_coarse(g, dm, lane, seg, c[0]);
                if (!grid_sum<1>(c, part2, g.bar, nb, abort, g.cluster)) goto aborted;
                a += c[0];
            }
            const float rz_new = a, err_now = b;
            const bool rz_bad = !(rz_new > 0.0f);
            beta = rz_new / rz0;
            rz0 = rz_new;
            const bool at_cap = iter >= g.max_iter;
            if (iter == next_check || at_cap || rz_bad) {
                const float reresid = err_now / err0;
                PcgResult out{iter, reresid, -1, broke, err0, break_val, 0u};
                if (reresid < g.tol) out.state = 0;
                else if (rz_bad) {
                    out.state = 2;
                    out.break_cause = 2;
                    out.break_val = rz_new;
                } else if (broke == 3) out.state = 1;
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

// Per-row contact block count: the sort key (descending count, rows without
// blocks last), the overflow beyond the slice cap, and the row maps reset.
__global__ void k_contact_rows(unsigned n, const unsigned *off, const unsigned *col,
                               const unsigned *tr_off, const uint2 *tr, const unsigned *mask,
                               unsigned *key, unsigned *perm, unsigned *row_ovf,
                               unsigned *row_flag, unsigned *index, unsigned *ovf_index,
                               unsigned *n_rows) {
    unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const unsigned c = dyn_row_count(i, off, col, tr_off, tr, mask);
    key[i] = c ? 0xFFFFu - (c < 0xFFFEu ? c : 0xFFFEu) : 0xFFFFu;
    perm[i] = i;
    const unsigned o = c > kDynSliceCap ? c - kDynSliceCap : 0u;
    row_ovf[i] = o;
    row_flag[i] = o ? 1u : 0u;
    index[i] = 0xFFFFFFFFu;
    ovf_index[i] = 0xFFFFFFFFu;
    if (c) atomicAdd(n_rows, 1u);
}

// Width of each contact slice: its first (longest) row's count, capped.
__global__ void k_contact_slice_k(unsigned max_slices, const unsigned *n_rows,
                                  const unsigned *key, unsigned *slice_k) {
    unsigned sl = blockIdx.x * blockDim.x + threadIdx.x;
    if (sl >= max_slices) return;
    const unsigned m = *n_rows;
    unsigned k = 0;
    if (sl * kSliceRows < m) {
        unsigned c = 0xFFFFu - key[sl * kSliceRows];
        k = c < kDynSliceCap ? c : kDynSliceCap;
    }
    slice_k[sl] = k;
}

// The contact layout's sizes from its scans. A layout sized for bounds that
// the totals would overrun (which the bounds rule out), or one whose row sort
// timed out, is left empty and flagged, so no later kernel writes past it.
__global__ void k_dyn_sizes(unsigned n, unsigned max_slices, const unsigned *counters,
                            const unsigned *slice_off, const unsigned *ovf_off,
                            const unsigned *flag_off, unsigned slot_cap, unsigned entry_cap,
                            unsigned *sizes, unsigned *status) {
    unsigned rows = counters[0], n_ovf = flag_off[n];
    const unsigned slots = slice_off[max_slices], entries = ovf_off[n];
    unsigned bad = 0u;
    if (counters[1]) bad |= STATUS_SORT_LOOKBACK_TIMEOUT;
    if (slots > slot_cap || entries > entry_cap) bad |= STATUS_BLOCK_OVERFLOW;
    if (bad) {
        rows = 0u;
        n_ovf = 0u;
        if (status) atomicOr(status, bad);
    }
    sizes[0] = rows;
    sizes[1] = n_ovf;
    sizes[2] = slots;
    sizes[3] = entries;
}

__device__ __forceinline__ void put_slot(unsigned *out_col, float *out_val, unsigned s,
                                         unsigned lane, unsigned j, const float (&m)[9]) {
    out_col[(size_t)s * kSliceRows + lane] = j;
    float *d = out_val + (size_t)s * 9 * kSliceRows + lane;
#pragma unroll
    for (int e = 0; e < 9; ++e) d[e * kSliceRows] = m[e];
}

struct DynFillOut {
    const unsigned *slice_off, *ovf_off, *flag_off, *perm, *n_rows;
    unsigned *col;
    float *val;
    unsigned *index, *ovf_row, *ovf_col, *ovf_index;
    uint2 *ovf_range;
    float *ovf_val;
    // the contact block each slot / overflow entry copies (bit 31:
    // transposed), or kPad
    unsigned *src, *ovf_src;
};

// Sorted position q: the row's entries in order, the first K (the slice
// width) to the slice slots, the rest to the row's overflow range.
__global__ void k_contact_fill(unsigned max_slices, const unsigned *off, const unsigned *col,
                               const float *upper, const unsigned *tr_off, const uint2 *tr,
                               const unsigned *mask, DynFillOut o) {
    unsigned q = blockIdx.x * blockDim.x + threadIdx.x;
    unsigned sl = q / kSliceRows, lane = q % kSliceRows;
    const unsigned m = *o.n_rows;
    if (sl >= max_slices || sl * kSliceRows >= m) return;
    const unsigned s0 = o.slice_off[sl], K = o.slice_off[sl + 1] - s0;
    const bool real = q < m;
    const unsigned i = real ? o.perm[q] : o.perm[m - 1];
    const unsigned obase = real ? o.ovf_off[i] : 0u;
    unsigned k = 0;
    auto put = [&](unsigned j, const float (&mm)[9], unsigned src) {
        if (k < K) {
            put_slot(o.col, o.val, s0 + k, lane, j, mm);
            o.src[(size_t)(s0 + k) * kSliceRows + lane] = src;
        } else {
            unsigned e = obase + (k - K);
            o.ovf_col[e] = j;
            o.ovf_src[e] = src;
#pragma unroll
            for (int t = 0; t < 9; ++t) o.ovf_val[9 * (size_t)e + t] = mm[t];
        }
        ++k;
    };
    if (real) {
        for (unsigned p = off[i]; p < off[i + 1]; ++p) {
            unsigned j = col[p];
            if (mask[j]) continue;
            const float *b = upper + 9 * (size_t)p;
            float mm[9];
#pragma unroll
            for (int e = 0; e < 9; ++e) mm[e] = b[e];
            put(j, mm, p);
        }
        for (unsigned p = tr_off[i]; p < tr_off[i + 1]; ++p) {
            uint2 rp = tr[p];
            if (mask[rp.x]) continue;
            const float *b = upper + 9 * (size_t)rp.y;
            float mm[9];
#pragma unroll
            for (int r = 0; r < 3; ++r)
#pragma unroll
                for (int c = 0; c < 3; ++c) mm[3 * c + r] = b[3 * r + c];
            put(rp.x, mm, rp.y | kTransposed);
        }
        o.index[i] = q;
    }
    const float zero[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    for (unsigned t = k; t < K; ++t) {
        put_slot(o.col, o.val, s0 + t, lane, i, zero);
        o.src[(size_t)(s0 + t) * kSliceRows + lane] = kPad;
    }
    if (real && k > K) {
        unsigned idx = o.flag_off[i];
        o.ovf_row[idx] = i;
        o.ovf_range[idx] = make_uint2(obase, k - K);
        o.ovf_index[i] = idx;
    }
}

// Estimated cost of each product task, in warp slot-steps: a half slice
// walks half its slots per lane; an overflow row walks its entries 32 at a
// time. The constant covers the per-task epilogue. Task order: overflow
// rows, contact half slices, fixed half slices (TaskSpace); entries past the
// solve's task count, up to the launch's bound, cost nothing.
__global__ void k_task_cost(PcgOperator A, unsigned bound, unsigned *cost) {
    unsigned t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= bound) return;
    const TaskSpace ts(A);
    unsigned c;
    if (t >= ts.total) {
        cost[t] = 0u;
        return;
    } else if (t < ts.t1) {
        c = (A.ovf.range[t].y + 31) / 32;
    } else if (t < ts.t2) {
        unsigned sl = (t - ts.t1) >> 1;
        c = (A.contact.sell.slice_off[sl + 1] - A.contact.sell.slice_off[sl] + 1) / 2;
    } else {
        unsigned sl = (t - ts.t2) >> 1;
        c = (A.fixed.slice_off[sl + 1] - A.fixed.slice_off[sl] + 1) / 2;
    }
    cost[t] = c + 2u;
}

// Block b takes the tasks whose cost prefix falls in [b Ws / nb,
// (b+1) Ws / nb), Ws the static share of the total cost W; start[nb] is the
// first task of the common pool.
__global__ void k_task_split(PcgOperator A, const unsigned *cost_off, unsigned nb,
                             unsigned sixteenths, unsigned *start) {
    unsigned b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b > nb) return;
    const unsigned T = TaskSpace(A).total;
    const unsigned long long W = (unsigned long long)cost_off[T] * sixteenths / 16u;
    const unsigned long long target = W * b / nb;
    unsigned lo = 0, hi = T; // first t with cost_off[t] >= target
    while (lo < hi) {
        unsigned mid = (lo + hi) >> 1;
        if ((unsigned long long)cost_off[mid] < target) lo = mid + 1;
        else hi = mid;
    }
    start[b] = lo;
}

} // namespace

void PcgWorkspace::reserve(unsigned n) {
    R.reserve(8 * (size_t)n);
    p.reserve(n);
    Ap.reserve(n);
    Y.reserve(n);
    if (grid == 0) {
        int dev = 0, sms = 0, per_sm = 0;
        PPF_CUDA(cudaGetDevice(&dev));
        PPF_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
        PPF_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_pcg, kThreads, 0));
        if (per_sm < 1) per_sm = 1;
        if (per_sm > 1) per_sm = 1;
        grid = (unsigned)(sms * per_sm);
        threads = kThreads;
        // the largest cluster the kernels can run as (one CTA per SM, so
        // the CTAs of a GPC): 16 when the device allows clusters that large
        const size_t schwarz_smem = (size_t)kWarps * kSchwarzWarpFloats * sizeof(float);
        PPF_CUDA(cudaFuncSetAttribute((const void *)k_pcg_schwarz,
                                      cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)schwarz_smem));
        max_cluster = 16;
        for (const void *kf : {(const void *)k_pcg, (const void *)k_pcg_factor,
                               (const void *)k_pcg_schwarz}) {
            if (cudaFuncSetAttribute(kf, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) !=
                cudaSuccess) {
                cudaGetLastError();
                max_cluster = std::min(max_cluster, 8u);
                continue;
            }
            cudaLaunchConfig_t cfg = {};
            cfg.gridDim = dim3(16);
            cfg.blockDim = dim3(kThreads);
            cfg.dynamicSmemBytes = kf == (const void *)k_pcg_schwarz ? schwarz_smem : 0;
            cudaLaunchAttribute attr[1];
            attr[0].id = cudaLaunchAttributeClusterDimension;
            attr[0].val.clusterDim.x = 16;
            attr[0].val.clusterDim.y = 1;
            attr[0].val.clusterDim.z = 1;
            cfg.attrs = attr;
            cfg.numAttrs = 1;
            int size = 0;
            if (cudaOccupancyMaxPotentialClusterSize(&size, kf, &cfg) != cudaSuccess) {
                cudaGetLastError();
                size = 0;
            }
            unsigned c = 1;
            while (2 * c <= (unsigned)std::max(size, 1)) c *= 2;
            max_cluster = std::min(max_cluster, c);
        }
        if (max_cluster < 2) max_cluster = 0;
    }
    partials.reserve(6 * (size_t)grid + 4);
    barrier.reserve(4);
    result.reserve(1);
}

void sell_build_fixed(unsigned n, const std::vector<unsigned> &off,
                      const std::vector<unsigned> &col, const std::vector<unsigned> &tr_off,
                      const std::vector<uint2> &tr, SellLayout &out) {
    const unsigned n_slices = (n + kSliceRows - 1) / kSliceRows;
    std::vector<unsigned> slice_off(n_slices + 1, 0u), slice_mid(n_slices, 0u);
    for (unsigned sl = 0; sl < n_slices; ++sl) {
        unsigned kl = 0, ku = 0;
        for (unsigned l = 0; l < kSliceRows; ++l) {
            unsigned i = sl * kSliceRows + l;
            if (i >= n) break;
            kl = std::max(kl, tr_off[i + 1] - tr_off[i]);
            ku = std::max(ku, off[i + 1] - off[i]);
        }
        slice_mid[sl] = slice_off[sl] + kl;
        slice_off[sl + 1] = slice_mid[sl] + ku;
    }
    const unsigned slots = slice_off[n_slices];
    std::vector<unsigned> c((size_t)slots * kSliceRows), src((size_t)slots * kSliceRows);
    for (unsigned sl = 0; sl < n_slices; ++sl)
        for (unsigned l = 0; l < kSliceRows; ++l) {
            unsigned i = sl * kSliceRows + l;
            unsigned self = i < n ? i : n - 1;
            auto put = [&](unsigned slot, unsigned j, unsigned s) {
                size_t e = (size_t)slot * kSliceRows + l;
                c[e] = j;
                src[e] = s;
            };
            unsigned k = slice_off[sl];
            if (i < n)
                for (unsigned q = tr_off[i]; q < tr_off[i + 1]; ++q)
                    put(k++, tr[q].x, tr[q].y | kTransposed);
            while (k < slice_mid[sl]) put(k++, self, kPad);
            if (i < n)
                for (unsigned q = off[i]; q < off[i + 1]; ++q) put(k++, col[q], q);
            while (k < slice_off[sl + 1]) put(k++, self, kPad);
        }
    out.n_slices = n_slices;
    out.slots = slots;
    out.slice_mid.reserve(n_slices + 1);
    if (n_slices)
        PPF_CUDA(cudaMemcpy(out.slice_mid.data(), slice_mid.data(), n_slices * 4,
                            cudaMemcpyHostToDevice));
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
                    DynLayout &D, cudaStream_t q, unsigned block_cap, unsigned *d_status) {
    const unsigned max_slices = (n + kSliceRows - 1) / kSliceRows;
    SellLayout &out = D.sell;
    out.slice_off.reserve(max_slices + 1);
    D.key.reserve(n + 1);
    D.perm.reserve(n + 1);
    D.index.reserve(n + 1);
    D.slice_k.reserve(max_slices + 1);
    D.row_ovf.reserve(n + 1);
    D.row_flag.reserve(n + 1);
    D.ovf_off.reserve(n + 1);
    D.flag_off.reserve(n + 1);
    D.ovf_index.reserve(n + 1);
    D.counters.reserve(4);
    D.sizes.reserve(4);
    D.scan_tmp.reserve(scan_tmp_size(n + 1));
    // Bounds for a layout sized before its totals are known: each contact
    // block sits in two rows, so the rows hold at most 2 block_cap entries;
    // with rows in order of decreasing count every slice after the first is
    // at most as wide as the mean of the 32 rows before it, so the slots are
    // at most one capped slice plus 2 block_cap / 32.
    const unsigned long long entry_cap = 2ull * block_cap;
    const unsigned long long slot_cap = kDynSliceCap + (entry_cap + kSliceRows - 1) / kSliceRows;
    if (block_cap) {
        if (slot_cap * kSliceRows * 9 >= 0xFFFFFFFFull || entry_cap * 9 >= 0xFFFFFFFFull)
            throw FatalError(4, "contact layout bound exceeds 32-bit indexing");
        out.col.reserve(slot_cap * kSliceRows + 1);
        out.val.reserve(slot_cap * kSliceRows * 9 + 1);
        out.src.reserve(slot_cap * kSliceRows + 1);
        D.ovf_src.reserve(entry_cap + 1);
        D.ovf_col.reserve(entry_cap + 1);
        D.ovf_val.reserve(9 * entry_cap + 1);
        D.ovf_row.reserve(n + 1);
        D.ovf_range.reserve(n + 1);
    }
    PPF_CUDA(cudaMemsetAsync(D.counters.data(), 0, 4 * sizeof(unsigned), q));
    k_contact_rows<<<div_up(n, 256u), 256, 0, q>>>(n, off, col, tr_off, tr, dof_mask,
                                                   D.key.data(), D.perm.data(),
                                                   D.row_ovf.data(), D.row_flag.data(),
                                                   D.index.data(), D.ovf_index.data(),
                                                   D.counters.data());
    PPF_LAUNCH_CHECK();
    // stable: rows of equal count keep their index order
    radix_sort_pairs(D.key.data(), D.perm.data(), n, 16, D.sort_ws, D.counters.data() + 1, q);
    k_contact_slice_k<<<div_up(max_slices, 256u), 256, 0, q>>>(max_slices, D.counters.data(),
                                                               D.key.data(), D.slice_k.data());
    PPF_LAUNCH_CHECK();
    exclusive_scan(D.slice_k.data(), out.slice_off.data(), max_slices, D.scan_tmp.data(), q);
    exclusive_scan(D.row_ovf.data(), D.ovf_off.data(), n, D.scan_tmp.data(), q);
    exclusive_scan(D.row_flag.data(), D.flag_off.data(), n, D.scan_tmp.data(), q);
    k_dyn_sizes<<<1, 1, 0, q>>>(n, max_slices, D.counters.data(), out.slice_off.data(),
                                D.ovf_off.data(), D.flag_off.data(),
                                block_cap ? (unsigned)slot_cap : 0xFFFFFFFFu,
                                block_cap ? (unsigned)entry_cap : 0xFFFFFFFFu, D.sizes.data(),
                                d_status);
    PPF_LAUNCH_CHECK();
    if (block_cap) {
        D.rows = n;
        out.n_slices = max_slices;
        out.slots = (unsigned)slot_cap;
        D.ovf_entries = (unsigned)entry_cap;
        D.n_ovf = n;
    } else {
        unsigned totals[5] = {0, 0, 0, 0, 0};
        PPF_CUDA(cudaMemcpyAsync(&totals[0], D.counters.data(), 2 * sizeof(unsigned),
                                 cudaMemcpyDeviceToHost, q));
        PPF_CUDA(cudaMemcpyAsync(&totals[2], out.slice_off.data() + max_slices,
                                 sizeof(unsigned), cudaMemcpyDeviceToHost, q));
        PPF_CUDA(cudaMemcpyAsync(&totals[3], D.ovf_off.data() + n, sizeof(unsigned),
                                 cudaMemcpyDeviceToHost, q));
        PPF_CUDA(cudaMemcpyAsync(&totals[4], D.flag_off.data() + n, sizeof(unsigned),
                                 cudaMemcpyDeviceToHost, q));
        PPF_CUDA(cudaStreamSynchronize(q));
        g_d2h_bytes += sizeof(totals);
        if (totals[1]) throw FatalError(4, "contact-row sort look-back timed out");
        D.rows = totals[0];
        out.n_slices = (D.rows + kSliceRows - 1) / kSliceRows;
        out.slots = totals[2];
        D.ovf_entries = totals[3];
        D.n_ovf = totals[4];
        out.col.reserve((size_t)out.slots * kSliceRows + 1);
        out.val.reserve((size_t)out.slots * kSliceRows * 9 + 1);
        out.src.reserve((size_t)out.slots * kSliceRows + 1);
        D.ovf_src.reserve(D.ovf_entries + 1);
        D.ovf_col.reserve(D.ovf_entries + 1);
        D.ovf_val.reserve(9 * (size_t)D.ovf_entries + 1);
        D.ovf_row.reserve(D.n_ovf + 1);
        D.ovf_range.reserve(D.n_ovf + 1);
        if (!D.rows) return;
    }
    DynFillOut o{out.slice_off.data(), D.ovf_off.data(), D.flag_off.data(), D.perm.data(),
                 D.sizes.data(),       out.col.data(),   out.val.data(),    D.index.data(),
                 D.ovf_row.data(),     D.ovf_col.data(), D.ovf_index.data(), D.ovf_range.data(),
                 D.ovf_val.data(),     out.src.data(),   D.ovf_src.data()};
    k_contact_fill<<<div_up(out.n_slices * kSliceRows, 256u), 256, 0, q>>>(
        out.n_slices, off, col, val, tr_off, tr, dof_mask, o);
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
                PcgWorkspace &ws, cudaStream_t q, const unsigned *run_if) {
    ws.reserve(A.n);
    PPF_CUDA(cudaMemsetAsync(ws.barrier.data(), 0, 4 * sizeof(unsigned), q));
    ws.Ap_ovf.reserve(A.ovf.count + 1);
    ws.Ap_c.reserve(A.contact.rows + 1);
    // balanced task ranges per block; the contact counts are an upper bound
    // here, the task kernels read the solve's own from the layout
    const unsigned T = 2 * A.fixed.n_slices + 2 * A.contact.sell.n_slices + A.ovf.count;
    ws.task_cost.reserve(T + 1);
    ws.task_off.reserve(T + 1);
    ws.task_start.reserve(ws.grid + 1);
    ws.scan_tmp.reserve(scan_tmp_size(T + 1));
    k_task_cost<<<div_up(T, 256u), 256, 0, q>>>(A, T, ws.task_cost.data());
    PPF_LAUNCH_CHECK();
    exclusive_scan(ws.task_cost.data(), ws.task_off.data(), T, ws.scan_tmp.data(), q);
    // the whole grid (a cooperative launch), or one cluster of ws.cluster CTAs
    const bool one_cluster = ws.cluster >= 2 && ws.cluster <= ws.max_cluster;
    const unsigned nb = one_cluster ? ws.cluster : ws.grid;
    const unsigned launch_cluster = one_cluster ? nb : 0u;
    k_task_split<<<div_up(nb + 1, 256u), 256, 0, q>>>(
        A, ws.task_off.data(), nb, ws.static_sixteenths ? ws.static_sixteenths : kStaticSixteenths,
        ws.task_start.data());
    PPF_LAUNCH_CHECK();
    // one counter per product phase: the initial product, then one (block-
    // Jacobi) or three (factored) per iteration, plus the factored start
    const unsigned n_ctr = 3 * max_iter + 8;
    ws.dyn_ctr.reserve(n_ctr);
    PPF_CUDA(cudaMemsetAsync(ws.dyn_ctr.data(), 0, n_ctr * sizeof(unsigned), q));
    PcgArgs g{A,
              ws.task_start.data(),
              ws.dyn_ctr.data(),
              n_ctr,
              x,
              r,
              ws.R.data(),
              ws.p.data(),
              ws.Ap.data(),
              ws.Ap_c.data(),
              ws.Ap_ovf.data(),
              ws.Y.data(),
              ws.partials.data(),
              ws.barrier.data(),
              launch_cluster,
              tol,
              max_iter,
              ws.result.data(),
              run_if};
    void *args[] = {(void *)&g};
    const void *kernel = A.schwarz.n_agg ? (const void *)k_pcg_schwarz
                         : A.factor.diag ? (const void *)k_pcg_factor
                                         : (const void *)k_pcg;
    const size_t dyn_smem =
        A.schwarz.n_agg ? (size_t)kWarps * kSchwarzWarpFloats * sizeof(float) : 0;
    if (launch_cluster == 0) {
        PPF_CUDA(cudaLaunchCooperativeKernel(kernel, dim3(nb), dim3(ws.threads), args, dyn_smem,
                                             q));
    } else {
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3(nb);
        cfg.blockDim = dim3(kernel == (const void *)k_pcg && ws.cluster_threads
                                ? ws.cluster_threads
                                : ws.threads);
        cfg.dynamicSmemBytes = dyn_smem;
        cfg.stream = q;
        cudaLaunchAttribute attr[1];
        attr[0].id = cudaLaunchAttributeClusterDimension;
        attr[0].val.clusterDim.x = launch_cluster;
        attr[0].val.clusterDim.y = 1;
        attr[0].val.clusterDim.z = 1;
        cfg.attrs = attr;
        cfg.numAttrs = 1;
        PPF_CUDA(cudaLaunchKernelExC(&cfg, kernel, args));
    }
    count_launches();
}

} // namespace gpu
} // namespace ppf
