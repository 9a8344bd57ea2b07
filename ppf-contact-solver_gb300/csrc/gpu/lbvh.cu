// lbvh.cu -- LBVH build and refit kernels.
//
// Arithmetic that decides the tree (centroids, bounds, Morton codes) uses the
// same single-precision operations in the same order as the reference's
// lbvh.cu:120-279, with no fused multiply-add (this translation unit is built
// with -fmad=false), so the codes -- and therefore the permutation and the
// topology -- are bit-identical to the CPU oracle's. The swept leaf box uses an
// explicit fmaf for `e * (y1 - y0) + y0`, the contraction the reference's
// default build applies to that expression.
#include "lbvh.cuh"

namespace ppf {
namespace gpu {

namespace {

constexpr unsigned kBlock = 256;

__device__ __forceinline__ Vec3 prim_centroid(PrimKind kind,
                                              const unsigned *prims,
                                              const float *x, unsigned i) {
    if (kind == PRIM_FACE) {
        unsigned a = prims[3 * i], b = prims[3 * i + 1], c = prims[3 * i + 2];
        Vec3 r;
#pragma unroll
        for (int d = 0; d < 3; ++d)
            r[d] = (x[3 * a + d] + x[3 * b + d] + x[3 * c + d]) / 3.0f;
        return r;
    } else if (kind == PRIM_EDGE) {
        unsigned a = prims[2 * i], b = prims[2 * i + 1];
        Vec3 r;
#pragma unroll
        for (int d = 0; d < 3; ++d) r[d] = (x[3 * a + d] + x[3 * b + d]) / 2.0f;
        return r;
    } else {
        unsigned a = prims ? prims[i] : i;
        return vec3(x[3 * a], x[3 * a + 1], x[3 * a + 2]);
    }
}

__global__ void k_init_bounds(unsigned *bounds) {
    unsigned t = threadIdx.x;
    if (t < 3) bounds[t] = 0xffffffffu;    // min: ordered(+inf) or larger
    else if (t < 6) bounds[t] = 0u;        // max
}

__global__ void k_bounds(PrimKind kind, const unsigned *prims, const float *x,
                         unsigned n, unsigned *bounds) {
    __shared__ float s_min[3][kBlock / 32], s_max[3][kBlock / 32];
    unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
    float lo[3] = {INFINITY, INFINITY, INFINITY};
    float hi[3] = {-INFINITY, -INFINITY, -INFINITY};
    if (i < n) {
        Vec3 c = prim_centroid(kind, prims, x, i);
#pragma unroll
        for (int d = 0; d < 3; ++d) lo[d] = hi[d] = c[d];
    }
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        for (int off = 16; off > 0; off >>= 1) {
            lo[d] = fminf(lo[d], __shfl_xor_sync(0xffffffffu, lo[d], off));
            hi[d] = fmaxf(hi[d], __shfl_xor_sync(0xffffffffu, hi[d], off));
        }
    }
    unsigned warp = threadIdx.x >> 5, lane = threadIdx.x & 31u;
    if (lane == 0) {
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            s_min[d][warp] = lo[d];
            s_max[d][warp] = hi[d];
        }
    }
    __syncthreads();
    if (threadIdx.x < 3) {
        int d = threadIdx.x;
        float a = INFINITY, b = -INFINITY;
        for (unsigned w = 0; w < blockDim.x / 32; ++w) {
            a = fminf(a, s_min[d][w]);
            b = fmaxf(b, s_max[d][w]);
        }
        if (a <= b) {
            atomicMin(&bounds[d], float_to_ordered(a));
            atomicMax(&bounds[d + 3], float_to_ordered(b));
        }
    }
}

__device__ __forceinline__ unsigned expand_bits10(unsigned v) {
    v = (v | (v << 16)) & 0x030000FFu;
    v = (v | (v << 8)) & 0x0300F00Fu;
    v = (v | (v << 4)) & 0x030C30C3u;
    v = (v | (v << 2)) & 0x09249249u;
    return v;
}

// Morton code of a centroid in the scene box (lbvh.cu:253-279).
__global__ void k_morton(PrimKind kind, const unsigned *prims, const float *x,
                         unsigned n, const unsigned *bounds, unsigned *keys,
                         unsigned *vals) {
    unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float lo[3], hi[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        lo[d] = ordered_to_float(bounds[d]);
        hi[d] = ordered_to_float(bounds[d + 3]);
    }
    Vec3 c = prim_centroid(kind, prims, x, i);
    unsigned q[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        float ext = hi[d] - lo[d];
        float scale = ext > 1e-10f ? 1023.0f / ext : 0.0f;
        q[d] = (unsigned)fminf(1023.0f, fmaxf(0.0f, (c[d] - lo[d]) * scale));
    }
    keys[i] = expand_bits10(q[0]) | (expand_bits10(q[1]) << 1) |
              (expand_bits10(q[2]) << 2);
    vals[i] = i;
}

// Length of the common prefix of keys i and j, ties broken by index
// (lbvh.cu:289-301). -1 outside [0, n).
__device__ __forceinline__ int common_prefix(const unsigned *keys, int n, int i,
                                             int j) {
    if (j < 0 || j >= n) return -1;
    unsigned ki = keys[i], kj = keys[j];
    if (ki == kj) return 32 + __clz((unsigned)(i ^ j));
    return __clz(ki ^ kj);
}

// Karras 2012 internal node i: range direction, range end, split.
__global__ void k_karras(const unsigned *keys, const unsigned *vals, unsigned n,
                         uint2 *node, unsigned *parent, unsigned *visit) {
    unsigned t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < n) node[t] = make_uint2(vals[t] + 1u, 0u);
    if (t + 1 >= n) return;
    int i = (int)t, N = (int)n;
    visit[i] = 0u;
    int d = common_prefix(keys, N, i, i + 1) > common_prefix(keys, N, i, i - 1)
                ? 1
                : -1;
    int dmin = common_prefix(keys, N, i, i - d);
    int lmax = 2;
    while (common_prefix(keys, N, i, i + lmax * d) > dmin) lmax *= 2;
    int l = 0;
    for (int step = lmax / 2; step >= 1; step /= 2)
        if (common_prefix(keys, N, i, i + (l + step) * d) > dmin) l += step;
    int j = i + l * d;
    int left = min(i, j), right = max(i, j);
    int dnode = common_prefix(keys, N, left, right);
    int s = 0, span = right - left;
    do {
        span = (span + 1) / 2;
        if (common_prefix(keys, N, left, left + s + span) > dnode) s += span;
    } while (span > 1);
    int split = left + s;
    unsigned lc = (left == split) ? (unsigned)left : n + (unsigned)split;
    unsigned rc = (split + 1 == right) ? (unsigned)right : n + (unsigned)split + 1u;
    unsigned self = n + t;
    node[self] = make_uint2(lc + 1u, rc + 1u);
    parent[lc] = self;
    parent[rc] = self;
    if (t == 0) parent[self] = self;
}

// One tree's arrays for a refit.
struct RefitTree {
    PrimKind kind;
    const unsigned *prims;
    const float *margin;
    const unsigned char *active;
    unsigned n;
    const uint2 *node;
    const unsigned *parent;
    float4 *bmin, *bmax;
    unsigned *visit;
    unsigned root;
};

// Leaf box of the sweep x0 -> x0 + e (x1 - x0), widened by the primitive's
// margin (lbvh.cu:623-731), then the climb to the root: the second child to
// arrive at a node merges both boxes (active-aware, lbvh.cu:778-823).
__device__ void refit_leaf(const RefitTree &t, unsigned leaf, const float *x0, const float *x1,
                           float e, unsigned *status) {
    const PrimKind kind = t.kind;
    const unsigned *prims = t.prims;
    const unsigned n = t.n, root = t.root;
    const uint2 *node = t.node;
    const unsigned *parent = t.parent;
    float4 *bmin = t.bmin, *bmax = t.bmax;
    unsigned *visit = t.visit;
    unsigned prim = node[leaf].x - 1u;
    unsigned v[3];
    int nv;
    if (kind == PRIM_FACE) {
        nv = 3;
        v[0] = prims[3 * prim];
        v[1] = prims[3 * prim + 1];
        v[2] = prims[3 * prim + 2];
    } else if (kind == PRIM_EDGE) {
        nv = 2;
        v[0] = prims[2 * prim];
        v[1] = prims[2 * prim + 1];
    } else {
        nv = 1;
        v[0] = prims ? prims[prim] : prim;
    }
    float mg = t.margin[prim];
    float lo[3], hi[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        float a0 = INFINITY, b0 = -INFINITY, a1 = INFINITY, b1 = -INFINITY;
        for (int k = 0; k < nv; ++k) {
            float y0 = x0[3 * v[k] + d];
            float y1 = x1[3 * v[k] + d];
            float z = fmaf(e, y1 - y0, y0);
            a0 = fminf(a0, y0);
            b0 = fmaxf(b0, y0);
            a1 = fminf(a1, z);
            b1 = fmaxf(b1, z);
        }
        lo[d] = fminf(a0, a1) - mg;
        hi[d] = fmaxf(b0, b1) + mg;
    }
    float act = (t.active && !t.active[prim]) ? 0.0f : 1.0f;
    bmin[leaf] = make_float4(lo[0], lo[1], lo[2], act);
    bmax[leaf] = make_float4(hi[0], hi[1], hi[2], 0.0f);

    unsigned cur = leaf;
    unsigned guard = 0;
    while (cur != root) {
        unsigned p = parent[cur];
        __threadfence();
        unsigned prev = atomicAdd(&visit[p - n], 1u);
        if (prev == 0u) return; // sibling not finished; it will continue
        visit[p - n] = 0u;      // last toucher resets for the next refit
        uint2 ch = node[p];
        unsigned l = ch.x - 1u, r = ch.y - 1u;
        float4 lmin = __ldcg(&bmin[l]), lmax = __ldcg(&bmax[l]);
        float4 rmin = __ldcg(&bmin[r]), rmax = __ldcg(&bmax[r]);
        float4 omin, omax;
        bool la = lmin.w != 0.0f, ra = rmin.w != 0.0f;
        if (la && ra) {
            omin = make_float4(lmin.x < rmin.x ? lmin.x : rmin.x,
                               lmin.y < rmin.y ? lmin.y : rmin.y,
                               lmin.z < rmin.z ? lmin.z : rmin.z, 1.0f);
            omax = make_float4(lmax.x > rmax.x ? lmax.x : rmax.x,
                               lmax.y > rmax.y ? lmax.y : rmax.y,
                               lmax.z > rmax.z ? lmax.z : rmax.z, 0.0f);
        } else if (la) {
            omin = lmin;
            omax = lmax;
        } else if (ra) {
            omin = rmin;
            omax = rmax;
        } else {
            omin = lmin;
            omin.w = 0.0f;
            omax = lmax;
        }
        __stcg(&bmin[p], omin);
        __stcg(&bmax[p], omax);
        cur = p;
        if (++guard > 2u * n + 64u) {
            atomicOr(status, STATUS_REFIT_CYCLE);
            return;
        }
    }
}

// Up to three trees refit in one launch: thread t takes leaf t of the first
// tree, then the second's, then the third's, so the climbs of all three run
// together instead of one launch after another.
struct RefitTrees {
    RefitTree tree[3];
    unsigned count;
};

__global__ void k_leaf_refit(RefitTrees ts, const float *x0, const float *x1, float e,
                             unsigned *status) {
    unsigned leaf = blockIdx.x * blockDim.x + threadIdx.x;
    for (unsigned k = 0; k < ts.count; ++k) {
        if (leaf < ts.tree[k].n) {
            refit_leaf(ts.tree[k], leaf, x0, x1, e, status);
            return;
        }
        leaf -= ts.tree[k].n;
    }
}

__global__ void k_single_leaf(PrimKind kind, const unsigned *prims, uint2 *node,
                              unsigned *parent, uint2 *link) {
    node[0] = make_uint2(1u, 0u);
    parent[0] = 0u;
    link[0] = make_uint2(0u | kLinkLeaf, kLinkEnd);
}

// Traversal links of every node: its left child (or primitive, for a leaf)
// and its escape node, the right sibling of the nearest ancestor-or-self that
// is a left child (kLinkEnd when there is none). A stackless depth-first walk
// goes to the left child on a box hit and to the escape node otherwise.
__global__ void k_links(unsigned n, const uint2 *node, const unsigned *parent, unsigned root,
                        uint2 *link, unsigned *status) {
    const unsigned t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= 2 * n - 1) return;
    const uint2 nd = node[t];
    const unsigned first = nd.y == 0u ? ((nd.x - 1u) | kLinkLeaf) : nd.x - 1u;
    unsigned esc = kLinkEnd, cur = t;
    for (unsigned guard = 0; cur != root; ++guard) {
        const unsigned p = parent[cur];
        const uint2 pn = node[p];
        if (pn.x - 1u == cur) {
            esc = pn.y - 1u;
            break;
        }
        cur = p;
        if (guard > 2 * n + 64u) {
            atomicOr(status, STATUS_REFIT_CYCLE);
            break;
        }
    }
    link[t] = make_uint2(first, esc);
}

} // namespace

void Lbvh::reserve(unsigned count) {
    unsigned nn = count == 0 ? 1 : 2 * count - 1;
    node.reserve(nn);
    link.reserve(nn);
    parent.reserve(nn);
    bmin.reserve(nn);
    bmax.reserve(nn);
    visit.reserve(count);
    keys.reserve(count);
    vals.reserve(count);
    bounds.reserve(8);
}

void Lbvh::release() {
    node.release();
    link.release();
    parent.release();
    bmin.release();
    bmax.release();
    visit.release();
    keys.release();
    vals.release();
    bounds.release();
}

void lbvh_build(Lbvh &bvh, const PrimSet &ps, const float *x_tree,
                const float *x0, const float *x1, float extrapolate,
                RadixSortWorkspace &ws, unsigned *d_status, cudaStream_t s, bool refit) {
    unsigned n = ps.count;
    bvh.reserve(n);
    bvh.n = n;
    if (n == 0) return;
    unsigned grid = div_up(n, kBlock);
    if (n == 1) {
        k_single_leaf<<<1, 1, 0, s>>>(ps.kind, ps.prims, bvh.node.data(),
                                      bvh.parent.data(), bvh.link.data());
        PPF_LAUNCH_CHECK();
        bvh.root = 0;
    } else {
        k_init_bounds<<<1, 32, 0, s>>>(bvh.bounds.data());
        PPF_LAUNCH_CHECK();
        k_bounds<<<grid, kBlock, 0, s>>>(ps.kind, ps.prims, x_tree, n,
                                         bvh.bounds.data());
        PPF_LAUNCH_CHECK();
        k_morton<<<grid, kBlock, 0, s>>>(ps.kind, ps.prims, x_tree, n,
                                         bvh.bounds.data(), bvh.keys.data(),
                                         bvh.vals.data());
        PPF_LAUNCH_CHECK();
        radix_sort_pairs(bvh.keys.data(), bvh.vals.data(), n, 30, ws, d_status,
                         s);
        k_karras<<<grid, kBlock, 0, s>>>(bvh.keys.data(), bvh.vals.data(), n,
                                         bvh.node.data(), bvh.parent.data(),
                                         bvh.visit.data());
        PPF_LAUNCH_CHECK();
        bvh.root = n;
        k_links<<<div_up(2 * n - 1, kBlock), kBlock, 0, s>>>(n, bvh.node.data(),
                                                             bvh.parent.data(), bvh.root,
                                                             bvh.link.data(), d_status);
        PPF_LAUNCH_CHECK();
    }
    if (refit) lbvh_refit(bvh, ps, x0, x1, extrapolate, d_status, s);
}

namespace {
RefitTree refit_tree(Lbvh &bvh, const PrimSet &ps) {
    return RefitTree{ps.kind,           ps.prims,          ps.margin,         ps.active,
                     bvh.n,             bvh.node.data(),   bvh.parent.data(), bvh.bmin.data(),
                     bvh.bmax.data(),   bvh.visit.data(),  bvh.root};
}
} // namespace

void lbvh_refit(Lbvh &bvh, const PrimSet &ps, const float *x0, const float *x1,
                float extrapolate, unsigned *d_status, cudaStream_t s) {
    Lbvh *trees[1] = {&bvh};
    lbvh_refit_many(trees, &ps, 1, x0, x1, extrapolate, d_status, s);
}

void lbvh_refit_many(Lbvh *const *trees, const PrimSet *ps, unsigned count, const float *x0,
                     const float *x1, float extrapolate, unsigned *d_status, cudaStream_t s) {
    RefitTrees ts{};
    unsigned total = 0;
    for (unsigned k = 0; k < count && k < 3; ++k) {
        if (trees[k]->n == 0) continue;
        ts.tree[ts.count++] = refit_tree(*trees[k], ps[k]);
        total += trees[k]->n;
    }
    if (total == 0) return;
    k_leaf_refit<<<div_up(total, kBlock), kBlock, 0, s>>>(ts, x0, x1, extrapolate, d_status);
    PPF_LAUNCH_CHECK();
}

} // namespace gpu
} // namespace ppf
