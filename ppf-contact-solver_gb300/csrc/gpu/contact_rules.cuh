// contact_rules.cuh -- BVH traversal and the contact pair rules.
//
// Pair acceptance restates crates/ppf-cts-solver/src/cpp/contact/contact.cu:
//   point-point  432-626  (index < query, multiplicity `count` over the
//                          incident edges / faces whose interior test does not
//                          already cover the pair, friction off when a
//                          neighbor element contains the query vertex)
//   point-edge   627-731  (interior closest point, face-neighbor count)
//   point-face   733-808  (interior closest point)
//   edge-edge    810-887  (edge < query edge, no shared vertex, interior)
// and the traversal of contact/aabb.hpp:78-107, restated stackless (escape
// links) with warp-synchronous leaf tests; a bounded walk latches
// STATUS_BVH_STACK_OVERFLOW instead of asserting.
#pragma once

#include <utility>

#include "../physics/contact_local.cuh"
#include "../physics/distance.cuh"
#include "lbvh.cuh"
#include "scene.cuh"

namespace ppf {
namespace gpu {

__device__ __forceinline__ bool box_overlap(const float4 &amin, const float4 &amax,
                                            const float4 &bmin, const float4 &bmax) {
    if (amin.w == 0.0f || bmin.w == 0.0f) return false;
    return (amin.x <= bmax.x && amax.x >= bmin.x) && (amin.y <= bmax.y && amax.y >= bmin.y) &&
           (amin.z <= bmax.z && amax.z >= bmin.z);
}

// Stackless traversal with warp-synchronous leaf tests. Every lane of the
// warp calls this together (a lane without a query passes active = false).
// Each lane walks the tree depth-first through the traversal links (left
// child on a box hit, escape node otherwise: no stack, no local memory)
// until it reaches its next overlapping leaf; then every lane that holds a
// leaf runs op(prim) in the same pass, so the narrow-phase test, the heavy
// part, executes once for the warp instead of once per diverged lane. The
// rounds repeat until no lane finds a leaf. With an exclusion box (xmin,
// xmax), leaves that also overlap it are skipped: the previous piece of a
// split query reports those. A walk longer than the tree allows latches
// STATUS_BVH_STACK_OVERFLOW (a corrupted tree) and ends.
// An op may define `bool pre(unsigned prim) const`, a cheap test (an index
// order, say) that the walk applies to a leaf before handing it over, so a
// leaf the narrow phase would reject at once costs no round of the warp.
template <class T> struct HasPre {
    template <class U>
    static auto test(int) -> decltype(std::declval<const U &>().pre(0u), char());
    template <class> static long test(...);
    static constexpr bool value = sizeof(test<T>(0)) == sizeof(char);
};

//
// Leaf tests taken in warp rounds pay off where the narrow phase is heavy and
// diverges (the CCD sweeps). Where it is light, the rounds cost more than
// they save: each round lasts as long as the lane whose next leaf is
// farthest along its walk, so a warp walks up to the sum over rounds of the
// longest step instead of the longest walk. kImmediate keeps the stackless
// walk and tests each leaf on the spot, lane by lane.
enum class LeafTests { kWarpRounds, kImmediate };

template <LeafTests MODE = LeafTests::kWarpRounds, class Op>
__device__ void warp_query(const BvhView &b, bool active, const float4 &qmin,
                           const float4 &qmax, Op &op, unsigned *status,
                           const float4 *xmin = nullptr, const float4 *xmax = nullptr) {
    if constexpr (MODE == LeafTests::kImmediate) {
        unsigned cur = (active && b.n != 0u && qmin.w != 0.0f) ? b.root : kLinkEnd;
        const unsigned bound = 4u * b.n + 64u;
        unsigned steps = 0;
        while (cur != kLinkEnd) {
            const float4 lo = b.bmin[cur], hi = b.bmax[cur];
            const uint2 ln = b.link[cur];
            if (++steps > bound) {
                atomicOr(status, STATUS_BVH_STACK_OVERFLOW);
                break;
            }
            if (box_overlap(lo, hi, qmin, qmax)) {
                if (!(ln.x & kLinkLeaf)) {
                    cur = ln.x;
                    continue;
                }
                cur = ln.y;
                const unsigned prim = ln.x & ~kLinkLeaf;
                bool take = !xmin || !box_overlap(lo, hi, *xmin, *xmax);
                if constexpr (HasPre<Op>::value) take = take && op.pre(prim);
                if (take) op(prim);
            } else {
                cur = ln.y;
            }
        }
        return;
    }
    unsigned cur = (active && b.n != 0u && qmin.w != 0.0f) ? b.root : kLinkEnd;
    const unsigned bound = 4u * b.n + 64u;
    unsigned steps = 0;
    while (true) {
        unsigned cand = kLinkEnd;
        while (cur != kLinkEnd) {
            const float4 lo = b.bmin[cur], hi = b.bmax[cur];
            const uint2 ln = b.link[cur];
            if (++steps > bound) {
                atomicOr(status, STATUS_BVH_STACK_OVERFLOW);
                cur = kLinkEnd;
                break;
            }
            if (box_overlap(lo, hi, qmin, qmax)) {
                if (!(ln.x & kLinkLeaf)) {
                    cur = ln.x;
                    continue;
                }
                cur = ln.y;
                const unsigned prim = ln.x & ~kLinkLeaf;
                bool take = !xmin || !box_overlap(lo, hi, *xmin, *xmax);
                if constexpr (HasPre<Op>::value) take = take && op.pre(prim);
                if (take) {
                    cand = prim;
                    break;
                }
            } else {
                cur = ln.y;
            }
        }
        if (!__any_sync(0xffffffffu, cand != kLinkEnd)) break;
        if (cand != kLinkEnd) op(cand);
    }
}

// Warp-aggregated slot reservation: the lanes that reach this call together
// take consecutive slots with one atomic add on the counter. Returns
// kSentinel past the capacity (the counter still counts, so the host sees
// the size a list needs).
__device__ __forceinline__ unsigned push_slot(unsigned *ctr, unsigned cap) {
    const unsigned mask = __activemask();
    const unsigned lane = threadIdx.x & 31u;
    const unsigned leader = __ffs(mask) - 1u;
    unsigned base = 0u;
    if (lane == leader) base = atomicAdd(ctr, (unsigned)__popc(mask));
    base = __shfl_sync(mask, base, leader);
    const unsigned slot = base + (unsigned)__popc(mask & ((1u << lane) - 1u));
    return slot < cap ? slot : kSentinel;
}

// Work items of a grid-stride loop taken a warp at a time, so that all 32
// lanes stay together for warp_query: item = base + lane, valid when below
// the total; `base` is the same on every lane of the warp.
struct WarpItems {
    unsigned base, stride, lane;
    __device__ __forceinline__ WarpItems() {
        lane = threadIdx.x & 31u;
        base = ((blockIdx.x * blockDim.x + threadIdx.x) >> 5) * 32u;
        stride = ((gridDim.x * blockDim.x) >> 5) * 32u;
    }
};

__device__ __forceinline__ Vec3 X(const float *x, unsigned i) {
    return vec3(x[3 * i], x[3 * i + 1], x[3 * i + 2]);
}

__device__ __forceinline__ bool interior(const Vec2 &c) {
    return c.max_coeff() < 1.0f && c.min_coeff() > 0.0f;
}
__device__ __forceinline__ bool interior(const Vec3 &c) {
    return c.max_coeff() < 1.0f && c.min_coeff() > 0.0f;
}
__device__ __forceinline__ bool interior(const Vec4 &c) {
    return c.max_coeff() < 1.0f && c.min_coeff() > 0.0f;
}

// ---- point-face -----------------------------------------------------------
__device__ __forceinline__ bool accept_point_face(const Scene &s, const float *x,
                                                  unsigned v, unsigned fi,
                                                  Vec3 *coef = nullptr) {
    const unsigned *f = s.face + 3 * fi;
    bool either_dyn = s.vprop[v].fix_index == 0 || !s.fprop[fi].fixed;
    bool both_collider = s.vprop[v].collider && s.vprop[f[0]].collider;
    if (f[0] == v || f[1] == v || f[2] == v || !either_dyn || both_collider) return false;
    Vec3 p = X(x, v), t0 = X(x, f[0]), t1 = X(x, f[1]), t2 = X(x, f[2]);
    Vec3 c = dist::point_triangle_coeff(p, t0, t1, t2);
    if (!interior(c)) return false;
    Vec3 e = c[0] * (p - t0) + c[1] * (p - t1) + c[2] * (p - t2);
    const PpfVertexParam &vp = s.vparam[s.vprop[v].param_index];
    const PpfFaceParam &fp = s.fparam[s.fprop[fi].param_index];
    float offset = vp.offset + fp.offset;
    float ghat = 0.5f * (vp.ghat + fp.ghat);
    if (!(e.squared_norm() < sqr(ghat + offset))) return false;
    if (coef) *coef = c;
    return true;
}

// ---- point-edge: returns multiplicity (0 = rejected) -----------------------
__device__ __forceinline__ unsigned accept_point_edge(const Scene &s, const float *x,
                                                      unsigned v, unsigned ei,
                                                      bool *friction, Vec2 *coef) {
    const unsigned *e = s.edge + 2 * ei;
    bool either_dyn = s.vprop[v].fix_index == 0 || !s.eprop[ei].fixed;
    bool both_collider = s.vprop[v].collider && s.vprop[e[0]].collider;
    if (e[0] == v || e[1] == v || !either_dyn || both_collider) return 0u;
    Vec3 p = X(x, v), t0 = X(x, e[0]), t1 = X(x, e[1]);
    Vec2 c = dist::point_edge_coeff(p, t0, t1);
    if (!interior(c)) return 0u;
    Vec3 d = c[0] * (p - t0) + c[1] * (p - t1);
    const PpfVertexParam &vp = s.vparam[s.vprop[v].param_index];
    const PpfEdgeParam &ep = s.eparam[s.eprop[ei].param_index];
    float offset = vp.offset + ep.offset;
    float ghat = 0.5f * (vp.ghat + ep.ghat);
    if (!(d.squared_norm() < sqr(ghat + offset))) return 0u;
    unsigned count = 0u;
    bool fr = true;
    unsigned k0 = s.ef_off[ei], k1 = s.ef_off[ei + 1];
    if (k1 > k0) {
        for (unsigned k = k0; k < k1; ++k) {
            const unsigned *f = s.face + 3 * s.ef[k];
            if (f[0] == v || f[1] == v || f[2] == v) {
                ++count;
                fr = false;
            } else {
                Vec3 cf = dist::point_triangle_coeff(p, X(x, f[0]), X(x, f[1]), X(x, f[2]));
                if (interior(cf)) continue;
                ++count;
            }
        }
    } else {
        count = 1u;
    }
    if (friction) *friction = fr;
    if (coef) *coef = c;
    return count;
}

// ---- point-point (index < v): returns multiplicity ----------------------------
__device__ __forceinline__ unsigned accept_point_point(const Scene &s, const float *x,
                                                       unsigned v, unsigned w,
                                                       bool *friction) {
    bool either_dyn = s.vprop[v].fix_index == 0 || s.vprop[w].fix_index == 0;
    bool both_collider = s.vprop[v].collider && s.vprop[w].collider;
    if (!(w < v) || !either_dyn || both_collider) return 0u;
    Vec3 p = X(x, v), q = X(x, w);
    Vec3 e = p - q;
    const PpfVertexParam &a = s.vparam[s.vprop[v].param_index];
    const PpfVertexParam &b = s.vparam[s.vprop[w].param_index];
    float offset = a.offset + b.offset;
    float ghat = 0.5f * (a.ghat + b.ghat);
    if (!(e.squared_norm() < sqr(ghat + offset))) return 0u;
    unsigned count = 0u;
    bool fr = true;
    unsigned e0 = s.ve_off[w], e1 = s.ve_off[w + 1];
    if (e1 > e0) {
        for (unsigned k = e0; k < e1; ++k) {
            const unsigned *ed = s.edge + 2 * s.ve[k];
            if (ed[0] == v || ed[1] == v) {
                ++count;
                fr = false;
            } else {
                Vec2 c = dist::point_edge_coeff(p, X(x, ed[0]), X(x, ed[1]));
                if (interior(c)) continue;
                ++count;
            }
        }
        unsigned f0 = s.vf_off[w], f1 = s.vf_off[w + 1];
        for (unsigned k = f0; k < f1; ++k) {
            const unsigned *f = s.face + 3 * s.vf[k];
            if (f[0] == v || f[1] == v || f[2] == v) {
                ++count;
                fr = false;
            } else {
                Vec3 c = dist::point_triangle_coeff(p, X(x, f[0]), X(x, f[1]), X(x, f[2]));
                if (interior(c)) continue;
                ++count;
            }
        }
    } else {
        count = 1u;
    }
    if (friction) *friction = fr;
    return count;
}

// ---- edge-edge (ei < ej) ------------------------------------------------------
__device__ __forceinline__ bool accept_edge_edge(const Scene &s, const float *x,
                                                 unsigned ei, unsigned ej,
                                                 Vec4 *coef = nullptr) {
    const unsigned *a = s.edge + 2 * ei;
    const unsigned *b = s.edge + 2 * ej;
    bool either_dyn = !s.eprop[ei].fixed || !s.eprop[ej].fixed;
    bool both_collider = s.vprop[a[0]].collider && s.vprop[b[0]].collider;
    bool shared = a[0] == b[0] || a[0] == b[1] || a[1] == b[0] || a[1] == b[1];
    if (!(ei < ej) || shared || !either_dyn || both_collider) return false;
    Vec3 p0 = X(x, a[0]), p1 = X(x, a[1]), q0 = X(x, b[0]), q1 = X(x, b[1]);
    Vec4 c = dist::edge_edge_coeff(p0, p1, q0, q1);
    if (!interior(c)) return false;
    Vec3 y0 = c[0] * p0 + c[1] * p1;
    Vec3 y1 = c[2] * q0 + c[3] * q1;
    Vec3 e = y0 - y1;
    const PpfEdgeParam &pa = s.eparam[s.eprop[ei].param_index];
    const PpfEdgeParam &pb = s.eparam[s.eprop[ej].param_index];
    float offset = pa.offset + pb.offset;
    float ghat = 0.5f * (pa.ghat + pb.ghat);
    if (!(e.squared_norm() < sqr(ghat + offset))) return false;
    if (coef) *coef = c;
    return true;
}

// ---- long edges query in pieces --------------------------------------------
// An edge much longer than its neighbours (a collider's face diagonal) has a
// query box covering thousands of leaves, and the one thread walking it
// holds up the launch. Such an edge is queried as K pieces of at most
// `piece_len`, one work item each. Pieces cover the segment (consecutive
// pieces share their split point), so every leaf within the query margin of
// the edge overlaps some piece box. Split points are monotone in each axis,
// so the pieces a leaf box overlaps are consecutive: reporting a leaf only
// from the first of them (the exclusion box is the previous piece) reports
// it once.
constexpr unsigned kMaxPieces = 1024;

struct EdgePieces {
    const unsigned *off; // n + 1: exclusive scan of the piece counts (tree order)
    unsigned n;          // edges
};

__device__ __forceinline__ unsigned piece_count(float len, float piece_len) {
    if (!(piece_len > 0.0f) || !(len > piece_len)) return 1u;
    float k = ceilf(len / piece_len);
    return k >= (float)kMaxPieces ? kMaxPieces : (unsigned)k;
}

// Split point k of K along a -> b, with the end points exact.
__device__ __forceinline__ Vec3 piece_point(const Vec3 &a, const Vec3 &b, unsigned k,
                                            unsigned K) {
    if (k == 0u) return a;
    if (k >= K) return b;
    const float u = (float)k / (float)K;
    return vec3(a[0] + u * (b[0] - a[0]), a[1] + u * (b[1] - a[1]), a[2] + u * (b[2] - a[2]));
}

// Tree slot of work item `item`: the largest t with off[t] <= item.
__device__ __forceinline__ unsigned piece_slot(const EdgePieces &ep, unsigned item) {
    unsigned lo = 0, hi = ep.n;
    while (hi - lo > 1u) {
        unsigned mid = (lo + hi) >> 1;
        if (ep.off[mid] <= item) lo = mid;
        else hi = mid;
    }
    return lo;
}

__device__ __forceinline__ void seg_box(const Vec3 &p, const Vec3 &q, float m, float4 &lo,
                                        float4 &hi) {
    lo = make_float4(fminf(p[0], q[0]) - m, fminf(p[1], q[1]) - m, fminf(p[2], q[2]) - m, 1.0f);
    hi = make_float4(fmaxf(p[0], q[0]) + m, fmaxf(p[1], q[1]) + m, fmaxf(p[2], q[2]) + m, 0.0f);
}

// Slot of block (i, j), i <= j, in the fixed upper pattern, or kSentinel.
__device__ __forceinline__ unsigned fixed_slot(const Scene &s, unsigned i, unsigned j) {
    unsigned lo = s.fixed_off[i], hi = s.fixed_off[i + 1];
    while (lo < hi) {
        unsigned mid = (lo + hi) >> 1;
        unsigned c = s.fixed_col[mid];
        if (c == j) return mid;
        if (c < j) lo = mid + 1;
        else hi = mid;
    }
    return kSentinel;
}

// Block (i, j) of the fixed matrix (either triangle), zero when absent.
__device__ __forceinline__ Mat3 fixed_block(const Scene &s, const float *val,
                                            unsigned i, unsigned j) {
    bool tr = i > j;
    unsigned a = tr ? j : i, b = tr ? i : j;
    unsigned slot = fixed_slot(s, a, b);
    Mat3 m = Mat3::zero();
    if (slot != kSentinel) {
        m = load_mat3(val + 9 * (size_t)slot);
        if (tr) m = m.transpose();
    }
    return m;
}

} // namespace gpu
} // namespace ppf
