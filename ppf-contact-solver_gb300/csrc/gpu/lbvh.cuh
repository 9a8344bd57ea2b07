// lbvh.cuh -- linear BVH over faces, edges or surface vertices.
//
// Topology and numbering follow the reference (crates/ppf-cts-solver/src/cpp/
// lbvh/lbvh.cu:253-385): leaves 0..n-1 in Morton order hold (prim + 1, 0),
// internal node n + i holds (left + 1, right + 1), children are leaves when
// their key range is a single element. The root is internal node n (Karras's
// node 0 spans the whole key range); a single primitive is its own root.
// Bounding boxes are refit bottom-up in one pass with per-node arrival
// counters instead of the reference's per-level launches.
#pragma once

#include "common.cuh"
#include "radix_sort.cuh"

namespace ppf {
namespace gpu {

enum PrimKind : int { PRIM_VERTEX = 1, PRIM_EDGE = 2, PRIM_FACE = 3 };

constexpr unsigned kLinkLeaf = 0x80000000u;
constexpr unsigned kLinkEnd = 0xFFFFFFFFu;

struct Lbvh {
    unsigned n = 0;            // primitives
    unsigned root = 0;         // node index of the root
    DevBuf<uint2> node;        // 2n-1
    // 2n-1 traversal links: x = left child of an internal node, or the
    // primitive | kLinkLeaf for a leaf; y = escape node (the node a
    // depth-first walk visits after this node's subtree), kLinkEnd after the
    // last one
    DevBuf<uint2> link;
    DevBuf<unsigned> parent;   // 2n-1 (root is its own parent)
    DevBuf<float4> bmin;       // 2n-1, w = 1 if active else 0
    DevBuf<float4> bmax;       // 2n-1
    DevBuf<unsigned> visit;    // n-1 arrival counters
    DevBuf<unsigned> keys;     // sorted Morton codes
    DevBuf<unsigned> vals;     // sorted primitive indices
    DevBuf<unsigned> bounds;   // 6 ordered-int scene bounds
    unsigned nodes() const { return n == 0 ? 0 : 2 * n - 1; }
    void reserve(unsigned count);
    void release();
};

// Primitive description shared by build and refit. `prims` holds `kind`
// vertex indices per primitive (null for PRIM_VERTEX: prim i is vertex i);
// `margin` is 0.5 ghat + offset per primitive; `active` (may be null) clears a
// leaf's active flag for collision-window filtering.
struct PrimSet {
    PrimKind kind;
    unsigned count;
    const unsigned *prims;
    const float *margin;
    const unsigned char *active;
};

// Full rebuild: centroids of `x_tree` -> bounds -> Morton -> sort -> Karras
// -> leaf boxes of the sweep x0 -> x0 + extrapolate (x1 - x0) -> refit.
void lbvh_build(Lbvh &bvh, const PrimSet &ps, const float *x_tree,
                const float *x0, const float *x1, float extrapolate,
                RadixSortWorkspace &ws, unsigned *d_status, cudaStream_t s,
                bool refit = true);

// Box-only update on the existing topology (lbvh.cu:1032-1097).
void lbvh_refit(Lbvh &bvh, const PrimSet &ps, const float *x0, const float *x1,
                float extrapolate, unsigned *d_status, cudaStream_t s);
// Up to three trees (built over the same positions) refit in one launch.
void lbvh_refit_many(Lbvh *const *trees, const PrimSet *ps, unsigned count, const float *x0,
                     const float *x1, float extrapolate, unsigned *d_status, cudaStream_t s);

} // namespace gpu
} // namespace ppf
