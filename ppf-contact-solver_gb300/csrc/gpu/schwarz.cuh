// schwarz.cuh -- the aggregate additive-Schwarz preconditioner of the PCG,
// the reference's second preconditioner (ParamSet::precond == Schwarz,
// crates/ppf-cts-solver/src/cpp/schwarz/schwarz.hpp:38-86, schwarz.cu).
//
// Vertices are grouped into non-overlapping, matrix-connected aggregates of at
// most kmax members (schwarz.cu:551-645: greedy heavy-edge growth, seeds in
// order of decreasing incident coupling). Per solve, each aggregate's dense
// block A_loc of the operator (3 m x 3 m) is gathered, its diagonal floored,
// factored A_loc = L L^T, and G = L^{-1} stored as a packed lower triangle
// (schwarz.cu:161-313). The preconditioner is z_seg = G^T (G r_seg) per
// aggregate (schwarz.cu:315-374), SPD by construction (r . z = |G r|^2).
//
// Two levels (ParamSet::schwarz_levels >= 2, the reference's default; its
// multilevel additive Schwarz, schwarz.cu:1043-1603) add a coarse
// correction: the aggregates become coarse nodes, C sums a vertex residual
// into its aggregate's node (piecewise-constant restriction), the coarse
// operator is the Galerkin product C A C^T (3 x 3 blocks summed over member
// pairs), the coarse nodes are grouped into domains of at most kmax nodes
// by the same heavy-edge growth on the Galerkin block norms, and
//     z = S_0 r + w C^T S_1 C r,   w = 1,
// with S_1 the per-domain G^T G of the Galerkin blocks. Still SPD.
//
// Because the aggregates do not overlap, z on an aggregate depends only on r
// on the same aggregate: the PCG applies S_0 in its update phase, one warp
// per aggregate, with no grid barrier beyond block-Jacobi's two; the coarse
// term needs the whole restricted residual, so it runs after the second
// barrier, one warp per domain, and adds a third.
#pragma once

#include <vector>

#include "pcg.cuh"
#include "scene.cuh"

namespace ppf {
namespace gpu {

// members per aggregate (schwarz.cu:1611)
constexpr unsigned kSchwarzKmax = kSchwarzMaxMembers;

// The reference's deepest hierarchy has 8 levels (schwarz.cu:403); this
// library builds at most the fine level and one coarse level. Each deeper
// level would add a grid barrier per PCG iteration and prolong one domain
// over ever more vertices from one warp; a request above 2 gets 2.
constexpr unsigned kSchwarzMaxLevels = 2;
// additive coarse-correction weight (schwarz.cu:429, coarse_weight)
constexpr float kSchwarzCoarseWeight = 1.0f;

struct SchwarzLayout {
    DevBuf<unsigned> agg;      // n: aggregate of each vertex
    DevBuf<unsigned> loc;      // n: position of the vertex among its members
    DevBuf<unsigned> agg_off;  // n_agg + 1: member offsets
    DevBuf<unsigned> members;  // n: vertices grouped by aggregate (ascending)
    DevBuf<unsigned> ainv_off; // n_agg + 1: float offsets of the packed factors
    DevBuf<float> ainv;        // packed lower triangles of G = L^{-1}
    // coarse level: aggregates as nodes, grouped into domains
    DevBuf<unsigned> dom;         // n_agg: domain of each aggregate
    DevBuf<unsigned> dom_loc;     // n_agg: position of the aggregate in its domain
    DevBuf<unsigned> dom_off;     // n_dom + 1
    DevBuf<unsigned> dom_members; // n_agg: aggregates grouped by domain (ascending)
    DevBuf<unsigned> ainv1_off;   // n_dom + 1
    DevBuf<float> ainv1;          // packed factors of the Galerkin domain blocks
    DevBuf<float4> rc;            // n_agg: restricted residual
    unsigned n = 0, n_agg = 0, max_members = 0;
    unsigned levels = 1, levels_req = 0, n_dom = 0, max_dom_members = 0;
    bool ready = false;
    SchwarzView view() const {
        return SchwarzView{n_agg,           agg_off.data(),     members.data(),
                           ainv_off.data(), ainv.data(),        n_dom,
                           dom_off.data(),  dom_members.data(), ainv1_off.data(),
                           ainv1.data(),    const_cast<float4 *>(rc.data()),
                           kSchwarzCoarseWeight};
    }
};

// Host: heavy-edge aggregation of the graph given as a both-triangle CSR
// (off, col) with the Frobenius norm of each stored block as its weight
// (schwarz.cu:478-645). Writes agg (aggregate per vertex) and returns the
// number of aggregates.
unsigned schwarz_aggregate(unsigned n, const std::vector<unsigned> &off,
                           const std::vector<unsigned> &col, const std::vector<float> &wgt,
                           unsigned kmax, std::vector<unsigned> &agg);

// Host: the coarse level's domains. The Galerkin blocks sum_{i in g, j in h}
// A(i, j) of distinct aggregates g != h, accumulated in float32 over the
// rows in order and each row's entries in order (blk: 9 floats per entry,
// column-major), weighted by their Frobenius norms, are grouped by
// schwarz_aggregate. Writes dom (domain per aggregate) and returns the
// number of domains.
unsigned schwarz_coarsen(unsigned n, const std::vector<unsigned> &off,
                         const std::vector<unsigned> &col, const float *blk,
                         const std::vector<unsigned> &agg, unsigned n_agg, unsigned kmax,
                         std::vector<unsigned> &dom);

// Aggregates the current operator (its pattern and blocks are read back
// once), builds the coarse domains when `levels` >= 2, and sizes the layout;
// called on a scene's first Schwarz solve.
void schwarz_setup(const PcgOperator &A, SchwarzLayout &S, unsigned levels, cudaStream_t q);

// Factors every aggregate's block of the current operator and, with the
// coarse level, every domain's Galerkin block; a non-finite pivot latches
// STATUS_PRECOND_NONSPD.
void launch_schwarz_factor(const PcgOperator &A, SchwarzLayout &S, unsigned *d_status,
                           cudaStream_t q);

} // namespace gpu
} // namespace ppf
