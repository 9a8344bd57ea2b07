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
// Because the aggregates do not overlap, z on an aggregate depends only on r
// on the same aggregate: the PCG applies it in its update phase, one warp per
// aggregate, with no grid barrier beyond block-Jacobi's two.
#pragma once

#include <vector>

#include "pcg.cuh"
#include "scene.cuh"

namespace ppf {
namespace gpu {

// members per aggregate (schwarz.cu:1611)
constexpr unsigned kSchwarzKmax = kSchwarzMaxMembers;

struct SchwarzLayout {
    DevBuf<unsigned> agg;      // n: aggregate of each vertex
    DevBuf<unsigned> loc;      // n: position of the vertex among its members
    DevBuf<unsigned> agg_off;  // n_agg + 1: member offsets
    DevBuf<unsigned> members;  // n: vertices grouped by aggregate (ascending)
    DevBuf<unsigned> ainv_off; // n_agg + 1: float offsets of the packed factors
    DevBuf<float> ainv;        // packed lower triangles of G = L^{-1}
    unsigned n = 0, n_agg = 0, max_members = 0;
    bool ready = false;
    SchwarzView view() const {
        return SchwarzView{n_agg, agg_off.data(), members.data(), ainv_off.data(),
                           ainv.data()};
    }
};

// Host: heavy-edge aggregation of the graph given as a both-triangle CSR
// (off, col) with the Frobenius norm of each stored block as its weight
// (schwarz.cu:478-645). Writes agg (aggregate per vertex) and returns the
// number of aggregates.
unsigned schwarz_aggregate(unsigned n, const std::vector<unsigned> &off,
                           const std::vector<unsigned> &col, const std::vector<float> &wgt,
                           unsigned kmax, std::vector<unsigned> &agg);

// Aggregates the current operator (its pattern and block norms are read back
// once) and sizes the layout; called on a scene's first Schwarz solve.
void schwarz_setup(const PcgOperator &A, SchwarzLayout &S, cudaStream_t q);

// Factors every aggregate's block of the current operator; a non-finite
// pivot latches STATUS_PRECOND_NONSPD.
void launch_schwarz_factor(const PcgOperator &A, SchwarzLayout &S, unsigned *d_status,
                           cudaStream_t q);

} // namespace gpu
} // namespace ppf
