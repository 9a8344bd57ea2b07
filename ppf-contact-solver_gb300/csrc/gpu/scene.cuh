// scene.cuh -- device-resident scene, per-step state and kernel entry points.
//
// Layout in HBM (one scene):
//   positions         float[3n] (curr, prev, eval_x, target), AoS like the ABI
//   topology          face u32[3F], edge u32[2E], hinge u32[4H] (hinge kept in
//                     its DataSet order; kernels remap (h2, h1, h0, h3))
//   props / params    the ABI structs, copied verbatim
//   fixed Hessian     upper-triangle 3x3 BSR on the builder's pattern: row
//                     offsets u32[n+1], columns u32[B_u], values float[9 B_u]
//                     (column-major blocks), plus the transpose table
//                     (row, slot) per lower entry for the symmetric SpMV
//   contact Hessian   upper-triangle blocks outside the fixed pattern, deduped
//                     per Newton iteration through a hash table, laid out as a
//                     CSR (offsets, columns, values) and a transpose table
//   diag              float[9n] (inertia, air, pull blocks)
//   vectors           force, dx, PCG work vectors: float[3n] each
#pragma once

#include "../../../include/ppf_gb300.h"
#include "common.cuh"
#include "lbvh.cuh"

namespace ppf {
namespace gpu {

constexpr unsigned kSentinel = 0xFFFFFFFFu;

struct BvhView {
    const uint2 *node;
    const float4 *bmin;
    const float4 *bmax;
    unsigned root;
    unsigned n;
    const uint2 *link; // traversal links (Lbvh::link)
};

struct CsrView {
    const unsigned *offset;
    const unsigned *col;
    float *val; // 9 per block
    const unsigned *tr_offset;
    const uint2 *tr; // (row, block index)
};

// How each traversal kernel tests the leaves its walk reaches: 0 in warp
// rounds (the leaves the lanes found are tested together), 1 on the spot.
// Both give the same pairs and times of impact; the faster form depends on
// the scene (ppf_autotune times them).
struct Tuning {
    unsigned char detect_vertex = 0, detect_edge = 1, ccd_vertex = 0, ccd_mesh_vertex = 0,
                  ccd_edge = 0, isect = 0;
    // the PCG's team: 0 the whole grid, else one cluster of this many CTAs
    unsigned char pcg_cluster = 0;
};

// Everything a kernel needs to read the scene (device pointers, by value).
struct Scene {
    unsigned n, n_surf, nf, ne, nh;
    unsigned nr;       // rod edges: edges 0 .. nr-1
    unsigned nf_shell; // shell faces: faces 0 .. nf_shell-1 (then solids' boundary faces)
    unsigned nt;       // tets
    const unsigned *tet;          // 4 per tet
    const PpfTetProp *tprop;
    const PpfTetParam *tparam;
    const float *inv_rest3;       // 9 per tet, column-major
    const unsigned *tet_slot;     // 16 per tet
    const unsigned char *hinge_type; // bit 0: next to a solid's face (no bending)
    unsigned nstitch;
    const PpfStitch *stitch;
    const unsigned *stitch_slot;  // 36 per stitch
    Tuning tune;
    const unsigned *face;
    const unsigned *edge;
    const unsigned *hinge;
    const PpfVertexProp *vprop;
    const PpfEdgeProp *eprop;
    const PpfFaceProp *fprop;
    const PpfHingeProp *hprop;
    const PpfVertexParam *vparam;
    const PpfEdgeParam *eparam;
    const PpfFaceParam *fparam;
    const PpfHingeParam *hparam;
    const float *inv_rest; // 4 per face, column-major
    const unsigned *vf_off, *vf; // vertex -> faces
    const unsigned *ve_off, *ve; // vertex -> edges
    const unsigned *ef_off, *ef; // edge -> faces
    const unsigned *fixed_off, *fixed_col;
    const unsigned *fixed_tr_off;
    const uint2 *fixed_tr;
    const unsigned *fixed_diag; // slot of (i, i)
    const unsigned *face_slot;  // 9 per face
    const unsigned *hinge_slot; // 16 per hinge, remapped order
    const unsigned *edge_slot;  // 4 per rod edge
    const unsigned *bend_slot;  // 9 per vertex: rod-bend stencil (j, i, k), or sentinels
    const unsigned *dof_mask;   // 1 = Dirichlet vertex
    const PpfFixPair *fix;
    unsigned nfix;
    const PpfPullPair *pull;
    unsigned npull;
    const PpfSphere *sphere;
    unsigned nsphere;
    const PpfFloor *floor;
    unsigned nfloor;
    const float *margin_face, *margin_edge, *margin_vert;
    // collision-window activity (null when every element is active)
    const unsigned char *vert_active, *edge_active;
    // static collision mesh (Constraint::mesh) and its trees (built once)
    unsigned ncv, ncf, nce;
    const float *cm_x;
    const unsigned *cm_face, *cm_edge;
    const PpfVertexProp *cm_vprop;
    const PpfFaceProp *cm_fprop;
    const PpfEdgeProp *cm_eprop;
    const PpfVertexParam *cm_vparam;
    const PpfFaceParam *cm_fparam;
    const PpfEdgeParam *cm_eparam;
    BvhView cm_face_bvh, cm_edge_bvh;
};

struct StepParams {
    float dt, prev_dt;
    float time;
    float air_friction, air_density, isotropic_air_friction;
    float friction_eps, eiganalysis_eps, constraint_tol;
    float line_search_max_t, ccd_eps;
    float gravity[3], wind[3];
    int barrier, friction_mode;
    int inactive_momentum;
    float fix_xz;
    float stitch_length_factor;
};

// Per-iteration scalars reduced on the device and read by the host once per
// Newton iteration (one small D2H copy).
struct IterStatus {
    unsigned n_pf, n_pe, n_pp, n_ee;   // detected pairs (may exceed capacity)
    unsigned n_dyn_keys, n_dyn;        // dynamic blocks: candidates, unique
    unsigned status;                   // StatusBits
    unsigned pin_infeasible;           // smallest pinned vertex index or ~0
    unsigned overlap;                  // CCD "starts overlapping" flag
    unsigned overlap_v0, overlap_v1, overlap_kind;
    unsigned toi_bits;                 // min contact toi (float bits, >= 0)
    unsigned toi_vf_bits;              // min vertex/face toi (seed for e-e)
    unsigned sl_toi_bits;              // min strain-limit toi
    unsigned max_dx_bits;              // max |dx_i|
    unsigned n_contact;                // active contact + constraint count
    unsigned n_isect;                  // intersection records found
    unsigned pcg_iter;
    float pcg_resid;
    int pcg_state;                     // 0 converged, 1 truncated, 2 failed
    float pcg_err0;
    int pcg_break_cause;               // 0 none, 1 negative curvature, 2 r^T z <= 0,
                                       // 3 unresolvable curvature
    float pcg_break_val;
    unsigned factor_iter;              // iterations of the factored solve
    unsigned fallback;                 // 1: it fell back to block-Jacobi
    float rescale;                     // min(1, max_dx / |dx|_max) of the step
};

} // namespace gpu
} // namespace ppf
