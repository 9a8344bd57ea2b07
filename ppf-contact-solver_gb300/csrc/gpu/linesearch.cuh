// linesearch.cuh -- feasible step fraction and post-step intersection check.
#pragma once

#include "assemble.cuh"

namespace ppf {
namespace gpu {

struct LineSearchArgs {
    const float *x0; // start of the sweep (target = previous iterate)
    const float *x1; // candidate iterate
    const float *curr; // start-of-step positions (strain limit rest reference)
    IterStatus *st;
    float max_t;
    float ccd_eps;
};

// Contact line search (crates/ppf-cts-solver/src/cpp/contact/contact.cu:
// 2472-2740): analytic colliders per vertex, point-face and point-point CCD
// per vertex, then edge-edge CCD per edge seeded with the vertex minimum.
// Results: st->toi_bits (min over every candidate, in units of the sweep),
// st->overlap, st->pin_infeasible.
void launch_contact_line_search(const Scene &s, const BvhView &fb, const BvhView &eb,
                                const BvhView &vb, const LineSearchArgs &a, float piece_len,
                                PieceBuffers &pb, cudaStream_t q);

// The analytic-collider part alone (sphere / floor crossings and infeasible
// pins), for scenes whose mesh contact is switched off -> st->toi_bits.
void launch_constraint_line_search(const Scene &s, const LineSearchArgs &a, cudaStream_t q);

// Strain-limit line search (strainlimiting.cu:247-305) -> st->sl_toi_bits.
void launch_strain_line_search(const Scene &s, const LineSearchArgs &a, cudaStream_t q);

// Intersection check of every edge (contact.cu:3056-3175): edge-triangle
// pierce against the face tree, and edge pairs nearer than their combined
// offset against the edge tree. Records go to `records` (at most
// PPF_MAX_INTERSECTION_RECORDS), the count to st->n_isect.
void launch_intersection_check(const Scene &s, const BvhView &fb, const BvhView &eb,
                               const float *x, PpfIntersectionRecord *records, IterStatus *st,
                               float piece_len, PieceBuffers &pb, cudaStream_t q);

} // namespace gpu
} // namespace ppf
