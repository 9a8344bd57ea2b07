// distance.cuh -- closest-point barycentric coefficients.
//
// Restates crates/ppf-cts-solver/src/cpp/contact/distance.hpp:
//   point_edge_coeff               distance.hpp:15-26
//   point_triangle_coeff           distance.hpp:48-84 (cross-product form,
//                                  longest-edge fallback for zero area)
//   edge_edge_coeff                distance.hpp:114-222 (five candidates,
//                                  first of equal distances wins)
//   point_triangle_coeff_unclassified  distance.hpp:224-284
//   point_edge_coeff_unclassified  distance.hpp:286-300
// The pair-acceptance tests (interior iff every coefficient is strictly in
// (0, 1)) read these exact values, so they are evaluated in the same order.
#pragma once

#include "linalg.cuh"

namespace ppf {
namespace dist {

PPF_HD float clamp_unit(float v) { return v > 0.0f ? (v < 1.0f ? v : 1.0f) : 0.0f; }

PPF_HD Vec2 point_edge_coeff(const Vec3 &p, const Vec3 &e0, const Vec3 &e1) {
    Vec3 r = e1 - e0;
    float d = r.dot(r);
    if (d > 0.0f) {
        float t = r.dot(p - e0) / d;
        return vec2(1.0f - t, t);
    }
    return vec2(0.5f, 0.5f);
}

PPF_HD Vec3 point_triangle_coeff(const Vec3 &p, const Vec3 &t0, const Vec3 &t1,
                                 const Vec3 &t2) {
    Vec3 r0 = t1 - t0;
    Vec3 r1 = t2 - t0;
    Vec3 d = p - t0;
    Vec3 n = cross(r0, r1);
    float nn = n.dot(n);
    if (nn > 0.0f) {
        float inv = 1.0f / nn;
        float u = cross(d, r1).dot(n) * inv;
        float v = cross(r0, d).dot(n) * inv;
        return vec3(1.0f - u - v, u, v);
    }
    // collinear: project onto the longest side
    Vec3 s1 = t2 - t1;
    Vec3 s2 = t0 - t2;
    float l0 = r0.dot(r0), l1 = s1.dot(s1), l2 = s2.dot(s2);
    if (l0 >= l1 && l0 >= l2) {
        Vec2 w = point_edge_coeff(p, t0, t1);
        return vec3(w[0], w[1], 0.0f);
    } else if (l1 >= l2) {
        Vec2 w = point_edge_coeff(p, t1, t2);
        return vec3(0.0f, w[0], w[1]);
    } else {
        Vec2 w = point_edge_coeff(p, t2, t0);
        return vec3(w[1], 0.0f, w[0]);
    }
}

PPF_HD Vec4 edge_edge_coeff(const Vec3 &a0, const Vec3 &a1, const Vec3 &b0,
                            const Vec3 &b1) {
    Vec3 r0 = a1 - a0;
    Vec3 r1 = b1 - b0;
    Vec3 d = a0 - b0;
    float a = r0.dot(r0);
    float e = r1.dot(r1);
    float b = r0.dot(r1);
    float c = r0.dot(d);
    float f = r1.dot(d);
    float inv_a = a > 0.0f ? 1.0f / a : 0.0f;
    float inv_e = e > 0.0f ? 1.0f / e : 0.0f;
    Vec3 n = cross(r0, r1);
    float nn = n.dot(n);
    float inv_nn = nn > 0.0f ? 1.0f / nn : 0.0f;
    float s_stat = clamp_unit(n.dot(cross(r1, d)) * inv_nn);
    float t_stat = clamp_unit((b * s_stat + f) * inv_e);
    float t_a0 = clamp_unit(f * inv_e);
    float t_a1 = clamp_unit((f + b) * inv_e);
    float s_b0 = clamp_unit(-c * inv_a);
    float s_b1 = clamp_unit((b - c) * inv_a);
    const float cs[5] = {s_stat, 0.0f, 1.0f, s_b0, s_b1};
    const float ct[5] = {t_stat, t_a0, t_a1, 0.0f, 1.0f};
    float best_s = 0.0f, best_t = 0.0f, best = 3.402823466e+38f;
#pragma unroll
    for (int i = 0; i < 5; ++i) {
        Vec3 v = d + cs[i] * r0 - ct[i] * r1;
        float dd = v.dot(v);
        if (dd < best) {
            best = dd;
            best_s = cs[i];
            best_t = ct[i];
        }
    }
    return vec4(1.0f - best_s, best_s, 1.0f - best_t, best_t);
}

PPF_HD Vec3 point_triangle_coeff_unclassified(const Vec3 &p, const Vec3 &t0,
                                              const Vec3 &t1, const Vec3 &t2) {
    Vec3 r0 = t1 - t0;
    Vec3 r1 = t2 - t0;
    Vec3 d = p - t0;
    Vec3 cand[4];
    bool ok[4] = {false, true, true, true};
    cand[0] = point_triangle_coeff(p, t0, t1, t2);
    ok[0] = cand[0].min_coeff() >= 0.0f;
    float s01 = clamp_unit(point_edge_coeff(p, t0, t1)[1]);
    float s12 = clamp_unit(point_edge_coeff(p, t1, t2)[1]);
    float s20 = clamp_unit(point_edge_coeff(p, t2, t0)[1]);
    cand[1] = vec3(1.0f - s01, s01, 0.0f);
    cand[2] = vec3(0.0f, 1.0f - s12, s12);
    cand[3] = vec3(s20, 0.0f, 1.0f - s20);
    Vec3 best = cand[1];
    float best_d = 3.402823466e+38f;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        if (!ok[i]) continue;
        Vec3 v = d - cand[i][1] * r0 - cand[i][2] * r1;
        float dd = v.dot(v);
        if (dd < best_d) {
            best_d = dd;
            best = cand[i];
        }
    }
    return best;
}

PPF_HD Vec2 point_edge_coeff_unclassified(const Vec3 &p, const Vec3 &e0,
                                          const Vec3 &e1) {
    Vec2 c = point_edge_coeff(p, e0, e1);
    if (c[0] >= 0.0f && c[0] <= 1.0f) return c;
    return c[0] > 1.0f ? vec2(1.0f, 0.0f) : vec2(0.0f, 1.0f);
}

} // namespace dist
} // namespace ppf
