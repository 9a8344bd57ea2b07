// contact_local.cuh -- per-pair and per-vertex contact terms.
//
// Restates:
//   friction coefficient combination          contact/contact.cu:64-74
//   pair force / Hessian with barrier stiffness, lagged friction, barycentric
//   extension                                 contact/contact.cu:262-354
//   analytic sphere / floor barrier + friction contact/contact.cu:1154-1381
//   edge-triangle pierce predicate            contact/intersect_core.hpp:33-82
//   edge-edge offset test of the check         contact/contact.cu:2774-2850
#pragma once

#include "barrier.cuh"
#include "distance.cuh"

namespace ppf {
namespace contact {

enum FrictionMode : int { FRICTION_MIN = 0, FRICTION_MAX = 1, FRICTION_MEAN = 2 };

PPF_HD float combine_friction(float a, float b, int mode) {
    if (mode == FRICTION_MAX) return fmaxf(a, b);
    if (mode == FRICTION_MEAN) return 0.5f * (a + b);
    return fminf(a, b);
}

// Force (3 x N, one column per vertex) and Hessian (3N x 3N) of one contact
// pair whose separation is ex = sum_i w_i x_i (weights sum to zero), already
// scaled by the pair's multiplicity `count`. `local` holds the elastic
// Hessian blocks of the pair's vertices (for the barrier stiffness); `x0` are
// the start-of-step positions (friction slip anchor).
template <int N>
PPF_HD void pair_force_hessian(const Vec3 (&x)[N], const Vec3 (&x0)[N],
                               const float (&w)[N], const float (&mass)[N],
                               const Mat<3 * N, 3 * N> &local, float ghat,
                               float offset, int barrier_kind, bool friction_on,
                               float mu, float friction_eps, float count,
                               Mat<3, N> &f_out, Mat<3 * N, 3 * N> &H_out) {
    Vec3 ex0 = Vec3::zero(), ex = Vec3::zero();
    const Vec3 a0 = x0[0], a = x[0];
#pragma unroll
    for (int i = 0; i < N; ++i) {
        ex0 += w[i] * (x0[i] - a0);
        ex += w[i] * (x[i] - a);
    }
    Vec3 dx = ex - ex0;
    Vec3 normal = ex.normalized();
    float k = barrier::stiffness<N>(w, mass, local, ex, offset);
    Vec3 f = k * barrier::edge_gradient(ex, ghat, offset, barrier_kind);
    Mat3 H = k * barrier::edge_hessian(ex, ghat, offset, barrier_kind);
    if (friction_on) {
        Friction fr(f, dx, normal, mu, friction_eps);
        f += fr.gradient();
        H += fr.hessian();
    }
#pragma unroll
    for (int i = 0; i < N; ++i) f_out.set_col(i, count * (w[i] * f));
#pragma unroll
    for (int i = 0; i < N; ++i)
#pragma unroll
        for (int j = 0; j < N; ++j)
            H_out.template set_block<3, 3>(3 * i, 3 * j, count * ((w[i] * w[j]) * H));
}

struct SphereC {
    Vec3 center;
    float ghat, friction, radius, thickness;
    bool bowl, reverse, kinematic;
};
struct FloorC {
    Vec3 ground;
    float ghat, friction, thickness;
    Vec3 up;
    bool kinematic;
};

// Barrier + friction of one analytic sphere on a free vertex of positive
// mass; returns 1 when active and accumulates into f, H.
PPF_HD unsigned sphere_constraint(const Vec3 &x, const Vec3 &x_start, float mass,
                                  float vfriction, const Mat3 &local,
                                  const SphereC &sp, int friction_mode,
                                  float friction_eps, Vec3 &f, Mat3 &H) {
    const Vec3 dx = x - x_start;
    float ghat = sp.ghat;
    float mu = combine_friction(sp.friction, vfriction, friction_mode);
    bool bowl = sp.bowl, reverse = sp.reverse;
    float radius = sp.radius;
    Vec3 center = (bowl && x[1] > sp.center[1]) ? vec3(sp.center[0], x[1], sp.center[2])
                                                : sp.center;
    float d2 = (x - center).squared_norm();
    if (sp.kinematic) {
        if (!d2) return 0u;
        Vec3 normal = (x - center).normalized();
        float eff = reverse ? (radius - ghat) : (radius + ghat);
        Vec3 target = eff * normal;
        Vec3 o = x - center;
        if (bowl) reverse = true;
        float k = mass / (ghat * ghat);
        float r2 = eff * eff;
        float dist = sqrtf(d2);
        float depth = reverse ? (dist - sp.radius) : (sp.radius - dist);
        if (sp.thickness > 0.0f && depth > sp.thickness) return 0u;
        if (reverse && d2 > r2) {
            f += k * push::gradient(o - target, -normal, ghat);
            H += k * push::hessian(o - target, -normal, ghat);
            return 1u;
        } else if (!reverse && d2 < r2) {
            f += k * push::gradient(o - target, normal, ghat);
            H += k * push::hessian(o - target, normal, ghat);
            return 1u;
        }
        return 0u;
    }
    radius = reverse ? radius - ghat : radius + ghat;
    float r2 = radius * radius;
    bool hit = reverse ? d2 > r2 : d2 < r2;
    if (!hit) return 0u;
    float dist = sqrtf(d2);
    float depth = reverse ? (dist - sp.radius) : (sp.radius - dist);
    if (sp.thickness > 0.0f && depth > sp.thickness) return 0u;
    Vec3 normal = (x - center).normalized();
    Vec3 projected = radius * normal;
    Vec3 o = x - center;
    if (reverse) normal = -normal;
    float gap = reverse ? sp.radius - sqrtf(d2) : sqrtf(d2) - sp.radius;
    float k = normal.dot(local * normal) + mass / (gap * gap);
    Vec3 fp = k * push::gradient(o - projected, normal, ghat);
    f += fp;
    H += k * push::hessian(o - projected, normal, ghat);
    Friction fr(fp, dx, normal, mu, friction_eps);
    f += fr.gradient();
    H += fr.hessian();
    return 1u;
}

// Barrier + friction of one analytic floor (half space) on a free vertex.
PPF_HD unsigned floor_constraint(const Vec3 &x, const Vec3 &x_start, float mass,
                                 float vfriction, const Mat3 &local, const FloorC &fl,
                                 int friction_mode, float friction_eps,
                                 float constraint_tol, Vec3 &f, Mat3 &H) {
    const Vec3 dx = x - x_start;
    float ghat = fl.ghat;
    float mu = combine_friction(fl.friction, vfriction, friction_mode);
    const Vec3 &up = fl.up;
    Vec3 ground = fl.ground + ghat * up;
    Vec3 e = x - ground;
    if (!(e.dot(up) < 0.0f)) return 0u;
    float depth = -e.dot(up);
    if (fl.thickness > 0.0f && depth > fl.thickness) return 0u;
    Vec3 projected = -e.dot(up) * up;
    float gap = (x - fl.ground).dot(up);
    if (fl.kinematic) gap = fmaxf(gap, constraint_tol * ghat);
    float k = up.dot(local * up) + mass / (gap * gap);
    Vec3 fp = k * push::gradient(-projected, up, ghat);
    f += fp;
    H += k * push::hessian(-projected, up, ghat);
    Friction fr(fp, dx, up, mu, friction_eps);
    f += fr.gradient();
    H += fr.hessian();
    return 1u;
}

// Segment (e0, e1) strictly crosses triangle (v0, v1, v2).
PPF_HD bool point_in_triangle(const Vec3 &p, const Vec3 &d1, const Vec3 &d2) {
    float a00 = d1.dot(d1), a01 = d1.dot(d2), a11 = d2.dot(d2);
    float b0 = d1.dot(p), b1 = d2.dot(p);
    float det = a00 * a11 - a01 * a01;
    if (det == 0.0f) return false;
    float w0 = (a11 * b0 - a01 * b1) / det;
    float w1 = (a00 * b1 - a01 * b0) / det;
    float w2 = 1.0f - w0 - w1;
    float wmin = fminf(fminf(w0, w1), w2);
    float wmax = fmaxf(fmaxf(w0, w1), w2);
    return wmin >= 0.0f && wmax <= 1.0f;
}

PPF_HD bool edge_triangle_intersect(const Vec3 &a0, const Vec3 &a1,
                                    const Vec3 &b0, const Vec3 &b1,
                                    const Vec3 &b2) {
    Vec3 d1 = b1 - b0, d2 = b2 - b0;
    Vec3 e0 = a0 - b0, e1 = a1 - b0;
    Vec3 n = cross(d1, d2);
    float s1 = e0.dot(n), s2 = e1.dot(n);
    if (s1 * s2 < 0.0f) {
        float t = s1 / (s1 - s2);
        Vec3 r = (1.0f - t) * e0 + t * e1;
        return point_in_triangle(r, d1, d2);
    }
    return false;
}

// Edge-edge part of the post-step intersection check
// (contact/contact.cu:2774-2850): two edges without a shared vertex whose
// closest points are nearer than their combined offset ...
PPF_HD bool edges_within_offset(const Vec3 &p0, const Vec3 &p1, const Vec3 &q0,
                                const Vec3 &q1, float offset) {
    Vec4 c = dist::edge_edge_coeff(p0, p1, q0, q1);
    Vec3 x0 = c[0] * p0 + c[1] * p1;
    Vec3 x1 = c[2] * q0 + c[3] * q1;
    Vec3 e = x0 - x1;
    return e.dot(e) < offset * offset;
}

// ... and for two edges sharing vertex s (free ends a, b), either free end
// nearer than the offset to the other edge.
PPF_HD bool shared_edges_within_offset(const Vec3 &s, const Vec3 &a, const Vec3 &b,
                                       float offset) {
    Vec2 c0 = dist::point_edge_coeff_unclassified(a, s, b);
    Vec2 c1 = dist::point_edge_coeff_unclassified(b, s, a);
    Vec3 e0 = (c0[0] * s + c0[1] * b) - a;
    Vec3 e1 = (c1[0] * s + c1[1] * a) - b;
    float d0 = e0.dot(e0), d1 = e1.dot(e1);
    return fminf(d0, d1) < offset * offset;
}

} // namespace contact
} // namespace ppf
