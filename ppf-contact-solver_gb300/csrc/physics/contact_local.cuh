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

// ---- static collision mesh (contact/contact.cu:899-1152) --------------------
// The push model of the analytic colliders, against the triangles and edges
// of a mesh without degrees of freedom. `local` is the elastic-only block(s)
// of the fixed Hessian the stiffness is read from.

// A free vertex at p (start of step x_start) against the static triangle
// (t0, t1, t2) (contact.cu:899-962). Force and Hessian of the vertex.
PPF_HD unsigned mesh_vertex_face(const Vec3 &p, const Vec3 &x_start, float mass,
                                 const Mat3 &local, const Vec3 &t0w, const Vec3 &t1w,
                                 const Vec3 &t2w, float offset, float ghat, float mu,
                                 float friction_eps, Vec3 &f, Mat3 &H) {
    const Vec3 q = x_start - p;
    const Vec3 t0 = t0w - p, t1 = t1w - p, t2 = t2w - p;
    const Vec3 c = dist::point_triangle_coeff_unclassified(Vec3::zero(), t0, t1, t2);
    const Vec3 y = c[0] * t0 + c[1] * t1 + c[2] * t2;
    const Vec3 e = -y;
    if (!(e.squared_norm() < sqr(offset + ghat))) return 0u;
    const Vec3 normal = e.normalized();
    const Vec3 proj_x = y + (offset + ghat) * normal;
    const float gap_squared = sqr(e.norm() - offset);
    const float stiff_k = normal.dot(local * normal) + mass / gap_squared;
    f = stiff_k * push::gradient(-proj_x, normal, ghat);
    H = stiff_k * push::hessian(-proj_x, normal, ghat);
    Friction fr(f, -q, normal, mu, friction_eps);
    f += fr.gradient();
    H += fr.hessian();
    return 1u;
}

// A static vertex y against the free triangle with vertices at t (start of
// step s) (contact.cu:964-1057): local is the 9x9 elastic block of the
// triangle, mass the triangle vertices' masses. Writes the 3 force columns
// and the 9x9 Hessian over the triangle's vertices.
PPF_HD unsigned mesh_face_vertex(const Vec3 &y, const Vec3 (&t)[3], const Vec3 (&s)[3],
                                 const float (&mass)[3], const Mat9 &local, float offset,
                                 float ghat, float mu, float friction_eps, Mat<3, 3> &ff,
                                 Mat9 &HH) {
    const Vec3 t0 = t[0] - y, t1 = t[1] - y, t2 = t[2] - y;
    const Vec3 s0 = s[0] - y, s1 = s[1] - y, s2 = s[2] - y;
    const Vec3 c = dist::point_triangle_coeff_unclassified(Vec3::zero(), t0, t1, t2);
    const Vec3 p = c[0] * t0 + c[1] * t1 + c[2] * t2;
    const Vec3 q = c[0] * s0 + c[1] * s1 + c[2] * s2;
    const Vec3 &e = p;
    if (!(e.squared_norm() < sqr(offset + ghat))) return 0u;
    const Vec3 normal = e.normalized();
    const float gap_squared = sqr(e.norm() - offset);
    Mat9 lh = local;
    for (int i = 0; i < 3; ++i)
        for (int k = 0; k < 3; ++k) lh(3 * i + k, 3 * i + k) += mass[i] / gap_squared;
    Vec9 ne;
    for (int j = 0; j < 9; ++j) ne[j] = c[j / 3] * normal[j % 3];
    const float stiff_k = (lh * ne).dot(ne) / ne.squared_norm();
    const Vec3 proj_x = (offset + ghat) * normal;
    Vec3 f = stiff_k * push::gradient(p - proj_x, normal, ghat);
    Mat3 H = stiff_k * push::hessian(p - proj_x, normal, ghat);
    Friction fr(f, p - q, normal, mu, friction_eps);
    f += fr.gradient();
    H += fr.hessian();
    for (int i = 0; i < 3; ++i) ff.set_col(i, c[i] * f);
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) HH.template set_block<3, 3>(3 * i, 3 * j, (c[i] * c[j]) * H);
    return 1u;
}

// A free edge (p0, p1; start of step b0, b1) against the static edge (q0, q1)
// (contact.cu:1059-1152): local is the edge's 6x6 elastic block. Writes the
// 2 force columns and the 6x6 Hessian over the edge's vertices.
PPF_HD unsigned mesh_edge_edge(const Vec3 &p0, const Vec3 &p1, const Vec3 &b0, const Vec3 &b1,
                               const Vec3 &q0, const Vec3 &q1, float m0, float m1,
                               const Mat6 &local, float offset, float ghat, float mu,
                               float friction_eps, Mat<3, 2> &ff, Mat6 &HH) {
    const Vec4 c = dist::edge_edge_coeff(p0, p1, q0, q1);
    const Vec3 x = c[0] * p0 + c[1] * p1;
    const Vec3 y = c[2] * q0 + c[3] * q1;
    const Vec3 z = c[0] * b0 + c[1] * b1;
    const Vec3 e = x - y;
    if (!(e.squared_norm() < sqr(offset + ghat))) return 0u;
    const Vec3 normal = e.normalized();
    const Vec3 proj_x = (offset + ghat) * normal;
    Vec6 ne;
    for (int j = 0; j < 6; ++j) ne[j] = c[j / 3] * normal[j % 3];
    const float gap_squared = sqr(e.norm() - offset);
    Mat6 lh = local;
    for (int k = 0; k < 3; ++k) {
        lh(k, k) += m0 / gap_squared;
        lh(3 + k, 3 + k) += m1 / gap_squared;
    }
    const float stiff_k = (lh * ne).dot(ne) / ne.squared_norm();
    Vec3 f = stiff_k * push::gradient(e - proj_x, normal, ghat);
    Mat3 H = stiff_k * push::hessian(e - proj_x, normal, ghat);
    Friction fr(f, x - z, normal, mu, friction_eps);
    f += fr.gradient();
    H += fr.hessian();
    for (int i = 0; i < 2; ++i) ff.set_col(i, c[i] * f);
    for (int i = 0; i < 2; ++i)
        for (int j = 0; j < 2; ++j) HH.template set_block<3, 3>(3 * i, 3 * j, (c[i] * c[j]) * H);
    return 1u;
}

} // namespace contact
} // namespace ppf
