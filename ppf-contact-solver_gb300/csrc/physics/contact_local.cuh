// contact_local.cuh -- per-pair and per-vertex contact terms.
//
// Restates:
//   friction coefficient combination          contact/contact.cu:64-74
//   pair force / Hessian with barrier stiffness, lagged friction, barycentric
//   extension                                 contact/contact.cu:262-354
//   analytic sphere / floor barrier + friction contact/contact.cu:1154-1381
//   edge-triangle pierce predicate            contact/intersect_core.hpp:33-82
#pragma once

#include "barrier.cuh"

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
            H_out.set_block<3, 3>(3 * i, 3 * j, count * ((w[i] * w[j]) * H));
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

// Sphere and floor barriers of one free vertex of positive mass; returns the
// number of active constraints and accumulates into f, H.
PPF_HD unsigned vertex_constraints(const Vec3 &x, const Vec3 &x_start, float mass,
                                   float vfriction, const Mat3 &local,
                                   const SphereC *spheres, unsigned ns,
                                   const FloorC *floors, unsigned nf,
                                   int friction_mode, float friction_eps,
                                   float constraint_tol, Vec3 &f, Mat3 &H) {
    unsigned nc = 0;
    const Vec3 dx = x - x_start;
    for (unsigned j = 0; j < ns; ++j) {
        const SphereC &sp = spheres[j];
        float ghat = sp.ghat;
        float mu = combine_friction(sp.friction, vfriction, friction_mode);
        bool bowl = sp.bowl, reverse = sp.reverse;
        float radius = sp.radius;
        Vec3 center = (bowl && x[1] > sp.center[1])
                          ? vec3(sp.center[0], x[1], sp.center[2])
                          : sp.center;
        float d2 = (x - center).squared_norm();
        if (sp.kinematic) {
            if (d2) {
                Vec3 normal = (x - center).normalized();
                float eff = reverse ? (radius - ghat) : (radius + ghat);
                Vec3 target = eff * normal;
                Vec3 o = x - center;
                if (bowl) reverse = true;
                float k = mass / (ghat * ghat);
                float r2 = eff * eff;
                float dist = sqrtf(d2);
                float depth = reverse ? (dist - sp.radius) : (sp.radius - dist);
                if (sp.thickness > 0.0f && depth > sp.thickness) continue;
                if (reverse && d2 > r2) {
                    ++nc;
                    f += k * push::gradient(o - target, -normal, ghat);
                    H += k * push::hessian(o - target, -normal, ghat);
                } else if (!reverse && d2 < r2) {
                    ++nc;
                    f += k * push::gradient(o - target, normal, ghat);
                    H += k * push::hessian(o - target, normal, ghat);
                }
            }
        } else {
            radius = reverse ? radius - ghat : radius + ghat;
            float r2 = radius * radius;
            bool hit = reverse ? d2 > r2 : d2 < r2;
            if (hit) {
                float dist = sqrtf(d2);
                float depth = reverse ? (dist - sp.radius) : (sp.radius - dist);
                if (sp.thickness > 0.0f && depth > sp.thickness) continue;
                ++nc;
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
            }
        }
    }
    for (unsigned j = 0; j < nf; ++j) {
        const FloorC &fl = floors[j];
        float ghat = fl.ghat;
        float mu = combine_friction(fl.friction, vfriction, friction_mode);
        const Vec3 &up = fl.up;
        Vec3 ground = fl.ground + ghat * up;
        Vec3 e = x - ground;
        if (e.dot(up) < 0.0f) {
            float depth = -e.dot(up);
            if (fl.thickness > 0.0f && depth > fl.thickness) continue;
            ++nc;
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
        }
    }
    return nc;
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

} // namespace contact
} // namespace ppf
