// barrier.cuh -- contact barrier potentials, friction, analytic pushes.
//
// Restates:
//   cubic / quadratic / log barrier       barrier/{cubic,quadratic,logarithm}.hpp
//   edge gradient / Hessian, stiffness    barrier/barrier.cu:49-113
//   strain-limit diff table               barrier/barrier.cu:116-131
//   regularized Coulomb friction          energy/model/friction.hpp:19-82
//   analytic push (sphere / floor)        energy/model/push.hpp:12-48
#pragma once

#include "linalg.cuh"

namespace ppf {
namespace barrier {

enum Kind : int { CUBIC = 0, QUAD = 1, LOG = 2 };

PPF_HD float energy(float g, float ghat, float offset, int kind) {
    g -= offset;
    if (kind == CUBIC) {
        float y = g - ghat;
        return y < 0.0f ? -2.0f * (y * y * y) / (3.0f * ghat) : 0.0f;
    } else if (kind == QUAD) {
        float y = ghat - g;
        return y > 0.0f ? y * y : 0.0f;
    } else {
        if (g <= 0.0f) return INFINITY;
        if (g >= ghat) return 0.0f;
        return -(g - ghat) * (g - ghat) * logf(g / ghat);
    }
}

PPF_HD float gradient(float g, float ghat, float offset, int kind) {
    g -= offset;
    if (kind == CUBIC) {
        float y = g - ghat;
        return y < 0.0f ? -2.0f * y * y / ghat : 0.0f;
    } else if (kind == QUAD) {
        float y = ghat - g;
        return y > 0.0f ? -2.0f * y : 0.0f;
    } else {
        if (g <= 0.0f) return -INFINITY;
        if (g >= ghat) return 0.0f;
        return (ghat - g) * (2.0f * g * logf(g / ghat) + g - ghat) / g;
    }
}

PPF_HD float curvature(float g, float ghat, float offset, int kind) {
    g -= offset;
    if (kind == CUBIC) {
        return g - ghat < 0.0f ? 4.0f * (1.0f - g / ghat) : 0.0f;
    } else if (kind == QUAD) {
        return ghat - g > 0.0f ? 2.0f : 0.0f;
    } else {
        if (g <= 0.0f) return INFINITY;
        if (g >= ghat) return 0.0f;
        return -2.0f * logf(g / ghat) + ghat * (ghat + 2.0f * g) / (g * g) - 3.0f;
    }
}

// Gradient of b(|e|) with respect to the separation e.
PPF_HD Vec3 edge_gradient(const Vec3 &e, float ghat, float offset, int kind) {
    float g = e.norm();
    Vec3 n = e / g;
    return n * gradient(g, ghat, offset, kind);
}

// Curvature-only Hessian c(|e|) e e^T / |e|^2.
PPF_HD Mat3 edge_hessian(const Vec3 &e, float ghat, float offset, int kind) {
    float c = curvature(e.norm(), ghat, offset, kind);
    float sq = e.squared_norm();
    Mat3 h;
#pragma unroll
    for (int j = 0; j < 3; ++j)
#pragma unroll
        for (int i = 0; i < 3; ++i) h(i, j) = (c * e[i]) * e[j] / sq;
    return h;
}

// Contact stiffness kappa = w^T (H_local + diag(m_i / g^2)) w, with
// w = normalize([c_0 e; ...; c_{N-1} e]). `local` holds the elastic blocks
// H(idx_i, idx_j) of the pair's vertices; zero masses (static vertices) take
// the largest mass of the pair (barrier.cu:49-86).
template <int N>
PPF_HD float stiffness(const float (&w)[N], const float (&mass)[N],
                       const Mat<3 * N, 3 * N> &local, const Vec3 &e,
                       float offset) {
    float g = e.norm() - offset;
    float gg = g * g;
    float m_max = 0.0f;
#pragma unroll
    for (int i = 0; i < N; ++i)
        if (mass[i] > m_max) m_max = mass[i];
    Mat<3 * N, 3 * N> h = local;
#pragma unroll
    for (int i = 0; i < N; ++i) {
        float mi = mass[i] > 0.0f ? mass[i] : m_max;
        float add = mi / gg;
#pragma unroll
        for (int k = 0; k < 3; ++k) h(3 * i + k, 3 * i + k) += add;
    }
    Vec<3 * N> v;
#pragma unroll
    for (int i = 0; i < N; ++i)
#pragma unroll
        for (int k = 0; k < 3; ++k) v[3 * i + k] = w[i] * e[k];
    v.normalize();
    return (h * v).dot(v);
}

// Strain-limit barrier table over the shifted singular values a_i = s_i - 1
// (barrier.cu:116-131): active where a_i > 0, on the gap ghat - a_i.
PPF_HD void strainlimit_table(const Vec2 &a, float ghat, int kind, Vec2 &deda,
                              Mat2 &d2ed2a) {
    deda = Vec2::zero();
    d2ed2a = Mat2::zero();
#pragma unroll
    for (int i = 0; i < 2; ++i) {
        float g = a[i];
        if (g > 0.0f) {
            float y = ghat - g;
            deda[i] = -gradient(y, ghat, 0.0f, kind);
            d2ed2a(i, i) = curvature(y, ghat, 0.0f, kind);
        }
    }
}

} // namespace barrier

// Regularized Coulomb friction with lagged normal force (friction.hpp).
struct Friction {
    Vec3 u;
    Vec3 n;
    Vec3 slip_dir;
    float lambda;
    bool kinetic;
    PPF_HD Friction(const Vec3 &force_contact, const Vec3 &dx, const Vec3 &normal,
                    float mu, float min_dx) {
        n = normal;
        float contact = -normal.dot(force_contact);
        u = dx - normal * normal.dot(dx);
        float un = sqrtf(u.squared_norm());
        kinetic = un > min_dx;
        slip_dir = kinetic ? u / un : Vec3::zero();
        lambda = mu > 0.0f ? mu * contact / fmaxf(min_dx, un) : 0.0f;
    }
    PPF_HD Vec3 gradient() const { return lambda * u; }
    PPF_HD Mat3 hessian() const {
        if (kinetic) {
            Vec3 w = cross(n, slip_dir);
            return lambda * outer<3>(w, w);
        }
        return lambda * (Mat3::identity() - outer<3>(n, n));
    }
};

namespace push {
PPF_HD Vec3 gradient(const Vec3 &e, const Vec3 &normal, float eps) {
    float d = e.dot(normal);
    if (d < 0.0f) return (-(d * d) / eps) * normal;
    return Vec3::zero();
}
PPF_HD Mat3 hessian(const Vec3 &e, const Vec3 &normal, float eps) {
    float d = e.dot(normal);
    float c = d < 0.0f ? -2.0f * d / eps : 0.0f;
    Mat3 h;
#pragma unroll
    for (int j = 0; j < 3; ++j)
#pragma unroll
        for (int i = 0; i < 3; ++i) h(i, j) = (c * normal[i]) * normal[j];
    return h;
}
} // namespace push

} // namespace ppf
