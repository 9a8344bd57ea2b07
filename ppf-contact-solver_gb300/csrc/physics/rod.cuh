// rod.cuh -- rod elements and the Rayleigh damping shared by every element.
//
// Restates:
//   stretch spring of one rod edge            energy/model/hook.hpp:21-37
//   bend angle gradient at a rod vertex       energy/model/dihedral_angle.hpp:397-425
//   bend force and projected Hessian          energy/model/dihedral_angle.hpp:451-541
//     (the closed-form angle-energy eigensystem of Wu & Kim 2023, "An
//     Eigenanalysis of Angle-Based Deformation Energies": four in-plane and
//     two out-of-plane eigenpairs, negative ones dropped)
//   bend stiffness of an interior rod vertex  energy/energy.cu:555-598
//   stretch strain-limit barrier and stiffness strainlimiting/strainlimiting.cu:100-190
//   stretch strain-limit line search          strainlimiting/strainlimiting.cu:192-245
//   stiffness-proportional damping            energy/energy.cu:90-181
//   stitch spring                             energy/energy.cu:796-884
#pragma once

#include "barrier.cuh"

namespace ppf {
namespace rod {

// Gradient (3 x 2: columns x0, x1) and Hessian (6 x 6) of
// weight * 1/2 (|x1 - x0| / l0 - 1)^2 with the compressive curvature
// clamped so the Hessian stays PSD.
PPF_HD void stretch(const Vec3 &x0, const Vec3 &x1, float l0, float weight, Mat3x2 &grad,
                    Mat6 &hess) {
    const Vec3 t = x1 - x0;
    const float l = t.norm();
    const Vec3 n = t / l;
    const Vec3 dedt = (l / l0 - 1.0f) * n;
    Vec6 g;
    for (int k = 0; k < 3; ++k) {
        g[k] = -n[k];
        g[3 + k] = n[k];
    }
    const float r = (l - l0) / l;
    const float c0 = fmaxf(0.0f, 1.0f - r) / l0;
    const float c1 = fmaxf(0.0f, r / l0);
    grad.set_col(0, -weight * dedt);
    grad.set_col(1, weight * dedt);
    for (int j = 0; j < 6; ++j)
        for (int i = 0; i < 6; ++i) {
            // (d t / d x)^T (d t / d x): +I on the diagonal blocks, -I off them
            const float s = (i % 3 != j % 3) ? 0.0f : ((i < 3) == (j < 3) ? c1 : -c1);
            hess(i, j) = weight * ((c0 * g[i]) * g[j] + s);
        }
}

// d theta / d (e0, e1) of the angle between e0 and e1; zero when they are
// (anti)parallel to within sin^2 < 1e-12.
PPF_HD Mat3x2 angle_gradient(const Vec3 &e0, const Vec3 &e1) {
    const Vec3 c = cross(e0, e1);
    const float cs = c.squared_norm();
    const float s0 = e0.dot(e0), s1 = e1.dot(e1);
    Mat3x2 G = Mat3x2::zero();
    if (cs <= 1e-12f * s0 * s1) return G;
    const Vec3 n = c / sqrtf(cs);
    G.set_col(0, cross(e0, n) / s0);
    G.set_col(1, (-cross(e1, n)) / s1);
    return G;
}

// Adds lam (J^T q)(J^T q)^T / |q|^2 for the 6-vector q = [qa; qb], mapped to
// the three vertices by J^T q = [qa; -qa - qb; qb]; skipped for lam <= 0.
PPF_HD void add_mode(float lam, const Vec3 &qa, const Vec3 &qb, Mat9 &hess) {
    if (lam <= 0.0f) return;
    const float n2 = qa.dot(qa) + qb.dot(qb);
    if (n2 <= 1e-20f) return;
    float p[9];
    for (int c = 0; c < 3; ++c) {
        p[c] = qa[c];
        p[3 + c] = -qa[c] - qb[c];
        p[6 + c] = qb[c];
    }
    const float s = lam / n2;
    for (int j = 0; j < 9; ++j)
        for (int i = 0; i < 9; ++i) hess(i, j) += s * p[i] * p[j];
}

// Force (3 x 3: columns x0, x1, x2) and PSD Hessian of
// 1/2 (theta - rest)^2 with theta the angle at x1 between x0 - x1 and
// x2 - x1. The caller scales both by the vertex's bend stiffness.
PPF_HD void bend(const Vec3 &x0, const Vec3 &x1, const Vec3 &x2, float rest, Mat3 &force,
                 Mat9 &hess) {
    const Vec3 e0 = x0 - x1, e1 = x2 - x1;
    const float theta = atan2f(cross(e0, e1).norm(), e0.dot(e1));
    const Mat3x2 G = angle_gradient(e0, e1);
    const float w = theta - rest;
    force.set_col(0, w * G.col(0));
    force.set_col(1, w * ((-G.col(0)) - G.col(1)));
    force.set_col(2, w * G.col(1));
    hess = Mat9::zero();
    const float l0 = e0.norm(), l1 = e1.norm();
    const Vec3 b = cross(e0, e1);
    const float lb = b.norm();
    if (lb <= 1e-9f * l0 * l1 || l0 <= 1e-9f || l1 <= 1e-9f) return;
    const Vec3 tb = b / lb;
    const Vec3 e0p = cross(e0, tb), e1p = cross(e1, tb);
    const float cos_t = e0.dot(e1) / (l0 * l1);
    const float sin_t = lb / (l0 * l1);
    const float gamma = (l1 * l1) / (l0 * l0);
    const float gm1 = gamma - 1.0f, gp1 = gamma + 1.0f;
    const float q = gm1 / gp1;
    const float r = sqrtf(4.0f * w * w * q * q + 1.0f);
    const float Rm = sqrtf(fmaxf(0.0f, 2.0f * (2.0f * w * w + 1.0f - r)));
    const float Rp = sqrtf(fmaxf(0.0f, 2.0f * (2.0f * w * w + 1.0f + r)));
    const float Lh = 1.0f / (l0 * l0) + 1.0f / (l1 * l1);
    const float cc = 4.0f * w / gp1;
    // in-plane pairs (sign of r, sign of R) = (-,-), (-,+), (+,-), (+,+); the
    // b component's R term carries the sign opposite to the paper's print
    for (int m = 0; m < 4; ++m) {
        const float sr = m < 2 ? -1.0f : 1.0f, sR = (m & 1) ? 1.0f : -1.0f;
        const float R = m < 2 ? Rm : Rp;
        const float a = w * (gm1 * gm1 / gp1 + sr * gp1 * r + sR * gm1 * R);
        const float bb = -0.5f * gamma * R * R + 2.0f * w * w -
                         sR * 0.5f * (gm1 + sr * gp1 * r) * R;
        const float d = 1.0f + sr * r + sR * R;
        add_mode(0.25f * Lh * d, a * e0 + bb * e0p, cc * e1 + d * e1p, hess);
    }
    // out-of-plane pairs
    const float beta = (l1 / l0 - l0 / l1) * cos_t;
    const float alpha0 = 0.5f * (-beta + sqrtf(beta * beta + 4.0f));
    const float ginv = w / sin_t;
    const float lam4 = ginv * (cos_t / (l1 * l1) - alpha0 / (l0 * l1));
    const float lam5 = ginv * (cos_t / (l1 * l1) + 1.0f / (alpha0 * l0 * l1));
    add_mode(lam4, alpha0 * tb, tb, hess);
    add_mode(lam5, tb, (-alpha0) * tb, hess);
}

// Bend stiffness of an interior rod vertex: bend * mass * (1 cm / l)^2 with
// l the Voronoi length, half the two incident rest lengths.
PPF_HD float bend_stiffness(float bend, float mass, float len0, float len1) {
    const float ref = 1e-2f;
    const float voronoi = 0.5f * (len0 + len1);
    return voronoi > 0.0f ? bend * mass * (ref * ref) / (voronoi * voronoi) : 0.0f;
}

// Strain-limit barrier of one stretched rod edge (g = |x1 - x0| / l0 - 1 > 0
// against `limit`): force (6) and PSD Hessian before the stiffness scale.
// Returns false when the edge is not stretched.
PPF_HD bool strain_barrier(const Vec3 &x0, const Vec3 &x1, float l0, float limit, int kind,
                           float &g, Vec6 &f, Mat6 &H) {
    const Vec3 d = x1 - x0;
    const float l = d.norm();
    g = l / l0 - 1.0f;
    if (!(g > 0.0f)) return false;
    const float y = limit - g;
    const float dEdg = -barrier::gradient(y, limit, 0.0f, kind);
    const float d2Edg2 = barrier::curvature(y, limit, 0.0f, kind);
    const Vec3 n = d / l;
    Vec6 J;
    for (int k = 0; k < 3; ++k) {
        J[k] = (-n[k]) / l0;
        J[3 + k] = n[k] / l0;
    }
    const float inv_ll0 = 1.0f / (l * l0);
    const float a = fmaxf(0.0f, d2Edg2), b = fmaxf(0.0f, dEdg);
    for (int j = 0; j < 6; ++j)
        for (int i = 0; i < 6; ++i) {
            const int r = i % 3, c = j % 3;
            const float P = (r == c ? 1.0f : 0.0f) - n[r] * n[c];
            const float hg = ((i < 3) == (j < 3)) ? inv_ll0 * P : (-inv_ll0) * P;
            H(i, j) = a * (J[i] * J[j]) + b * hg;
        }
    f = dEdg * J;
    return true;
}

// Barrier stiffness of a rod edge: w^T H_e w + m / (limit - g)^2 with w the
// edge's centered start-of-step positions and H_e its elastic blocks.
PPF_HD float strain_stiffness(const Vec3 &c0, const Vec3 &c1, const Mat6 &local, float mass,
                              float g, float limit) {
    const Vec3 center = 0.5f * c0 + 0.5f * c1;
    Vec6 w;
    const Vec3 r0 = c0 - center, r1 = c1 - center;
    for (int k = 0; k < 3; ++k) {
        w[k] = r0[k];
        w[3 + k] = r1[k];
    }
    const float d = limit - g;
    return w.dot(local * w) + mass / (d * d);
}

// Largest t in [0, max_t] with |d0 + t (d1 - d0)| / l0 - 1 below `limit`,
// by bisection to float resolution (d0, d1: the edge vector at the previous
// iterate and at the candidate).
PPF_HD float strain_line_search(const Vec3 &d0, const Vec3 &d1, float l0, float limit,
                                float max_t) {
    const Vec3 dd = d1 - d0;
    float t = max_t;
    if ((d0 + t * dd).norm() / l0 - 1.0f >= limit) {
        float upper = t, lower = 0.0f, window = upper - lower;
        while (true) {
            t = 0.5f * (upper + lower);
            if ((d0 + t * dd).norm() / l0 - 1.0f - limit < 0.0f) lower = t;
            else upper = t;
            const float nw = upper - lower;
            if (nw == window) break;
            window = nw;
        }
        t = lower;
    }
    return t;
}

} // namespace rod

namespace stitch {

// A stitch spring between the barycentric points sum w_a x_a (a < 3) and
// sum w_a x_a (a >= 3), taken about their centroid, stretched against rest
// length l0 with the length capped at l_cap (energy.cu:822-876): gradient
// (3 x 6, one column per index) and Hessian (18 x 18), before the stitch's
// stiffness scale.
PPF_HD void spring(const Vec3 (&x)[6], const float (&w)[6], float l0, float l_cap,
                   Mat<3, 6> &grad, Mat<18, 18> &hess) {
    const float s = 1.0f / 6.0f;
    Vec3 cog = s * x[0];
    for (int a = 1; a < 6; ++a) cog = cog + s * x[a];
    const Vec3 z0 = (w[0] * (x[0] - cog) + w[1] * (x[1] - cog)) + w[2] * (x[2] - cog);
    const Vec3 z1 = (w[3] * (x[3] - cog) + w[4] * (x[4] - cog)) + w[5] * (x[5] - cog);
    const Vec3 t = z0 - z1;
    const float l = fminf(l_cap, t.norm());
    const Vec3 n = t / l;
    float coef[6];
    for (int a = 0; a < 6; ++a) coef[a] = a < 3 ? w[a] : -w[a];
    const Vec3 dedt = (l / l0 - 1.0f) * n;
    float g[18];
    for (int a = 0; a < 6; ++a)
        for (int k = 0; k < 3; ++k) g[3 * a + k] = coef[a] * n[k];
    const float r = (l - l0) / l;
    const float c0 = fmaxf(0.0f, 1.0f - r) / l0;
    const float c1 = fmaxf(0.0f, r / l0);
    for (int a = 0; a < 6; ++a) grad.set_col(a, coef[a] * dedt);
    for (int j = 0; j < 18; ++j)
        for (int i = 0; i < 18; ++i) {
            const float jj = (i % 3 == j % 3) ? (c1 * coef[i / 3]) * coef[j / 3] : 0.0f;
            hess(i, j) = (c0 * g[i]) * g[j] + jj;
        }
}

} // namespace stitch

namespace damping {

// Stiffness-proportional damping of one element of N vertices with elastic
// Hessian K and displacement u = x - x_start over the step: the gradient
// gains (beta / dt) K u and the Hessian becomes (1 + beta / dt) K.
template <int N>
PPF_HD void stiffness(float beta, float dt, const Vec<3 * N> &u, Mat<3, N> &dedx,
                      Mat<3 * N, 3 * N> &H) {
    if (beta <= 0.0f || dt <= 0.0f) return;
    const float s = beta / dt;
    for (int a = 0; a < N; ++a) {
        float f0 = 0.0f, f1 = 0.0f, f2 = 0.0f;
        for (int b = 0; b < 3 * N; ++b) {
            f0 += H(3 * a, b) * u[b];
            f1 += H(3 * a + 1, b) * u[b];
            f2 += H(3 * a + 2, b) * u[b];
        }
        dedx(0, a) += s * f0;
        dedx(1, a) += s * f1;
        dedx(2, a) += s * f2;
    }
    H *= (1.0f + s);
}

// The same with the damping operator K_lag evaluated at the start-of-step
// positions (for the fast-varying bending Hessians): the gradient gains
// (beta / dt) K_lag u and the Hessian (beta / dt) K_lag.
template <int N>
PPF_HD void lagged(float beta, float dt, const Vec<3 * N> &u, const Mat<3 * N, 3 * N> &K_lag,
                   Mat<3, N> &dedx, Mat<3 * N, 3 * N> &H) {
    if (beta <= 0.0f || dt <= 0.0f) return;
    const float s = beta / dt;
    for (int a = 0; a < N; ++a) {
        float f0 = 0.0f, f1 = 0.0f, f2 = 0.0f;
        for (int b = 0; b < 3 * N; ++b) {
            f0 += K_lag(3 * a, b) * u[b];
            f1 += K_lag(3 * a + 1, b) * u[b];
            f2 += K_lag(3 * a + 2, b) * u[b];
        }
        dedx(0, a) += s * f0;
        dedx(1, a) += s * f1;
        dedx(2, a) += s * f2;
    }
    for (int c = 0; c < 3 * N; ++c)
        for (int r = 0; r < 3 * N; ++r) H(r, c) += s * K_lag(r, c);
}

} // namespace damping
} // namespace ppf
