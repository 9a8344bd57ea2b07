// strainlimit.cuh -- singular-value strain-limit barrier of one shell face.
//
// Restates:
//   eigen-analysis force / projected Hessian   eigenanalysis/eigenanalysis.cu:11-74
//   per-face barrier force / Hessian           strainlimiting/strainlimiting.cu:46-98
//   stiffness from the elastic Hessian         strainlimiting/strainlimiting.cu:21-44
//   bisection line search on sigma_max - 1     strainlimiting/strainlimiting.cu:247-305
#pragma once

#include "barrier.cuh"
#include "bw.cuh"
#include "eig.cuh"

namespace ppf {
namespace strain {

// F = U diag(S) Vt (U 3x2, S ascending, Vt 2x2).
struct Svd32 {
    Mat3x2 U;
    Vec2 S;
    Mat2 Vt;
};

PPF_HD Svd32 svd(const Mat3x2 &F) {
    Svd32 r;
    Mat2 V;
    eig::svd3x2(F, r.U, r.S, V);
    r.Vt = V.transpose();
    return r;
}

PPF_HD Vec2 singular_values_minus_one(const Mat3x2 &F) {
    Svd32 s = svd(F);
    return vec2(s.S[0] - 1.0f, s.S[1] - 1.0f);
}

PPF_HD Mat3x2 eigen_force(const Vec2 &deda, const Svd32 &s) {
    Mat2 D = Mat2::zero();
    D(0, 0) = deda[0];
    D(1, 1) = deda[1];
    return (s.U * D) * s.Vt;
}

PPF_HD Mat3x2 rows3x2(float a, float b, float c, float d, float e, float f) {
    Mat3x2 m;
    m(0, 0) = a;
    m(0, 1) = b;
    m(1, 0) = c;
    m(1, 1) = d;
    m(2, 0) = e;
    m(2, 1) = f;
    return m;
}

PPF_HD Mat6 eigen_hessian(const Vec2 &deda, const Mat2 &d2, const Svd32 &s,
                          float eps) {
    Vec2 ev;
    Mat2 evec;
    eig::symm2(d2, ev, evec);
    const float is2 = 0.7071067811865475f;
    Mat3 U = mat3_cols(s.U.col(0), s.U.col(1), cross(s.U.col(0), s.U.col(1)));
    Mat3x2 Q[6];
    Q[0] = is2 * rows3x2(0.0f, 1.0f, -1.0f, 0.0f, 0.0f, 0.0f);
    Q[1] = is2 * rows3x2(0.0f, 1.0f, 1.0f, 0.0f, 0.0f, 0.0f);
    Q[2] = rows3x2(0.0f, 0.0f, 0.0f, 0.0f, 1.0f, 0.0f);
    Q[3] = rows3x2(0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 1.0f);
    Q[4] = Mat3x2::zero();
    Q[5] = Mat3x2::zero();
    for (int i = 0; i < 2; ++i) {
        Q[4](i, i) = evec(i, 0);
        Q[5](i, i) = evec(i, 1);
    }
    float a0 = s.S[0], a1 = s.S[1];
    float den = a0 - a1;
    float lam[6];
    lam[0] = fmaxf(0.0f, (deda[0] + deda[1]) / (a0 + a1));
    lam[1] = fmaxf(0.0f, fabsf(den) > eps
                             ? (deda[0] - deda[1]) / den
                             : 0.5f * (d2(0, 0) + d2(1, 1)) - 0.5f * (d2(0, 1) + d2(1, 0)));
    lam[2] = fmaxf(0.0f, deda[0] / a0);
    lam[3] = fmaxf(0.0f, deda[1] / a1);
    lam[4] = fmaxf(0.0f, ev[0]);
    lam[5] = fmaxf(0.0f, ev[1]);
    Mat6 r = Mat6::zero();
    for (int i = 0; i < 6; ++i) {
        if (lam[i]) {
            Mat3x2 t = (U * Q[i]) * s.Vt;
            Vec6 q;
            for (int k = 0; k < 6; ++k) q[k] = t.m[k];
            r += outer<6>(lam[i] * q, q);
        }
    }
    return r;
}

// Limit on sigma - 1 after the rest-shape shrink (strainlimiting.cu:62-63).
PPF_HD float effective_limit(float strainlimit, float shrink_x, float shrink_y) {
    float shrink_min = fminf(shrink_x, shrink_y);
    return (strainlimit + 1.0f) / shrink_min - 1.0f;
}

// Barrier stiffness: w^T H_e w + m / d^2 with w the face's centered
// start-of-step positions and d = limit - max(sigma - 1).
PPF_HD float stiffness(const Vec3 &c0, const Vec3 &c1, const Vec3 &c2,
                       const Mat9 &local, float mass, float sigma_max_shifted,
                       float limit) {
    const float s = 1.0f / 3.0f;
    Vec3 center = s * c0 + s * c1 + s * c2;
    Vec9 w;
    Vec3 r0 = c0 - center, r1 = c1 - center, r2 = c2 - center;
    for (int k = 0; k < 3; ++k) {
        w[k] = r0[k];
        w[3 + k] = r1[k];
        w[6 + k] = r2[k];
    }
    float d = limit - sigma_max_shifted;
    return w.dot(local * w) + mass / (d * d);
}

// Force / Hessian of the face barrier; returns false when inactive. The
// caller multiplies both by `stiffness`.
PPF_HD bool face_barrier(const Mat3x2 &F, const Mat2 &inv_rest, float strainlimit,
                         int barrier_kind, float eig_eps, Svd32 &sv, Mat3 &dedx,
                         Mat9 &d2edx2) {
    sv = svd(F);
    sv.S[0] -= 1.0f;
    sv.S[1] -= 1.0f;
    if (!(sv.S.max_coeff() > 0.0f)) return false;
    Vec2 deda;
    Mat2 d2;
    barrier::strainlimit_table(sv.S, strainlimit, barrier_kind, deda, d2);
    Svd32 s1 = sv;
    s1.S[0] += 1.0f;
    s1.S[1] += 1.0f;
    Mat3x2 dedF = eigen_force(deda, s1);
    Mat6 d2edF2 = eigen_hessian(deda, d2, s1, eig_eps);
    dedx = bw::convert_force(dedF, inv_rest);
    d2edx2 = bw::convert_hessian(d2edF2, inv_rest);
    return true;
}

// Largest t in [0, max_t] with sigma_max(F0 + t dF) - 1 below `limit`,
// located by bisection to float resolution (strainlimiting.cu:270-296).
PPF_HD float line_search(const Mat3x2 &F0, const Mat3x2 &F1, float limit,
                         float max_t) {
    Mat3x2 dF = F1 - F0;
    float t = max_t;
    if (singular_values_minus_one(F0 + t * dF).max_coeff() >= limit) {
        float upper = t, lower = 0.0f;
        float window = upper - lower;
        while (true) {
            t = 0.5f * (upper + lower);
            float diff = singular_values_minus_one(F0 + t * dF).max_coeff() - limit;
            if (diff < 0.0f) lower = t;
            else upper = t;
            float nw = upper - lower;
            if (nw == window) break;
            window = nw;
        }
        t = lower;
    }
    return t;
}

} // namespace strain
} // namespace ppf
