// bw.cuh -- Baraff-Witkin shell membrane and the F -> x chain rule.
//
// Restates:
//   deformation gradient          utility/utility.cu:276-282
//   dE/dF -> dE/dx, d2E/dF2 -> x  utility/utility.cu:185-245
//   stretch / shear energy terms  energy/model/baraffwitkin.hpp:27-225
// The stretch and shear Hessians are the reference's PSD eigen-constructions,
// built from the same candidate vectors and the same tie-breaking, because the
// shear construction does not coincide with the nearest-PSD projection of the
// exact shear Hessian and parity with the reference requires its values.
// 6-vectors are laid out [column 0 of F; column 1 of F].
#pragma once

#include "linalg.cuh"

namespace ppf {
namespace bw {

PPF_HD Mat3x2 deformation_grad(const Vec3 &x0, const Vec3 &x1, const Vec3 &x2,
                               const Mat2 &inv_rest) {
    Mat3x2 dx = mat3x2_cols(x1 - x0, x2 - x0);
    return dx * inv_rest;
}

PPF_HD void shape_grads(const Mat2 &inv_rest, Vec2 g[3]) {
    Vec2 r0 = vec2(inv_rest(0, 0), inv_rest(0, 1));
    Vec2 r1 = vec2(inv_rest(1, 0), inv_rest(1, 1));
    g[0] = -r0 - r1;
    g[1] = r0;
    g[2] = r1;
}

PPF_HD Mat3 convert_force(const Mat3x2 &dedF, const Mat2 &inv_rest) {
    Vec2 g[3];
    shape_grads(inv_rest, g);
    Mat3 r;
    for (int d = 0; d < 3; ++d)
        for (int a = 0; a < 3; ++a)
            r(d, a) = g[a][0] * dedF(d, 0) + g[a][1] * dedF(d, 1);
    return r;
}

PPF_HD Mat9 convert_hessian(const Mat6 &h, const Mat2 &inv_rest) {
    Vec2 g[3];
    shape_grads(inv_rest, g);
    Mat9 r;
    for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b) {
            Mat3 blk = Mat3::zero();
            for (int d = 0; d < 2; ++d)
                for (int e = 0; e < 2; ++e)
                    blk += (g[a][d] * g[b][e]) * h.block<3, 3>(3 * d, 3 * e);
            r.set_block<3, 3>(3 * a, 3 * b, blk);
        }
    return r;
}

PPF_HD Mat3x2 stretch_gradient(const Mat3x2 &F, float mu) {
    Vec3 fu = F.col(0), fv = F.col(1);
    float nu = fu.norm(), nv = fv.norm();
    Mat3x2 r = mat3x2_cols((fu * (nu - 1.0f)) / nu, (fv * (nv - 1.0f)) / nv);
    return mu * r;
}

PPF_HD Mat3x2 shear_gradient(const Mat3x2 &F, float lmd) {
    float w = F.col(0).dot(F.col(1));
    return lmd * mat3x2_cols(w * F.col(1), w * F.col(0));
}

// Orthonormal frame {q1 = f/|f|, q2, q3} of one column and its PSD stretch
// block max(0,1) q1 q1^T + max(0, 1 - 1/|f|) (q2 q2^T + q3 q3^T), with q2
// the largest of three cross-product candidates (strict comparisons; ties
// fall to the third candidate).
PPF_HD Mat3 stretch_column_block(const Vec3 &f) {
    float nrm = f.norm();
    Vec3 q1 = f;
    Vec3 c1 = cross(vec3(f[2], 0.0f, -f[0]), q1);
    Vec3 c2 = cross(vec3(0.0f, f[2], -f[1]), q1);
    Vec3 c3 = cross(vec3(f[1], -f[0], 0.0f), q1);
    float n1 = c1.squared_norm(), n2 = c2.squared_norm(), n3 = c3.squared_norm();
    Vec3 q2 = (n1 > n2 && n1 > n3) ? c1 : ((n2 > n1 && n2 > n3) ? c2 : c3);
    Vec3 q3 = cross(q1, q2);
    q1.normalize();
    q2.normalize();
    q3.normalize();
    float l1 = 1.0f;
    float l2 = 1.0f - 1.0f / nrm;
    Mat3 H = Mat3::zero();
    H += outer<3>(fmaxf(0.0f, l1) * q1, q1);
    H += outer<3>(fmaxf(0.0f, l2) * q2, q2);
    H += outer<3>(fmaxf(0.0f, l2) * q3, q3);
    return H;
}

PPF_HD Mat6 stretch_hessian(const Mat3x2 &F, float mu) {
    Mat6 H = Mat6::zero();
    H.set_block<3, 3>(0, 0, stretch_column_block(F.col(0)));
    H.set_block<3, 3>(3, 3, stretch_column_block(F.col(1)));
    return mu * H;
}

PPF_HD Vec6 vec6(float a, float b, float c, float d, float e, float f) {
    Vec6 r;
    r[0] = a;
    r[1] = b;
    r[2] = c;
    r[3] = d;
    r[4] = e;
    r[5] = f;
    return r;
}

PPF_HD Vec6 pick_largest6(const Vec6 &a, const Vec6 &b, const Vec6 &c) {
    float na = a.squared_norm(), nb = b.squared_norm(), nc = c.squared_norm();
    if (na > nb && na > nc) return a;
    if (nb > na && nb > nc) return b;
    return c;
}

// Rows-first 2x2 (a, b; c, d) helpers.
PPF_HD float det_rows(float a, float b, float c, float d) { return a * d - b * c; }

PPF_HD Mat6 shear_hessian(const Mat3x2 &F, float lmd) {
    float I6 = F.col(0).dot(F.col(1));
    float I2 = F.squared_norm();
    Vec6 g, Hg;
    for (int k = 0; k < 3; ++k) {
        g[k] = F(k, 1);
        g[3 + k] = F(k, 0);
        Hg[k] = F(k, 0);
        Hg[3 + k] = F(k, 1);
    }
    float root = sqrtf(I2 * I2 + 12.0f * I6 * I6);
    float lmd0 = I2 + root;
    Vec6 q0 = 2.0f * I6 * Hg + lmd0 * g;
    Vec6 z, w1, w2, w3;
    float lmd1;
    if (I6 > 0) {
        z = q0;
        lmd1 = 2.0f * I6;
        w1 = vec6(1, 1, 0, 0, 0, 0);
        w2 = vec6(0, 0, 1, 1, 0, 0);
        w3 = vec6(0, 0, 0, 0, 1, 1);
    } else {
        lmd1 = -2.0f * I6;
        float tmp = I2 - root;
        z = 2.0f * I6 * Hg + tmp * g;
        w1 = vec6(1, -1, 0, 0, 0, 0);
        w2 = vec6(0, 0, 1, -1, 0, 0);
        w3 = vec6(0, 0, 0, 0, 1, -1);
    }
    float a1 = z.dot(w1), a2 = z.dot(w2), a3 = z.dot(w3);
    Vec6 q1 = pick_largest6(a3 * w1 + a3 * w2 - (a1 - a2) * w3,
                            a2 * w1 - (a1 - a3) * w2 + a2 * w3,
                            -(a2 - a3) * w1 + a1 * w2 + a1 * w3);
    float b1 = q1.dot(w1), b2 = q1.dot(w2), b3 = q1.dot(w3);
    // A1 = [a2 a3; b2 b3], A2 = [a3 a1; b3 b1], A3 = [a1 a2; b1 b2]
    float detA1 = det_rows(a2, a3, b2, b3);
    float detA2 = det_rows(a3, a1, b3, b1);
    float detA3 = det_rows(a1, a2, b1, b2);
    // adj(A) * rhs with adj([p q; r s]) = [s -q; -r p] and rhs = (-x, -y)
    auto adj_mul = [](float p, float q, float r, float s, float x, float y) {
        return vec2(s * x + (-q) * y, (-r) * x + p * y);
    };
    Vec2 c45 = adj_mul(a1, a2, b1, b2, -a3, -b3);
    Vec2 c56 = adj_mul(a2, a3, b2, b3, -a1, -b1);
    Vec2 c64 = adj_mul(a3, a1, b3, b1, -a2, -b2);
    Vec6 q2 = pick_largest6(c45[0] * w1 + c45[1] * w2 + detA3 * w3,
                            detA1 * w1 + c56[0] * w2 + c56[1] * w3,
                            c64[1] * w1 + detA2 * w2 + c64[0] * w3);
    q0.normalize();
    q1.normalize();
    q2.normalize();
    Mat6 r = Mat6::zero();
    r += fmaxf(0.0f, lmd0) * outer<6>(q0, q0);
    r += fmaxf(0.0f, lmd1) * outer<6>(q1, q1);
    r += fmaxf(0.0f, lmd1) * outer<6>(q2, q2);
    return (0.5f * lmd) * r;
}

// Membrane force (3x3, column a = vertex a) and 9x9 Hessian of one face,
// scaled by its mass (energy/energy.cu:304-364, BaraffWitkin branch).
PPF_HD void membrane(const Vec3 &x0, const Vec3 &x1, const Vec3 &x2,
                     const Mat2 &inv_rest, float mu, float lambda, float mass,
                     Mat3 &dedx, Mat9 &d2edx2) {
    Mat3x2 F = deformation_grad(x0, x1, x2, inv_rest);
    Mat3x2 dedF = stretch_gradient(F, mu) + shear_gradient(F, lambda);
    Mat6 d2edF2 = stretch_hessian(F, mu) + shear_hessian(F, lambda);
    dedx = mass * convert_force(dedF, inv_rest);
    d2edx2 = mass * convert_hessian(d2edF2, inv_rest);
}

} // namespace bw
} // namespace ppf
