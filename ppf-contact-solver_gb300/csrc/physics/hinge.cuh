// hinge.cuh -- discrete-shell dihedral bending of one hinge.
//
// Restates energy/model/dihedral_angle.hpp:15-374 and the hinge stiffness of
// energy/energy.cu:448-553:
//   remap (h2, h1, h0, h3), signed angle by atan2 (dihedral_angle.hpp:86-105),
//   exact angle gradient (dihedral_angle.hpp:19-43),
//   projected Hessian = F-part (six eigenpairs of the angle energy mapped by
//   the projected-edge Jacobian) + W-part (rank-4 term in the p-basis, PSD
//   projected by cyclic Jacobi), both as the reference assembles them
//   (Wu & Kim 2023, "An Eigenanalysis of Angle-Based Deformation Energies").
#pragma once

#include "eig.cuh"

namespace ppf {
namespace hinge {

PPF_HD float dihedral_angle(const Vec3 &v0, const Vec3 &v1, const Vec3 &v2,
                            const Vec3 &v3) {
    Vec3 n1 = cross(v1 - v0, v2 - v0);
    Vec3 n2 = cross(v2 - v3, v1 - v3);
    Vec3 e = v1 - v2;
    float en = e.norm();
    if (en <= 0.0f) return 0.0f;
    float s = cross(n2, n1).dot(e) / en;
    float c = n1.dot(n2);
    return atan2f(s, c);
}

PPF_HD Mat3x4 angle_gradient(const Vec3 &v2, const Vec3 &v0, const Vec3 &v1,
                             const Vec3 &v3) {
    Vec3 e0 = v1 - v0, e1 = v2 - v0, e2 = v3 - v0, e3 = v2 - v1, e4 = v3 - v1;
    Vec3 n1 = cross(e0, e1), n2 = cross(e2, e0);
    float n1s = n1.squared_norm(), n2s = n2.squared_norm();
    float e0n = e0.norm();
    Mat3x4 r;
    r.set_col(0, (-e0n / n1s) * n1);
    r.set_col(1, (-e0.dot(e3) / (e0n * n1s)) * n1 - (e0.dot(e4) / (e0n * n2s)) * n2);
    r.set_col(2, (e0.dot(e1) / (e0n * n1s)) * n1 + (e0.dot(e2) / (e0n * n2s)) * n2);
    r.set_col(3, (-e0n / n2s) * n2);
    return r;
}

// Force (3x4, columns in remapped order X0..X3) and projected 12x12 Hessian of
// E = 1/2 (theta - rest)^2 for the remapped hinge X = (h2, h1, h0, h3).
PPF_HD void force_hessian(const Vec3 &X0, const Vec3 &X1, const Vec3 &X2,
                          const Vec3 &X3, float rest_angle, Mat3x4 &force,
                          Mat12 &hess) {
    const float angle = dihedral_angle(X0, X1, X2, X3);
    force = (angle - rest_angle) * angle_gradient(X0, X1, X2, X3);
    hess = Mat12::zero();

    // paper stencil (P0, P1 = edge, P2, P3 = flaps) = (X2, X1, X0, X3)
    const Vec3 y1 = X1 - X2, y2 = X0 - X2, y3 = X3 - X2;
    const float ly1 = y1.norm();
    if (ly1 <= 1e-9f) return;
    const Vec3 t1 = y1 / ly1;
    const Mat3 sigma = Mat3::identity() - outer<3>(t1, t1);
    const Vec3 z0 = y2 - t1 * t1.dot(y2);
    const Vec3 z1 = y3 - t1 * t1.dot(y3);
    const float l0 = z0.norm(), l1 = z1.norm();
    const Vec3 bc = cross(z0, z1);
    const float lb = bc.norm();
    if (l0 <= 1e-9f || l1 <= 1e-9f || lb <= 1e-9f * l0 * l1) return;
    const Vec3 tb = bc / lb;
    const float sgeom = tb.dot(t1) >= 0.0f ? 1.0f : -1.0f;
    const float g = angle - rest_angle;

    Mat12 Hp = Mat12::zero();

    // ---- F-part
    const Vec3 e0p = cross(z0, tb), e1p = cross(z1, tb);
    const float w = -sgeom * g;
    const float gamma = (l1 * l1) / (l0 * l0);
    const float gm1 = gamma - 1.0f, gp1 = gamma + 1.0f;
    const float r = sqrtf(4.0f * w * w * (gm1 / gp1) * (gm1 / gp1) + 1.0f);
    const float Rm = sqrtf(fmaxf(0.0f, 2.0f * (2.0f * w * w + 1.0f - r)));
    const float Rp = sqrtf(fmaxf(0.0f, 2.0f * (2.0f * w * w + 1.0f + r)));
    const float Lh = 1.0f / (l0 * l0) + 1.0f / (l1 * l1);
    const float cc = 4.0f * w / gp1;
    const Mat3 eta2 = (-1.0f / ly1) * (t1.dot(y2) * sigma + outer<3>(t1, z0));
    const Mat3 eta3 = (-1.0f / ly1) * (t1.dot(y3) * sigma + outer<3>(t1, z1));
    const Mat3 e2T = eta2.transpose(), e3T = eta3.transpose();
    const Mat3 m0 = -e2T - sigma, m1 = -e3T - sigma;
    auto accF = [&](float lam, const Vec3 &qa, const Vec3 &qb) {
        if (lam <= 0.0f) return;
        const float n2 = qa.dot(qa) + qb.dot(qb);
        if (n2 <= 1e-20f) return;
        const Vec3 b0 = m0 * qa + m1 * qb;
        const Vec3 b1 = e2T * qa + e3T * qb;
        const Vec3 b2 = sigma * qa;
        const Vec3 b3 = sigma * qb;
        float p[12];
        for (int c = 0; c < 3; ++c) {
            p[c] = b0[c];
            p[3 + c] = b1[c];
            p[6 + c] = b2[c];
            p[9 + c] = b3[c];
        }
        const float s = lam / n2;
        for (int i = 0; i < 12; ++i)
            for (int j = 0; j < 12; ++j) Hp(i, j) += s * p[i] * p[j];
    };
    const float sr[4] = {-1.0f, -1.0f, 1.0f, 1.0f};
    const float RR[4] = {Rm, Rm, Rp, Rp};
    const float sR[4] = {-1.0f, 1.0f, -1.0f, 1.0f};
    for (int mm = 0; mm < 4; ++mm) {
        const float R = RR[mm];
        const float a = w * (gm1 * gm1 / gp1 + sr[mm] * gp1 * r + sR[mm] * gm1 * R);
        const float b = -0.5f * gamma * R * R + 2.0f * w * w -
                        sR[mm] * 0.5f * (gm1 + sr[mm] * gp1 * r) * R;
        const float d = 1.0f + sr[mm] * r + sR[mm] * R;
        accF(0.25f * Lh * d, a * z0 + b * e0p, cc * z1 + d * e1p);
    }
    const float cos_t = z0.dot(z1) / (l0 * l1);
    const float sin_t = lb / (l0 * l1);
    const float beta = (l1 / l0 - l0 / l1) * cos_t;
    const float alpha0 = 0.5f * (-beta + sqrtf(beta * beta + 4.0f));
    const float ginv = w / sin_t;
    accF(ginv * (cos_t / (l1 * l1) - alpha0 / (l0 * l1)), alpha0 * tb, tb);
    accF(ginv * (cos_t / (l1 * l1) + 1.0f / (alpha0 * l0 * l1)), tb, (-alpha0) * tb);

    // ---- W-part
    const Vec3 tau0 = z0 / l0, tau1 = z1 / l1;
    const Vec3 tau1p = cross(tau1, tb);
    const float a0 = t1.dot(y2) / (ly1 * l0);
    const float a1 = t1.dot(y3) / (ly1 * l1);
    const float c0 = 1.0f / l0, c1 = 1.0f / l1;
    const float k0 = -4.0f * tau0.dot(tau1p) / (ly1 * ly1);
    const float k1 = 2.0f * tau0.dot(tau1p) / ly1;
    const Vec3 s01 = tau0 + tau1, d01 = tau0 - tau1;
    float pc[4][12];
    for (int c = 0; c < 3; ++c) {
        pc[0][c] = s01[c];
        pc[0][3 + c] = -s01[c];
        pc[0][6 + c] = 0.0f;
        pc[0][9 + c] = 0.0f;
        pc[1][c] = d01[c];
        pc[1][3 + c] = -d01[c];
        pc[1][6 + c] = 0.0f;
        pc[1][9 + c] = 0.0f;
        pc[2][c] = (-a1 - a0 + c1 + c0) * t1[c];
        pc[2][3 + c] = (a1 + a0) * t1[c];
        pc[2][6 + c] = -c0 * t1[c];
        pc[2][9 + c] = -c1 * t1[c];
        pc[3][c] = (-a1 + a0 + c1 - c0) * t1[c];
        pc[3][3 + c] = (a1 - a0) * t1[c];
        pc[3][6 + c] = c0 * t1[c];
        pc[3][9 + c] = -c1 * t1[c];
    }
    float gg[4], g23 = 0.0f;
    for (int i = 0; i < 4; ++i) {
        float s = 0.0f;
        for (int m = 0; m < 12; ++m) s += pc[i][m] * pc[i][m];
        gg[i] = s;
    }
    for (int m = 0; m < 12; ++m) g23 += pc[2][m] * pc[3][m];
    const float det23 = gg[2] * gg[3] - g23 * g23;
    if (gg[0] > 1e-5f && gg[1] > 1e-5f && det23 > 1e-6f * gg[2] * gg[3]) {
        const float we = -g * sgeom;
        float E[4][4] = {{0.0f}};
        E[0][0] = we * (-k0 * gg[0]);
        E[1][1] = we * (k0 * gg[1]);
        E[0][2] = E[2][0] = we * (k1 * gg[2]);
        E[0][3] = E[3][0] = we * (k1 * g23);
        E[1][2] = E[2][1] = we * (k1 * g23);
        E[1][3] = E[3][1] = we * (k1 * gg[3]);
        float Li[4][4] = {{0.0f}};
        Li[0][0] = 1.0f / sqrtf(gg[0]);
        Li[1][1] = 1.0f / sqrtf(gg[1]);
        const float L22 = sqrtf(gg[2]);
        const float L32 = g23 / L22;
        const float L33 = sqrtf(fmaxf(1e-30f, gg[3] - L32 * L32));
        Li[2][2] = 1.0f / L22;
        Li[3][3] = 1.0f / L33;
        Li[3][2] = -L32 / (L22 * L33);
        float LiE[4][4];
        for (int i = 0; i < 4; ++i)
            for (int j = 0; j < 4; ++j) {
                float s = 0.0f;
                for (int k = 0; k < 4; ++k) s += Li[i][k] * E[k][j];
                LiE[i][j] = s;
            }
        Mat<4, 4> Ss;
        for (int i = 0; i < 4; ++i)
            for (int j = 0; j < 4; ++j) {
                float s = 0.0f;
                for (int k = 0; k < 4; ++k) s += LiE[i][k] * Li[j][k];
                Ss(i, j) = s;
            }
        eig::psd_project<4>(Ss, 0.0f);
        float LtS[4][4];
        for (int i = 0; i < 4; ++i)
            for (int j = 0; j < 4; ++j) {
                float s = 0.0f;
                for (int k = 0; k < 4; ++k) s += Li[k][i] * Ss(k, j);
                LtS[i][j] = s;
            }
        float Core[4][4];
        for (int i = 0; i < 4; ++i)
            for (int j = 0; j < 4; ++j) {
                float s = 0.0f;
                for (int k = 0; k < 4; ++k) s += LtS[i][k] * Li[k][j];
                Core[i][j] = s;
            }
        float PC[12][4];
        for (int m = 0; m < 12; ++m)
            for (int j = 0; j < 4; ++j) {
                float s = 0.0f;
                for (int i = 0; i < 4; ++i) s += pc[i][m] * Core[i][j];
                PC[m][j] = s;
            }
        for (int m = 0; m < 12; ++m)
            for (int n = 0; n < 12; ++n) {
                float s = 0.0f;
                for (int j = 0; j < 4; ++j) s += PC[m][j] * pc[j][n];
                Hp(m, n) += s;
            }
    }

    // paper order (P0..P3) -> remapped order (X0..X3): swap blocks 0 and 2
    const int perm[4] = {2, 1, 0, 3};
    for (int a = 0; a < 4; ++a)
        for (int b = 0; b < 4; ++b)
            for (int i = 0; i < 3; ++i)
                for (int j = 0; j < 3; ++j)
                    hess(3 * perm[a] + i, 3 * perm[b] + j) = Hp(3 * a + i, 3 * b + j);
}

// Hinge bending stiffness (energy/energy.cu:458-519): density-normalized,
// resolution-independent |e|^2 / (A1 + A2) coefficient times BEND_SCALE.
PPF_HD float stiffness(float bend, float bend_warp, float bend_weft,
                       float uv_edge_sin2, float length, float area,
                       float areal_density) {
    const float kBendScale = 1.28e-5f;
    float b = uv_edge_sin2 < 0.0f
                  ? bend
                  : bend + bend_warp * uv_edge_sin2 + bend_weft * (1.0f - uv_edge_sin2);
    return area > 1e-12f ? kBendScale * b * (length * length / area) * areal_density
                         : 0.0f;
}

} // namespace hinge
} // namespace ppf
