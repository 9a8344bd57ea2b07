// elastic.cuh -- the isotropic singular-value models of shells and solids.
//
// Restates:
//   ARAP, StVK (+ the volume term), stable Neo-Hookean diff tables over the
//     singular values                     energy/model/{arap,stvk,detsqr,snhk}.hpp
//   one-sided Jacobi SVD of a 3x3 matrix (five sweeps) and its rotation-variant
//     sign fix                            utility/utility.cu:60-183
//   deformation gradient, force conversion of a tet
//                                         utility/utility.cu:200-215, 284-291
//   force U diag(de/da) V^T and the tet Hessian assembled from the nine
//     projected eigenmodes                eigenanalysis/eigenanalysis.cu:82-180
//   shell (non-Baraff-Witkin) and tet element force / Hessian
//                                         energy/energy.cu:304-446
#pragma once

#include "bw.cuh"
#include "eig.cuh"
#include "strainlimit.cuh"

namespace ppf {
namespace elastic {

template <int N> struct Table {
    Vec<N> deda;
    Mat<N, N> d2;
};

// ---- models over the singular values a --------------------------------------

PPF_HD Table<2> arap(const Vec2 &a, float mu, float lmd) {
    Table<2> t;
    const float tr = (a[0] - 1.0f) + (a[1] - 1.0f);
    for (int i = 0; i < 2; ++i) t.deda[i] = 2.0f * mu * (a[i] - 1.0f) + lmd * tr;
    for (int j = 0; j < 2; ++j)
        for (int i = 0; i < 2; ++i) t.d2(i, j) = (i == j ? 2.0f * mu : 0.0f) + lmd;
    return t;
}
PPF_HD Table<3> arap(const Vec3 &a, float mu, float lmd) {
    Table<3> t;
    const float tr = (a[0] - 1.0f) + (a[1] - 1.0f) + (a[2] - 1.0f);
    for (int i = 0; i < 3; ++i) t.deda[i] = 2.0f * mu * (a[i] - 1.0f) + lmd * tr;
    for (int j = 0; j < 3; ++j)
        for (int i = 0; i < 3; ++i) t.d2(i, j) = (i == j ? 2.0f * mu : 0.0f) + lmd;
    return t;
}

// lmd/2 (prod a - 1)^2, the volume term of StVK
PPF_HD Table<2> det_sqr(const Vec2 &a, float lmd) {
    Table<2> t;
    const float J = a[0] * a[1];
    t.deda[0] = lmd * a[1] * (J - 1.0f);
    t.deda[1] = lmd * a[0] * (J - 1.0f);
    t.d2(0, 0) = lmd * sqr(a[1]);
    t.d2(1, 1) = lmd * sqr(a[0]);
    t.d2(0, 1) = lmd * (2.0f * a[0] * a[1] - 1.0f);
    t.d2(1, 0) = t.d2(0, 1);
    return t;
}
PPF_HD Table<3> det_sqr(const Vec3 &a, float lmd) {
    Table<3> t;
    const float J = a[0] * a[1] * a[2];
    t.deda[0] = lmd * a[1] * a[2] * (J - 1.0f);
    t.deda[1] = lmd * a[0] * a[2] * (J - 1.0f);
    t.deda[2] = lmd * a[0] * a[1] * (J - 1.0f);
    t.d2(0, 0) = lmd * sqr(a[1] * a[2]);
    t.d2(1, 1) = lmd * sqr(a[0] * a[2]);
    t.d2(2, 2) = lmd * sqr(a[0] * a[1]);
    t.d2(0, 1) = lmd * a[2] * (2.0f * J - 1.0f);
    t.d2(0, 2) = lmd * a[1] * (2.0f * J - 1.0f);
    t.d2(1, 2) = lmd * a[0] * (2.0f * J - 1.0f);
    t.d2(1, 0) = t.d2(0, 1);
    t.d2(2, 0) = t.d2(0, 2);
    t.d2(2, 1) = t.d2(1, 2);
    return t;
}

// mu/4 sum (a_i - 1)^4 + the volume term
template <int N> PPF_HD Table<N> stvk(const Vec<N> &a, float mu, float lmd) {
    Table<N> t = det_sqr(a, lmd);
    for (int i = 0; i < N; ++i) {
        const float s = a[i] - 1.0f;
        t.deda[i] = mu * (s * s * s) + t.deda[i];
    }
    for (int j = 0; j < N; ++j)
        for (int i = 0; i < N; ++i) {
            float h = 0.0f;
            if (i == j) {
                const float s = a[i] - 1.0f;
                h = 3.0f * s * s;
            }
            t.d2(i, j) = mu * h + t.d2(i, j);
        }
    return t;
}

PPF_HD Table<2> snhk(const Vec2 &S, float mu, float lmd) {
    Table<2> t;
    const float a = S[0], b = S[1];
    t.deda[0] = lmd * b * (a * b - 1.0f) + mu * (a - b);
    t.deda[1] = lmd * a * (a * b - 1.0f) + mu * (b - a);
    t.d2(0, 0) = lmd * b * b + mu;
    t.d2(1, 1) = lmd * a * a + mu;
    t.d2(0, 1) = 2.0f * lmd * a * b - lmd - mu;
    t.d2(1, 0) = t.d2(0, 1);
    return t;
}
PPF_HD Table<3> snhk(const Vec3 &S, float mu, float lmd) {
    Table<3> t;
    const float a = S[0], b = S[1], c = S[2];
    const float I3 = a * b * c;
    t.deda[0] = lmd * b * c * (I3 - 1.0f) + mu * (a - b * c);
    t.deda[1] = lmd * a * c * (I3 - 1.0f) + mu * (b - a * c);
    t.deda[2] = lmd * a * b * (I3 - 1.0f) + mu * (c - a * b);
    t.d2(0, 0) = lmd * b * b * c * c + mu;
    t.d2(1, 1) = lmd * a * a * c * c + mu;
    t.d2(2, 2) = lmd * a * a * b * b + mu;
    t.d2(0, 1) = lmd * I3 * c + lmd * c * (I3 - 1.0f) - mu * c;
    t.d2(0, 2) = lmd * I3 * b + lmd * b * (I3 - 1.0f) - mu * b;
    t.d2(1, 2) = lmd * I3 * a + lmd * a * (I3 - 1.0f) - mu * a;
    t.d2(1, 0) = t.d2(0, 1);
    t.d2(2, 0) = t.d2(0, 2);
    t.d2(2, 1) = t.d2(1, 2);
    return t;
}

// The table of model id `model` (PPF_MODEL_ARAP / STVK / SNHK); false for
// any other model.
template <int N>
PPF_HD bool table(int model, const Vec<N> &a, float mu, float lmd, Table<N> &t) {
    if (model == 0) t = arap(a, mu, lmd);
    else if (model == 1) t = stvk<N>(a, mu, lmd);
    else if (model == 3) t = snhk(a, mu, lmd);
    else return false;
    return true;
}

// ---- 3x3 SVD ----------------------------------------------------------------

struct Svd33 {
    Mat3 U;
    Vec3 S;
    Mat3 Vt;
};

// One-sided Jacobi SVD with five fixed sweeps over the column pairs (0,1),
// (0,2), (1,2): singular values ascending as column norms of the rotated F,
// U its normalized columns, V the accumulated rotations.
PPF_HD Svd33 svd3x3(const Mat3 &F) {
    float A[3][3], Vv[3][3];
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) {
            A[r][c] = F(r, c);
            Vv[r][c] = r == c ? 1.0f : 0.0f;
        }
    for (int sweep = 0; sweep < 5; ++sweep)
        for (int p = 0; p < 3; ++p)
            for (int q = p + 1; q < 3; ++q) {
                float a = 0.0f, b = 0.0f, g = 0.0f;
                for (int r = 0; r < 3; ++r) {
                    a += A[r][p] * A[r][p];
                    b += A[r][q] * A[r][q];
                    g += A[r][p] * A[r][q];
                }
                const float zeta = (b - a) / (2.0f * g);
                const float t = (g == 0.0f) ? 0.0f
                                            : (zeta >= 0.0f ? 1.0f : -1.0f) /
                                                  (fabsf(zeta) + sqrtf(1.0f + zeta * zeta));
                const float c = 1.0f / sqrtf(1.0f + t * t), s = c * t;
                for (int r = 0; r < 3; ++r) {
                    const float ap = A[r][p], aq = A[r][q];
                    A[r][p] = c * ap - s * aq;
                    A[r][q] = s * ap + c * aq;
                }
                for (int r = 0; r < 3; ++r) {
                    const float vp = Vv[r][p], vq = Vv[r][q];
                    Vv[r][p] = c * vp - s * vq;
                    Vv[r][q] = s * vp + c * vq;
                }
            }
    float sv[3], u[3][3];
    for (int c = 0; c < 3; ++c) {
        float n2 = 0.0f;
        for (int r = 0; r < 3; ++r) n2 += A[r][c] * A[r][c];
        const float n = sqrtf(n2);
        sv[c] = n;
        const float inv = n > 0.0f ? 1.0f / n : 0.0f;
        for (int r = 0; r < 3; ++r) u[r][c] = A[r][c] * inv;
    }
    int idx[3] = {0, 1, 2};
    for (int i = 0; i < 3; ++i)
        for (int j = i + 1; j < 3; ++j)
            if (sv[idx[j]] < sv[idx[i]]) {
                const int k = idx[i];
                idx[i] = idx[j];
                idx[j] = k;
            }
    Svd33 out;
    for (int c = 0; c < 3; ++c) {
        out.S[c] = sv[idx[c]];
        for (int r = 0; r < 3; ++r) {
            out.U(r, c) = u[r][idx[c]];
            out.Vt(c, r) = Vv[r][idx[c]];
        }
    }
    return out;
}

// The rotation-variant SVD: when exactly one of U, V^T is a reflection, the
// smallest singular value turns negative and that column of U (or row of
// V^T) flips, so both factors are rotations.
PPF_HD Svd33 svd3x3_rv(const Mat3 &F) {
    Svd33 s = svd3x3(F);
    const float du = det3(s.U), dv = det3(s.Vt);
    int k = 0;
    for (int i = 1; i < 3; ++i)
        if (s.S[i] < s.S[k]) k = i;
    if (du < 0.0f && dv > 0.0f) {
        for (int r = 0; r < 3; ++r) s.U(r, k) = -s.U(r, k);
        s.S[k] *= -1.0f;
    } else if (du > 0.0f && dv < 0.0f) {
        for (int c = 0; c < 3; ++c) s.Vt(k, c) = -s.Vt(k, c);
        s.S[k] *= -1.0f;
    }
    return s;
}

// ---- tets -------------------------------------------------------------------

PPF_HD Mat3 deformation_grad(const Vec3 &x0, const Vec3 &x1, const Vec3 &x2, const Vec3 &x3,
                             const Mat3 &inv_rest) {
    return mat3_cols(x1 - x0, x2 - x0, x3 - x0) * inv_rest;
}

// d(vec F)/dx of a tet contracts with the shape-gradient columns
// g_0 = -(r_0 + r_1 + r_2), g_k = r_{k-1} (r: rows of the inverse rest matrix).
PPF_HD Mat3x4 shape_gradients(const Mat3 &inv_rest) {
    Mat3x4 G;
    const Vec3 r0 = inv_rest.row(0).transpose(), r1 = inv_rest.row(1).transpose(),
               r2 = inv_rest.row(2).transpose();
    G.set_col(0, ((-r0) - r1) - r2);
    G.set_col(1, r0);
    G.set_col(2, r1);
    G.set_col(3, r2);
    return G;
}

PPF_HD Mat3x4 convert_force(const Mat3 &dedF, const Mat3 &inv_rest) {
    const Mat3x4 G = shape_gradients(inv_rest);
    Mat3x4 out;
    for (int d = 0; d < 3; ++d) {
        const Vec3 row = dedF.row(d).transpose();
        for (int a = 0; a < 4; ++a) out(d, a) = G.col(a).dot(row);
    }
    return out;
}

// U diag(de/da) V^T
PPF_HD Mat3 eigen_force(const Vec3 &deda, const Svd33 &s) {
    Mat3 D = Mat3::zero();
    for (int i = 0; i < 3; ++i) D(i, i) = deda[i];
    return (s.U * D) * s.Vt;
}

// Adds mass * sum_i lambda_i vec(P_i) vec(P_i)^T to `out`, with the nine
// eigenmodes of the singular-value energy (three twists, three flips, three
// scalings from the table's Hessian) clamped at zero and P_i = U Q_i V^T G.
PPF_HD void tet_hessian(const Table<3> &t, const Svd33 &s, float eps, const Mat3 &inv_rest,
                        float mass, Mat12 &out) {
    Vec3 ev;
    Mat3 evec;
    eig::symm3(t.d2, ev, evec);
    const float a = s.S[0], b = s.S[1], c = s.S[2];
    float lam[9];
    lam[0] = fmaxf(0.0f, (t.deda[0] + t.deda[1]) / (a + b));
    lam[1] = fmaxf(0.0f, (t.deda[0] + t.deda[2]) / (a + c));
    lam[2] = fmaxf(0.0f, (t.deda[1] + t.deda[2]) / (b + c));
    const int pi[3] = {0, 0, 1}, pj[3] = {1, 2, 2};
    for (int m = 0; m < 3; ++m) {
        const int i = pi[m], j = pj[m];
        const float den = s.S[i] - s.S[j];
        lam[3 + m] = fmaxf(0.0f, fabsf(den) > eps
                                     ? (t.deda[i] - t.deda[j]) / den
                                     : 0.5f * (t.d2(i, i) + t.d2(j, j)) -
                                           0.5f * (t.d2(i, j) + t.d2(j, i)));
    }
    for (int m = 0; m < 3; ++m) lam[6 + m] = fmaxf(0.0f, ev[m]);
    const Mat3x4 W = s.Vt * shape_gradients(inv_rest);
    const float is2 = 0.7071067811865475f;
    for (int m = 0; m < 9; ++m) {
        if (lam[m] == 0.0f) continue;
        float P[12]; // column-major 3 x 4
        if (m < 6) {
            const float s2 = m < 3 ? -1.0f : 1.0f;
            const int r = pi[m % 3], cc = pj[m % 3];
            for (int col = 0; col < 4; ++col)
                for (int k = 0; k < 3; ++k)
                    P[3 * col + k] =
                        is2 * (W(cc, col) * s.U(k, r) + s2 * W(r, col) * s.U(k, cc));
        } else {
            const Vec3 v = evec.col(m - 6);
            for (int col = 0; col < 4; ++col)
                for (int k = 0; k < 3; ++k)
                    P[3 * col + k] = v[0] * W(0, col) * s.U(k, 0) +
                                     v[1] * W(1, col) * s.U(k, 1) +
                                     v[2] * W(2, col) * s.U(k, 2);
        }
        const float sc = mass * lam[m];
        for (int r = 0; r < 12; ++r) {
            const float sr = sc * P[r];
            for (int q = 0; q < 12; ++q) out(r, q) += sr * P[q];
        }
    }
}

// Force (3 x 4) and projected Hessian of one tet; false for a model without
// a singular-value table.
PPF_HD bool tet(const Vec3 &x0, const Vec3 &x1, const Vec3 &x2, const Vec3 &x3,
                const Mat3 &inv_rest, int model, float mu, float lmd, float mass, float eps,
                Mat3x4 &dedx, Mat12 &H) {
    const Svd33 s = svd3x3_rv(deformation_grad(x0, x1, x2, x3, inv_rest));
    Table<3> t;
    if (!table<3>(model, s.S, mu, lmd, t)) return false;
    dedx = mass * convert_force(eigen_force(t.deda, s), inv_rest);
    H = Mat12::zero();
    tet_hessian(t, s, eps, inv_rest, mass, H);
    return true;
}

// ---- shells under the singular-value models -----------------------------------

// Force (3 x 3) and projected Hessian of a shell face under ARAP, StVK or
// SNHk (energy.cu:336-355); false for any other model.
PPF_HD bool shell(const Vec3 &x0, const Vec3 &x1, const Vec3 &x2, const Mat2 &inv_rest,
                  int model, float mu, float lmd, float mass, float eps, Mat3 &dedx, Mat9 &H) {
    const strain::Svd32 s = strain::svd(bw::deformation_grad(x0, x1, x2, inv_rest));
    Table<2> t;
    if (!table<2>(model, s.S, mu, lmd, t)) return false;
    const Mat3x2 dedF = strain::eigen_force(t.deda, s);
    const Mat6 d2 = strain::eigen_hessian(t.deda, t.d2, s, eps);
    dedx = mass * bw::convert_force(dedF, inv_rest);
    H = mass * bw::convert_hessian(d2, inv_rest);
    return true;
}

} // namespace elastic
} // namespace ppf
