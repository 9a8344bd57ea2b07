// eig.cuh -- small symmetric eigen-solvers, PSD projection, SVD, and the
// block-Jacobi inverse.
//
// Restates:
//   symmetric 2x2 / 3x3 closed forms   linalg/eigsolve.hpp:33-240 (max-abs
//                                      scaling, clamped Cardano acos,
//                                      ascending output)
//   PSD projection (cyclic Jacobi)     linalg/eigsolve.hpp:245-320
//   one-sided Jacobi SVD of 3x2        utility/utility.cu:60-150 (one sweep)
//   block-Jacobi 3x3 inverse           solver/solver.cu:357-400
#pragma once

#include "linalg.cuh"

namespace ppf {
namespace eig {

constexpr float kPi = 3.14159265358979323846f;

PPF_HD Vec2 rot90(const Vec2 &x) { return vec2(x[1], -x[0]); }

// Symmetric 2x2: eigenvalues ascending, eigenvectors as columns.
PPF_HD void symm2(const Mat2 &A, Vec2 &val, Mat2 &vec) {
    float scale = 0.0f;
#pragma unroll
    for (int i = 0; i < 4; ++i) scale = fmaxf(scale, fabsf(A.m[i]));
    if (scale <= 0.0f) {
        val = Vec2::zero();
        vec = Mat2::identity();
        return;
    }
    Mat2 B = A / scale;
    float tmp = B(0, 0) - B(1, 1);
    float D = 0.5f * sqrtf(tmp * tmp + 4.0f * B(0, 1) * B(0, 1));
    float mid = 0.5f * (B(0, 0) + B(1, 1));
    Vec2 lmd = vec2(mid - D, mid + D);
    Mat2 M = B;
    M(0, 0) -= lmd[0];
    M(1, 1) -= lmd[0];
    const float sqr_eps = 1e-7f * 1e-7f;
    Vec2 u = rot90(M.col(0));
    Vec2 v = rot90(M.col(1));
    Vec2 e0;
    if (u.squared_norm() > sqr_eps) e0 = u.normalized();
    else if (v.squared_norm() > sqr_eps) e0 = v.normalized();
    else e0 = rot90(vec2(0.0f, 1.0f));
    vec.set_col(0, e0);
    vec.set_col(1, rot90(e0));
    val = scale * lmd;
}

// Eigenvalues of a symmetric 3x3, DESCENDING (Cardano).
PPF_HD Vec3 eigvalues3(const Mat3 &A) {
    float p1 = A(0, 1) * A(0, 1) + A(0, 2) * A(0, 2) + A(1, 2) * A(1, 2);
    float q = A.trace() / 3.0f;
    float p2 = (A(0, 0) - q) * (A(0, 0) - q) + (A(1, 1) - q) * (A(1, 1) - q) +
               (A(2, 2) - q) * (A(2, 2) - q) + 2.0f * p1;
    float p = sqrtf(p2 / 6.0f);
    if (fabsf(p) < 1e-8f) return Vec3::zero();
    Mat3 B = A;
#pragma unroll
    for (int i = 0; i < 3; ++i) B(i, i) -= q;
    B = (1.0f / p) * B;
    float r = det3(B) / 2.0f;
    r = r < -1.0f ? -1.0f : (r > 1.0f ? 1.0f : r);
    float phi = acosf(r) / 3.0f;
    float e1 = q + 2.0f * p * cosf(phi);
    float e3 = q + 2.0f * p * cosf(phi + 2.0f * kPi / 3.0f);
    float e2 = 3.0f * q - e1 - e3;
    return vec3(e1, e2, e3);
}

PPF_HD Vec3 pick_largest(const Vec3 &a, const Vec3 &b, const Vec3 &c) {
    float an = a.squared_norm(), bn = b.squared_norm(), cn = c.squared_norm();
    if (an > bn) return an > cn ? a : c;
    return bn > cn ? b : c;
}

// Null-space directions of a (near-)singular symmetric 3x3: one vector when
// the null space is a line, two when it is a plane (second slot zero
// otherwise).
PPF_HD void null_dirs(const Mat3 &A, Vec3 &v1, Vec3 &v2) {
    const float eps = 1e-7f;
    Vec3 u = A.col(0), v = A.col(1), w = A.col(2);
    Vec3 q = pick_largest(cross(u, v), cross(v, w), cross(w, u));
    if (q.squared_norm() < eps) {
        Vec3 pp = pick_largest(u, v, w);
        Vec3 x = cross(pp, vec3(1.0f, 0.0f, 0.0f));
        if (x.squared_norm() < eps) x = cross(pp, vec3(0.0f, 1.0f, 0.0f));
        Vec3 y = cross(pp, x);
        v1 = x.normalized();
        v2 = y.normalized();
    } else {
        v1 = q.normalized();
        v2 = Vec3::zero();
    }
}

PPF_HD Mat3 eigvectors3(const Mat3 &A, const Vec3 &lmd) {
    Mat3 M = A;
#pragma unroll
    for (int i = 0; i < 3; ++i) M(i, i) -= lmd[0];
    Vec3 v1, v2;
    null_dirs(M, v1, v2);
    if (v2.squared_norm() == 0.0f) {
        Mat3 M1 = A;
#pragma unroll
        for (int i = 0; i < 3; ++i) M1(i, i) -= lmd[1];
        Vec3 t1, t2;
        null_dirs(M1, t1, t2);
        Vec3 g = t1 - v1.dot(t1) * v1;
        v2 = g.normalized();
    }
    Vec3 w = cross(v1, v2).normalized();
    v2 = cross(w, v1);
    if (v1.squared_norm() < 0.5f || w.squared_norm() < 0.5f) return Mat3::identity();
    return mat3_cols(v1, v2, w);
}

// Symmetric 3x3: eigenvalues ascending, eigenvectors as columns.
PPF_HD void symm3(const Mat3 &A, Vec3 &val, Mat3 &vec) {
    float scale = 0.0f;
#pragma unroll
    for (int i = 0; i < 9; ++i) scale = fmaxf(scale, fabsf(A.m[i]));
    if (scale <= 0.0f) {
        val = Vec3::zero();
        vec = Mat3::identity();
        return;
    }
    Mat3 B = (1.0f / scale) * A;
    Vec3 lmd = eigvalues3(B);
    Mat3 ev;
    if (lmd.squared_norm() > 0.0f) {
        ev = eigvectors3(B, lmd);
    } else {
        ev = Mat3::identity();
        float q = B.trace() / 3.0f;
        lmd = vec3(q, q, q);
    }
    val = vec3(scale * lmd[2], scale * lmd[1], scale * lmd[0]);
    vec = mat3_cols(ev.col(2), ev.col(1), ev.col(0));
}

// Nearest PSD matrix (eigenvalues clamped at `floor`) by cyclic Jacobi.
template <int N> PPF_HD void psd_project(Mat<N, N> &A, float floor) {
    Mat<N, N> V = Mat<N, N>::identity();
    float scale = 0.0f;
    for (int i = 0; i < N * N; ++i) scale = fmaxf(scale, fabsf(A.m[i]));
    if (scale == 0.0f) {
        if (floor > 0.0f)
            for (int i = 0; i < N; ++i) A(i, i) = floor;
        return;
    }
    const float tiny = 1e-7f * scale;
    for (int sweep = 0; sweep < 24; ++sweep) {
        float off = 0.0f;
        for (int p = 0; p < N; ++p)
            for (int q = p + 1; q < N; ++q) off = fmaxf(off, fabsf(A(p, q)));
        if (off <= tiny) break;
        for (int p = 0; p < N; ++p) {
            for (int q = p + 1; q < N; ++q) {
                const float apq = A(p, q);
                if (fabsf(apq) <= tiny) continue;
                const float app = A(p, p), aqq = A(q, q);
                const float tau = (aqq - app) / (2.0f * apq);
                const float t = (tau >= 0.0f ? 1.0f : -1.0f) /
                                (fabsf(tau) + sqrtf(1.0f + tau * tau));
                const float c = 1.0f / sqrtf(1.0f + t * t);
                const float s = t * c;
                A(p, p) = c * c * app - 2.0f * s * c * apq + s * s * aqq;
                A(q, q) = s * s * app + 2.0f * s * c * apq + c * c * aqq;
                A(p, q) = 0.0f;
                A(q, p) = 0.0f;
                for (int k = 0; k < N; ++k) {
                    if (k == p || k == q) continue;
                    const float akp = A(k, p), akq = A(k, q);
                    const float np = c * akp - s * akq;
                    const float nq = s * akp + c * akq;
                    A(k, p) = np;
                    A(p, k) = np;
                    A(k, q) = nq;
                    A(q, k) = nq;
                }
                for (int k = 0; k < N; ++k) {
                    const float vkp = V(k, p), vkq = V(k, q);
                    V(k, p) = c * vkp - s * vkq;
                    V(k, q) = s * vkp + c * vkq;
                }
            }
        }
    }
    float lam[N];
    for (int i = 0; i < N; ++i) lam[i] = fmaxf(A(i, i), floor);
    for (int i = 0; i < N; ++i)
        for (int j = i; j < N; ++j) {
            float sum = 0.0f;
            for (int k = 0; k < N; ++k) sum += V(i, k) * lam[k] * V(j, k);
            A(i, j) = sum;
            A(j, i) = sum;
        }
}

// One-sided Jacobi SVD of a 3x2 matrix, one rotation (exact for two
// columns). sigma ascending, U with unit columns, V 2x2.
PPF_HD void svd3x2(const Mat3x2 &F, Mat3x2 &U, Vec2 &sigma, Mat2 &V) {
    float A[3][2];
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 2; ++c) A[r][c] = F(r, c);
    float Vv[2][2] = {{1.0f, 0.0f}, {0.0f, 1.0f}};
    {
        float a = 0.0f, b = 0.0f, g = 0.0f;
        for (int r = 0; r < 3; ++r) {
            a += A[r][0] * A[r][0];
            b += A[r][1] * A[r][1];
            g += A[r][0] * A[r][1];
        }
        float zeta = (b - a) / (2.0f * g);
        float t = (g == 0.0f) ? 0.0f
                              : (zeta >= 0.0f ? 1.0f : -1.0f) /
                                    (fabsf(zeta) + sqrtf(1.0f + zeta * zeta));
        float c = 1.0f / sqrtf(1.0f + t * t), s = c * t;
        for (int r = 0; r < 3; ++r) {
            float ap = A[r][0], aq = A[r][1];
            A[r][0] = c * ap - s * aq;
            A[r][1] = s * ap + c * aq;
        }
        for (int r = 0; r < 2; ++r) {
            float vp = Vv[r][0], vq = Vv[r][1];
            Vv[r][0] = c * vp - s * vq;
            Vv[r][1] = s * vp + c * vq;
        }
    }
    float sv[2], u[3][2];
    for (int c = 0; c < 2; ++c) {
        float n2 = 0.0f;
        for (int r = 0; r < 3; ++r) n2 += A[r][c] * A[r][c];
        float n = sqrtf(n2);
        sv[c] = n;
        float inv = n > 0.0f ? 1.0f / n : 0.0f;
        for (int r = 0; r < 3; ++r) u[r][c] = A[r][c] * inv;
    }
    int i0 = 0, i1 = 1;
    if (sv[1] < sv[0]) {
        i0 = 1;
        i1 = 0;
    }
    const int idx[2] = {i0, i1};
    for (int c = 0; c < 2; ++c) {
        sigma[c] = sv[idx[c]];
        for (int r = 0; r < 3; ++r) U(r, c) = u[r][idx[c]];
        for (int r = 0; r < 2; ++r) V(r, c) = Vv[r][idx[c]];
    }
}

// Block-Jacobi inverse of a 3x3 diagonal block via its symmetrized
// eigendecomposition, eigenvalues floored at 1e-6 of the largest. Returns
// false when the largest eigenvalue is not positive and finite (the
// reference asserts there; here the caller latches a status bit).
PPF_HD bool invert_spd(const Mat3 &m, Mat3 &out) {
    Mat3 s;
    for (int a = 0; a < 3; ++a) {
        s(a, a) = m(a, a);
        for (int b = a + 1; b < 3; ++b) {
            float v = 0.5f * (m(a, b) + m(b, a));
            s(a, b) = v;
            s(b, a) = v;
        }
    }
    Vec3 lam;
    Mat3 Q;
    symm3(s, lam, Q);
    float lmax = fmaxf(lam[0], fmaxf(lam[1], lam[2]));
    out = Mat3::zero();
    bool ok = isfinite(lmax) && lmax > 0.0f;
    const float floor_ = lmax * 1.0e-6f;
    for (int k = 0; k < 3; ++k) {
        float inv = 1.0f / fmaxf(lam[k], floor_);
        float q0 = Q(0, k), q1 = Q(1, k), q2 = Q(2, k);
        out(0, 0) += inv * q0 * q0;
        out(0, 1) += inv * q0 * q1;
        out(0, 2) += inv * q0 * q2;
        out(1, 1) += inv * q1 * q1;
        out(1, 2) += inv * q1 * q2;
        out(2, 2) += inv * q2 * q2;
    }
    out(1, 0) = out(0, 1);
    out(2, 0) = out(0, 2);
    out(2, 1) = out(1, 2);
    return ok;
}

} // namespace eig
} // namespace ppf
