// linalg.cuh -- fixed-size column-major float matrices for the element math.
//
// Compiled twice: by nvcc into the sm_103a kernels and by g++ into the CPU
// oracle library, so every function is host+device and free of CUDA-only
// intrinsics. Storage is column-major (element (i, j) at m[i + R * j]) because
// that is the byte layout of the 3x3 / 2x2 blocks exchanged through the C ABI
// (data.hpp Mat3x3f / Mat2x2f). Reductions run left to right from zero, the
// order the reference's smat.hpp uses, and normalize() leaves an exact-zero
// vector at zero instead of producing 0/0.
#pragma once

#include <math.h>

#if defined(__CUDACC__)
#define PPF_HD __host__ __device__ __forceinline__
#define PPF_HDI __host__ __device__ inline
#else
#define PPF_HD inline
#define PPF_HDI inline
#endif

namespace ppf {

PPF_HD float fmin2(float a, float b) { return fminf(a, b); }
PPF_HD float fmax2(float a, float b) { return fmaxf(a, b); }
PPF_HD float sqr(float x) { return x * x; }

template <int R, int C> struct Mat {
    float m[R * C];

    PPF_HD float &operator()(int i, int j) { return m[i + R * j]; }
    PPF_HD float operator()(int i, int j) const { return m[i + R * j]; }
    PPF_HD float &operator[](int i) { return m[i]; }
    PPF_HD float operator[](int i) const { return m[i]; }

    PPF_HD static Mat zero() {
        Mat r;
#pragma unroll
        for (int i = 0; i < R * C; ++i) r.m[i] = 0.0f;
        return r;
    }
    PPF_HD static Mat identity() {
        Mat r = zero();
#pragma unroll
        for (int i = 0; i < (R < C ? R : C); ++i) r(i, i) = 1.0f;
        return r;
    }
    PPF_HD static Mat constant(float v) {
        Mat r;
#pragma unroll
        for (int i = 0; i < R * C; ++i) r.m[i] = v;
        return r;
    }
    PPF_HD Mat<R, 1> col(int j) const {
        Mat<R, 1> r;
#pragma unroll
        for (int i = 0; i < R; ++i) r.m[i] = m[i + R * j];
        return r;
    }
    PPF_HD void set_col(int j, const Mat<R, 1> &v) {
#pragma unroll
        for (int i = 0; i < R; ++i) m[i + R * j] = v.m[i];
    }
    PPF_HD Mat<1, C> row(int i) const {
        Mat<1, C> r;
#pragma unroll
        for (int j = 0; j < C; ++j) r.m[j] = m[i + R * j];
        return r;
    }
    PPF_HD Mat<C, R> transpose() const {
        Mat<C, R> r;
#pragma unroll
        for (int i = 0; i < R; ++i)
#pragma unroll
            for (int j = 0; j < C; ++j) r(j, i) = (*this)(i, j);
        return r;
    }
    template <int BR, int BC> PPF_HD Mat<BR, BC> block(int i0, int j0) const {
        Mat<BR, BC> r;
#pragma unroll
        for (int j = 0; j < BC; ++j)
#pragma unroll
            for (int i = 0; i < BR; ++i) r(i, j) = (*this)(i0 + i, j0 + j);
        return r;
    }
    template <int BR, int BC>
    PPF_HD void set_block(int i0, int j0, const Mat<BR, BC> &b) {
#pragma unroll
        for (int j = 0; j < BC; ++j)
#pragma unroll
            for (int i = 0; i < BR; ++i) (*this)(i0 + i, j0 + j) = b(i, j);
    }
    template <int BR, int BC>
    PPF_HD void add_block(int i0, int j0, const Mat<BR, BC> &b) {
#pragma unroll
        for (int j = 0; j < BC; ++j)
#pragma unroll
            for (int i = 0; i < BR; ++i) (*this)(i0 + i, j0 + j) += b(i, j);
    }
    PPF_HD float dot(const Mat &o) const {
        float acc = 0.0f;
#pragma unroll
        for (int i = 0; i < R * C; ++i) acc = acc + m[i] * o.m[i];
        return acc;
    }
    PPF_HD float squared_norm() const { return dot(*this); }
    PPF_HD float norm() const { return sqrtf(squared_norm()); }
    PPF_HD void normalize() {
        float n = norm();
        if (n > 0.0f) {
#pragma unroll
            for (int i = 0; i < R * C; ++i) m[i] = m[i] / n;
        }
    }
    PPF_HD Mat normalized() const {
        Mat r = *this;
        r.normalize();
        return r;
    }
    PPF_HD float max_coeff() const {
        float r = m[0];
#pragma unroll
        for (int i = 1; i < R * C; ++i) r = m[i] > r ? m[i] : r;
        return r;
    }
    PPF_HD float min_coeff() const {
        float r = m[0];
#pragma unroll
        for (int i = 1; i < R * C; ++i) r = m[i] < r ? m[i] : r;
        return r;
    }
    PPF_HD Mat cwise_abs() const {
        Mat r;
#pragma unroll
        for (int i = 0; i < R * C; ++i) r.m[i] = fabsf(m[i]);
        return r;
    }
    PPF_HD float trace() const {
        float t = 0.0f;
#pragma unroll
        for (int i = 0; i < (R < C ? R : C); ++i) t = t + (*this)(i, i);
        return t;
    }
    PPF_HD bool is_zero() const {
#pragma unroll
        for (int i = 0; i < R * C; ++i)
            if (m[i] != 0.0f) return false;
        return true;
    }
    PPF_HD Mat &operator+=(const Mat &o) {
#pragma unroll
        for (int i = 0; i < R * C; ++i) m[i] += o.m[i];
        return *this;
    }
    PPF_HD Mat &operator-=(const Mat &o) {
#pragma unroll
        for (int i = 0; i < R * C; ++i) m[i] -= o.m[i];
        return *this;
    }
    PPF_HD Mat &operator*=(float s) {
#pragma unroll
        for (int i = 0; i < R * C; ++i) m[i] *= s;
        return *this;
    }
};

template <int N> using Vec = Mat<N, 1>;
using Vec2 = Mat<2, 1>;
using Vec3 = Mat<3, 1>;
using Vec4 = Mat<4, 1>;
using Vec6 = Mat<6, 1>;
using Vec9 = Mat<9, 1>;
using Vec12 = Mat<12, 1>;
using Mat2 = Mat<2, 2>;
using Mat3 = Mat<3, 3>;
using Mat3x2 = Mat<3, 2>;
using Mat3x4 = Mat<3, 4>;
using Mat6 = Mat<6, 6>;
using Mat9 = Mat<9, 9>;
using Mat12 = Mat<12, 12>;

template <int R, int C>
PPF_HD Mat<R, C> operator+(const Mat<R, C> &a, const Mat<R, C> &b) {
    Mat<R, C> r;
#pragma unroll
    for (int i = 0; i < R * C; ++i) r.m[i] = a.m[i] + b.m[i];
    return r;
}
template <int R, int C>
PPF_HD Mat<R, C> operator-(const Mat<R, C> &a, const Mat<R, C> &b) {
    Mat<R, C> r;
#pragma unroll
    for (int i = 0; i < R * C; ++i) r.m[i] = a.m[i] - b.m[i];
    return r;
}
template <int R, int C> PPF_HD Mat<R, C> operator-(const Mat<R, C> &a) {
    Mat<R, C> r;
#pragma unroll
    for (int i = 0; i < R * C; ++i) r.m[i] = -a.m[i];
    return r;
}
template <int R, int C> PPF_HD Mat<R, C> operator*(float s, const Mat<R, C> &a) {
    Mat<R, C> r;
#pragma unroll
    for (int i = 0; i < R * C; ++i) r.m[i] = s * a.m[i];
    return r;
}
template <int R, int C> PPF_HD Mat<R, C> operator*(const Mat<R, C> &a, float s) {
    Mat<R, C> r;
#pragma unroll
    for (int i = 0; i < R * C; ++i) r.m[i] = a.m[i] * s;
    return r;
}
template <int R, int C> PPF_HD Mat<R, C> operator/(const Mat<R, C> &a, float s) {
    Mat<R, C> r;
#pragma unroll
    for (int i = 0; i < R * C; ++i) r.m[i] = a.m[i] / s;
    return r;
}
// Matrix product; each entry is a left-to-right sum over k.
template <int R, int K, int C>
PPF_HD Mat<R, C> operator*(const Mat<R, K> &a, const Mat<K, C> &b) {
    Mat<R, C> r;
#pragma unroll
    for (int j = 0; j < C; ++j)
#pragma unroll
        for (int i = 0; i < R; ++i) {
            float acc = 0.0f;
#pragma unroll
            for (int k = 0; k < K; ++k) acc = acc + a(i, k) * b(k, j);
            r(i, j) = acc;
        }
    return r;
}

PPF_HD Vec2 vec2(float a, float b) {
    Vec2 r;
    r.m[0] = a;
    r.m[1] = b;
    return r;
}
PPF_HD Vec3 vec3(float a, float b, float c) {
    Vec3 r;
    r.m[0] = a;
    r.m[1] = b;
    r.m[2] = c;
    return r;
}
PPF_HD Vec4 vec4(float a, float b, float c, float d) {
    Vec4 r;
    r.m[0] = a;
    r.m[1] = b;
    r.m[2] = c;
    r.m[3] = d;
    return r;
}
PPF_HD Vec3 cross(const Vec3 &a, const Vec3 &b) {
    return vec3(a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2],
                a[0] * b[1] - a[1] * b[0]);
}
template <int N> PPF_HD Mat<N, N> outer(const Vec<N> &a, const Vec<N> &b) {
    Mat<N, N> r;
#pragma unroll
    for (int j = 0; j < N; ++j)
#pragma unroll
        for (int i = 0; i < N; ++i) r(i, j) = a[i] * b[j];
    return r;
}
PPF_HD Mat3 mat3_cols(const Vec3 &a, const Vec3 &b, const Vec3 &c) {
    Mat3 r;
    r.set_col(0, a);
    r.set_col(1, b);
    r.set_col(2, c);
    return r;
}
PPF_HD Mat3x2 mat3x2_cols(const Vec3 &a, const Vec3 &b) {
    Mat3x2 r;
    r.set_col(0, a);
    r.set_col(1, b);
    return r;
}
PPF_HD float det2(const Mat2 &a) { return a(0, 0) * a(1, 1) - a(0, 1) * a(1, 0); }
PPF_HD float det3(const Mat3 &a) {
    return a(0, 0) * (a(1, 1) * a(2, 2) - a(1, 2) * a(2, 1)) -
           a(0, 1) * (a(1, 0) * a(2, 2) - a(1, 2) * a(2, 0)) +
           a(0, 2) * (a(1, 0) * a(2, 1) - a(1, 1) * a(2, 0));
}
template <int N> PPF_HD Vec<N> load_vec(const float *p) {
    Vec<N> r;
#pragma unroll
    for (int i = 0; i < N; ++i) r.m[i] = p[i];
    return r;
}
template <int R, int C> PPF_HD void store(float *p, const Mat<R, C> &a) {
#pragma unroll
    for (int i = 0; i < R * C; ++i) p[i] = a.m[i];
}
PPF_HD Mat3 load_mat3(const float *p) {
    Mat3 r;
#pragma unroll
    for (int i = 0; i < 9; ++i) r.m[i] = p[i];
    return r;
}

} // namespace ppf
