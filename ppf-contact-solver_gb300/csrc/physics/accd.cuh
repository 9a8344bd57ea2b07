// accd.cuh -- additive continuous collision detection of one primitive pair.
//
// Restates crates/ppf-cts-solver/src/cpp/contact/accd.hpp:
//   centerize / rescale into a unit frame       accd.hpp:63-120
//   Lipschitz bound over inter-primitive pairs  accd.hpp:141-151
//   directional advance certificate             accd.hpp:241-281
//   park floor 1e-2 ghat                        accd.hpp:289
//   conservative advance (<= 4096 probes) then bisection to float resolution,
//   park / dip hysteresis                       accd.hpp:291-471
//   pair entry points                           accd.hpp:565-696
// A pair that starts inside its contact offset (or whose sweep frame
// collapses) returns 0 and reports it through `CcdFlag` instead of a device
// global, so the same code serves the CPU oracle and the kernels; the kernels
// fold the flags into the step's status block.
#pragma once

#include "distance.cuh"

namespace ppf {
namespace accd {

struct CcdFlag {
    bool overlap = false;
    float d2 = -1.0f;
    float offset = -1.0f;
};

template <int C> PPF_HD void centerize(Mat<3, C> &x) {
    Vec3 mov = Vec3::zero();
    const float s = (float)(1.0 / C);
#pragma unroll
    for (int k = 0; k < C; ++k) mov += s * x.col(k);
#pragma unroll
    for (int k = 0; k < C; ++k) x.set_col(k, x.col(k) - mov);
}

template <int C>
PPF_HD float rescale(Mat<3, C> &x, Mat<3, C> &dx, float max_t, CcdFlag *flag) {
    float m = fmaxf(x.cwise_abs().max_coeff(), (x + max_t * dx).cwise_abs().max_coeff());
    float scale = 0.99f / m;
    if (!(scale > 0.0f) || !isfinite(scale)) {
        if (flag) {
            flag->overlap = true;
            flag->d2 = 0.0f;
            flag->offset = -1.0f;
        }
        return 0.0f;
    }
    float scaled = 1.0f;
    const float s = 8.0f;
    while (true) {
        if (scale > s) {
            x *= s;
            dx *= s;
            scaled *= s;
            scale /= s;
        } else {
            x *= scale;
            dx *= scale;
            scaled *= scale;
            break;
        }
    }
    return scaled;
}

template <int C, int SPLIT> PPF_HD float max_relative_u(const Mat<3, C> &u) {
    float mu = 0.0f;
#pragma unroll
    for (int i = 0; i < SPLIT; ++i)
#pragma unroll
        for (int j = SPLIT; j < C; ++j) {
            Vec3 du = u.col(i) - u.col(j);
            mu = fmaxf(mu, du.squared_norm());
        }
    return sqrtf(mu);
}

template <int C, int SPLIT>
PPF_HD float directional_advance(const Mat<3, C> &x, const Mat<3, C> &dx,
                                 const Vec3 &w, float w_norm, float dip,
                                 float park, float max_t) {
    const float round_slack = 2.0f * 1.19209290e-7f;
    const float coord_slack = 6.2e-7f;
    Vec3 wa = w.cwise_abs();
    float dip_w = dip * w_norm;
    float park_w = park * w_norm;
    float step = 3.402823466e+38f;
#pragma unroll
    for (int i = 0; i < SPLIT; ++i)
#pragma unroll
        for (int j = SPLIT; j < C; ++j) {
            Vec3 gap = x.col(j) - x.col(i);
            Vec3 rel = dx.col(i) - dx.col(j);
            float err = round_slack * (wa.dot(gap.cwise_abs()) +
                                       max_t * wa.dot(rel.cwise_abs()) + park_w) +
                        coord_slack * w_norm;
            float projected = w.dot(gap) - err;
            if (!(projected - dip_w > 0.0f)) return 0.0f;
            float rate = w.dot(rel);
            if (rate > 0.0f) step = fminf(step, fmaxf(0.0f, projected - park_w) / rate);
        }
    return step;
}

PPF_HD float park_floor(float ghat) { return 1e-2f * ghat; }

// squared distance of the sweep state x and the direction from primitive A's
// closest point to primitive B's (A = columns [0, SPLIT)).
struct PointTriangleDist {
    PPF_HD float operator()(const Mat<3, 4> &x, Vec3 &dir) const {
        Vec3 p = x.col(0), t0 = x.col(1), t1 = x.col(2), t2 = x.col(3);
        Vec3 c = dist::point_triangle_coeff_unclassified(p, t0, t1, t2);
        dir = c[0] * (t0 - p) + c[1] * (t1 - p) + c[2] * (t2 - p);
        return dir.dot(dir);
    }
};
struct PointEdgeDist {
    PPF_HD float operator()(const Mat<3, 3> &x, Vec3 &dir) const {
        Vec3 p = x.col(0), q0 = x.col(1), q1 = x.col(2);
        Vec2 c = dist::point_edge_coeff_unclassified(p, q0, q1);
        dir = (c[0] * q0 + c[1] * q1) - p;
        return dir.dot(dir);
    }
};
struct PointPointDist {
    PPF_HD float operator()(const Mat<3, 2> &x, Vec3 &dir) const {
        dir = x.col(1) - x.col(0);
        return dir.dot(dir);
    }
};
struct EdgeEdgeDist {
    PPF_HD float operator()(const Mat<3, 4> &x, Vec3 &dir) const {
        Vec3 p0 = x.col(0), p1 = x.col(1), q0 = x.col(2), q1 = x.col(3);
        Vec4 c = dist::edge_edge_coeff(p0, p1, q0, q1);
        Vec3 a = c[0] * p0 + c[1] * p1;
        Vec3 b = c[2] * q0 + c[3] * q1;
        dir = b - a;
        return dir.dot(dir);
    }
};

template <class F, int C, int SPLIT>
PPF_HD float ccd_helper(const Mat<3, C> &x0, const Mat<3, C> &dx, float u_max,
                        const F &dist2, float offset, float eps, float floor_gap,
                        float max_t, CcdFlag *flag) {
    Mat<3, C> x = x0;
    Vec3 w;
    float lower_t = 0.0f, toi = 0.0f;
    float d2 = dist2(x0, w);
    float target2 = offset * offset;
    if (!(d2 > target2)) {
        if (flag) {
            flag->overlap = true;
            flag->d2 = d2;
            flag->offset = offset;
        }
        return 0.0f;
    }
    float clearance = sqrtf(d2) - offset;
    float floor_clear = fmaxf(2.0f * eps, floor_gap);
    float park = offset + fminf(floor_clear, fmaxf(clearance - 0.5f * eps, 0.5f * clearance));
    float overshoot = fmaxf(0.0f, (park - offset) - 0.5f * floor_clear);
    float dip = park - overshoot;
    float park2 = fminf(park * park, nextafterf(d2, 0.0f));
    float inv_u = 1.0f / u_max;
    const unsigned max_probes = 4096u;
    unsigned probes = 0;
    while (true) {
        if (!(d2 > park2)) break;
        lower_t = toi;
        float dist = sqrtf(d2);
        float step = (dist - dip) * inv_u;
        if (toi + step <= max_t) {
            step = fmaxf(step, directional_advance<C, SPLIT>(
                                   x, dx, w, dist * (1.0f + 2.0f * 1.19209290e-7f),
                                   dip, park, max_t));
        }
        toi += step;
        if (toi > max_t) return max_t;
        if (++probes > max_probes) return lower_t;
        x = x0 + toi * dx;
        d2 = dist2(x, w);
    }
    float upper_t = toi;
    float window = upper_t - lower_t;
    while (true) {
        toi = 0.5f * (upper_t + lower_t);
        x = x0 + toi * dx;
        Vec3 wd;
        d2 = dist2(x, wd);
        if (d2 > park2) lower_t = toi;
        else upper_t = toi;
        float nw = upper_t - lower_t;
        if (nw == window) break;
        window = nw;
    }
    if (!(lower_t > 0.0f)) {
        if (flag) {
            flag->overlap = true;
            flag->d2 = d2;
            flag->offset = offset;
        }
        return 0.0f;
    }
    return lower_t;
}

template <class F, int C, int SPLIT>
PPF_HD float sweep_ccd(Mat<3, C> x0, Mat<3, C> dx, float offset, float ghat,
                       float max_t, float ccd_eps, CcdFlag *flag) {
    centerize<C>(x0);
    centerize<C>(dx);
    float scale = rescale<C>(x0, dx, max_t, flag);
    if (!(scale > 0.0f)) return 0.0f;
    float u_max = max_relative_u<C, SPLIT>(dx);
    if (u_max) {
        F f;
        return ccd_helper<F, C, SPLIT>(x0, dx, u_max, f, scale * offset,
                                       scale * ccd_eps, scale * park_floor(ghat),
                                       max_t, flag);
    }
    return max_t;
}

PPF_HD float point_triangle(const Vec3 &p0, const Vec3 &p1, const Vec3 &t00,
                            const Vec3 &t01, const Vec3 &t02, const Vec3 &t10,
                            const Vec3 &t11, const Vec3 &t12, float offset,
                            float ghat, float max_t, float ccd_eps, CcdFlag *flag) {
    Mat<3, 4> x, d;
    x.set_col(0, p0);
    x.set_col(1, t00);
    x.set_col(2, t01);
    x.set_col(3, t02);
    d.set_col(0, p1 - p0);
    d.set_col(1, t10 - t00);
    d.set_col(2, t11 - t01);
    d.set_col(3, t12 - t02);
    return sweep_ccd<PointTriangleDist, 4, 1>(x, d, offset, ghat, max_t, ccd_eps, flag);
}

PPF_HD float point_edge(const Vec3 &p0, const Vec3 &p1, const Vec3 &e00,
                        const Vec3 &e01, const Vec3 &e10, const Vec3 &e11,
                        float offset, float ghat, float max_t, float ccd_eps,
                        CcdFlag *flag) {
    Mat<3, 3> x, d;
    x.set_col(0, p0);
    x.set_col(1, e00);
    x.set_col(2, e01);
    d.set_col(0, p1 - p0);
    d.set_col(1, e10 - e00);
    d.set_col(2, e11 - e01);
    return sweep_ccd<PointEdgeDist, 3, 1>(x, d, offset, ghat, max_t, ccd_eps, flag);
}

PPF_HD float point_point(const Vec3 &p0, const Vec3 &p1, const Vec3 &q0,
                         const Vec3 &q1, float offset, float ghat, float max_t,
                         float ccd_eps, CcdFlag *flag) {
    Mat<3, 2> x, d;
    x.set_col(0, p0);
    x.set_col(1, q0);
    d.set_col(0, p1 - p0);
    d.set_col(1, q1 - q0);
    return sweep_ccd<PointPointDist, 2, 1>(x, d, offset, ghat, max_t, ccd_eps, flag);
}

PPF_HD float edge_edge(const Vec3 &a00, const Vec3 &a01, const Vec3 &b00,
                       const Vec3 &b01, const Vec3 &a10, const Vec3 &a11,
                       const Vec3 &b10, const Vec3 &b11, float offset, float ghat,
                       float max_t, float ccd_eps, CcdFlag *flag) {
    Mat<3, 4> x, d;
    x.set_col(0, a00);
    x.set_col(1, a01);
    x.set_col(2, b00);
    x.set_col(3, b01);
    d.set_col(0, a10 - a00);
    d.set_col(1, a11 - a01);
    d.set_col(2, b10 - b00);
    d.set_col(3, b11 - b01);
    return sweep_ccd<EdgeEdgeDist, 4, 2>(x, d, offset, ghat, max_t, ccd_eps, flag);
}

} // namespace accd
} // namespace ppf
