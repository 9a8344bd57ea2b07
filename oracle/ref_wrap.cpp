// ref_wrap.cpp -- extern "C" wrappers around the reference's own element math
// (TEST INFRASTRUCTURE).
//
// Compiled by oracle/Makefile with g++ straight from the reference's header
// and .cu sources where they lie (REF_CPP points at
// crates/ppf-cts-solver/src/cpp); the output goes only to oracle/_ref/. The
// reference's common.hpp defines __device__/__host__ away when nvcc is absent,
// so its element math compiles as host code. The few device-runtime pieces it
// touches are supplied here as serial host shims: the DISPATCH macros run the
// lambda in a loop, atomicAdd is a plain add, and the fixed Hessian the
// stiffness functions read is a small dense block table.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>

using std::isfinite;
using std::max;
using std::min;

// ---- shims that must precede the reference headers ------------------------
#define DISPATCHER_HPP
#ifndef __global__
#define __global__
#endif
#define DISPATCH_START(n)                                                      \
    {                                                                          \
        const unsigned n_threads(n);                                           \
        auto kernel =
#define DISPATCH_END                                                           \
    ;                                                                          \
    for (unsigned i_ = 0; i_ < n_threads; ++i_) kernel(i_);                    \
    }
inline float atomicAdd(float *p, float v) {
    float old = *p;
    *p += v;
    return old;
}
inline unsigned atomicAdd(unsigned *p, unsigned v) {
    unsigned old = *p;
    *p += v;
    return old;
}

#include "data.hpp"
#include "barrier/barrier.cu"
#include "contact/distance.hpp"
#include "energy/model/baraffwitkin.hpp"
#include "energy/model/dihedral_angle.hpp"
#include "energy/model/friction.hpp"
#include "energy/model/hook.hpp"
#include "energy/model/arap.hpp"
#include "energy/model/snhk.hpp"
#include "energy/model/stvk.hpp"
#include "energy/model/push.hpp"
#include "linalg/eigsolve.hpp"
#include "utility/utility.cu"
#include "eigenanalysis/eigenanalysis.cu"

namespace accd {
unsigned g_ccd_overlap = 0u, g_ccd_overlap_v0 = 0xffffffffu,
         g_ccd_overlap_v1 = 0xffffffffu, g_ccd_overlap_kind = 0xffffffffu;
float g_ccd_overlap_d2 = -1.0f, g_ccd_overlap_offset = -1.0f;
} // namespace accd
#include "contact/accd.hpp"
#include "contact/intersect_core.hpp"

extern "C" {
unsigned char g_ppf_fatal_code = 0;
char g_ppf_fatal_detail[512] = {0};
void print_rust(const char *m) { std::puts(m); }
}

// Dense block table standing in for the fixed Hessian: block (i, j) of the
// pair's local vertices 0..N-1.
static float g_blocks[4][4][9];
__device__ Mat3x3f FixedCSRMat::operator()(unsigned i, unsigned j) const {
    Mat3x3f m;
    for (int k = 0; k < 9; ++k) m.m[k] = g_blocks[i][j][k];
    return m;
}

// The strain-limit unit scatters into the fixed matrix; the wrappers never
// call those scatter paths, so the two members only need to exist.
__device__ bool FixedCSRMat::push(unsigned, unsigned, const Mat3x3f &) {
    return false;
}
__device__ void FixedCSRMat::push_at(unsigned, const Mat3x3f &) {}

namespace kernels {
template <class T> T max_array(const T *a, unsigned n, T init) {
    T r = init;
    for (unsigned i = 0; i < n; ++i) r = a[i] > r ? a[i] : r;
    return r;
}
template <class T> T min_array(const T *a, unsigned n, T init) {
    T r = init;
    for (unsigned i = 0; i < n; ++i) r = a[i] < r ? a[i] : r;
    return r;
}
} // namespace kernels

// strainlimiting.cu's compute_stiffness (strainlimiting.cu:21-44) is reached
// by including the whole unit; its DISPATCH loops run serially via the shim.
#include "strainlimiting/strainlimiting.cu"

namespace {
Vec3f v3(const float *p) { return Vec3f(p[0], p[1], p[2]); }
void put(float *dst, const float *src, int n) { std::memcpy(dst, src, n * 4); }
ParamSet ccd_param(float max_t, float eps) {
    ParamSet p{};
    p.line_search_max_t = max_t;
    p.ccd_eps = eps;
    return p;
}
} // namespace

extern "C" {

int ref_wrap_version() { return 4; }

void ref_pe_coeff(const float *p, const float *a, const float *b, float *out) {
    Vec2f c = distance::point_edge_distance_coeff<float, float>(v3(p), v3(a), v3(b));
    out[0] = c[0];
    out[1] = c[1];
}
void ref_pt_coeff(const float *p, const float *a, const float *b, const float *c,
                  float *out) {
    Vec3f r = distance::point_triangle_distance_coeff<float, float>(v3(p), v3(a), v3(b), v3(c));
    put(out, r.m, 3);
}
void ref_ee_coeff(const float *a0, const float *a1, const float *b0,
                  const float *b1, float *out) {
    Vec4f r = distance::edge_edge_distance_coeff<float, float>(v3(a0), v3(a1), v3(b0), v3(b1));
    put(out, r.m, 4);
}
void ref_pt_coeff_unclassified(const float *p, const float *a, const float *b,
                               const float *c, float *out) {
    Vec3f r = distance::point_triangle_distance_coeff_unclassified<float, float>(
        v3(p), v3(a), v3(b), v3(c));
    put(out, r.m, 3);
}
void ref_pe_coeff_unclassified(const float *p, const float *a, const float *b,
                               float *out) {
    Vec2f r = distance::point_edge_distance_coeff_unclassified<float, float>(v3(p), v3(a), v3(b));
    put(out, r.m, 2);
}
void ref_barrier(int kind, float g, float ghat, float offset, float *out) {
    Barrier b = (Barrier)kind;
    out[0] = barrier::energy(g, ghat, offset, b);
    out[1] = barrier::gradient(g, ghat, offset, b);
    out[2] = barrier::curvature(g, ghat, offset, b);
}
void ref_edge_grad_hess(const float *e, float ghat, float offset, int kind,
                        float *g, float *h) {
    Vec3f gr = barrier::compute_edge_gradient(v3(e), ghat, offset, (Barrier)kind);
    Mat3x3f hs = barrier::compute_edge_hessian(v3(e), ghat, offset, (Barrier)kind);
    put(g, gr.m, 3);
    put(h, hs.m, 9);
}
// local: (3N)x(3N) column-major elastic blocks of the pair's N vertices.
float ref_stiffness(int n, const float *w, const float *mass, const float *local,
                    const float *e, float ghat, float offset) {
    for (int i = 0; i < n; ++i)
        for (int j = 0; j < n; ++j)
            for (int c = 0; c < 3; ++c)
                for (int r = 0; r < 3; ++r)
                    g_blocks[i][j][r + 3 * c] = local[(3 * i + r) + 3 * n * (3 * j + c)];
    FixedCSRMat fake{};
    ParamSet prm{};
    if (n == 2) {
        Proximity<2> p;
        p.index = Vec2u(0, 1);
        p.value = Vec2f(w[0], w[1]);
        return barrier::compute_stiffness<2>(p, SVecf<2>(mass[0], mass[1]), fake, v3(e), ghat, offset, prm);
    } else if (n == 3) {
        Proximity<3> p;
        p.index = Vec3u(0, 1, 2);
        p.value = Vec3f(w[0], w[1], w[2]);
        return barrier::compute_stiffness<3>(p, SVecf<3>(mass[0], mass[1], mass[2]), fake, v3(e), ghat, offset, prm);
    } else {
        Proximity<4> p;
        p.index = Vec4u(0, 1, 2, 3);
        p.value = Vec4f(w[0], w[1], w[2], w[3]);
        return barrier::compute_stiffness<4>(p, SVecf<4>(mass[0], mass[1], mass[2], mass[3]), fake, v3(e), ghat, offset, prm);
    }
}
void ref_friction(const float *force, const float *dx, const float *normal,
                  float mu, float eps, float *g, float *h) {
    Friction f(v3(force), v3(dx), v3(normal), mu, eps);
    Vec3f gr = f.gradient();
    Mat3x3f hs = f.hessian();
    put(g, gr.m, 3);
    put(h, hs.m, 9);
}
void ref_push(const float *e, const float *normal, float eps, float *g, float *h) {
    Vec3f gr = push::gradient(v3(e), v3(normal), eps);
    Mat3x3f hs = push::hessian(v3(e), v3(normal), eps);
    put(g, gr.m, 3);
    put(h, hs.m, 9);
}
void ref_bw(const float *F6, float mu, float lmd, float *sg, float *sh, float *hg,
            float *hh) {
    Mat3x2f F;
    put(F.m, F6, 6);
    put(sg, BaraffWitkin::stretch_gradient(F, mu).m, 6);
    put(sh, BaraffWitkin::stretch_hessian(F, mu).m, 36);
    put(hg, BaraffWitkin::shear_gradient(F, lmd).m, 6);
    put(hh, BaraffWitkin::shear_hessian(F, lmd).m, 36);
}
void ref_deformation_grad(const float *x0, const float *x1, const float *x2,
                          const float *inv4, float *out6) {
    Mat3x3f X;
    X << v3(x0), v3(x1), v3(x2);
    Mat2x2f inv;
    put(inv.m, inv4, 4);
    put(out6, utility::compute_deformation_grad(X, inv).m, 6);
}
void ref_convert(const float *dedF6, const float *d2_36, const float *inv4,
                 float *f9, float *h81) {
    Mat3x2f g;
    put(g.m, dedF6, 6);
    Mat6x6f h;
    put(h.m, d2_36, 36);
    Mat2x2f inv;
    put(inv.m, inv4, 4);
    put(f9, utility::convert_force(g, inv).m, 9);
    put(h81, utility::convert_hessian(h, inv).m, 81);
}
// x12: positions of the ORIGINAL hinge order (h0, h1, h2, h3).
void ref_hinge(const float *x12, float rest, float *angle, float *force12,
               float *hess144) {
    Vec3f xs[4] = {v3(x12), v3(x12 + 3), v3(x12 + 6), v3(x12 + 9)};
    Vec<Vec3f> vv;
    vv.data = xs;
    vv.size = 4;
    vv.allocated = 4;
    Vec4u hinge(0, 1, 2, 3);
    Mat3x4f f;
    Mat12x12f h;
    dihedral_angle::face_compute_force_hessian(vv, hinge, rest, f, h);
    Vec4u rh = dihedral_angle::remap(Vec4u(0, 1, 2, 3));
    *angle = dihedral_angle::face_dihedral_angle(xs[rh[0]], xs[rh[1]], xs[rh[2]], xs[rh[3]]);
    put(force12, f.m, 12);
    put(hess144, h.m, 144);
}
// hook.hpp:21-37: rod stretch gradient (3 x 2) and Hessian (6 x 6).
void ref_hook(const float *x0, const float *x1, float l0, float weight, float *grad6,
              float *hess36) {
    Mat3x2f g;
    Mat6x6f h;
    hook::make_diff_table(v3(x0), v3(x1), l0, weight, g, h);
    put(grad6, g.m, 6);
    put(hess36, h.m, 36);
}
// dihedral_angle.hpp:451-541: rod bend force (3 x 3) and projected Hessian.
void ref_strand(const float *x0, const float *x1, const float *x2, float rest, float *f9,
                float *h81) {
    Mat3x3f f;
    Mat9x9f h;
    dihedral_angle::strand_compute_force_hessian(v3(x0), v3(x1), v3(x2), rest, f, h);
    put(f9, f.m, 9);
    put(h81, h.m, 81);
}
// energy/model/{arap,stvk,snhk}.hpp: singular-value tables (dim 2 or 3).
void ref_model_table(int model, int dim, const float *a, float mu, float lmd, float *deda,
                     float *d2) {
    if (dim == 2) {
        Vec2f v(a[0], a[1]);
        DiffTable2 t = model == 0 ? ARAP::make_diff_table2(v, mu, lmd)
                       : model == 1 ? StVK::make_diff_table2(v, mu, lmd)
                                    : SNHk::make_diff_table2(v, mu, lmd);
        put(deda, t.deda.m, 2);
        put(d2, t.d2ed2a.m, 4);
    } else {
        Vec3f v(a[0], a[1], a[2]);
        DiffTable3 t = model == 0 ? ARAP::make_diff_table3(v, mu, lmd)
                       : model == 1 ? StVK::make_diff_table3(v, mu, lmd)
                                    : SNHk::make_diff_table3(v, mu, lmd);
        put(deda, t.deda.m, 3);
        put(d2, t.d2ed2a.m, 9);
    }
}
// utility.cu:167-183: rotation-variant 3x3 SVD.
void ref_svd33(const float *F9, float *U9, float *S3, float *Vt9) {
    Mat3x3f F;
    put(F.m, F9, 9);
    Svd3x3 s = utility::svd3x3_rv(F);
    put(U9, s.U.m, 9);
    put(S3, s.S.m, 3);
    put(Vt9, s.Vt.m, 9);
}
// energy.cu:395-446 without damping: the tet element's force and Hessian.
void ref_tet(const float *x12, const float *inv9, int model, float mu, float lmd, float mass,
             float eps, float *f12, float *h144) {
    Mat3x4f X;
    for (int k = 0; k < 4; ++k)
        for (int d = 0; d < 3; ++d) X(d, k) = x12[3 * k + d];
    Mat3x3f inv;
    put(inv.m, inv9, 9);
    Mat3x3f F = utility::compute_deformation_grad(X, inv);
    Svd3x3 svd = utility::svd3x3_rv(F);
    DiffTable3 table = model == 0 ? ARAP::make_diff_table3(svd.S, mu, lmd)
                       : model == 1 ? StVK::make_diff_table3(svd.S, mu, lmd)
                                    : SNHk::make_diff_table3(svd.S, mu, lmd);
    Mat3x3f dedF = eigenanalysis::compute_force(table, svd);
    Mat3x4f dedx = Mat3x4f::Zero();
    Mat12x12f h = Mat12x12f::Zero();
    dedx += mass * utility::convert_force(dedF, inv);
    eigenanalysis::accumulate_hessian_tet_fused(table, svd, eps, inv, mass, h);
    put(f12, dedx.m, 12);
    put(h144, h.m, 144);
}
// energy.cu:336-355: a shell face under ARAP / StVK / SNHk.
void ref_shell_model(const float *x9, const float *inv4, int model, float mu, float lmd,
                     float mass, float eps, float *f9, float *h81) {
    Mat3x3f X;
    put(X.m, x9, 9);
    Mat2x2f inv;
    put(inv.m, inv4, 4);
    Mat3x2f F = utility::compute_deformation_grad(X, inv);
    const Svd3x2 svd = utility::svd3x2(F);
    DiffTable2 table = model == 0 ? ARAP::make_diff_table2(svd.S, mu, lmd)
                       : model == 1 ? StVK::make_diff_table2(svd.S, mu, lmd)
                                    : SNHk::make_diff_table2(svd.S, mu, lmd);
    Mat3x2f dedF = eigenanalysis::compute_force(table, svd);
    Mat6x6f d2edF2 = eigenanalysis::compute_hessian(table, svd, eps);
    Mat3x3f dedx = Mat3x3f::Zero();
    Mat9x9f h = Mat9x9f::Zero();
    dedx += mass * utility::convert_force(dedF, inv);
    h += mass * utility::convert_hessian(d2edF2, inv);
    put(f9, dedx.m, 9);
    put(h81, h.m, 81);
}
void ref_symm2(const float *A4, float *val, float *vec) {
    Mat2x2f A;
    put(A.m, A4, 4);
    linalg::eig::V2 v;
    linalg::eig::M2 e;
    linalg::eig::symm2x2(A, v, e);
    put(val, v.m, 2);
    put(vec, e.m, 4);
}
void ref_symm3(const float *A9, float *val, float *vec) {
    Mat3x3f A;
    put(A.m, A9, 9);
    linalg::eig::V3 v;
    linalg::eig::M3 e;
    linalg::eig::symm3x3(A, v, e);
    put(val, v.m, 3);
    put(vec, e.m, 9);
}
void ref_psd4(float *A16) {
    SMat<float, 4, 4> A;
    put(A.m, A16, 16);
    linalg::psd_project_symmetric<4>(A, 0.0f);
    put(A16, A.m, 16);
}
void ref_svd32(const float *F6, float *U6, float *S2, float *Vt4) {
    Mat3x2f F;
    put(F.m, F6, 6);
    Svd3x2 s = utility::svd3x2(F);
    put(U6, s.U.m, 6);
    put(S2, s.S.m, 2);
    put(Vt4, s.Vt.m, 4);
}
void ref_strainlimit_table(const float *a2, float ghat, int kind, float *deda,
                           float *d2) {
    DiffTable2 t = barrier::compute_strainlimiting_diff_table(Vec2f(a2[0], a2[1]), ghat, (Barrier)kind);
    put(deda, t.deda.m, 2);
    put(d2, t.d2ed2a.m, 4);
}
void ref_eigen_force_hessian(const float *deda, const float *d2, const float *U6,
                             const float *S2, const float *Vt4, float eps,
                             float *f6, float *h36) {
    DiffTable2 t;
    put(t.deda.m, deda, 2);
    put(t.d2ed2a.m, d2, 4);
    Svd3x2 s;
    put(s.U.m, U6, 6);
    put(s.S.m, S2, 2);
    put(s.Vt.m, Vt4, 4);
    put(f6, eigenanalysis::compute_force(t, s).m, 6);
    put(h36, eigenanalysis::compute_hessian(t, s, eps).m, 36);
}
float ref_strain_stiffness(const float *x9, const float *local81, float mass,
                           const float *S2, float limit) {
    Vec3f xs[3] = {v3(x9), v3(x9 + 3), v3(x9 + 6)};
    Vec<Vec3f> vv;
    vv.data = xs;
    vv.size = 3;
    vv.allocated = 3;
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j)
            for (int c = 0; c < 3; ++c)
                for (int r = 0; r < 3; ++r)
                    g_blocks[i][j][r + 3 * c] = local81[(3 * i + r) + 9 * (3 * j + c)];
    Svd3x2 s{};
    s.S = Vec2f(S2[0], S2[1]);
    FixedCSRMat fake{};
    return strainlimiting::compute_stiffness(vv, Vec3u(0, 1, 2), fake, mass, s, limit);
}
float ref_singular_minus_one_max(const float *F6) {
    Mat3x2f F;
    put(F.m, F6, 6);
    return utility::singular_vals_minus_one(F).maxCoeff();
}
// CCD: x holds the sweep start of every column, then the sweep end.
float ref_ccd(int kind, const float *x0, const float *x1, float offset,
              float ghat, float max_t, float eps, int *overlap) {
    accd::g_ccd_overlap = 0u;
    ParamSet p = ccd_param(max_t, eps);
    float r;
    if (kind == 0)
        r = accd::point_triangle_ccd(v3(x0), v3(x1), v3(x0 + 3), v3(x0 + 6), v3(x0 + 9),
                                     v3(x1 + 3), v3(x1 + 6), v3(x1 + 9), offset, ghat, p);
    else if (kind == 1)
        r = accd::point_edge_ccd(v3(x0), v3(x1), v3(x0 + 3), v3(x0 + 6), v3(x1 + 3),
                                 v3(x1 + 6), offset, ghat, p);
    else if (kind == 2)
        r = accd::point_point_ccd(v3(x0), v3(x1), v3(x0 + 3), v3(x1 + 3), offset, ghat, p);
    else
        r = accd::edge_edge_ccd(v3(x0), v3(x0 + 3), v3(x0 + 6), v3(x0 + 9), v3(x1),
                                v3(x1 + 3), v3(x1 + 6), v3(x1 + 9), offset, ghat, p);
    *overlap = (int)accd::g_ccd_overlap;
    return r;
}
int ref_edge_triangle(const float *e0, const float *e1, const float *t0,
                      const float *t1, const float *t2) {
    float z[3] = {0, 0, 0};
    float a[3], b[3], d1[3], d2[3];
    for (int k = 0; k < 3; ++k) {
        a[k] = e0[k] - t0[k];
        b[k] = e1[k] - t0[k];
        d1[k] = t1[k] - t0[k];
        d2[k] = t2[k] - t0[k];
    }
    return ppf_isect::edge_triangle_intersect<float>(a, b, z, d1, d2) ? 1 : 0;
}

} // extern "C"
