// oracle_elem.cpp -- CPU entry points for the element math (TEST INFRASTRUCTURE).
//
// Exposes the element-level functions that the sm_103a kernels evaluate
// (ppf-contact-solver_gb300/csrc/physics/*.cuh, compiled here as host code)
// with the same signatures as oracle/ref_wrap.cpp exposes the reference's, so
// tests can check each formula against the reference's own code on the same
// inputs and against the golden vectors frozen from it.
#include "../ppf-contact-solver_gb300/csrc/physics/accd.cuh"
#include "../ppf-contact-solver_gb300/csrc/physics/bw.cuh"
#include "../ppf-contact-solver_gb300/csrc/physics/contact_local.cuh"
#include "../ppf-contact-solver_gb300/csrc/physics/elastic.cuh"
#include "../ppf-contact-solver_gb300/csrc/physics/hinge.cuh"
#include "../ppf-contact-solver_gb300/csrc/physics/rod.cuh"
#include "../ppf-contact-solver_gb300/csrc/physics/strainlimit.cuh"

#include <cstring>

using namespace ppf;

namespace {
Vec3 v3(const float *p) { return vec3(p[0], p[1], p[2]); }
template <int R, int C> void put(float *dst, const Mat<R, C> &m) {
    std::memcpy(dst, m.m, sizeof(float) * R * C);
}
template <int R, int C> Mat<R, C> get(const float *src) {
    Mat<R, C> m;
    std::memcpy(m.m, src, sizeof(float) * R * C);
    return m;
}
} // namespace

extern "C" {

void orc_pe_coeff(const float *p, const float *a, const float *b, float *out) {
    put(out, dist::point_edge_coeff(v3(p), v3(a), v3(b)));
}
void orc_pt_coeff(const float *p, const float *a, const float *b, const float *c,
                  float *out) {
    put(out, dist::point_triangle_coeff(v3(p), v3(a), v3(b), v3(c)));
}
void orc_ee_coeff(const float *a0, const float *a1, const float *b0,
                  const float *b1, float *out) {
    put(out, dist::edge_edge_coeff(v3(a0), v3(a1), v3(b0), v3(b1)));
}
void orc_pt_coeff_unclassified(const float *p, const float *a, const float *b,
                               const float *c, float *out) {
    put(out, dist::point_triangle_coeff_unclassified(v3(p), v3(a), v3(b), v3(c)));
}
void orc_pe_coeff_unclassified(const float *p, const float *a, const float *b,
                               float *out) {
    put(out, dist::point_edge_coeff_unclassified(v3(p), v3(a), v3(b)));
}
void orc_barrier(int kind, float g, float ghat, float offset, float *out) {
    out[0] = barrier::energy(g, ghat, offset, kind);
    out[1] = barrier::gradient(g, ghat, offset, kind);
    out[2] = barrier::curvature(g, ghat, offset, kind);
}
void orc_edge_grad_hess(const float *e, float ghat, float offset, int kind,
                        float *g, float *h) {
    put(g, barrier::edge_gradient(v3(e), ghat, offset, kind));
    put(h, barrier::edge_hessian(v3(e), ghat, offset, kind));
}
float orc_stiffness(int n, const float *w, const float *mass, const float *local,
                    const float *e, float ghat, float offset) {
    (void)ghat;
    if (n == 2) {
        float ww[2] = {w[0], w[1]}, mm[2] = {mass[0], mass[1]};
        return barrier::stiffness<2>(ww, mm, get<6, 6>(local), v3(e), offset);
    } else if (n == 3) {
        float ww[3] = {w[0], w[1], w[2]}, mm[3] = {mass[0], mass[1], mass[2]};
        return barrier::stiffness<3>(ww, mm, get<9, 9>(local), v3(e), offset);
    }
    float ww[4] = {w[0], w[1], w[2], w[3]}, mm[4] = {mass[0], mass[1], mass[2], mass[3]};
    return barrier::stiffness<4>(ww, mm, get<12, 12>(local), v3(e), offset);
}
void orc_friction(const float *force, const float *dx, const float *normal,
                  float mu, float eps, float *g, float *h) {
    Friction f(v3(force), v3(dx), v3(normal), mu, eps);
    put(g, f.gradient());
    put(h, f.hessian());
}
void orc_push(const float *e, const float *normal, float eps, float *g, float *h) {
    put(g, push::gradient(v3(e), v3(normal), eps));
    put(h, push::hessian(v3(e), v3(normal), eps));
}
void orc_bw(const float *F6, float mu, float lmd, float *sg, float *sh, float *hg,
            float *hh) {
    Mat3x2 F = get<3, 2>(F6);
    put(sg, bw::stretch_gradient(F, mu));
    put(sh, bw::stretch_hessian(F, mu));
    put(hg, bw::shear_gradient(F, lmd));
    put(hh, bw::shear_hessian(F, lmd));
}
void orc_deformation_grad(const float *x0, const float *x1, const float *x2,
                          const float *inv4, float *out6) {
    put(out6, bw::deformation_grad(v3(x0), v3(x1), v3(x2), get<2, 2>(inv4)));
}
void orc_convert(const float *dedF6, const float *d2_36, const float *inv4,
                 float *f9, float *h81) {
    Mat2 inv = get<2, 2>(inv4);
    put(f9, bw::convert_force(get<3, 2>(dedF6), inv));
    put(h81, bw::convert_hessian(get<6, 6>(d2_36), inv));
}
void orc_hinge(const float *x12, float rest, float *angle, float *force12,
               float *hess144) {
    // remap (h2, h1, h0, h3)
    Vec3 X0 = v3(x12 + 6), X1 = v3(x12 + 3), X2 = v3(x12), X3 = v3(x12 + 9);
    Mat3x4 f;
    Mat12 h;
    hinge::force_hessian(X0, X1, X2, X3, rest, f, h);
    *angle = hinge::dihedral_angle(X0, X1, X2, X3);
    put(force12, f);
    put(hess144, h);
}
void orc_hook(const float *x0, const float *x1, float l0, float weight, float *grad6,
              float *hess36) {
    Mat3x2 g;
    Mat6 h;
    rod::stretch(v3(x0), v3(x1), l0, weight, g, h);
    put(grad6, g);
    put(hess36, h);
}
void orc_strand(const float *x0, const float *x1, const float *x2, float rest, float *f9,
                float *h81) {
    Mat3 f;
    Mat9 h;
    rod::bend(v3(x0), v3(x1), v3(x2), rest, f, h);
    put(f9, f);
    put(h81, h);
}
void orc_model_table(int model, int dim, const float *a, float mu, float lmd, float *deda,
                     float *d2) {
    if (dim == 2) {
        elastic::Table<2> t;
        elastic::table<2>(model, vec2(a[0], a[1]), mu, lmd, t);
        put(deda, t.deda);
        put(d2, t.d2);
    } else {
        elastic::Table<3> t;
        elastic::table<3>(model, vec3(a[0], a[1], a[2]), mu, lmd, t);
        put(deda, t.deda);
        put(d2, t.d2);
    }
}
void orc_svd33(const float *F9, float *U9, float *S3, float *Vt9) {
    elastic::Svd33 s = elastic::svd3x3_rv(get<3, 3>(F9));
    put(U9, s.U);
    put(S3, s.S);
    put(Vt9, s.Vt);
}
void orc_tet(const float *x12, const float *inv9, int model, float mu, float lmd, float mass,
             float eps, float *f12, float *h144) {
    Mat3x4 f;
    Mat12 h;
    elastic::tet(v3(x12), v3(x12 + 3), v3(x12 + 6), v3(x12 + 9), get<3, 3>(inv9), model, mu, lmd,
                 mass, eps, f, h);
    put(f12, f);
    put(h144, h);
}
void orc_shell_model(const float *x9, const float *inv4, int model, float mu, float lmd,
                     float mass, float eps, float *f9, float *h81) {
    Mat3 f;
    Mat9 h;
    elastic::shell(v3(x9), v3(x9 + 3), v3(x9 + 6), get<2, 2>(inv4), model, mu, lmd, mass, eps, f,
                   h);
    put(f9, f);
    put(h81, h);
}
void orc_symm2(const float *A4, float *val, float *vec) {
    Vec2 v;
    Mat2 e;
    eig::symm2(get<2, 2>(A4), v, e);
    put(val, v);
    put(vec, e);
}
void orc_symm3(const float *A9, float *val, float *vec) {
    Vec3 v;
    Mat3 e;
    eig::symm3(get<3, 3>(A9), v, e);
    put(val, v);
    put(vec, e);
}
void orc_psd4(float *A16) {
    Mat<4, 4> A = get<4, 4>(A16);
    eig::psd_project<4>(A, 0.0f);
    put(A16, A);
}
void orc_svd32(const float *F6, float *U6, float *S2, float *Vt4) {
    strain::Svd32 s = strain::svd(get<3, 2>(F6));
    put(U6, s.U);
    put(S2, s.S);
    put(Vt4, s.Vt);
}
void orc_strainlimit_table(const float *a2, float ghat, int kind, float *deda,
                           float *d2) {
    Vec2 dd;
    Mat2 hh;
    barrier::strainlimit_table(vec2(a2[0], a2[1]), ghat, kind, dd, hh);
    put(deda, dd);
    put(d2, hh);
}
void orc_eigen_force_hessian(const float *deda, const float *d2, const float *U6,
                             const float *S2, const float *Vt4, float eps,
                             float *f6, float *h36) {
    strain::Svd32 s;
    s.U = get<3, 2>(U6);
    s.S = get<2, 1>(S2);
    s.Vt = get<2, 2>(Vt4);
    Vec2 dd = get<2, 1>(deda);
    put(f6, strain::eigen_force(dd, s));
    put(h36, strain::eigen_hessian(dd, get<2, 2>(d2), s, eps));
}
float orc_strain_stiffness(const float *x9, const float *local81, float mass,
                           const float *S2, float limit) {
    return strain::stiffness(v3(x9), v3(x9 + 3), v3(x9 + 6), get<9, 9>(local81),
                             mass, fmaxf(S2[0], S2[1]), limit);
}
float orc_singular_minus_one_max(const float *F6) {
    return strain::singular_values_minus_one(get<3, 2>(F6)).max_coeff();
}
float orc_ccd(int kind, const float *x0, const float *x1, float offset,
              float ghat, float max_t, float eps, int *overlap) {
    accd::CcdFlag flag;
    float r;
    if (kind == 0)
        r = accd::point_triangle(v3(x0), v3(x1), v3(x0 + 3), v3(x0 + 6), v3(x0 + 9),
                                 v3(x1 + 3), v3(x1 + 6), v3(x1 + 9), offset, ghat,
                                 max_t, eps, &flag);
    else if (kind == 1)
        r = accd::point_edge(v3(x0), v3(x1), v3(x0 + 3), v3(x0 + 6), v3(x1 + 3),
                             v3(x1 + 6), offset, ghat, max_t, eps, &flag);
    else if (kind == 2)
        r = accd::point_point(v3(x0), v3(x1), v3(x0 + 3), v3(x1 + 3), offset, ghat,
                              max_t, eps, &flag);
    else
        r = accd::edge_edge(v3(x0), v3(x0 + 3), v3(x0 + 6), v3(x0 + 9), v3(x1),
                            v3(x1 + 3), v3(x1 + 6), v3(x1 + 9), offset, ghat, max_t,
                            eps, &flag);
    *overlap = flag.overlap ? 1 : 0;
    return r;
}
int orc_edge_triangle(const float *e0, const float *e1, const float *t0,
                      const float *t1, const float *t2) {
    return contact::edge_triangle_intersect(v3(e0), v3(e1), v3(t0), v3(t1), v3(t2)) ? 1 : 0;
}
void orc_invert_spd(const float *A9, float *out9, int *ok) {
    Mat3 o;
    *ok = eig::invert_spd(get<3, 3>(A9), o) ? 1 : 0;
    put(out9, o);
}

} // extern "C"
