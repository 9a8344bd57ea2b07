// oracle_solver.cpp -- CPU restatement of the per-step contact solve
// (TEST INFRASTRUCTURE: used only by tests/, the smoke check and the CPU
// baseline arm of bench.py).
//
// Follows crates/ppf-cts-solver/src/cpp/main/main.cu:267-1649 (advance):
//   trees from x_curr, inertial target (main.cu:491-511), Newton loop:
//     inertia / air / pull          energy/energy.cu:182-270
//     membrane + bending            energy/energy.cu:304-553, 718-794
//     elastic copy, strain limit    strainlimiting/strainlimiting.cu:46-98
//     contact: pair rules           contact/contact.cu:432-887
//              pair assembly        contact/contact.cu:262-354
//     sphere / floor                contact/contact.cu:1154-1381
//     Dirichlet elimination         main/main.cu:954-1049
//     block-Jacobi PCG              solver/solver.cu:357-400, 921-1383
//     rescale by max_dx             main/main.cu:1142-1188
//     CCD line search               contact/contact.cu:2095-2740
//     strain-limit line search      strainlimiting/strainlimiting.cu:247-305
//     toi accounting, final step    main/main.cu:1356-1513
//   intersection check, commit      main/main.cu:1516-1588
// Sparse blocks are kept in plain maps; loops run serially or as OpenMP
// loops whose results are combined in index order, so a run is reproducible.
#include "../ppf-contact-solver_gb300/csrc/physics/accd.cuh"
#include "../ppf-contact-solver_gb300/csrc/physics/bw.cuh"
#include "../ppf-contact-solver_gb300/csrc/physics/contact_local.cuh"
#include "../ppf-contact-solver_gb300/csrc/physics/hinge.cuh"
#include "../ppf-contact-solver_gb300/csrc/physics/strainlimit.cuh"
#include "oracle.h"

#include <algorithm>
#include <array>
#include <chrono>
#include <cmath>
#include <cstring>
#include <unordered_map>
#include <vector>

using namespace ppf;

namespace {

struct Tree {
    unsigned n = 0, root = 0;
    std::vector<unsigned> node; // 2 per node
    std::vector<float> box;     // 8 per node
};

struct Pair {
    unsigned a, b, count;
    bool friction;
};

struct StepStatsO {
    unsigned newton = 0, pcg_iters = 0, max_contacts = 0;
    float step_ms = 0.0f;
};

struct Oracle {
    PpfParamSet prm{};
    unsigned n = 0, nsurf = 0, nf = 0, ne = 0, nh = 0;
    std::vector<unsigned> face, edge, hinge;
    std::vector<PpfVertexProp> vprop;
    std::vector<PpfEdgeProp> eprop;
    std::vector<PpfFaceProp> fprop;
    std::vector<PpfHingeProp> hprop;
    std::vector<PpfVertexParam> vparam;
    std::vector<PpfEdgeParam> eparam;
    std::vector<PpfFaceParam> fparam;
    std::vector<PpfHingeParam> hparam;
    std::vector<float> inv_rest;
    std::vector<std::vector<unsigned>> vf, ve, ef;
    std::vector<unsigned> foff, fcol; // fixed upper pattern
    std::vector<PpfFixPair> fix;
    std::vector<PpfPullPair> pull;
    std::vector<PpfSphere> sphere;
    std::vector<PpfFloor> floor_;
    std::vector<float> margin_f, margin_e, margin_v;
    std::vector<float> curr, prev;
    // per Newton iteration
    std::vector<float> x, target, force, dx, diag;
    std::vector<float> fval, ftmp; // fixed values (9 per block)
    std::unordered_map<unsigned long long, Mat3> dyn;
    std::vector<Pair> pf, pe, pp, ee;
    Tree tf, te, tv;
    // static collision mesh (Constraint::mesh) and its trees, built once
    unsigned ncv = 0, ncf = 0, nce = 0;
    std::vector<float> cm_x;
    std::vector<unsigned> cm_face, cm_edge;
    std::vector<PpfVertexProp> cm_vprop;
    std::vector<PpfFaceProp> cm_fprop;
    std::vector<PpfEdgeProp> cm_eprop;
    std::vector<PpfVertexParam> cm_vparam;
    std::vector<PpfFaceParam> cm_fparam;
    std::vector<PpfEdgeParam> cm_eparam;
    std::vector<float> cm_margin_f, cm_margin_e;
    Tree tcf, tce;
    StepStatsO stats;
    // the line-search inputs of the last Newton iterations (x0: the previous
    // iterate, x1: the candidate) with their contact and strain-limit times,
    // newest last, for reproducing a failing step
    struct LsTrace {
        std::vector<float> x0, x1;
        float toi_contact, toi_strain;
    };
    std::vector<LsTrace> ls_trace;
    unsigned last_pcg_iters = 0;
    bool dirichlet = true; // eliminate fix pins after assembly (main.cu:954-1049)
    float last_pcg_resid = 0.0f;

    Vec3 X(const std::vector<float> &v, unsigned i) const {
        return vec3(v[3 * i], v[3 * i + 1], v[3 * i + 2]);
    }
    Vec3 CX(unsigned i) const { return X(cm_x, i); }
    static void point_box(const Vec3 &p, float m, float q[8]) {
        q[0] = p[0] - m; q[1] = p[1] - m; q[2] = p[2] - m; q[3] = 1.0f;
        q[4] = p[0] + m; q[5] = p[1] + m; q[6] = p[2] + m; q[7] = 0.0f;
    }
    unsigned slot(unsigned i, unsigned j) const {
        auto b = fcol.begin() + foff[i], e = fcol.begin() + foff[i + 1];
        auto it = std::lower_bound(b, e, j);
        return (it != e && *it == j) ? (unsigned)(it - fcol.begin()) : 0xFFFFFFFFu;
    }
    Mat3 fixed_block(const std::vector<float> &val, unsigned i, unsigned j) const {
        bool tr = i > j;
        unsigned s = tr ? slot(j, i) : slot(i, j);
        if (s == 0xFFFFFFFFu) return Mat3::zero();
        Mat3 m = load_mat3(&val[9 * (size_t)s]);
        return tr ? m.transpose() : m;
    }
    void add_block(unsigned i, unsigned j, const Mat3 &m) {
        unsigned s = slot(i, j);
        if (s != 0xFFFFFFFFu) {
            for (int k = 0; k < 9; ++k)
                if (m.m[k] != 0.0f) fval[9 * (size_t)s + k] += m.m[k];
        } else {
            Mat3 &d = dyn.try_emplace(((unsigned long long)i << 32) | j, Mat3::zero()).first->second;
            d += m;
        }
    }

    // ---- trees (oracle_lbvh.cpp) ----
    void build(Tree &t, int kind, unsigned count, const unsigned *prims, const float *margin,
               const std::vector<float> &x0, const std::vector<float> &x1, float e) {
        t.n = count;
        if (!count) return;
        t.node.assign(2 * (2 * count - 1), 0u);
        t.box.assign(8 * (2 * count - 1), 0.0f);
        t.root = oracle_lbvh_build(kind, x0.data(), x1.data(), (unsigned)(x0.size() / 3), prims,
                                   count, margin, e, t.node.data(), t.box.data(), nullptr);
    }
    template <class Op>
    void query(const Tree &t, const float q[8], Op &&op) const {
        if (!t.n || q[3] == 0.0f) return;
        std::vector<unsigned> st;
        st.push_back(t.root);
        while (!st.empty()) {
            unsigned id = st.back();
            st.pop_back();
            const float *b = &t.box[8 * (size_t)id];
            if (b[3] == 0.0f) continue;
            if (!(b[0] <= q[4] && b[4] >= q[0] && b[1] <= q[5] && b[5] >= q[1] &&
                  b[2] <= q[6] && b[6] >= q[2]))
                continue;
            if (t.node[2 * id + 1] == 0u) op(t.node[2 * id] - 1u);
            else {
                st.push_back(t.node[2 * id] - 1u);
                st.push_back(t.node[2 * id + 1] - 1u);
            }
        }
    }
    void trees(const std::vector<float> &x0, const std::vector<float> &x1, float e) {
        build(tf, 3, nf, face.data(), margin_f.data(), x0, x1, e);
        build(te, 2, ne, edge.data(), margin_e.data(), x0, x1, e);
        build(tv, 1, nsurf, nullptr, margin_v.data(), x0, x1, e);
    }

    bool init(const PpfDataSet *ds, const PpfParamSet *p);
    void compute_target(float dt);
    void assemble(float dt);
    void detect();
    int solve(unsigned &iters, float &resid);
    Vec3 spmv_row(const std::vector<float> &v, unsigned i,
                  const std::vector<std::vector<std::pair<unsigned, const Mat3 *>>> &dy_rows,
                  Vec3 &abssum) const;
    float line_search(unsigned &pin_bad, bool &overlap);
    float strain_line_search() const;
    bool intersection_free(const std::vector<float> &xx);
    void intersections(const std::vector<float> &xx, std::vector<std::array<unsigned, 3>> &out,
                       bool first_only);
    PpfStepResult advance();
    void set_constraint(const PpfConstraint *c);
};

bool Oracle::init(const PpfDataSet *ds, const PpfParamSet *p) {
    prm = *p;
    n = ds->vertex.curr.size;
    nsurf = ds->surface_vert_count;
    nf = ds->mesh.mesh.face.size;
    ne = ds->mesh.mesh.edge.size;
    nh = ds->mesh.mesh.hinge.size;
    const unsigned *F = (const unsigned *)ds->mesh.mesh.face.data;
    const unsigned *E = (const unsigned *)ds->mesh.mesh.edge.data;
    const unsigned *H = (const unsigned *)ds->mesh.mesh.hinge.data;
    face.assign(F, F + 3 * (size_t)nf);
    edge.assign(E, E + 2 * (size_t)ne);
    hinge.assign(H, H + 4 * (size_t)nh);
    vprop.assign(ds->prop.vertex.data, ds->prop.vertex.data + n);
    eprop.assign(ds->prop.edge.data, ds->prop.edge.data + ne);
    fprop.assign(ds->prop.face.data, ds->prop.face.data + nf);
    hprop.assign(ds->prop.hinge.data, ds->prop.hinge.data + nh);
    vparam.assign(ds->param_arrays.vertex.data, ds->param_arrays.vertex.data + ds->param_arrays.vertex.size);
    eparam.assign(ds->param_arrays.edge.data, ds->param_arrays.edge.data + ds->param_arrays.edge.size);
    fparam.assign(ds->param_arrays.face.data, ds->param_arrays.face.data + ds->param_arrays.face.size);
    hparam.assign(ds->param_arrays.hinge.data, ds->param_arrays.hinge.data + ds->param_arrays.hinge.size);
    const float *ir = (const float *)ds->inv_rest2x2.data;
    inv_rest.assign(ir, ir + 4 * (size_t)ds->inv_rest2x2.size);
    auto rows = [](const PpfVecVecU32 &v, unsigned count) {
        std::vector<std::vector<unsigned>> r(count);
        for (unsigned i = 0; i < count && i < v.size; ++i)
            r[i].assign(v.data + v.offset[i], v.data + v.offset[i + 1]);
        return r;
    };
    vf = rows(ds->mesh.neighbor.vertex.face, n);
    ve = rows(ds->mesh.neighbor.vertex.edge, n);
    ef = rows(ds->mesh.neighbor.edge.face, ne);
    foff.assign(ds->fixed_index_table.offset, ds->fixed_index_table.offset + n + 1);
    fcol.assign(ds->fixed_index_table.data, ds->fixed_index_table.data + foff[n]);
    margin_f.resize(nf);
    margin_e.resize(ne);
    margin_v.resize(n);
    for (unsigned i = 0; i < nf; ++i) {
        const PpfFaceParam &q = fparam[fprop[i].param_index];
        margin_f[i] = 0.5f * q.ghat + q.offset;
    }
    for (unsigned i = 0; i < ne; ++i) {
        const PpfEdgeParam &q = eparam[eprop[i].param_index];
        margin_e[i] = 0.5f * q.ghat + q.offset;
    }
    for (unsigned i = 0; i < n; ++i) {
        const PpfVertexParam &q = vparam[vprop[i].param_index];
        margin_v[i] = 0.5f * q.ghat + q.offset;
    }
    {
        const PpfCollisionMesh &cm = ds->constraint.mesh;
        ncv = cm.vertex.size;
        ncf = cm.face.size;
        nce = cm.edge.size;
        const float *cx = (const float *)cm.vertex.data;
        cm_x.assign(cx, cx + 3 * (size_t)ncv);
        cm_face.assign((const unsigned *)cm.face.data, (const unsigned *)cm.face.data + 3 * (size_t)ncf);
        cm_edge.assign((const unsigned *)cm.edge.data, (const unsigned *)cm.edge.data + 2 * (size_t)nce);
        cm_vprop.assign(cm.prop.vertex.data, cm.prop.vertex.data + cm.prop.vertex.size);
        cm_fprop.assign(cm.prop.face.data, cm.prop.face.data + cm.prop.face.size);
        cm_eprop.assign(cm.prop.edge.data, cm.prop.edge.data + cm.prop.edge.size);
        cm_vparam.assign(cm.param_arrays.vertex.data, cm.param_arrays.vertex.data + cm.param_arrays.vertex.size);
        cm_fparam.assign(cm.param_arrays.face.data, cm.param_arrays.face.data + cm.param_arrays.face.size);
        cm_eparam.assign(cm.param_arrays.edge.data, cm.param_arrays.edge.data + cm.param_arrays.edge.size);
        cm_margin_f.resize(ncf);
        cm_margin_e.resize(nce);
        for (unsigned i = 0; i < ncf; ++i) {
            const PpfFaceParam &q = cm_fparam[cm_fprop[i].param_index];
            cm_margin_f[i] = 0.5f * q.ghat + q.offset;
        }
        for (unsigned i = 0; i < nce; ++i) {
            const PpfEdgeParam &q = cm_eparam[cm_eprop[i].param_index];
            cm_margin_e[i] = 0.5f * q.ghat + q.offset;
        }
        // lbvh/lbvh.cu:1100-1118: static trees over the mesh as it is
        build(tcf, 3, ncf, cm_face.data(), cm_margin_f.data(), cm_x, cm_x, 1.0f);
        build(tce, 2, nce, cm_edge.data(), cm_margin_e.data(), cm_x, cm_x, 1.0f);
    }
    const float *c = (const float *)ds->vertex.curr.data;
    const float *pv = (const float *)ds->vertex.prev.data;
    curr.assign(c, c + 3 * (size_t)n);
    prev.assign(pv, pv + 3 * (size_t)n);
    set_constraint(&ds->constraint);
    if (!prm.disable_contact) {
        trees(curr, curr, 1.0f);
        if (!intersection_free(prev) || !intersection_free(curr)) return false;
    }
    return true;
}

void Oracle::set_constraint(const PpfConstraint *c) {
    fix.assign(c->fix.data, c->fix.data + c->fix.size);
    pull.assign(c->pull.data, c->pull.data + c->pull.size);
    sphere.assign(c->sphere.data, c->sphere.data + c->sphere.size);
    floor_.assign(c->floor.data, c->floor.data + c->floor.size);
    for (auto &v : vprop) v.fix_index = v.pull_index = 0;
    for (size_t i = 0; i < fix.size(); ++i) vprop[fix[i].index].fix_index = (unsigned)i + 1;
    for (size_t i = 0; i < pull.size(); ++i) vprop[pull[i].index].pull_index = (unsigned)i + 1;
    auto fx = [&](unsigned v) { return vprop[v].fix_index > 0; };
    for (unsigned i = 0; i < nf; ++i)
        fprop[i].fixed = fx(face[3 * i]) && fx(face[3 * i + 1]) && fx(face[3 * i + 2]);
    for (unsigned i = 0; i < ne; ++i) eprop[i].fixed = fx(edge[2 * i]) && fx(edge[2 * i + 1]);
    for (unsigned i = 0; i < nh; ++i)
        hprop[i].fixed = fx(hinge[4 * i]) && fx(hinge[4 * i + 1]) && fx(hinge[4 * i + 2]) &&
                         fx(hinge[4 * i + 3]);
}

void Oracle::compute_target(float dt) {
    target.resize(3 * (size_t)n);
    for (unsigned i = 0; i < n; ++i) {
        if (vprop[i].fix_index > 0) {
            for (int d = 0; d < 3; ++d) target[3 * i + d] = fix[vprop[i].fix_index - 1].position.v[d];
            continue;
        }
        float tr = dt / prm.prev_dt, h2 = dt * dt;
        for (int d = 0; d < 3; ++d) {
            float x1 = curr[3 * i + d], x0 = prev[3 * i + d];
            float y = (x1 - x0) * tr + h2 * prm.gravity.v[d];
            target[3 * i + d] = prm.inactive_momentum ? x1 : x1 + y;
        }
    }
}

// Query widening of the proximity search: the trees hold tight boxes at x;
// the guard keeps fp32 rounding of the box corners from dropping a pair at
// the distance threshold (the distance test alone decides acceptance).
static float detect_guard(const Vec3 &p) {
    return 1e-6f * (1.0f + std::fmax(std::fmax(std::fabs(p[0]), std::fabs(p[1])), std::fabs(p[2])));
}

// Contact pair detection over trees of tight boxes at x
// (contact.cu:1398-1787, stage 0).
void Oracle::detect() {
    trees(x, x, 1.0f);
    pf.clear();
    pe.clear();
    pp.clear();
    ee.clear();
    std::vector<std::vector<Pair>> lpf(nsurf), lpe(nsurf), lpp(nsurf), lee(ne);
#pragma omp parallel for schedule(dynamic, 64)
    for (long long vi = 0; vi < (long long)nsurf; ++vi) {
        unsigned v = (unsigned)vi;
        Vec3 p = X(x, v);
        float m = margin_v[v] + detect_guard(p);
        float q[8] = {p[0] - m, p[1] - m, p[2] - m, 1.0f, p[0] + m, p[1] + m, p[2] + m, 0.0f};
        const PpfVertexParam &vp = vparam[vprop[v].param_index];
        query(tf, q, [&](unsigned fi) {
            const unsigned *f = &face[3 * fi];
            bool either = vprop[v].fix_index == 0 || !fprop[fi].fixed;
            bool bc = vprop[v].collider && vprop[f[0]].collider;
            if (f[0] == v || f[1] == v || f[2] == v || !either || bc) return;
            Vec3 t0 = X(x, f[0]), t1 = X(x, f[1]), t2 = X(x, f[2]);
            Vec3 c = dist::point_triangle_coeff(p, t0, t1, t2);
            if (!(c.max_coeff() < 1.0f && c.min_coeff() > 0.0f)) return;
            Vec3 e = c[0] * (p - t0) + c[1] * (p - t1) + c[2] * (p - t2);
            const PpfFaceParam &fp = fparam[fprop[fi].param_index];
            float off = vp.offset + fp.offset, gh = 0.5f * (vp.ghat + fp.ghat);
            if (e.squared_norm() < sqr(gh + off)) lpf[v].push_back({v, fi, 1u, true});
        });
        query(te, q, [&](unsigned ei) {
            const unsigned *ed = &edge[2 * ei];
            bool either = vprop[v].fix_index == 0 || !eprop[ei].fixed;
            bool bc = vprop[v].collider && vprop[ed[0]].collider;
            if (ed[0] == v || ed[1] == v || !either || bc) return;
            Vec3 t0 = X(x, ed[0]), t1 = X(x, ed[1]);
            Vec2 c = dist::point_edge_coeff(p, t0, t1);
            if (!(c.max_coeff() < 1.0f && c.min_coeff() > 0.0f)) return;
            Vec3 e = c[0] * (p - t0) + c[1] * (p - t1);
            const PpfEdgeParam &ep = eparam[eprop[ei].param_index];
            float off = vp.offset + ep.offset, gh = 0.5f * (vp.ghat + ep.ghat);
            if (!(e.squared_norm() < sqr(gh + off))) return;
            unsigned count = 0;
            bool fr = true;
            if (!ef[ei].empty()) {
                for (unsigned fi : ef[ei]) {
                    const unsigned *f = &face[3 * fi];
                    if (f[0] == v || f[1] == v || f[2] == v) {
                        ++count;
                        fr = false;
                    } else {
                        Vec3 cf = dist::point_triangle_coeff(p, X(x, f[0]), X(x, f[1]), X(x, f[2]));
                        if (cf.max_coeff() < 1.0f && cf.min_coeff() > 0.0f) continue;
                        ++count;
                    }
                }
            } else {
                count = 1;
            }
            if (count) lpe[v].push_back({v, ei, count, fr});
        });
        query(tv, q, [&](unsigned w) {
            bool either = vprop[v].fix_index == 0 || vprop[w].fix_index == 0;
            bool bc = vprop[v].collider && vprop[w].collider;
            if (!(w < v) || !either || bc) return;
            Vec3 y = X(x, w);
            Vec3 e = p - y;
            const PpfVertexParam &wp = vparam[vprop[w].param_index];
            float off = vp.offset + wp.offset, gh = 0.5f * (vp.ghat + wp.ghat);
            if (!(e.squared_norm() < sqr(gh + off))) return;
            unsigned count = 0;
            bool fr = true;
            if (!ve[w].empty()) {
                for (unsigned ei : ve[w]) {
                    const unsigned *ed = &edge[2 * ei];
                    if (ed[0] == v || ed[1] == v) {
                        ++count;
                        fr = false;
                    } else {
                        Vec2 c = dist::point_edge_coeff(p, X(x, ed[0]), X(x, ed[1]));
                        if (c.max_coeff() < 1.0f && c.min_coeff() > 0.0f) continue;
                        ++count;
                    }
                }
                for (unsigned fi : vf[w]) {
                    const unsigned *f = &face[3 * fi];
                    if (f[0] == v || f[1] == v || f[2] == v) {
                        ++count;
                        fr = false;
                    } else {
                        Vec3 c = dist::point_triangle_coeff(p, X(x, f[0]), X(x, f[1]), X(x, f[2]));
                        if (c.max_coeff() < 1.0f && c.min_coeff() > 0.0f) continue;
                        ++count;
                    }
                }
            } else {
                count = 1;
            }
            if (count) lpp[v].push_back({v, w, count, fr});
        });
    }
#pragma omp parallel for schedule(dynamic, 64)
    for (long long eii = 0; eii < (long long)ne; ++eii) {
        unsigned ei = (unsigned)eii;
        const unsigned *a = &edge[2 * ei];
        Vec3 pa = X(x, a[0]), pb = X(x, a[1]);
        float m = margin_e[ei] + std::fmax(detect_guard(pa), detect_guard(pb));
        float q[8] = {std::fmin(pa[0], pb[0]) - m, std::fmin(pa[1], pb[1]) - m,
                      std::fmin(pa[2], pb[2]) - m, 1.0f, std::fmax(pa[0], pb[0]) + m,
                      std::fmax(pa[1], pb[1]) + m, std::fmax(pa[2], pb[2]) + m, 0.0f};
        query(te, q, [&](unsigned ej) {
            const unsigned *b = &edge[2 * ej];
            bool either = !eprop[ei].fixed || !eprop[ej].fixed;
            bool bc = vprop[a[0]].collider && vprop[b[0]].collider;
            bool shared = a[0] == b[0] || a[0] == b[1] || a[1] == b[0] || a[1] == b[1];
            if (!(ei < ej) || shared || !either || bc) return;
            Vec3 q0 = X(x, b[0]), q1 = X(x, b[1]);
            Vec4 c = dist::edge_edge_coeff(pa, pb, q0, q1);
            if (!(c.max_coeff() < 1.0f && c.min_coeff() > 0.0f)) return;
            Vec3 y0 = c[0] * pa + c[1] * pb, y1 = c[2] * q0 + c[3] * q1;
            Vec3 e = y0 - y1;
            const PpfEdgeParam &p0 = eparam[eprop[ei].param_index];
            const PpfEdgeParam &p1 = eparam[eprop[ej].param_index];
            float off = p0.offset + p1.offset, gh = 0.5f * (p0.ghat + p1.ghat);
            if (e.squared_norm() < sqr(gh + off)) lee[ei].push_back({ei, ej, 1u, true});
        });
    }
    for (unsigned v = 0; v < nsurf; ++v) {
        pf.insert(pf.end(), lpf[v].begin(), lpf[v].end());
        pe.insert(pe.end(), lpe[v].begin(), lpe[v].end());
        pp.insert(pp.end(), lpp[v].begin(), lpp[v].end());
    }
    for (unsigned e = 0; e < ne; ++e) ee.insert(ee.end(), lee[e].begin(), lee[e].end());
}

template <int N> struct LocalPair {
    unsigned idx[N];
    Mat<3, N> f;
    Mat<3 * N, 3 * N> H;
};

void Oracle::assemble(float dt) {
    const size_t n3 = 3 * (size_t)n;
    force.assign(n3, 0.0f);
    diag.assign(9 * (size_t)n, 0.0f);
    fval.assign(9 * (size_t)foff[n], 0.0f);
    dyn.clear();
    dx.assign(n3, 0.0f);
    for (unsigned i = 0; i < n; ++i)
        if (vprop[i].fix_index > 0)
            for (int d = 0; d < 3; ++d) dx[3 * i + d] = x[3 * i + d] - target[3 * i + d];
    const float dt2 = dt * dt;
    // inertia, air, pull
    for (unsigned i = 0; i < n; ++i) {
        const PpfVertexProp &vp = vprop[i];
        if (vp.fix_index != 0) continue;
        Vec3 xs = X(curr, i), y = X(x, i);
        Vec3 nrm = Vec3::zero();
        for (unsigned fi : vf[i]) {
            const unsigned *f = &face[3 * fi];
            Vec3 z0 = X(x, f[0]), z1 = X(x, f[1]), z2 = X(x, f[2]);
            nrm += cross(z1 - z0, z2 - z0);
        }
        if (nrm.squared_norm()) nrm.normalize();
        Vec3 wind = Vec3::zero();
        if (!prm.inactive_momentum) {
            float w = 0.25f * (0.5f * (1.0f + std::sin(30.0f * (float)prm.time))) + 0.75f;
            wind = w * vec3(prm.wind.v[0], prm.wind.v[1], prm.wind.v[2]);
        }
        Vec3 f = Vec3::zero();
        Mat3 H = Mat3::zero();
        if (!nrm.is_zero() && prm.air_density) {
            Vec3 z = (y - xs) - dt * wind;
            Mat3 P = Mat3::identity() - outer<3>(nrm, nrm);
            Vec3 g = (nrm * nrm.dot(z)) / dt2 + ((prm.air_friction * P) * z) / dt2;
            Mat3 h = outer<3>(nrm, nrm) / dt2 + (prm.air_friction * P) / dt2;
            f += (vp.area * prm.air_density) * g;
            H += (vp.area * prm.air_density) * h;
        }
        bool pulled = false;
        if (vp.pull_index > 0) {
            const PpfPullPair &q = pull[vp.pull_index - 1];
            f += q.weight * (y - vec3(q.position.v[0], q.position.v[1], q.position.v[2]));
            H += q.weight * Mat3::identity();
            pulled = true;
        }
        if (!pulled) {
            f += vp.mass * ((y - X(target, i)) / dt2);
            H += vp.mass * (Mat3::identity() / dt2);
        }
        if (prm.isotropic_air_friction) {
            f += (prm.isotropic_air_friction * (y - xs)) / dt2;
            H += (prm.isotropic_air_friction / dt2) * Mat3::identity();
        }
        if (prm.fix_xz && y[1] > (float)prm.fix_xz) {
            float t = std::fmin(1.0f, y[1] - (float)prm.fix_xz);
            Mat3 P = Mat3::identity();
            P(1, 1) = 0.0f;
            f += ((P * t) * vp.mass) * (y - xs) / dt2;
            H += (P * t) * vp.mass * dt2;
        }
        for (int d = 0; d < 3; ++d) force[3 * i + d] += f[d];
        for (int k = 0; k < 9; ++k) diag[9 * i + k] += H.m[k];
    }
    // membrane
    {
        std::vector<Mat3> ff(nf);
        std::vector<Mat9> hh(nf);
        std::vector<char> on(nf, 0);
#pragma omp parallel for schedule(static)
        for (long long ii = 0; ii < (long long)nf; ++ii) {
            unsigned i = (unsigned)ii;
            const PpfFaceProp &pr = fprop[i];
            if (pr.fixed || pr.rest_excluded || pr.collider) continue;
            const PpfFaceParam &fp = fparam[pr.param_index];
            if (!(fp.mu > 0.0f)) continue;
            const unsigned *f = &face[3 * i];
            Mat2 inv;
            for (int k = 0; k < 4; ++k) inv.m[k] = inv_rest[4 * i + k];
            bw::membrane(X(x, f[0]), X(x, f[1]), X(x, f[2]), inv, fp.mu, fp.lambda, pr.mass,
                         ff[i], hh[i]);
            on[i] = 1;
        }
        for (unsigned i = 0; i < nf; ++i) {
            if (!on[i]) continue;
            const unsigned *f = &face[3 * i];
            for (int a = 0; a < 3; ++a)
                for (int d = 0; d < 3; ++d) force[3 * f[a] + d] += ff[i](d, a);
            for (int a = 0; a < 3; ++a)
                for (int b = 0; b < 3; ++b)
                    if (f[a] <= f[b]) add_block(f[a], f[b], hh[i].block<3, 3>(3 * a, 3 * b));
        }
    }
    // bending
    {
        std::vector<Mat3x4> ff(nh);
        std::vector<Mat12> hh(nh);
        std::vector<char> on(nh, 0);
#pragma omp parallel for schedule(static)
        for (long long ii = 0; ii < (long long)nh; ++ii) {
            unsigned i = (unsigned)ii;
            const PpfHingeProp &pr = hprop[i];
            if (pr.fixed || pr.collider) continue;
            const PpfHingeParam &hp = hparam[pr.param_index];
            const unsigned *h = &hinge[4 * i];
            float rho = 0.0f;
            int cnt = 0;
            for (int k = 0; k < 4; ++k) {
                float a = vprop[h[k]].area;
                if (a > 0.0f) {
                    rho += vprop[h[k]].mass / a;
                    ++cnt;
                }
            }
            if (cnt > 0) rho /= cnt;
            float k = hinge::stiffness(hp.bend, hp.bend_warp, hp.bend_weft, pr.uv_edge_sin2,
                                       pr.length, pr.area, rho);
            if (!(k > 0.0f)) continue;
            hinge::force_hessian(X(x, h[2]), X(x, h[1]), X(x, h[0]), X(x, h[3]), pr.rest_angle,
                                 ff[i], hh[i]);
            ff[i] *= k;
            hh[i] *= k;
            on[i] = 1;
        }
        for (unsigned i = 0; i < nh; ++i) {
            if (!on[i]) continue;
            const unsigned *h = &hinge[4 * i];
            const unsigned r[4] = {h[2], h[1], h[0], h[3]};
            for (int a = 0; a < 4; ++a)
                for (int d = 0; d < 3; ++d) force[3 * r[a] + d] += ff[i](d, a);
            for (int a = 0; a < 4; ++a)
                for (int b = 0; b < 4; ++b)
                    if (r[a] <= r[b]) add_block(r[a], r[b], hh[i].block<3, 3>(3 * a, 3 * b));
        }
    }
    ftmp = fval;
    // strain limit
    {
        std::vector<Mat3> ff(nf);
        std::vector<Mat9> hh(nf);
        std::vector<char> on(nf, 0);
#pragma omp parallel for schedule(static)
        for (long long ii = 0; ii < (long long)nf; ++ii) {
            unsigned i = (unsigned)ii;
            const PpfFaceProp &pr = fprop[i];
            const PpfFaceParam &fp = fparam[pr.param_index];
            if (pr.fixed || pr.rest_excluded || !(fp.strainlimit > 0.0f)) continue;
            float limit = strain::effective_limit(fp.strainlimit, fp.shrink_x, fp.shrink_y);
            const unsigned *f = &face[3 * i];
            Mat2 inv;
            for (int k = 0; k < 4; ++k) inv.m[k] = inv_rest[4 * i + k];
            Mat3x2 F = bw::deformation_grad(X(x, f[0]), X(x, f[1]), X(x, f[2]), inv);
            strain::Svd32 sv;
            Mat3 de;
            Mat9 H;
            if (!strain::face_barrier(F, inv, fp.strainlimit, prm.barrier, prm.eiganalysis_eps, sv,
                                      de, H))
                continue;
            Mat9 local;
            for (int a = 0; a < 3; ++a)
                for (int b = 0; b < 3; ++b)
                    local.set_block<3, 3>(3 * a, 3 * b, fixed_block(ftmp, f[a], f[b]));
            float k = strain::stiffness(X(curr, f[0]), X(curr, f[1]), X(curr, f[2]), local,
                                        pr.mass, sv.S.max_coeff(), limit);
            ff[i] = k * de;
            hh[i] = k * H;
            on[i] = 1;
        }
        for (unsigned i = 0; i < nf; ++i) {
            if (!on[i]) continue;
            const unsigned *f = &face[3 * i];
            for (int a = 0; a < 3; ++a)
                for (int d = 0; d < 3; ++d) force[3 * f[a] + d] += ff[i](d, a);
            for (int a = 0; a < 3; ++a)
                for (int b = 0; b < 3; ++b)
                    if (f[a] <= f[b]) add_block(f[a], f[b], hh[i].block<3, 3>(3 * a, 3 * b));
        }
    }
    // contact
    if (!prm.disable_contact) {
        detect();
        stats.max_contacts = std::max(stats.max_contacts,
                                      (unsigned)(pf.size() + pe.size() + pp.size() + ee.size()));
        auto run = [&](auto tag, const std::vector<Pair> &list, int type) {
            constexpr int N = decltype(tag)::value;
            std::vector<LocalPair<N>> out(list.size());
#pragma omp parallel for schedule(static)
            for (long long kk = 0; kk < (long long)list.size(); ++kk) {
                const Pair &pr = list[kk];
                LocalPair<N> &lp = out[kk];
                float w[N];
                float ghat, offset, mu;
                bool fr = pr.friction;
                if constexpr (N == 4) {
                    if (type == 0) {
                        const unsigned *f = &face[3 * pr.b];
                        lp.idx[0] = pr.a;
                        lp.idx[1] = f[0];
                        lp.idx[2] = f[1];
                        lp.idx[3] = f[2];
                        Vec3 c = dist::point_triangle_coeff(X(x, lp.idx[0]), X(x, lp.idx[1]),
                                                            X(x, lp.idx[2]), X(x, lp.idx[3]));
                        w[0] = 1.0f;
                        w[1] = -c[0];
                        w[2] = -c[1];
                        w[3] = -c[2];
                        const PpfVertexParam &vp = vparam[vprop[pr.a].param_index];
                        const PpfFaceParam &fp = fparam[fprop[pr.b].param_index];
                        offset = vp.offset + fp.offset;
                        ghat = 0.5f * (vp.ghat + fp.ghat);
                        mu = contact::combine_friction(vp.friction, fp.friction, prm.friction_mode);
                    } else {
                        const unsigned *a = &edge[2 * pr.a];
                        const unsigned *b = &edge[2 * pr.b];
                        lp.idx[0] = a[0];
                        lp.idx[1] = a[1];
                        lp.idx[2] = b[0];
                        lp.idx[3] = b[1];
                        Vec4 c = dist::edge_edge_coeff(X(x, a[0]), X(x, a[1]), X(x, b[0]), X(x, b[1]));
                        w[0] = c[0];
                        w[1] = c[1];
                        w[2] = -c[2];
                        w[3] = -c[3];
                        const PpfEdgeParam &p0 = eparam[eprop[pr.a].param_index];
                        const PpfEdgeParam &p1 = eparam[eprop[pr.b].param_index];
                        offset = p0.offset + p1.offset;
                        ghat = 0.5f * (p0.ghat + p1.ghat);
                        mu = contact::combine_friction(p0.friction, p1.friction, prm.friction_mode);
                    }
                } else if constexpr (N == 3) {
                    const unsigned *e = &edge[2 * pr.b];
                    lp.idx[0] = pr.a;
                    lp.idx[1] = e[0];
                    lp.idx[2] = e[1];
                    Vec2 c = dist::point_edge_coeff(X(x, pr.a), X(x, e[0]), X(x, e[1]));
                    w[0] = 1.0f;
                    w[1] = -c[0];
                    w[2] = -c[1];
                    const PpfVertexParam &vp = vparam[vprop[pr.a].param_index];
                    const PpfEdgeParam &ep = eparam[eprop[pr.b].param_index];
                    offset = vp.offset + ep.offset;
                    ghat = 0.5f * (vp.ghat + ep.ghat);
                    mu = contact::combine_friction(vp.friction, ep.friction, prm.friction_mode);
                } else {
                    lp.idx[0] = pr.a;
                    lp.idx[1] = pr.b;
                    w[0] = 1.0f;
                    w[1] = -1.0f;
                    const PpfVertexParam &a = vparam[vprop[pr.a].param_index];
                    const PpfVertexParam &b = vparam[vprop[pr.b].param_index];
                    offset = a.offset + b.offset;
                    ghat = 0.5f * (a.ghat + b.ghat);
                    mu = contact::combine_friction(a.friction, b.friction, prm.friction_mode);
                }
                Vec3 xs[N], x0s[N];
                float mass[N];
                Mat<3 * N, 3 * N> local;
                for (int a = 0; a < N; ++a) {
                    xs[a] = X(x, lp.idx[a]);
                    x0s[a] = X(curr, lp.idx[a]);
                    mass[a] = vprop[lp.idx[a]].mass;
                }
                for (int a = 0; a < N; ++a)
                    for (int b = 0; b < N; ++b)
                        local.template set_block<3, 3>(3 * a, 3 * b, fixed_block(ftmp, lp.idx[a], lp.idx[b]));
                contact::pair_force_hessian<N>(xs, x0s, w, mass, local, ghat, offset, prm.barrier,
                                               fr, mu, prm.friction_eps, (float)pr.count, lp.f, lp.H);
            }
            for (auto &lp : out) {
                for (int a = 0; a < N; ++a)
                    for (int d = 0; d < 3; ++d) force[3 * lp.idx[a] + d] += lp.f(d, a);
                for (int a = 0; a < N; ++a)
                    for (int b = 0; b < N; ++b)
                        if (lp.idx[a] <= lp.idx[b])
                            add_block(lp.idx[a], lp.idx[b], lp.H.template block<3, 3>(3 * a, 3 * b));
            }
        };
        run(std::integral_constant<int, 4>{}, pf, 0);
        run(std::integral_constant<int, 3>{}, pe, 1);
        run(std::integral_constant<int, 2>{}, pp, 2);
        run(std::integral_constant<int, 4>{}, ee, 3);
    }
    // sphere / floor
    for (unsigned i = 0; i < nsurf; ++i) {
        const PpfVertexProp &vp = vprop[i];
        if (vp.fix_index > 0 || !(vp.mass > 0.0f)) continue;
        Mat3 local = fixed_block(ftmp, i, i);
        Vec3 f = Vec3::zero();
        Mat3 H = Mat3::zero();
        unsigned nc = 0;
        const float vfr = vparam[vp.param_index].friction;
        for (auto &q : sphere) {
            contact::SphereC sp{vec3(q.center.v[0], q.center.v[1], q.center.v[2]), q.ghat, q.friction,
                                q.radius, q.thickness, q.bowl, q.reverse, q.kinematic};
            nc += contact::sphere_constraint(X(x, i), X(curr, i), vp.mass, vfr, local, sp,
                                             prm.friction_mode, prm.friction_eps, f, H);
        }
        for (auto &q : floor_) {
            contact::FloorC fl{vec3(q.ground.v[0], q.ground.v[1], q.ground.v[2]), q.ghat, q.friction,
                               q.thickness, vec3(q.up.v[0], q.up.v[1], q.up.v[2]), q.kinematic};
            nc += contact::floor_constraint(X(x, i), X(curr, i), vp.mass, vfr, local, fl,
                                            prm.friction_mode, prm.friction_eps,
                                            prm.constraint_tol, f, H);
        }
        if (nc) {
            for (int d = 0; d < 3; ++d) force[3 * i + d] += f[d];
            add_block(i, i, H);
        }
    }
    // static collision mesh (contact/contact.cu:1834-1947; element math at
    // 899-1152): free vertices against its faces, its vertices against the
    // free faces, free edges against its edges; every block lands in the
    // fixed pattern
    if (!prm.disable_contact && ncv) {
        for (unsigned i = 0; i < nsurf; ++i) {
            const PpfVertexProp &vp = vprop[i];
            const PpfVertexParam &vq = vparam[vp.param_index];
            float q[8];
            point_box(X(x, i), 0.5f * vq.ghat + vq.offset, q);
            const Mat3 local = fixed_block(ftmp, i, i);
            query(tcf, q, [&](unsigned fi) {
                if (!(vp.fix_index == 0 && vp.mass > 0.0f)) return;
                const unsigned *cf = &cm_face[3 * fi];
                const PpfFaceParam &fq = cm_fparam[cm_fprop[fi].param_index];
                Vec3 f;
                Mat3 H;
                if (contact::mesh_vertex_face(
                        X(x, i), X(curr, i), vp.mass, local, CX(cf[0]), CX(cf[1]), CX(cf[2]),
                        vq.offset + fq.offset, 0.5f * (vq.ghat + fq.ghat),
                        contact::combine_friction(vq.friction, fq.friction, prm.friction_mode),
                        prm.friction_eps, f, H)) {
                    for (int d = 0; d < 3; ++d) force[3 * i + d] += f[d];
                    add_block(i, i, H);
                }
            });
        }
        for (unsigned v = 0; v < ncv; ++v) {
            const PpfVertexParam &cq = cm_vparam[cm_vprop[v].param_index];
            float q[8];
            point_box(CX(v), 0.5f * cq.ghat + cq.offset, q);
            query(tf, q, [&](unsigned fi) {
                const PpfFaceProp &fp = fprop[fi];
                if (fp.fixed || !(fp.mass > 0.0f)) return;
                const unsigned *fc = &face[3 * fi];
                const PpfFaceParam &fq = fparam[fp.param_index];
                Vec3 t[3], s[3];
                float m[3];
                Mat9 local;
                for (int a = 0; a < 3; ++a) {
                    t[a] = X(x, fc[a]);
                    s[a] = X(curr, fc[a]);
                    m[a] = vprop[fc[a]].mass;
                    for (int b = 0; b < 3; ++b)
                        local.set_block<3, 3>(3 * a, 3 * b, fixed_block(ftmp, fc[a], fc[b]));
                }
                Mat<3, 3> ff;
                Mat9 HH;
                if (contact::mesh_face_vertex(
                        CX(v), t, s, m, local, fq.offset + cq.offset, 0.5f * (fq.ghat + cq.ghat),
                        contact::combine_friction(fq.friction, cq.friction, prm.friction_mode),
                        prm.friction_eps, ff, HH)) {
                    for (int a = 0; a < 3; ++a)
                        for (int d = 0; d < 3; ++d) force[3 * fc[a] + d] += ff(d, a);
                    for (int a = 0; a < 3; ++a)
                        for (int b = 0; b < 3; ++b)
                            if (fc[a] <= fc[b]) add_block(fc[a], fc[b], HH.block<3, 3>(3 * a, 3 * b));
                }
            });
        }
        for (unsigned ei = 0; ei < ne; ++ei) {
            const PpfEdgeProp &ep = eprop[ei];
            const PpfEdgeParam &eq = eparam[ep.param_index];
            const unsigned *ed = &edge[2 * ei];
            const Vec3 a = X(x, ed[0]), b = X(x, ed[1]);
            const float m = 0.5f * eq.ghat + eq.offset;
            float q[8] = {std::fmin(a[0], b[0]) - m, std::fmin(a[1], b[1]) - m, std::fmin(a[2], b[2]) - m,
                          1.0f, std::fmax(a[0], b[0]) + m, std::fmax(a[1], b[1]) + m,
                          std::fmax(a[2], b[2]) + m, 0.0f};
            Mat6 local;
            for (int u = 0; u < 2; ++u)
                for (int w = 0; w < 2; ++w)
                    local.set_block<3, 3>(3 * u, 3 * w, fixed_block(ftmp, ed[u], ed[w]));
            query(tce, q, [&](unsigned ce) {
                if (ep.fixed || !(ep.mass > 0.0f)) return;
                const unsigned *cedge = &cm_edge[2 * ce];
                const PpfEdgeParam &cq = cm_eparam[cm_eprop[ce].param_index];
                Mat<3, 2> ff;
                Mat6 HH;
                if (contact::mesh_edge_edge(
                        a, b, X(curr, ed[0]), X(curr, ed[1]), CX(cedge[0]), CX(cedge[1]),
                        vprop[ed[0]].mass, vprop[ed[1]].mass, local, eq.offset + cq.offset,
                        0.5f * (eq.ghat + cq.ghat),
                        contact::combine_friction(eq.friction, cq.friction, prm.friction_mode),
                        prm.friction_eps, ff, HH)) {
                    for (int u = 0; u < 2; ++u)
                        for (int d = 0; d < 3; ++d) force[3 * ed[u] + d] += ff(d, u);
                    for (int u = 0; u < 2; ++u)
                        for (int w = 0; w < 2; ++w)
                            if (ed[u] <= ed[w]) add_block(ed[u], ed[w], HH.block<3, 3>(3 * u, 3 * w));
                }
            });
        }
    }
    // Dirichlet elimination
    if (dirichlet && !fix.empty()) {
        auto mask = [&](unsigned v) { return vprop[v].fix_index > 0 && vprop[v].pdrd_body_index == 0; };
        auto presc = [&](unsigned v) { return X(x, v) - X(target, v); };
        auto lift = [&](unsigned row, const Mat3 &blk, const Vec3 &pv, bool tr) {
            Vec3 c = tr ? blk.transpose() * pv : blk * pv;
            for (int d = 0; d < 3; ++d) force[3 * row + d] -= c[d];
        };
        auto elim = [&](unsigned i, unsigned j, Mat3 &blk) {
            bool mi = mask(i), mj = mask(j);
            if (mi != mj) {
                if (mj) lift(i, blk, presc(j), false);
                else lift(j, blk, presc(i), true);
            }
            if (mi || mj) blk = Mat3::zero();
        };
        for (auto &kv : dyn) elim((unsigned)(kv.first >> 32), (unsigned)kv.first, kv.second);
        for (unsigned i = 0; i < n; ++i)
            for (unsigned k = foff[i]; k < foff[i + 1]; ++k) {
                Mat3 blk = load_mat3(&fval[9 * (size_t)k]);
                elim(i, fcol[k], blk);
                store(&fval[9 * (size_t)k], blk);
            }
        for (unsigned i = 0; i < n; ++i)
            if (mask(i)) {
                for (int k = 0; k < 9; ++k) diag[9 * i + k] = (k % 4 == 0) ? 1.0f : 0.0f;
                Vec3 pv = presc(i);
                for (int d = 0; d < 3; ++d) force[3 * i + d] = pv[d];
            }
    }
    // fold the per-vertex diagonal into the fixed diagonal blocks
    for (unsigned i = 0; i < n; ++i) {
        unsigned s = slot(i, i);
        for (int k = 0; k < 9; ++k) fval[9 * (size_t)s + k] += diag[9 * i + k];
    }
}

// Row i of A v and the component-wise sum of |term| over its block terms
// (solver/solver.cu:804-884: the scale of the round-off bound on p^T A p).
Vec3 Oracle::spmv_row(const std::vector<float> &v, unsigned i,
                      const std::vector<std::vector<std::pair<unsigned, const Mat3 *>>> &rows,
                      Vec3 &abssum) const {
    Vec3 acc = Vec3::zero();
    abssum = Vec3::zero();
    for (unsigned k = foff[i]; k < foff[i + 1]; ++k) {
        Vec3 t = load_mat3(&fval[9 * (size_t)k]) * X(v, fcol[k]);
        acc += t;
        abssum += t.cwise_abs();
    }
    for (auto &e : rows[i]) {
        Vec3 t = (e.first & 0x80000000u) ? e.second->transpose() * X(v, e.first & 0x7fffffffu)
                                         : (*e.second) * X(v, e.first);
        acc += t;
        abssum += t.cwise_abs();
    }
    return acc;
}

// Block-Jacobi PCG, L1 residual against the seeded residual, checks at
// iterations 1, 5, 9, ... and every iteration once below 8 tol.
int Oracle::solve(unsigned &iters, float &resid) {
    // rows: fixed lower entries (transposed) + contact blocks, both triangles
    std::vector<std::vector<std::pair<unsigned, const Mat3 *>>> rows(n);
    std::vector<Mat3> lower_store;
    for (unsigned i = 0; i < n; ++i)
        for (unsigned k = foff[i]; k < foff[i + 1]; ++k)
            if (fcol[k] != i) lower_store.push_back(load_mat3(&fval[9 * (size_t)k]));
    size_t li = 0;
    for (unsigned i = 0; i < n; ++i)
        for (unsigned k = foff[i]; k < foff[i + 1]; ++k)
            if (fcol[k] != i) rows[fcol[k]].push_back({i | 0x80000000u, &lower_store[li++]});
    for (auto &kv : dyn) {
        unsigned i = (unsigned)(kv.first >> 32), j = (unsigned)kv.first;
        rows[i].push_back({j, &kv.second});
        rows[j].push_back({i | 0x80000000u, &kv.second});
    }
    const size_t n3 = 3 * (size_t)n;
    std::vector<Mat3> P(n);
    for (unsigned i = 0; i < n; ++i) eig::invert_spd(load_mat3(&fval[9 * (size_t)slot(i, i)]), P[i]);
    std::vector<float> r(force), z(n3), p(n3), Ap(n3);
    std::vector<float> &xx = dx;
    std::vector<float> abss(n3);
    auto spmv = [&](const std::vector<float> &v, std::vector<float> &out) {
#pragma omp parallel for schedule(static)
        for (long long ii = 0; ii < (long long)n; ++ii) {
            Vec3 ab;
            Vec3 a = spmv_row(v, (unsigned)ii, rows, ab);
            for (int d = 0; d < 3; ++d) {
                out[3 * ii + d] = a[d];
                abss[3 * ii + d] = ab[d];
            }
        }
    };
    spmv(xx, Ap);
    float err0 = 0.0f;
    for (size_t k = 0; k < n3; ++k) {
        r[k] -= Ap[k];
        err0 += std::fabs(r[k]);
    }
    if (err0 == 0.0f) {
        iters = 1;
        resid = 0.0f;
        return 0;
    }
    float rz0 = 0.0f;
    for (unsigned i = 0; i < n; ++i) {
        Vec3 zi = P[i] * X(r, i);
        for (int d = 0; d < 3; ++d) {
            z[3 * i + d] = zi[d];
            p[3 * i + d] = zi[d];
            rz0 += r[3 * i + d] * zi[d];
        }
    }
    unsigned stride = 4, next_check = 1;
    int broke = 0;
    const float tol = prm.cg_tol;
    for (unsigned iter = 1;; ++iter) {
        spmv(p, Ap);
        float pap = 0.0f, absdot = 0.0f;
        for (size_t k = 0; k < n3; ++k) {
            pap += p[k] * Ap[k];
            absdot += std::fabs(p[k]) * abss[k];
        }
        float bound = 256.0f * 1.19209290e-7f * absdot;
        float alpha = 0.0f;
        if (pap > bound) alpha = rz0 / pap;
        else if (!broke) broke = (pap < -bound || pap != pap) ? 1 : 3;
        float rz1 = 0.0f, err = 0.0f;
        for (unsigned i = 0; i < n; ++i) {
            Vec3 ri;
            for (int d = 0; d < 3; ++d) {
                size_t k = 3 * i + d;
                xx[k] += alpha * p[k];
                ri[d] = r[k] - alpha * Ap[k];
                r[k] = ri[d];
            }
            Vec3 zi = P[i] * ri;
            for (int d = 0; d < 3; ++d) {
                z[3 * i + d] = zi[d];
                rz1 += ri[d] * zi[d];
                err += std::fabs(ri[d]);
            }
        }
        float beta = rz1 / rz0;
        rz0 = rz1;
        for (size_t k = 0; k < n3; ++k) p[k] = z[k] + beta * p[k];
        bool at_cap = iter >= prm.cg_max_iter;
        if (iter == next_check || at_cap) {
            float rr = err / err0;
            iters = iter;
            resid = rr;
            if (rr < tol) return 0;
            if (broke == 3) return 1;
            if (broke == 1 || !std::isfinite(rr) || at_cap) return 2;
            if (rr < 8.0f * tol) stride = 1;
            next_check = iter + stride;
        }
    }
}

// Strain-limit line search of the shells from target to x
// (strainlimiting/strainlimiting.cu:247-305): the largest t <= T along it.
float Oracle::strain_line_search() const {
    const float T = prm.line_search_max_t;
    float sl = T;
    for (unsigned i = 0; i < nf; ++i) {
        const PpfFaceProp &pr = fprop[i];
        const PpfFaceParam &fp = fparam[pr.param_index];
        if (pr.fixed || pr.rest_excluded || !(fp.strainlimit > 0.0f)) continue;
        float limit = strain::effective_limit(fp.strainlimit, fp.shrink_x, fp.shrink_y);
        const unsigned *f = &face[3 * i];
        Mat2 inv;
        for (int k = 0; k < 4; ++k) inv.m[k] = inv_rest[4 * i + k];
        Mat3x2 F0 = bw::deformation_grad(X(target, f[0]), X(target, f[1]), X(target, f[2]), inv);
        Mat3x2 F1 = bw::deformation_grad(X(x, f[0]), X(x, f[1]), X(x, f[2]), inv);
        sl = std::fmin(sl, strain::line_search(F0, F1, limit, T));
    }
    return sl;
}

float Oracle::line_search(unsigned &pin_bad, bool &overlap) {
    const float T = prm.line_search_max_t;
    pin_bad = 0xFFFFFFFFu;
    overlap = false;
    const std::vector<float> &x0 = target; // previous iterate
    auto end_of = [&](unsigned i, float t) {
        return vec3(std::fma(t, x[3 * i] - x0[3 * i], x0[3 * i]),
                    std::fma(t, x[3 * i + 1] - x0[3 * i + 1], x0[3 * i + 1]),
                    std::fma(t, x[3 * i + 2] - x0[3 * i + 2], x0[3 * i + 2]));
    };
    std::vector<float> vtoi(nsurf, T);
    std::vector<unsigned> bad(nsurf, 0xFFFFFFFFu);
    std::vector<char> ov(nsurf, 0);
#pragma omp parallel for schedule(dynamic, 64)
    for (long long vi = 0; vi < (long long)nsurf; ++vi) {
        unsigned v = (unsigned)vi;
        const Vec3 a = X(x0, v), b = end_of(v, T);
        const PpfVertexProp &vp = vprop[v];
        float toi = T;
        // analytic colliders
        for (auto &sp : sphere) {
            if (sp.kinematic) continue;
            Vec3 c = vec3(sp.center.v[0], sp.center.v[1], sp.center.v[2]);
            Vec3 c0 = (sp.bowl && a[1] > c[1]) ? vec3(c[0], a[1], c[2]) : c;
            Vec3 c1 = (sp.bowl && b[1] > c[1]) ? vec3(c[0], b[1], c[2]) : c;
            float r0 = (a - c0).norm(), r1 = (b - c1).norm(), r = sp.radius;
            if (vp.fix_index > 0) {
                float d0 = sp.reverse ? (r - r0) : (r0 - r), d1 = sp.reverse ? (r - r1) : (r1 - r);
                if (d0 >= 0.0f && d1 < 0.0f) bad[v] = std::min(bad[v], v);
            } else if (vp.mass > 0.0f) {
                float depth0 = sp.reverse ? (r0 - r) : (r - r0);
                if (sp.thickness > 0.0f && depth0 > sp.thickness) continue;
                if ((r0 - r) * (r1 - r) <= 0.0f) toi = std::fmin(toi, T * ((r - r0) / (r1 - r0)));
            }
        }
        for (auto &fl : floor_) {
            if (fl.kinematic) continue;
            Vec3 up = vec3(fl.up.v[0], fl.up.v[1], fl.up.v[2]);
            Vec3 g = vec3(fl.ground.v[0], fl.ground.v[1], fl.ground.v[2]);
            float h0 = up.dot(a - g), h1 = up.dot(b - g);
            if (vp.fix_index > 0) {
                if (h0 >= 0.0f && h1 < 0.0f) bad[v] = std::min(bad[v], v);
            } else if (vp.mass > 0.0f) {
                if (fl.thickness > 0.0f && -h0 > fl.thickness) continue;
                if (h1 < 0.0f) toi = std::fmin(toi, T * (-h0 / (h1 - h0)));
            }
        }
        if (!prm.disable_contact) {
            float m = margin_v[v];
            float q[8] = {std::fmin(a[0], b[0]) - m, std::fmin(a[1], b[1]) - m, std::fmin(a[2], b[2]) - m,
                          1.0f, std::fmax(a[0], b[0]) + m, std::fmax(a[1], b[1]) + m,
                          std::fmax(a[2], b[2]) + m, 0.0f};
            const PpfVertexParam &pv = vparam[vp.param_index];
            query(tf, q, [&](unsigned fi) {
                const unsigned *f = &face[3 * fi];
                bool either = vp.fix_index == 0 || !fprop[fi].fixed;
                bool bc = vp.collider && vprop[f[0]].collider;
                if (!either || bc) return;
                int dup = -1;
                for (int k = 0; k < 3; ++k)
                    if (f[k] == v) {
                        dup = k;
                        break;
                    }
                accd::CcdFlag flag;
                float r;
                if (dup < 0) {
                    const PpfFaceParam &fp = fparam[fprop[fi].param_index];
                    r = accd::point_triangle(X(x0, v), X(x, v), X(x0, f[0]), X(x0, f[1]), X(x0, f[2]),
                                             X(x, f[0]), X(x, f[1]), X(x, f[2]), pv.offset + fp.offset,
                                             0.5f * (pv.ghat + fp.ghat), T, prm.ccd_eps, &flag);
                } else {
                    unsigned i0 = f[dup], j = f[(dup + 1) % 3], k = f[(dup + 2) % 3];
                    r = accd::point_edge(X(x0, i0), X(x, i0), X(x0, j), X(x0, k), X(x, j), X(x, k),
                                         2.0f * pv.offset, pv.ghat, T, prm.ccd_eps, &flag);
                }
                if (r < T) {
                    toi = std::fmin(toi, r);
                    if (r == 0.0f) ov[v] = 1;
                }
            });
            query(tv, q, [&](unsigned w) {
                bool either = vp.fix_index == 0 || vprop[w].fix_index == 0;
                bool bc = vp.collider && vprop[w].collider;
                if (!(w < v) || !either || bc) return;
                const PpfVertexParam &pw = vparam[vprop[w].param_index];
                accd::CcdFlag flag;
                float r = accd::point_point(X(x0, v), X(x, v), X(x0, w), X(x, w), pv.offset + pw.offset,
                                            0.5f * (pv.ghat + pw.ghat), T, prm.ccd_eps, &flag);
                if (r < T) {
                    toi = std::fmin(toi, r);
                    if (r == 0.0f) ov[v] = 1;
                }
            });
            // against the static collision mesh's faces (contact.cu:2596-2626)
            if (vp.fix_index == 0 && vp.mass > 0.0f)
                query(tcf, q, [&](unsigned fi) {
                    const unsigned *cf = &cm_face[3 * fi];
                    const PpfFaceParam &fp = cm_fparam[cm_fprop[fi].param_index];
                    accd::CcdFlag flag;
                    float r = accd::point_triangle(X(x0, v), X(x, v), CX(cf[0]), CX(cf[1]), CX(cf[2]),
                                                   CX(cf[0]), CX(cf[1]), CX(cf[2]), pv.offset + fp.offset,
                                                   0.5f * (pv.ghat + fp.ghat), T, prm.ccd_eps, &flag);
                    if (r < T) {
                        toi = std::fmin(toi, r);
                        if (r == 0.0f) ov[v] = 1;
                    }
                });
        }
        vtoi[v] = toi;
    }
    // the collision mesh's vertices against the free faces (contact.cu:2628-2655)
    std::vector<float> ctoi(ncv, T);
    std::vector<char> cov(ncv, 0);
    if (!prm.disable_contact) {
#pragma omp parallel for schedule(dynamic, 64)
        for (long long cvi = 0; cvi < (long long)ncv; ++cvi) {
            const unsigned cv = (unsigned)cvi;
            const PpfVertexParam &cq = cm_vparam[cm_vprop[cv].param_index];
            const Vec3 y = CX(cv);
            float q[8];
            point_box(y, 0.5f * cq.ghat + cq.offset, q);
            float toi = T;
            query(tf, q, [&](unsigned fi) {
                const PpfFaceProp &fp = fprop[fi];
                if (fp.fixed || !(fp.mass > 0.0f)) return;
                const unsigned *f = &face[3 * fi];
                const PpfFaceParam &fq = fparam[fp.param_index];
                accd::CcdFlag flag;
                float r = accd::point_triangle(y, y, X(x0, f[0]), X(x0, f[1]), X(x0, f[2]), X(x, f[0]),
                                               X(x, f[1]), X(x, f[2]), fq.offset + cq.offset,
                                               0.5f * (fq.ghat + cq.ghat), T, prm.ccd_eps, &flag);
                if (r < T) {
                    toi = std::fmin(toi, r);
                    if (r == 0.0f) cov[cv] = 1;
                }
            });
            ctoi[cv] = toi;
        }
    }
    float seed = T;
    for (unsigned v = 0; v < nsurf; ++v) {
        seed = std::fmin(seed, vtoi[v]);
        pin_bad = std::min(pin_bad, bad[v]);
        if (ov[v]) overlap = true;
    }
    for (unsigned cv = 0; cv < ncv; ++cv) {
        seed = std::fmin(seed, ctoi[cv]);
        if (cov[cv]) overlap = true;
    }
    std::vector<float> te_(ne, T);
    std::vector<char> ove(ne, 0);
    if (!prm.disable_contact) {
#pragma omp parallel for schedule(dynamic, 64)
        for (long long eii = 0; eii < (long long)ne; ++eii) {
            unsigned e = (unsigned)eii;
            const unsigned *ed = &edge[2 * e];
            float m = margin_e[e];
            Vec3 p0 = X(x0, ed[0]), p1 = X(x0, ed[1]), q0 = end_of(ed[0], seed), q1 = end_of(ed[1], seed);
            float q[8] = {std::fmin(std::fmin(p0[0], p1[0]) - m, std::fmin(q0[0], q1[0]) - m),
                          std::fmin(std::fmin(p0[1], p1[1]) - m, std::fmin(q0[1], q1[1]) - m),
                          std::fmin(std::fmin(p0[2], p1[2]) - m, std::fmin(q0[2], q1[2]) - m), 1.0f,
                          std::fmax(std::fmax(p0[0], p1[0]) + m, std::fmax(q0[0], q1[0]) + m),
                          std::fmax(std::fmax(p0[1], p1[1]) + m, std::fmax(q0[1], q1[1]) + m),
                          std::fmax(std::fmax(p0[2], p1[2]) + m, std::fmax(q0[2], q1[2]) + m), 0.0f};
            float toi = seed;
            query(te, q, [&](unsigned o) {
                const unsigned *e1 = &edge[2 * o];
                bool either = !eprop[e].fixed || !eprop[o].fixed;
                bool bc = vprop[ed[0]].collider && vprop[e1[0]].collider;
                if (!(e < o) || !either || bc) return;
                const PpfEdgeParam &pa = eparam[eprop[e].param_index];
                const PpfEdgeParam &pb = eparam[eprop[o].param_index];
                float off = pa.offset + pb.offset, gh = 0.5f * (pa.ghat + pb.ghat);
                float r = T;
                accd::CcdFlag flag;
                bool shared = ed[0] == e1[0] || ed[0] == e1[1] || ed[1] == e1[0] || ed[1] == e1[1];
                if (!shared) {
                    r = accd::edge_edge(X(x0, ed[0]), X(x0, ed[1]), X(x0, e1[0]), X(x0, e1[1]), X(x, ed[0]),
                                        X(x, ed[1]), X(x, e1[0]), X(x, e1[1]), off, gh, T, prm.ccd_eps, &flag);
                } else {
                    const unsigned ij[4][2] = {{0, 0}, {0, 1}, {1, 0}, {1, 1}};
                    for (int k = 0; k < 4; ++k) {
                        unsigned i = ij[k][0], j = ij[k][1];
                        if (ed[i] == e1[j]) {
                            unsigned i0 = ed[i], i1 = ed[1 - i], i2 = e1[1 - j];
                            float t0 = accd::point_edge(X(x0, i1), X(x, i1), X(x0, i0), X(x0, i2), X(x, i0),
                                                        X(x, i2), off, gh, T, prm.ccd_eps, &flag);
                            float t1 = accd::point_edge(X(x0, i2), X(x, i2), X(x0, i0), X(x0, i1), X(x, i0),
                                                        X(x, i1), off, gh, T, prm.ccd_eps, &flag);
                            r = std::fmin(t0, t1);
                            break;
                        }
                    }
                }
                if (r < T) {
                    toi = std::fmin(toi, r);
                    if (r == 0.0f) ove[e] = 1;
                }
            });
            // against the static collision mesh's edges (contact.cu:2697-2732)
            if (!eprop[e].fixed && eprop[e].mass > 0.0f)
                query(tce, q, [&](unsigned ce) {
                    const unsigned *c = &cm_edge[2 * ce];
                    const PpfEdgeParam &pa = eparam[eprop[e].param_index];
                    const PpfEdgeParam &pb = cm_eparam[cm_eprop[ce].param_index];
                    accd::CcdFlag flag;
                    float r = accd::edge_edge(X(x0, ed[0]), X(x0, ed[1]), CX(c[0]), CX(c[1]), X(x, ed[0]),
                                              X(x, ed[1]), CX(c[0]), CX(c[1]), pa.offset + pb.offset,
                                              0.5f * (pa.ghat + pb.ghat), T, prm.ccd_eps, &flag);
                    if (r < T) {
                        toi = std::fmin(toi, r);
                        if (r == 0.0f) ove[e] = 1;
                    }
                });
            te_[e] = toi;
        }
    }
    float toi = seed;
    for (unsigned e = 0; e < ne; ++e) {
        toi = std::fmin(toi, te_[e]);
        if (ove[e]) overlap = true;
    }
    return toi / T;
}

// Post-step intersection check over the current face / edge trees
// (contact/contact.cu:3056-3175, testers at 2762-2960). Every intersecting
// pair goes to `out` as (type, elem0, elem1) with the reference's record
// types: 0 face-edge (face, edge), 1 edge-edge (edge, earlier edge),
// 2 collision face-edge (collision face, edge). With first_only the walk
// stops after the edge that produced the first record.
void Oracle::intersections(const std::vector<float> &xx,
                           std::vector<std::array<unsigned, 3>> &out, bool first_only) {
    for (unsigned e = 0; e < ne && !(first_only && !out.empty()); ++e) {
        const unsigned *ed = &edge[2 * e];
        Vec3 a = X(xx, ed[0]), b = X(xx, ed[1]);
        float q[8] = {std::fmin(a[0], b[0]), std::fmin(a[1], b[1]), std::fmin(a[2], b[2]), 1.0f,
                      std::fmax(a[0], b[0]), std::fmax(a[1], b[1]), std::fmax(a[2], b[2]), 0.0f};
        query(tf, q, [&](unsigned fi) {
            const unsigned *f = &face[3 * fi];
            bool either = !fprop[fi].fixed || !eprop[e].fixed;
            bool nonzero = fprop[fi].mass > 0.0f || eprop[e].mass > 0.0f;
            bool bc = vprop[ed[0]].collider && vprop[f[0]].collider;
            if (!either || !nonzero || bc) return;
            for (int k = 0; k < 3; ++k)
                if (ed[0] == f[k] || ed[1] == f[k]) return;
            if (contact::edge_triangle_intersect(a, b, X(xx, f[0]), X(xx, f[1]), X(xx, f[2])))
                out.push_back({0u, fi, e});
        });
        // against the static collision mesh's faces (contact.cu:3114-3122)
        if (eprop[e].mass > 0.0f)
            query(tcf, q, [&](unsigned fi) {
                const unsigned *f = &cm_face[3 * fi];
                if (contact::edge_triangle_intersect(a, b, CX(f[0]), CX(f[1]), CX(f[2])))
                    out.push_back({2u, fi, e});
            });
        query(te, q, [&](unsigned o) {
            if (!(o < e)) return;
            const unsigned *e1 = &edge[2 * o];
            bool either = !eprop[e].fixed || !eprop[o].fixed;
            bool nonzero = eprop[e].mass > 0.0f || eprop[o].mass > 0.0f;
            bool bc = vprop[ed[0]].collider && vprop[e1[0]].collider;
            if (!either || !nonzero || bc) return;
            float off = eparam[eprop[e].param_index].offset + eparam[eprop[o].param_index].offset;
            bool shared = ed[0] == e1[0] || ed[0] == e1[1] || ed[1] == e1[0] || ed[1] == e1[1];
            bool hit = false;
            if (!shared) {
                hit = contact::edges_within_offset(a, b, X(xx, e1[0]), X(xx, e1[1]), off);
            } else {
                const unsigned ij[4][2] = {{0, 0}, {0, 1}, {1, 0}, {1, 1}};
                for (int k = 0; k < 4 && !hit; ++k) {
                    unsigned i = ij[k][0], j = ij[k][1];
                    if (ed[i] == e1[j])
                        hit = contact::shared_edges_within_offset(X(xx, ed[i]), X(xx, ed[1 - i]),
                                                                  X(xx, e1[1 - j]), off);
                }
            }
            if (hit) out.push_back({1u, e, o});
        });
    }
}

bool Oracle::intersection_free(const std::vector<float> &xx) {
    std::vector<std::array<unsigned, 3>> hits;
    intersections(xx, hits, true);
    return hits.empty();
}

PpfStepResult Oracle::advance() {
    auto t0 = std::chrono::steady_clock::now();
    PpfStepResult res{};
    res.ccd_success = res.pcg_success = res.intersection_free = true;
    res.newton_progress = res.pin_feasible = res.contact_separated = true;
    stats = StepStatsO{};
    float dt = prm.dt * prm.playback;
    if (!prm.disable_contact) trees(curr, curr, 1.0f);
    compute_target(dt);
    x = curr;
    double toi_adv = 0.0;
    unsigned step = 1;
    bool final_step = false;
    const float T = prm.line_search_max_t;
    while (true) {
        if (!final_step && prm.max_newton_steps > 0 && step >= prm.max_newton_steps) {
            res.newton_progress = false;
            return res;
        }
        if (final_step) {
            if (toi_adv < 1.0)
                for (auto &f : fix)
                    if (f.kinematic)
                        for (int d = 0; d < 3; ++d)
                            f.position.v[d] = f.position.v[d] - (1.0f - (float)toi_adv) * f.step_delta.v[d];
            dt *= (float)toi_adv;
            compute_target(dt);
        }
        assemble(dt);
        unsigned iters = 0;
        float resid = 0.0f;
        int state = solve(iters, resid);
        stats.newton++;
        stats.pcg_iters += iters;
        last_pcg_iters = iters;
        last_pcg_resid = resid;
        if (state == 2) {
            res.pcg_success = false;
            return res;
        }
        float max_dx = 0.0f;
        for (unsigned i = 0; i < n; ++i) max_dx = std::fmax(max_dx, X(dx, i).norm());
        float rescale = std::fmin(1.0f, prm.max_dx / max_dx);
        target = x;
        for (size_t k = 0; k < x.size(); ++k) x[k] = x[k] - rescale * dx[k];
        if (!prm.disable_contact) trees(target, x, T);
        unsigned bad;
        bool overlap;
        float toi = line_search(bad, overlap);
        if (bad != 0xFFFFFFFFu) {
            res.pin_feasible = false;
            return res;
        }
        if (overlap) {
            res.contact_separated = false;
            return res;
        }
        {
            const float sl = strain_line_search();
            if (ls_trace.size() >= 8) ls_trace.erase(ls_trace.begin());
            ls_trace.push_back(LsTrace{target, x, toi, sl});
            toi = std::fmin(toi, sl / T);
        }
        if (toi <= 1.19209290e-7f) {
            res.ccd_success = false;
            return res;
        }
        if (!final_step) toi_adv += std::max(0.0, 1.0 - toi_adv) * (double)(rescale * toi);
        for (size_t k = 0; k < x.size(); ++k) {
            float d = toi * (x[k] - target[k]);
            x[k] = target[k] + d;
        }
        if (final_step) break;
        if (toi_adv >= prm.target_toi && step >= prm.min_newton_steps) final_step = true;
        else {
            ++step;
            compute_target(dt);
        }
    }
    if (!prm.disable_contact) {
        trees(x, x, 1.0f);
        if (!intersection_free(x)) res.intersection_free = false;
    }
    prm.prev_dt = dt;
    prm.time += (double)(prm.prev_dt / prm.playback);
    prev = curr;
    curr = x;
    res.time = prm.time;
    stats.step_ms = std::chrono::duration<float, std::milli>(std::chrono::steady_clock::now() - t0).count();
    return res;
}

Oracle *g_oracle = nullptr;

} // namespace

extern "C" {

bool oracle_initialize(const PpfDataSet *ds, const PpfParamSet *param) {
    delete g_oracle;
    g_oracle = new Oracle();
    return g_oracle->init(ds, param);
}

void oracle_advance(PpfStepResult *result) { *result = g_oracle->advance(); }

void oracle_fetch(float *curr, float *prev) {
    std::memcpy(curr, g_oracle->curr.data(), g_oracle->curr.size() * sizeof(float));
    if (prev) std::memcpy(prev, g_oracle->prev.data(), g_oracle->prev.size() * sizeof(float));
}

double oracle_time(void) { return g_oracle->prm.time; }

// Intersection check of an arbitrary state of the initialized scene (trees
// rebuilt at x): true when free of intersections.
bool oracle_check_intersection(const float *x) {
    Oracle &o = *g_oracle;
    std::vector<float> xx(x, x + 3 * (size_t)o.n);
    o.trees(xx, xx, 1.0f);
    return o.intersection_free(xx);
}

// Every intersecting pair of an arbitrary state (trees rebuilt at x), as
// (type, elem0, elem1) triples in `out` (3 * max_count); returns the count,
// which may exceed max_count.
unsigned oracle_intersection_records(const float *x, unsigned *out, unsigned max_count) {
    Oracle &o = *g_oracle;
    std::vector<float> xx(x, x + 3 * (size_t)o.n);
    o.trees(xx, xx, 1.0f);
    std::vector<std::array<unsigned, 3>> hits;
    o.intersections(xx, hits, false);
    for (size_t k = 0; k < hits.size() && k < max_count; ++k)
        for (int d = 0; d < 3; ++d) out[3 * k + d] = hits[k][d];
    return (unsigned)hits.size();
}

void oracle_update_constraint(const PpfConstraint *c) { g_oracle->set_constraint(c); }

// Line-search record k of the last (up to 8) Newton iterations, 0 the
// newest: x0 (previous iterate), x1 (candidate), and the contact and raw
// strain-limit times of impact. Returns false past the records kept.
bool oracle_ls_trace(unsigned k, float *x0, float *x1, float *toi_contact, float *toi_strain) {
    const auto &t = g_oracle->ls_trace;
    if (k >= t.size()) return false;
    const auto &r = t[t.size() - 1 - k];
    std::memcpy(x0, r.x0.data(), r.x0.size() * sizeof(float));
    std::memcpy(x1, r.x1.data(), r.x1.size() * sizeof(float));
    *toi_contact = r.toi_contact;
    *toi_strain = r.toi_strain;
    return true;
}

void oracle_step_stats(unsigned *newton, unsigned *pcg_iters, float *step_ms) {
    *newton = g_oracle->stats.newton;
    *pcg_iters = g_oracle->stats.pcg_iters;
    *step_ms = g_oracle->stats.step_ms;
}

int oracle_newton_system(float *dx, unsigned *iters, float *resid) {
    Oracle &o = *g_oracle;
    float dt = o.prm.dt * o.prm.playback;
    if (!o.prm.disable_contact) o.trees(o.curr, o.curr, 1.0f);
    o.compute_target(dt);
    o.x = o.curr;
    o.assemble(dt);
    int st = o.solve(*iters, *resid);
    std::memcpy(dx, o.dx.data(), o.dx.size() * sizeof(float));
    return st;
}

// Sizes / copies of the system kept by oracle_newton_system, in the layout of
// ppf_debug_system (dynamic blocks sorted by row then column).
void oracle_system_sizes(unsigned *sizes) {
    Oracle &o = *g_oracle;
    sizes[0] = (unsigned)o.fcol.size();
    sizes[1] = (unsigned)o.dyn.size();
    sizes[2] = (unsigned)o.pf.size();
    sizes[3] = (unsigned)o.pe.size();
    sizes[4] = (unsigned)o.pp.size();
    sizes[5] = (unsigned)o.ee.size();
}

void oracle_system(unsigned *f_off, unsigned *f_col, float *f_val, unsigned *d_off,
                   unsigned *d_col, float *d_val, float *diag, float *force, unsigned *pf,
                   unsigned *pe, unsigned *pp, unsigned *ee) {
    Oracle &o = *g_oracle;
    if (f_off) std::memcpy(f_off, o.foff.data(), o.foff.size() * 4);
    if (f_col) std::memcpy(f_col, o.fcol.data(), o.fcol.size() * 4);
    if (f_val) std::memcpy(f_val, o.fval.data(), o.fval.size() * 4);
    std::vector<std::pair<unsigned long long, const Mat3 *>> blocks;
    for (auto &kv : o.dyn) blocks.push_back({kv.first, &kv.second});
    std::sort(blocks.begin(), blocks.end(),
              [](const auto &a, const auto &b) { return a.first < b.first; });
    if (d_off) {
        std::vector<unsigned> off(o.n + 1, 0u);
        for (auto &b : blocks) off[(unsigned)(b.first >> 32) + 1]++;
        for (unsigned i = 0; i < o.n; ++i) off[i + 1] += off[i];
        std::memcpy(d_off, off.data(), off.size() * 4);
    }
    for (size_t k = 0; k < blocks.size(); ++k) {
        if (d_col) d_col[k] = (unsigned)blocks[k].first;
        if (d_val) std::memcpy(d_val + 9 * k, blocks[k].second->m, 36);
    }
    if (diag) std::memcpy(diag, o.diag.data(), o.diag.size() * 4);
    if (force) std::memcpy(force, o.force.data(), o.force.size() * 4);
    auto put2 = [](unsigned *dst, const std::vector<Pair> &v) {
        if (!dst) return;
        for (size_t k = 0; k < v.size(); ++k) {
            dst[2 * k] = v[k].a;
            dst[2 * k + 1] = v[k].b;
        }
    };
    auto put3 = [](unsigned *dst, const std::vector<Pair> &v) {
        if (!dst) return;
        for (size_t k = 0; k < v.size(); ++k) {
            dst[3 * k] = v[k].a;
            dst[3 * k + 1] = v[k].b;
            dst[3 * k + 2] = v[k].count | (v[k].friction ? 0x80000000u : 0u);
        }
    };
    put2(pf, o.pf);
    put3(pe, o.pe);
    put3(pp, o.pp);
    put2(ee, o.ee);
}

// The first Newton system of the step at the current state, assembled and
// kept without solving; `dirichlet` = 0 keeps the fix-pin rows as assembled.
// Writes the step's target and returns dt.
float oracle_assemble_first(int dirichlet, float *target_out) {
    Oracle &o = *g_oracle;
    float dt = o.prm.dt * o.prm.playback;
    o.compute_target(dt);
    o.x = o.curr;
    o.dirichlet = dirichlet != 0;
    o.assemble(dt);
    o.dirichlet = true;
    if (target_out) std::memcpy(target_out, o.target.data(), o.target.size() * sizeof(float));
    return dt;
}

void oracle_param(PpfParamSet *out) { *out = g_oracle->prm; }

// Contact line search and strain-limit line search from x0 to x1 (trees
// swept over x0 -> x0 + T (x1 - x0)), as one Newton iteration runs them.
float oracle_line_search_at(const float *x0, const float *x1, unsigned *pin_bad, int *overlap) {
    Oracle &o = *g_oracle;
    o.target.assign(x0, x0 + 3 * (size_t)o.n);
    o.x.assign(x1, x1 + 3 * (size_t)o.n);
    o.trees(o.target, o.x, o.prm.line_search_max_t);
    bool ov = false;
    float toi = o.line_search(*pin_bad, ov);
    *overlap = ov ? 1 : 0;
    return toi;
}

float oracle_strain_line_search_at(const float *x0, const float *x1) {
    Oracle &o = *g_oracle;
    o.target.assign(x0, x0 + 3 * (size_t)o.n);
    o.x.assign(x1, x1 + 3 * (size_t)o.n);
    return o.strain_line_search();
}

} // extern "C"
