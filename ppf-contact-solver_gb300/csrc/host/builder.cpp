// builder.cpp -- host-side scene builder: meshes + materials -> DataSet.
//
// Restates, for shells, the reference driver's preparation of the DataSet:
//   mesh topology (edges, hinges, neighbor tables)   mesh.rs:66-293
//   face / vertex / hinge / edge props and params    scene.rs:1655-1840,
//                                                   builder.rs:339-1020,
//                                                   main.rs:205-250
//   inverse rest matrices (tangent-plane frame)      builder.rs:157-230
//   fixed sparsity, transpose table, slot tables     builder.rs:1244-1420
//   ParamSet defaults                                params.rs:207-289,
//                                                   builder.rs:1629-1681
#include "../../../include/ppf_gb300_scene.h"

#include <algorithm>
#include <array>
#include <cmath>
#include <cstring>
#include <map>
#include <string>
#include <unordered_map>
#include <vector>

namespace {

template <class T> void set_vec(T *&data, unsigned &size, unsigned &alloc,
                                std::vector<T> &src) {
    data = src.empty() ? nullptr : src.data();
    size = (unsigned)src.size();
    alloc = size;
}

struct VecVecStore {
    std::vector<unsigned> data;
    std::vector<unsigned> offset;
    void from(const std::vector<std::vector<unsigned>> &rows) {
        data.clear();
        offset.assign(1, 0u);
        for (auto &r : rows) {
            data.insert(data.end(), r.begin(), r.end());
            offset.push_back((unsigned)data.size());
        }
    }
    void fill(PpfVecVecU32 &v) {
        v.data = data.empty() ? nullptr : data.data();
        v.offset = offset.data();
        v.size = (unsigned)offset.size() - 1;
        v.nnz = (unsigned)data.size();
        v.nnz_allocated = v.nnz;
        v.offset_allocated = (unsigned)offset.size();
    }
};

template <class P> unsigned dedup(std::vector<P> &store, const P &p) {
    for (size_t i = 0; i < store.size(); ++i)
        if (std::memcmp(&store[i], &p, sizeof(P)) == 0) return (unsigned)i;
    store.push_back(p);
    return (unsigned)store.size() - 1;
}

struct V3 {
    float x, y, z;
};
V3 sub(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
V3 crs(V3 a, V3 b) {
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
float dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
float nrm(V3 a) { return std::sqrt(dot(a, a)); }
V3 unscale(V3 a, float s) { return {a.x / s, a.y / s, a.z / s}; }

} // namespace

struct PpfScene {
    // inputs
    std::vector<float> x;                 // 3 n
    std::vector<float> vel;               // 3 n
    std::vector<unsigned> faces;          // 3 F
    std::vector<unsigned> face_material;  // per face
    std::vector<PpfShellMaterial> materials;
    std::vector<unsigned> rods;           // 2 R, global vertex indices
    std::vector<unsigned> rod_material;   // per rod edge
    std::vector<PpfRodMaterial> rod_materials;
    std::vector<unsigned> tets;           // 4 T, global vertex indices
    std::vector<unsigned> tet_material;   // per tet
    std::vector<PpfSolidMaterial> solid_materials;
    std::vector<PpfStitch> seams;         // stitches, indices as added
    std::vector<PpfStitch> stitch;        // the DataSet's, indices in DataSet order
    std::vector<unsigned> solid_faces;    // 3 per boundary face of the solids
    std::vector<unsigned> solid_face_material;

    // vertex order of the built DataSet (mesh.rs:78-95): vpos maps an added
    // vertex to its DataSet index, vorder the reverse; identity unless a
    // solid has interior vertices, which go last
    std::vector<unsigned> vpos, vorder;
    unsigned n_interior = 0;
    std::vector<float> bx, bvel;          // positions / velocities in DataSet order
    std::vector<unsigned> bfaces, brods, btets;
    std::vector<unsigned> pin_index;
    std::vector<unsigned char> pin_kinematic;
    std::vector<std::pair<unsigned, float>> pulls;
    std::vector<PpfSphere> spheres;
    std::vector<PpfFloor> floors;
    // static collision mesh (Constraint::mesh): triangles and one contact
    // parameter set per added mesh
    std::vector<float> cm_x;
    std::vector<unsigned> cm_faces, cm_face_param;
    std::vector<PpfVertexParam> cm_params;

    // outputs
    std::vector<PpfVec3f> curr, prev;
    std::vector<PpfVec3u> face;
    std::vector<PpfVec2u> edge;
    std::vector<PpfVec4u> hinge;
    VecVecStore nb_vface, nb_vhinge, nb_vedge, nb_vrod, nb_hface, nb_eface;
    std::vector<char> type_face, type_vertex, type_hinge;
    std::vector<PpfVertexProp> vprop;
    std::vector<PpfEdgeProp> eprop;
    std::vector<PpfFaceProp> fprop;
    std::vector<PpfHingeProp> hprop;
    std::vector<PpfVertexParam> vparam;
    std::vector<PpfEdgeParam> eparam;
    std::vector<PpfFaceParam> fparam;
    std::vector<PpfHingeParam> hparam;
    std::vector<PpfMat2x2f> inv_rest;
    std::vector<PpfFixPair> fix;
    std::vector<PpfPullPair> pull;
    VecVecStore fixed_table;
    std::vector<PpfVec2u> transpose_data;
    std::vector<unsigned> transpose_offset;
    std::vector<unsigned> face_slots, hinge_slots, edge_slots, rod_bend_slots, tet_slots,
        stitch_slots;
    std::vector<PpfVec4u> tet;
    std::vector<PpfTetProp> tprop;
    std::vector<PpfTetParam> tparam;
    std::vector<PpfMat3x3f> inv_rest3;
    std::vector<PpfVec3f> cm_vertex;
    std::vector<PpfVec3u> cm_face;
    std::vector<PpfVec2u> cm_edge;
    std::vector<PpfVertexProp> cm_vprop;
    std::vector<PpfEdgeProp> cm_eprop;
    std::vector<PpfFaceProp> cm_fprop;
    std::vector<PpfVertexParam> cm_vparam;
    std::vector<PpfEdgeParam> cm_eparam;
    std::vector<PpfFaceParam> cm_fparam;
    PpfDataSet ds;
    PpfParamSet param;
    bool built = false;
};

extern "C" {

PpfScene *ppf_scene_create(void) { return new PpfScene(); }
void ppf_scene_destroy(PpfScene *s) { delete s; }
unsigned ppf_scene_vertex_count(PpfScene *s) { return (unsigned)s->x.size() / 3; }

// Host copies of curr / prev in the order the vertices were added (the
// DataSet holds a solid's interior vertices last).
void ppf_scene_positions(PpfScene *s, float *curr, float *prev) {
    const size_t n = s->curr.size();
    for (size_t i = 0; i < n && s->vpos.size() == n; ++i)
        for (int d = 0; d < 3; ++d) {
            if (curr) curr[3 * i + d] = s->curr[s->vpos[i]].v[d];
            if (prev) prev[3 * i + d] = s->prev[s->vpos[i]].v[d];
        }
}

void ppf_scene_set_positions(PpfScene *s, const float *curr, const float *prev) {
    const size_t n = s->curr.size();
    for (size_t i = 0; i < n && s->vpos.size() == n; ++i)
        for (int d = 0; d < 3; ++d) {
            if (curr) s->curr[s->vpos[i]].v[d] = curr[3 * i + d];
            if (prev) s->prev[s->vpos[i]].v[d] = prev[3 * i + d];
        }
}

void ppf_scene_default_param(PpfParamSet *p) {
    std::memset(p, 0, sizeof(*p));
    const float dt = 1e-3f;
    p->time = 0.0;
    p->air_friction = 0.2f;
    p->air_density = 1e-3f;
    p->constraint_tol = 0.01f;
    p->prev_dt = dt;
    p->dt = dt;
    p->playback = 1.0f;
    p->min_newton_steps = 0;
    p->target_toi = 0.25f;
    p->stitch_length_factor = 10.0f;
    p->cg_max_iter = 10000;
    p->cg_tol = 1e-3f;
    p->line_search_max_t = 1.25f;
    p->ccd_eps = 1e-7f;
    p->max_dx = 1.0f;
    p->eiganalysis_eps = 1e-2f;
    p->friction_eps = 1e-5f;
    p->isotropic_air_friction = 0.0f;
    p->gravity = {{0.0f, -9.8f, 0.0f}};
    p->wind = {{0.0f, 0.0f, 0.0f}};
    p->barrier = PPF_BARRIER_CUBIC;
    p->friction_mode = PPF_FRICTION_MIN;
    p->csrmat_max_nnz = 10000000u;
    p->fix_xz = 0.0f;
    p->disable_contact = false;
    p->inactive_momentum = false;
    p->precond = 0;
    p->schwarz_levels = 2;
    p->max_newton_steps = 2048;
    p->disable_pin_dof_removal = false;
}

unsigned ppf_scene_add_shell(PpfScene *s, const float *v, unsigned nv,
                             const unsigned *f, unsigned nf,
                             const PpfShellMaterial *mat) {
    unsigned base = (unsigned)s->x.size() / 3;
    s->x.insert(s->x.end(), v, v + 3 * nv);
    s->vel.insert(s->vel.end(), 3 * nv, 0.0f);
    unsigned mi = (unsigned)s->materials.size();
    s->materials.push_back(*mat);
    for (unsigned i = 0; i < 3 * nf; ++i) s->faces.push_back(base + f[i]);
    s->face_material.insert(s->face_material.end(), nf, mi);
    s->built = false;
    return base;
}

unsigned ppf_scene_add_rod(PpfScene *s, const float *v, unsigned nv, const unsigned *e,
                           unsigned ne, const PpfRodMaterial *mat) {
    unsigned base = (unsigned)s->x.size() / 3;
    s->x.insert(s->x.end(), v, v + 3 * nv);
    s->vel.insert(s->vel.end(), 3 * nv, 0.0f);
    unsigned mi = (unsigned)s->rod_materials.size();
    s->rod_materials.push_back(*mat);
    for (unsigned i = 0; i < 2 * ne; ++i) s->rods.push_back(base + e[i]);
    s->rod_material.insert(s->rod_material.end(), ne, mi);
    s->built = false;
    return base;
}

unsigned ppf_scene_add_solid(PpfScene *s, const float *v, unsigned nv, const unsigned *t,
                             unsigned nt, const PpfSolidMaterial *mat) {
    unsigned base = (unsigned)s->x.size() / 3;
    s->x.insert(s->x.end(), v, v + 3 * (size_t)nv);
    s->vel.insert(s->vel.end(), 3 * (size_t)nv, 0.0f);
    const unsigned mi = (unsigned)s->solid_materials.size();
    s->solid_materials.push_back(*mat);
    // boundary faces: the tet faces that no other tet shares, oriented away
    // from the tet's fourth vertex
    std::map<std::array<unsigned, 3>, std::pair<int, std::array<unsigned, 3>>> faces;
    for (unsigned i = 0; i < nt; ++i) {
        const unsigned a = base + t[4 * i], b = base + t[4 * i + 1], c = base + t[4 * i + 2],
                       d = base + t[4 * i + 3];
        s->tets.insert(s->tets.end(), {a, b, c, d});
        s->tet_material.push_back(mi);
        const std::array<unsigned, 3> fs[4] = {{b, c, d}, {a, d, c}, {a, b, d}, {a, c, b}};
        for (const auto &f : fs) {
            std::array<unsigned, 3> key = f;
            std::sort(key.begin(), key.end());
            auto it = faces.find(key);
            if (it == faces.end()) faces.emplace(key, std::make_pair(1, f));
            else ++it->second.first;
        }
    }
    // in tet order, so the surface is deterministic
    for (unsigned i = 0; i < nt; ++i) {
        const unsigned a = base + t[4 * i], b = base + t[4 * i + 1], c = base + t[4 * i + 2],
                       d = base + t[4 * i + 3];
        const std::array<unsigned, 3> fs[4] = {{b, c, d}, {a, d, c}, {a, b, d}, {a, c, b}};
        for (const auto &f : fs) {
            std::array<unsigned, 3> key = f;
            std::sort(key.begin(), key.end());
            if (faces[key].first != 1) continue;
            s->solid_faces.insert(s->solid_faces.end(), f.begin(), f.end());
            s->solid_face_material.push_back(mi);
        }
    }
    s->built = false;
    return base;
}

int ppf_scene_add_stitch(PpfScene *s, const unsigned *index, const float *weight,
                         float stiffness) {
    const unsigned n = (unsigned)s->x.size() / 3;
    PpfStitch st{};
    for (int k = 0; k < 6; ++k) {
        if (index[k] >= n) return -1;
        st.index.v[k] = index[k];
        st.weight.v[k] = weight[k];
    }
    st.stiffness = stiffness;
    s->seams.push_back(st);
    s->built = false;
    return 0;
}

int ppf_scene_add_rod_edges(PpfScene *s, const unsigned *e, unsigned ne,
                            const unsigned *edge_material, const PpfRodMaterial *materials,
                            unsigned n_materials) {
    const unsigned n = (unsigned)s->x.size() / 3;
    for (unsigned i = 0; i < ne; ++i)
        if (e[2 * i] >= n || e[2 * i + 1] >= n || edge_material[i] >= n_materials) return -1;
    const unsigned base = (unsigned)s->rod_materials.size();
    s->rod_materials.insert(s->rod_materials.end(), materials, materials + n_materials);
    s->rods.insert(s->rods.end(), e, e + 2 * ne);
    for (unsigned i = 0; i < ne; ++i) s->rod_material.push_back(base + edge_material[i]);
    s->built = false;
    return 0;
}

unsigned ppf_scene_add_shell_faces(PpfScene *s, const float *v, unsigned nv, const unsigned *f,
                                   unsigned nf, const unsigned *face_material,
                                   const PpfShellMaterial *materials, unsigned n_materials) {
    if (n_materials == 0 && nf > 0) return 0xFFFFFFFFu;
    for (unsigned i = 0; i < nf; ++i)
        if (face_material[i] >= n_materials) return 0xFFFFFFFFu;
    unsigned base = (unsigned)s->x.size() / 3;
    s->x.insert(s->x.end(), v, v + 3 * (size_t)nv);
    s->vel.insert(s->vel.end(), 3 * (size_t)nv, 0.0f);
    unsigned m0 = (unsigned)s->materials.size();
    s->materials.insert(s->materials.end(), materials, materials + n_materials);
    for (unsigned i = 0; i < 3 * nf; ++i) s->faces.push_back(base + f[i]);
    for (unsigned i = 0; i < nf; ++i) s->face_material.push_back(m0 + face_material[i]);
    s->built = false;
    return base;
}

void ppf_scene_set_velocity(PpfScene *s, const float *velocity) {
    std::memcpy(s->vel.data(), velocity, s->vel.size() * sizeof(float));
}

void ppf_scene_pin(PpfScene *s, const unsigned *idx, unsigned n, int kinematic) {
    for (unsigned i = 0; i < n; ++i) {
        s->pin_index.push_back(idx[i]);
        s->pin_kinematic.push_back(kinematic ? 1 : 0);
    }
}

void ppf_scene_pull(PpfScene *s, const unsigned *idx, unsigned n, float weight) {
    for (unsigned i = 0; i < n; ++i) s->pulls.push_back({idx[i], weight});
}

void ppf_scene_add_sphere(PpfScene *s, const float *c, float r, float gap,
                          float friction, int reverse, int bowl) {
    PpfSphere sp{};
    sp.center = {{c[0], c[1], c[2]}};
    sp.ghat = gap;
    sp.friction = friction;
    sp.radius = r;
    sp.thickness = 0.0f;
    sp.bowl = bowl != 0;
    sp.reverse = reverse != 0;
    sp.kinematic = false;
    s->spheres.push_back(sp);
}

void ppf_scene_add_collision_mesh(PpfScene *s, const float *v, unsigned nv, const unsigned *f,
                                  unsigned nf, float gap, float offset, float friction) {
    const unsigned base = (unsigned)s->cm_x.size() / 3;
    const unsigned param = (unsigned)s->cm_params.size();
    s->cm_x.insert(s->cm_x.end(), v, v + 3 * (size_t)nv);
    for (unsigned i = 0; i < 3 * nf; ++i) s->cm_faces.push_back(base + f[i]);
    s->cm_face_param.insert(s->cm_face_param.end(), nf, param);
    s->cm_params.push_back(PpfVertexParam{gap, offset, friction});
}

void ppf_scene_add_floor(PpfScene *s, const float *g, const float *up, float gap,
                         float friction) {
    PpfFloor fl{};
    fl.ground = {{g[0], g[1], g[2]}};
    fl.ghat = gap;
    fl.friction = friction;
    fl.thickness = 0.0f;
    fl.up = {{up[0], up[1], up[2]}};
    fl.kinematic = false;
    s->floors.push_back(fl);
}

int ppf_scene_build(PpfScene *s, const PpfParamSet *prm) {
    const unsigned n = (unsigned)s->x.size() / 3;
    s->n_interior = 0;
    // vertex order (mesh.rs:78-95): every vertex a face or rod uses, then the
    // vertices only tets use (a solid's interior), each group in added order
    {
        std::vector<char> surf(n, 0), in_tet(n, 0);
        for (unsigned v : s->faces) surf[v] = 1;
        for (unsigned v : s->solid_faces) surf[v] = 1;
        for (unsigned v : s->rods) surf[v] = 1;
        for (unsigned v : s->tets) in_tet[v] = 1;
        s->vpos.assign(n, 0u);
        s->vorder.clear();
        for (int pass = 0; pass < 2; ++pass)
            for (unsigned i = 0; i < n; ++i) {
                const bool interior = in_tet[i] && !surf[i];
                if (interior == (pass == 1)) {
                    s->vpos[i] = (unsigned)s->vorder.size();
                    s->vorder.push_back(i);
                    s->n_interior += interior ? 1u : 0u;
                }
            }
        s->bx.resize(3 * (size_t)n);
        s->bvel.resize(3 * (size_t)n);
        for (unsigned k = 0; k < n; ++k)
            for (int d = 0; d < 3; ++d) {
                s->bx[3 * k + d] = s->x[3 * s->vorder[k] + d];
                s->bvel[3 * k + d] = s->vel[3 * s->vorder[k] + d];
            }
        auto remap = [&](const std::vector<unsigned> &in, std::vector<unsigned> &out) {
            out.resize(in.size());
            for (size_t k = 0; k < in.size(); ++k) out[k] = s->vpos[in[k]];
        };
        std::vector<unsigned> all_faces(s->faces);
        all_faces.insert(all_faces.end(), s->solid_faces.begin(), s->solid_faces.end());
        remap(all_faces, s->bfaces);
        remap(s->rods, s->brods);
        remap(s->tets, s->btets);
        s->stitch = s->seams;
        for (auto &st : s->stitch)
            for (int k = 0; k < 6; ++k) st.index.v[k] = s->vpos[st.index.v[k]];
    }
    const unsigned nf_shell = (unsigned)s->faces.size() / 3;
    const unsigned nf = (unsigned)s->bfaces.size() / 3;
    const unsigned nt = (unsigned)s->btets.size() / 4;
    auto X = [&](unsigned i) { return V3{s->bx[3 * i], s->bx[3 * i + 1], s->bx[3 * i + 2]}; };
    s->param = *prm;
    const float dt = prm->dt;

    // positions
    s->curr.resize(n);
    s->prev.resize(n);
    for (unsigned i = 0; i < n; ++i)
        for (int d = 0; d < 3; ++d) {
            s->curr[i].v[d] = s->bx[3 * i + d];
            s->prev[i].v[d] = s->bx[3 * i + d] - s->bvel[3 * i + d] * dt;
        }

    // faces
    s->face.resize(nf);
    for (unsigned i = 0; i < nf; ++i)
        for (int k = 0; k < 3; ++k) s->face[i].v[k] = s->bfaces[3 * i + k];

    // edges (mesh.rs:188-229): the rod edges as given, then the face edges in
    // first-seen order with their incident faces
    const unsigned nr = (unsigned)s->brods.size() / 2;
    std::map<std::pair<unsigned, unsigned>, unsigned> edge_id;
    std::vector<std::vector<unsigned>> edge_faces(nr);
    s->edge.clear();
    for (unsigned i = 0; i < nr; ++i) s->edge.push_back({{s->brods[2 * i], s->brods[2 * i + 1]}});
    for (unsigned i = 0; i < nf; ++i)
        for (int j = 0; j < 3; ++j) {
            unsigned a = s->bfaces[3 * i + j], b = s->bfaces[3 * i + (j + 1) % 3];
            auto key = std::make_pair(std::min(a, b), std::max(a, b));
            auto it = edge_id.find(key);
            if (it == edge_id.end()) {
                edge_id[key] = (unsigned)s->edge.size();
                s->edge.push_back({{a, b}});
                edge_faces.push_back({i});
            } else if (edge_faces[it->second].size() < 2) {
                edge_faces[it->second].push_back(i);
            }
        }
    // hinges (mesh.rs:231-293): shared edge as seen in its first face, the
    // first face's opposite corner, then the second face's opposite corner;
    // edges with more than two faces carry no hinge.
    struct HingeAcc {
        unsigned e0, e1, o0, o1, f0, f1, count;
    };
    std::map<std::pair<unsigned, unsigned>, unsigned> hinge_key;
    std::vector<HingeAcc> hacc;
    for (unsigned i = 0; i < nf; ++i)
        for (int j = 0; j < 3; ++j) {
            unsigned a = s->bfaces[3 * i + j], b = s->bfaces[3 * i + (j + 1) % 3],
                     c = s->bfaces[3 * i + (j + 2) % 3];
            auto key = std::make_pair(std::min(a, b), std::max(a, b));
            auto it = hinge_key.find(key);
            if (it == hinge_key.end()) {
                hinge_key[key] = (unsigned)hacc.size();
                hacc.push_back({a, b, c, 0u, i, 0u, 1u});
            } else {
                HingeAcc &h = hacc[it->second];
                if (h.count == 1) {
                    h.o1 = c;
                    h.f1 = i;
                }
                ++h.count;
            }
        }
    s->hinge.clear();
    std::vector<std::vector<unsigned>> hinge_faces;
    for (auto &h : hacc)
        if (h.count == 2) {
            s->hinge.push_back({{h.e0, h.e1, h.o0, h.o1}});
            hinge_faces.push_back({h.f0, h.f1});
        }
    const unsigned ne = (unsigned)s->edge.size(), nh = (unsigned)s->hinge.size();

    // neighbor tables (mesh.rs:172-186)
    std::vector<std::vector<unsigned>> vf(n), vh(n), ve(n), vr(n);
    for (unsigned i = 0; i < nf; ++i)
        for (int k = 0; k < 3; ++k) vf[s->face[i].v[k]].push_back(i);
    for (unsigned i = 0; i < nh; ++i)
        for (int k = 0; k < 4; ++k) vh[s->hinge[i].v[k]].push_back(i);
    for (unsigned i = 0; i < ne; ++i)
        for (int k = 0; k < 2; ++k) ve[s->edge[i].v[k]].push_back(i);
    for (unsigned i = 0; i < nr; ++i)
        for (int k = 0; k < 2; ++k) vr[s->edge[i].v[k]].push_back(i);
    s->nb_vface.from(vf);
    s->nb_vhinge.from(vh);
    s->nb_vedge.from(ve);
    s->nb_vrod.from(vr);
    s->nb_hface.from(hinge_faces);
    s->nb_eface.from(edge_faces);
    // element types (builder.rs:1497-1518): bit 0 marks a solid's boundary
    // face, a tet vertex, and a hinge next to a solid face (no bending)
    s->type_face.assign(nf, 0);
    s->type_vertex.assign(n, 0);
    s->type_hinge.assign(nh, 0);
    for (unsigned i = nf_shell; i < nf; ++i) s->type_face[i] = 1;
    for (unsigned v : s->btets) s->type_vertex[v] = 1;
    for (unsigned i = 0; i < nh; ++i)
        for (unsigned f : hinge_faces[i])
            if (f >= nf_shell) s->type_hinge[i] = 1;

    // pins
    std::vector<char> fixed_v(n, 0);
    s->fix.clear();
    for (size_t i = 0; i < s->pin_index.size(); ++i) {
        unsigned v = s->vpos[s->pin_index[i]];
        PpfFixPair fp{};
        for (int d = 0; d < 3; ++d) fp.position.v[d] = s->bx[3 * v + d];
        fp.ghat = 1e-3f;
        fp.index = v;
        fp.kinematic = s->pin_kinematic[i] != 0;
        s->fix.push_back(fp);
        fixed_v[v] = 1;
    }
    s->pull.clear();
    for (auto &p : s->pulls) {
        PpfPullPair pp{};
        const unsigned v = s->vpos[p.first];
        for (int d = 0; d < 3; ++d) pp.position.v[d] = s->bx[3 * v + d];
        pp.weight = p.second;
        pp.index = v;
        s->pull.push_back(pp);
    }

    // face props / params (scene.rs:1655-1840)
    s->fparam.clear();
    s->fprop.assign(nf, PpfFaceProp{});
    std::vector<float> face_area(nf);
    for (unsigned i = nf_shell; i < nf; ++i) {
        // a solid's boundary face: contact parameters of its solid, no
        // membrane energy (energy.cu:748-760 runs over the shell faces only)
        const PpfSolidMaterial &m = s->solid_materials[s->solid_face_material[i - nf_shell]];
        V3 a = X(s->face[i].v[0]), b = X(s->face[i].v[1]), c = X(s->face[i].v[2]);
        const float area = 0.5f * nrm(crs(sub(b, a), sub(c, a)));
        face_area[i] = area;
        PpfFaceParam fp{};
        fp.model = m.model;
        fp.friction = m.friction;
        fp.ghat = m.contact_gap;
        fp.offset = m.contact_offset;
        fp.shrink_x = 1.0f;
        fp.shrink_y = 1.0f;
        PpfFaceProp pr{};
        pr.area = area;
        pr.mass = m.density * area;
        pr.fixed = fixed_v[s->face[i].v[0]] && fixed_v[s->face[i].v[1]] &&
                   fixed_v[s->face[i].v[2]];
        pr.param_index = dedup(s->fparam, fp);
        s->fprop[i] = pr;
    }
    for (unsigned i = 0; i < nf_shell; ++i) {
        const PpfShellMaterial &m = s->materials[s->face_material[i]];
        V3 a = X(s->face[i].v[0]), b = X(s->face[i].v[1]), c = X(s->face[i].v[2]);
        float area = 0.5f * nrm(crs(sub(b, a), sub(c, a)));
        face_area[i] = area;
        PpfFaceParam fp{};
        fp.model = m.model;
        float E = m.young_mod, nu = m.poiss_rat;
        fp.mu = E / (2.0f * (1.0f + nu));
        fp.lambda = E * nu / ((1.0f + nu) * (1.0f - 2.0f * nu));
        fp.friction = m.friction;
        fp.ghat = m.contact_gap;
        fp.offset = m.contact_offset;
        fp.bend = m.bend;
        fp.strainlimit = m.strain_limit;
        fp.shrink_x = 1.0f;
        fp.shrink_y = 1.0f;
        fp.deform_damping = m.deform_damping;
        fp.bend_damping = m.bend_damping;
        PpfFaceProp pr{};
        pr.area = area;
        pr.mass = m.density * area;
        pr.fixed = fixed_v[s->face[i].v[0]] && fixed_v[s->face[i].v[1]] &&
                   fixed_v[s->face[i].v[2]];
        pr.param_index = dedup(s->fparam, fp);
        s->fprop[i] = pr;
    }

    // rod edge props / params (scene.rs:1540-1655): mass from the initial
    // length, rest length scaled by the length factor; fixed when both ends
    // are pinned (builder.rs:409-419)
    s->eparam.clear();
    s->eprop.assign(ne, PpfEdgeProp{});
    for (unsigned i = 0; i < nr; ++i) {
        const PpfRodMaterial &m = s->rod_materials[s->rod_material[i]];
        const float len = nrm(sub(X(s->edge[i].v[1]), X(s->edge[i].v[0])));
        PpfEdgeParam ep{};
        ep.stiffness = m.young_mod;
        ep.bend = m.bend;
        ep.ghat = m.contact_gap;
        ep.offset = m.contact_offset;
        ep.friction = m.friction;
        ep.strainlimit = m.strain_limit;
        ep.bend_rest_from_geometry = m.bend_rest_from_geometry != 0;
        ep.deform_damping = m.deform_damping;
        ep.bend_damping = m.bend_damping;
        PpfEdgeProp pr{};
        pr.length = len * m.length_factor;
        pr.initial_length = len;
        pr.mass = m.density * len;
        pr.fixed = fixed_v[s->edge[i].v[0]] && fixed_v[s->edge[i].v[1]];
        pr.param_index = dedup(s->eparam, ep);
        s->eprop[i] = pr;
    }

    // vertex props (builder.rs:476-720) and params (builder.rs:780-870)
    s->vprop.assign(n, PpfVertexProp{});
    for (unsigned i = 0; i < n; ++i) s->vprop[i].rest_bend_angle = 3.14159265358979323846f;
    for (size_t i = 0; i < s->fix.size(); ++i) s->vprop[s->fix[i].index].fix_index = (unsigned)i + 1;
    for (size_t i = 0; i < s->pull.size(); ++i) s->vprop[s->pull[i].index].pull_index = (unsigned)i + 1;
    // rest bend angle of an interior rod vertex (two rod edges, no face)
    // whose edges ask for it from the initial shape (builder.rs:521-569)
    for (unsigned j = 0; j < n; ++j) {
        std::vector<unsigned> re;
        for (unsigned ei : ve[j])
            if (ei < nr) re.push_back(ei);
        if (re.size() != 2 || !vf[j].empty()) continue;
        if (!s->eparam[s->eprop[re[0]].param_index].bend_rest_from_geometry &&
            !s->eparam[s->eprop[re[1]].param_index].bend_rest_from_geometry)
            continue;
        const PpfVec2u &a = s->edge[re[0]], &b = s->edge[re[1]];
        const unsigned o0 = a.v[0] == j ? a.v[1] : a.v[0], o1 = b.v[0] == j ? b.v[1] : b.v[0];
        V3 e0 = sub(X(o0), X(j)), e1 = sub(X(o1), X(j));
        float n0 = nrm(e0), n1 = nrm(e1);
        if (n0 <= 0.0f || n1 <= 0.0f) continue;
        float c = dot(e0, e1) / (n0 * n1);
        c = std::min(1.0f, std::max(-1.0f, c));
        s->vprop[j].rest_bend_angle = std::acos(c);
    }
    for (unsigned i = 0; i < nf; ++i)
        for (int k = 0; k < 3; ++k) s->vprop[s->face[i].v[k]].area += s->fprop[i].area / 3.0f;
    // mass: shell faces (not a solid's boundary faces), rod edges, tets
    // (builder.rs:589-660)
    for (unsigned i = 0; i < nf_shell; ++i)
        for (int k = 0; k < 3; ++k) s->vprop[s->face[i].v[k]].mass += s->fprop[i].mass / 3.0f;
    for (unsigned i = 0; i < nr; ++i)
        for (int k = 0; k < 2; ++k) s->vprop[s->edge[i].v[k]].mass += s->eprop[i].mass / 2.0f;
    // tets (scene.rs:1840-1921): volume |(e0 x e1) . e2| / 6, mass density x
    // volume, Lame parameters from (E, nu); a quarter of each to its vertices
    s->tet.resize(nt);
    s->tprop.assign(nt, PpfTetProp{});
    s->tparam.clear();
    for (unsigned i = 0; i < nt; ++i) {
        const unsigned *t = &s->btets[4 * i];
        s->tet[i] = {{t[0], t[1], t[2], t[3]}};
        const PpfSolidMaterial &m = s->solid_materials[s->tet_material[i]];
        const V3 x0 = X(t[0]);
        const float vol = std::fabs(dot(crs(sub(X(t[1]), x0), sub(X(t[2]), x0)), sub(X(t[3]), x0))) / 6.0f;
        PpfTetParam tp{};
        tp.model = m.model;
        const float E = m.young_mod, nu = m.poiss_rat;
        tp.mu = E / (2.0f * (1.0f + nu));
        tp.lambda = E * nu / ((1.0f + nu) * (1.0f - 2.0f * nu));
        tp.shrink = 1.0f;
        tp.deform_damping = m.deform_damping;
        PpfTetProp pr{};
        pr.mass = m.density * vol;
        pr.volume = vol;
        pr.fixed = fixed_v[t[0]] && fixed_v[t[1]] && fixed_v[t[2]] && fixed_v[t[3]];
        pr.param_index = dedup(s->tparam, tp);
        s->tprop[i] = pr;
    }
    for (unsigned i = 0; i < nt; ++i)
        for (int k = 0; k < 4; ++k) {
            s->vprop[s->tet[i].v[k]].mass += s->tprop[i].mass / 4.0f;
            s->vprop[s->tet[i].v[k]].volume += s->tprop[i].volume / 4.0f;
        }
    s->vparam.clear();
    for (unsigned j = 0; j < n; ++j) {
        // faces weighted by area, rod edges by rest length
        float gs = 0, os = 0, fs = 0, ws = 0;
        for (unsigned fi : vf[j]) {
            const PpfFaceParam &p = s->fparam[s->fprop[fi].param_index];
            float w = s->fprop[fi].area;
            gs += w * p.ghat;
            os += w * p.offset;
            fs += w * p.friction;
            ws += w;
        }
        for (unsigned ei : ve[j]) {
            if (ei >= nr) continue;
            const PpfEdgeParam &p = s->eparam[s->eprop[ei].param_index];
            float w = s->eprop[ei].length;
            gs += w * p.ghat;
            os += w * p.offset;
            fs += w * p.friction;
            ws += w;
        }
        if (ws > 0.0f) {
            PpfVertexParam vp{gs / ws, os / ws, fs / ws};
            s->vprop[j].param_index = dedup(s->vparam, vp);
        }
    }

    // hinge props / params (builder.rs:873-1020)
    s->hparam.clear();
    s->hprop.assign(nh, PpfHingeProp{});
    for (unsigned i = 0; i < nh; ++i) {
        const PpfVec4u &h = s->hinge[i];
        float length = nrm(sub(X(h.v[0]), X(h.v[1])));
        float os = 0, gs = 0, bs = 0, ds = 0, as = 0;
        bool all_fixed = true;
        for (unsigned fi : hinge_faces[i]) {
            const PpfFaceParam &p = s->fparam[s->fprop[fi].param_index];
            float a = s->fprop[fi].area;
            all_fixed = all_fixed && s->fprop[fi].fixed;
            os += a * p.offset;
            gs += a * p.ghat;
            bs += a * p.bend;
            ds += a * p.bend_damping;
            as += a;
        }
        PpfHingeParam hp{};
        hp.bend = all_fixed ? 0.0f : bs / as;
        hp.bend_damping = all_fixed ? 0.0f : ds / as;
        hp.ghat = gs / as;
        hp.offset = os / as;
        PpfHingeProp pr{};
        pr.length = length;
        pr.area = as;
        pr.rest_angle = 0.0f;
        pr.uv_edge_sin2 = -1.0f;
        pr.fixed = fixed_v[h.v[0]] && fixed_v[h.v[1]] && fixed_v[h.v[2]] && fixed_v[h.v[3]];
        pr.collider = false;
        pr.param_index = dedup(s->hparam, hp);
        s->hprop[i] = pr;
    }

    // face-edge props (main.rs:205-250): zero mass, area-averaged contact
    for (unsigned i = nr; i < ne; ++i) {
        float gs = 0, os = 0, fs = 0, as = 0;
        for (unsigned fi : edge_faces[i]) {
            const PpfFaceParam &p = s->fparam[s->fprop[fi].param_index];
            float a = face_area[fi];
            gs += a * p.ghat;
            os += a * p.offset;
            fs += a * p.friction;
            as += a;
        }
        PpfEdgeParam ep{};
        ep.ghat = gs / as;
        ep.offset = os / as;
        ep.friction = fs / as;
        PpfEdgeProp pr{};
        pr.length = nrm(sub(X(s->edge[i].v[0]), X(s->edge[i].v[1])));
        pr.initial_length = pr.length;
        pr.mass = 0.0f;
        pr.fixed = fixed_v[s->edge[i].v[0]] && fixed_v[s->edge[i].v[1]];
        pr.param_index = dedup(s->eparam, ep);
        s->eprop[i] = pr;
    }

    // inverse rest matrices of the tets: [x1-x0, x2-x0, x3-x0]^-1 (builder.rs:
    // 232-262, shrink 1), by cofactors, column-major
    s->inv_rest3.resize(nt);
    for (unsigned i = 0; i < nt; ++i) {
        const unsigned *t = &s->btets[4 * i];
        const V3 x0 = X(t[0]);
        const V3 c[3] = {sub(X(t[1]), x0), sub(X(t[2]), x0), sub(X(t[3]), x0)};
        // m(r, k) = c[k] component r
        auto m = [&](int r, int k) { return r == 0 ? c[k].x : r == 1 ? c[k].y : c[k].z; };
        const float det = m(0, 0) * (m(1, 1) * m(2, 2) - m(1, 2) * m(2, 1)) -
                          m(0, 1) * (m(1, 0) * m(2, 2) - m(1, 2) * m(2, 0)) +
                          m(0, 2) * (m(1, 0) * m(2, 1) - m(1, 1) * m(2, 0));
        if (!(std::fabs(det) > 0.0f)) return 1;
        PpfMat3x3f inv;
        for (int r = 0; r < 3; ++r)
            for (int k = 0; k < 3; ++k) {
                // inverse(r, k) = cofactor(k, r) / det
                const int r1 = (k + 1) % 3, r2 = (k + 2) % 3, c1 = (r + 1) % 3, c2 = (r + 2) % 3;
                inv.m[r + 3 * k] = (m(r1, c1) * m(r2, c2) - m(r1, c2) * m(r2, c1)) / det;
            }
        s->inv_rest3[i] = inv;
    }
    // inverse rest matrices in the face's tangent frame (builder.rs:157-230),
    // shell faces only
    s->inv_rest.resize(nf_shell);
    for (unsigned i = 0; i < nf_shell; ++i) {
        V3 x0 = X(s->face[i].v[0]), x1 = X(s->face[i].v[1]), x2 = X(s->face[i].v[2]);
        V3 d0 = sub(x1, x0), d1 = sub(x2, x0);
        V3 nn = crs(d0, d1);
        // normalize divides by the norm (nalgebra's normalize), which rounds
        // differently from multiplying by its reciprocal
        V3 e2 = crs(nn, d0);
        e2 = unscale(e2, nrm(e2));
        V3 e1 = unscale(d0, nrm(d0));
        float a = dot(e1, d0), b = dot(e1, d1), c = dot(e2, d0), d = dot(e2, d1);
        float det = a * d - c * b;
        if (!(std::fabs(det) > 0.0f)) return 1;
        PpfMat2x2f inv;
        // column-major [[d, -b], [-c, a]] / det
        inv.m[0] = d / det;
        inv.m[1] = -c / det;
        inv.m[2] = -b / det;
        inv.m[3] = a / det;
        s->inv_rest[i] = inv;
    }

    // fixed sparsity: diagonal, edge, face and hinge stencils, upper triangle
    // sorted by column (builder.rs:1244-1340)
    std::vector<std::vector<unsigned>> rows(n);
    auto insert = [&](unsigned i, unsigned j) {
        if (i > j) return;
        auto &r = rows[i];
        auto it = std::lower_bound(r.begin(), r.end(), j);
        if (it == r.end() || *it != j) r.insert(it, j);
    };
    for (unsigned i = 0; i < n; ++i) insert(i, i);
    for (auto &e : s->edge)
        for (int a = 0; a < 2; ++a)
            for (int b = 0; b < 2; ++b) insert(e.v[a], e.v[b]);
    for (auto &f : s->face)
        for (int a = 0; a < 3; ++a)
            for (int b = 0; b < 3; ++b) insert(f.v[a], f.v[b]);
    for (auto &h : s->hinge)
        for (int a = 0; a < 4; ++a)
            for (int b = 0; b < 4; ++b) insert(h.v[a], h.v[b]);
    for (auto &t : s->tet)
        for (int a = 0; a < 4; ++a)
            for (int b = 0; b < 4; ++b) insert(t.v[a], t.v[b]);
    for (auto &st : s->stitch) // builder.rs:1314-1320
        for (int a = 0; a < 6; ++a)
            for (int b = 0; b < 6; ++b) insert(st.index.v[a], st.index.v[b]);
    // rod-bend stencil (j, i, k) of every vertex with two edges and no face
    // (builder.rs:1289-1313)
    std::vector<std::array<unsigned, 3>> bend_stencil(n, {{0xFFFFFFFFu, 0u, 0u}});
    for (unsigned i = 0; i < n; ++i) {
        if (ve[i].size() != 2 || !vf[i].empty()) continue;
        const PpfVec2u &a = s->edge[ve[i][0]], &b = s->edge[ve[i][1]];
        const unsigned j = a.v[0] == i ? a.v[1] : a.v[0], k = b.v[0] == i ? b.v[1] : b.v[0];
        bend_stencil[i] = {{j, i, k}};
        for (unsigned x : bend_stencil[i])
            for (unsigned y : bend_stencil[i]) insert(x, y);
    }
    s->fixed_table.from(rows);
    std::vector<std::vector<PpfVec2u>> tr(n);
    unsigned base = 0;
    for (unsigned i = 0; i < n; ++i) {
        for (size_t k = 0; k < rows[i].size(); ++k)
            if (rows[i][k] != i) tr[rows[i][k]].push_back({{i, base + (unsigned)k}});
        base += (unsigned)rows[i].size();
    }
    s->transpose_data.clear();
    s->transpose_offset.assign(1, 0u);
    for (auto &r : tr) {
        s->transpose_data.insert(s->transpose_data.end(), r.begin(), r.end());
        s->transpose_offset.push_back((unsigned)s->transpose_data.size());
    }
    auto slot_of = [&](unsigned i, unsigned j) -> unsigned {
        if (i > j) return 0xFFFFFFFFu;
        auto &r = rows[i];
        auto it = std::lower_bound(r.begin(), r.end(), j);
        return s->fixed_table.offset[i] + (unsigned)(it - r.begin());
    };
    s->face_slots.clear();
    for (auto &f : s->face)
        for (int a = 0; a < 3; ++a)
            for (int b = 0; b < 3; ++b) s->face_slots.push_back(slot_of(f.v[a], f.v[b]));
    s->hinge_slots.clear();
    for (auto &h : s->hinge) {
        unsigned r[4] = {h.v[2], h.v[1], h.v[0], h.v[3]}; // remapped order
        for (int a = 0; a < 4; ++a)
            for (int b = 0; b < 4; ++b) s->hinge_slots.push_back(slot_of(r[a], r[b]));
    }
    s->stitch_slots.clear();
    for (auto &st : s->stitch)
        for (int a = 0; a < 6; ++a)
            for (int b = 0; b < 6; ++b)
                s->stitch_slots.push_back(slot_of(st.index.v[a], st.index.v[b]));
    s->tet_slots.clear();
    for (auto &t : s->tet)
        for (int a = 0; a < 4; ++a)
            for (int b = 0; b < 4; ++b) s->tet_slots.push_back(slot_of(t.v[a], t.v[b]));
    // rod edges: 4 blocks each; rod-bend stencils: 9 per vertex (sentinels
    // where a vertex has none), builder.rs:1424-1466
    s->edge_slots.clear();
    for (unsigned i = 0; i < nr; ++i)
        for (int a = 0; a < 2; ++a)
            for (int b = 0; b < 2; ++b)
                s->edge_slots.push_back(slot_of(s->edge[i].v[a], s->edge[i].v[b]));
    s->rod_bend_slots.assign(nr ? 9 * (size_t)n : 0, 0xFFFFFFFFu);
    if (nr)
        for (unsigned i = 0; i < n; ++i) {
            if (bend_stencil[i][0] == 0xFFFFFFFFu) continue;
            for (int a = 0; a < 3; ++a)
                for (int b = 0; b < 3; ++b)
                    s->rod_bend_slots[9 * (size_t)i + 3 * a + b] =
                        slot_of(bend_stencil[i][a], bend_stencil[i][b]);
        }

    // assemble the DataSet view
    PpfDataSet &ds = s->ds;
    std::memset(&ds, 0, sizeof(ds));
    set_vec(ds.vertex.prev.data, ds.vertex.prev.size, ds.vertex.prev.allocated, s->prev);
    set_vec(ds.vertex.curr.data, ds.vertex.curr.size, ds.vertex.curr.allocated, s->curr);
    set_vec(ds.mesh.mesh.face.data, ds.mesh.mesh.face.size, ds.mesh.mesh.face.allocated, s->face);
    set_vec(ds.mesh.mesh.hinge.data, ds.mesh.mesh.hinge.size, ds.mesh.mesh.hinge.allocated, s->hinge);
    set_vec(ds.mesh.mesh.edge.data, ds.mesh.mesh.edge.size, ds.mesh.mesh.edge.allocated, s->edge);
    s->nb_vface.fill(ds.mesh.neighbor.vertex.face);
    s->nb_vhinge.fill(ds.mesh.neighbor.vertex.hinge);
    s->nb_vedge.fill(ds.mesh.neighbor.vertex.edge);
    s->nb_vrod.fill(ds.mesh.neighbor.vertex.rod);
    s->nb_hface.fill(ds.mesh.neighbor.hinge.face);
    s->nb_eface.fill(ds.mesh.neighbor.edge.face);
    set_vec(ds.mesh.type.face.data, ds.mesh.type.face.size, ds.mesh.type.face.allocated, s->type_face);
    set_vec(ds.mesh.type.vertex.data, ds.mesh.type.vertex.size, ds.mesh.type.vertex.allocated, s->type_vertex);
    set_vec(ds.mesh.type.hinge.data, ds.mesh.type.hinge.size, ds.mesh.type.hinge.allocated, s->type_hinge);
    set_vec(ds.prop.vertex.data, ds.prop.vertex.size, ds.prop.vertex.allocated, s->vprop);
    set_vec(ds.prop.edge.data, ds.prop.edge.size, ds.prop.edge.allocated, s->eprop);
    set_vec(ds.prop.face.data, ds.prop.face.size, ds.prop.face.allocated, s->fprop);
    set_vec(ds.prop.hinge.data, ds.prop.hinge.size, ds.prop.hinge.allocated, s->hprop);
    set_vec(ds.param_arrays.vertex.data, ds.param_arrays.vertex.size, ds.param_arrays.vertex.allocated, s->vparam);
    set_vec(ds.param_arrays.edge.data, ds.param_arrays.edge.size, ds.param_arrays.edge.allocated, s->eparam);
    set_vec(ds.param_arrays.face.data, ds.param_arrays.face.size, ds.param_arrays.face.allocated, s->fparam);
    set_vec(ds.param_arrays.hinge.data, ds.param_arrays.hinge.size, ds.param_arrays.hinge.allocated, s->hparam);
    set_vec(ds.inv_rest2x2.data, ds.inv_rest2x2.size, ds.inv_rest2x2.allocated, s->inv_rest);
    set_vec(ds.constraint.fix.data, ds.constraint.fix.size, ds.constraint.fix.allocated, s->fix);
    set_vec(ds.constraint.pull.data, ds.constraint.pull.size, ds.constraint.pull.allocated, s->pull);
    set_vec(ds.constraint.sphere.data, ds.constraint.sphere.size, ds.constraint.sphere.allocated, s->spheres);
    set_vec(ds.constraint.floor.data, ds.constraint.floor.size, ds.constraint.floor.allocated, s->floors);
    // collision mesh (builder.rs:1823-1935): vertices, faces, the edges in
    // first-seen order; every element takes its mesh's contact parameters
    // (one set per mesh: the reference's area-weighted averages of equal
    // values), props carry no mass
    {
        const unsigned ncv = (unsigned)s->cm_x.size() / 3, ncf = (unsigned)s->cm_faces.size() / 3;
        s->cm_vertex.resize(ncv);
        for (unsigned i = 0; i < ncv; ++i)
            s->cm_vertex[i] = {{s->cm_x[3 * i], s->cm_x[3 * i + 1], s->cm_x[3 * i + 2]}};
        s->cm_face.resize(ncf);
        s->cm_edge.clear();
        s->cm_fprop.assign(ncf, PpfFaceProp{});
        s->cm_fparam.clear();
        s->cm_eprop.clear();
        s->cm_eparam.clear();
        s->cm_vparam = s->cm_params;
        s->cm_vprop.assign(ncv, PpfVertexProp{});
        std::map<std::pair<unsigned, unsigned>, unsigned> cm_edge_id;
        for (const PpfVertexParam &p : s->cm_params) {
            PpfFaceParam fp{};
            fp.model = PPF_MODEL_BARAFF_WITKIN;
            fp.ghat = p.ghat;
            fp.offset = p.offset;
            fp.friction = p.friction;
            s->cm_fparam.push_back(fp);
            PpfEdgeParam ep{};
            ep.ghat = p.ghat;
            ep.offset = p.offset;
            ep.friction = p.friction;
            s->cm_eparam.push_back(ep);
        }
        for (unsigned i = 0; i < ncf; ++i) {
            const unsigned *t = &s->cm_faces[3 * i];
            const unsigned param = s->cm_face_param[i];
            s->cm_face[i] = {{t[0], t[1], t[2]}};
            s->cm_fprop[i].param_index = param;
            for (int k = 0; k < 3; ++k) {
                s->cm_vprop[t[k]].param_index = param;
                s->cm_vprop[t[k]].rest_bend_angle = 3.14159265358979f;
                const unsigned a = std::min(t[k], t[(k + 1) % 3]), b = std::max(t[k], t[(k + 1) % 3]);
                if (cm_edge_id.emplace(std::make_pair(a, b), (unsigned)s->cm_edge.size()).second) {
                    s->cm_edge.push_back({{a, b}});
                    PpfEdgeProp ep{};
                    ep.param_index = param;
                    s->cm_eprop.push_back(ep);
                }
            }
        }
        PpfCollisionMesh &cm = ds.constraint.mesh;
        set_vec(cm.vertex.data, cm.vertex.size, cm.vertex.allocated, s->cm_vertex);
        set_vec(cm.face.data, cm.face.size, cm.face.allocated, s->cm_face);
        set_vec(cm.edge.data, cm.edge.size, cm.edge.allocated, s->cm_edge);
        set_vec(cm.prop.vertex.data, cm.prop.vertex.size, cm.prop.vertex.allocated, s->cm_vprop);
        set_vec(cm.prop.face.data, cm.prop.face.size, cm.prop.face.allocated, s->cm_fprop);
        set_vec(cm.prop.edge.data, cm.prop.edge.size, cm.prop.edge.allocated, s->cm_eprop);
        set_vec(cm.param_arrays.vertex.data, cm.param_arrays.vertex.size,
                cm.param_arrays.vertex.allocated, s->cm_vparam);
        set_vec(cm.param_arrays.face.data, cm.param_arrays.face.size,
                cm.param_arrays.face.allocated, s->cm_fparam);
        set_vec(cm.param_arrays.edge.data, cm.param_arrays.edge.size,
                cm.param_arrays.edge.allocated, s->cm_eparam);
    }
    s->fixed_table.fill(ds.fixed_index_table);
    ds.transpose_table.data = s->transpose_data.empty() ? nullptr : s->transpose_data.data();
    ds.transpose_table.offset = s->transpose_offset.data();
    ds.transpose_table.size = n;
    ds.transpose_table.nnz = (unsigned)s->transpose_data.size();
    ds.transpose_table.nnz_allocated = ds.transpose_table.nnz;
    ds.transpose_table.offset_allocated = n + 1;
    ds.rod_count = nr;
    ds.shell_face_count = nf_shell;
    ds.surface_vert_count = n - s->n_interior;
    set_vec(ds.mesh.mesh.tet.data, ds.mesh.mesh.tet.size, ds.mesh.mesh.tet.allocated, s->tet);
    set_vec(ds.prop.tet.data, ds.prop.tet.size, ds.prop.tet.allocated, s->tprop);
    set_vec(ds.param_arrays.tet.data, ds.param_arrays.tet.size, ds.param_arrays.tet.allocated,
            s->tparam);
    set_vec(ds.inv_rest3x3.data, ds.inv_rest3x3.size, ds.inv_rest3x3.allocated, s->inv_rest3);
    set_vec(ds.tet_hess_slots.data, ds.tet_hess_slots.size, ds.tet_hess_slots.allocated,
            s->tet_slots);
    set_vec(ds.constraint.stitch.data, ds.constraint.stitch.size, ds.constraint.stitch.allocated,
            s->stitch);
    set_vec(ds.stitch_hess_slots.data, ds.stitch_hess_slots.size,
            ds.stitch_hess_slots.allocated, s->stitch_slots);
    set_vec(ds.face_hess_slots.data, ds.face_hess_slots.size, ds.face_hess_slots.allocated, s->face_slots);
    set_vec(ds.hinge_hess_slots.data, ds.hinge_hess_slots.size, ds.hinge_hess_slots.allocated, s->hinge_slots);
    set_vec(ds.edge_hess_slots.data, ds.edge_hess_slots.size, ds.edge_hess_slots.allocated, s->edge_slots);
    set_vec(ds.rod_bend_hess_slots.data, ds.rod_bend_hess_slots.size,
            ds.rod_bend_hess_slots.allocated, s->rod_bend_slots);
    s->built = true;
    return 0;
}

PpfDataSet *ppf_scene_dataset(PpfScene *s) { return s->built ? &s->ds : nullptr; }
PpfParamSet *ppf_scene_param(PpfScene *s) { return s->built ? &s->param : nullptr; }
PpfConstraint *ppf_scene_constraint(PpfScene *s) {
    return s->built ? &s->ds.constraint : nullptr;
}

// Byte size of a named array of the built scene, copied to `out` when it is
// not NULL; (size_t)-1 for an unknown name or an unbuilt scene.
size_t ppf_scene_array(PpfScene *s, const char *name, void *out) {
    if (!s->built || !name) return (size_t)-1;
    std::vector<float> tmp;
    const void *src = nullptr;
    size_t bytes = 0;
    auto take = [&](const auto &v) {
        src = v.data();
        bytes = v.size() * sizeof(v[0]);
    };
    auto per = [&](const auto &props, auto get) {
        tmp.resize(props.size());
        for (size_t i = 0; i < props.size(); ++i) tmp[i] = get(props[i]);
        take(tmp);
    };
    const std::string n(name);
    if (n == "face") take(s->face);
    else if (n == "edge") take(s->edge);
    else if (n == "hinge") take(s->hinge);
    else if (n == "inv_rest2x2") take(s->inv_rest);
    else if (n == "fixed_offset") take(s->fixed_table.offset);
    else if (n == "fixed_index") take(s->fixed_table.data);
    else if (n == "transpose_offset") take(s->transpose_offset);
    else if (n == "transpose") take(s->transpose_data);
    else if (n == "face_slots") take(s->face_slots);
    else if (n == "hinge_slots") take(s->hinge_slots);
    else if (n == "edge_face_offset") take(s->nb_eface.offset);
    else if (n == "edge_face") take(s->nb_eface.data);
    else if (n == "vertex_mass") per(s->vprop, [](const PpfVertexProp &p) { return p.mass; });
    else if (n == "vertex_area") per(s->vprop, [](const PpfVertexProp &p) { return p.area; });
    else if (n == "face_area") per(s->fprop, [](const PpfFaceProp &p) { return p.area; });
    else if (n == "face_mass") per(s->fprop, [](const PpfFaceProp &p) { return p.mass; });
    else if (n == "vertex_order") take(s->vpos);
    else if (n == "tet") take(s->tet);
    else if (n == "tet_slots") take(s->tet_slots);
    else if (n == "stitch_slots") take(s->stitch_slots);
    else if (n == "stitch") take(s->stitch);
    else if (n == "inv_rest3x3") take(s->inv_rest3);
    else if (n == "tet_mass") per(s->tprop, [](const PpfTetProp &p) { return p.mass; });
    else if (n == "tet_volume") per(s->tprop, [](const PpfTetProp &p) { return p.volume; });
    else if (n == "vertex_volume") per(s->vprop, [](const PpfVertexProp &p) { return p.volume; });
    else if (n == "face_type") take(s->type_face);
    else if (n == "hinge_type") take(s->type_hinge);
    else if (n == "edge_slots") take(s->edge_slots);
    else if (n == "rod_bend_slots") take(s->rod_bend_slots);
    else if (n == "edge_length") per(s->eprop, [](const PpfEdgeProp &p) { return p.length; });
    else if (n == "edge_initial_length")
        per(s->eprop, [](const PpfEdgeProp &p) { return p.initial_length; });
    else if (n == "edge_mass") per(s->eprop, [](const PpfEdgeProp &p) { return p.mass; });
    else if (n == "edge_stiffness")
        per(s->eprop, [&](const PpfEdgeProp &p) { return s->eparam[p.param_index].stiffness; });
    else if (n == "edge_bend")
        per(s->eprop, [&](const PpfEdgeProp &p) { return s->eparam[p.param_index].bend; });
    else if (n == "rest_bend_angle")
        per(s->vprop, [](const PpfVertexProp &p) { return p.rest_bend_angle; });
    else if (n == "vertex_ghat")
        per(s->vprop, [&](const PpfVertexProp &p) { return s->vparam.empty() ? 0.0f : s->vparam[p.param_index].ghat; });
    else if (n == "vertex_offset")
        per(s->vprop, [&](const PpfVertexProp &p) { return s->vparam.empty() ? 0.0f : s->vparam[p.param_index].offset; });
    else if (n == "vertex_friction")
        per(s->vprop, [&](const PpfVertexProp &p) { return s->vparam.empty() ? 0.0f : s->vparam[p.param_index].friction; });
    else if (n == "hinge_length") per(s->hprop, [](const PpfHingeProp &p) { return p.length; });
    else if (n == "hinge_area") per(s->hprop, [](const PpfHingeProp &p) { return p.area; });
    else if (n == "face_mu")
        per(s->fprop, [&](const PpfFaceProp &p) { return s->fparam[p.param_index].mu; });
    else if (n == "face_lambda")
        per(s->fprop, [&](const PpfFaceProp &p) { return s->fparam[p.param_index].lambda; });
    else if (n == "hinge_bend")
        per(s->hprop, [&](const PpfHingeProp &p) { return s->hparam[p.param_index].bend; });
    else return (size_t)-1;
    if (out && bytes) std::memcpy(out, src, bytes);
    return bytes;
}

void ppf_scene_set_pin_targets(PpfScene *s, const float *pos, const float *delta) {
    for (size_t i = 0; i < s->fix.size(); ++i)
        for (int d = 0; d < 3; ++d) {
            s->fix[i].position.v[d] = pos[3 * i + d];
            s->fix[i].step_delta.v[d] = delta ? delta[3 * i + d] : 0.0f;
        }
}

} // extern "C"
