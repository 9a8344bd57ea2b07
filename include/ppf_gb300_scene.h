/*
 * ppf_gb300_scene.h -- host-side scene builder of libppf_gb300.so.
 *
 * Builds the DataSet / ParamSet / Constraint that initialize() consumes from
 * plain meshes and material parameters, the way the reference's driver does
 * before its first initialize() call (crates/ppf-cts-solver/src/builder.rs
 * build() and make_param(), crates/ppf-cts-solver/src/scene.rs make_props(),
 * crates/ppf-cts-solver/src/mesh.rs Mesh::new, and the face-edge props of
 * crates/ppf-cts-solver/src/main.rs:205-250). Covered: shells (any model
 * field, Baraff-Witkin evaluated), rods, fix pins (static or kinematic), pull
 * pins, analytic spheres and floors, static collision meshes, solids (tets),
 * stitches. Not covered: PDRD bodies, sand grains, UV anisotropy.
 *
 * Edge and hinge order: the reference extracts them from a hash map, whose
 * iteration order is not reproducible; here they are listed in first-seen
 * order over the faces, which is deterministic.
 */
#ifndef PPF_GB300_SCENE_H
#define PPF_GB300_SCENE_H

#include "ppf_gb300.h"

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct PpfScene PpfScene;

/* Per-object shell material, in the reference's parameter units
 * (crates/ppf-cts-core/src/datamodel/params.rs object_param). */
typedef struct {
    int model;            /* PPF_MODEL_* ; default Baraff-Witkin */
    float density;        /* kg/m^2 */
    float young_mod;      /* Young's modulus pre-divided by density (Pa/rho) */
    float poiss_rat;      /* (0, 0.5) */
    float bend;           /* dimensionless bending stiffness */
    float strain_limit;   /* 0 disables */
    float contact_gap;    /* ghat */
    float contact_offset;
    float friction;
    float deform_damping; /* Rayleigh damping of the membrane (0: none) */
    float bend_damping;   /* Rayleigh damping of the bending (0: none) */
} PpfShellMaterial;

/* Per-object solid material (the reference scene's tet parameters,
 * scene.rs:1840-1921). */
typedef struct {
    int model;            /* PPF_MODEL_ARAP / STVK / SNHK */
    float density;        /* kg/m^3 */
    float young_mod;      /* Young's modulus (pre-divided by density, as shells) */
    float poiss_rat;      /* (0, 0.5) */
    float contact_gap;    /* ghat of the boundary faces */
    float contact_offset;
    float friction;
    float deform_damping; /* Rayleigh damping (0: none) */
} PpfSolidMaterial;

/* Per-object rod material (the reference scene's rod-* parameters,
 * scene.rs:1540-1660). */
typedef struct {
    float density;        /* kg/m: edge mass = density x rest length */
    float young_mod;      /* stretch stiffness, scaled by the edge mass */
    float bend;           /* bending stiffness (0: none) */
    float length_factor;  /* rest length = factor x initial length */
    float strain_limit;   /* 0 disables */
    float contact_gap;    /* ghat */
    float contact_offset;
    float friction;
    float deform_damping; /* Rayleigh damping of the stretch */
    float bend_damping;   /* Rayleigh damping of the bending */
    int bend_rest_from_geometry; /* rest bend angle from the initial shape */
} PpfRodMaterial;

PpfScene *ppf_scene_create(void);
void ppf_scene_destroy(PpfScene *scene);

/* Reference defaults of every ParamSet field (params.rs app_param through
 * builder.rs make_param), with dt = 1e-3. */
void ppf_scene_default_param(PpfParamSet *out);

/* Appends a shell object; returns the global index of its first vertex. */
unsigned ppf_scene_add_shell(PpfScene *scene, const float *vertices,
                             unsigned n_vertices, const unsigned *faces,
                             unsigned n_faces, const PpfShellMaterial *mat);
/* A shell whose faces carry their own materials (the reference scene's
 * per-face tri-* parameter arrays, scene.rs:1660-1830): face i uses
 * materials[face_material[i]]. Vertices are appended as by
 * ppf_scene_add_shell; returns the index of the first, or 0xffffffff when a
 * face names a material past n_materials. */
unsigned ppf_scene_add_shell_faces(PpfScene *scene, const float *vertices, unsigned nv,
                                   const unsigned *faces, unsigned nf,
                                   const unsigned *face_material,
                                   const PpfShellMaterial *materials, unsigned n_materials);
/* Appends a rod object: nv vertices and ne edges (2 vertex indices each,
 * local to this object). Rod edges come first in the DataSet's edge list
 * (mesh.rs:188-229), so the rods of every added object precede the shells'
 * edges. Returns the global index of the first vertex. */
unsigned ppf_scene_add_rod(PpfScene *scene, const float *vertices, unsigned nv,
                           const unsigned *edges, unsigned ne, const PpfRodMaterial *mat);
/* Rod edges between vertices already added (global indices, 2 per edge),
 * edge i with materials[edge_material[i]]: the reference scene's rod.bin and
 * per-rod rod-* parameter arrays over its shared vertex array
 * (scene.rs:512-719, 1540-1655). Returns 0, or -1 when an index is out of
 * range (nothing is added then). */
int ppf_scene_add_rod_edges(PpfScene *scene, const unsigned *edges, unsigned ne,
                            const unsigned *edge_material, const PpfRodMaterial *materials,
                            unsigned n_materials);
/* Appends a solid object: nv vertices and nt tets (4 vertex indices each,
 * local, positively oriented). Its boundary faces (the tet faces no other
 * tet shares, outward) become contact faces after every shell face
 * (shell_face_count stays the shells'); the vertices only tets use become
 * the DataSet's last vertices (surface_vert_count counts the rest,
 * mesh.rs:78-95). Vertex indices in this API stay in the order vertices were
 * added; "vertex_order" (ppf_scene_array) maps them to DataSet indices.
 * Returns the index of the first vertex. */
unsigned ppf_scene_add_solid(PpfScene *scene, const float *vertices, unsigned nv,
                             const unsigned *tets, unsigned nt, const PpfSolidMaterial *mat);
/* A stitch (Constraint::stitch, energy.cu:796-884): a spring between the
 * barycentric point index[0..2] / weight[0..2] and index[3..5] /
 * weight[3..5] (vertex indices as added; weights of each side sum to 1; a
 * single vertex s is {s, s, s} with {1, 0, 0}), rest length half the
 * weighted contact gap, with the given stiffness. Returns 0, or -1 for an
 * index out of range. */
int ppf_scene_add_stitch(PpfScene *scene, const unsigned *index, const float *weight,
                         float stiffness);
/* Initial velocity of every vertex (3 floats each); prev = curr - v dt. */
void ppf_scene_set_velocity(PpfScene *scene, const float *velocity);
/* Fix pins at the vertices' current positions. kinematic != 0 marks pins
 * whose targets the host moves each step (ppf_scene_set_pin_targets). */
void ppf_scene_pin(PpfScene *scene, const unsigned *indices, unsigned count,
                   int kinematic);
/* Soft pull pins toward the current positions with the given weight. */
void ppf_scene_pull(PpfScene *scene, const unsigned *indices, unsigned count,
                    float weight);
void ppf_scene_add_sphere(PpfScene *scene, const float *center, float radius,
                          float contact_gap, float friction, int reverse,
                          int bowl);
/* A static collision mesh (Constraint::mesh, builder.rs:1823-1935): nv
 * vertices and nf triangles, with its contact gap, offset and friction. Its
 * edges are extracted at build; meshes added in turn are concatenated. */
void ppf_scene_add_collision_mesh(PpfScene *scene, const float *vertices, unsigned nv,
                                  const unsigned *faces, unsigned nf, float contact_gap,
                                  float contact_offset, float friction);
void ppf_scene_add_floor(PpfScene *scene, const float *ground, const float *up,
                         float contact_gap, float friction);

/* Builds the DataSet and ParamSet; `param` supplies the global parameters
 * (dt, gravity, tolerances ...). Returns 0 on success. */
int ppf_scene_build(PpfScene *scene, const PpfParamSet *param);
PpfDataSet *ppf_scene_dataset(PpfScene *scene);
PpfParamSet *ppf_scene_param(PpfScene *scene);
PpfConstraint *ppf_scene_constraint(PpfScene *scene);
/* Moves the kinematic pins: target positions at the end of the coming step
 * and their displacement over it (3 floats per pin, in pin order). */
void ppf_scene_set_pin_targets(PpfScene *scene, const float *position,
                               const float *step_delta);
unsigned ppf_scene_vertex_count(PpfScene *scene);
/* Host copies of the built DataSet's vertex.curr / vertex.prev (3 floats per
 * vertex, in the order the vertices were added). fetch() writes the device
 * state into these arrays, so after it ppf_scene_positions returns the
 * solver's state; ppf_scene_set_positions overwrites them before
 * initialize(). Either pointer may be NULL. */
void ppf_scene_positions(PpfScene *scene, float *curr, float *prev);
void ppf_scene_set_positions(PpfScene *scene, const float *curr,
                             const float *prev);
/* Byte size of one named array of the built scene, copied into `out` when it
 * is not NULL ((size_t)-1 for an unknown name or an unbuilt scene). It has no
 * counterpart in the reference: it exposes what the builder computed so a
 * host can check it. Names: face, edge, hinge (u32 per corner);
 * inv_rest2x2 (4 f32 per face, column-major); fixed_offset, fixed_index
 * (the upper-triangle fixed pattern, u32); transpose_offset, transpose (u32
 * (row, slot) pairs per lower entry); face_slots (9 u32 per face),
 * hinge_slots (16 u32 per hinge); edge_slots (4 u32 per rod edge),
 * rod_bend_slots (9 u32 per vertex); edge_face_offset, edge_face (u32); and
 * f32 per element: vertex_mass, vertex_area, face_area, face_mass,
 * edge_length, edge_initial_length, edge_mass, edge_stiffness, edge_bend,
 * rest_bend_angle (per vertex), hinge_length, hinge_area, face_mu,
 * stitch (the DataSet's stitches), stitch_slots (36 u32 per stitch),
 * tet (4 u32 per tet), tet_slots (16 u32 per tet), inv_rest3x3 (9 f32 per
 * tet, column-major), tet_mass, tet_volume, vertex_volume (f32),
 * vertex_order (u32: DataSet index of each added vertex), face_type,
 * hinge_type (u8, bit 0: a solid's boundary face / a hinge next to one),
 * face_lambda, hinge_bend; vertex_ghat, vertex_offset, vertex_friction (the
 * contact parameters of each vertex's param). */
size_t ppf_scene_array(PpfScene *scene, const char *name, void *out);

#ifdef __cplusplus
}
#endif

#endif
