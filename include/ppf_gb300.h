/*
 * ppf_gb300.h -- C ABI of the GB300-native per-step contact solve.
 *
 * The library libppf_gb300.so is a drop-in for the reference's CUDA backend
 * (libsimbackend_cuda.so) on the per-step path: it exports the same extern "C"
 * entry points, with the same argument meaning, and reads/writes host structs
 * whose byte layout is identical to the reference's repr(C) data model.
 *
 *   reference struct definitions : crates/ppf-cts-solver/src/cpp/data.hpp
 *   reference Rust mirror        : crates/ppf-cts-solver/src/data.rs
 *   reference extern block       : crates/ppf-cts-solver/src/backend.rs:28-62
 *   reference implementation     : crates/ppf-cts-solver/src/cpp/main/main.cu:1673-2350
 *
 * Layout conventions (data.hpp / vec.hpp / smat.hpp):
 *   Vec<T>    = { T *data; u32 size; u32 allocated; }
 *   VecVec<T> = { T *data; u32 *offset; u32 size, nnz, nnz_allocated,
 *                 offset_allocated; }
 *   SVec/SMat = plain float/u32 arrays, column-major, no extra alignment.
 *   enums     = 4-byte ints, bool = 1 byte.
 * The layout is checked field by field against the reference headers by the
 * layout fixture in tests/golden (see tests/test_abi_layout.py).
 *
 * Ownership and threading follow the reference: the host owns every DataSet
 * array; initialize() deep-copies them to the device and keeps the host
 * DataSet / ParamSet by pointer; advance() writes param->time and
 * param->prev_dt through that pointer; fetch() writes vertex.curr/prev back
 * into the host arrays.  Single host thread, not re-entrant.
 */
#ifndef PPF_GB300_H
#define PPF_GB300_H

#include <stdbool.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- small fixed-size values (SVec / SMat, column-major) ---------------- */
typedef struct { float v[3]; } PpfVec3f;
typedef struct { float v[6]; } PpfVec6f;
typedef struct { unsigned v[2]; } PpfVec2u;
typedef struct { unsigned v[3]; } PpfVec3u;
typedef struct { unsigned v[4]; } PpfVec4u;
typedef struct { unsigned v[6]; } PpfVec6u;
typedef struct { float m[4]; } PpfMat2x2f;
typedef struct { float m[9]; } PpfMat3x3f;

/* ---- containers --------------------------------------------------------- */
#define PPF_DECLARE_VEC(NAME, T)                                               \
    typedef struct {                                                           \
        T *data;                                                               \
        unsigned size;                                                         \
        unsigned allocated;                                                    \
    } NAME
#define PPF_DECLARE_VECVEC(NAME, T)                                            \
    typedef struct {                                                           \
        T *data;                                                               \
        unsigned *offset;                                                      \
        unsigned size;                                                         \
        unsigned nnz;                                                          \
        unsigned nnz_allocated;                                                \
        unsigned offset_allocated;                                             \
    } NAME

/* enums (data.hpp:77-83) */
typedef int PpfModel;        /* 0 ARAP, 1 StVK, 2 BaraffWitkin, 3 SNHk, 4 Pdrd */
typedef int PpfBarrier;      /* 0 Cubic, 1 Quad, 2 Log */
typedef int PpfFrictionMode; /* 0 Min, 1 Max, 2 Mean */
typedef int PpfPrecondMode;  /* 0 BlockJacobi, 1 Schwarz */
enum { PPF_MODEL_ARAP = 0, PPF_MODEL_STVK = 1, PPF_MODEL_BARAFF_WITKIN = 2,
       PPF_MODEL_SNHK = 3, PPF_MODEL_PDRD = 4 };
enum { PPF_BARRIER_CUBIC = 0, PPF_BARRIER_QUAD = 1, PPF_BARRIER_LOG = 2 };
enum { PPF_FRICTION_MIN = 0, PPF_FRICTION_MAX = 1, PPF_FRICTION_MEAN = 2 };

/* ---- per-element params and props (data.hpp:115-330) -------------------- */
typedef struct { float ghat, offset, friction; } PpfVertexParam;
typedef struct {
    float stiffness, bend, ghat, offset, friction, strainlimit, plasticity,
        plasticity_threshold;
    bool bend_rest_from_geometry;
    float deform_damping, bend_damping;
} PpfEdgeParam;
typedef struct {
    PpfModel model;
    float mu, lambda, friction, ghat, offset, bend, strainlimit, shrink_x,
        shrink_y, pressure, plasticity, plasticity_threshold, bend_plasticity,
        bend_plasticity_threshold;
    bool bend_rest_from_geometry;
    float deform_damping, bend_damping, bend_warp, bend_weft;
} PpfFaceParam;
typedef struct {
    float bend, ghat, offset, plasticity, plasticity_threshold, bend_damping,
        bend_warp, bend_weft;
} PpfHingeParam;
typedef struct {
    PpfModel model;
    float mu, lambda, shrink, plasticity, plasticity_threshold, deform_damping;
} PpfTetParam;
typedef struct {
    float area, volume, mass, rest_bend_angle;
    unsigned fix_index, pull_index, param_index, pdrd_body_index;
    bool collider;
} PpfVertexProp;
typedef struct {
    float length, initial_length, mass;
    bool fixed;
    unsigned param_index;
} PpfEdgeProp;
typedef struct {
    float area, mass;
    bool fixed, rest_excluded, collider;
    unsigned param_index;
} PpfFaceProp;
typedef struct {
    float length, area, rest_angle, uv_edge_sin2;
    bool fixed, collider;
    unsigned param_index;
} PpfHingeProp;
typedef struct {
    float mass, volume;
    bool fixed, rest_excluded;
    unsigned param_index;
} PpfTetProp;
typedef struct {
    PpfVec3f rest_centroid;
    PpfMat3x3f rest_gram_inv;
    float volume;
    unsigned vertex_start, vertex_count;
    float mass_per_vertex;
    unsigned joint_mode;
    PpfVec3f joint_axis, joint_pin;
} PpfPdrdBodyProp;

/* ---- constraints (data.hpp:372-488) ------------------------------------- */
typedef struct {
    PpfVec3f position, step_delta;
    float ghat;
    unsigned index;
    bool kinematic;
} PpfFixPair;
typedef struct { PpfVec3f position; float weight; unsigned index; } PpfPullPair;
typedef struct {
    unsigned axis_component, vertex_start, vertex_count, hint_vertex;
} PpfTorqueGroup;
typedef struct { float magnitude; unsigned index, group_id; } PpfTorqueVertex;
typedef struct { PpfVec6u index; PpfVec6f weight; float stiffness; } PpfStitch;
typedef struct {
    PpfVec3f center;
    float ghat, friction, radius, thickness;
    bool bowl, reverse, kinematic;
} PpfSphere;
typedef struct {
    PpfVec3f ground;
    float ghat, friction, thickness;
    PpfVec3f up;
    bool kinematic;
} PpfFloor;
typedef struct {
    PpfVec3f axis;
    float total_mass;
    unsigned pdrd_body_index, dmap_index;
    PpfVec3f rotation_axis;
    unsigned rotation_mode;
    PpfVec3f anchor;
} PpfTranslationLock;

PPF_DECLARE_VEC(PpfVecVec3f, PpfVec3f);
PPF_DECLARE_VEC(PpfVecVec3u, PpfVec3u);
PPF_DECLARE_VEC(PpfVecVec4u, PpfVec4u);
PPF_DECLARE_VEC(PpfVecVec2u, PpfVec2u);
PPF_DECLARE_VEC(PpfVecChar, char);
PPF_DECLARE_VEC(PpfVecU8, unsigned char);
PPF_DECLARE_VEC(PpfVecU32, unsigned);
PPF_DECLARE_VEC(PpfVecF32, float);
PPF_DECLARE_VEC(PpfVecMat2x2f, PpfMat2x2f);
PPF_DECLARE_VEC(PpfVecMat3x3f, PpfMat3x3f);
PPF_DECLARE_VEC(PpfVecVertexParam, PpfVertexParam);
PPF_DECLARE_VEC(PpfVecEdgeParam, PpfEdgeParam);
PPF_DECLARE_VEC(PpfVecFaceParam, PpfFaceParam);
PPF_DECLARE_VEC(PpfVecHingeParam, PpfHingeParam);
PPF_DECLARE_VEC(PpfVecTetParam, PpfTetParam);
PPF_DECLARE_VEC(PpfVecVertexProp, PpfVertexProp);
PPF_DECLARE_VEC(PpfVecEdgeProp, PpfEdgeProp);
PPF_DECLARE_VEC(PpfVecFaceProp, PpfFaceProp);
PPF_DECLARE_VEC(PpfVecHingeProp, PpfHingeProp);
PPF_DECLARE_VEC(PpfVecTetProp, PpfTetProp);
PPF_DECLARE_VEC(PpfVecPdrdBodyProp, PpfPdrdBodyProp);
PPF_DECLARE_VEC(PpfVecFixPair, PpfFixPair);
PPF_DECLARE_VEC(PpfVecPullPair, PpfPullPair);
PPF_DECLARE_VEC(PpfVecTorqueGroup, PpfTorqueGroup);
PPF_DECLARE_VEC(PpfVecTorqueVertex, PpfTorqueVertex);
PPF_DECLARE_VEC(PpfVecSphere, PpfSphere);
PPF_DECLARE_VEC(PpfVecFloor, PpfFloor);
PPF_DECLARE_VEC(PpfVecStitch, PpfStitch);
PPF_DECLARE_VEC(PpfVecTranslationLock, PpfTranslationLock);
PPF_DECLARE_VECVEC(PpfVecVecU32, unsigned);
PPF_DECLARE_VECVEC(PpfVecVecVec2u, PpfVec2u);

typedef struct {
    PpfVecVecU32 face, hinge, edge, rod;
} PpfVertexNeighbor;
typedef struct { PpfVecVecU32 face; } PpfHingeNeighbor;
typedef struct { PpfVecVecU32 face; } PpfEdgeNeighbor;

typedef struct {
    struct {
        PpfVecVec3u face;
        PpfVecVec4u hinge;
        PpfVecVec2u edge;
        PpfVecVec4u tet;
    } mesh;
    struct {
        PpfVertexNeighbor vertex;
        PpfHingeNeighbor hinge;
        PpfEdgeNeighbor edge;
    } neighbor;
    struct {
        PpfVecChar face, vertex, hinge;
    } type;
} PpfMeshInfo;

typedef struct {
    PpfVecVertexProp vertex;
    PpfVecEdgeProp edge;
    PpfVecFaceProp face;
    PpfVecHingeProp hinge;
    PpfVecTetProp tet;
    PpfVecPdrdBodyProp pdrd_body;
} PpfPropSet;

typedef struct {
    PpfVecVertexParam vertex;
    PpfVecEdgeParam edge;
    PpfVecFaceParam face;
    PpfVecHingeParam hinge;
    PpfVecTetParam tet;
} PpfParamArrays;

typedef struct {
    PpfVecVec3f vertex;
    PpfVecVec3u face;
    PpfVecVec2u edge;
    struct {
        PpfVecVertexProp vertex;
        PpfVecFaceProp face;
        PpfVecEdgeProp edge;
    } prop;
    struct {
        PpfVecVertexParam vertex;
        PpfVecFaceParam face;
        PpfVecEdgeParam edge;
    } param_arrays;
    struct {
        PpfVertexNeighbor vertex;
        PpfHingeNeighbor hinge;
        PpfEdgeNeighbor edge;
    } neighbor;
} PpfCollisionMesh;

typedef struct {
    PpfVecFixPair fix;
    PpfVecPullPair pull;
    PpfVecTorqueGroup torque_groups;
    PpfVecTorqueVertex torque_vertices;
    PpfVecSphere sphere;
    PpfVecFloor floor;
    PpfVecStitch stitch;
    PpfCollisionMesh mesh;
} PpfConstraint;

typedef struct {
    PpfVecMat2x2f inv_rest2x2;
    PpfVecMat3x3f inv_rest3x3;
    PpfVecU8 exclude_face;
    PpfVecU8 exclude_tet;
} PpfRestShapeUpdate;

/* ParamSet (data.hpp:515-568) */
typedef struct {
    double time;
    float air_friction, air_density, constraint_tol, prev_dt, dt, playback;
    unsigned min_newton_steps;
    float target_toi, stitch_length_factor;
    unsigned cg_max_iter;
    float cg_tol, line_search_max_t, ccd_eps, max_dx, eiganalysis_eps,
        friction_eps, isotropic_air_friction;
    PpfVec3f gravity, wind;
    PpfBarrier barrier;
    PpfFrictionMode friction_mode;
    unsigned csrmat_max_nnz;
    float fix_xz;
    bool disable_contact, inactive_momentum;
    PpfPrecondMode precond;
    unsigned schwarz_levels;
    unsigned max_newton_steps;
    bool disable_pin_dof_removal;
} PpfParamSet;

/* StepResult (data.hpp:570-595) */
typedef struct {
    double time;
    bool ccd_success, pcg_success, intersection_free, newton_progress,
        pin_feasible, contact_separated;
} PpfStepResult;

typedef struct { PpfVecVec3f prev, curr; } PpfVertexSet;

/* DataSet (data.hpp:624-720) */
typedef struct {
    PpfVertexSet vertex;
    PpfMeshInfo mesh;
    PpfPropSet prop;
    PpfParamArrays param_arrays;
    PpfVecMat2x2f inv_rest2x2;
    PpfVecMat3x3f inv_rest3x3;
    PpfConstraint constraint;
    PpfVecVecU32 fixed_index_table;
    PpfVecVecVec2u transpose_table;
    unsigned rod_count, shell_face_count, surface_vert_count;
    PpfVecU32 pdrd_vert_list;
    PpfVecVec3f pdrd_rest_centered;
    PpfVecVec3f grain_omega;
    PpfVecF32 grain_inv_inertia;
    PpfVecVec3f grain_torque;
    PpfVecF32 grain_ang_stiff;
    PpfVecVec3f grain_contact_normal;
    PpfVecF32 grain_inv_inertia_center;
    PpfVecVec3f grain_omega_prev;
    PpfVecMat3x3f grain_A, grain_B;
    PpfVecVec3f grain_grot;
    PpfVecU32 tet_hess_slots, face_hess_slots, edge_hess_slots,
        hinge_hess_slots, rod_bend_hess_slots, stitch_hess_slots;
    PpfVecTranslationLock translation_lock;
    PpfVecU32 translation_lock_index;
    PpfVecVec3f translation_lock_initial;
    PpfVecU32 statistics_object_index, statistics_static_object_index,
        statistics_contact_count;
} PpfDataSet;

#define PPF_MAX_INTERSECTION_RECORDS 256
/* IntersectionRecord (data.hpp:741-748) */
typedef struct {
    unsigned type, elem0, elem1, num_verts0, num_verts1;
    float positions[15];
} PpfIntersectionRecord;

/* =========================================================================
 * Reference entry points (drop-in).  Each replaces the function of the same
 * name in crates/ppf-cts-solver/src/cpp/main/main.cu; the Rust declarations
 * they satisfy are crates/ppf-cts-solver/src/backend.rs:28-62.
 * ========================================================================= */

/* main.cu:1877-1920.  Copies the DataSet to the device, builds the BVHs and
 * runs the initial intersection check on prev and curr.  Returns false (with
 * ppf_fatal_code() == PPF_FATAL_INIT_INTERSECTION) when the scene starts
 * self-intersecting. */
bool initialize(PpfDataSet *dataset, PpfParamSet *param);
/* main.cu:1922-1924 -> main_helper::advance (main.cu:267-1649).  One step:
 * BVH rebuild, inertial target, Newton loop (assembly, block-Jacobi PCG,
 * additive-CCD line search, strain-limit line search), commit. */
void advance(PpfStepResult *result);
/* main.cu:1926-1937.  Device -> host copy of vertex.curr/prev. The optional
 * per-object contact statistics (statistics_contact_count) are not counted
 * by this library; a host array given for them is left as it is. */
void fetch(void);
/* main.cu:1939-1948.  Device -> host copy of the rest-shape inverses
 * (inv_rest2x2; update_rest_shape is what changes them on the device). */
void fetch_inv_rest(void);
/* main.cu:1950-1968.  Device -> host copy of the hinge and vertex props,
 * which carry the rest angles. Nothing on the device changes them in this
 * library (bend plasticity is not built), so the copy returns what the host
 * last uploaded. */
void fetch_rest_angles(void);
/* main.cu:1970-1977.  Size of the carried dynamic contact pattern: the
 * last assembly's, or the one update_dyn restored since. */
void fetch_dyn_counts(unsigned *n_value, unsigned *n_offset);
/* main.cu:1979-1982.  Carried dynamic contact pattern (row offsets and
 * column indices of the upper-triangle contact blocks outside the fixed
 * pattern); value may be NULL. */
void fetch_dyn(unsigned *index, PpfMat3x3f *value, unsigned *offset);
/* main.cu:1984-1986.  Restores a carried pattern (checkpoint resume). The
 * pattern only seeds capacity; it never changes values. It reserves the
 * contact-block buffers for its count and is what fetch_dyn_counts /
 * fetch_dyn report until the next assembly. */
void update_dyn(unsigned *index, unsigned *offset);
/* main.cu:1988-2077 */
void update_constraint(const PpfConstraint *constraint);
/* main.cu:2079-2121 */
void update_rest_shape(const PpfRestShapeUpdate *update);
/* main.cu:2123-2150 */
void override_velocity(const unsigned *indices, unsigned count, float vx,
                       float vy, float vz, float dt);
/* main.cu:2158-2185 */
void gather_current_positions(const unsigned *indices, unsigned count,
                              float *out);
/* main.cu:2195-2227 */
void override_angular_velocity(const unsigned *indices, unsigned count,
                               float wx, float wy, float wz, float cx,
                               float cy, float cz, float dt);
/* main.cu:2229-2263 */
void init_collision_windows(const unsigned *vert_dmap, unsigned vert_count,
                            const float *windows,
                            const unsigned *window_counts, unsigned n_groups);
/* main.cu:2265-2325 */
void refresh_collision_active(float time);
/* main.cu:2339-2350 */
unsigned fetch_intersection_records(PpfIntersectionRecord *out,
                                    unsigned max_count);
/* main.cu:1662-1668 */
unsigned char ppf_fatal_code(void);
const char *ppf_fatal_detail(void);
/* main.cu:1680-1682.  Creates data_dir and appends per-step logs there in
 * SimpleLog's format: advance.out ("time msec") and advance.<channel>.out
 * for the channels iter, toi, num_contact, newton_steps and final_dt. */
void set_log_path(const char *data_dir);

/* Fatal codes (crates/ppf-cts-solver/src/cpp/main/fatal.hpp:48-55). */
enum {
    PPF_FATAL_NONE = 0,
    PPF_FATAL_INIT_INTERSECTION = 1,
    PPF_FATAL_OOM = 2,
    PPF_FATAL_CUDA_DRIVER = 3,
    PPF_FATAL_SOLVER_INVARIANT = 4,
    PPF_FATAL_DEVICE_ASSERT = 5,
    PPF_FATAL_WATCHDOG_TIMEOUT = 6
};

#ifdef __cplusplus
}
#endif

#endif /* PPF_GB300_H */
