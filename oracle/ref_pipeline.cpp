// ref_pipeline.cpp -- the reference's own Newton-system assembly, contact
// detection, CCD line search and intersection check, run as host code
// (TEST INFRASTRUCTURE).
//
// Compiled by oracle/Makefile with g++ straight from the reference's sources
// where they lie (crates/ppf-cts-solver/src/cpp: csrmat.cu, buffer.cu,
// energy.cu, strainlimiting.cu, contact.cu, utility.cu, eigenanalysis.cu,
// barrier.cu); the output goes only to oracle/_ref/. None of those files
// launch kernels themselves: their DISPATCH lambdas run here as serial loops.
// The device runtime they touch is supplied as host shims: allocations are
// host heap memory, copies are memcpy, atomics are plain read-modify-writes,
// and the fill / reduction kernels of kernels/*.cu are host loops.
//
// The entry points mirror main_helper::advance's assembly sequence
// (main/main.cu:713-874) and line search (main.cu:1213-1340) on one state, so
// the oracle's restatement can be compared with the reference's own code on
// the same inputs.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <vector>

using std::isfinite;
using std::max;
using std::min;

// ---- CUDA runtime stand-ins (host memory) ---------------------------------
#define CUDA_UTILS_HPP
typedef int cudaError_t;
enum : int { cudaSuccess = 0 };
enum cudaMemcpyKind {
    cudaMemcpyHostToHost,
    cudaMemcpyHostToDevice,
    cudaMemcpyDeviceToHost,
    cudaMemcpyDeviceToDevice,
    cudaMemcpyDefault
};
typedef void *cudaStream_t;
template <class T> inline cudaError_t cudaMalloc(T **p, size_t n) {
    *p = (T *)std::calloc(n ? n : 1, 1);
    return cudaSuccess;
}
inline cudaError_t cudaFree(void *p) {
    std::free(p);
    return cudaSuccess;
}
inline cudaError_t cudaMemcpy(void *d, const void *s, size_t n, cudaMemcpyKind) {
    if (n) std::memmove(d, s, n);
    return cudaSuccess;
}
inline cudaError_t cudaMemset(void *p, int v, size_t n) {
    std::memset(p, v, n);
    return cudaSuccess;
}
template <class T>
inline cudaError_t cudaMemcpyToSymbol(T &sym, const void *src, size_t n, size_t off = 0,
                                      cudaMemcpyKind = cudaMemcpyHostToDevice) {
    std::memcpy((char *)&sym + off, src, n);
    return cudaSuccess;
}
template <class T>
inline cudaError_t cudaMemcpyFromSymbol(void *dst, const T &sym, size_t n, size_t off = 0,
                                        cudaMemcpyKind = cudaMemcpyDeviceToHost) {
    std::memcpy(dst, (const char *)&sym + off, n);
    return cudaSuccess;
}
inline cudaError_t cudaDeviceSynchronize() { return cudaSuccess; }
#define CUDA_HANDLE_ERROR(err) ((void)(err))
#ifndef __host__
#define __host__
#endif
#ifndef __device__
#define __device__
#endif
#ifndef __global__
#define __global__
#endif
#ifndef __forceinline__
#define __forceinline__ inline
#endif
template <class Y> inline Y pinned_read(const Y *dev) { return *dev; }
inline void *pinned_scratch(size_t bytes) {
    static std::vector<char> buf;
    if (buf.size() < bytes) buf.resize(bytes);
    return buf.data();
}
unsigned long long g_device_alloc_count = 0, g_device_free_count = 0;
int g_ppf_kernel_timeout_enabled = -1;

// ---- serial dispatch and atomics --------------------------------------------
#define DISPATCHER_HPP
#define DISPATCH_START(n)                                                      \
    {                                                                          \
        const unsigned n_threads(n);                                           \
        auto kernel =
#define DISPATCH_END                                                           \
    ;                                                                          \
    for (unsigned i_ = 0; i_ < n_threads; ++i_) kernel(i_);                    \
    }
inline float atomicAdd(float *p, float v) {
    float o = *p;
    *p += v;
    return o;
}
inline unsigned atomicAdd(unsigned *p, unsigned v) {
    unsigned o = *p;
    *p += v;
    return o;
}
inline int atomicAdd(int *p, int v) {
    int o = *p;
    *p += v;
    return o;
}
inline unsigned long long atomicAdd(unsigned long long *p, unsigned long long v) {
    unsigned long long o = *p;
    *p += v;
    return o;
}
inline unsigned atomicCAS(unsigned *p, unsigned cmp, unsigned v) {
    unsigned o = *p;
    if (o == cmp) *p = v;
    return o;
}
inline unsigned atomicMin(unsigned *p, unsigned v) {
    unsigned o = *p;
    if (v < o) *p = v;
    return o;
}
inline unsigned atomicMax(unsigned *p, unsigned v) {
    unsigned o = *p;
    if (v > o) *p = v;
    return o;
}
inline unsigned atomicOr(unsigned *p, unsigned v) {
    unsigned o = *p;
    *p |= v;
    return o;
}
inline unsigned atomicExch(unsigned *p, unsigned v) {
    unsigned o = *p;
    *p = v;
    return o;
}
inline void __threadfence() {}

// ---- logging / profiling stand-ins ------------------------------------------
#define SIMPLELOG_H
struct SimpleLog {
    explicit SimpleLog(const char * = nullptr) {}
    template <class... A> void push(A...) {}
    void pop() {}
    template <class... A> void mark(A...) {}
    template <class... A> static void message(A...) {}
    template <class... A> static void set(A...) {}
};
#define ASM_PROFILE_HPP
namespace asm_profile {
inline bool enabled() { return false; }
inline double tick() { return 0.0; }
inline double ms_since(double) { return 0.0; }
inline void report_widths(const char *, std::vector<unsigned> &) {}
} // namespace asm_profile

// PDRD rigid bodies are outside the path; energy.cu includes their kernels but
// calls none of them.
#define PDRD_RIGID_HPP
#include "data.hpp"
#include "kernels/reduce.hpp"
#include "kernels/vec_ops.hpp"
#include "main/fatal.hpp"

extern "C" {
unsigned char g_ppf_fatal_code = 0;
char g_ppf_fatal_detail[512] = {0};
void print_rust(const char *m) { std::puts(m); }
}

// ---- kernels/*.cu as host loops ---------------------------------------------
namespace kernels {
template <typename T> void set(T *array, unsigned n, T value, cudaStream_t) {
    for (unsigned i = 0; i < n; ++i) array[i] = value;
}
// kernels/exclusive_scan.cu:96-190: in-place exclusive prefix sum, returning
// the total.
unsigned exclusive_scan(unsigned *d, unsigned n) {
    unsigned run = 0;
    for (unsigned i = 0; i < n; ++i) {
        const unsigned v = d[i];
        d[i] = run;
        run += v;
    }
    return run;
}
void exclusive_scan_nocopy(unsigned *d, unsigned n) { (void)exclusive_scan(d, n); }
template <typename T> void copy(const T *src, T *dst, unsigned n, cudaStream_t) {
    if (n) std::memmove(dst, src, sizeof(T) * n);
}
template <class T> T sum_array(const T *array, unsigned size) {
    T s = T();
    for (unsigned i = 0; i < size; ++i) s += array[i];
    return s;
}
template <class T> T min_array(const T *array, unsigned size, T init) {
    T s = init;
    for (unsigned i = 0; i < size; ++i) s = std::min(s, array[i]);
    return s;
}
template <class T> T max_array(const T *array, unsigned size, T init) {
    T s = init;
    for (unsigned i = 0; i < size; ++i) s = std::max(s, array[i]);
    return s;
}
} // namespace kernels

#include "buffer/buffer.cu"
#include "csrmat/csrmat.cu"
#include "barrier/barrier.cu"
#include "utility/utility.cu"
#include "eigenanalysis/eigenanalysis.cu"
#include "energy/energy.cu"
#include "strainlimiting/strainlimiting.cu"
#include "contact/contact.cu"

// ---- BVH storage and collision windows --------------------------------------
namespace bvh_storage {
BVHSet &get_bvh() {
    static BVHSet s;
    return s;
}
BVHSet &get_collision_mesh_bvh() {
    static BVHSet s;
    return s;
}
} // namespace bvh_storage
const bool *contact::get_vert_collision_active() { return nullptr; }
const bool *contact::get_edge_collision_active() { return nullptr; }
const bool *contact::get_face_collision_active() { return nullptr; }

// ---- entry points -------------------------------------------------------------
namespace {

// Trees over the primitives' boxes: the reference's node format (leaf k holds
// (prim + 1, 0), internal nodes (left + 1, right + 1), boxes per node), built
// by median splits. Which valid tree the query walks does not change what it
// finds, so the reference's own LBVH builder (device code) is not needed.
struct HostTrees {
    std::vector<Vec2u> node[5]; // faces, edges, vertices, collision faces, collision edges
    std::vector<AABB> box[5];
};

AABB join_box(const AABB &a, const AABB &b) {
    AABB r;
    for (int d = 0; d < 3; ++d) {
        r.min[d] = std::fmin(a.min[d], b.min[d]);
        r.max[d] = std::fmax(a.max[d], b.max[d]);
    }
    r.active = a.active && b.active;
    return r;
}

unsigned split_build(std::vector<unsigned> &perm, const std::vector<AABB> &leaf, unsigned lo,
                     unsigned hi, unsigned &next, std::vector<Vec2u> &node,
                     std::vector<AABB> &box) {
    if (hi - lo == 1) {
        node[lo] = Vec2u(perm[lo] + 1, 0);
        box[lo] = leaf[perm[lo]];
        return lo;
    }
    float lo_c[3] = {INFINITY, INFINITY, INFINITY}, hi_c[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (unsigned k = lo; k < hi; ++k)
        for (int d = 0; d < 3; ++d) {
            float c = 0.5f * (leaf[perm[k]].min[d] + leaf[perm[k]].max[d]);
            lo_c[d] = std::fmin(lo_c[d], c);
            hi_c[d] = std::fmax(hi_c[d], c);
        }
    int ax = 0;
    for (int d = 1; d < 3; ++d)
        if (hi_c[d] - lo_c[d] > hi_c[ax] - lo_c[ax]) ax = d;
    const unsigned mid = lo + (hi - lo) / 2;
    std::nth_element(perm.begin() + lo, perm.begin() + mid, perm.begin() + hi,
                     [&](unsigned a, unsigned b) {
                         float ca = leaf[a].min[ax] + leaf[a].max[ax];
                         float cb = leaf[b].min[ax] + leaf[b].max[ax];
                         return ca < cb || (ca == cb && a < b);
                     });
    const unsigned id = next++;
    const unsigned l = split_build(perm, leaf, lo, mid, next, node, box);
    const unsigned r = split_build(perm, leaf, mid, hi, next, node, box);
    node[id] = Vec2u(l + 1, r + 1);
    box[id] = join_box(box[l], box[r]);
    return id;
}

void install_tree(BVH &bvh, Vec<AABB> &aabb, std::vector<Vec2u> &node, std::vector<AABB> &box,
                  const std::vector<AABB> &leaf) {
    const unsigned n = (unsigned)leaf.size();
    bvh.node.data = nullptr;
    bvh.node.size = 0;
    if (!n) return;
    node.assign(2 * n - 1, Vec2u(0, 0));
    box.assign(2 * n - 1, AABB());
    std::vector<unsigned> perm(n);
    for (unsigned i = 0; i < n; ++i) perm[i] = i;
    unsigned next = n;
    bvh.root = split_build(perm, leaf, 0, n, next, node, box);
    bvh.node.data = node.data();
    bvh.node.size = 2 * n - 1;
    bvh.node.allocated = 2 * n - 1;
    // the reference keeps the boxes in contact.cu's storage, sized 2n - 1
    std::memcpy(aabb.data, box.data(), sizeof(AABB) * (2 * n - 1));
}

// Leaf boxes of lbvh/lbvh.cu:623-721: the primitive at x0 and at
// x0 + e (x1 - x0), widened by 0.5 ghat + offset of its parameter set.
AABB leaf_box(const Vec3f *y0, const Vec3f *y1, unsigned k, float e, float margin) {
    AABB b;
    for (int d = 0; d < 3; ++d) {
        float mn0 = INFINITY, mx0 = -INFINITY, mn1 = INFINITY, mx1 = -INFINITY;
        for (unsigned a = 0; a < k; ++a) {
            float z = e * (y1[a][d] - y0[a][d]) + y0[a][d];
            mn0 = std::fmin(mn0, y0[a][d]);
            mx0 = std::fmax(mx0, y0[a][d]);
            mn1 = std::fmin(mn1, z);
            mx1 = std::fmax(mx1, z);
        }
        b.min[d] = std::fmin(mn0, mn1) - margin;
        b.max[d] = std::fmax(mx0, mx1) + margin;
    }
    b.active = true;
    return b;
}

struct RefPipe {
    DataSet data;
    ParamSet prm;
    unsigned n = 0;
    std::vector<Vec3f> curr, prev, velocity, eval_x, target, x0, x1;
    std::vector<float> force;
    std::vector<Mat3x3f> diag;
    DynCSRMat dyn;
    FixedCSRMat fixed, tmp_fixed;
    HostTrees trees;
    unsigned num_contact = 0;
    // The reference's scene builder sizes the grain arrays to the vertex
    // count in every scene and contact.cu reads them unconditionally; a
    // DataSet that leaves them empty gets zeroed ones (no grains).
    std::vector<float> grain_f[3];
    std::vector<Vec3f> grain_v[5];
    std::vector<Mat3x3f> grain_m[2];

    template <class T> void fill_empty(Vec<T> &v, std::vector<T> &store, const T &zero) {
        if (v.size) return;
        store.assign(n, zero);
        v = view(store);
    }
    void fill_grains() {
        const Vec3f z3 = Vec3f::Zero();
        fill_empty(data.grain_inv_inertia, grain_f[0], 0.0f);
        fill_empty(data.grain_ang_stiff, grain_f[1], 0.0f);
        fill_empty(data.grain_inv_inertia_center, grain_f[2], 0.0f);
        fill_empty(data.grain_omega, grain_v[0], z3);
        fill_empty(data.grain_torque, grain_v[1], z3);
        fill_empty(data.grain_contact_normal, grain_v[2], z3);
        fill_empty(data.grain_omega_prev, grain_v[3], z3);
        fill_empty(data.grain_grot, grain_v[4], z3);
        fill_empty(data.grain_A, grain_m[0], Mat3x3f::Zero());
        fill_empty(data.grain_B, grain_m[1], Mat3x3f::Zero());
    }

    template <class T> static Vec<T> view(std::vector<T> &v) {
        Vec<T> r;
        r.data = v.data();
        r.size = (unsigned)v.size();
        r.allocated = r.size;
        return r;
    }

    void build_trees(const std::vector<Vec3f> &a, const std::vector<Vec3f> &b, float e) {
        const Vec3f *pa = a.data(), *pb = b.data();
        std::vector<AABB> leaf;
        const unsigned nf = data.mesh.mesh.face.size;
        leaf.resize(nf);
        for (unsigned i = 0; i < nf; ++i) {
            const Vec3u f = data.mesh.mesh.face[i];
            Vec3f y0[3] = {pa[f[0]], pa[f[1]], pa[f[2]]}, y1[3] = {pb[f[0]], pb[f[1]], pb[f[2]]};
            const FaceParam &fp = data.param_arrays.face[data.prop.face[i].param_index];
            leaf[i] = leaf_box(y0, y1, 3, e, 0.5f * fp.ghat + fp.offset);
        }
        install_tree(bvh_storage::get_bvh().face, contact::get_face_aabb(), trees.node[0],
                     trees.box[0], leaf);
        const unsigned ne = data.mesh.mesh.edge.size;
        leaf.resize(ne);
        for (unsigned i = 0; i < ne; ++i) {
            const Vec2u g = data.mesh.mesh.edge[i];
            Vec3f y0[2] = {pa[g[0]], pa[g[1]]}, y1[2] = {pb[g[0]], pb[g[1]]};
            const EdgeParam &ep = data.param_arrays.edge[data.prop.edge[i].param_index];
            leaf[i] = leaf_box(y0, y1, 2, e, 0.5f * ep.ghat + ep.offset);
        }
        install_tree(bvh_storage::get_bvh().edge, contact::get_edge_aabb(), trees.node[1],
                     trees.box[1], leaf);
        const unsigned nv = data.surface_vert_count;
        leaf.resize(nv);
        for (unsigned i = 0; i < nv; ++i) {
            const VertexParam &vp = data.param_arrays.vertex[data.prop.vertex[i].param_index];
            leaf[i] = leaf_box(pa + i, pb + i, 1, e, 0.5f * vp.ghat + vp.offset);
        }
        install_tree(bvh_storage::get_bvh().vertex, contact::get_vertex_aabb(), trees.node[2],
                     trees.box[2], leaf);
    }

    // The static collision mesh's trees (lbvh/lbvh.cu:1100-1118: boxes of the
    // mesh as it is, widened by its parameters' 0.5 ghat + offset).
    void build_collision_trees() {
        const CollisionMesh &cm = data.constraint.mesh;
        const Vec3f *v = cm.vertex.data;
        std::vector<AABB> leaf(cm.face.size);
        for (unsigned i = 0; i < cm.face.size; ++i) {
            const Vec3u f = cm.face[i];
            Vec3f y[3] = {v[f[0]], v[f[1]], v[f[2]]};
            const FaceParam &fp = cm.param_arrays.face[cm.prop.face[i].param_index];
            leaf[i] = leaf_box(y, y, 3, 1.0f, 0.5f * fp.ghat + fp.offset);
        }
        install_tree(bvh_storage::get_collision_mesh_bvh().face,
                     contact::get_collision_mesh_face_aabb(), trees.node[3], trees.box[3], leaf);
        leaf.resize(cm.edge.size);
        for (unsigned i = 0; i < cm.edge.size; ++i) {
            const Vec2u g = cm.edge[i];
            Vec3f y[2] = {v[g[0]], v[g[1]]};
            const EdgeParam &ep = cm.param_arrays.edge[cm.prop.edge[i].param_index];
            leaf[i] = leaf_box(y, y, 2, 1.0f, 0.5f * ep.ghat + ep.offset);
        }
        install_tree(bvh_storage::get_collision_mesh_bvh().edge,
                     contact::get_collision_mesh_edge_aabb(), trees.node[4], trees.box[4], leaf);
    }
};

RefPipe *g_pipe = nullptr;

void load3(std::vector<Vec3f> &dst, const float *src, unsigned n) {
    dst.resize(n);
    for (unsigned i = 0; i < n; ++i) dst[i] = Vec3f(src[3 * i], src[3 * i + 1], src[3 * i + 2]);
}

} // namespace

extern "C" {

// main.cu:159-180: the matrices and contact storage of one scene. The
// DataSet is read in place (its arrays are host memory here); the state
// arrays come from refpipe_state.
bool refpipe_init(const DataSet *ds, const ParamSet *param) {
    delete g_pipe;
    g_pipe = new RefPipe();
    RefPipe &p = *g_pipe;
    p.data = *ds;
    p.prm = *param;
    p.n = ds->vertex.curr.size;
    p.fill_grains();
    p.dyn = DynCSRMat::alloc(p.n, param->csrmat_max_nnz);
    p.fixed = FixedCSRMat::alloc(p.data.fixed_index_table, p.data.transpose_table);
    p.tmp_fixed = FixedCSRMat::alloc(p.data.fixed_index_table, p.data.transpose_table);
    contact::initialize(p.data, p.prm);
    p.build_collision_trees();
    return true;
}

// The step's start state and parameters; velocity as main.cu:376-390.
void refpipe_state(const float *curr, const float *prev, const ParamSet *param) {
    RefPipe &p = *g_pipe;
    p.prm = *param;
    load3(p.curr, curr, p.n);
    load3(p.prev, prev, p.n);
    p.data.vertex.curr = RefPipe::view(p.curr);
    p.data.vertex.prev = RefPipe::view(p.prev);
    p.velocity.resize(p.n);
    for (unsigned i = 0; i < p.n; ++i) p.velocity[i] = (p.curr[i] - p.prev[i]) / p.prm.prev_dt;
}

// One Newton system at eval_x (main.cu:713-874, the scene features in
// scope): inertia and per-vertex terms, elastic, stitches, strain limit,
// contact over trees at eval_x, analytic constraints. Returns the contact
// count.
unsigned refpipe_assemble(const float *eval_x, const float *target, float dt) {
    RefPipe &p = *g_pipe;
    load3(p.eval_x, eval_x, p.n);
    load3(p.target, target, p.n);
    Vec<Vec3f> ex = RefPipe::view(p.eval_x), tg = RefPipe::view(p.target),
               vel = RefPipe::view(p.velocity);
    p.dyn.clear();
    p.diag.assign(p.n, Mat3x3f::Zero());
    p.fixed.clear();
    p.force.assign(3 * (size_t)p.n, 0.0f);
    Vec<float> force = RefPipe::view(p.force);
    Vec<Mat3x3f> diag = RefPipe::view(p.diag);
    std::vector<TorqueGroupResult> torque(std::max(1u, p.data.constraint.torque_groups.size));
    Vec<TorqueGroupResult> torque_v = RefPipe::view(torque);
    energy::compute_torque_groups(p.data, ex, torque_v);
    energy::embed_momentum_force_hessian(p.data, ex, vel, dt, tg, force, diag, p.prm, torque_v);
    energy::embed_elastic_force_hessian(p.data, ex, force, p.fixed, dt, p.prm);
    if (p.data.constraint.stitch.size)
        energy::embed_stitch_force_hessian(p.data, ex, force, p.fixed, p.prm);
    p.tmp_fixed.copy(p.fixed);
    if (p.data.shell_face_count > 0)
        strainlimiting::embed_strainlimiting_force_hessian(p.data, ex, force, p.tmp_fixed,
                                                           p.fixed, p.prm);
    if (p.data.rod_count > 0)
        strainlimiting::embed_rod_strainlimiting_force_hessian(p.data, ex, force, p.tmp_fixed,
                                                               p.fixed, p.prm);
    unsigned num = 0;
    if (!p.prm.disable_contact) {
        p.build_trees(p.eval_x, p.eval_x, 1.0f);
        unsigned max_nnz_row = 0;
        float consumed = 0.0f;
        num += contact::embed_contact_force_hessian(p.data, ex, force, p.tmp_fixed, p.fixed,
                                                    p.dyn, max_nnz_row, consumed, dt, p.prm);
    }
    num += contact::embed_constraint_force_hessian(p.data, ex, force, p.tmp_fixed, p.fixed, dt,
                                                   p.prm);
    p.num_contact = num;
    return num;
}

// Every stored block of the last system, upper triangle (row <= col):
// fixed pattern, contact rows, then the per-vertex diagonal. A (row, col) may
// repeat; the matrix is the sum. Returns the count; copies when row != null.
unsigned refpipe_blocks(unsigned *row, unsigned *col, float *val) {
    RefPipe &p = *g_pipe;
    unsigned k = 0;
    auto put = [&](unsigned i, unsigned j, const Mat3x3f &m) {
        if (row) {
            row[k] = i;
            col[k] = j;
            std::memcpy(val + 9 * (size_t)k, &m, 36);
        }
        ++k;
    };
    const VecVec<unsigned> &ix = p.fixed.index;
    for (unsigned i = 0; i < ix.size; ++i)
        for (unsigned s = ix.offset[i]; s < ix.offset[i + 1]; ++s)
            put(i, ix.data[s], p.fixed.value.data[s]);
    for (unsigned i = 0; i < p.dyn.rows.size; ++i) {
        const Row &r = p.dyn.rows.data[i];
        for (unsigned s = 0; s < r.head; ++s) put(i, r.index[s], r.value[s]);
    }
    for (unsigned i = 0; i < p.n; ++i) put(i, i, p.diag[i]);
    return k;
}

void refpipe_force(float *out) {
    std::memcpy(out, g_pipe->force.data(), g_pipe->force.size() * sizeof(float));
}

// main.cu:1213-1250: trees swept from x0 to x0 + T (x1 - x0), then the
// contact line search; the fraction of x1 - x0 it allows.
float refpipe_line_search(const float *a, const float *b, unsigned *pin_bad, int *overlap) {
    RefPipe &p = *g_pipe;
    load3(p.x0, a, p.n);
    load3(p.x1, b, p.n);
    p.build_trees(p.x0, p.x1, p.prm.line_search_max_t);
    contact::clear_ccd_overlap();
    unsigned pin = 0xFFFFFFFFu;
    const float toi = contact::line_search(p.data, RefPipe::view(p.x0), RefPipe::view(p.x1),
                                           p.prm, &pin);
    *pin_bad = pin;
    *overlap = contact::ccd_overlap_detected() ? 1 : 0;
    return toi;
}

// main.cu:1320-1325: the shells' strain-limit line search from x0 to x1.
float refpipe_strain_line_search(const float *a, const float *b) {
    RefPipe &p = *g_pipe;
    load3(p.x0, a, p.n);
    load3(p.x1, b, p.n);
    std::vector<float> tmp(std::max(1u, p.data.shell_face_count));
    Vec<float> tmp_v = RefPipe::view(tmp);
    return strainlimiting::line_search(p.data, RefPipe::view(p.x1), RefPipe::view(p.x0), tmp_v,
                                       p.prm);
}

// main.cu:1336-1341: the rods' strain-limit line search from x0 to x1.
float refpipe_rod_strain_line_search(const float *a, const float *b) {
    RefPipe &p = *g_pipe;
    load3(p.x0, a, p.n);
    load3(p.x1, b, p.n);
    std::vector<float> tmp(std::max(1u, p.data.rod_count));
    Vec<float> tmp_v = RefPipe::view(tmp);
    return strainlimiting::rod_line_search(p.data, RefPipe::view(p.x1), RefPipe::view(p.x0),
                                           tmp_v, p.prm);
}

// main.cu:1519-1536: trees at x, then the intersection check.
bool refpipe_check_intersection(const float *x) {
    RefPipe &p = *g_pipe;
    load3(p.x0, x, p.n);
    p.build_trees(p.x0, p.x0, 1.0f);
    return contact::check_intersection(p.data, RefPipe::view(p.x0), p.prm);
}

} // extern "C"
