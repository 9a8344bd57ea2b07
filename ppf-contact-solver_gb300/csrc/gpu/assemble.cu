// assemble.cu -- Newton system assembly kernels.
//
// Stage order follows crates/ppf-cts-solver/src/cpp/main/main.cu:713-1049:
// inertia / air / pull -> membrane + bending -> (copy elastic Hessian) ->
// strain limit -> contact (detect, dedupe blocks, assemble) -> sphere / floor
// -> Dirichlet elimination. Element formulas live in ../physics (shared with
// the CPU oracle); these kernels gather, evaluate and scatter.
#include "../physics/bw.cuh"
#include "../physics/elastic.cuh"
#include "../physics/hinge.cuh"
#include "../physics/rod.cuh"
#include "../physics/strainlimit.cuh"
#include "assemble.cuh"

namespace ppf {
namespace gpu {

namespace {

constexpr unsigned kB = 256;
constexpr unsigned long long kEmptyKey = 0xFFFFFFFFFFFFFFFFull;

__device__ __forceinline__ void atomic_add_block(float *dst, const Mat3 &m) {
#pragma unroll
    for (int k = 0; k < 9; ++k) {
        float v = m.m[k];
        if (v != 0.0f) atomicAdd(dst + k, v);
    }
}

__device__ __forceinline__ Mat3 load_block(const float *p) { return load_mat3(p); }

__device__ __forceinline__ Mat2 load_inv_rest(const float *p) {
    Mat2 m;
    m.m[0] = p[0];
    m.m[1] = p[1];
    m.m[2] = p[2];
    m.m[3] = p[3];
    return m;
}

// ---- inertia, air drag, pull pins (energy.cu:182-270, 700-716) ------------
__global__ void k_vertex_energy(Scene s, AssemblyBuffers b) {
    const StepParams &p = *b.params;
    unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= s.n) return;
    const PpfVertexProp &vp = s.vprop[i];
    if (vp.fix_index != 0) return;
    const float dt = p.dt, dt2 = dt * dt;
    Vec3 x = X(b.x0, i), y = X(b.x, i);
    Vec3 normal = Vec3::zero();
    for (unsigned k = s.vf_off[i]; k < s.vf_off[i + 1]; ++k) {
        const unsigned *f = s.face + 3 * s.vf[k];
        Vec3 z0 = X(b.x, f[0]), z1 = X(b.x, f[1]), z2 = X(b.x, f[2]);
        normal += cross(z1 - z0, z2 - z0);
    }
    if (normal.squared_norm()) normal.normalize();
    Vec3 wind = Vec3::zero();
    if (!p.inactive_momentum) {
        float ang = 30.0f * p.time;
        float w = 0.25f * (0.5f * (1.0f + sinf(ang))) + (1.0f - 0.25f);
        wind = w * vec3(p.wind[0], p.wind[1], p.wind[2]);
    }
    Vec3 f = Vec3::zero();
    Mat3 H = Mat3::zero();
    if (!normal.is_zero() && p.air_density) {
        Vec3 z = (y - x) - dt * wind;
        Mat3 P = Mat3::identity() - outer<3>(normal, normal);
        Vec3 g = (normal * normal.dot(z)) / dt2 + ((p.air_friction * P) * z) / dt2;
        Mat3 h = outer<3>(normal, normal) / dt2 + (p.air_friction * P) / dt2;
        float s0 = vp.area * p.air_density;
        f += s0 * g;
        H += s0 * h;
    }
    bool pulled = false;
    if (vp.pull_index > 0) {
        const PpfPullPair &pp = s.pull[vp.pull_index - 1];
        Vec3 pos = vec3(pp.position.v[0], pp.position.v[1], pp.position.v[2]);
        f += pp.weight * (y - pos);
        H += pp.weight * Mat3::identity();
        pulled = true;
    }
    if (!pulled) {
        Vec3 t = X(b.target, i);
        f += vp.mass * ((y - t) / dt2);
        H += vp.mass * (Mat3::identity() / dt2);
    }
    if (p.isotropic_air_friction) {
        f += (p.isotropic_air_friction * (y - x)) / dt2;
        H += (p.isotropic_air_friction / dt2) * Mat3::identity();
    }
    if (p.fix_xz && y[1] > p.fix_xz) {
        float t = fminf(1.0f, y[1] - p.fix_xz);
        Mat3 P = Mat3::identity();
        P(1, 1) = 0.0f;
        f += ((P * t) * vp.mass) * (y - x) / dt2;
        H += (P * t) * vp.mass * dt2;
    }
    float *fo = b.force + 3 * i;
    fo[0] += f[0];
    fo[1] += f[1];
    fo[2] += f[2];
    float *d = b.diag + 9 * i;
#pragma unroll
    for (int k = 0; k < 9; ++k) d[k] += H.m[k];
}

// ---- Baraff-Witkin membrane (energy.cu:304-364) ----------------------------
// Displacement of an element's N vertices over the step, x - x_start.
template <int N>
__device__ __forceinline__ Vec<3 * N> step_displacement(const AssemblyBuffers &b,
                                                         const unsigned (&v)[N]) {
    Vec<3 * N> u;
#pragma unroll
    for (int k = 0; k < N; ++k) {
        const Vec3 d = X(b.x, v[k]) - X(b.x0, v[k]);
        u[3 * k] = d[0];
        u[3 * k + 1] = d[1];
        u[3 * k + 2] = d[2];
    }
    return u;
}

// Scatters an element's N x N Hessian blocks through its slot table
// (sentinel: a lower-triangle block, which the upper pattern does not hold).
template <int N>
__device__ __forceinline__ void scatter_blocks(float *fixed_val, const unsigned *slot,
                                               const Mat<3 * N, 3 * N> &H) {
    for (int a = 0; a < N; ++a)
        for (int c = 0; c < N; ++c) {
            const unsigned sl = slot[N * a + c];
            if (sl != kSentinel)
                atomic_add_block(fixed_val + 9 * (size_t)sl, H.template block<3, 3>(3 * a, 3 * c));
        }
}

__global__ void k_face_energy(Scene s, AssemblyBuffers b) {
    const StepParams &p = *b.params;
    unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= s.nf_shell) return;
    const PpfFaceProp &pr = s.fprop[i];
    if (pr.fixed || pr.rest_excluded || pr.collider) return;
    const PpfFaceParam &fp = s.fparam[pr.param_index];
    if (!(fp.mu > 0.0f)) return;
    const unsigned *f = s.face + 3 * i;
    Mat3 dedx;
    Mat9 H;
    if (fp.model == PPF_MODEL_BARAFF_WITKIN) {
        bw::membrane(X(b.x, f[0]), X(b.x, f[1]), X(b.x, f[2]),
                     load_inv_rest(s.inv_rest + 4 * i), fp.mu, fp.lambda, pr.mass, dedx, H);
    } else if (!elastic::shell(X(b.x, f[0]), X(b.x, f[1]), X(b.x, f[2]),
                               load_inv_rest(s.inv_rest + 4 * i), fp.model, fp.mu, fp.lambda,
                               pr.mass, p.eiganalysis_eps, dedx, H)) {
        return;
    }
    if (fp.deform_damping > 0.0f) { // energy.cu:359-360
        const unsigned v[3] = {f[0], f[1], f[2]};
        damping::stiffness<3>(fp.deform_damping, p.dt, step_displacement<3>(b, v), dedx, H);
    }
    for (int a = 0; a < 3; ++a) atomic_add3(b.force + 3 * f[a], dedx.col(a));
    const unsigned *slot = s.face_slot + 9 * i;
    for (int a = 0; a < 3; ++a)
        for (int c = 0; c < 3; ++c) {
            unsigned sl = slot[3 * a + c];
            if (sl != kSentinel)
                atomic_add_block(b.fixed_val + 9 * (size_t)sl, H.block<3, 3>(3 * a, 3 * c));
        }
}

// ---- dihedral bending (energy.cu:448-553) ----------------------------------
__global__ void k_hinge_energy(Scene s, AssemblyBuffers b) {
    const StepParams &p = *b.params;
    unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= s.nh) return;
    const PpfHingeProp &pr = s.hprop[i];
    if (pr.fixed || pr.collider || (s.hinge_type[i] & 1u)) return;
    const PpfHingeParam &hp = s.hparam[pr.param_index];
    const unsigned *h = s.hinge + 4 * i;
    float rho = 0.0f;
    int cnt = 0;
    for (int k = 0; k < 4; ++k) {
        float a = s.vprop[h[k]].area;
        if (a > 0.0f) {
            rho += s.vprop[h[k]].mass / a;
            ++cnt;
        }
    }
    if (cnt > 0) rho /= cnt;
    float k = hinge::stiffness(hp.bend, hp.bend_warp, hp.bend_weft, pr.uv_edge_sin2,
                               pr.length, pr.area, rho);
    if (!(k > 0.0f)) return;
    const unsigned r[4] = {h[2], h[1], h[0], h[3]};
    Mat3x4 dedx;
    Mat12 H;
    hinge::force_hessian(X(b.x, r[0]), X(b.x, r[1]), X(b.x, r[2]), X(b.x, r[3]),
                         pr.rest_angle, dedx, H);
    dedx *= k;
    H *= k;
    if (hp.bend_damping > 0.0f) { // lagged, at the start-of-step positions (energy.cu:528-540)
        Mat3x4 f_lag;
        Mat12 K_lag;
        hinge::force_hessian(X(b.x0, r[0]), X(b.x0, r[1]), X(b.x0, r[2]), X(b.x0, r[3]),
                             pr.rest_angle, f_lag, K_lag);
        K_lag *= k;
        damping::lagged<4>(hp.bend_damping, p.dt, step_displacement<4>(b, r), K_lag, dedx, H);
    }
    for (int a = 0; a < 4; ++a) atomic_add3(b.force + 3 * r[a], dedx.col(a));
    const unsigned *slot = s.hinge_slot + 16 * i;
    for (int a = 0; a < 4; ++a)
        for (int c = 0; c < 4; ++c) {
            unsigned sl = slot[4 * a + c];
            if (sl != kSentinel)
                atomic_add_block(b.fixed_val + 9 * (size_t)sl, H.block<3, 3>(3 * a, 3 * c));
        }
}

// ---- rod stretch (energy.cu:272-302) ---------------------------------------
__global__ void k_rod_energy(Scene s, AssemblyBuffers b) {
    const StepParams &p = *b.params;
    unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= s.nr) return;
    const PpfEdgeProp &pr = s.eprop[i];
    if (pr.fixed) return;
    const PpfEdgeParam &ep = s.eparam[pr.param_index];
    if (!(ep.stiffness > 0.0f)) return;
    const unsigned v[2] = {s.edge[2 * i], s.edge[2 * i + 1]};
    Mat3x2 dedx;
    Mat6 H;
    rod::stretch(X(b.x, v[0]), X(b.x, v[1]), pr.length, ep.stiffness * pr.mass, dedx, H);
    if (ep.deform_damping > 0.0f)
        damping::stiffness<2>(ep.deform_damping, p.dt, step_displacement<2>(b, v), dedx, H);
    for (int a = 0; a < 2; ++a) atomic_add3(b.force + 3 * v[a], dedx.col(a));
    scatter_blocks<2>(b.fixed_val, s.edge_slot + 4 * i, H);
}

// ---- rod bending at an interior rod vertex (energy.cu:555-641) -------------
__global__ void k_rod_bend(Scene s, AssemblyBuffers b) {
    const StepParams &p = *b.params;
    unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= s.n_surf) return;
    const PpfVertexProp &vp = s.vprop[i];
    if (vp.fix_index != 0) return;
    if (s.ve_off[i + 1] - s.ve_off[i] != 2 || s.vf_off[i + 1] != s.vf_off[i]) return;
    const unsigned e0 = s.ve[s.ve_off[i]], e1 = s.ve[s.ve_off[i] + 1];
    const PpfEdgeParam &p0 = s.eparam[s.eprop[e0].param_index];
    const PpfEdgeParam &p1 = s.eparam[s.eprop[e1].param_index];
    const float bend = 0.5f * (p0.bend + p1.bend);
    const float bend_damping = 0.5f * (p0.bend_damping + p1.bend_damping);
    const float k = rod::bend_stiffness(bend, vp.mass, s.eprop[e0].length, s.eprop[e1].length);
    if (!(vp.mass > 0.0f && k > 0.0f)) return;
    const unsigned *E0 = s.edge + 2 * e0, *E1 = s.edge + 2 * e1;
    const unsigned v[3] = {E0[0] == i ? E0[1] : E0[0], i, E1[0] == i ? E1[1] : E1[0]};
    Mat3 dedx;
    Mat9 H;
    rod::bend(X(b.x, v[0]), X(b.x, v[1]), X(b.x, v[2]), vp.rest_bend_angle, dedx, H);
    dedx *= k;
    H *= k;
    if (bend_damping > 0.0f) {
        Mat3 f_lag;
        Mat9 K_lag;
        rod::bend(X(b.x0, v[0]), X(b.x0, v[1]), X(b.x0, v[2]), vp.rest_bend_angle, f_lag, K_lag);
        K_lag *= k;
        damping::lagged<3>(bend_damping, p.dt, step_displacement<3>(b, v), K_lag, dedx, H);
    }
    for (int a = 0; a < 3; ++a) atomic_add3(b.force + 3 * v[a], dedx.col(a));
    scatter_blocks<3>(b.fixed_val, s.bend_slot + 9 * (size_t)i, H);
}

// ---- stitches (energy.cu:796-884) ---------------------------------------------
__global__ void k_stitch_energy(Scene s, AssemblyBuffers b) {
    const StepParams &p = *b.params;
    unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= s.nstitch) return;
    const PpfStitch &st = s.stitch[i];
    Vec3 x[6];
    float w[6], ghat = 0.0f;
    float off_src = -INFINITY, off_tgt = -INFINITY;
    for (int a = 0; a < 6; ++a) {
        const unsigned v = st.index.v[a];
        x[a] = X(b.x, v);
        w[a] = st.weight.v[a];
        const PpfVertexParam &vp = s.vparam[s.vprop[v].param_index];
        ghat += w[a] * vp.ghat;
        if (a < 3) off_src = a ? fmaxf(off_src, vp.offset) : vp.offset;
        else off_tgt = a > 3 ? fmaxf(off_tgt, vp.offset) : vp.offset;
    }
    const float l0 = ghat / 2.0f;
    const float l_cap = p.stitch_length_factor * l0 + off_src + off_tgt;
    Mat<3, 6> dedx;
    Mat<18, 18> H;
    stitch::spring(x, w, l0, l_cap, dedx, H);
    for (int a = 0; a < 6; ++a) atomic_add3(b.force + 3 * st.index.v[a], st.stiffness * dedx.col(a));
    H *= st.stiffness;
    scatter_blocks<6>(b.fixed_val, s.stitch_slot + 36 * (size_t)i, H);
}

// ---- solids (energy.cu:395-446) ------------------------------------------------
__global__ void k_tet_energy(Scene s, AssemblyBuffers b) {
    const StepParams &p = *b.params;
    unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= s.nt) return;
    const PpfTetProp &pr = s.tprop[i];
    if (pr.fixed || pr.rest_excluded) return;
    const PpfTetParam &tp = s.tparam[pr.param_index];
    if (!(tp.mu > 0.0f)) return;
    const unsigned v[4] = {s.tet[4 * i], s.tet[4 * i + 1], s.tet[4 * i + 2], s.tet[4 * i + 3]};
    const Mat3 inv = load_mat3(s.inv_rest3 + 9 * (size_t)i);
    Mat3x4 dedx;
    Mat12 H;
    if (!elastic::tet(X(b.x, v[0]), X(b.x, v[1]), X(b.x, v[2]), X(b.x, v[3]), inv, tp.model,
                      tp.mu, tp.lambda, pr.mass, p.eiganalysis_eps, dedx, H))
        return;
    if (tp.deform_damping > 0.0f)
        damping::stiffness<4>(tp.deform_damping, p.dt, step_displacement<4>(b, v), dedx, H);
    for (int a = 0; a < 4; ++a) atomic_add3(b.force + 3 * v[a], dedx.col(a));
    scatter_blocks<4>(b.fixed_val, s.tet_slot + 16 * (size_t)i, H);
}

// ---- strain-limit barrier (strainlimiting.cu:46-98) -------------------------
__global__ void k_strain_limit(Scene s, AssemblyBuffers b) {
    const StepParams &p = *b.params;
    unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= s.nf_shell) return;
    const PpfFaceProp &pr = s.fprop[i];
    const PpfFaceParam &fp = s.fparam[pr.param_index];
    if (pr.fixed || pr.rest_excluded || !(fp.strainlimit > 0.0f)) return;
    float limit = strain::effective_limit(fp.strainlimit, fp.shrink_x, fp.shrink_y);
    const unsigned *f = s.face + 3 * i;
    Mat2 inv = load_inv_rest(s.inv_rest + 4 * i);
    Mat3x2 F = bw::deformation_grad(X(b.x, f[0]), X(b.x, f[1]), X(b.x, f[2]), inv);
    strain::Svd32 sv;
    Mat3 dedx;
    Mat9 H;
    if (!strain::face_barrier(F, inv, fp.strainlimit, p.barrier, p.eiganalysis_eps, sv,
                              dedx, H))
        return;
    Mat9 local;
    for (int a = 0; a < 3; ++a)
        for (int c = 0; c < 3; ++c)
            local.set_block<3, 3>(3 * a, 3 * c, fixed_block(s, b.fixed_tmp, f[a], f[c]));
    float k = strain::stiffness(X(b.x0, f[0]), X(b.x0, f[1]), X(b.x0, f[2]), local,
                                pr.mass, sv.S.max_coeff(), limit);
    Mat3 kf = k * dedx;
    Mat9 kH = k * H;
    for (int a = 0; a < 3; ++a) atomic_add3(b.force + 3 * f[a], kf.col(a));
    const unsigned *slot = s.face_slot + 9 * i;
    for (int a = 0; a < 3; ++a)
        for (int c = 0; c < 3; ++c) {
            unsigned sl = slot[3 * a + c];
            if (sl != kSentinel)
                atomic_add_block(b.fixed_val + 9 * (size_t)sl, kH.block<3, 3>(3 * a, 3 * c));
        }
}

// ---- rod strain-limit barrier (strainlimiting.cu:122-190) --------------------
__global__ void k_rod_strain_limit(Scene s, AssemblyBuffers b) {
    const StepParams &p = *b.params;
    unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= s.nr) return;
    const PpfEdgeProp &pr = s.eprop[i];
    const PpfEdgeParam &ep = s.eparam[pr.param_index];
    if (pr.fixed || !(ep.strainlimit > 0.0f)) return;
    const float l0 = pr.initial_length;
    if (l0 <= 0.0f) return;
    const unsigned v[2] = {s.edge[2 * i], s.edge[2 * i + 1]};
    float g;
    Vec6 f;
    Mat6 H;
    if (!rod::strain_barrier(X(b.x, v[0]), X(b.x, v[1]), l0, ep.strainlimit, p.barrier, g, f, H))
        return;
    Mat6 local;
    for (int a = 0; a < 2; ++a)
        for (int c = 0; c < 2; ++c)
            local.set_block<3, 3>(3 * a, 3 * c, fixed_block(s, b.fixed_tmp, v[a], v[c]));
    const float k = rod::strain_stiffness(X(b.x0, v[0]), X(b.x0, v[1]), local, pr.mass, g,
                                          ep.strainlimit);
    H = k * H;
    f = k * f;
    atomic_add3(b.force + 3 * v[0], vec3(f[0], f[1], f[2]));
    atomic_add3(b.force + 3 * v[1], vec3(f[3], f[4], f[5]));
    scatter_blocks<2>(b.fixed_val, s.edge_slot + 4 * i, H);
}

// ---- contact detection (contact.cu:1398-1787, stage 0) ----------------------
// The trees are refit to tight boxes at the evaluated positions before this
// runs (the reference queries the swept boxes left by the last line search).
// A pair passes the distance test only if its tight boxes overlap in exact
// arithmetic; the query is widened by this guard so fp32 rounding of the box
// corners cannot drop a pair at the threshold. The accepted set is decided by
// the distance test alone, as in the reference.
__device__ __forceinline__ float detect_guard(const Vec3 &p) {
    return 1e-6f * (1.0f + fmaxf(fmaxf(fabsf(p[0]), fabsf(p[1])), fabsf(p[2])));
}

__device__ __forceinline__ unsigned push_pair(unsigned *ctr, unsigned cap) {
    return push_slot(ctr, cap);
}

struct VertexQueryOp {
    const Scene &s;
    const float *x;
    unsigned v;
    int kind; // 0 face, 1 edge, 2 vertex
    PairLists &pl;
    IterStatus *st;
    unsigned found;
    // a point-point pair is kept from its higher-index vertex
    __device__ bool pre(unsigned prim) const { return kind != 2 || prim < v; }
    __device__ void operator()(unsigned prim) {
        if (kind == 0) {
            if (accept_point_face(s, x, v, prim)) {
                unsigned k = push_pair(&st->n_pf, pl.cap_pf);
                if (k != kSentinel) pl.pf[k] = make_uint2(v, prim);
                ++found;
            }
        } else if (kind == 1) {
            bool fr = true;
            Vec2 c;
            unsigned cnt = accept_point_edge(s, x, v, prim, &fr, &c);
            if (cnt) {
                unsigned k = push_pair(&st->n_pe, pl.cap_pe);
                if (k != kSentinel) pl.pe[k] = make_uint3(v, prim, cnt | (fr ? 0x80000000u : 0u));
                ++found;
            }
        } else {
            bool fr = true;
            unsigned cnt = accept_point_point(s, x, v, prim, &fr);
            if (cnt) {
                unsigned k = push_pair(&st->n_pp, pl.cap_pp);
                if (k != kSentinel) pl.pp[k] = make_uint3(v, prim, cnt | (fr ? 0x80000000u : 0u));
                ++found;
            }
        }
    }
};

// One lane per surface vertex, in the vertex tree's Morton order, so a warp's
// queries are neighbours in space; all lanes of a warp query together.
template <LeafTests M>
__global__ void k_detect_vertex(Scene s, BvhView fb, BvhView eb, BvhView vb,
                                const float *x, PairLists pl, IterStatus *st) {
    const unsigned t = blockIdx.x * blockDim.x + threadIdx.x;
    const bool act = t < s.n_surf;
    const unsigned v = act ? vb.node[t].x - 1u : 0u;
    float4 qmin = make_float4(0.0f, 0.0f, 0.0f, 0.0f), qmax = qmin;
    if (act) {
        Vec3 p = X(x, v);
        float m = s.margin_vert[v] + detect_guard(p);
        qmin = make_float4(p[0] - m, p[1] - m, p[2] - m, 1.0f);
        qmax = make_float4(p[0] + m, p[1] + m, p[2] + m, 0.0f);
    }
    VertexQueryOp op{s, x, v, 0, pl, st, 0u};
    warp_query<M>(fb, act, qmin, qmax, op, &st->status);
    op.kind = 1;
    warp_query<M>(eb, act, qmin, qmax, op, &st->status);
    op.kind = 2;
    warp_query<M>(vb, act, qmin, qmax, op, &st->status);
    if (op.found) atomicAdd(&st->n_contact, op.found);
}

struct EdgeQueryOp {
    const Scene &s;
    const float *x;
    unsigned e;
    PairLists &pl;
    IterStatus *st;
    unsigned found;
    // accept_edge_edge keeps the pair with the query edge first
    __device__ bool pre(unsigned other) const { return e < other; }
    __device__ void operator()(unsigned other) {
        if (accept_edge_edge(s, x, e, other)) {
            unsigned k = push_pair(&st->n_ee, pl.cap_ee);
            if (k != kSentinel) pl.ee[k] = make_uint2(e, other);
            ++found;
        }
    }
};

// One work item per edge piece (edges in the tree's Morton order).
// Work items (edge pieces in the tree's Morton order) are taken a warp at a
// time; a piece after the first excludes the leaves its predecessor reports.
template <LeafTests M>
__global__ void k_detect_edge(Scene s, BvhView eb, const float *x, PairLists pl,
                              IterStatus *st, EdgePieces ep) {
    const unsigned total = ep.off[ep.n];
    for (WarpItems w; w.base < total; w.base += w.stride) {
        const unsigned item = w.base + w.lane;
        const bool act = item < total;
        unsigned e = 0u;
        float4 qmin = make_float4(0.0f, 0.0f, 0.0f, 0.0f), qmax = qmin;
        float4 xmin = make_float4(0.0f, 0.0f, 0.0f, 0.0f), xmax = xmin;
        bool excl = false;
        if (act) {
            const unsigned t = piece_slot(ep, item);
            const unsigned k = item - ep.off[t], K = ep.off[t + 1] - ep.off[t];
            e = eb.node[t].x - 1u;
            const unsigned *ed = s.edge + 2 * e;
            Vec3 a = X(x, ed[0]), c = X(x, ed[1]);
            float m = s.margin_edge[e] + fmaxf(detect_guard(a), detect_guard(c));
            seg_box(piece_point(a, c, k, K), piece_point(a, c, k + 1, K), m, qmin, qmax);
            if (k > 0u) {
                seg_box(piece_point(a, c, k - 1, K), piece_point(a, c, k, K), m, xmin, xmax);
                excl = true;
            }
        }
        EdgeQueryOp op{s, x, e, pl, st, 0u};
        // a lane without an exclusion box gets one that overlaps nothing
        if (!excl) xmin.w = 0.0f;
        warp_query<M>(eb, act, qmin, qmax, op, &st->status, &xmin, &xmax);
        if (op.found) atomicAdd(&st->n_contact, op.found);
    }
}

// Piece counts of every edge (tree order) for a query over positions x, or
// over the sweep x -> x + t (x1 - x) when x1 is given (t read from t_bits).
__global__ void k_edge_piece_count(unsigned ne, const uint2 *node, const unsigned *edge,
                                   const float *x, const float *x1, const unsigned *t_bits,
                                   float piece_len, unsigned *count) {
    unsigned t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= ne) return;
    const unsigned e = node[t].x - 1u;
    const unsigned *ed = edge + 2 * e;
    Vec3 a = X(x, ed[0]), b = X(x, ed[1]);
    float len = (b - a).norm();
    if (x1) {
        const float tt = __uint_as_float(*t_bits);
        Vec3 a1 = vec3(fmaf(tt, x1[3 * ed[0]] - a[0], a[0]), fmaf(tt, x1[3 * ed[0] + 1] - a[1], a[1]),
                       fmaf(tt, x1[3 * ed[0] + 2] - a[2], a[2]));
        Vec3 b1 = vec3(fmaf(tt, x1[3 * ed[1]] - b[0], b[0]), fmaf(tt, x1[3 * ed[1] + 1] - b[1], b[1]),
                       fmaf(tt, x1[3 * ed[1] + 2] - b[2], b[2]));
        len = fmaxf(len, (b1 - a1).norm());
    }
    count[t] = piece_count(len, piece_len);
}

// ---- dynamic contact blocks: hash dedupe + CSR layout ----------------------
__device__ __forceinline__ unsigned hash_key(unsigned long long k) {
    k ^= k >> 33;
    k *= 0xff51afd7ed558ccdull;
    k ^= k >> 33;
    k *= 0xc4ceb9fe1a85ec53ull;
    k ^= k >> 33;
    return (unsigned)k;
}

__device__ void hash_insert(DynMatrix &dm, unsigned long long key, IterStatus *st) {
    // past the block capacity the iteration is repeated with a larger one:
    // stop inserting (the table, sized at least twice the capacity plus the
    // threads in flight, never fills)
    if (*(volatile unsigned *)&st->n_dyn > dm.cap) return;
    unsigned mask = dm.hcap - 1u;
    unsigned h = hash_key(key) & mask;
    for (unsigned probe = 0; probe < dm.hcap; ++probe) {
        unsigned long long prev = atomicCAS(&dm.hkey[h], kEmptyKey, key);
        if (prev == kEmptyKey) {
            atomicAdd(&st->n_dyn, 1u);
            return;
        }
        if (prev == key) return;
        h = (h + 1u) & mask;
    }
    // a full table: more blocks than the capacity it was sized for
    atomicOr(&st->status, STATUS_PAIR_OVERFLOW);
}

__device__ unsigned hash_find(const DynMatrix &dm, unsigned long long key) {
    unsigned mask = dm.hcap - 1u;
    unsigned h = hash_key(key) & mask;
    for (unsigned probe = 0; probe < dm.hcap; ++probe) {
        unsigned long long k = dm.hkey[h];
        if (k == key) return dm.hval[h];
        if (k == kEmptyKey) return kSentinel;
        h = (h + 1u) & mask;
    }
    return kSentinel;
}

template <int N>
__device__ void insert_pair_keys(const Scene &s, DynMatrix &dm, const unsigned (&idx)[N],
                                 IterStatus *st) {
#pragma unroll
    for (int a = 0; a < N; ++a)
#pragma unroll
        for (int c = 0; c < N; ++c) {
            unsigned i = idx[a], j = idx[c];
            if (i < j && fixed_slot(s, i, j) == kSentinel)
                hash_insert(dm, ((unsigned long long)i << 32) | j, st);
        }
}

__device__ __forceinline__ void pair_indices_pf(const Scene &s, uint2 pr, unsigned (&idx)[4]) {
    const unsigned *f = s.face + 3 * pr.y;
    idx[0] = pr.x;
    idx[1] = f[0];
    idx[2] = f[1];
    idx[3] = f[2];
}
__device__ __forceinline__ void pair_indices_pe(const Scene &s, uint3 pr, unsigned (&idx)[3]) {
    const unsigned *e = s.edge + 2 * pr.y;
    idx[0] = pr.x;
    idx[1] = e[0];
    idx[2] = e[1];
}
__device__ __forceinline__ void pair_indices_ee(const Scene &s, uint2 pr, unsigned (&idx)[4]) {
    const unsigned *a = s.edge + 2 * pr.x;
    const unsigned *c = s.edge + 2 * pr.y;
    idx[0] = a[0];
    idx[1] = a[1];
    idx[2] = c[0];
    idx[3] = c[1];
}

// Pair counts as detected, clamped to the lists' capacities; none in an
// iteration flagged for a repeat (a list or the block capacity overran).
struct PairCounts {
    unsigned pf = 0, pe = 0, pp = 0, ee = 0;
    __device__ __forceinline__ PairCounts(const PairLists &pl, const IterStatus *st) {
        if (st->status & STATUS_PAIR_OVERFLOW) return;
        pf = min(st->n_pf, pl.cap_pf);
        pe = min(st->n_pe, pl.cap_pe);
        pp = min(st->n_pp, pl.cap_pp);
        ee = min(st->n_ee, pl.cap_ee);
    }
};

__global__ void k_dyn_insert(Scene s, PairLists pl, DynMatrix dm, IterStatus *st) {
    const PairCounts n(pl, st);
    unsigned t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < n.pf) {
        unsigned idx[4];
        pair_indices_pf(s, pl.pf[t], idx);
        insert_pair_keys<4>(s, dm, idx, st);
        return;
    }
    t -= n.pf;
    if (t < n.pe) {
        unsigned idx[3];
        pair_indices_pe(s, pl.pe[t], idx);
        insert_pair_keys<3>(s, dm, idx, st);
        return;
    }
    t -= n.pe;
    if (t < n.pp) {
        unsigned idx[2] = {pl.pp[t].x, pl.pp[t].y};
        insert_pair_keys<2>(s, dm, idx, st);
        return;
    }
    t -= n.pp;
    if (t < n.ee) {
        unsigned idx[4];
        pair_indices_ee(s, pl.ee[t], idx);
        insert_pair_keys<4>(s, dm, idx, st);
    }
}

// Zeroes the values of the n_dyn unique contact blocks (grid-stride).
__global__ void k_zero_dyn_val(DynMatrix dm, const IterStatus *st) {
    const size_t m = 9 * (size_t)min(st->n_dyn, dm.cap);
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < m;
         e += (size_t)gridDim.x * blockDim.x)
        dm.val[e] = 0.0f;
}

// Marks an iteration whose pair lists were too short for what detection
// found: its pair sets were cut at the capacities, so the host grows the
// lists and repeats the iteration (the step's rescale turns it into a no-op).
__global__ void k_pair_capacity(PairLists pl, IterStatus *st) {
    if (st->n_pf > pl.cap_pf || st->n_pe > pl.cap_pe || st->n_pp > pl.cap_pp ||
        st->n_ee > pl.cap_ee)
        atomicOr(&st->status, STATUS_PAIR_OVERFLOW);
}

// More unique contact blocks than the block capacity: flag the iteration for
// a repeat with a larger one, and leave the contact CSR empty (the counts and
// the fill below skip a flagged iteration, the pair kernels see no pairs).
__global__ void k_dyn_capacity(DynMatrix dm, IterStatus *st) {
    if (st->n_dyn > dm.cap) atomicOr(&st->status, STATUS_PAIR_OVERFLOW);
}

__global__ void k_dyn_count(DynMatrix dm, const IterStatus *st) {
    unsigned h = blockIdx.x * blockDim.x + threadIdx.x;
    if (h >= dm.hcap || (st->status & STATUS_PAIR_OVERFLOW)) return;
    unsigned long long k = dm.hkey[h];
    if (k == kEmptyKey) return;
    atomicAdd(&dm.cnt[(unsigned)(k >> 32)], 1u);
    atomicAdd(&dm.cnt2[(unsigned)k], 1u);
}

__global__ void k_dyn_fill(DynMatrix dm, const IterStatus *st) {
    unsigned h = blockIdx.x * blockDim.x + threadIdx.x;
    if (h >= dm.hcap || (st->status & STATUS_PAIR_OVERFLOW)) return;
    unsigned long long k = dm.hkey[h];
    if (k == kEmptyKey) return;
    unsigned r = (unsigned)(k >> 32), c = (unsigned)k;
    unsigned pos = dm.off[r] + atomicAdd(&dm.cnt[r], 1u);
    dm.col[pos] = c;
    dm.hval[h] = pos;
    unsigned tpos = dm.tr_off[c] + atomicAdd(&dm.cnt2[c], 1u);
    dm.tr[tpos] = make_uint2(r, pos);
}

// ---- contact pair assembly (contact.cu:262-354, stage 1) ---------------------
template <int N>
__device__ void scatter_pair(const Scene &s, const AssemblyBuffers &b, const DynMatrix &dm,
                             const unsigned (&idx)[N], const Mat<3, N> &f,
                             const Mat<3 * N, 3 * N> &H, IterStatus *st) {
#pragma unroll
    for (int a = 0; a < N; ++a) atomic_add3(b.force + 3 * idx[a], f.col(a));
#pragma unroll
    for (int a = 0; a < N; ++a)
#pragma unroll
        for (int c = 0; c < N; ++c) {
            unsigned i = idx[a], j = idx[c];
            if (i > j) continue;
            Mat3 blk = H.template block<3, 3>(3 * a, 3 * c);
            unsigned sl = fixed_slot(s, i, j);
            if (sl != kSentinel) {
                atomic_add_block(b.fixed_val + 9 * (size_t)sl, blk);
            } else {
                unsigned pos = hash_find(dm, ((unsigned long long)i << 32) | j);
                if (pos == kSentinel) {
                    atomicOr(&st->status, STATUS_BAD_SLOT);
                } else {
                    atomic_add_block(dm.val + 9 * (size_t)pos, blk);
                }
            }
        }
}

template <int N>
__device__ void assemble_pair(const Scene &s, const AssemblyBuffers &b,
                              const DynMatrix &dm, const unsigned (&idx)[N],
                              const float (&w)[N], float ghat, float offset, float mu,
                              bool friction_on, float count) {
    const StepParams &p = *b.params;
    Vec3 x[N], x0[N];
    float mass[N];
    Mat<3 * N, 3 * N> local;
#pragma unroll
    for (int a = 0; a < N; ++a) {
        x[a] = X(b.x, idx[a]);
        x0[a] = X(b.x0, idx[a]);
        mass[a] = s.vprop[idx[a]].mass;
    }
#pragma unroll
    for (int a = 0; a < N; ++a)
#pragma unroll
        for (int c = 0; c < N; ++c)
            local.template set_block<3, 3>(3 * a, 3 * c, fixed_block(s, b.fixed_tmp, idx[a], idx[c]));
    Mat<3, N> f;
    Mat<3 * N, 3 * N> H;
    contact::pair_force_hessian<N>(x, x0, w, mass, local, ghat, offset, p.barrier,
                                   friction_on, mu, p.friction_eps, count, f, H);
    scatter_pair<N>(s, b, dm, idx, f, H, b.st);
}

__global__ void k_assemble_pf(Scene s, AssemblyBuffers b, PairLists pl, DynMatrix dm) {
    const StepParams &p = *b.params;
    unsigned t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= PairCounts(pl, b.st).pf) return;
    uint2 pr = pl.pf[t];
    unsigned idx[4];
    pair_indices_pf(s, pr, idx);
    Vec3 c = dist::point_triangle_coeff(X(b.x, idx[0]), X(b.x, idx[1]), X(b.x, idx[2]),
                                        X(b.x, idx[3]));
    float w[4] = {1.0f, -c[0], -c[1], -c[2]};
    const PpfVertexParam &vp = s.vparam[s.vprop[pr.x].param_index];
    const PpfFaceParam &fp = s.fparam[s.fprop[pr.y].param_index];
    float offset = vp.offset + fp.offset;
    float ghat = 0.5f * (vp.ghat + fp.ghat);
    float mu = contact::combine_friction(vp.friction, fp.friction, p.friction_mode);
    assemble_pair<4>(s, b, dm, idx, w, ghat, offset, mu, true, 1.0f);
}

__global__ void k_assemble_pe(Scene s, AssemblyBuffers b, PairLists pl, DynMatrix dm) {
    const StepParams &p = *b.params;
    unsigned t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= PairCounts(pl, b.st).pe) return;
    uint3 pr = pl.pe[t];
    unsigned idx[3];
    pair_indices_pe(s, pr, idx);
    Vec2 c = dist::point_edge_coeff(X(b.x, idx[0]), X(b.x, idx[1]), X(b.x, idx[2]));
    float w[3] = {1.0f, -c[0], -c[1]};
    const PpfVertexParam &vp = s.vparam[s.vprop[pr.x].param_index];
    const PpfEdgeParam &ep = s.eparam[s.eprop[pr.y].param_index];
    float offset = vp.offset + ep.offset;
    float ghat = 0.5f * (vp.ghat + ep.ghat);
    float mu = contact::combine_friction(vp.friction, ep.friction, p.friction_mode);
    bool fr = (pr.z & 0x80000000u) != 0u;
    float count = (float)(pr.z & 0x7fffffffu);
    assemble_pair<3>(s, b, dm, idx, w, ghat, offset, mu, fr, count);
}

__global__ void k_assemble_pp(Scene s, AssemblyBuffers b, PairLists pl, DynMatrix dm) {
    const StepParams &p = *b.params;
    unsigned t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= PairCounts(pl, b.st).pp) return;
    uint3 pr = pl.pp[t];
    unsigned idx[2] = {pr.x, pr.y};
    float w[2] = {1.0f, -1.0f};
    const PpfVertexParam &a = s.vparam[s.vprop[pr.x].param_index];
    const PpfVertexParam &c = s.vparam[s.vprop[pr.y].param_index];
    float offset = a.offset + c.offset;
    float ghat = 0.5f * (a.ghat + c.ghat);
    float mu = contact::combine_friction(a.friction, c.friction, p.friction_mode);
    bool fr = (pr.z & 0x80000000u) != 0u;
    float count = (float)(pr.z & 0x7fffffffu);
    assemble_pair<2>(s, b, dm, idx, w, ghat, offset, mu, fr, count);
}

__global__ void k_assemble_ee(Scene s, AssemblyBuffers b, PairLists pl, DynMatrix dm) {
    const StepParams &p = *b.params;
    unsigned t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= PairCounts(pl, b.st).ee) return;
    uint2 pr = pl.ee[t];
    unsigned idx[4];
    pair_indices_ee(s, pr, idx);
    Vec4 c = dist::edge_edge_coeff(X(b.x, idx[0]), X(b.x, idx[1]), X(b.x, idx[2]),
                                   X(b.x, idx[3]));
    float w[4] = {c[0], c[1], -c[2], -c[3]};
    const PpfEdgeParam &pa = s.eparam[s.eprop[pr.x].param_index];
    const PpfEdgeParam &pb = s.eparam[s.eprop[pr.y].param_index];
    float offset = pa.offset + pb.offset;
    float ghat = 0.5f * (pa.ghat + pb.ghat);
    float mu = contact::combine_friction(pa.friction, pb.friction, p.friction_mode);
    assemble_pair<4>(s, b, dm, idx, w, ghat, offset, mu, true, 1.0f);
}

// ---- analytic sphere / floor (contact.cu:1154-1381) --------------------------
__global__ void k_vertex_constraints(Scene s, AssemblyBuffers b) {
    const StepParams &p = *b.params;
    unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= s.n_surf) return;
    const PpfVertexProp &vp = s.vprop[i];
    if (vp.fix_index > 0 || !(vp.mass > 0.0f)) return;
    if (s.nsphere == 0 && s.nfloor == 0) return;
    Mat3 local = load_block(b.fixed_tmp + 9 * (size_t)s.fixed_diag[i]);
    Vec3 f = Vec3::zero();
    Mat3 H = Mat3::zero();
    const float vfr = s.vparam[vp.param_index].friction;
    const Vec3 x = X(b.x, i), xs = X(b.x0, i);
    unsigned nc = 0;
    for (unsigned k = 0; k < s.nsphere; ++k) {
        const PpfSphere &q = s.sphere[k];
        contact::SphereC sp{vec3(q.center.v[0], q.center.v[1], q.center.v[2]), q.ghat,
                            q.friction, q.radius, q.thickness, q.bowl, q.reverse,
                            q.kinematic};
        nc += contact::sphere_constraint(x, xs, vp.mass, vfr, local, sp, p.friction_mode,
                                         p.friction_eps, f, H);
    }
    for (unsigned k = 0; k < s.nfloor; ++k) {
        const PpfFloor &q = s.floor[k];
        contact::FloorC fl{vec3(q.ground.v[0], q.ground.v[1], q.ground.v[2]), q.ghat,
                           q.friction, q.thickness, vec3(q.up.v[0], q.up.v[1], q.up.v[2]),
                           q.kinematic};
        nc += contact::floor_constraint(x, xs, vp.mass, vfr, local, fl, p.friction_mode,
                                        p.friction_eps, p.constraint_tol, f, H);
    }
    if (nc == 0) return;
    atomic_add3(b.force + 3 * i, f);
    atomic_add_block(b.fixed_val + 9 * (size_t)s.fixed_diag[i], H);
    atomicAdd(&b.st->n_contact, nc);
}

// ---- static collision mesh (contact/contact.cu:1834-1947) -------------------
// Push-model contacts against a mesh without degrees of freedom (element math
// in contact_local.cuh). Every block they touch is in the fixed pattern: a
// vertex's diagonal, a face's and an edge's own blocks.

// A free vertex against the collision faces.
struct MeshFaceOp {
    const Scene &s;
    const StepParams &p;
    const AssemblyBuffers &b;
    unsigned v;
    Mat3 local;
    Vec3 f;
    Mat3 H;
    unsigned n;
    __device__ void operator()(unsigned fi) {
        const PpfVertexProp &vp = s.vprop[v];
        const unsigned *cf = s.cm_face + 3 * fi;
        const PpfVertexParam &vq = s.vparam[vp.param_index];
        const PpfFaceParam &fq = s.cm_fparam[s.cm_fprop[fi].param_index];
        Vec3 fo;
        Mat3 Ho;
        if (contact::mesh_vertex_face(X(b.x, v), X(b.x0, v), vp.mass, local, X(s.cm_x, cf[0]),
                                      X(s.cm_x, cf[1]), X(s.cm_x, cf[2]), vq.offset + fq.offset,
                                      0.5f * (vq.ghat + fq.ghat),
                                      contact::combine_friction(vq.friction, fq.friction,
                                                                p.friction_mode),
                                      p.friction_eps, fo, Ho)) {
            f += fo;
            H += Ho;
            ++n;
        }
    }
};

__global__ void k_mesh_vertex_face(Scene s, AssemblyBuffers b) {
    const StepParams &p = *b.params;
    const unsigned v = blockIdx.x * blockDim.x + threadIdx.x;
    bool act = v < s.n_surf;
    if (act) act = s.vprop[v].fix_index == 0 && s.vprop[v].mass > 0.0f;
    float4 qmin = make_float4(0.0f, 0.0f, 0.0f, 0.0f), qmax = qmin;
    Mat3 local = Mat3::zero();
    if (act) {
        const PpfVertexParam &vq = s.vparam[s.vprop[v].param_index];
        const Vec3 x = X(b.x, v);
        const float m = 0.5f * vq.ghat + vq.offset + detect_guard(x);
        qmin = make_float4(x[0] - m, x[1] - m, x[2] - m, 1.0f);
        qmax = make_float4(x[0] + m, x[1] + m, x[2] + m, 0.0f);
        local = load_block(b.fixed_tmp + 9 * (size_t)s.fixed_diag[v]);
    }
    MeshFaceOp op{s, p, b, act ? v : 0u, local, Vec3::zero(), Mat3::zero(), 0u};
    warp_query(s.cm_face_bvh, act, qmin, qmax, op, &b.st->status);
    if (!op.n) return;
    atomic_add3(b.force + 3 * v, op.f);
    atomic_add_block(b.fixed_val + 9 * (size_t)s.fixed_diag[v], op.H);
    atomicAdd(&b.st->n_contact, op.n);
}

// A collision vertex against the free faces.
struct MeshVertexOp {
    const Scene &s;
    const StepParams &p;
    const AssemblyBuffers &b;
    unsigned cv;
    unsigned n;
    __device__ void operator()(unsigned fi) {
        const PpfFaceProp &fp = s.fprop[fi];
        if (fp.fixed || !(fp.mass > 0.0f)) return;
        const unsigned *fc = s.face + 3 * fi;
        const PpfFaceParam &fq = s.fparam[fp.param_index];
        const PpfVertexParam &cq = s.cm_vparam[s.cm_vprop[cv].param_index];
        Vec3 t[3], sx[3];
        float m[3];
        Mat9 local;
        for (int a = 0; a < 3; ++a) {
            t[a] = X(b.x, fc[a]);
            sx[a] = X(b.x0, fc[a]);
            m[a] = s.vprop[fc[a]].mass;
            for (int c = 0; c < 3; ++c)
                local.set_block<3, 3>(3 * a, 3 * c, fixed_block(s, b.fixed_tmp, fc[a], fc[c]));
        }
        Mat<3, 3> ff;
        Mat9 HH;
        if (!contact::mesh_face_vertex(X(s.cm_x, cv), t, sx, m, local, fq.offset + cq.offset,
                                       0.5f * (fq.ghat + cq.ghat),
                                       contact::combine_friction(fq.friction, cq.friction,
                                                                 p.friction_mode),
                                       p.friction_eps, ff, HH))
            return;
        for (int a = 0; a < 3; ++a) atomic_add3(b.force + 3 * fc[a], ff.col(a));
        const unsigned *slot = s.face_slot + 9 * fi;
        for (int a = 0; a < 3; ++a)
            for (int c = 0; c < 3; ++c) {
                const unsigned sl = slot[3 * a + c];
                if (sl != kSentinel)
                    atomic_add_block(b.fixed_val + 9 * (size_t)sl, HH.block<3, 3>(3 * a, 3 * c));
            }
        ++n;
    }
};

__global__ void k_mesh_face_vertex(Scene s, AssemblyBuffers b, BvhView fb) {
    const StepParams &p = *b.params;
    const unsigned cv = blockIdx.x * blockDim.x + threadIdx.x;
    const bool act = cv < s.ncv;
    float4 qmin = make_float4(0.0f, 0.0f, 0.0f, 0.0f), qmax = qmin;
    if (act) {
        const PpfVertexParam &cq = s.cm_vparam[s.cm_vprop[cv].param_index];
        const Vec3 y = X(s.cm_x, cv);
        const float m = 0.5f * cq.ghat + cq.offset + detect_guard(y);
        qmin = make_float4(y[0] - m, y[1] - m, y[2] - m, 1.0f);
        qmax = make_float4(y[0] + m, y[1] + m, y[2] + m, 0.0f);
    }
    MeshVertexOp op{s, p, b, act ? cv : 0u, 0u};
    warp_query(fb, act, qmin, qmax, op, &b.st->status);
    if (op.n) atomicAdd(&b.st->n_contact, op.n);
}

// A free edge of positive mass against the collision edges (a shell's edges
// carry no mass, so for cloth this finds nothing, as in the reference).
struct MeshEdgeOp {
    const Scene &s;
    const StepParams &p;
    const AssemblyBuffers &b;
    unsigned e;
    unsigned n;
    __device__ void operator()(unsigned ce) {
        const unsigned *ed = s.edge + 2 * e, *c = s.cm_edge + 2 * ce;
        const PpfEdgeParam &eq = s.eparam[s.eprop[e].param_index];
        const PpfEdgeParam &cq = s.cm_eparam[s.cm_eprop[ce].param_index];
        Mat6 local;
        for (int u = 0; u < 2; ++u)
            for (int w = 0; w < 2; ++w)
                local.set_block<3, 3>(3 * u, 3 * w, fixed_block(s, b.fixed_tmp, ed[u], ed[w]));
        Mat<3, 2> ff;
        Mat6 HH;
        if (!contact::mesh_edge_edge(X(b.x, ed[0]), X(b.x, ed[1]), X(b.x0, ed[0]), X(b.x0, ed[1]),
                                     X(s.cm_x, c[0]), X(s.cm_x, c[1]), s.vprop[ed[0]].mass,
                                     s.vprop[ed[1]].mass, local, eq.offset + cq.offset,
                                     0.5f * (eq.ghat + cq.ghat),
                                     contact::combine_friction(eq.friction, cq.friction,
                                                               p.friction_mode),
                                     p.friction_eps, ff, HH))
            return;
        for (int u = 0; u < 2; ++u) atomic_add3(b.force + 3 * ed[u], ff.col(u));
        for (int u = 0; u < 2; ++u)
            for (int w = 0; w < 2; ++w)
                if (ed[u] <= ed[w]) {
                    const unsigned sl = fixed_slot(s, ed[u], ed[w]);
                    if (sl != kSentinel)
                        atomic_add_block(b.fixed_val + 9 * (size_t)sl,
                                         HH.block<3, 3>(3 * u, 3 * w));
                }
        ++n;
    }
};

__global__ void k_mesh_edge_edge(Scene s, AssemblyBuffers b) {
    const StepParams &p = *b.params;
    const unsigned e = blockIdx.x * blockDim.x + threadIdx.x;
    bool act = e < s.ne;
    if (act) act = !s.eprop[e].fixed && s.eprop[e].mass > 0.0f;
    float4 qmin = make_float4(0.0f, 0.0f, 0.0f, 0.0f), qmax = qmin;
    if (act) {
        const unsigned *ed = s.edge + 2 * e;
        const PpfEdgeParam &eq = s.eparam[s.eprop[e].param_index];
        const Vec3 a = X(b.x, ed[0]), c = X(b.x, ed[1]);
        seg_box(a, c, 0.5f * eq.ghat + eq.offset + fmaxf(detect_guard(a), detect_guard(c)),
                qmin, qmax);
    }
    MeshEdgeOp op{s, p, b, act ? e : 0u, 0u};
    warp_query(s.cm_edge_bvh, act, qmin, qmax, op, &b.st->status);
    if (op.n) atomicAdd(&b.st->n_contact, op.n);
}

// ---- Dirichlet elimination of pinned vertices (main.cu:954-1049) -------------
__device__ __forceinline__ void lift_sub(float *force, unsigned row, const Mat3 &blk,
                                         const Vec3 &pv, bool transposed) {
    Vec3 c;
    if (transposed) {
        c[0] = blk(0, 0) * pv[0] + blk(1, 0) * pv[1] + blk(2, 0) * pv[2];
        c[1] = blk(0, 1) * pv[0] + blk(1, 1) * pv[1] + blk(2, 1) * pv[2];
        c[2] = blk(0, 2) * pv[0] + blk(1, 2) * pv[1] + blk(2, 2) * pv[2];
    } else {
        c[0] = blk(0, 0) * pv[0] + blk(0, 1) * pv[1] + blk(0, 2) * pv[2];
        c[1] = blk(1, 0) * pv[0] + blk(1, 1) * pv[1] + blk(1, 2) * pv[2];
        c[2] = blk(2, 0) * pv[0] + blk(2, 1) * pv[1] + blk(2, 2) * pv[2];
    }
    atomicAdd(force + 3 * row + 0, -c[0]);
    atomicAdd(force + 3 * row + 1, -c[1]);
    atomicAdd(force + 3 * row + 2, -c[2]);
}

__device__ __forceinline__ void eliminate_row(const Scene &s, const AssemblyBuffers &b,
                                              unsigned i, unsigned k0, unsigned k1,
                                              const unsigned *col, float *val) {
    const bool mi = s.dof_mask[i] != 0u;
    for (unsigned k = k0; k < k1; ++k) {
        unsigned j = col[k];
        const bool mj = s.dof_mask[j] != 0u;
        float *blkp = val + 9 * (size_t)k;
        if (mi != mj) {
            Mat3 blk = load_block(blkp);
            if (mj) lift_sub(b.force, i, blk, X(b.x, j) - X(b.target, j), false);
            else lift_sub(b.force, j, blk, X(b.x, i) - X(b.target, i), true);
        }
        if (mi || mj)
            for (int q = 0; q < 9; ++q) blkp[q] = 0.0f;
    }
}

__global__ void k_dirichlet_lift(Scene s, AssemblyBuffers b, DynMatrix dm) {
    unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= s.n) return;
    eliminate_row(s, b, i, dm.off[i], dm.off[i + 1], dm.col, dm.val);
    eliminate_row(s, b, i, s.fixed_off[i], s.fixed_off[i + 1], s.fixed_col, b.fixed_val);
}

__global__ void k_dirichlet_rows(Scene s, AssemblyBuffers b) {
    unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= s.n || s.dof_mask[i] == 0u) return;
    float *d = b.diag + 9 * i;
    for (int q = 0; q < 9; ++q) d[q] = (q % 4 == 0) ? 1.0f : 0.0f;
    Vec3 pv = X(b.x, i) - X(b.target, i);
    store3(b.force + 3 * i, pv);
}

// ---- exclusive scan ----------------------------------------------------------
constexpr unsigned kScanBlock = 1024;

__global__ void k_scan_blocks(const unsigned *in, unsigned *out, unsigned n,
                              unsigned *block_sums) {
    __shared__ unsigned s_warp[32];
    unsigned i = blockIdx.x * kScanBlock + threadIdx.x;
    unsigned v = i < n ? in[i] : 0u;
    unsigned lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    unsigned x = v;
    for (int off = 1; off < 32; off <<= 1) {
        unsigned y = __shfl_up_sync(0xffffffffu, x, off);
        if (lane >= (unsigned)off) x += y;
    }
    if (lane == 31) s_warp[warp] = x;
    __syncthreads();
    if (warp == 0) {
        unsigned w = s_warp[lane];
        for (int off = 1; off < 32; off <<= 1) {
            unsigned y = __shfl_up_sync(0xffffffffu, w, off);
            if (lane >= (unsigned)off) w += y;
        }
        s_warp[lane] = w;
    }
    __syncthreads();
    unsigned incl = x + (warp ? s_warp[warp - 1] : 0u);
    if (i < n) out[i] = incl - v;
    if (threadIdx.x == kScanBlock - 1) block_sums[blockIdx.x] = incl;
}

__global__ void k_scan_add(unsigned *out, unsigned n, const unsigned *block_offsets) {
    unsigned i = blockIdx.x * kScanBlock + threadIdx.x;
    if (i < n && blockIdx.x > 0) out[i] += block_offsets[blockIdx.x];
}

__global__ void k_scan_total(const unsigned *in, unsigned *out, unsigned n) {
    out[n] = (n ? out[n - 1] + in[n - 1] : 0u);
}

// Up to kScanSmall values scanned by one block, total included: each thread
// takes `items` consecutive values, the block scans the threads' sums. One
// launch where the general path takes three or four.
constexpr unsigned kScanItems = 16, kScanSmall = kScanBlock * kScanItems;

__global__ void k_scan_small(const unsigned *in, unsigned *out, unsigned n) {
    __shared__ unsigned s_warp[32];
    const unsigned items = (n + kScanBlock - 1) / kScanBlock;
    const unsigned base = threadIdx.x * items;
    unsigned v[kScanItems];
    unsigned sum = 0;
#pragma unroll
    for (unsigned k = 0; k < kScanItems; ++k) {
        v[k] = (k < items && base + k < n) ? in[base + k] : 0u;
        sum += v[k];
    }
    const unsigned lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    unsigned x = sum;
    for (int off = 1; off < 32; off <<= 1) {
        unsigned y = __shfl_up_sync(0xffffffffu, x, off);
        if (lane >= (unsigned)off) x += y;
    }
    if (lane == 31) s_warp[warp] = x;
    __syncthreads();
    if (warp == 0) {
        unsigned w = s_warp[lane];
        for (int off = 1; off < 32; off <<= 1) {
            unsigned y = __shfl_up_sync(0xffffffffu, w, off);
            if (lane >= (unsigned)off) w += y;
        }
        s_warp[lane] = w;
    }
    __syncthreads();
    unsigned run = x - sum + (warp ? s_warp[warp - 1] : 0u);
#pragma unroll
    for (unsigned k = 0; k < kScanItems; ++k) {
        if (k < items && base + k < n) out[base + k] = run;
        run += v[k];
    }
    if (threadIdx.x == kScanBlock - 1) out[n] = run;
}

} // namespace

size_t scan_tmp_size(unsigned n) {
    // per level: block sums + their scanned offsets (+1), then the next level
    size_t total = 0;
    unsigned m = n;
    do {
        unsigned b = div_up(m < 1u ? 1u : m, kScanBlock);
        total += 2 * (size_t)b + 1;
        m = b;
    } while (m > 1);
    return total + 2;
}

static void scan_rec(const unsigned *in, unsigned *out, unsigned n, unsigned *tmp,
                     cudaStream_t q) {
    unsigned blocks = div_up(n, kScanBlock);
    unsigned *sums = tmp;
    unsigned *offs = tmp + blocks;
    k_scan_blocks<<<blocks, kScanBlock, 0, q>>>(in, out, n, sums);
    PPF_LAUNCH_CHECK();
    if (blocks > 1) {
        scan_rec(sums, offs, blocks, offs + blocks + 1, q);
        k_scan_add<<<blocks, kScanBlock, 0, q>>>(out, n, offs);
        PPF_LAUNCH_CHECK();
    }
}

void exclusive_scan(const unsigned *in, unsigned *out, unsigned n, unsigned *tmp,
                    cudaStream_t q) {
    if (n <= kScanSmall) {
        k_scan_small<<<1, kScanBlock, 0, q>>>(in, out, n);
        PPF_LAUNCH_CHECK();
        return;
    }
    scan_rec(in, out, n, tmp, q);
    k_scan_total<<<1, 1, 0, q>>>(in, out, n);
    PPF_LAUNCH_CHECK();
}

void launch_vertex_energy(const Scene &s, const AssemblyBuffers &b,
                          cudaStream_t q) {
    if (!s.n) return;
    k_vertex_energy<<<div_up(s.n, kB), kB, 0, q>>>(s, b);
    PPF_LAUNCH_CHECK();
}

void launch_elastic(const Scene &s, const AssemblyBuffers &b,
                    cudaStream_t q) {
    if (s.nr) {
        k_rod_bend<<<div_up(s.n_surf, kB), kB, 0, q>>>(s, b);
        PPF_LAUNCH_CHECK();
        k_rod_energy<<<div_up(s.nr, kB), kB, 0, q>>>(s, b);
        PPF_LAUNCH_CHECK();
    }
    if (s.nf_shell) {
        k_face_energy<<<div_up(s.nf_shell, kB), kB, 0, q>>>(s, b);
        PPF_LAUNCH_CHECK();
    }
    if (s.nt) {
        k_tet_energy<<<div_up(s.nt, kB), kB, 0, q>>>(s, b);
        PPF_LAUNCH_CHECK();
    }
    if (s.nh) {
        k_hinge_energy<<<div_up(s.nh, kB), kB, 0, q>>>(s, b);
        PPF_LAUNCH_CHECK();
    }
    if (s.nstitch) { // after the elastic terms, before the copy (main.cu:794-797)
        k_stitch_energy<<<div_up(s.nstitch, kB), kB, 0, q>>>(s, b);
        PPF_LAUNCH_CHECK();
    }
}

void launch_strain_limit(const Scene &s, const AssemblyBuffers &b,
                         cudaStream_t q) {
    if (s.nf_shell) {
        k_strain_limit<<<div_up(s.nf_shell, kB), kB, 0, q>>>(s, b);
        PPF_LAUNCH_CHECK();
    }
    if (s.nr) {
        k_rod_strain_limit<<<div_up(s.nr, kB), kB, 0, q>>>(s, b);
        PPF_LAUNCH_CHECK();
    }
}

void launch_edge_pieces(const Scene &s, const BvhView &eb, const float *x, const float *x1,
                        const unsigned *t_bits, float piece_len, PieceBuffers &pb,
                        cudaStream_t q) {
    if (!s.ne) return;
    k_edge_piece_count<<<div_up(s.ne, kB), kB, 0, q>>>(s.ne, eb.node, s.edge, x, x1, t_bits,
                                                       piece_len, pb.count);
    PPF_LAUNCH_CHECK();
    exclusive_scan(pb.count, pb.off, s.ne, pb.scan_tmp, q);
}

unsigned piece_grid(unsigned ne, unsigned block) { return div_up(ne, block) + 2 * kNumSMs; }

void launch_detect(const Scene &s, const BvhView &fb, const BvhView &eb,
                   const BvhView &vb, const AssemblyBuffers &b, PairLists &pl,
                   const PieceBuffers &pb, cudaStream_t q) {
    if (s.n_surf) {
        if (s.tune.detect_vertex)
            k_detect_vertex<LeafTests::kImmediate>
                <<<div_up(s.n_surf, 128u), 128, 0, q>>>(s, fb, eb, vb, b.x, pl, b.st);
        else
            k_detect_vertex<LeafTests::kWarpRounds>
                <<<div_up(s.n_surf, 128u), 128, 0, q>>>(s, fb, eb, vb, b.x, pl, b.st);
        PPF_LAUNCH_CHECK();
    }
    if (s.ne) {
        if (s.tune.detect_edge)
            k_detect_edge<LeafTests::kImmediate>
                <<<piece_grid(s.ne, 128u), 128, 0, q>>>(s, eb, b.x, pl, b.st,
                                                            EdgePieces{pb.off, s.ne});
        else
            k_detect_edge<LeafTests::kWarpRounds>
                <<<piece_grid(s.ne, 128u), 128, 0, q>>>(s, eb, b.x, pl, b.st,
                                                            EdgePieces{pb.off, s.ne});
        PPF_LAUNCH_CHECK();
    }
}

void launch_dyn_build(const Scene &s, const AssemblyBuffers &b, const PairLists &pl,
                      const unsigned bound[4], DynMatrix &dm, unsigned *d_scan_tmp,
                      cudaStream_t q) {
    PPF_CUDA(cudaMemsetAsync(dm.hkey, 0xff, (size_t)dm.hcap * sizeof(unsigned long long), q));
    PPF_CUDA(cudaMemsetAsync(dm.cnt, 0, s.n * sizeof(unsigned), q));
    PPF_CUDA(cudaMemsetAsync(dm.cnt2, 0, s.n * sizeof(unsigned), q));
    const unsigned total = bound[0] + bound[1] + bound[2] + bound[3];
    if (total) {
        k_dyn_insert<<<div_up(total, kB), kB, 0, q>>>(s, pl, dm, b.st);
        PPF_LAUNCH_CHECK();
    }
    k_dyn_capacity<<<1, 1, 0, q>>>(dm, b.st);
    PPF_LAUNCH_CHECK();
    k_dyn_count<<<div_up(dm.hcap, kB), kB, 0, q>>>(dm, b.st);
    PPF_LAUNCH_CHECK();
    exclusive_scan(dm.cnt, dm.off, s.n, d_scan_tmp, q);
    exclusive_scan(dm.cnt2, dm.tr_off, s.n, d_scan_tmp, q);
    PPF_CUDA(cudaMemsetAsync(dm.cnt, 0, s.n * sizeof(unsigned), q));
    PPF_CUDA(cudaMemsetAsync(dm.cnt2, 0, s.n * sizeof(unsigned), q));
    k_dyn_fill<<<div_up(dm.hcap, kB), kB, 0, q>>>(dm, b.st);
    PPF_LAUNCH_CHECK();
    k_zero_dyn_val<<<2 * kNumSMs, kB, 0, q>>>(dm, b.st);
    PPF_LAUNCH_CHECK();
}

void launch_pair_capacity(const PairLists &pl, IterStatus *st, cudaStream_t q) {
    k_pair_capacity<<<1, 1, 0, q>>>(pl, st);
    PPF_LAUNCH_CHECK();
}

void launch_contact_assemble(const Scene &s, const AssemblyBuffers &b, const PairLists &pl,
                             const unsigned bound[4], DynMatrix &dm, cudaStream_t q) {
    if (bound[0]) {
        k_assemble_pf<<<div_up(bound[0], 128u), 128, 0, q>>>(s, b, pl, dm);
        PPF_LAUNCH_CHECK();
    }
    if (bound[1]) {
        k_assemble_pe<<<div_up(bound[1], 128u), 128, 0, q>>>(s, b, pl, dm);
        PPF_LAUNCH_CHECK();
    }
    if (bound[2]) {
        k_assemble_pp<<<div_up(bound[2], 128u), 128, 0, q>>>(s, b, pl, dm);
        PPF_LAUNCH_CHECK();
    }
    if (bound[3]) {
        k_assemble_ee<<<div_up(bound[3], 128u), 128, 0, q>>>(s, b, pl, dm);
        PPF_LAUNCH_CHECK();
    }
}

void launch_vertex_constraints(const Scene &s, const AssemblyBuffers &b, cudaStream_t q) {
    if (!s.n_surf || (s.nsphere == 0 && s.nfloor == 0)) return;
    k_vertex_constraints<<<div_up(s.n_surf, kB), kB, 0, q>>>(s, b);
    PPF_LAUNCH_CHECK();
}

void launch_collision_mesh(const Scene &s, const AssemblyBuffers &b,
                           const BvhView &fb, cudaStream_t q) {
    if (!s.ncv) return;
    if (s.ncf && s.n_surf) {
        k_mesh_vertex_face<<<div_up(s.n_surf, kB), kB, 0, q>>>(s, b);
        PPF_LAUNCH_CHECK();
    }
    k_mesh_face_vertex<<<div_up(s.ncv, kB), kB, 0, q>>>(s, b, fb);
    PPF_LAUNCH_CHECK();
    if (s.nce && s.ne) {
        k_mesh_edge_edge<<<div_up(s.ne, kB), kB, 0, q>>>(s, b);
        PPF_LAUNCH_CHECK();
    }
}

void launch_dirichlet(const Scene &s, const AssemblyBuffers &b, const DynMatrix &dm,
                      float *dx, cudaStream_t q) {
    (void)dx;
    if (s.nfix == 0) return;
    k_dirichlet_lift<<<div_up(s.n, kB), kB, 0, q>>>(s, b, dm);
    PPF_LAUNCH_CHECK();
    k_dirichlet_rows<<<div_up(s.n, kB), kB, 0, q>>>(s, b);
    PPF_LAUNCH_CHECK();
}

} // namespace gpu
} // namespace ppf
