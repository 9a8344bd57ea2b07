// linesearch.cu -- additive-CCD step filter, strain-limit bisection, and the
// post-step intersection check. The per-pair sweeps are the shared element
// functions of ../physics/accd.cuh.
#include "../physics/accd.cuh"
#include "../physics/bw.cuh"
#include "../physics/rod.cuh"
#include "../physics/strainlimit.cuh"
#include "assemble.cuh"
#include "linesearch.cuh"

namespace ppf {
namespace gpu {

namespace {

constexpr unsigned kB = 128;

__device__ __forceinline__ Vec3 sweep_end(const float *x0, const float *x1, unsigned i,
                                          float t) {
    return vec3(fmaf(t, x1[3 * i] - x0[3 * i], x0[3 * i]),
                fmaf(t, x1[3 * i + 1] - x0[3 * i + 1], x0[3 * i + 1]),
                fmaf(t, x1[3 * i + 2] - x0[3 * i + 2], x0[3 * i + 2]));
}

__device__ __forceinline__ void record_overlap(IterStatus *st, const accd::CcdFlag &fl,
                                               unsigned v0, unsigned v1, unsigned kind) {
    if (!fl.overlap) return;
    atomicOr(&st->overlap, 1u);
    if (atomicCAS(&st->overlap_v0, 0xFFFFFFFFu, v0) == 0xFFFFFFFFu) {
        st->overlap_v1 = v1;
        st->overlap_kind = kind;
    }
}

// Sphere / floor crossing of one vertex's sweep (contact.cu:2318-2470).
__device__ float vertex_constraint_toi(const Scene &s, const LineSearchArgs &a, unsigned i) {
    const Vec3 x0 = X(a.x0, i);
    const Vec3 x1 = sweep_end(a.x0, a.x1, i, a.max_t);
    const PpfVertexProp &vp = s.vprop[i];
    float toi = a.max_t;
    if (vp.fix_index > 0) {
        for (unsigned j = 0; j < s.nsphere; ++j) {
            const PpfSphere &sp = s.sphere[j];
            if (sp.kinematic) continue;
            Vec3 c = vec3(sp.center.v[0], sp.center.v[1], sp.center.v[2]);
            Vec3 c0 = (sp.bowl && x0[1] > c[1]) ? vec3(c[0], x0[1], c[2]) : c;
            Vec3 c1 = (sp.bowl && x1[1] > c[1]) ? vec3(c[0], x1[1], c[2]) : c;
            float r0 = (x0 - c0).norm(), r1 = (x1 - c1).norm();
            float d0 = sp.reverse ? (sp.radius - r0) : (r0 - sp.radius);
            float d1 = sp.reverse ? (sp.radius - r1) : (r1 - sp.radius);
            if (d0 >= 0.0f && d1 < 0.0f) atomicMin(&a.st->pin_infeasible, i);
        }
        for (unsigned j = 0; j < s.nfloor; ++j) {
            const PpfFloor &fl = s.floor[j];
            if (fl.kinematic) continue;
            Vec3 up = vec3(fl.up.v[0], fl.up.v[1], fl.up.v[2]);
            Vec3 g = vec3(fl.ground.v[0], fl.ground.v[1], fl.ground.v[2]);
            float h0 = up.dot(x0 - g), h1 = up.dot(x1 - g);
            if (h0 >= 0.0f && h1 < 0.0f) atomicMin(&a.st->pin_infeasible, i);
        }
    } else if (vp.mass > 0.0f) {
        for (unsigned j = 0; j < s.nsphere; ++j) {
            const PpfSphere &sp = s.sphere[j];
            if (sp.kinematic) continue;
            Vec3 c = vec3(sp.center.v[0], sp.center.v[1], sp.center.v[2]);
            Vec3 c0 = (sp.bowl && x0[1] > c[1]) ? vec3(c[0], x0[1], c[2]) : c;
            Vec3 c1 = (sp.bowl && x1[1] > c[1]) ? vec3(c[0], x1[1], c[2]) : c;
            float r = sp.radius;
            float r0 = (x0 - c0).norm(), r1 = (x1 - c1).norm();
            float depth0 = sp.reverse ? (r0 - r) : (r - r0);
            if (sp.thickness > 0.0f && depth0 > sp.thickness) continue;
            if ((r0 - r) * (r1 - r) <= 0.0f) {
                float t = (r - r0) / (r1 - r0);
                toi = fminf(toi, a.max_t * t);
            }
        }
        for (unsigned j = 0; j < s.nfloor; ++j) {
            const PpfFloor &fl = s.floor[j];
            if (fl.kinematic) continue;
            Vec3 up = vec3(fl.up.v[0], fl.up.v[1], fl.up.v[2]);
            Vec3 g = vec3(fl.ground.v[0], fl.ground.v[1], fl.ground.v[2]);
            float h0 = up.dot(x0 - g), h1 = up.dot(x1 - g);
            if (fl.thickness > 0.0f && -h0 > fl.thickness) continue;
            if (h1 < 0.0f) {
                float t = -h0 / (h1 - h0);
                toi = fminf(toi, a.max_t * t);
            }
        }
    }
    return toi;
}

struct PointFaceCcdOp {
    const Scene &s;
    const LineSearchArgs &a;
    unsigned v;
    float toi;
    __device__ void operator()(unsigned fi) {
        const unsigned *f = s.face + 3 * fi;
        bool either_dyn = s.vprop[v].fix_index == 0 || !s.fprop[fi].fixed;
        bool both_collider = s.vprop[v].collider && s.vprop[f[0]].collider;
        if (!either_dyn || both_collider) return;
        int dup = -1;
        for (int k = 0; k < 3; ++k)
            if (f[k] == v) {
                dup = k;
                break;
            }
        accd::CcdFlag fl;
        float r;
        const PpfVertexParam &vp = s.vparam[s.vprop[v].param_index];
        if (dup < 0) {
            const PpfFaceParam &fp = s.fparam[s.fprop[fi].param_index];
            float offset = vp.offset + fp.offset;
            float ghat = 0.5f * (vp.ghat + fp.ghat);
            r = accd::point_triangle(X(a.x0, v), X(a.x1, v), X(a.x0, f[0]), X(a.x0, f[1]),
                                     X(a.x0, f[2]), X(a.x1, f[0]), X(a.x1, f[1]),
                                     X(a.x1, f[2]), offset, ghat, a.max_t, a.ccd_eps, &fl);
        } else {
            unsigned i = f[dup], j = f[(dup + 1) % 3], k = f[(dup + 2) % 3];
            r = accd::point_edge(X(a.x0, i), X(a.x1, i), X(a.x0, j), X(a.x0, k), X(a.x1, j),
                                 X(a.x1, k), 2.0f * vp.offset, vp.ghat, a.max_t, a.ccd_eps,
                                 &fl);
        }
        if (r < a.max_t) {
            toi = fminf(toi, r);
            if (r == 0.0f) {
                record_overlap(a.st, fl, v, f[0], 0u);
                if (!fl.overlap) atomicOr(&a.st->overlap, 1u);
            }
        }
    }
};

struct PointPointCcdOp {
    const Scene &s;
    const LineSearchArgs &a;
    unsigned v;
    float toi;
    __device__ bool pre(unsigned w) const { return w < v; }
    __device__ void operator()(unsigned w) {
        bool either_dyn = s.vprop[v].fix_index == 0 || s.vprop[w].fix_index == 0;
        bool both_collider = s.vprop[v].collider && s.vprop[w].collider;
        if (!(w < v) || !either_dyn || both_collider) return;
        const PpfVertexParam &pa = s.vparam[s.vprop[v].param_index];
        const PpfVertexParam &pb = s.vparam[s.vprop[w].param_index];
        accd::CcdFlag fl;
        float r = accd::point_point(X(a.x0, v), X(a.x1, v), X(a.x0, w), X(a.x1, w),
                                    pa.offset + pb.offset, 0.5f * (pa.ghat + pb.ghat),
                                    a.max_t, a.ccd_eps, &fl);
        if (r < a.max_t) {
            toi = fminf(toi, r);
            if (r == 0.0f) {
                record_overlap(a.st, fl, v, w, 2u);
                if (!fl.overlap) atomicOr(&a.st->overlap, 1u);
            }
        }
    }
};

// ---- static collision mesh (contact/contact.cu:1956-2094, 2596-2732) --------
// A free vertex's sweep against the collision faces.
struct MeshPointFaceCcdOp {
    const Scene &s;
    const LineSearchArgs &a;
    unsigned v;
    float toi;
    __device__ void operator()(unsigned fi) {
        const unsigned *cf = s.cm_face + 3 * fi;
        const PpfVertexParam &vq = s.vparam[s.vprop[v].param_index];
        const PpfFaceParam &fq = s.cm_fparam[s.cm_fprop[fi].param_index];
        const Vec3 t0 = X(s.cm_x, cf[0]), t1 = X(s.cm_x, cf[1]), t2 = X(s.cm_x, cf[2]);
        accd::CcdFlag fl;
        float r = accd::point_triangle(X(a.x0, v), X(a.x1, v), t0, t1, t2, t0, t1, t2,
                                       vq.offset + fq.offset, 0.5f * (vq.ghat + fq.ghat), a.max_t,
                                       a.ccd_eps, &fl);
        if (r < a.max_t) {
            toi = fminf(toi, r);
            if (r == 0.0f) {
                record_overlap(a.st, fl, v, cf[0], 3u);
                if (!fl.overlap) atomicOr(&a.st->overlap, 1u);
            }
        }
    }
};

// A collision vertex against the free faces' sweeps.
struct MeshVertexCcdOp {
    const Scene &s;
    const LineSearchArgs &a;
    unsigned cv;
    float toi;
    __device__ void operator()(unsigned fi) {
        const PpfFaceProp &fp = s.fprop[fi];
        if (fp.fixed || !(fp.mass > 0.0f)) return;
        const unsigned *f = s.face + 3 * fi;
        const PpfFaceParam &fq = s.fparam[fp.param_index];
        const PpfVertexParam &cq = s.cm_vparam[s.cm_vprop[cv].param_index];
        const Vec3 y = X(s.cm_x, cv);
        accd::CcdFlag fl;
        float r = accd::point_triangle(y, y, X(a.x0, f[0]), X(a.x0, f[1]), X(a.x0, f[2]),
                                       X(a.x1, f[0]), X(a.x1, f[1]), X(a.x1, f[2]),
                                       fq.offset + cq.offset, 0.5f * (fq.ghat + cq.ghat), a.max_t,
                                       a.ccd_eps, &fl);
        if (r < a.max_t) {
            toi = fminf(toi, r);
            if (r == 0.0f) {
                record_overlap(a.st, fl, f[0], cv, 4u);
                if (!fl.overlap) atomicOr(&a.st->overlap, 1u);
            }
        }
    }
};

// A free edge of positive mass against the collision edges.
struct MeshEdgeCcdOp {
    const Scene &s;
    const LineSearchArgs &a;
    unsigned e;
    float toi;
    __device__ void operator()(unsigned ce) {
        const unsigned *ed = s.edge + 2 * e, *c = s.cm_edge + 2 * ce;
        const PpfEdgeParam &pa = s.eparam[s.eprop[e].param_index];
        const PpfEdgeParam &pb = s.cm_eparam[s.cm_eprop[ce].param_index];
        const Vec3 q0 = X(s.cm_x, c[0]), q1 = X(s.cm_x, c[1]);
        accd::CcdFlag fl;
        float r = accd::edge_edge(X(a.x0, ed[0]), X(a.x0, ed[1]), q0, q1, X(a.x1, ed[0]),
                                  X(a.x1, ed[1]), q0, q1, pa.offset + pb.offset,
                                  0.5f * (pa.ghat + pb.ghat), a.max_t, a.ccd_eps, &fl);
        if (r < a.max_t) {
            toi = fminf(toi, r);
            if (r == 0.0f) {
                record_overlap(a.st, fl, ed[0], c[0], 5u);
                if (!fl.overlap) atomicOr(&a.st->overlap, 1u);
            }
        }
    }
};

// The warp's minimum of a per-lane time of impact, taken into `bits` with one
// atomic by lane 0 (every lane of the warp calls this).
__device__ __forceinline__ void warp_min_toi(unsigned *bits, float toi) {
    for (int off = 16; off > 0; off >>= 1)
        toi = fminf(toi, __shfl_xor_sync(0xffffffffu, toi, off));
    if ((threadIdx.x & 31u) == 0u) atomicMin(bits, __float_as_uint(toi));
}

template <LeafTests M>
__global__ void k_ccd_mesh_vertex(Scene s, BvhView fb, LineSearchArgs a) {
    const unsigned cv = blockIdx.x * blockDim.x + threadIdx.x;
    const bool act = cv < s.ncv;
    float4 qmin = make_float4(0.0f, 0.0f, 0.0f, 0.0f), qmax = qmin;
    if (act) {
        const PpfVertexParam &cq = s.cm_vparam[s.cm_vprop[cv].param_index];
        const Vec3 y = X(s.cm_x, cv);
        const float m = 0.5f * cq.ghat + cq.offset;
        qmin = make_float4(y[0] - m, y[1] - m, y[2] - m, 1.0f);
        qmax = make_float4(y[0] + m, y[1] + m, y[2] + m, 0.0f);
    }
    MeshVertexCcdOp op{s, a, act ? cv : 0u, a.max_t};
    warp_query<M>(fb, act, qmin, qmax, op, &a.st->status);
    warp_min_toi(&a.st->toi_vf_bits, op.toi);
}

// One lane per surface vertex in the vertex tree's Morton order; the warp's
// lanes walk the face, vertex and collision-face trees together.
template <LeafTests M>
__global__ void k_ccd_vertex(Scene s, BvhView fb, BvhView vb, LineSearchArgs a) {
    const unsigned t = blockIdx.x * blockDim.x + threadIdx.x;
    const bool act = t < s.n_surf;
    const unsigned v = act ? vb.node[t].x - 1u : 0u;
    float toi = a.max_t;
    float4 qmin = make_float4(0.0f, 0.0f, 0.0f, 0.0f), qmax = qmin;
    bool mesh = false;
    if (act) {
        toi = vertex_constraint_toi(s, a, v);
        float m = s.margin_vert[v];
        Vec3 p0 = X(a.x0, v), p1 = sweep_end(a.x0, a.x1, v, a.max_t);
        qmin = make_float4(fminf(p0[0], p1[0]) - m, fminf(p0[1], p1[1]) - m,
                           fminf(p0[2], p1[2]) - m, 1.0f);
        qmax = make_float4(fmaxf(p0[0], p1[0]) + m, fmaxf(p0[1], p1[1]) + m,
                           fmaxf(p0[2], p1[2]) + m, 0.0f);
        const PpfVertexProp &vp = s.vprop[v];
        mesh = s.ncf && vp.fix_index == 0 && vp.mass > 0.0f;
    }
    PointFaceCcdOp pf{s, a, v, a.max_t};
    warp_query<M>(fb, act, qmin, qmax, pf, &a.st->status);
    PointPointCcdOp pp{s, a, v, a.max_t};
    warp_query<M>(vb, act, qmin, qmax, pp, &a.st->status);
    toi = fminf(toi, fminf(pf.toi, pp.toi));
    if (s.ncf) {
        MeshPointFaceCcdOp mf{s, a, v, a.max_t};
        warp_query<M>(s.cm_face_bvh, mesh, qmin, qmax, mf, &a.st->status);
        toi = fminf(toi, mf.toi);
    }
    warp_min_toi(&a.st->toi_vf_bits, toi);
}

struct EdgeEdgeCcdOp {
    const Scene &s;
    const LineSearchArgs &a;
    unsigned e;
    float toi;
    __device__ bool pre(unsigned o) const { return e < o; }
    __device__ void operator()(unsigned o) {
        const unsigned *e0 = s.edge + 2 * e;
        const unsigned *e1 = s.edge + 2 * o;
        bool either_dyn = !s.eprop[e].fixed || !s.eprop[o].fixed;
        bool both_collider = s.vprop[e0[0]].collider && s.vprop[e1[0]].collider;
        if (!(e < o) || !either_dyn || both_collider) return;
        const PpfEdgeParam &pa = s.eparam[s.eprop[e].param_index];
        const PpfEdgeParam &pb = s.eparam[s.eprop[o].param_index];
        float offset = pa.offset + pb.offset;
        float ghat = 0.5f * (pa.ghat + pb.ghat);
        float r = a.max_t;
        accd::CcdFlag fl;
        bool shared = e0[0] == e1[0] || e0[0] == e1[1] || e0[1] == e1[0] || e0[1] == e1[1];
        if (!shared) {
            r = accd::edge_edge(X(a.x0, e0[0]), X(a.x0, e0[1]), X(a.x0, e1[0]), X(a.x0, e1[1]),
                                X(a.x1, e0[0]), X(a.x1, e0[1]), X(a.x1, e1[0]), X(a.x1, e1[1]),
                                offset, ghat, a.max_t, a.ccd_eps, &fl);
        } else {
            const unsigned ij[4][2] = {{0, 0}, {0, 1}, {1, 0}, {1, 1}};
            for (int k = 0; k < 4; ++k) {
                unsigned i = ij[k][0], j = ij[k][1];
                if (e0[i] == e1[j]) {
                    unsigned i0 = e0[i], i1 = e0[1 - i], i2 = e1[1 - j];
                    accd::CcdFlag f0, f1;
                    float t0 = accd::point_edge(X(a.x0, i1), X(a.x1, i1), X(a.x0, i0),
                                                X(a.x0, i2), X(a.x1, i0), X(a.x1, i2), offset,
                                                ghat, a.max_t, a.ccd_eps, &f0);
                    float t1 = accd::point_edge(X(a.x0, i2), X(a.x1, i2), X(a.x0, i0),
                                                X(a.x0, i1), X(a.x1, i0), X(a.x1, i1), offset,
                                                ghat, a.max_t, a.ccd_eps, &f1);
                    r = fminf(t0, t1);
                    fl.overlap = f0.overlap || f1.overlap;
                    break;
                }
            }
        }
        if (r < a.max_t) {
            toi = fminf(toi, r);
            if (r == 0.0f) {
                record_overlap(a.st, fl, e0[0], e1[0], 1u);
                if (!fl.overlap) atomicOr(&a.st->overlap, 1u);
            }
        }
    }
};

// One work item per edge piece: the piece swept from the previous iterate to
// the vertex/face seed time. A leaf found by two pieces is tested twice;
// the result is a minimum, so that changes nothing.
template <LeafTests M>
__global__ void k_ccd_edge(Scene s, BvhView eb, LineSearchArgs a, EdgePieces ep) {
    const unsigned total = ep.off[ep.n];
    const float seed = __uint_as_float(a.st->toi_vf_bits);
    for (WarpItems w; w.base < total; w.base += w.stride) {
        const unsigned item = w.base + w.lane;
        const bool act = item < total;
        unsigned e = 0u;
        bool mesh = false;
        float4 qmin = make_float4(0.0f, 0.0f, 0.0f, 0.0f), qmax = qmin;
        if (act) {
            const unsigned t = piece_slot(ep, item);
            const unsigned k = item - ep.off[t], K = ep.off[t + 1] - ep.off[t];
            e = eb.node[t].x - 1u;
            const unsigned *ed = s.edge + 2 * e;
            float m = s.margin_edge[e];
            Vec3 a0 = X(a.x0, ed[0]), b0 = X(a.x0, ed[1]);
            Vec3 a1 = sweep_end(a.x0, a.x1, ed[0], seed), b1 = sweep_end(a.x0, a.x1, ed[1], seed);
            Vec3 p0 = piece_point(a0, b0, k, K), p1 = piece_point(a0, b0, k + 1, K);
            Vec3 q0 = piece_point(a1, b1, k, K), q1 = piece_point(a1, b1, k + 1, K);
            qmin.x = fminf(fminf(p0[0], p1[0]) - m, fminf(q0[0], q1[0]) - m);
            qmin.y = fminf(fminf(p0[1], p1[1]) - m, fminf(q0[1], q1[1]) - m);
            qmin.z = fminf(fminf(p0[2], p1[2]) - m, fminf(q0[2], q1[2]) - m);
            qmin.w = 1.0f;
            qmax.x = fmaxf(fmaxf(p0[0], p1[0]) + m, fmaxf(q0[0], q1[0]) + m);
            qmax.y = fmaxf(fmaxf(p0[1], p1[1]) + m, fmaxf(q0[1], q1[1]) + m);
            qmax.z = fmaxf(fmaxf(p0[2], p1[2]) + m, fmaxf(q0[2], q1[2]) + m);
            qmax.w = 0.0f;
            mesh = s.nce && !s.eprop[e].fixed && s.eprop[e].mass > 0.0f;
        }
        EdgeEdgeCcdOp op{s, a, e, seed};
        warp_query<M>(eb, act, qmin, qmax, op, &a.st->status);
        if (s.nce) {
            MeshEdgeCcdOp me{s, a, e, op.toi};
            warp_query<M>(s.cm_edge_bvh, mesh, qmin, qmax, me, &a.st->status);
            op.toi = me.toi;
        }
        warp_min_toi(&a.st->toi_bits, op.toi);
    }
}

// Analytic colliders alone, for scenes whose mesh contact is switched off
// (contact.cu:2523-2528 runs this part unconditionally).
__global__ void k_constraint_toi(Scene s, LineSearchArgs a) {
    unsigned v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= s.n_surf) return;
    atomicMin(&a.st->toi_bits, __float_as_uint(vertex_constraint_toi(s, a, v)));
}

__global__ void k_fold_vertex_toi(IterStatus *st) {
    atomicMin(&st->toi_bits, st->toi_vf_bits);
}

__global__ void k_strain_ls(Scene s, LineSearchArgs a) {
    unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= s.nf_shell) return;
    float t = a.max_t;
    const PpfFaceProp &pr = s.fprop[i];
    const PpfFaceParam &fp = s.fparam[pr.param_index];
    if (!pr.fixed && !pr.rest_excluded && fp.strainlimit > 0.0f) {
        float limit = strain::effective_limit(fp.strainlimit, fp.shrink_x, fp.shrink_y);
        const unsigned *f = s.face + 3 * i;
        const float *ir = s.inv_rest + 4 * i;
        Mat2 inv;
        for (int k = 0; k < 4; ++k) inv.m[k] = ir[k];
        // a.x1 is the candidate, a.x0 the previous iterate (strainlimiting.cu:262-268)
        Mat3x2 F0 = bw::deformation_grad(X(a.x0, f[0]), X(a.x0, f[1]), X(a.x0, f[2]), inv);
        Mat3x2 F1 = bw::deformation_grad(X(a.x1, f[0]), X(a.x1, f[1]), X(a.x1, f[2]), inv);
        t = strain::line_search(F0, F1, limit, a.max_t);
    }
    atomicMin(&a.st->sl_toi_bits, __float_as_uint(t));
}

// Rod edges (strainlimiting.cu:192-245): a.x0 the previous iterate, a.x1 the
// candidate, as for the faces.
__global__ void k_rod_strain_ls(Scene s, LineSearchArgs a) {
    unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= s.nr) return;
    float t = a.max_t;
    const PpfEdgeProp &pr = s.eprop[i];
    const PpfEdgeParam &ep = s.eparam[pr.param_index];
    if (!pr.fixed && ep.strainlimit > 0.0f && pr.initial_length > 0.0f) {
        const unsigned *e = s.edge + 2 * i;
        t = rod::strain_line_search(X(a.x0, e[1]) - X(a.x0, e[0]), X(a.x1, e[1]) - X(a.x1, e[0]),
                                    pr.initial_length, ep.strainlimit, a.max_t);
    }
    atomicMin(&a.st->sl_toi_bits, __float_as_uint(t));
}

struct FaceEdgeIsectOp {
    const Scene &s;
    const float *x;
    unsigned e;
    PpfIntersectionRecord *records;
    IterStatus *st;
    __device__ void operator()(unsigned fi) {
        const unsigned *f = s.face + 3 * fi;
        const unsigned *ed = s.edge + 2 * e;
        bool either_dyn = !s.fprop[fi].fixed || !s.eprop[e].fixed;
        bool nonzero = s.fprop[fi].mass > 0.0f || s.eprop[e].mass > 0.0f;
        bool both_collider = s.vprop[ed[0]].collider && s.vprop[f[0]].collider;
        if (!either_dyn || !nonzero || both_collider) return;
        for (int k = 0; k < 3; ++k)
            if (ed[0] == f[k] || ed[1] == f[k]) return;
        Vec3 t0 = X(x, f[0]), t1 = X(x, f[1]), t2 = X(x, f[2]);
        Vec3 y0 = X(x, ed[0]), y1 = X(x, ed[1]);
        if (!contact::edge_triangle_intersect(y0, y1, t0, t1, t2)) return;
        unsigned slot = atomicAdd(&st->n_isect, 1u);
        if (slot < PPF_MAX_INTERSECTION_RECORDS) {
            PpfIntersectionRecord &r = records[slot];
            r.type = 0;
            r.elem0 = fi;
            r.elem1 = e;
            r.num_verts0 = 3;
            r.num_verts1 = 2;
            const Vec3 vs[5] = {t0, t1, t2, y0, y1};
            for (int k = 0; k < 5; ++k)
                for (int d = 0; d < 3; ++d) r.positions[3 * k + d] = vs[k][d];
        }
    }
};

struct EdgeEdgeIsectOp {
    const Scene &s;
    const float *x;
    unsigned e;
    PpfIntersectionRecord *records;
    IterStatus *st;
    __device__ bool pre(unsigned o) const { return o < e; }
    __device__ void operator()(unsigned o) {
        if (!(o < e)) return;
        const unsigned *e0 = s.edge + 2 * e;
        const unsigned *e1 = s.edge + 2 * o;
        bool either_dyn = !s.eprop[e].fixed || !s.eprop[o].fixed;
        bool nonzero = s.eprop[e].mass > 0.0f || s.eprop[o].mass > 0.0f;
        bool both_collider = s.vprop[e0[0]].collider && s.vprop[e1[0]].collider;
        if (!either_dyn || !nonzero || both_collider) return;
        float offset = s.eparam[s.eprop[e].param_index].offset +
                       s.eparam[s.eprop[o].param_index].offset;
        bool hit = false;
        bool shared = e0[0] == e1[0] || e0[0] == e1[1] || e0[1] == e1[0] || e0[1] == e1[1];
        if (!shared) {
            hit = contact::edges_within_offset(X(x, e0[0]), X(x, e0[1]), X(x, e1[0]),
                                               X(x, e1[1]), offset);
        } else {
            const unsigned ij[4][2] = {{0, 0}, {0, 1}, {1, 0}, {1, 1}};
            for (int k = 0; k < 4 && !hit; ++k) {
                unsigned i = ij[k][0], j = ij[k][1];
                if (e0[i] == e1[j])
                    hit = contact::shared_edges_within_offset(X(x, e0[i]), X(x, e0[1 - i]),
                                                              X(x, e1[1 - j]), offset);
            }
        }
        if (!hit) return;
        unsigned slot = atomicAdd(&st->n_isect, 1u);
        if (slot < PPF_MAX_INTERSECTION_RECORDS) {
            PpfIntersectionRecord &r = records[slot];
            r.type = 1;
            r.elem0 = e;
            r.elem1 = o;
            r.num_verts0 = 2;
            r.num_verts1 = 2;
            const unsigned vs[4] = {e0[0], e0[1], e1[0], e1[1]};
            for (int k = 0; k < 4; ++k)
                for (int d = 0; d < 3; ++d) r.positions[3 * k + d] = x[3 * vs[k] + d];
        }
    }
};

// One work item per edge piece, each leaf reported from its first piece.
// Piece boxes carry the edge's contact offset plus a rounding guard: every
// pierced face contains the pierce point, and every edge nearer than the
// combined offset lies within the edge's offset plus its own leaf margin.
// A free edge of positive mass piercing a collision face
// (contact/contact.cu:2955-2987, 3114-3122).
struct MeshFaceEdgeIsectOp {
    const Scene &s;
    const float *x;
    unsigned e;
    PpfIntersectionRecord *records;
    IterStatus *st;
    __device__ void operator()(unsigned fi) {
        const unsigned *f = s.cm_face + 3 * fi;
        const unsigned *ed = s.edge + 2 * e;
        const Vec3 t0 = X(s.cm_x, f[0]), t1 = X(s.cm_x, f[1]), t2 = X(s.cm_x, f[2]);
        const Vec3 y0 = X(x, ed[0]), y1 = X(x, ed[1]);
        if (!contact::edge_triangle_intersect(y0, y1, t0, t1, t2)) return;
        unsigned slot = atomicAdd(&st->n_isect, 1u);
        if (slot < PPF_MAX_INTERSECTION_RECORDS) {
            PpfIntersectionRecord &r = records[slot];
            r.type = 2;
            r.elem0 = fi;
            r.elem1 = e;
            r.num_verts0 = 3;
            r.num_verts1 = 2;
            const Vec3 vs[5] = {t0, t1, t2, y0, y1};
            for (int k = 0; k < 5; ++k)
                for (int d = 0; d < 3; ++d) r.positions[3 * k + d] = vs[k][d];
        }
    }
};

template <LeafTests M>
__global__ void k_isect(Scene s, BvhView fb, BvhView eb, const float *x,
                        PpfIntersectionRecord *rec, IterStatus *st, EdgePieces ep) {
    const unsigned total = ep.off[ep.n];
    for (WarpItems w; w.base < total; w.base += w.stride) {
        const unsigned item = w.base + w.lane;
        const bool act = item < total;
        unsigned e = 0u;
        bool mesh = false;
        float4 qmin = make_float4(0.0f, 0.0f, 0.0f, 0.0f), qmax = qmin;
        float4 xmin = make_float4(0.0f, 0.0f, 0.0f, 0.0f), xmax = xmin;
        if (act) {
            const unsigned t = piece_slot(ep, item);
            const unsigned k = item - ep.off[t], K = ep.off[t + 1] - ep.off[t];
            e = eb.node[t].x - 1u;
            const unsigned *ed = s.edge + 2 * e;
            Vec3 a = X(x, ed[0]), b = X(x, ed[1]);
            const float guard =
                1e-6f * (1.0f + fmaxf(fmaxf(fmaxf(fabsf(a[0]), fabsf(a[1])),
                                            fmaxf(fabsf(a[2]), fabsf(b[0]))),
                                      fmaxf(fabsf(b[1]), fabsf(b[2]))));
            const float m = s.eparam[s.eprop[e].param_index].offset + guard;
            seg_box(piece_point(a, b, k, K), piece_point(a, b, k + 1, K), m, qmin, qmax);
            // a piece after the first excludes what its predecessor reports;
            // the first piece's exclusion box (w = 0) overlaps nothing
            if (k > 0u)
                seg_box(piece_point(a, b, k - 1, K), piece_point(a, b, k, K), m, xmin, xmax);
            mesh = s.ncf && s.eprop[e].mass > 0.0f;
        }
        FaceEdgeIsectOp op{s, x, e, rec, st};
        warp_query<M>(fb, act, qmin, qmax, op, &st->status, &xmin, &xmax);
        EdgeEdgeIsectOp op2{s, x, e, rec, st};
        warp_query<M>(eb, act, qmin, qmax, op2, &st->status, &xmin, &xmax);
        if (s.ncf) {
            MeshFaceEdgeIsectOp op3{s, x, e, rec, st};
            warp_query<M>(s.cm_face_bvh, mesh, qmin, qmax, op3, &st->status, &xmin, &xmax);
        }
    }
}

} // namespace

void launch_contact_line_search(const Scene &s, const BvhView &fb, const BvhView &eb,
                                const BvhView &vb, const LineSearchArgs &a, float piece_len,
                                PieceBuffers &pb, cudaStream_t q) {
    if (s.n_surf) {
        if (s.tune.ccd_vertex)
            k_ccd_vertex<LeafTests::kImmediate><<<div_up(s.n_surf, kB), kB, 0, q>>>(s, fb, vb, a);
        else
            k_ccd_vertex<LeafTests::kWarpRounds><<<div_up(s.n_surf, kB), kB, 0, q>>>(s, fb, vb, a);
        PPF_LAUNCH_CHECK();
    }
    if (s.ncv) { // before the edge seed is read
        if (s.tune.ccd_mesh_vertex)
            k_ccd_mesh_vertex<LeafTests::kImmediate><<<div_up(s.ncv, kB), kB, 0, q>>>(s, fb, a);
        else
            k_ccd_mesh_vertex<LeafTests::kWarpRounds><<<div_up(s.ncv, kB), kB, 0, q>>>(s, fb, a);
        PPF_LAUNCH_CHECK();
    }
    if (s.ne) {
        launch_edge_pieces(s, eb, a.x0, a.x1, &a.st->toi_vf_bits, piece_len, pb, q);
        const EdgePieces ep{pb.off, s.ne};
        if (s.tune.ccd_edge)
            k_ccd_edge<LeafTests::kImmediate><<<piece_grid(s.ne, kB), kB, 0, q>>>(s, eb, a, ep);
        else
            k_ccd_edge<LeafTests::kWarpRounds><<<piece_grid(s.ne, kB), kB, 0, q>>>(s, eb, a, ep);
        PPF_LAUNCH_CHECK();
    }
    k_fold_vertex_toi<<<1, 1, 0, q>>>(a.st);
    PPF_LAUNCH_CHECK();
}

void launch_constraint_line_search(const Scene &s, const LineSearchArgs &a, cudaStream_t q) {
    if (!s.n_surf || (!s.nsphere && !s.nfloor)) return;
    k_constraint_toi<<<div_up(s.n_surf, kB), kB, 0, q>>>(s, a);
    PPF_LAUNCH_CHECK();
}

void launch_strain_line_search(const Scene &s, const LineSearchArgs &a, cudaStream_t q) {
    if (s.nf_shell) {
        k_strain_ls<<<div_up(s.nf_shell, kB), kB, 0, q>>>(s, a);
        PPF_LAUNCH_CHECK();
    }
    if (s.nr) {
        k_rod_strain_ls<<<div_up(s.nr, kB), kB, 0, q>>>(s, a);
        PPF_LAUNCH_CHECK();
    }
}

void launch_intersection_check(const Scene &s, const BvhView &fb, const BvhView &eb,
                               const float *x, PpfIntersectionRecord *records, IterStatus *st,
                               float piece_len, PieceBuffers &pb, cudaStream_t q) {
    if (!s.ne) return;
    launch_edge_pieces(s, eb, x, nullptr, nullptr, piece_len, pb, q);
    const EdgePieces ep{pb.off, s.ne};
    if (s.tune.isect)
        k_isect<LeafTests::kImmediate>
            <<<piece_grid(s.ne, kB), kB, 0, q>>>(s, fb, eb, x, records, st, ep);
    else
        k_isect<LeafTests::kWarpRounds>
            <<<piece_grid(s.ne, kB), kB, 0, q>>>(s, fb, eb, x, records, st, ep);
    PPF_LAUNCH_CHECK();
}

} // namespace gpu
} // namespace ppf
