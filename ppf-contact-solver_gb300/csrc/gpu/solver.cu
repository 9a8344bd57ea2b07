// solver.cu -- per-step Newton solve (crates/ppf-cts-solver/src/cpp/main/
// main.cu:267-1649) on the device, driven from the host with two small
// synchronizations per Newton iteration (contact-pair counts after detection,
// the iteration's status block after the line search).
#include "fatal.cuh"
#include "solver.cuh"
#include "fsai.cuh"

#include <algorithm>
#include <chrono>
#include <cstring>

namespace ppf {
namespace gpu {

namespace {

constexpr unsigned kB = 256;

template <class T> void upload(DevBuf<T> &d, const T *h, size_t n) {
    d.reserve(n ? n : 1);
    if (n) PPF_CUDA(cudaMemcpy(d.data(), h, n * sizeof(T), cudaMemcpyHostToDevice));
    g_h2d_bytes += n * sizeof(T);
}
template <class T> void upload(DevBuf<T> &d, const std::vector<T> &h) {
    upload(d, h.data(), h.size());
}

// target = x + (x - x_prev) dt / dt_prev + dt^2 g; pinned: the pin's position
// (main.cu:491-511).
__global__ void k_compute_target(unsigned n, const float *curr, const float *prev,
                                 const PpfVertexProp *vprop, const PpfFixPair *fix,
                                 float *target, float dt, float prev_dt, float gx, float gy,
                                 float gz, int inactive) {
    unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    if (vprop[i].fix_index > 0) {
        const PpfFixPair &f = fix[vprop[i].fix_index - 1];
        for (int d = 0; d < 3; ++d) target[3 * i + d] = f.position.v[d];
        return;
    }
    float tr = dt / prev_dt, h2 = dt * dt;
    const float g[3] = {gx, gy, gz};
    for (int d = 0; d < 3; ++d) {
        float x1 = curr[3 * i + d], x0 = prev[3 * i + d];
        float y = (x1 - x0) * tr + h2 * g[d];
        target[3 * i + d] = inactive ? x1 : x1 + y;
    }
}

__global__ void k_rewind_fix(unsigned nfix, PpfFixPair *fix, float back) {
    unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nfix) return;
    PpfFixPair &f = fix[i];
    if (f.kinematic)
        for (int d = 0; d < 3; ++d) f.position.v[d] = f.position.v[d] - back * f.step_delta.v[d];
}

__global__ void k_seed_dx(unsigned n, const PpfVertexProp *vprop, const float *x,
                          const float *target, float *dx) {
    unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    if (vprop[i].fix_index > 0)
        for (int d = 0; d < 3; ++d) dx[3 * i + d] = x[3 * i + d] - target[3 * i + d];
}

__global__ void k_fold_diag(unsigned n, const unsigned *diag_slot, const float *diag,
                            float *fixed_val) {
    unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float *d = fixed_val + 9 * (size_t)diag_slot[i];
    for (int k = 0; k < 9; ++k) d[k] += diag[9 * i + k];
}

__global__ void k_max_dx(unsigned n, const float *dx, IterStatus *st) {
    unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
    float m = 0.0f;
    if (i < n) {
        float a = dx[3 * i], b = dx[3 * i + 1], c = dx[3 * i + 2];
        m = sqrtf(a * a + b * b + c * c);
    }
    for (int off = 16; off > 0; off >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, off));
    if ((threadIdx.x & 31u) == 0 && m > 0.0f) atomicMax(&st->max_dx_bits, __float_as_uint(m));
}

// target <- eval_x; eval_x -= min(1, max_dx / |dx|_max) dx (main.cu:1142-1188)
// An iteration flagged for a repeat (a pair list or the contact-block
// capacity overran) leaves both untouched.
__global__ void k_apply_dx(unsigned n, float *x, float *target, const float *dx,
                           IterStatus *st, float max_dx_param) {
    unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
    if (st->status & STATUS_PAIR_OVERFLOW) return;
    float mdx = __uint_as_float(st->max_dx_bits);
    float rescale = fminf(1.0f, max_dx_param / mdx);
    if (i == 0) st->rescale = rescale;
    if (i >= n) return;
    for (int d = 0; d < 3; ++d) {
        float v = x[3 * i + d];
        target[3 * i + d] = v;
        x[3 * i + d] = v - rescale * dx[3 * i + d];
    }
}

__global__ void k_apply_toi(unsigned n, float *x, const float *target, float toi) {
    unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    for (int d = 0; d < 3; ++d) {
        float t = target[3 * i + d];
        float dd = toi * (x[3 * i + d] - t);
        x[3 * i + d] = t + dd;
    }
}

__global__ void k_init_ls(IterStatus *st, float max_t, PcgResult *res) {
    st->toi_bits = __float_as_uint(max_t);
    st->toi_vf_bits = __float_as_uint(max_t);
    st->sl_toi_bits = __float_as_uint(max_t);
    st->pin_infeasible = 0xFFFFFFFFu;
    st->overlap = 0u;
    st->overlap_v0 = 0xFFFFFFFFu;
    st->overlap_v1 = 0xFFFFFFFFu;
    st->overlap_kind = 0xFFFFFFFFu;
    st->pcg_iter = res->iter;
    st->pcg_resid = res->resid;
    st->pcg_state = res->state;
    st->pcg_err0 = res->err0;
    st->pcg_break_cause = res->break_cause;
    st->pcg_break_val = res->break_val;
    st->status |= res->status;
}

// After a factored solve: when it did not converge (stalled, broke down or
// reached the block-Jacobi count), restore the solve's start (r = b,
// dx = dx0) and flag the block-Jacobi solve that follows to run. After a
// Schwarz solve (any_failure 0) only a non-positive r^T z does that.
__global__ void k_factor_verdict(unsigned n3, const PcgResult *res, int any_failure,
                                 const float *b, const float *dx0, float *r, float *dx,
                                 unsigned *run_plain, IterStatus *st) {
    const unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
    const bool redo = any_failure ? res->state != 0 : (res->state == 2 && res->break_cause == 2);
    if (i == 0) {
        *run_plain = redo ? 1u : 0u;
        st->factor_iter = res->iter;
        st->fallback = redo ? 1u : 0u;
    }
    if (redo && i < n3) {
        r[i] = b[i];
        dx[i] = dx0[i];
    }
}

__global__ void k_override_velocity(const unsigned *idx, unsigned count, const float *curr,
                                    float *prev, float vx, float vy, float vz) {
    unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count) return;
    unsigned v = idx[i];
    prev[3 * v] = curr[3 * v] - vx;
    prev[3 * v + 1] = curr[3 * v + 1] - vy;
    prev[3 * v + 2] = curr[3 * v + 2] - vz;
}

__global__ void k_override_angular(const unsigned *idx, unsigned count, const float *curr,
                                   float *prev, float wx, float wy, float wz, float cx,
                                   float cy, float cz, float dt) {
    unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count) return;
    unsigned v = idx[i];
    float rx = curr[3 * v] - cx, ry = curr[3 * v + 1] - cy, rz = curr[3 * v + 2] - cz;
    float ux = wy * rz - wz * ry, uy = wz * rx - wx * rz, uz = wx * ry - wy * rx;
    prev[3 * v] = prev[3 * v] - ux * dt;
    prev[3 * v + 1] = prev[3 * v + 1] - uy * dt;
    prev[3 * v + 2] = prev[3 * v + 2] - uz * dt;
}

float bits_to_float(unsigned u) {
    float f;
    std::memcpy(&f, &u, sizeof(f));
    return f;
}

unsigned next_pow2(unsigned long long v) {
    unsigned long long p = 1024;
    while (p < v) p <<= 1;
    return (unsigned)p;
}

} // namespace

Solver &solver_instance() {
    static Solver s;
    return s;
}

Scene Solver::scene() const {
    Scene s{};
    s.n = n_;
    s.n_surf = n_surf_;
    s.nf = nf_;
    s.ne = ne_;
    s.nh = nh_;
    s.nr = nr_;
    s.nf_shell = nf_shell_;
    s.nt = nt_;
    s.tet = tet_.data();
    s.tprop = tprop_.data();
    s.tparam = tparam_.data();
    s.inv_rest3 = inv_rest3_.data();
    s.tet_slot = tet_slot_.data();
    s.hinge_type = hinge_type_.data();
    s.tune = tune_;
    s.nstitch = nstitch_;
    s.stitch = stitch_.data();
    s.stitch_slot = stitch_slot_.data();
    s.face = face_.data();
    s.edge = edge_.data();
    s.hinge = hinge_.data();
    s.vprop = vprop_.data();
    s.eprop = eprop_.data();
    s.fprop = fprop_.data();
    s.hprop = hprop_.data();
    s.vparam = vparam_.data();
    s.eparam = eparam_.data();
    s.fparam = fparam_.data();
    s.hparam = hparam_.data();
    s.inv_rest = inv_rest_.data();
    s.vf_off = vf_off_.data();
    s.vf = vf_.data();
    s.ve_off = ve_off_.data();
    s.ve = ve_.data();
    s.ef_off = ef_off_.data();
    s.ef = ef_.data();
    s.fixed_off = fixed_off_.data();
    s.fixed_col = fixed_col_.data();
    s.fixed_tr_off = fixed_tr_off_.data();
    s.fixed_tr = fixed_tr_.data();
    s.fixed_diag = fixed_diag_.data();
    s.face_slot = face_slot_.data();
    s.hinge_slot = hinge_slot_.data();
    s.edge_slot = edge_slot_.data();
    s.bend_slot = bend_slot_.data();
    s.dof_mask = dof_mask_.data();
    s.fix = fix_.data();
    s.nfix = nfix_;
    s.pull = pull_.data();
    s.npull = npull_;
    s.sphere = sphere_.data();
    s.nsphere = nsphere_;
    s.floor = floor_.data();
    s.nfloor = nfloor_;
    s.margin_face = margin_face_.data();
    s.margin_edge = margin_edge_.data();
    s.margin_vert = margin_vert_.data();
    s.vert_active = use_active_ ? vert_active_.data() : nullptr;
    s.edge_active = use_active_ ? edge_active_.data() : nullptr;
    s.ncv = ncv_;
    s.ncf = ncf_;
    s.nce = nce_;
    s.cm_x = cm_x_.data();
    s.cm_face = cm_face_.data();
    s.cm_edge = cm_edge_.data();
    s.cm_vprop = cm_vprop_.data();
    s.cm_fprop = cm_fprop_.data();
    s.cm_eprop = cm_eprop_.data();
    s.cm_vparam = cm_vparam_.data();
    s.cm_fparam = cm_fparam_.data();
    s.cm_eparam = cm_eparam_.data();
    s.cm_face_bvh = view(cm_bvh_face_);
    s.cm_edge_bvh = view(cm_bvh_edge_);
    return s;
}

// The collision mesh as the DataSet gives it, and its face and edge trees
// over the mesh as it is (lbvh/lbvh.cu:1100-1118), built once.
void Solver::upload_collision_mesh(const PpfCollisionMesh &cm) {
    ncv_ = cm.vertex.size;
    ncf_ = cm.face.size;
    nce_ = cm.edge.size;
    if (!ncv_) return;
    upload(cm_x_, (const float *)cm.vertex.data, 3 * (size_t)ncv_);
    upload(cm_face_, (const unsigned *)cm.face.data, 3 * (size_t)ncf_);
    upload(cm_edge_, (const unsigned *)cm.edge.data, 2 * (size_t)nce_);
    upload(cm_vprop_, cm.prop.vertex.data, cm.prop.vertex.size);
    upload(cm_fprop_, cm.prop.face.data, cm.prop.face.size);
    upload(cm_eprop_, cm.prop.edge.data, cm.prop.edge.size);
    upload(cm_vparam_, cm.param_arrays.vertex.data, cm.param_arrays.vertex.size);
    upload(cm_fparam_, cm.param_arrays.face.data, cm.param_arrays.face.size);
    upload(cm_eparam_, cm.param_arrays.edge.data, cm.param_arrays.edge.size);
    std::vector<float> mf(ncf_), me(nce_);
    for (unsigned i = 0; i < ncf_; ++i) {
        const PpfFaceParam &p = cm.param_arrays.face.data[cm.prop.face.data[i].param_index];
        mf[i] = 0.5f * p.ghat + p.offset;
    }
    for (unsigned i = 0; i < nce_; ++i) {
        const PpfEdgeParam &p = cm.param_arrays.edge.data[cm.prop.edge.data[i].param_index];
        me[i] = 0.5f * p.ghat + p.offset;
    }
    upload(cm_margin_f_, mf);
    upload(cm_margin_e_, me);
    unsigned *status = &st_.data()->status;
    const float *x = cm_x_.data();
    PrimSet pf{PRIM_FACE, ncf_, cm_face_.data(), cm_margin_f_.data(), nullptr};
    PrimSet pe{PRIM_EDGE, nce_, cm_edge_.data(), cm_margin_e_.data(), nullptr};
    if (ncf_) lbvh_build(cm_bvh_face_, pf, x, x, x, 1.0f, sort_ws_, status, q_);
    if (nce_) lbvh_build(cm_bvh_edge_, pe, x, x, x, 1.0f, sort_ws_, status, q_);
}

StepParams Solver::step_params(float dt) const {
    StepParams p{};
    p.dt = dt;
    p.prev_dt = param->prev_dt;
    p.time = (float)param->time;
    p.air_friction = param->air_friction;
    p.air_density = param->air_density;
    p.isotropic_air_friction = param->isotropic_air_friction;
    p.friction_eps = param->friction_eps;
    p.eiganalysis_eps = param->eiganalysis_eps;
    p.constraint_tol = param->constraint_tol;
    p.line_search_max_t = param->line_search_max_t;
    p.ccd_eps = param->ccd_eps;
    for (int d = 0; d < 3; ++d) {
        p.gravity[d] = param->gravity.v[d];
        p.wind[d] = param->wind.v[d];
    }
    p.barrier = param->barrier;
    p.friction_mode = param->friction_mode;
    p.inactive_momentum = param->inactive_momentum ? 1 : 0;
    p.fix_xz = param->fix_xz;
    p.stitch_length_factor = param->stitch_length_factor;
    return p;
}

AssemblyBuffers Solver::abuf() {
    AssemblyBuffers b{};
    b.force = force_.data();
    b.diag = diag_.data();
    b.fixed_val = fixed_val_.data();
    b.fixed_tmp = fixed_tmp_.data();
    b.x = eval_x_.data();
    b.x0 = curr_.data();
    b.target = target_.data();
    b.st = st_.data();
    b.params = sp_dev_.data();
    return b;
}

PcgOperator Solver::pcg_operator() const {
    return PcgOperator{n_,
                       sell_view(fixed_sell_),
                       contact_view(dyn_layout_),
                       overflow_view(dyn_layout_),
                       inv_diag_.data(),
                       factor_active_ ? factor_.view(factor_eps_) : PcgFactor{},
                       schwarz_active_ ? schwarz_.view() : SchwarzView{}};
}

bool Solver::set_preconditioner(int kind, float param) {
    if (kind < 0 || kind > 4 || kind == 3 || (kind == 2 && !learned_ready_)) return false;
    precond_kind_ = kind;
    if (kind == 1) precond_param_ = param > 0.0f ? param : 0.5f;
    plain_iters_ = 0;
    return true;
}

// The factor of the assembled operator (after the block-Jacobi inverse).
void Solver::build_factor() {
    const PcgOperator A = PcgOperator{n_, sell_view(fixed_sell_), contact_view(dyn_layout_),
                                      overflow_view(dyn_layout_), inv_diag_.data(),
                                      PcgFactor{}};
    reserve_factor(A, fixed_sell_.slots, dyn_layout_.sell.slots, dyn_layout_.ovf_entries,
                   factor_);
    launch_chol_inv(n_, fixed_val_.data(), fixed_diag_.data(), factor_.cinv.data(),
                    &st_.data()->status, q_);
    if (precond_kind_ == 4) {
        FsaiSystem S{n_,
                     fixed_off_.data(),
                     fixed_col_.data(),
                     fixed_val_.data(),
                     fixed_tr_off_.data(),
                     fixed_tr_.data(),
                     dyn_.off,
                     dyn_.col,
                     dyn_.val,
                     dyn_.tr_off,
                     dyn_.tr,
                     fixed_diag_.data(),
                     dof_mask_.data()};
        launch_factor_fsai(A, S, nnz_fixed_, dyn_.cap, fixed_sell_.src.data(),
                           dyn_layout_.sell.src.data(), dyn_layout_.ovf_src.data(), factor_,
                           &st_.data()->status, q_);
    } else if (precond_kind_ == 2) {
        LearnedGraph g;
        g.n = n_;
        g.fixed = LearnedPart{fixed_off_.data(), fixed_col_.data(), fixed_val_.data(),
                              fixed_tr_off_.data(), fixed_tr_.data(), nnz_fixed_};
        // the contact part's edge numbering is only used by the trainer
        g.contact = LearnedPart{dyn_.off, dyn_.col, dyn_.val, dyn_.tr_off, dyn_.tr, 0u};
        g.diag_slot = fixed_diag_.data();
        g.dof_mask = dof_mask_.data();
        g.mass = mass_.data();
        g.cinv = factor_.cinv.data();
        learned_forward_nodes(g, learned_w_.data(), learned_nodes_, q_);
        launch_factor_learned(A, dof_mask_.data(), learned_nodes_.Y.data(), learned_w_.data(),
                              factor_, q_);
    } else {
        launch_factor_first_order(A, dof_mask_.data(), precond_param_, factor_, q_);
    }
}

bool Solver::set_learned_weights(const unsigned short *w, unsigned count) {
    if (!w || count != learned::kWeights) return false;
    learned_w_.reserve(count);
    PPF_CUDA(cudaMemcpy(learned_w_.data(), w, count * sizeof(unsigned short),
                        cudaMemcpyHostToDevice));
    learned_ready_ = true;
    return true;
}

PieceBuffers Solver::pieces() {
    return PieceBuffers{piece_cnt_.data(), piece_off_.data(), piece_tmp_.data()};
}

BvhView Solver::view(const Lbvh &b) const {
    return BvhView{b.node.data(), b.bmin.data(), b.bmax.data(), b.root, b.n, b.link.data()};
}

void Solver::upload_props() {
    upload(vprop_, h_vprop_);
    upload(fprop_, h_fprop_);
    upload(eprop_, h_eprop_);
    upload(hprop_, h_hprop_);
    std::vector<unsigned> mask(n_, 0u);
    for (unsigned i = 0; i < n_; ++i)
        mask[i] = (h_vprop_[i].fix_index > 0 && h_vprop_[i].pdrd_body_index == 0) ? 1u : 0u;
    upload(dof_mask_, mask);
    std::vector<float> mass(n_);
    for (unsigned i = 0; i < n_; ++i) mass[i] = h_vprop_[i].mass;
    upload(mass_, mass);
}

bool Solver::initialize(PpfDataSet *ds, PpfParamSet *prm) {
    host = ds;
    param = prm;
    plain_iters_ = 0; // a new scene's first solve is block-Jacobi again
    schwarz_.ready = false;
    n_ = ds->vertex.curr.size;
    n_surf_ = ds->surface_vert_count;
    nf_ = ds->mesh.mesh.face.size;
    ne_ = ds->mesh.mesh.edge.size;
    nh_ = ds->mesh.mesh.hinge.size;
    nr_ = std::min(ds->rod_count, ne_);
    nf_shell_ = std::min(ds->shell_face_count, nf_);
    nt_ = ds->mesh.mesh.tet.size;
    if (nt_ && ds->inv_rest3x3.size != nt_)
        throw FatalError(4, "inv_rest3x3 does not match the tets");
    if (!q_) PPF_CUDA(cudaStreamCreateWithFlags(&q_, cudaStreamNonBlocking));
    if (!ev0_) {
        PPF_CUDA(cudaEventCreate(&ev0_));
        PPF_CUDA(cudaEventCreate(&ev1_));
        PPF_CUDA(cudaEventCreate(&evs0_));
        PPF_CUDA(cudaEventCreate(&evs1_));
    }
    // topology
    upload(face_, (const unsigned *)ds->mesh.mesh.face.data, 3 * (size_t)nf_);
    upload(edge_, (const unsigned *)ds->mesh.mesh.edge.data, 2 * (size_t)ne_);
    upload(hinge_, (const unsigned *)ds->mesh.mesh.hinge.data, 4 * (size_t)nh_);
    h_vprop_.assign(ds->prop.vertex.data, ds->prop.vertex.data + ds->prop.vertex.size);
    h_fprop_.assign(ds->prop.face.data, ds->prop.face.data + ds->prop.face.size);
    h_eprop_.assign(ds->prop.edge.data, ds->prop.edge.data + ds->prop.edge.size);
    h_hprop_.assign(ds->prop.hinge.data, ds->prop.hinge.data + ds->prop.hinge.size);
    upload_props();
    upload(vparam_, ds->param_arrays.vertex.data, ds->param_arrays.vertex.size);
    upload(eparam_, ds->param_arrays.edge.data, ds->param_arrays.edge.size);
    upload(fparam_, ds->param_arrays.face.data, ds->param_arrays.face.size);
    upload(hparam_, ds->param_arrays.hinge.data, ds->param_arrays.hinge.size);
    upload(inv_rest_, (const float *)ds->inv_rest2x2.data, 4 * (size_t)ds->inv_rest2x2.size);
    auto up_vv = [&](const PpfVecVecU32 &v, DevBuf<unsigned> &off, DevBuf<unsigned> &dat,
                     unsigned rows) {
        std::vector<unsigned> o(rows + 1, 0u);
        if (v.size && v.offset)
            for (unsigned i = 0; i <= rows && i <= v.size; ++i) o[i] = v.offset[i];
        for (unsigned i = v.size + 1; i <= rows; ++i) o[i] = o[v.size];
        upload(off, o);
        upload(dat, v.data, v.nnz);
    };
    up_vv(ds->mesh.neighbor.vertex.face, vf_off_, vf_, n_);
    up_vv(ds->mesh.neighbor.vertex.edge, ve_off_, ve_, n_);
    up_vv(ds->mesh.neighbor.edge.face, ef_off_, ef_, ne_);
    // fixed pattern (builder.rs:1244-1356), diagonal slots, element slots
    const PpfVecVecU32 &ft = ds->fixed_index_table;
    std::vector<unsigned> foff(ft.offset, ft.offset + n_ + 1);
    std::vector<unsigned> fcol(ft.data, ft.data + foff[n_]);
    nnz_fixed_ = foff[n_];
    upload(fixed_off_, foff);
    upload(fixed_col_, fcol);
    const PpfVecVecVec2u &tt = ds->transpose_table;
    std::vector<unsigned> toff(tt.offset, tt.offset + n_ + 1);
    std::vector<uint2> tr(toff[n_]);
    for (unsigned k = 0; k < toff[n_]; ++k) tr[k] = make_uint2(tt.data[k].v[0], tt.data[k].v[1]);
    upload(fixed_tr_off_, toff);
    upload(fixed_tr_, tr);
    sell_build_fixed(n_, foff, fcol, toff, tr, fixed_sell_);
    auto slot_of = [&](unsigned i, unsigned j) -> unsigned {
        if (i > j) return kSentinel;
        auto b = fcol.begin() + foff[i], e = fcol.begin() + foff[i + 1];
        auto it = std::lower_bound(b, e, j);
        if (it == e || *it != j) return kSentinel;
        return (unsigned)(it - fcol.begin());
    };
    std::vector<unsigned> dslot(n_);
    for (unsigned i = 0; i < n_; ++i) {
        dslot[i] = slot_of(i, i);
        if (dslot[i] == kSentinel) throw FatalError(4, "fixed pattern lacks a diagonal block");
    }
    upload(fixed_diag_, dslot);
    std::vector<unsigned> fs(9 * (size_t)nf_), hs(16 * (size_t)nh_);
    const unsigned *F = (const unsigned *)ds->mesh.mesh.face.data;
    for (unsigned f = 0; f < nf_; ++f)
        for (int a = 0; a < 3; ++a)
            for (int b = 0; b < 3; ++b) fs[9 * f + 3 * a + b] = slot_of(F[3 * f + a], F[3 * f + b]);
    const unsigned *Hh = (const unsigned *)ds->mesh.mesh.hinge.data;
    for (unsigned h = 0; h < nh_; ++h) {
        const unsigned r[4] = {Hh[4 * h + 2], Hh[4 * h + 1], Hh[4 * h], Hh[4 * h + 3]};
        for (int a = 0; a < 4; ++a)
            for (int b = 0; b < 4; ++b) hs[16 * h + 4 * a + b] = slot_of(r[a], r[b]);
    }
    upload(face_slot_, fs);
    upload(hinge_slot_, hs);
    // rod edges: 4 blocks each; the rod-bend stencil (j, i, k) of every vertex
    // with two edges and no face (energy.cu:555-565): 9 blocks, else sentinels
    const unsigned *E = (const unsigned *)ds->mesh.mesh.edge.data;
    std::vector<unsigned> es(4 * (size_t)nr_), bs;
    for (unsigned e = 0; e < nr_; ++e)
        for (int a = 0; a < 2; ++a)
            for (int b = 0; b < 2; ++b) es[4 * e + 2 * a + b] = slot_of(E[2 * e + a], E[2 * e + b]);
    if (nr_) {
        bs.assign(9 * (size_t)n_, kSentinel);
        const PpfVecVecU32 &ve = ds->mesh.neighbor.vertex.edge, &vf = ds->mesh.neighbor.vertex.face;
        auto count = [&](const PpfVecVecU32 &v, unsigned i) -> unsigned {
            return (v.offset && i < v.size) ? v.offset[i + 1] - v.offset[i] : 0u;
        };
        for (unsigned i = 0; i < n_surf_; ++i) {
            if (count(ve, i) != 2 || count(vf, i) != 0) continue;
            const unsigned e0 = ve.data[ve.offset[i]], e1 = ve.data[ve.offset[i] + 1];
            const unsigned st[3] = {E[2 * e0] == i ? E[2 * e0 + 1] : E[2 * e0], i,
                                    E[2 * e1] == i ? E[2 * e1 + 1] : E[2 * e1]};
            for (int a = 0; a < 3; ++a)
                for (int b = 0; b < 3; ++b) {
                    const unsigned sl = slot_of(st[a], st[b]);
                    if (st[a] <= st[b] && sl == kSentinel)
                        throw FatalError(4, "fixed pattern lacks a rod-bend block");
                    bs[9 * (size_t)i + 3 * a + b] = sl;
                }
        }
    }
    upload(edge_slot_, es);
    upload(bend_slot_, bs);
    // tets: topology, props, params, inverse rest matrices, 16 slots each
    {
        const unsigned *T = (const unsigned *)ds->mesh.mesh.tet.data;
        upload(tet_, T, 4 * (size_t)nt_);
        upload(tprop_, ds->prop.tet.data, nt_);
        upload(tparam_, ds->param_arrays.tet.data, ds->param_arrays.tet.size);
        upload(inv_rest3_, (const float *)ds->inv_rest3x3.data, 9 * (size_t)nt_);
        std::vector<unsigned> ts(16 * (size_t)nt_);
        for (unsigned t = 0; t < nt_; ++t)
            for (int a = 0; a < 4; ++a)
                for (int b = 0; b < 4; ++b) {
                    const unsigned sl = slot_of(T[4 * t + a], T[4 * t + b]);
                    if (T[4 * t + a] <= T[4 * t + b] && sl == kSentinel)
                        throw FatalError(4, "fixed pattern lacks a tet block");
                    ts[16 * t + 4 * a + b] = sl;
                }
        upload(tet_slot_, ts);
        // stitches: 36 slots each over the six indices (builder.rs:1314-1320);
        // update_constraint may change their weights and stiffness, not
        // their vertices
        nstitch_ = ds->constraint.stitch.size;
        std::vector<unsigned> ss(36 * (size_t)nstitch_);
        for (unsigned k = 0; k < nstitch_; ++k) {
            const unsigned *I = ds->constraint.stitch.data[k].index.v;
            for (int a = 0; a < 6; ++a)
                for (int b = 0; b < 6; ++b) {
                    const unsigned sl = slot_of(I[a], I[b]);
                    if (I[a] <= I[b] && sl == kSentinel)
                        throw FatalError(4, "fixed pattern lacks a stitch block");
                    ss[36 * k + 6 * a + b] = sl;
                }
        }
        upload(stitch_slot_, ss);
        std::vector<unsigned char> ht(nh_, 0);
        const PpfVecChar &hty = ds->mesh.type.hinge;
        for (unsigned h = 0; h < nh_ && hty.data && h < hty.size; ++h)
            ht[h] = (unsigned char)hty.data[h];
        upload(hinge_type_, ht);
    }
    // per-primitive margins 0.5 ghat + offset
    std::vector<float> mf(nf_), me(ne_), mv(n_);
    for (unsigned i = 0; i < nf_; ++i) {
        const PpfFaceParam &p = ds->param_arrays.face.data[h_fprop_[i].param_index];
        mf[i] = 0.5f * p.ghat + p.offset;
    }
    for (unsigned i = 0; i < ne_; ++i) {
        const PpfEdgeParam &p = ds->param_arrays.edge.data[h_eprop_[i].param_index];
        me[i] = 0.5f * p.ghat + p.offset;
    }
    for (unsigned i = 0; i < n_; ++i) {
        const PpfVertexParam &p = ds->param_arrays.vertex.data[h_vprop_[i].param_index];
        mv[i] = 0.5f * p.ghat + p.offset;
    }
    upload(margin_face_, mf);
    upload(margin_edge_, me);
    upload(margin_vert_, mv);
    // edge queries split into pieces of about twice the median rest length
    {
        std::vector<float> len(ne_);
        const float *x = (const float *)ds->vertex.curr.data;
        const unsigned *E = (const unsigned *)ds->mesh.mesh.edge.data;
        for (unsigned i = 0; i < ne_; ++i) {
            float d0 = x[3 * E[2 * i]] - x[3 * E[2 * i + 1]];
            float d1 = x[3 * E[2 * i] + 1] - x[3 * E[2 * i + 1] + 1];
            float d2 = x[3 * E[2 * i] + 2] - x[3 * E[2 * i + 1] + 2];
            len[i] = std::sqrt(d0 * d0 + d1 * d1 + d2 * d2);
        }
        piece_len_ = 0.0f;
        if (ne_) {
            std::nth_element(len.begin(), len.begin() + ne_ / 2, len.end());
            piece_len_ = 2.0f * len[ne_ / 2];
        }
        piece_cnt_.reserve(ne_ + 1);
        piece_off_.reserve(ne_ + 1);
        piece_tmp_.reserve(scan_tmp_size(ne_ + 1));
    }
    // constraints
    update_constraint(&ds->constraint);
    // state
    upload(curr_, (const float *)ds->vertex.curr.data, 3 * (size_t)n_);
    upload(prev_, (const float *)ds->vertex.prev.data, 3 * (size_t)n_);
    const size_t n3 = 3 * (size_t)n_;
    eval_x_.reserve(n3);
    target_.reserve(n3);
    force_.reserve(n3);
    dx_.reserve(n3);
    r_.reserve(n3);
    diag_.reserve(9 * (size_t)n_);
    inv_diag_.reserve(9 * (size_t)fixed_sell_.n_slices * kSliceRows);
    fixed_val_.reserve(9 * (size_t)nnz_fixed_);
    fixed_tmp_.reserve(9 * (size_t)nnz_fixed_);
    st_.reserve(1);
    sp_dev_.reserve(1);
    isect_.reserve(PPF_MAX_INTERSECTION_RECORDS);
    if (!st_host_) PPF_CUDA(cudaMallocHost(&st_host_, sizeof(IterStatus)));
    // pair lists and contact-block buffers start at a size proportional to the
    // mesh and grow on demand
    unsigned cap0 = std::max(1u << 14, 2 * std::max(n_, ne_));
    pf_buf_.reserve(cap0);
    pe_buf_.reserve(cap0);
    pp_buf_.reserve(cap0);
    ee_buf_.reserve(cap0);
    pairs_.pf = pf_buf_.data();
    pairs_.pe = pe_buf_.data();
    pairs_.pp = pp_buf_.data();
    pairs_.ee = ee_buf_.data();
    pairs_.cap_pf = pairs_.cap_pe = pairs_.cap_pp = pairs_.cap_ee = cap0;
    doff_buf_.reserve(n_ + 1);
    dtroff_buf_.reserve(n_ + 1);
    dcnt_buf_.reserve(n_ + 1);
    dcnt2_buf_.reserve(n_ + 1);
    scan_tmp_.reserve(scan_tmp_size(n_ + 1));
    pcg_.reserve(n_);
    if (pcg_team_auto_) tune_.pcg_cluster = auto_pcg_team();
    pcg_.cluster = tune_.pcg_cluster;
    if (cta_auto_) pcg_.cluster_threads = auto_cta_threads();
    upload_collision_mesh(ds->constraint.mesh);
    initialized_ = true;
    carried_ = false;
    ++scene_version_;
    // initial trees and intersection check on prev and curr (main.cu:196-262)
    if (!param->disable_contact) {
        build_trees(curr_.data(), curr_.data(), 1.0f, true);
        bool ok = check_intersection(prev_.data());
        build_trees(curr_.data(), curr_.data(), 1.0f, false);
        ok = ok && check_intersection(curr_.data());
        if (!ok) {
            set_fatal(1, "the scene is already self-intersecting at t=0; the solver "
                         "advances from a separated configuration and cannot untangle one");
            return false;
        }
    }
    return true;
}

void Solver::update_constraint(const PpfConstraint *c) {
    ++scene_version_;
    nfix_ = c->fix.size;
    npull_ = c->pull.size;
    nsphere_ = c->sphere.size;
    nfloor_ = c->floor.size;
    upload(fix_, c->fix.data, nfix_);
    upload(pull_, c->pull.data, npull_);
    upload(sphere_, c->sphere.data, nsphere_);
    upload(floor_, c->floor.data, nfloor_);
    if (c->stitch.size != nstitch_ && !h_vprop_.empty())
        throw FatalError(4, "update_constraint changed the number of stitches");
    upload(stitch_, c->stitch.data, c->stitch.size);
    if (h_vprop_.empty()) return;
    // rebuild fix/pull indices and element `fixed` flags (main.cu:2012-2077).
    // The reference re-uploads every prop array on each call; when the pinned
    // and pulled vertices and their order are those of the last call, the
    // props it would upload are the ones already on the device, so only the
    // constraint arrays above are copied.
    {
        bool same = true;
        std::vector<unsigned> fix_of(n_, 0u), pull_of(n_, 0u);
        for (unsigned i = 0; i < nfix_; ++i) fix_of[c->fix.data[i].index] = i + 1;
        for (unsigned i = 0; i < npull_; ++i) pull_of[c->pull.data[i].index] = i + 1;
        for (unsigned v = 0; v < n_ && same; ++v)
            same = h_vprop_[v].fix_index == fix_of[v] && h_vprop_[v].pull_index == pull_of[v];
        if (same) return;
    }
    for (auto &v : h_vprop_) v.fix_index = v.pull_index = 0;
    for (unsigned i = 0; i < nfix_; ++i) h_vprop_[c->fix.data[i].index].fix_index = i + 1;
    for (unsigned i = 0; i < npull_; ++i) h_vprop_[c->pull.data[i].index].pull_index = i + 1;
    auto fixed = [&](unsigned v) { return h_vprop_[v].fix_index > 0; };
    const unsigned *F = (const unsigned *)host->mesh.mesh.face.data;
    for (unsigned i = 0; i < nf_; ++i)
        h_fprop_[i].fixed = fixed(F[3 * i]) && fixed(F[3 * i + 1]) && fixed(F[3 * i + 2]);
    const unsigned *E = (const unsigned *)host->mesh.mesh.edge.data;
    for (unsigned i = 0; i < ne_; ++i) h_eprop_[i].fixed = fixed(E[2 * i]) && fixed(E[2 * i + 1]);
    const unsigned *H = (const unsigned *)host->mesh.mesh.hinge.data;
    for (unsigned i = 0; i < nh_; ++i)
        h_hprop_[i].fixed = fixed(H[4 * i]) && fixed(H[4 * i + 1]) && fixed(H[4 * i + 2]) &&
                            fixed(H[4 * i + 3]);
    if (nt_) {
        const unsigned *T = (const unsigned *)host->mesh.mesh.tet.data;
        PpfTetProp *tp = host->prop.tet.data;
        for (unsigned i = 0; i < nt_; ++i)
            tp[i].fixed = fixed(T[4 * i]) && fixed(T[4 * i + 1]) && fixed(T[4 * i + 2]) &&
                          fixed(T[4 * i + 3]);
        upload(tprop_, tp, nt_);
    }
    upload_props();
    // mirror into the host DataSet props, as the reference does
    std::memcpy(host->prop.vertex.data, h_vprop_.data(), n_ * sizeof(PpfVertexProp));
    std::memcpy(host->prop.face.data, h_fprop_.data(), nf_ * sizeof(PpfFaceProp));
    std::memcpy(host->prop.edge.data, h_eprop_.data(), ne_ * sizeof(PpfEdgeProp));
    std::memcpy(host->prop.hinge.data, h_hprop_.data(), nh_ * sizeof(PpfHingeProp));
}

void Solver::update_rest_shape(const PpfRestShapeUpdate *u) {
    if (u->inv_rest2x2.size) {
        PPF_CUDA(cudaMemcpy(inv_rest_.data(), u->inv_rest2x2.data,
                            u->inv_rest2x2.size * sizeof(PpfMat2x2f), cudaMemcpyHostToDevice));
        g_h2d_bytes += u->inv_rest2x2.size * sizeof(PpfMat2x2f);
    }
    if (u->exclude_face.size) {
        for (unsigned i = 0; i < u->exclude_face.size && i < nf_; ++i)
            h_fprop_[i].rest_excluded = u->exclude_face.data[i] != 0;
        upload(fprop_, h_fprop_);
    }
    if (u->inv_rest3x3.size && nt_) {
        const size_t k = std::min<size_t>(u->inv_rest3x3.size, nt_);
        PPF_CUDA(cudaMemcpy(inv_rest3_.data(), u->inv_rest3x3.data, k * sizeof(PpfMat3x3f),
                            cudaMemcpyHostToDevice));
        g_h2d_bytes += k * sizeof(PpfMat3x3f);
    }
    if (u->exclude_tet.size && nt_) {
        PpfTetProp *tp = host->prop.tet.data;
        for (unsigned i = 0; i < u->exclude_tet.size && i < nt_; ++i)
            tp[i].rest_excluded = u->exclude_tet.data[i] != 0;
        upload(tprop_, tp, nt_);
    }
}

void Solver::build_trees(const float *x0, const float *x1, float extrap, bool rebuild) {
    PrimSet pf{PRIM_FACE, nf_, face_.data(), margin_face_.data(),
               use_active_ ? face_active_.data() : nullptr};
    PrimSet pe{PRIM_EDGE, ne_, edge_.data(), margin_edge_.data(),
               use_active_ ? edge_active_.data() : nullptr};
    PrimSet pv{PRIM_VERTEX, n_surf_, nullptr, margin_vert_.data(),
               use_active_ ? vert_active_.data() : nullptr};
    unsigned *status = &st_.data()->status;
    if (rebuild) {
        lbvh_build(bvh_face_, pf, x1, x0, x1, extrap, sort_ws_, status, q_, false);
        lbvh_build(bvh_edge_, pe, x1, x0, x1, extrap, sort_ws_, status, q_, false);
        lbvh_build(bvh_vert_, pv, x1, x0, x1, extrap, sort_ws_, status, q_, false);
    }
    // the three trees' boxes and climbs in one launch
    Lbvh *trees[3] = {&bvh_face_, &bvh_edge_, &bvh_vert_};
    const PrimSet sets[3] = {pf, pe, pv};
    lbvh_refit_many(trees, sets, 3, x0, x1, extrap, status, q_);
}

void Solver::compute_target(float dt) {
    k_compute_target<<<div_up(n_, kB), kB, 0, q_>>>(
        n_, curr_.data(), prev_.data(), vprop_.data(), fix_.data(), target_.data(), dt,
        param->prev_dt, param->gravity.v[0], param->gravity.v[1], param->gravity.v[2],
        param->inactive_momentum ? 1 : 0);
    PPF_LAUNCH_CHECK();
}

bool Solver::check_intersection(const float *x) {
    PPF_CUDA(cudaMemsetAsync(&st_.data()->n_isect, 0, sizeof(unsigned), q_));
    PieceBuffers pb = pieces();
    launch_intersection_check(scene(), view(bvh_face_), view(bvh_edge_), x, isect_.data(),
                              st_.data(), piece_len_, pb, q_);
    unsigned cnt = 0;
    PPF_CUDA(cudaMemcpyAsync(&cnt, &st_.data()->n_isect, sizeof(unsigned),
                             cudaMemcpyDeviceToHost, q_));
    wait();
    isect_count_ = std::min(cnt, (unsigned)PPF_MAX_INTERSECTION_RECORDS);
    isect_host_.resize(isect_count_);
    if (isect_count_)
        PPF_CUDA(cudaMemcpy(isect_host_.data(), isect_.data(),
                            isect_count_ * sizeof(PpfIntersectionRecord), cudaMemcpyDeviceToHost));
    g_d2h_bytes += sizeof(unsigned) + isect_count_ * sizeof(PpfIntersectionRecord);
    return cnt == 0;
}

unsigned Solver::fetch_intersection_records(PpfIntersectionRecord *out, unsigned max_count) {
    unsigned c = std::min(isect_count_, max_count);
    if (c) std::memcpy(out, isect_host_.data(), c * sizeof(PpfIntersectionRecord));
    return c;
}

// Waits for the solver's stream: spinning (the default, lowest latency), or
// with blocking_sync_ by an event the thread sleeps on, so that more host
// threads than cores can each wait on their own scene.
void Solver::wait() {
    if (blocking_sync_) {
        if (!ev_done_)
            PPF_CUDA(cudaEventCreateWithFlags(&ev_done_,
                                              cudaEventBlockingSync | cudaEventDisableTiming));
        PPF_CUDA(cudaEventRecord(ev_done_, q_));
        PPF_CUDA(cudaEventSynchronize(ev_done_));
    } else {
        PPF_CUDA(cudaStreamSynchronize(q_));
    }
}

void Solver::read_status() {
    PPF_CUDA(cudaMemcpyAsync(st_host_, st_.data(), sizeof(IterStatus), cudaMemcpyDeviceToHost, q_));
    wait();
    g_d2h_bytes += sizeof(IterStatus);
}

__global__ void k_set_step_params(StepParams p, StepParams *dst) { *dst = p; }

// The step's parameters to their device copy, by a kernel argument: the
// assembly kernels read them there, so a captured iteration serves every
// step (their time step and clock change per step).
void Solver::upload_step_params(float dt) {
    sp_dev_.reserve(1);
    k_set_step_params<<<1, 1, 0, q_>>>(step_params(dt), sp_dev_.data());
    PPF_LAUNCH_CHECK();
}

void Solver::grow_pairs(const unsigned counts[4]) {
    auto grow_to = [](unsigned c) { return std::max(1u << 14, (unsigned)(2ull * c)); };
    if (counts[0] > pairs_.cap_pf) pf_buf_.reserve(grow_to(counts[0]));
    if (counts[1] > pairs_.cap_pe) pe_buf_.reserve(grow_to(counts[1]));
    if (counts[2] > pairs_.cap_pp) pp_buf_.reserve(grow_to(counts[2]));
    if (counts[3] > pairs_.cap_ee) ee_buf_.reserve(grow_to(counts[3]));
    pairs_.pf = pf_buf_.data();
    pairs_.pe = pe_buf_.data();
    pairs_.pp = pp_buf_.data();
    pairs_.ee = ee_buf_.data();
    pairs_.cap_pf = (unsigned)pf_buf_.cap;
    pairs_.cap_pe = (unsigned)pe_buf_.cap;
    pairs_.cap_pp = (unsigned)pp_buf_.cap;
    pairs_.cap_ee = (unsigned)ee_buf_.cap;
}

// Assembly of the Newton system at eval_x (main.cu:713-1049).
void Solver::assemble(float dt) {
    upload_step_params(dt);
    assemble_stage(false);
}

// The assembly launches. With `capacity` false the pair counts and the
// contact layout's totals are read back to size the launches and buffers
// (two synchronizations); with it true everything is sized by capacities
// (the pair lists' and dyn_cap_ contact blocks), no value is read back, and
// an iteration whose counts overran them is flagged (STATUS_PAIR_OVERFLOW)
// for the host to grow them and repeat it.
void Solver::assemble_stage(bool capacity) {
    const Scene s = scene();
    const size_t n3 = 3 * (size_t)n_;
    PPF_CUDA(cudaMemsetAsync(force_.data(), 0, n3 * sizeof(float), q_));
    PPF_CUDA(cudaMemsetAsync(diag_.data(), 0, 9 * (size_t)n_ * sizeof(float), q_));
    PPF_CUDA(cudaMemsetAsync(fixed_val_.data(), 0, 9 * (size_t)nnz_fixed_ * sizeof(float), q_));
    PPF_CUDA(cudaMemsetAsync(dx_.data(), 0, n3 * sizeof(float), q_));
    k_seed_dx<<<div_up(n_, kB), kB, 0, q_>>>(n_, vprop_.data(), eval_x_.data(), target_.data(),
                                            dx_.data());
    PPF_LAUNCH_CHECK();
    AssemblyBuffers b = abuf();
    launch_vertex_energy(s, b, q_);
    launch_elastic(s, b, q_);
    PPF_CUDA(cudaMemcpyAsync(fixed_tmp_.data(), fixed_val_.data(),
                             9 * (size_t)nnz_fixed_ * sizeof(float), cudaMemcpyDeviceToDevice, q_));
    launch_strain_limit(s, b, q_);
    unsigned bound[4] = {0, 0, 0, 0};
    if (!param->disable_contact) {
        // tight boxes at the evaluated positions for the proximity queries
        build_trees(eval_x_.data(), eval_x_.data(), 1.0f, false);
        if (capacity) {
            PPF_CUDA(cudaMemsetAsync(st_.data(), 0, 4 * sizeof(unsigned), q_));
            PieceBuffers pb = pieces();
            launch_edge_pieces(s, view(bvh_edge_), eval_x_.data(), nullptr, nullptr, piece_len_,
                               pb, q_);
            launch_detect(s, view(bvh_face_), view(bvh_edge_), view(bvh_vert_), b, pairs_, pb, q_);
            launch_pair_capacity(pairs_, st_.data(), q_);
            bound[0] = pairs_.cap_pf;
            bound[1] = pairs_.cap_pe;
            bound[2] = pairs_.cap_pp;
            bound[3] = pairs_.cap_ee;
        } else {
            for (int attempt = 0; attempt < 3; ++attempt) {
                PPF_CUDA(cudaMemsetAsync(st_.data(), 0, 4 * sizeof(unsigned), q_));
                PieceBuffers pb = pieces();
                launch_edge_pieces(s, view(bvh_edge_), eval_x_.data(), nullptr, nullptr,
                                   piece_len_, pb, q_);
                launch_detect(s, view(bvh_face_), view(bvh_edge_), view(bvh_vert_), b, pairs_, pb,
                              q_);
                read_status();
                bound[0] = st_host_->n_pf;
                bound[1] = st_host_->n_pe;
                bound[2] = st_host_->n_pp;
                bound[3] = st_host_->n_ee;
                bool grow = bound[0] > pairs_.cap_pf || bound[1] > pairs_.cap_pe ||
                            bound[2] > pairs_.cap_pp || bound[3] > pairs_.cap_ee;
                if (!grow) break;
                grow_pairs(bound);
                PPF_CUDA(cudaMemsetAsync(&st_.data()->n_contact, 0, sizeof(unsigned), q_));
            }
            if (bound[0] > pairs_.cap_pf || bound[1] > pairs_.cap_pe ||
                bound[2] > pairs_.cap_pp || bound[3] > pairs_.cap_ee)
                throw FatalError(4, "contact pair lists still overflow after growing them");
        }
    }
    // contact blocks outside the fixed pattern: at most 6, 3, 1, 6 per pair
    // (upper triangle); the hash table is kept at most half full
    unsigned hcap, dcap;
    if (capacity) {
        dcap = dyn_cap_;
        hcap = next_pow2(4ull * dcap);
    } else {
        unsigned long long keys =
            6ull * bound[0] + 3ull * bound[1] + bound[2] + 6ull * bound[3];
        hcap = next_pow2(2 * keys + 16);
        dcap = (unsigned)std::max<unsigned long long>(keys, 16ull);
    }
    hkey_buf_.reserve(hcap);
    hval_buf_.reserve(hcap);
    dcol_buf_.reserve(dcap);
    dtr_buf_.reserve(dcap);
    dval_buf_.reserve(9 * (size_t)dcap);
    dyn_.hkey = hkey_buf_.data();
    dyn_.hval = hval_buf_.data();
    dyn_.hcap = hcap;
    dyn_.off = doff_buf_.data();
    dyn_.col = dcol_buf_.data();
    dyn_.val = dval_buf_.data();
    dyn_.tr_off = dtroff_buf_.data();
    dyn_.tr = dtr_buf_.data();
    dyn_.cnt = dcnt_buf_.data();
    dyn_.cnt2 = dcnt2_buf_.data();
    dyn_.cap = dcap;
    PPF_CUDA(cudaMemsetAsync(&st_.data()->n_dyn, 0, sizeof(unsigned), q_));
    launch_dyn_build(s, b, pairs_, bound, dyn_, scan_tmp_.data(), q_);
    carried_ = false;
    launch_contact_assemble(s, b, pairs_, bound, dyn_, q_);
    launch_vertex_constraints(s, b, q_);
    if (!param->disable_contact) launch_collision_mesh(s, b, view(bvh_face_), q_);
    launch_dirichlet(s, b, dyn_, dx_.data(), q_);
    k_fold_diag<<<div_up(n_, kB), kB, 0, q_>>>(n_, fixed_diag_.data(), diag_.data(),
                                              fixed_val_.data());
    PPF_LAUNCH_CHECK();
    // the operator in the PCG's slice layout, and its block-Jacobi inverse
    sell_pack_fixed(fixed_sell_, fixed_val_.data(), q_);
    sell_build_dyn(n_, dyn_.off, dyn_.col, dyn_.val, dyn_.tr_off, dyn_.tr, dof_mask_.data(),
                   dyn_layout_, q_, capacity ? dcap : 0u, &st_.data()->status);
    launch_block_jacobi(n_, fixed_val_.data(), fixed_diag_.data(), inv_diag_.data(),
                        &st_.data()->status, q_);
    // the factored preconditioner once a block-Jacobi solve has set the
    // iteration count it must stay within (never in a capacity-sized
    // iteration: its build reads the layout's sizes on the host)
    factor_active_ = !capacity && precond_kind_ != 0 && (plain_iters_ != 0 || force_factor_);
    if (factor_active_) build_factor();
    // the reference's aggregate Schwarz when the scene asks for it
    schwarz_active_ = precond_kind_ == 0 && param->precond == 1;
    if (schwarz_active_) {
        PcgOperator A{n_, sell_view(fixed_sell_), contact_view(dyn_layout_),
                      overflow_view(dyn_layout_), inv_diag_.data(), PcgFactor{}, SchwarzView{}};
        if (!schwarz_ready()) {
            if (capacity) throw FatalError(4, "Schwarz layout not set up before a captured iteration");
            schwarz_setup(A, schwarz_, schwarz_levels(), q_);
        }
        launch_schwarz_factor(A, schwarz_, &st_.data()->status, q_);
    }
}

// Levels as the reference reads ParamSet::schwarz_levels (0: unset, 2), built
// up to kSchwarzMaxLevels (schwarz.cu:1650-1666).
unsigned Solver::schwarz_levels() const {
    unsigned levels = param->schwarz_levels ? param->schwarz_levels : 2u;
    return std::min(levels, kSchwarzMaxLevels);
}

bool Solver::schwarz_ready() const {
    return schwarz_.ready && schwarz_.n == n_ && schwarz_.levels_req == schwarz_levels();
}

void Solver::record_event(cudaEvent_t ev, bool capturing) {
    if (capturing) PPF_CUDA(cudaEventRecordWithFlags(ev, q_, cudaEventRecordExternal));
    else PPF_CUDA(cudaEventRecord(ev, q_));
}

// The linear solve of the assembled system, bracketed by the PCG timing
// events. A factored or Schwarz solve runs first; block-Jacobi solves again
// from the same start if it stalled or reached the block-Jacobi count (a
// factored one), or if r^T z <= 0 (a Schwarz one, solver/solver.cu:1627-1676),
// decided on the device.
void Solver::enqueue_solve(bool capturing) {
    const size_t n3 = 3 * (size_t)n_;
    PPF_CUDA(cudaMemcpyAsync(r_.data(), force_.data(), n3 * sizeof(float),
                             cudaMemcpyDeviceToDevice, q_));
    PcgOperator A = pcg_operator();
    pcg_.cluster = tune_.pcg_cluster;
    record_event(ev0_, capturing);
    if (factor_active_ || schwarz_active_) {
        dx0_.reserve(n3);
        run_plain_.reserve(1);
        PPF_CUDA(cudaMemcpyAsync(dx0_.data(), dx_.data(), n3 * sizeof(float),
                                 cudaMemcpyDeviceToDevice, q_));
        launch_pcg(A, dx_.data(), r_.data(), param->cg_tol,
                   factor_active_ ? std::min(plain_iters_, param->cg_max_iter)
                                  : param->cg_max_iter,
                   pcg_, q_);
        k_factor_verdict<<<div_up(n3, (size_t)kB), kB, 0, q_>>>(
            (unsigned)n3, pcg_.result.data(), factor_active_ ? 1 : 0, force_.data(),
            dx0_.data(), r_.data(), dx_.data(), run_plain_.data(), st_.data());
        PPF_LAUNCH_CHECK();
        A.schwarz = SchwarzView{};
        PcgOperator J = A;
        J.factor = PcgFactor{};
        launch_pcg(J, dx_.data(), r_.data(), param->cg_tol, param->cg_max_iter, pcg_, q_,
                   run_plain_.data());
    } else {
        launch_pcg(A, dx_.data(), r_.data(), param->cg_tol, param->cg_max_iter, pcg_, q_);
    }
    record_event(ev1_, capturing);
}

// Everything a captured iteration bakes in: the scene's arrays and counts,
// the parameters (but the per-step clock), the pair lists, the contact-block
// capacity, the fixed operator's and the Schwarz layout's sizes, and the
// buffer epoch (every device pointer). A constraint update that rewrites the
// device arrays in place leaves it as it is.
Solver::IterKey Solver::iteration_key() const {
    IterKey k;
    memset(&k, 0, sizeof(k));
    const Scene sc = scene();
    memcpy(&k.scene, &sc, sizeof(Scene));
    memcpy(&k.param, param, sizeof(PpfParamSet));
    k.param.time = 0.0;
    k.param.prev_dt = 0.0f;
    memcpy(&k.pairs, &pairs_, sizeof(PairLists));
    k.piece_len = piece_len_;
    k.dyn_cap = dyn_cap_;
    k.use_active = use_active_ ? 1u : 0u;
    k.schwarz = schwarz_ready() ? 1u : 0u;
    k.nnz_fixed = nnz_fixed_;
    k.fixed_slices = fixed_sell_.n_slices;
    k.fixed_slots = fixed_sell_.slots;
    if (k.schwarz) {
        k.agg[0] = schwarz_.n;
        k.agg[1] = schwarz_.n_agg;
        k.agg[2] = schwarz_.max_members;
        k.agg[3] = schwarz_.levels;
        k.agg[4] = schwarz_.n_dom;
        k.agg[5] = schwarz_.max_dom_members;
    }
    k.epoch = g_buffer_epoch;
    return k;
}

// A Newton iteration can be captured when its assembly needs no read-back:
// block-Jacobi, or Schwarz once its layout is set up.
bool Solver::iteration_graph_ok() const {
    if (!graph_enabled_ || precond_kind_ != 0) return false;
    return param->precond != 1 || schwarz_ready();
}

// The iteration's launches, sized by capacities, in stream order: status
// reset, assembly, solve, line search, status copy to the host.
void Solver::enqueue_iteration(bool capturing) {
    PPF_CUDA(cudaMemsetAsync(st_.data(), 0, sizeof(IterStatus), q_));
    assemble_stage(true);
    enqueue_solve(capturing);
    enqueue_line_search();
}

// One Newton iteration through its CUDA graph. The first iteration under a
// new key runs its launches directly (sizing every buffer for the current
// capacities), the next one captures them, and later ones replay the graph.
void Solver::iteration_graph(float dt) {
    upload_step_params(dt);
    IterKey key = iteration_key();
    if (it_graph_ && memcmp(&key, &it_key_, sizeof(IterKey)) == 0) {
        PPF_CUDA(cudaGraphLaunch(it_graph_, q_));
        count_launches(it_launches_);
        ++graph_stats_.replays;
        return;
    }
    if (it_graph_) {
        PPF_CUDA(cudaGraphExecDestroy(it_graph_));
        it_graph_ = nullptr;
    }
    if (!it_eager_valid_ || memcmp(&key, &it_eager_key_, sizeof(IterKey)) != 0) {
        enqueue_iteration(false);
        it_eager_key_ = iteration_key();
        it_eager_valid_ = true;
        ++graph_stats_.direct;
        return;
    }
    cudaGraph_t graph = nullptr;
    const unsigned long long l0 = t_kernel_launches;
    PPF_CUDA(cudaStreamBeginCapture(q_, cudaStreamCaptureModeThreadLocal));
    g_capturing = true;
    try {
        enqueue_iteration(true);
    } catch (...) {
        g_capturing = false;
        cudaGraph_t aborted = nullptr;
        cudaStreamEndCapture(q_, &aborted);
        if (aborted) cudaGraphDestroy(aborted);
        throw;
    }
    g_capturing = false;
    PPF_CUDA(cudaStreamEndCapture(q_, &graph));
    it_launches_ = (unsigned)(t_kernel_launches - l0);
    uncount_launches(it_launches_);
    PPF_CUDA(cudaGraphInstantiate(&it_graph_, graph, 0ull));
    PPF_CUDA(cudaGraphDestroy(graph));
    it_key_ = key;
    ++graph_stats_.captures;
    PPF_CUDA(cudaGraphLaunch(it_graph_, q_));
    count_launches(it_launches_);
    ++graph_stats_.replays;
}

// The line-search stage of a Newton iteration (main.cu:1142-1354): the
// rescaled step, the swept-box refits, contact (or analytic-collider) and
// strain-limit line searches, and the status block's copy to pinned host
// memory. Its launches depend only on the scene's buffers and constants, so
// the sequence is captured once as a CUDA graph and replayed every
// iteration; the capture is redone when the scene changes (scene_version_).
void Solver::enqueue_line_search() {
    const Scene s = scene();
    const float max_t = param->line_search_max_t;
    k_max_dx<<<div_up(n_, kB), kB, 0, q_>>>(n_, dx_.data(), st_.data());
    PPF_LAUNCH_CHECK();
    k_apply_dx<<<div_up(n_, kB), kB, 0, q_>>>(n_, eval_x_.data(), target_.data(), dx_.data(),
                                               st_.data(), param->max_dx);
    PPF_LAUNCH_CHECK();
    k_init_ls<<<1, 1, 0, q_>>>(st_.data(), max_t, pcg_.result.data());
    PPF_LAUNCH_CHECK();
    LineSearchArgs la{target_.data(), eval_x_.data(), curr_.data(), st_.data(), max_t,
                      param->ccd_eps};
    if (!param->disable_contact) {
        build_trees(target_.data(), eval_x_.data(), max_t, false);
        PieceBuffers pb = pieces();
        launch_contact_line_search(s, view(bvh_face_), view(bvh_edge_), view(bvh_vert_), la,
                                   piece_len_, pb, q_);
    } else {
        launch_constraint_line_search(s, la, q_);
    }
    launch_strain_line_search(s, la, q_);
    PPF_CUDA(cudaMemcpyAsync(st_host_, st_.data(), sizeof(IterStatus), cudaMemcpyDeviceToHost,
                             q_));
}

void Solver::line_search_stage() {
    const unsigned long long key = scene_version_ * 4ull + (param->disable_contact ? 1u : 0u) +
                                   (use_active_ ? 2u : 0u);
    if (!ls_graph_ || ls_key_ != key || ls_max_t_ != param->line_search_max_t ||
        ls_max_dx_ != param->max_dx || ls_ccd_eps_ != param->ccd_eps) {
        if (ls_graph_) {
            PPF_CUDA(cudaGraphExecDestroy(ls_graph_));
            ls_graph_ = nullptr;
        }
        cudaGraph_t graph = nullptr;
        const unsigned long long l0 = t_kernel_launches;
        PPF_CUDA(cudaStreamBeginCapture(q_, cudaStreamCaptureModeThreadLocal));
        try {
            enqueue_line_search();
        } catch (...) {
            cudaGraph_t aborted = nullptr;
            cudaStreamEndCapture(q_, &aborted);
            if (aborted) cudaGraphDestroy(aborted);
            throw;
        }
        PPF_CUDA(cudaStreamEndCapture(q_, &graph));
        ls_launches_ = (unsigned)(t_kernel_launches - l0);
        uncount_launches(ls_launches_);
        PPF_CUDA(cudaGraphInstantiate(&ls_graph_, graph, 0ull));
        PPF_CUDA(cudaGraphDestroy(graph));
        ls_key_ = key;
        ls_max_t_ = param->line_search_max_t;
        ls_max_dx_ = param->max_dx;
        ls_ccd_eps_ = param->ccd_eps;
    }
    PPF_CUDA(cudaGraphLaunch(ls_graph_, q_));
    count_launches(ls_launches_);
    ++ls_replays_;
}

PpfStepResult Solver::advance() {
    PpfStepResult result{};
    result.ccd_success = result.pcg_success = result.intersection_free = true;
    result.newton_progress = result.pin_feasible = result.contact_separated = true;
    auto t_start = std::chrono::steady_clock::now();
    stats_ = StepStats{};
    const size_t n3 = 3 * (size_t)n_;
    float dt = param->dt * param->playback;
    const float max_t = param->line_search_max_t;
    PPF_CUDA(cudaMemsetAsync(st_.data(), 0, sizeof(IterStatus), q_));
    if (!param->disable_contact) build_trees(curr_.data(), curr_.data(), 1.0f, true);
    compute_target(dt);
    PPF_CUDA(cudaMemcpyAsync(eval_x_.data(), curr_.data(), n3 * sizeof(float),
                             cudaMemcpyDeviceToDevice, q_));
    double toi_advanced = 0.0;
    unsigned step = 1;
    bool final_step = false;
    bool repeat = false;   // the last iteration overran a capacity: run it again
    unsigned repeats = 0;
    while (true) {
        if (!repeat) {
            if (!final_step && param->max_newton_steps > 0 &&
                step >= param->max_newton_steps) {
                result.newton_progress = false;
                return result;
            }
            if (final_step) {
                if (toi_advanced < 1.0 && nfix_) {
                    k_rewind_fix<<<div_up(nfix_, kB), kB, 0, q_>>>(nfix_, fix_.data(),
                                                                   1.0f - (float)toi_advanced);
                    PPF_LAUNCH_CHECK();
                }
                dt *= (float)toi_advanced;
                compute_target(dt);
            }
        }
        repeat = false;
        const bool graphed = iteration_graph_ok();
        if (graphed) {
            // assembly, solve and line search as one CUDA graph, sized by
            // capacities, with no read-back before the status copy
            iteration_graph(dt);
        } else {
            PPF_CUDA(cudaMemsetAsync(st_.data(), 0, sizeof(IterStatus), q_));
            assemble(dt);
            enqueue_solve(false);
            // rescaled Newton step, swept boxes, line search, status to the
            // host: a fixed sequence of launches over this scene's buffers,
            // replayed as one CUDA graph
            line_search_stage();
        }
        wait();
        g_d2h_bytes += sizeof(IterStatus);
        const float rescale = st_host_->rescale;
        const IterStatus st = *st_host_;
        if (st.status & STATUS_PAIR_OVERFLOW) {
            // a capacity-sized iteration found more pairs or contact blocks
            // than it could hold; it changed nothing, so grow and repeat it
            if (!graphed || ++repeats > 8)
                throw FatalError(4, "contact capacities still overflow after growing them");
            const unsigned counts[4] = {st.n_pf, st.n_pe, st.n_pp, st.n_ee};
            const bool lists = st.n_pf > pairs_.cap_pf || st.n_pe > pairs_.cap_pe ||
                               st.n_pp > pairs_.cap_pp || st.n_ee > pairs_.cap_ee;
            if (lists) {
                // the blocks were not counted: grow the lists first
                grow_pairs(counts);
            } else {
                dyn_cap_ = (unsigned)std::min<unsigned long long>(
                    2ull * std::max(st.n_dyn, dyn_cap_), 0x3FFFFFFFull);
            }
            ++graph_stats_.repeats;
            repeat = true;
            continue;
        }
        float pcg_ms = 0.0f;
        PPF_CUDA(cudaEventElapsedTime(&pcg_ms, ev0_, ev1_));
        stats_.newton_iters++;
        stats_.pcg_solves++;
        unsigned iters = st.pcg_iter;
        if (schwarz_active_) {
            if (st.fallback) {
                stats_.fallbacks++;
                iters += st.factor_iter;
            }
        } else if (factor_active_) {
            stats_.factor_iters_total += st.factor_iter;
            if (st.fallback) {
                stats_.fallbacks++;
                plain_iters_ = std::max(st.pcg_iter, 1u);
                iters += st.factor_iter;
            }
        } else if (precond_kind_ != 0) {
            plain_iters_ = std::max(st.pcg_iter, 1u);
        }
        stats_.pcg_iters_total += iters;
        stats_.last_state = st.pcg_state;
        stats_.last_break_cause = st.pcg_break_cause;
        stats_.last_resid = st.pcg_resid;
        stats_.last_break_val = st.pcg_break_val;
        stats_.pcg_ms_total += pcg_ms;
        stats_.pcg_ms.push_back(pcg_ms);
        stats_.pcg_iters.push_back(iters);
        stats_.dyn_blocks.push_back(st.n_dyn);
        stats_.max_contacts = std::max(stats_.max_contacts, st.n_contact);
        stats_.max_dyn_blocks = std::max(stats_.max_dyn_blocks, st.n_dyn);
        if (st.status & (STATUS_BVH_STACK_OVERFLOW | STATUS_BLOCK_OVERFLOW | STATUS_BAD_SLOT |
                         STATUS_SORT_LOOKBACK_TIMEOUT | STATUS_REFIT_CYCLE)) {
            char buf[160];
            snprintf(buf, sizeof(buf), "device status 0x%x during the Newton step", st.status);
            throw FatalError(4, buf);
        }
        if (st.pcg_state == 2) {
            result.pcg_success = false;
            return result;
        }
        if (st.pin_infeasible != 0xFFFFFFFFu) {
            result.pin_feasible = false;
            return result;
        }
        if (st.overlap) {
            result.contact_separated = false;
            return result;
        }
        float toi = std::min(1.0f, bits_to_float(st.toi_bits) / max_t);
        float sl_toi = bits_to_float(st.sl_toi_bits) / max_t;
        toi = std::min(toi, sl_toi);
        stats_.toi.push_back(toi);
        if (toi <= 1.19209290e-7f) {
            result.ccd_success = false;
            return result;
        }
        if (!final_step)
            toi_advanced += std::max(0.0, 1.0 - toi_advanced) * (double)(rescale * toi);
        k_apply_toi<<<div_up(n_, kB), kB, 0, q_>>>(n_, eval_x_.data(), target_.data(), toi);
        PPF_LAUNCH_CHECK();
        if (final_step) break;
        if (toi_advanced >= param->target_toi && step >= param->min_newton_steps) {
            final_step = true;
        } else {
            ++step;
            compute_target(dt);
        }
    }
    if (!param->disable_contact) {
        build_trees(eval_x_.data(), eval_x_.data(), 1.0f, false);
        if (!check_intersection(eval_x_.data())) result.intersection_free = false;
    }
    param->prev_dt = dt;
    param->time += (double)(param->prev_dt / param->playback);
    PPF_CUDA(cudaMemcpyAsync(prev_.data(), curr_.data(), n3 * sizeof(float),
                             cudaMemcpyDeviceToDevice, q_));
    PPF_CUDA(cudaMemcpyAsync(curr_.data(), eval_x_.data(), n3 * sizeof(float),
                             cudaMemcpyDeviceToDevice, q_));
    wait();
    result.time = param->time;
    stats_.step_ms = std::chrono::duration<float, std::milli>(std::chrono::steady_clock::now() -
                                                              t_start)
                         .count();
    return result;
}

void Solver::fetch() {
    PPF_CUDA(cudaStreamSynchronize(q_));
    PPF_CUDA(cudaMemcpy(host->vertex.curr.data, curr_.data(), 3 * (size_t)n_ * sizeof(float),
                        cudaMemcpyDeviceToHost));
    PPF_CUDA(cudaMemcpy(host->vertex.prev.data, prev_.data(), 3 * (size_t)n_ * sizeof(float),
                        cudaMemcpyDeviceToHost));
    g_d2h_bytes += 2 * 3 * (size_t)n_ * sizeof(float);
}

void Solver::fetch_dyn_counts(unsigned *n_value, unsigned *n_offset) {
    *n_offset = n_ + 1;
    if (carried_) {
        *n_value = carried_off_[n_];
        return;
    }
    unsigned v = 0;
    PPF_CUDA(cudaStreamSynchronize(q_));
    if (dyn_.off) PPF_CUDA(cudaMemcpy(&v, dyn_.off + n_, sizeof(unsigned), cudaMemcpyDeviceToHost));
    *n_value = v;
}

// The reference restores its carried contact pattern from a saved state
// (main.cu:1985-1987, csrmat.cu:146-153). That pattern seeds the capacity of
// the next assembly and never changes its values. Here the contact blocks are
// re-derived every Newton iteration, so the restored pattern reserves the
// contact-block buffers for its count and is what fetch_dyn reports until an
// assembly replaces it: a state saved, restored and saved again writes the
// same pattern.
void Solver::update_dyn(const unsigned *index, const unsigned *offset) {
    if (!initialized_ || !offset) return;
    carried_off_.assign(offset, offset + n_ + 1);
    for (unsigned i = 0; i < n_; ++i)
        if (carried_off_[i + 1] < carried_off_[i])
            throw FatalError(4, "update_dyn: row offsets decrease");
    const unsigned nnz = carried_off_[n_];
    carried_col_.assign(index, index + nnz);
    for (unsigned c : carried_col_)
        if (c >= n_) throw FatalError(4, "update_dyn: column index out of range");
    carried_ = true;
    const unsigned cap = std::max(nnz, 16u);
    dcol_buf_.reserve(cap);
    dtr_buf_.reserve(cap);
    dval_buf_.reserve(9 * (size_t)cap);
}

void Solver::fetch_inv_rest() {
    PPF_CUDA(cudaStreamSynchronize(q_));
    const size_t n = host->inv_rest2x2.size;
    if (n && inv_rest_.data())
        PPF_CUDA(cudaMemcpy(host->inv_rest2x2.data, inv_rest_.data(), n * sizeof(PpfMat2x2f),
                            cudaMemcpyDeviceToHost));
}

void Solver::fetch_rest_angles() {
    PPF_CUDA(cudaStreamSynchronize(q_));
    if (nh_ && host->prop.hinge.size)
        PPF_CUDA(cudaMemcpy(host->prop.hinge.data, hprop_.data(), nh_ * sizeof(PpfHingeProp),
                            cudaMemcpyDeviceToHost));
    if (n_ && host->prop.vertex.size)
        PPF_CUDA(cudaMemcpy(host->prop.vertex.data, vprop_.data(), n_ * sizeof(PpfVertexProp),
                            cudaMemcpyDeviceToHost));
}

void Solver::fetch_dyn(unsigned *index, PpfMat3x3f *value, unsigned *offset) {
    if (carried_) {
        std::memcpy(offset, carried_off_.data(), (n_ + 1) * sizeof(unsigned));
        if (!carried_col_.empty())
            std::memcpy(index, carried_col_.data(), carried_col_.size() * sizeof(unsigned));
        if (value) std::memset(value, 0, carried_col_.size() * sizeof(PpfMat3x3f));
        return;
    }
    PPF_CUDA(cudaStreamSynchronize(q_));
    std::vector<unsigned> off(n_ + 1, 0u);
    if (dyn_.off)
        PPF_CUDA(cudaMemcpy(off.data(), dyn_.off, (n_ + 1) * sizeof(unsigned), cudaMemcpyDeviceToHost));
    std::vector<unsigned> col(off[n_]);
    std::vector<float> val(9 * (size_t)off[n_]);
    if (off[n_]) {
        PPF_CUDA(cudaMemcpy(col.data(), dyn_.col, off[n_] * sizeof(unsigned), cudaMemcpyDeviceToHost));
        PPF_CUDA(cudaMemcpy(val.data(), dyn_.val, 9 * (size_t)off[n_] * sizeof(float),
                            cudaMemcpyDeviceToHost));
    }
    // rows sorted by column, as the reference's carried pattern is
    for (unsigned i = 0; i < n_; ++i) {
        std::vector<unsigned> order(off[i + 1] - off[i]);
        for (unsigned k = 0; k < order.size(); ++k) order[k] = off[i] + k;
        std::sort(order.begin(), order.end(), [&](unsigned a, unsigned b) { return col[a] < col[b]; });
        for (unsigned k = 0; k < order.size(); ++k) {
            index[off[i] + k] = col[order[k]];
            if (value) std::memcpy(value[off[i] + k].m, &val[9 * (size_t)order[k]], 9 * sizeof(float));
        }
    }
    std::memcpy(offset, off.data(), (n_ + 1) * sizeof(unsigned));
}

void Solver::override_velocity(const unsigned *idx, unsigned count, float vx, float vy,
                               float vz, float dt) {
    if (count == 0 || dt <= 0.0f) return;
    DevBuf<unsigned> d;
    upload(d, idx, count);
    k_override_velocity<<<div_up(count, kB), kB, 0, q_>>>(d.data(), count, curr_.data(),
                                                         prev_.data(), vx * dt, vy * dt, vz * dt);
    PPF_LAUNCH_CHECK();
    PPF_CUDA(cudaStreamSynchronize(q_));
    d.release();
}

void Solver::override_angular_velocity(const unsigned *idx, unsigned count, float wx, float wy,
                                       float wz, float cx, float cy, float cz, float dt) {
    if (count == 0 || dt <= 0.0f) return;
    DevBuf<unsigned> d;
    upload(d, idx, count);
    k_override_angular<<<div_up(count, kB), kB, 0, q_>>>(d.data(), count, curr_.data(),
                                                        prev_.data(), wx, wy, wz, cx, cy, cz, dt);
    PPF_LAUNCH_CHECK();
    PPF_CUDA(cudaStreamSynchronize(q_));
    d.release();
}

void Solver::gather_current_positions(const unsigned *idx, unsigned count, float *out) {
    std::vector<float> all(3 * (size_t)n_);
    PPF_CUDA(cudaStreamSynchronize(q_));
    PPF_CUDA(cudaMemcpy(all.data(), curr_.data(), all.size() * sizeof(float), cudaMemcpyDeviceToHost));
    for (unsigned i = 0; i < count; ++i)
        for (int d = 0; d < 3; ++d) out[3 * i + d] = all[3 * idx[i] + d];
}

void Solver::set_active(const std::vector<unsigned char> &va) {
    std::vector<unsigned char> fa(nf_), ea(ne_);
    const unsigned *F = (const unsigned *)host->mesh.mesh.face.data;
    const unsigned *E = (const unsigned *)host->mesh.mesh.edge.data;
    for (unsigned i = 0; i < nf_; ++i) fa[i] = va[F[3 * i]] || va[F[3 * i + 1]] || va[F[3 * i + 2]];
    for (unsigned i = 0; i < ne_; ++i) ea[i] = va[E[2 * i]] || va[E[2 * i + 1]];
    upload(vert_active_, va);
    upload(face_active_, fa);
    upload(edge_active_, ea);
    use_active_ = true;
    ++scene_version_;
}

void Solver::debug_matrix(std::vector<unsigned> &f_off, std::vector<unsigned> &f_col,
                          std::vector<float> &f_val, std::vector<unsigned> &d_off,
                          std::vector<unsigned> &d_col, std::vector<float> &d_val,
                          std::vector<float> &diag, std::vector<float> &force) {
    PPF_CUDA(cudaStreamSynchronize(q_));
    f_off.resize(n_ + 1);
    PPF_CUDA(cudaMemcpy(f_off.data(), fixed_off_.data(), (n_ + 1) * 4, cudaMemcpyDeviceToHost));
    f_col.resize(nnz_fixed_);
    PPF_CUDA(cudaMemcpy(f_col.data(), fixed_col_.data(), nnz_fixed_ * 4, cudaMemcpyDeviceToHost));
    f_val.resize(9 * (size_t)nnz_fixed_);
    PPF_CUDA(cudaMemcpy(f_val.data(), fixed_val_.data(), f_val.size() * 4, cudaMemcpyDeviceToHost));
    d_off.assign(n_ + 1, 0u);
    if (dyn_.off) PPF_CUDA(cudaMemcpy(d_off.data(), dyn_.off, (n_ + 1) * 4, cudaMemcpyDeviceToHost));
    d_col.resize(d_off[n_]);
    d_val.resize(9 * (size_t)d_off[n_]);
    if (d_off[n_]) {
        PPF_CUDA(cudaMemcpy(d_col.data(), dyn_.col, d_off[n_] * 4, cudaMemcpyDeviceToHost));
        PPF_CUDA(cudaMemcpy(d_val.data(), dyn_.val, d_val.size() * 4, cudaMemcpyDeviceToHost));
    }
    diag.resize(9 * (size_t)n_);
    PPF_CUDA(cudaMemcpy(diag.data(), diag_.data(), diag.size() * 4, cudaMemcpyDeviceToHost));
    force.resize(3 * (size_t)n_);
    PPF_CUDA(cudaMemcpy(force.data(), force_.data(), force.size() * 4, cudaMemcpyDeviceToHost));
}

void Solver::debug_vertex_info(std::vector<float> &mass, std::vector<unsigned> &dof) {
    PPF_CUDA(cudaStreamSynchronize(q_));
    mass.resize(n_);
    dof.resize(n_);
    PPF_CUDA(cudaMemcpy(mass.data(), mass_.data(), n_ * sizeof(float), cudaMemcpyDeviceToHost));
    PPF_CUDA(cudaMemcpy(dof.data(), dof_mask_.data(), n_ * sizeof(unsigned),
                        cudaMemcpyDeviceToHost));
}

void Solver::debug_factor_diag(std::vector<float> &diag) {
    PPF_CUDA(cudaStreamSynchronize(q_));
    diag.assign(9 * (size_t)n_, 0.0f);
    if (factor_.diag.cap >= diag.size())
        PPF_CUDA(cudaMemcpy(diag.data(), factor_.diag.data(), diag.size() * sizeof(float),
                            cudaMemcpyDeviceToHost));
}

void Solver::debug_pairs(std::vector<unsigned> &pf, std::vector<unsigned> &pe,
                         std::vector<unsigned> &pp, std::vector<unsigned> &ee) {
    read_status();
    unsigned c[4] = {std::min(st_host_->n_pf, pairs_.cap_pf), std::min(st_host_->n_pe, pairs_.cap_pe),
                     std::min(st_host_->n_pp, pairs_.cap_pp), std::min(st_host_->n_ee, pairs_.cap_ee)};
    pf.resize(2 * (size_t)c[0]);
    pe.resize(3 * (size_t)c[1]);
    pp.resize(3 * (size_t)c[2]);
    ee.resize(2 * (size_t)c[3]);
    if (c[0]) PPF_CUDA(cudaMemcpy(pf.data(), pairs_.pf, pf.size() * 4, cudaMemcpyDeviceToHost));
    if (c[1]) PPF_CUDA(cudaMemcpy(pe.data(), pairs_.pe, pe.size() * 4, cudaMemcpyDeviceToHost));
    if (c[2]) PPF_CUDA(cudaMemcpy(pp.data(), pairs_.pp, pp.size() * 4, cudaMemcpyDeviceToHost));
    if (c[3]) PPF_CUDA(cudaMemcpy(ee.data(), pairs_.ee, ee.size() * 4, cudaMemcpyDeviceToHost));
}

// One assembly + linear solve at the current state (target from curr/prev,
// eval_x = curr), exposing the first Newton iteration of a step.
int Solver::debug_assemble_solve(std::vector<float> &dx, unsigned &iters, float &resid) {
    const size_t n3 = 3 * (size_t)n_;
    float dt = param->dt * param->playback;
    PPF_CUDA(cudaMemsetAsync(st_.data(), 0, sizeof(IterStatus), q_));
    if (!param->disable_contact) build_trees(curr_.data(), curr_.data(), 1.0f, true);
    compute_target(dt);
    PPF_CUDA(cudaMemcpyAsync(eval_x_.data(), curr_.data(), n3 * sizeof(float),
                             cudaMemcpyDeviceToDevice, q_));
    force_factor_ = true; // with a factored kind set, solve with it alone
    assemble(dt);
    force_factor_ = false;
    PPF_CUDA(cudaMemcpyAsync(r_.data(), force_.data(), n3 * sizeof(float),
                             cudaMemcpyDeviceToDevice, q_));
    PcgOperator A = pcg_operator();
    launch_pcg(A, dx_.data(), r_.data(), param->cg_tol, param->cg_max_iter, pcg_, q_);
    PcgResult res;
    PPF_CUDA(cudaMemcpyAsync(&res, pcg_.result.data(), sizeof(PcgResult), cudaMemcpyDeviceToHost, q_));
    PPF_CUDA(cudaStreamSynchronize(q_));
    dx.resize(n3);
    PPF_CUDA(cudaMemcpy(dx.data(), dx_.data(), n3 * sizeof(float), cudaMemcpyDeviceToHost));
    iters = res.iter;
    resid = res.resid;
    return res.state;
}

int Solver::debug_pcg(const float *b, std::vector<float> &x, unsigned max_iter, unsigned &iters,
                      float &resid) {
    const size_t n3 = 3 * (size_t)n_;
    PPF_CUDA(cudaMemcpyAsync(r_.data(), b, n3 * sizeof(float), cudaMemcpyHostToDevice, q_));
    PPF_CUDA(cudaMemsetAsync(dx_.data(), 0, n3 * sizeof(float), q_));
    PcgOperator A = pcg_operator();
    launch_pcg(A, dx_.data(), r_.data(), param->cg_tol, max_iter, pcg_, q_);
    PcgResult res;
    PPF_CUDA(cudaMemcpyAsync(&res, pcg_.result.data(), sizeof(PcgResult), cudaMemcpyDeviceToHost, q_));
    PPF_CUDA(cudaStreamSynchronize(q_));
    x.resize(n3);
    PPF_CUDA(cudaMemcpy(x.data(), dx_.data(), n3 * sizeof(float), cudaMemcpyDeviceToHost));
    iters = res.iter;
    resid = res.resid;
    return res.state;
}

float Solver::debug_strain_line_search(const float *x0, const float *x1) {
    const size_t n3 = 3 * (size_t)n_;
    const float max_t = param->line_search_max_t;
    PPF_CUDA(cudaMemcpyAsync(target_.data(), x0, n3 * sizeof(float), cudaMemcpyHostToDevice, q_));
    PPF_CUDA(cudaMemcpyAsync(eval_x_.data(), x1, n3 * sizeof(float), cudaMemcpyHostToDevice, q_));
    const unsigned bits = __builtin_bit_cast(unsigned, max_t);
    PPF_CUDA(cudaMemcpyAsync(&st_.data()->sl_toi_bits, &bits, sizeof(unsigned),
                             cudaMemcpyHostToDevice, q_));
    LineSearchArgs la{target_.data(), eval_x_.data(), curr_.data(), st_.data(), max_t,
                      param->ccd_eps};
    launch_strain_line_search(scene(), la, q_);
    unsigned out = 0;
    PPF_CUDA(cudaMemcpyAsync(&out, &st_.data()->sl_toi_bits, sizeof(unsigned),
                             cudaMemcpyDeviceToHost, q_));
    PPF_CUDA(cudaStreamSynchronize(q_));
    return __builtin_bit_cast(float, out) / max_t;
}

void Solver::set_contact_capacity(unsigned pair_cap, unsigned block_cap) {
    if (pair_cap) {
        pairs_.cap_pf = std::min<unsigned>(pair_cap, (unsigned)pf_buf_.cap);
        pairs_.cap_pe = std::min<unsigned>(pair_cap, (unsigned)pe_buf_.cap);
        pairs_.cap_pp = std::min<unsigned>(pair_cap, (unsigned)pp_buf_.cap);
        pairs_.cap_ee = std::min<unsigned>(pair_cap, (unsigned)ee_buf_.cap);
    }
    if (block_cap) dyn_cap_ = std::max(block_cap, 16u);
}

void Solver::set_tuning(const Tuning &t) {
    const unsigned char team = tune_.pcg_cluster;
    tune_ = t;
    tune_.pcg_cluster = team;
    ++scene_version_; // the line-search graph holds the kernels it chose
}

Tuning Solver::autotune() {
    const size_t n3 = 3 * (size_t)n_;
    const float max_t = param->line_search_max_t;
    pcg_.reserve(n_); // k_init_ls copies the last solve's result block
    PPF_CUDA(cudaStreamSynchronize(q_));
    // min of three timed runs of `run` on the solver's stream, in ms
    auto time = [&](auto &&run) {
        float best = 1e30f;
        for (int k = 0; k < 3; ++k) {
            PPF_CUDA(cudaEventRecord(ev0_, q_));
            run();
            PPF_CUDA(cudaEventRecord(ev1_, q_));
            PPF_CUDA(cudaEventSynchronize(ev1_));
            float ms = 0.0f;
            PPF_CUDA(cudaEventElapsedTime(&ms, ev0_, ev1_));
            best = std::min(best, ms);
        }
        return best;
    };
    // each field in turn, the others held: the kernels run one after another
    // and do not interact, so the per-field choices compose
    auto pick = [&](unsigned char &field, auto &&run) {
        float t[2];
        for (unsigned char v = 0; v < 2; ++v) {
            field = v;
            t[v] = time(run);
        }
        field = t[1] < t[0] ? 1 : 0;
    };
    if (!param->disable_contact && n_surf_) {
        build_trees(curr_.data(), curr_.data(), 1.0f, true);
        PPF_CUDA(cudaMemcpyAsync(eval_x_.data(), curr_.data(), n3 * sizeof(float),
                                 cudaMemcpyDeviceToDevice, q_));
        AssemblyBuffers b = abuf();
        auto detect = [&]() {
            PPF_CUDA(cudaMemsetAsync(st_.data(), 0, sizeof(IterStatus), q_));
            PieceBuffers pb = pieces();
            const Scene sc = scene();
            launch_edge_pieces(sc, view(bvh_edge_), eval_x_.data(), nullptr, nullptr, piece_len_,
                               pb, q_);
            launch_detect(sc, view(bvh_face_), view(bvh_edge_), view(bvh_vert_), b, pairs_, pb,
                          q_);
        };
        pick(tune_.detect_vertex, detect);
        pick(tune_.detect_edge, detect);
        // the CCD over the inertial step from the current positions
        compute_target(param->dt * param->playback);
        build_trees(curr_.data(), target_.data(), max_t, false);
        LineSearchArgs la{curr_.data(), target_.data(), curr_.data(), st_.data(), max_t,
                          param->ccd_eps};
        auto ccd = [&]() {
            k_init_ls<<<1, 1, 0, q_>>>(st_.data(), max_t, pcg_.result.data());
            PPF_LAUNCH_CHECK();
            PieceBuffers pb = pieces();
            launch_contact_line_search(scene(), view(bvh_face_), view(bvh_edge_),
                                       view(bvh_vert_), la, piece_len_, pb, q_);
        };
        pick(tune_.ccd_vertex, ccd);
        if (ncv_) pick(tune_.ccd_mesh_vertex, ccd);
        pick(tune_.ccd_edge, ccd);
        build_trees(curr_.data(), curr_.data(), 1.0f, false);
        auto isect = [&]() {
            PPF_CUDA(cudaMemsetAsync(&st_.data()->n_isect, 0, sizeof(unsigned), q_));
            PieceBuffers pb = pieces();
            launch_intersection_check(scene(), view(bvh_face_), view(bvh_edge_), curr_.data(),
                                      isect_.data(), st_.data(), piece_len_, pb, q_);
        };
        pick(tune_.isect, isect);
    }
    // the PCG's team, by the time of 40 iterations on the Newton system at
    // the current positions (tolerance 0: no early exit), block-Jacobi
    if (pcg_.max_cluster >= 2 && n_) {
        const float dt = param->dt * param->playback;
        PPF_CUDA(cudaMemcpyAsync(eval_x_.data(), curr_.data(), n3 * sizeof(float),
                                 cudaMemcpyDeviceToDevice, q_));
        compute_target(dt);
        PPF_CUDA(cudaMemsetAsync(st_.data(), 0, sizeof(IterStatus), q_));
        assemble(dt);
        PcgOperator A = pcg_operator();
        A.factor = PcgFactor{};
        A.schwarz = SchwarzView{};
        auto solve = [&]() {
            PPF_CUDA(cudaMemcpyAsync(r_.data(), force_.data(), n3 * sizeof(float),
                                     cudaMemcpyDeviceToDevice, q_));
            PPF_CUDA(cudaMemsetAsync(dx_.data(), 0, n3 * sizeof(float), q_));
            launch_pcg(A, dx_.data(), r_.data(), 0.0f, 40u, pcg_, q_);
        };
        float best = 1e30f;
        unsigned char choice = 0;
        for (unsigned c : {0u, pcg_.max_cluster, pcg_.max_cluster / 2}) {
            if (c == 1) continue;
            pcg_.cluster = c;
            const float t = time(solve);
            if (t < best) {
                best = t;
                choice = (unsigned char)c;
            }
        }
        tune_.pcg_cluster = choice;
        pcg_.cluster = choice;
        pcg_team_auto_ = false;
    }
    PPF_CUDA(cudaMemsetAsync(st_.data(), 0, sizeof(IterStatus), q_));
    PPF_CUDA(cudaStreamSynchronize(q_));
    ++scene_version_;
    return tune_;
}

bool Solver::set_pcg_team(int ctas) {
    pcg_.reserve(std::max(n_, 1u));
    if (ctas < 0) {
        pcg_team_auto_ = true;
        tune_.pcg_cluster = auto_pcg_team();
    } else if (ctas == 0 || (ctas >= 2 && (unsigned)ctas <= pcg_.max_cluster)) {
        pcg_team_auto_ = false;
        tune_.pcg_cluster = (unsigned char)ctas;
    } else {
        return false;
    }
    pcg_.cluster = tune_.pcg_cluster;
    return true;
}

// Systems up to kClusterPcgRows vertices solve on one cluster: their
// iterations are bound by the two reductions, which a cluster's hardware
// barrier makes several times cheaper than a grid barrier through L2.
unsigned char Solver::auto_pcg_team() const {
    return n_ <= kClusterPcgRows && pcg_.max_cluster >= 2 ? (unsigned char)pcg_.max_cluster : 0;
}

float Solver::debug_contact_line_search(const float *x0, const float *x1, unsigned &overlap) {
    const size_t n3 = 3 * (size_t)n_;
    const float max_t = param->line_search_max_t;
    pcg_.reserve(n_); // k_init_ls copies the last solve's result block
    PPF_CUDA(cudaMemcpyAsync(target_.data(), x0, n3 * sizeof(float), cudaMemcpyHostToDevice, q_));
    PPF_CUDA(cudaMemcpyAsync(eval_x_.data(), x1, n3 * sizeof(float), cudaMemcpyHostToDevice, q_));
    PPF_CUDA(cudaMemsetAsync(st_.data(), 0, sizeof(IterStatus), q_));
    build_trees(target_.data(), target_.data(), 1.0f, true);
    build_trees(target_.data(), eval_x_.data(), max_t, false);
    k_init_ls<<<1, 1, 0, q_>>>(st_.data(), max_t, pcg_.result.data());
    PPF_LAUNCH_CHECK();
    LineSearchArgs la{target_.data(), eval_x_.data(), curr_.data(), st_.data(), max_t,
                      param->ccd_eps};
    PieceBuffers pb = pieces();
    launch_contact_line_search(scene(), view(bvh_face_), view(bvh_edge_), view(bvh_vert_), la,
                               piece_len_, pb, q_);
    IterStatus st;
    PPF_CUDA(cudaMemcpyAsync(&st, st_.data(), sizeof(IterStatus), cudaMemcpyDeviceToHost, q_));
    PPF_CUDA(cudaStreamSynchronize(q_));
    overlap = st.overlap;
    return bits_to_float(st.toi_bits) / max_t;
}

void Solver::debug_schwarz(unsigned *sizes, std::vector<unsigned> &agg,
                           std::vector<unsigned> &dom) {
    const SchwarzLayout &S = schwarz_;
    sizes[0] = S.ready ? S.n_agg : 0u;
    sizes[1] = S.ready ? S.n_dom : 0u;
    sizes[2] = S.ready ? S.levels : 0u;
    agg.assign(S.ready ? S.n : 0u, 0u);
    dom.assign(sizes[1] ? S.n_agg : 0u, 0u);
    if (!agg.empty())
        PPF_CUDA(cudaMemcpy(agg.data(), S.agg.data(), agg.size() * 4, cudaMemcpyDeviceToHost));
    if (!dom.empty())
        PPF_CUDA(cudaMemcpy(dom.data(), S.dom.data(), dom.size() * 4, cudaMemcpyDeviceToHost));
}

Solver::~Solver() {
    if (q_) cudaStreamSynchronize(q_);
    if (it_graph_) cudaGraphExecDestroy(it_graph_);
    if (ls_graph_) cudaGraphExecDestroy(ls_graph_);
    for (cudaEvent_t e : {ev0_, ev1_, evs0_, evs1_, ev_done_})
        if (e) cudaEventDestroy(e);
    if (st_host_) cudaFreeHost(st_host_);
    if (q_) cudaStreamDestroy(q_);
}

void Solver::release() {
    if (q_) cudaStreamSynchronize(q_);
    initialized_ = false;
}

} // namespace gpu
} // namespace ppf
