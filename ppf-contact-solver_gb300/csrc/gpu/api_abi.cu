// api_abi.cu -- the reference's extern "C" backend entry points
// (crates/ppf-cts-solver/src/cpp/main/main.cu:1673-2350) and the stats /
// stage-inspection extensions of include/ppf_gb300_ext.h.
#include "../../../include/ppf_gb300_ext.h"
#include "fatal.cuh"
#include "learned.cuh"
#include "schwarz.cuh"
#include "solver.cuh"
#include "stats.cuh"

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <sys/stat.h>
#include <vector>

using ppf::FatalError;
using ppf::gpu::solver_instance;

namespace {

bool return_on_fatal() {
    const char *e = std::getenv("PPF_RETURN_ON_FATAL");
    return e && e[0] == '1';
}

// Records the error as the reference's fatal path does, then exits with
// status 1 unless the host asked to get the failure back instead.
void fatal(const FatalError &e) {
    ppf::set_fatal(e.code, e.detail.c_str());
    fprintf(stderr, "[ppf_gb300] fatal: %s\n", e.detail.c_str());
    fflush(stderr);
    if (!return_on_fatal()) std::exit(1);
}

struct DebugCache {
    std::vector<unsigned> f_off, f_col, d_off, d_col, pf, pe, pp, ee;
    std::vector<float> f_val, d_val, diag, force;
} g_dbg;

std::vector<unsigned char> g_window_dmap_active;
struct Windows {
    std::vector<unsigned> dmap;
    std::vector<float> windows;
    std::vector<unsigned> counts;
    bool on = false;
} g_win;
constexpr unsigned kMaxCollisionWindows = 8; // main.cu:45

// Per-step log files in the directory set_log_path names, in the format of
// the reference's SimpleLog (simplelog/SimpleLog.cpp:86-120): `advance.out`
// holds "time msec" per step, and `advance.<channel>.out` one "time value"
// line per value marked in the step (integers as %d, others as %e), with
// time the simulation time at the start of the step (main.cu:329).
struct StepLog {
    std::string dir;
    void line(const char *channel, double t, double v) const {
        std::string path = dir + "/advance" + (channel[0] ? "." : "") + channel + ".out";
        FILE *fp = std::fopen(path.c_str(), "a");
        if (!fp) return;
        if (std::fmod(v, 1.0) == 0.0 && std::fabs(v) < 2e9)
            std::fprintf(fp, "%f %d\n", t, (int)v);
        else
            std::fprintf(fp, "%f %e\n", t, v);
        std::fclose(fp);
    }
    void step(double t, const ppf::gpu::StepStats &s, double final_dt) const {
        if (dir.empty()) return;
        FILE *fp = std::fopen((dir + "/advance.out").c_str(), "a");
        if (fp) {
            std::fprintf(fp, "%f %lu\n", t, (unsigned long)s.step_ms);
            std::fclose(fp);
        }
        for (size_t k = 0; k < s.pcg_iters.size(); ++k) line("iter", t, s.pcg_iters[k]);
        for (size_t k = 0; k < s.toi.size(); ++k) line("toi", t, s.toi[k]);
        line("num_contact", t, s.max_contacts);
        line("newton_steps", t, s.newton_iters);
        line("final_dt", t, final_dt);
    }
} g_log;

} // namespace

extern "C" {

bool initialize(PpfDataSet *dataset, PpfParamSet *param) {
    try {
        // a new session starts without the previous one's fatal report (a
        // host that gets failures back may initialize again in one process)
        ppf::set_fatal(0, "");
        int count = 0;
        if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0) {
            throw FatalError(PPF_FATAL_CUDA_DRIVER, "no CUDA device is visible to this process");
        }
        return solver_instance().initialize(dataset, param);
    } catch (const FatalError &e) {
        fatal(e);
        return false;
    }
}

void advance(PpfStepResult *result) {
    try {
        const double t0 = solver_instance().param ? solver_instance().param->time : 0.0;
        *result = solver_instance().advance();
        if (!g_log.dir.empty())
            g_log.step(t0, solver_instance().stats(), solver_instance().param->prev_dt);
    } catch (const FatalError &e) {
        fatal(e);
        std::memset(result, 0, sizeof(*result));
    }
}

void fetch(void) {
    try {
        solver_instance().fetch();
    } catch (const FatalError &e) {
        fatal(e);
    }
}

void fetch_inv_rest(void) {
    try {
        solver_instance().fetch_inv_rest();
    } catch (const FatalError &e) {
        fatal(e);
    }
}

void fetch_rest_angles(void) {
    try {
        solver_instance().fetch_rest_angles();
    } catch (const FatalError &e) {
        fatal(e);
    }
}

void fetch_dyn_counts(unsigned *n_value, unsigned *n_offset) {
    try {
        solver_instance().fetch_dyn_counts(n_value, n_offset);
    } catch (const FatalError &e) {
        fatal(e);
    }
}

void fetch_dyn(unsigned *index, PpfMat3x3f *value, unsigned *offset) {
    try {
        solver_instance().fetch_dyn(index, value, offset);
    } catch (const FatalError &e) {
        fatal(e);
    }
}

void update_dyn(unsigned *index, unsigned *offset) {
    try {
        solver_instance().update_dyn(index, offset);
    } catch (const FatalError &e) {
        fatal(e);
    }
}

void update_constraint(const PpfConstraint *constraint) {
    try {
        solver_instance().host->constraint = *constraint;
        solver_instance().update_constraint(constraint);
    } catch (const FatalError &e) {
        fatal(e);
    }
}

void update_rest_shape(const PpfRestShapeUpdate *update) {
    try {
        solver_instance().update_rest_shape(update);
    } catch (const FatalError &e) {
        fatal(e);
    }
}

void override_velocity(const unsigned *indices, unsigned count, float vx, float vy,
                       float vz, float dt) {
    try {
        solver_instance().override_velocity(indices, count, vx, vy, vz, dt);
    } catch (const FatalError &e) {
        fatal(e);
    }
}

void gather_current_positions(const unsigned *indices, unsigned count, float *out) {
    try {
        solver_instance().gather_current_positions(indices, count, out);
    } catch (const FatalError &e) {
        fatal(e);
    }
}

void override_angular_velocity(const unsigned *indices, unsigned count, float wx, float wy,
                               float wz, float cx, float cy, float cz, float dt) {
    try {
        solver_instance().override_angular_velocity(indices, count, wx, wy, wz, cx, cy, cz, dt);
    } catch (const FatalError &e) {
        fatal(e);
    }
}

void init_collision_windows(const unsigned *vert_dmap, unsigned vert_count,
                            const float *windows, const unsigned *window_counts,
                            unsigned n_groups) {
    g_win.dmap.assign(vert_dmap, vert_dmap + vert_count);
    g_win.windows.assign(windows, windows + (size_t)n_groups * kMaxCollisionWindows * 2);
    g_win.counts.assign(window_counts, window_counts + n_groups);
    g_win.on = true;
}

void refresh_collision_active(float time) {
    if (!g_win.on) return;
    try {
        std::vector<unsigned char> active(g_win.dmap.size());
        for (size_t i = 0; i < g_win.dmap.size(); ++i) {
            unsigned dm = g_win.dmap[i];
            unsigned cnt = g_win.counts[dm];
            bool a = cnt == 0;
            for (unsigned w = 0; w < cnt && !a; ++w) {
                float ts = g_win.windows[dm * kMaxCollisionWindows * 2 + w * 2];
                float te = g_win.windows[dm * kMaxCollisionWindows * 2 + w * 2 + 1];
                a = time >= ts && time < te;
            }
            active[i] = a ? 1 : 0;
        }
        solver_instance().set_active(active);
    } catch (const FatalError &e) {
        fatal(e);
    }
}

unsigned fetch_intersection_records(PpfIntersectionRecord *out, unsigned max_count) {
    return solver_instance().fetch_intersection_records(out, max_count);
}

unsigned char ppf_fatal_code(void) { return g_ppf_fatal_code; }
const char *ppf_fatal_detail(void) { return g_ppf_fatal_detail; }
void set_log_path(const char *data_dir) {
    g_log.dir = data_dir ? data_dir : "";
    if (!g_log.dir.empty()) mkdir(g_log.dir.c_str(), 0775);
}

// ---- extensions -------------------------------------------------------------
void ppf_step_stats(PpfStepStats *out) { ppf::gpu::fill_step_stats(solver_instance(), out); }
}

namespace ppf {
namespace gpu {
void fill_step_stats(const Solver &solver, PpfStepStats *out) {
    const ppf::gpu::StepStats &s = solver.stats();
    std::memset(out, 0, sizeof(*out));
    out->newton_iters = s.newton_iters;
    out->pcg_iters_total = s.pcg_iters_total;
    out->pcg_solves = s.pcg_solves;
    out->pcg_ms_total = s.pcg_ms_total;
    out->step_ms = s.step_ms;
    out->max_contacts = s.max_contacts;
    out->max_dyn_blocks = s.max_dyn_blocks;
    unsigned k = s.pcg_solves < PPF_STATS_MAX_SOLVES ? s.pcg_solves : PPF_STATS_MAX_SOLVES;
    for (unsigned i = 0; i < k; ++i) {
        out->pcg_ms[i] = s.pcg_ms[i];
        out->pcg_iters[i] = s.pcg_iters[i];
        out->toi[i] = i < s.toi.size() ? s.toi[i] : 0.0f;
        out->dyn_blocks[i] = i < s.dyn_blocks.size() ? s.dyn_blocks[i] : 0u;
    }
    out->fixed_blocks = solver.fixed_blocks();
    out->vertices = solver.vertices();
    out->precond_kind = (unsigned)solver.preconditioner();
    out->fallbacks = s.fallbacks;
    out->factor_iters_total = s.factor_iters_total;
    out->last_pcg_state = s.last_state;
    out->last_break_cause = s.last_break_cause;
    out->last_pcg_resid = s.last_resid;
    out->last_break_val = s.last_break_val;
}
} // namespace gpu
} // namespace ppf

extern "C" {

unsigned ppf_schwarz_aggregate(unsigned n, const unsigned *off, const unsigned *col,
                               const float *wgt, unsigned kmax, unsigned *agg) {
    std::vector<unsigned> o(off, off + n + 1), c(col, col + off[n]), a;
    std::vector<float> w(wgt, wgt + off[n]);
    const unsigned n_agg = ppf::gpu::schwarz_aggregate(n, o, c, w, kmax, a);
    std::copy(a.begin(), a.end(), agg);
    return n_agg;
}

unsigned ppf_schwarz_coarsen(unsigned n, const unsigned *off, const unsigned *col,
                             const float *blocks, const unsigned *agg, unsigned n_agg,
                             unsigned kmax, unsigned *dom) {
    std::vector<unsigned> o(off, off + n + 1), c(col, col + off[n]), a(agg, agg + n), d;
    const unsigned n_dom = ppf::gpu::schwarz_coarsen(n, o, c, blocks, a, n_agg, kmax, d);
    std::copy(d.begin(), d.end(), dom);
    return n_dom;
}

int ppf_set_preconditioner(int kind, float param) {
    return solver_instance().set_preconditioner(kind, param) ? 0 : -1;
}

void *ppf_stream(void) { return (void *)solver_instance().stream(); }

unsigned long long ppf_kernel_launches(void) { return ppf::gpu::g_kernel_launches; }
unsigned long long ppf_graph_launches(void) {
    return solver_instance().ls_replays_ + solver_instance().graph_stats_.replays;
}
int ppf_set_pcg_team(int ctas) {
    try {
        return solver_instance().set_pcg_team(ctas) ? 0 : -1;
    } catch (const ppf::FatalError &e) {
        ppf::set_fatal(e.code, e.what());
        return -1;
    }
}
int ppf_pcg_team(void) { return (int)solver_instance().pcg_team(); }
int ppf_set_pcg_cta_threads(unsigned threads) {
    return solver_instance().set_pcg_cta_threads(threads) ? 0 : -1;
}
int ppf_set_pcg_static_share(unsigned sixteenths) {
    if (sixteenths > 16) return -1;
    solver_instance().set_pcg_static_share(sixteenths);
    return 0;
}
void ppf_set_iteration_graph(int enable) { solver_instance().graph_enabled_ = enable != 0; }
void ppf_iteration_graph_stats(unsigned long long *out) {
    const auto &g = solver_instance().graph_stats_;
    out[0] = g.direct;
    out[1] = g.captures;
    out[2] = g.replays;
    out[3] = g.repeats;
}
void ppf_debug_set_contact_capacity(unsigned pair_cap, unsigned block_cap) {
    solver_instance().set_contact_capacity(pair_cap, block_cap);
}
void ppf_transfer_bytes(unsigned long long *h2d, unsigned long long *d2h) {
    if (h2d) *h2d = ppf::gpu::g_h2d_bytes;
    if (d2h) *d2h = ppf::gpu::g_d2h_bytes;
}

int ppf_debug_newton_system(float *dx, unsigned *iters, float *resid) {
    try {
        std::vector<float> d;
        int state = solver_instance().debug_assemble_solve(d, *iters, *resid);
        std::memcpy(dx, d.data(), d.size() * sizeof(float));
        solver_instance().debug_matrix(g_dbg.f_off, g_dbg.f_col, g_dbg.f_val, g_dbg.d_off,
                                       g_dbg.d_col, g_dbg.d_val, g_dbg.diag, g_dbg.force);
        solver_instance().debug_pairs(g_dbg.pf, g_dbg.pe, g_dbg.pp, g_dbg.ee);
        return state;
    } catch (const FatalError &e) {
        fatal(e);
        return -1;
    }
}

void ppf_debug_system_sizes(unsigned *sizes) {
    sizes[0] = (unsigned)g_dbg.f_col.size();
    sizes[1] = (unsigned)g_dbg.d_col.size();
    sizes[2] = (unsigned)g_dbg.pf.size() / 2;
    sizes[3] = (unsigned)g_dbg.pe.size() / 3;
    sizes[4] = (unsigned)g_dbg.pp.size() / 3;
    sizes[5] = (unsigned)g_dbg.ee.size() / 2;
}

void ppf_debug_system(unsigned *f_off, unsigned *f_col, float *f_val, unsigned *d_off,
                      unsigned *d_col, float *d_val, float *diag, float *force,
                      unsigned *pf, unsigned *pe, unsigned *pp, unsigned *ee) {
    auto cp = [](void *dst, const auto &v) {
        if (dst && !v.empty()) std::memcpy(dst, v.data(), v.size() * sizeof(v[0]));
    };
    cp(f_off, g_dbg.f_off);
    cp(f_col, g_dbg.f_col);
    cp(f_val, g_dbg.f_val);
    cp(d_off, g_dbg.d_off);
    cp(d_col, g_dbg.d_col);
    cp(d_val, g_dbg.d_val);
    cp(diag, g_dbg.diag);
    cp(force, g_dbg.force);
    cp(pf, g_dbg.pf);
    cp(pe, g_dbg.pe);
    cp(pp, g_dbg.pp);
    cp(ee, g_dbg.ee);
}

void ppf_debug_vertex_info(float *mass, unsigned *dof_mask) {
    try {
        std::vector<float> m;
        std::vector<unsigned> d;
        solver_instance().debug_vertex_info(m, d);
        if (mass) std::memcpy(mass, m.data(), m.size() * sizeof(float));
        if (dof_mask) std::memcpy(dof_mask, d.data(), d.size() * sizeof(unsigned));
    } catch (const FatalError &e) {
        fatal(e);
    }
}

int ppf_debug_pcg(const float *b, float *x, unsigned max_iter, unsigned *iters, float *resid) {
    try {
        std::vector<float> v;
        const int state = solver_instance().debug_pcg(b, v, max_iter, *iters, *resid);
        std::memcpy(x, v.data(), v.size() * sizeof(float));
        return state;
    } catch (const FatalError &e) {
        fatal(e);
        return -1;
    }
}

namespace {
void tuning_out(const ppf::gpu::Tuning &t, unsigned char *m) {
    m[0] = t.detect_vertex;
    m[1] = t.detect_edge;
    m[2] = t.ccd_vertex;
    m[3] = t.ccd_mesh_vertex;
    m[4] = t.ccd_edge;
    m[5] = t.isect;
}
} // namespace

int ppf_autotune(unsigned char *modes) {
    try {
        const ppf::gpu::Tuning t = solver_instance().autotune();
        if (modes) tuning_out(t, modes);
        return 0;
    } catch (const FatalError &e) {
        fatal(e);
        return -1;
    }
}

void ppf_get_tuning(unsigned char *modes) { tuning_out(solver_instance().tuning(), modes); }

int ppf_set_tuning(const unsigned char *m) {
    for (int k = 0; k < 6; ++k)
        if (m[k] > 1) return -1;
    ppf::gpu::Tuning t;
    t.detect_vertex = m[0];
    t.detect_edge = m[1];
    t.ccd_vertex = m[2];
    t.ccd_mesh_vertex = m[3];
    t.ccd_edge = m[4];
    t.isect = m[5];
    solver_instance().set_tuning(t);
    return 0;
}

float ppf_debug_contact_line_search(const float *x0, const float *x1, unsigned *overlap) {
    try {
        unsigned ov = 0;
        const float t = solver_instance().debug_contact_line_search(x0, x1, ov);
        if (overlap) *overlap = ov;
        return t;
    } catch (const FatalError &e) {
        fatal(e);
        return -1.0f;
    }
}

float ppf_debug_strain_line_search(const float *x0, const float *x1) {
    try {
        return solver_instance().debug_strain_line_search(x0, x1);
    } catch (const FatalError &e) {
        fatal(e);
        return -1.0f;
    }
}

void ppf_debug_schwarz_layout(unsigned *sizes, unsigned *agg, unsigned *dom) {
    try {
        std::vector<unsigned> a, d;
        solver_instance().debug_schwarz(sizes, a, d);
        if (agg && !a.empty()) std::memcpy(agg, a.data(), a.size() * 4);
        if (dom && !d.empty()) std::memcpy(dom, d.data(), d.size() * 4);
    } catch (const FatalError &e) {
        fatal(e);
    }
}

void ppf_debug_factor_diag(float *out) {
    try {
        std::vector<float> d;
        solver_instance().debug_factor_diag(d);
        std::memcpy(out, d.data(), d.size() * sizeof(float));
    } catch (const FatalError &e) {
        fatal(e);
    }
}

int ppf_set_learned_weights(const unsigned short *bf16, unsigned count) {
    try {
        return solver_instance().set_learned_weights(bf16, count) ? 0 : -1;
    } catch (const FatalError &e) {
        fatal(e);
        return -1;
    }
}

int ppf_learned_add_sample(unsigned n, const unsigned *f_off, const unsigned *f_col,
                           const float *f_val, const unsigned *c_off, const unsigned *c_col,
                           const float *c_val, const unsigned *dof_mask, const float *mass) {
    try {
        return ppf::gpu::learned_add_sample(n, f_off, f_col, f_val, c_off, c_col, c_val,
                                            dof_mask, mass);
    } catch (const FatalError &e) {
        fatal(e);
        return -1;
    }
}

void ppf_learned_clear_samples(void) {
    try {
        ppf::gpu::learned_clear_samples();
    } catch (const FatalError &e) {
        fatal(e);
    }
}

int ppf_learned_tensor_path(int tc) { return ppf::gpu::learned_tensor_path(tc); }

unsigned ppf_learned_tc_status(void) {
    try {
        return ppf::gpu::learned_tc_status();
    } catch (const FatalError &e) {
        fatal(e);
        return ~0u;
    }
}

int ppf_learned_sample_info(int sample, unsigned *n, unsigned *edges, unsigned *n_free) {
    return ppf::gpu::learned_sample_info(sample, n, edges, n_free);
}

static bool aligned16(const void *p) { return ((uintptr_t)p & 15u) == 0; }

int ppf_learned_forward(int sample, const void *d_weights, float *h_alpha, float *h_q) {
    if (!aligned16(d_weights)) return -1;
    try {
        return ppf::gpu::learned_forward(sample, (const ppf::gpu::bf16_t *)d_weights, h_alpha,
                                         h_q);
    } catch (const FatalError &e) {
        fatal(e);
        return -1;
    }
}

int ppf_learned_loss_grad(int sample, const void *d_weights, const float *d_probes,
                          unsigned n_probes, float *d_grad, float *h_loss, void *stream) {
    if (!aligned16(d_weights)) return -1;
    try {
        return ppf::gpu::learned_loss_grad(sample, (const ppf::gpu::bf16_t *)d_weights, d_probes,
                                           n_probes, d_grad, h_loss, (cudaStream_t)stream);
    } catch (const FatalError &e) {
        fatal(e);
        return -1;
    }
}

} // extern "C"
