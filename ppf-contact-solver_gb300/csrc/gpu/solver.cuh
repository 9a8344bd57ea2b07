// solver.cuh -- the per-step solve behind the reference's C ABI.
#pragma once

#include <vector>

#include "assemble.cuh"
#include "lbvh.cuh"
#include "linesearch.cuh"
#include "pcg.cuh"
#include "precond.cuh"
#include "schwarz.cuh"

namespace ppf {
namespace gpu {

constexpr unsigned kClusterPcgRows = 16384;
// One-cluster solves of systems up to this size run on 512-thread CTAs (per
// PCG iteration on the 64 x 64 cloth: 8.0 against 10.1 us with 1024; at
// 96 x 96 and above 1024 is faster)
constexpr unsigned kSmallCtaRows = 6144;

// Per-step statistics (GB300 extension, ppf_step_stats in ppf_gb300_ext.h).
struct StepStats {
    unsigned newton_iters = 0;
    unsigned pcg_iters_total = 0;
    unsigned pcg_solves = 0;
    float pcg_ms_total = 0.0f;
    float step_ms = 0.0f;
    unsigned max_contacts = 0;
    unsigned max_dyn_blocks = 0;
    std::vector<float> pcg_ms;        // per solve
    std::vector<unsigned> pcg_iters;  // per solve
    std::vector<float> toi;           // per Newton iteration
    std::vector<unsigned> dyn_blocks; // per solve
    unsigned fallbacks = 0;           // factored solves redone with block-Jacobi
    unsigned factor_iters_total = 0;  // iterations of the factored solves
    // the last solve's verdict
    int last_state = 0, last_break_cause = 0;
    float last_resid = 0.0f, last_break_val = 0.0f;
};

class Solver {
  public:
    Solver() = default;
    Solver(const Solver &) = delete;
    Solver &operator=(const Solver &) = delete;
    // its stream, graphs, events and pinned status (device buffers free
    // themselves)
    ~Solver();
    bool initialize(PpfDataSet *ds, PpfParamSet *param);
    PpfStepResult advance();
    void fetch();
    void update_constraint(const PpfConstraint *c);
    void update_rest_shape(const PpfRestShapeUpdate *u);
    void fetch_dyn_counts(unsigned *n_value, unsigned *n_offset);
    void fetch_dyn(unsigned *index, PpfMat3x3f *value, unsigned *offset);
    void update_dyn(const unsigned *index, const unsigned *offset);
    void fetch_inv_rest();
    void fetch_rest_angles();
    void override_velocity(const unsigned *idx, unsigned count, float vx, float vy,
                           float vz, float dt);
    void override_angular_velocity(const unsigned *idx, unsigned count, float wx,
                                   float wy, float wz, float cx, float cy, float cz,
                                   float dt);
    void gather_current_positions(const unsigned *idx, unsigned count, float *out);
    void set_active(const std::vector<unsigned char> &vert_active);
    unsigned fetch_intersection_records(PpfIntersectionRecord *out, unsigned max_count);
    const StepStats &stats() const { return stats_; }
    cudaStream_t stream() const { return q_; }
    unsigned fixed_blocks() const { return nnz_fixed_; }
    unsigned vertices() const { return n_; }
    // PPF_PRECOND_* of ppf_gb300_ext.h; false for an unknown kind
    bool set_preconditioner(int kind, float param);
    // bf16 weight blob of the learned preconditioner (learned.cuh); false
    // when count is not the network's size
    bool set_learned_weights(const unsigned short *w, unsigned count);
    // the kind of the last solve: PPF_PRECOND_* (3: aggregate Schwarz)
    int preconditioner() const { return schwarz_active_ ? 3 : precond_kind_; }
    // debug views (host copies) for stage parity checks
    void debug_matrix(std::vector<unsigned> &f_off, std::vector<unsigned> &f_col,
                      std::vector<float> &f_val, std::vector<unsigned> &d_off,
                      std::vector<unsigned> &d_col, std::vector<float> &d_val,
                      std::vector<float> &diag, std::vector<float> &force);
    // per-vertex mass and Dirichlet mask; G(i, i) of the last factor built
    void debug_vertex_info(std::vector<float> &mass, std::vector<unsigned> &dof);
    void debug_factor_diag(std::vector<float> &diag);
    void debug_pairs(std::vector<unsigned> &pf, std::vector<unsigned> &pe,
                     std::vector<unsigned> &pp, std::vector<unsigned> &ee);
    // one assembly + solve at the current positions, without line search
    int debug_assemble_solve(std::vector<float> &dx, unsigned &iters, float &resid);
    // Solves the operator (and preconditioner) of the last debug_assemble_solve
    // with right-hand side b from x = 0, at most max_iter iterations.
    int debug_pcg(const float *b, std::vector<float> &x, unsigned max_iter, unsigned &iters,
                  float &resid);
    // The strain-limit line search (faces and rods) from x0 to x1, as the
    // fraction of x1 - x0 it admits (the time of impact over max_t).
    float debug_strain_line_search(const float *x0, const float *x1);
    // The contact line search (CCD over trees swept from x0 to x1), as the
    // fraction of x1 - x0 it admits; `overlap` reports a start inside an offset.
    float debug_contact_line_search(const float *x0, const float *x1, unsigned &overlap);
    // The Schwarz layout of the last solve: sizes {n_agg, n_dom, levels},
    // the aggregate of each vertex and the domain of each aggregate.
    void debug_schwarz(unsigned *sizes, std::vector<unsigned> &agg, std::vector<unsigned> &dom);
    // Times both leaf-test forms of every traversal kernel on the current
    // state (detection at the positions, the CCD over the inertial step, the
    // intersection check) and keeps the faster of each; returns the choice.
    Tuning autotune();
    Tuning tuning() const { return tune_; }
    // the traversal leaf-test forms (the PCG team is kept)
    void set_tuning(const Tuning &t);
    // The PCG's team: -1 automatic (one cluster up to kClusterPcgRows
    // vertices, else the whole grid), 0 the whole grid, 2 to the largest
    // cluster the device runs: one cluster of that many CTAs. False for a
    // size the device cannot run.
    bool set_pcg_team(int ctas);
    unsigned pcg_team() const { return tune_.pcg_cluster; }
    // the PCG's static share of the product work, in sixteenths (1 to 16;
    // 0 the default)
    void set_pcg_static_share(unsigned sixteenths) { pcg_.static_sixteenths = sixteenths; }
    // threads per CTA of a one-cluster block-Jacobi solve: 256, 512 or 1024;
    // 0 restores the automatic choice (512 up to kSmallCtaRows vertices, else
    // 1024); false for another value
    bool set_pcg_cta_threads(unsigned threads) {
        if (threads != 0 && threads != 256 && threads != 512 && threads != 1024) return false;
        cta_auto_ = threads == 0;
        pcg_.cluster_threads = cta_auto_ ? auto_cta_threads() : threads;
        return true;
    }
    // Caps the pair lists at pair_cap entries each and a capacity-sized
    // iteration at block_cap contact blocks (0 leaves one as it is); larger
    // counts then take the overrun-and-repeat path.
    void set_contact_capacity(unsigned pair_cap, unsigned block_cap);
    void release();

    PpfDataSet *host = nullptr;
    PpfParamSet *param = nullptr;

  private:
    Scene scene() const;
    StepParams step_params(float dt) const;
    AssemblyBuffers abuf();
    PcgOperator pcg_operator() const;
    void upload_props();
    void build_trees(const float *x0, const float *x1, float extrap, bool rebuild);
    BvhView view(const Lbvh &b) const;
    void compute_target(float dt);
    void upload_step_params(float dt);
    void grow_pairs(const unsigned counts[4]);
    void assemble(float dt);
    void assemble_stage(bool capacity);
    unsigned schwarz_levels() const;
    bool schwarz_ready() const;
    void record_event(cudaEvent_t ev, bool capturing);
    void enqueue_solve(bool capturing);
    bool check_intersection(const float *x);
    void enqueue_line_search();
    void line_search_stage();
    void read_status();
    void wait();
    cudaEvent_t ev_done_ = nullptr;

    unsigned n_ = 0, n_surf_ = 0, nf_ = 0, ne_ = 0, nh_ = 0, nr_ = 0, nf_shell_ = 0, nt_ = 0;
    cudaStream_t q_ = nullptr;
    // topology / props / params
    DevBuf<unsigned> face_, edge_, hinge_;
    DevBuf<PpfVertexProp> vprop_;
    DevBuf<PpfEdgeProp> eprop_;
    DevBuf<PpfFaceProp> fprop_;
    DevBuf<PpfHingeProp> hprop_;
    DevBuf<PpfVertexParam> vparam_;
    DevBuf<PpfEdgeParam> eparam_;
    DevBuf<PpfFaceParam> fparam_;
    DevBuf<PpfHingeParam> hparam_;
    DevBuf<float> inv_rest_;
    DevBuf<unsigned> vf_off_, vf_, ve_off_, ve_, ef_off_, ef_;
    DevBuf<unsigned> fixed_off_, fixed_col_, fixed_tr_off_, fixed_diag_;
    DevBuf<uint2> fixed_tr_;
    DevBuf<unsigned> face_slot_, hinge_slot_, edge_slot_, bend_slot_, dof_mask_, tet_, tet_slot_;
    DevBuf<PpfTetProp> tprop_;
    DevBuf<PpfTetParam> tparam_;
    DevBuf<float> inv_rest3_;
    DevBuf<unsigned char> hinge_type_;
    DevBuf<PpfStitch> stitch_;
    DevBuf<unsigned> stitch_slot_;
    unsigned nstitch_ = 0;
    DevBuf<PpfFixPair> fix_;
    DevBuf<PpfPullPair> pull_;
    DevBuf<PpfSphere> sphere_;
    DevBuf<PpfFloor> floor_;
    unsigned nfix_ = 0, npull_ = 0, nsphere_ = 0, nfloor_ = 0;
    DevBuf<float> margin_face_, margin_edge_, margin_vert_;
    DevBuf<unsigned char> vert_active_, edge_active_, face_active_;
    bool use_active_ = false;
    std::vector<PpfVertexProp> h_vprop_;
    std::vector<PpfFaceProp> h_fprop_;
    std::vector<PpfEdgeProp> h_eprop_;
    std::vector<PpfHingeProp> h_hprop_;
    unsigned nnz_fixed_ = 0;
    // state
    DevBuf<float> curr_, prev_, eval_x_, target_, force_, dx_, diag_, r_;
    DevBuf<float> fixed_val_, fixed_tmp_, inv_diag_;
    Lbvh bvh_face_, bvh_edge_, bvh_vert_;
    RadixSortWorkspace sort_ws_;
    PairLists pairs_;
    DevBuf<uint2> pf_buf_, ee_buf_;
    DevBuf<uint3> pe_buf_, pp_buf_;
    DynMatrix dyn_;
    DevBuf<unsigned long long> hkey_buf_;
    DevBuf<unsigned> hval_buf_, doff_buf_, dcol_buf_, dtroff_buf_, dcnt_buf_, dcnt2_buf_;
    DevBuf<uint2> dtr_buf_;
    DevBuf<float> dval_buf_;
    DevBuf<unsigned> scan_tmp_;
    // contact pattern restored by update_dyn (a resumed run's carried
    // pattern): reported by fetch_dyn until the next assembly replaces it
    std::vector<unsigned> carried_off_, carried_col_;
    bool carried_ = false;
    PcgWorkspace pcg_;
    // factored preconditioner (block-Jacobi stays the fallback)
    int precond_kind_ = 0;
    float precond_param_ = 0.5f;
    float factor_eps_ = 1e-3f;
    unsigned plain_iters_ = 0; // iterations of the last block-Jacobi solve
    bool factor_active_ = false;
    bool learned_ready_ = false; // network weights loaded
    bool force_factor_ = false;  // the debug solve uses the factor directly
    FactorBuffers factor_;
    DevBuf<bf16_t> learned_w_;
    LearnedNodes learned_nodes_;
    DevBuf<float> mass_;
    // static collision mesh
    unsigned ncv_ = 0, ncf_ = 0, nce_ = 0;
    DevBuf<float> cm_x_, cm_margin_f_, cm_margin_e_;
    DevBuf<unsigned> cm_face_, cm_edge_;
    DevBuf<PpfVertexProp> cm_vprop_;
    DevBuf<PpfFaceProp> cm_fprop_;
    DevBuf<PpfEdgeProp> cm_eprop_;
    DevBuf<PpfVertexParam> cm_vparam_;
    DevBuf<PpfFaceParam> cm_fparam_;
    DevBuf<PpfEdgeParam> cm_eparam_;
    Lbvh cm_bvh_face_, cm_bvh_edge_;
    void upload_collision_mesh(const PpfCollisionMesh &cm);
    // aggregate Schwarz (ParamSet::precond == 1), aggregated once per scene
    bool schwarz_active_ = false;
    SchwarzLayout schwarz_;
    DevBuf<float> dx0_;
    DevBuf<unsigned> run_plain_;
    void build_factor();
    SellLayout fixed_sell_;
    DynLayout dyn_layout_;
    DevBuf<unsigned> piece_cnt_, piece_off_, piece_tmp_;
    float piece_len_ = 0.0f;
    PieceBuffers pieces();
    DevBuf<IterStatus> st_;
    IterStatus *st_host_ = nullptr;
    // the line-search stage captured as a CUDA graph, keyed on the scene
    cudaGraphExec_t ls_graph_ = nullptr;
    unsigned long long scene_version_ = 0, ls_key_ = ~0ull;
    Tuning tune_;
    float ls_max_t_ = 0.0f, ls_max_dx_ = 0.0f, ls_ccd_eps_ = 0.0f;
    unsigned ls_launches_ = 0;
  public:
    unsigned long long ls_replays_ = 0; // graph launches of the line-search stage
    // Newton iterations run through the iteration graph: directly (the first
    // under a new key), captured, replayed, and repeated after a capacity
    // overran
    struct GraphStats {
        unsigned long long direct = 0, captures = 0, replays = 0, repeats = 0;
    } graph_stats_;
    // the whole Newton iteration as one CUDA graph (on by default; off runs
    // the sized-by-read-back assembly and the line-search graph alone)
    bool graph_enabled_ = true;
    // waits for the stream sleep on an event instead of spinning (many
    // solvers stepped by more host threads than cores)
    bool blocking_sync_ = false;
  private:
    struct IterKey {
        Scene scene;
        PpfParamSet param;
        PairLists pairs;
        float piece_len;
        unsigned dyn_cap, use_active, schwarz;
        unsigned nnz_fixed, fixed_slices, fixed_slots;
        unsigned agg[6]; // Schwarz: n, n_agg, max_members, levels, n_dom, max_dom_members
        unsigned long long epoch;
    };
    IterKey iteration_key() const;
    bool iteration_graph_ok() const;
    void enqueue_iteration(bool capturing);
    void iteration_graph(float dt);
    cudaGraphExec_t it_graph_ = nullptr;
    IterKey it_key_{}, it_eager_key_{};
    bool it_eager_valid_ = false;
    unsigned it_launches_ = 0;
    // contact blocks a capacity-sized iteration holds; doubled past the count
    // an overrun iteration reached
    unsigned dyn_cap_ = 1u << 18;
    DevBuf<StepParams> sp_dev_;
    bool pcg_team_auto_ = true;
    unsigned char auto_pcg_team() const;
    bool cta_auto_ = true;
    unsigned auto_cta_threads() const { return n_ <= kSmallCtaRows ? 512u : 0u; }
    DevBuf<PpfIntersectionRecord> isect_;
    std::vector<PpfIntersectionRecord> isect_host_;
    unsigned isect_count_ = 0;
    cudaEvent_t ev0_ = nullptr, ev1_ = nullptr, evs0_ = nullptr, evs1_ = nullptr;
    StepStats stats_;
    bool initialized_ = false;
};

Solver &solver_instance();

} // namespace gpu
} // namespace ppf
