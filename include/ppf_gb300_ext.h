/*
 * ppf_gb300_ext.h -- stage-level entry points of libppf_gb300.so.
 *
 * The reference runs these stages only inside advance(); it has no separate
 * entry point for them. They exist here so a host can run, check and time a
 * single stage of the per-step solve with plain pointers. Host-pointer
 * variants copy in and out; device-pointer variants take device memory and a
 * cudaStream_t passed as void*.
 */
#ifndef PPF_GB300_EXT_H
#define PPF_GB300_EXT_H

#include "ppf_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

/* LBVH build of one primitive set, standing in for lbvh::build_face_bvh /
 * build_edge_bvh / build_vertex_bvh (crates/ppf-cts-solver/src/cpp/lbvh/
 * lbvh.cu:863-1030) run on their own.
 *   kind    1 = surface vertices, 2 = edges, 3 = faces
 *   x0, x1  3 * n_verts floats; the tree is ordered by centroids of x1 and the
 *           leaf boxes cover the sweep x0 -> x0 + extrapolate (x1 - x0)
 *   prims   kind * n_prims vertex indices (ignored for kind 1)
 *   margin  n_prims floats, 0.5 * ghat + offset of each primitive
 * Outputs (any may be NULL):
 *   out_node  2 * (2 n_prims - 1) u32: leaves (prim + 1, 0) in Morton order,
 *             internal node n_prims + i as (left + 1, right + 1)
 *   out_box   8 * (2 n_prims - 1) floats: min xyz, active flag, max xyz, 0
 *   out_keys  n_prims sorted Morton codes
 * Returns the root node index, or 0xffffffff on failure. */
unsigned ppf_lbvh_build_host(int kind, const float *x0, const float *x1,
                             unsigned n_verts, const unsigned *prims,
                             unsigned n_prims, const float *margin,
                             float extrapolate, unsigned *out_node,
                             float *out_box, unsigned *out_keys);

/* Stable radix sort of n (key, value) pairs by the low key_bits bits, standing
 * in for kernels::radix_sort_pairs (crates/ppf-cts-solver/src/cpp/kernels/
 * radix_sort.cu:126-159). Host memory in, host memory out. Returns 0, a set of
 * device status bits, or -1 on a CUDA error. */
int ppf_radix_sort_host(unsigned *keys, unsigned *vals, unsigned n,
                        int key_bits);

/* Same sort on device memory, asynchronous on `stream`; scratch is allocated
 * by the library on first use and kept. Returns 0, or -1 on a CUDA error at
 * launch. The sort's own status (a look-back wait that ran out, which leaves
 * the pairs unsorted) is reset at the start of every call and read with
 * ppf_radix_sort_device_status. */
int ppf_radix_sort_device(unsigned *d_keys, unsigned *d_vals, unsigned n,
                          int key_bits, void *stream);

/* Status bits of the last ppf_radix_sort_device call ordered before this one
 * on `stream`. Waits for the stream, then returns 0 (sorted) or a set of
 * device status bits (1: a look-back wait ran out; the pairs are not
 * sorted), or -1 on a CUDA error. */
int ppf_radix_sort_device_status(void *stream);

/* The same sort with no allocation at all. It has no counterpart in the
 * reference. Its scratch (two ping-pong arrays, look-back words, histograms,
 * counters, a status word) lives in static device arrays sized for at most
 * PPF_NOALLOC_SORT_MAX_PAIRS pairs (about 8.5 MB per device). It is for
 * callers that must not allocate: a per-frame loop where a cudaMalloc /
 * cudaFree would synchronize the device, or a host whose allocator owns the
 * device memory.
 *   - The static scratch is reserved when the library's device code is
 *     loaded on a device. Under lazy module loading (CUDA_MODULE_LOADING=LAZY,
 *     the CUDA 12+ default) that happens at the first call on each device,
 *     which can fail when the host's pool already owns the device memory. A
 *     caller that must not allocate later makes one warm-up call at its own
 *     initialisation, for example with n = 0: that call performs the set-up
 *     below and sorts nothing.
 *   - n > PPF_NOALLOC_SORT_MAX_PAIRS: returns -2, prints one line to stderr
 *     and touches nothing.
 *   - The first call on each device looks up the scratch addresses
 *     (cudaGetSymbolAddress) with that device current; make it before any
 *     stream capture begins. Concurrent first calls from several host
 *     threads are safe (the set-up runs once per device).
 *   - Every call resets the status word, histograms, counters and look-back
 *     words it uses on `stream`; nothing needs zeroing by the caller.
 *   - There is one scratch set per device: calls that overlap in time (on any
 *     streams) race on it, so the caller orders them.
 * Asynchronous on `stream`: the result is ready once the stream is. A
 * look-back wait that runs out leaves the pairs unsorted and is reported by
 * ppf_radix_sort_noalloc_status, not by this return code. */
#define PPF_NOALLOC_SORT_MAX_PAIRS (1u << 20)
int ppf_radix_sort_device_noalloc(unsigned *d_keys, unsigned *d_vals,
                                  unsigned n, int key_bits, void *stream);

/* Status bits of the last ppf_radix_sort_device_noalloc call ordered before
 * this one on `stream` (the current device's static status word). Waits for
 * the stream, then returns 0 (sorted), 1 (a look-back wait ran out: the pairs
 * are not sorted), or -1 on a CUDA error. Allocates nothing. The next sort
 * on the device resets the word, so read it before the next call. */
int ppf_radix_sort_noalloc_status(void *stream);

/* ---- per-step statistics ------------------------------------------------
 * The reference logs these per step through SimpleLog channels (newton_steps,
 * pcg_iter, pcg_linsolve, toi: crates/ppf-cts-solver/src/cpp/main/main.cu:
 * 1090-1111, 1354, 1547-1560); here they are returned to the host. */
#define PPF_STATS_MAX_SOLVES 256
typedef struct {
    unsigned newton_iters;     /* Newton iterations of the last advance() */
    unsigned pcg_iters_total;  /* PCG iterations summed over its solves */
    unsigned pcg_solves;
    float pcg_ms_total;        /* device time of the PCG solves */
    float step_ms;             /* host wall time of advance() */
    unsigned max_contacts;     /* largest active contact count of the step */
    unsigned max_dyn_blocks;   /* largest number of contact-only blocks */
    float pcg_ms[PPF_STATS_MAX_SOLVES];
    unsigned pcg_iters[PPF_STATS_MAX_SOLVES];
    float toi[PPF_STATS_MAX_SOLVES];
    /* sizes of the operator each solve ran on: unique upper-triangle blocks
     * of the fixed pattern (diagonal included), vertices, and the unique
     * contact blocks outside the pattern per solve */
    unsigned fixed_blocks;
    unsigned vertices;
    unsigned dyn_blocks[PPF_STATS_MAX_SOLVES];
    /* the preconditioner of the step's solves (PPF_PRECOND_*), how many of
     * its solves fell back to block-Jacobi, and the iterations the factored
     * preconditioner ran (included in pcg_iters_total and pcg_iters) */
    unsigned precond_kind;
    unsigned fallbacks;
    unsigned factor_iters_total;
    /* the last solve's verdict: state (0 converged, 1 truncated, 2 failed),
     * break cause (0 none, 1 negative curvature, 2 r^T z <= 0, 3 curvature
     * within round-off), relative residual at return, the offending value */
    int last_pcg_state;
    int last_break_cause;
    float last_pcg_resid;
    float last_break_val;
} PpfStepStats;
void ppf_step_stats(PpfStepStats *out);

/* ---- preconditioner --------------------------------------------------------
 * The reference's PCG uses block-Jacobi (solver/solver.cu:357-400), the
 * default here. The factored kinds use P = G^T G + eps D^{-1} with G block
 * lower-triangular on the operator's own pattern (D: the diagonal blocks):
 *   PPF_PRECOND_FIRST_ORDER  G from the block-Jacobi-normalised operator,
 *                            G = I - param * (strict lower part); param 0.5
 *   PPF_PRECOND_LEARNED      G emitted by the message-passing network whose
 *                            weights ppf_set_learned_weights loaded
 *   PPF_PRECOND_FSAI         the factorised sparse approximate inverse
 *                            (Kolotilina-Yeremin) on each row's strongest 15
 *                            lower neighbours: (G A G^T)(i, i) = I and
 *                            (G A)(i, j) = 0 on the row's pattern
 * These kinds have no counterpart in the reference. A factored solve runs to the same relative residual with at most as many
 * iterations as the last block-Jacobi solve took; when it stalls or reaches
 * that count, the Newton iteration solves again with block-Jacobi from the
 * same start (the first solve of a session is block-Jacobi, which sets the
 * count). Returns 0, or -1 for an unknown kind or a learned kind without
 * weights. */
#define PPF_PRECOND_BLOCK_JACOBI 0
#define PPF_PRECOND_FIRST_ORDER 1
#define PPF_PRECOND_LEARNED 2
#define PPF_PRECOND_FSAI 4
int ppf_set_preconditioner(int kind, float param);
/* ---- learned preconditioner -------------------------------------------------
 * The reference has no learned preconditioner; these entry points have no
 * counterpart in it. A message-passing network (hidden width 32, bf16 weights,
 * fp32 accumulation) over the Newton system's own sparsity emits the factor G
 * of PPF_PRECOND_LEARNED: in the block-Jacobi-normalised operator
 * Â = C^-1 A C^-T (A(i,i) = C(i) C(i)^T), G(i,i) = d_i C(i)^-1 and
 * G(hi,lo) = -alpha_e Â(hi,lo) C(lo)^-1 per matrix edge. The weights are one
 * flat bf16 blob of PPF_LEARNED_WEIGHTS values (row-major [out][in] layers:
 * W0 32x16, W1..W3 32x80, Wh 80x48, Wf 32x16, wo 48).
 *
 * Loads the weights (host memory, bf16 bit patterns). Returns 0, or -1 when
 * count != PPF_LEARNED_WEIGHTS. */
#define PPF_LEARNED_WEIGHTS 12592
int ppf_set_learned_weights(const unsigned short *bf16, unsigned count);

/* Training on the device. A sample is one Newton system as the solver dumps
 * it (ppf_debug_system after ppf_debug_newton_system): the fixed pattern's
 * upper CSR (n + 1 offsets, columns, 9 column-major floats per block, the
 * diagonal blocks included), the contact blocks' upper CSR (offsets may be
 * NULL for none), the Dirichlet mask and the vertex masses
 * (ppf_debug_vertex_info). It is copied to the device and kept. Returns the
 * sample's index, or -1 for an invalid system. */
int ppf_learned_add_sample(unsigned n, const unsigned *f_off, const unsigned *f_col,
                           const float *f_val, const unsigned *c_off,
                           const unsigned *c_col, const float *c_val,
                           const unsigned *dof_mask, const float *mass);
void ppf_learned_clear_samples(void);
/* n, edges (upper entries of both parts: the length of h_alpha below) and
 * free vertices of a sample; -1 for an unknown index. */
int ppf_learned_sample_info(int sample, unsigned *n, unsigned *edges,
                            unsigned *n_free);
/* The network on a sample with device weights (16-byte aligned): alpha per
 * upper entry (fixed entries first, then contact ones; 0 where the entry is
 * diagonal or touches a Dirichlet vertex) and the head output q per vertex
 * (d = exp(clamp(q, -4, 4))), into host arrays (either may be NULL). */
int ppf_learned_forward(int sample, const void *d_weights, float *h_alpha,
                        float *h_q);
/* Kaporin's condition number of M = Ĝ Â Ĝ^T as the training loss,
 *   L = ln(tr(M) / N) - (1/N) ln det(Ĝ)^2,  N = 3 (free vertices),
 * with tr(M) estimated by n_probes probe vectors (d_probes: n_probes x n x 3
 * floats, +-1, on the device), and its gradient with respect to the weights
 * (d_grad: PPF_LEARNED_WEIGHTS floats on the device, overwritten). Runs on
 * `stream` and waits for it; writes the loss to *h_loss. Returns 0 or -1. */
int ppf_learned_loss_grad(int sample, const void *d_weights, const float *d_probes,
                          unsigned n_probes, float *d_grad, float *h_loss,
                          void *stream);

/* The network's forward layers run on the tensor cores either as tcgen05
 * tiles (M = 128, accumulator in tensor memory; tc = 1) or as mma.sync tiles
 * (tc = 0); tc = -1 only reads the setting. Returns the previous setting.
 * ppf_learned_tc_status is nonzero once a tcgen05 tile gave up waiting for its
 * accumulator (bounded wait; its outputs are then not written). */
int ppf_learned_tensor_path(int tc);
unsigned ppf_learned_tc_status(void);

/* Reported by PpfStepStats.precond_kind when the scene's ParamSet asks for the
 * reference's aggregate additive-Schwarz preconditioner (precond == 1,
 * schwarz/schwarz.hpp:38-86). */
#define PPF_PRECOND_SCHWARZ 3

/* ---- batched PCG ------------------------------------------------------------
 * Many independent Newton systems (one per scene of a batch of uneven scenes)
 * solved by the reference's block-Jacobi PCG (solver/solver.cu:357-400,
 * 431-571, 1002-1278; x0 = 0, relative L1 residual tol, the same check
 * schedule and curvature verdict) in ONE launch: one 512-thread CTA (or a
 * cluster of them) per system with block barriers only, so each system stops on its own iteration
 * count. No counterpart in the reference, which solves one scene per process.
 *   row_off   n_sys + 1 vertex-row offsets: system s owns rows
 *             [row_off[s], row_off[s+1])
 *   off, col, val   both-triangle block rows over all rows (off: rows + 1;
 *             col: the global row of each block's column, inside the same
 *             system; val: 9 column-major floats per block)
 *   rhs       3 floats per row
 *   precond   PPF_PRECOND_BLOCK_JACOBI (the reference's), or PPF_PRECOND_FSAI:
 *             each system's FSAI factor (each row's 15 strongest lower
 *             couplings; rows sorted by column required), built on the device
 *             in the timed region, applied as P = G^T G + 1e-3 D^{-1}
 *   one_by_one  nonzero: one launch per system instead (for comparison)
 * A system's team is one CTA or a thread-block cluster of 2 to 16 CTAs,
 * chosen by its size bucket (ppf_batch_team_ctas); systems of one team size
 * share one launch, the launches run on concurrent streams.
 * Host memory in and out (any output may be NULL): x (3 per row), the
 * iterations, relative residual and state (0 converged, 1 truncated, 2
 * failed) per system, and the device time of the launch(es) in ms.
 * Returns 0, or -1 for an invalid batch (a column outside its system's rows
 * included). */
int ppf_batch_pcg(unsigned n_sys, const unsigned *row_off, const unsigned *off,
                  const unsigned *col, const float *val, const float *rhs,
                  float tol, unsigned max_iter, int precond, int one_by_one,
                  float *x_out,
                  unsigned *iters_out, float *resid_out, int *state_out,
                  float *ms_out);
/* The team size (CTAs; 1, 2, 4, 8 or 16) of each of the 5 system-size
 * buckets: at most 1024, 2048, 4096, 8192 rows, and more. set = 0 reads the
 * table into table[5], set != 0 replaces it (-1 for a size not listed).
 * Defaults: 1, 1, 8, 8, 8. */
int ppf_batch_team_ctas(unsigned *table, int set);
/* The autotuner of the batched PCG: for every size bucket present in the
 * batch (layout as ppf_batch_pcg), solves all of the bucket's systems in one
 * launch with teams of 1, 2, 4, 8 and 16 CTAs (sizes that would leave half
 * the team idle on the bucket's largest system, and cluster sizes the device
 * cannot schedule, are skipped), three times each, and keeps the fastest in
 * the table that ppf_batch_pcg uses. Writes
 * the table to table_out[5] and the best time of each (bucket, size) to
 * ms_out[5 * 5] (-1 where not tried; both may be NULL). Returns 0 or -1. */
int ppf_batch_autotune(unsigned n_sys, const unsigned *row_off, const unsigned *off,
                       const unsigned *col, const float *val, const float *rhs,
                       float tol, unsigned max_iter, unsigned *table_out,
                       float *ms_out);

/* The Schwarz aggregation on the host (schwarz/schwarz.cu:551-645): the graph
 * as a both-triangle CSR (n + 1 offsets, columns, one weight per entry: the
 * Frobenius norm of the block), aggregates of at most kmax matrix-connected
 * vertices grown greedily by the heaviest coupling, seeds in decreasing order
 * of summed coupling. Writes the aggregate of each vertex to agg (n) and
 * returns the number of aggregates. */
unsigned ppf_schwarz_aggregate(unsigned n, const unsigned *off, const unsigned *col,
                               const float *wgt, unsigned kmax, unsigned *agg);
/* The Schwarz coarse level on the host (the reference's two-level form,
 * schwarz/schwarz.cu:1225-1327 and 1416-1470): for the same CSR with the 9
 * values of every block (column-major, 9 floats per entry) and the
 * aggregation agg (n entries, n_agg aggregates), the Galerkin blocks of
 * distinct aggregate pairs summed in float32 (rows in order, each row's
 * entries in order), grouped by the aggregation above with their Frobenius
 * norms as weights. Writes the domain of each aggregate to dom (n_agg) and
 * returns the number of domains. */
unsigned ppf_schwarz_coarsen(unsigned n, const unsigned *off, const unsigned *col,
                             const float *blocks, const unsigned *agg, unsigned n_agg,
                             unsigned kmax, unsigned *dom);

/* The project's autotuner for the traversal kernels (no counterpart in the
 * reference). Each of the six traversal kernels (vertex and edge proximity
 * detection, vertex, collision-mesh vertex and edge CCD, the intersection
 * check) tests the leaves its stackless walk reaches either in warp rounds
 * (0: the leaves the lanes found are tested together) or on the spot (1).
 * Both forms find the same pairs and times of impact; which is faster depends
 * on the scene. ppf_autotune times both forms of each on the initialized
 * scene's current state (three runs each, the minimum kept: detection at the
 * positions, the CCD over the inertial step, the intersection check), keeps
 * the faster and writes the six choices to modes (may be NULL); it returns
 * 0, or -1 on a fatal error. ppf_get_tuning / ppf_set_tuning read and set
 * the six choices (set returns -1 for a value other than 0 or 1). Defaults:
 * 0 1 0 0 0 0. */
int ppf_autotune(unsigned char *modes);
/* The PCG's team. Each solve is one persistent launch: over the whole grid
 * (one 1024-thread block per SM, a cooperative launch whose two reductions
 * per iteration meet at grid barriers through L2), or as one thread-block
 * cluster of up to 16 CTAs, whose hardware barrier stands for the grid
 * barrier. A small system's iterations are bound by those reductions, so it
 * solves faster on one cluster. ppf_set_pcg_team(-1) (the default) picks one
 * cluster of the largest size the device runs for scenes up to 16,384
 * vertices and the whole grid above, at each initialize; 0 sets the whole
 * grid; 2 to 16 one cluster of that many CTAs (returns -1 for a size the
 * device cannot run). ppf_autotune also times the whole grid against the
 * largest cluster and half of it on the current Newton system and keeps the
 * fastest. ppf_pcg_team returns the current team (0: the whole grid). */
int ppf_set_pcg_team(int ctas);
int ppf_pcg_team(void);
/* The share of a PCG product phase's work, in sixteenths of its estimated
 * cost, that is split into one contiguous range per block; the rest is a
 * common pool taken by whichever warps finish first. 0 restores the default
 * (12); returns -1 above 16. */
int ppf_set_pcg_static_share(unsigned sixteenths);
/* Threads per CTA of a one-cluster block-Jacobi solve: 256, 512 or 1024; 0
 * (the default) picks 512 up to 6,144 vertices and 1024 above, at each
 * initialize. Smaller CTAs let several solves share an SM. Returns -1 for
 * another value. */
int ppf_set_pcg_cta_threads(unsigned threads);
void ppf_get_tuning(unsigned char *modes);
int ppf_set_tuning(const unsigned char *modes);
/* The CUDA stream (cudaStream_t, as void*) every kernel of advance() runs
 * on, so a host can time the step with its own events on that stream. NULL
 * before initialize(). */
void *ppf_stream(void);
/* Number of kernels this library has launched since it was loaded (the
 * kernels of a replayed CUDA graph count each time). */
unsigned long long ppf_kernel_launches(void);
/* Launches of a CUDA graph that holds a Newton iteration's line-search stage
 * (the rescaled step, the swept-box refits, the contact and strain-limit line
 * searches and the status copy): the whole-iteration graph below, or, for an
 * iteration that runs outside it, a graph of that stage alone. No counterpart
 * in the reference (which captures its PCG iteration,
 * solver/solver.cu:1195-1244). */
unsigned long long ppf_graph_launches(void);
/* The whole Newton iteration as one CUDA graph: status reset, assembly
 * (elastic terms, detection, contact blocks, the PCG's operator layout and
 * preconditioner), the PCG solve, the line search and the status copy, with
 * no read-back until the status copy. Its launches are sized by capacities
 * (the pair lists and a contact-block capacity) and read the counts on the
 * device; an iteration whose counts overran a capacity changes nothing and
 * is repeated after the host grows it. The first iteration under a new
 * capture key (scene, parameters but the clock, capacities, device buffers)
 * runs its launches directly, the next captures them, later ones replay the
 * graph. It serves block-Jacobi and (once its layout is set up) Schwarz
 * solves; the factored preconditioners size their builds on the host and run
 * outside it. On by default; ppf_set_iteration_graph(0) turns it off (the
 * assembly then reads the counts back and sizes to them, and the line-search
 * stage alone is a graph). ppf_iteration_graph_stats writes four counts since
 * the library was loaded: iterations run directly, graphs captured, graph
 * replays, iterations repeated after an overrun. */
void ppf_set_iteration_graph(int enable);
void ppf_iteration_graph_stats(unsigned long long *out);
/* ---- many scenes stepped together -------------------------------------------
 * No counterpart in the reference, whose backend holds one scene per process.
 * ppf_multi_create initializes one solver per scene (its own stream, device
 * buffers and Newton-iteration graph; datasets[i] and params[i] stay owned by
 * the caller and must outlive the handle), `threads` host threads at a time.
 * ppf_multi_advance steps every scene by one time step (advance()), the
 * scenes taken by the host threads as they come free, so their launches
 * overlap on the device; results may be NULL. A scene up to 16,384 vertices
 * solves its PCG on one cluster sized to it (2 to 16 CTAs of 512 threads; set
 * per scene with ppf_multi_set_pcg_team and ppf_multi_set_pcg_cta_threads, as
 * their single-scene forms). The others mirror
 * update_constraint, fetch and ppf_step_stats for scene i. Each
 * returns 0, or -1 on a fatal error (ppf_fatal_code / ppf_fatal_detail; the
 * handle of a failed create is NULL). The single-scene entry points keep
 * their own solver. */
typedef struct PpfMulti PpfMulti;
PpfMulti *ppf_multi_create(unsigned count, PpfDataSet *const *datasets,
                           PpfParamSet *const *params, unsigned threads);
int ppf_multi_advance(PpfMulti *m, PpfStepResult *results);
int ppf_multi_update_constraint(PpfMulti *m, unsigned i, const PpfConstraint *constraint);
int ppf_multi_fetch(PpfMulti *m, unsigned i);
int ppf_multi_step_stats(PpfMulti *m, unsigned i, PpfStepStats *out);
int ppf_multi_set_pcg_team(PpfMulti *m, unsigned i, int ctas);
int ppf_multi_set_pcg_cta_threads(PpfMulti *m, unsigned i, unsigned threads);
int ppf_multi_pcg_team(PpfMulti *m, unsigned i);
void ppf_multi_destroy(PpfMulti *m);
/* Debug: caps the pair lists at pair_cap entries each and the iteration
 * graph's contact-block capacity at block_cap (0 leaves one as it is), to
 * exercise the overrun-and-repeat path. The capacities grow again as counts
 * require. */
void ppf_debug_set_contact_capacity(unsigned pair_cap, unsigned block_cap);
/* Bytes copied host -> device and device -> host by the library since it was
 * loaded, counted at the copies of the per-step path: update_constraint's
 * uploads, the status and count reads inside advance(), intersection
 * records and fetch(). No counterpart in the reference. Either pointer may
 * be NULL. */
void ppf_transfer_bytes(unsigned long long *h2d, unsigned long long *d2h);

/* ---- stage inspection (parity checks) -------------------------------------
 * Assembles and solves the first Newton system of a step at the current
 * state (what advance() does before its first line search, main.cu:683-1120),
 * writes the solution dx (3n floats) and keeps host copies of the system for
 * ppf_debug_system. Returns the PCG state: 0 converged, 1 truncated, 2 failed. */
int ppf_debug_newton_system(float *dx, unsigned *iters, float *resid);
/* sizes[6]: fixed blocks, contact blocks, point-face, point-edge, point-point
 * and edge-edge pairs of the system kept by ppf_debug_newton_system. */
void ppf_debug_system_sizes(unsigned *sizes);
/* Copies the kept system: fixed pattern (n+1 offsets, columns, 9 floats per
 * block, per-vertex diagonal already folded in), contact blocks (offsets,
 * columns, values), the per-vertex diagonal (9n), the right-hand side (3n)
 * and the pair lists (pf: 2 u32, pe / pp: 3 u32 with the multiplicity and the
 * friction flag in bit 31, ee: 2 u32 per pair). Any pointer may be NULL. */
void ppf_debug_system(unsigned *f_off, unsigned *f_col, float *f_val,
                      unsigned *d_off, unsigned *d_col, float *d_val,
                      float *diag, float *force, unsigned *pf, unsigned *pe,
                      unsigned *pp, unsigned *ee);
/* The vertex masses (n floats) and Dirichlet mask (n u32, nonzero = pinned)
 * of the initialized scene, and the diagonal blocks G(i,i) (9n floats,
 * column-major) of the last factor a factored preconditioner built. */
void ppf_debug_vertex_info(float *mass, unsigned *dof_mask);
void ppf_debug_factor_diag(float *out);
/* Solves the operator of the last ppf_debug_newton_system, with the same
 * preconditioner, for the right-hand side b (3n floats) from x = 0 with at
 * most max_iter iterations; writes x (3n floats). With max_iter = 1,
 * x = alpha P b: the direction of the preconditioner's first output.
 * Returns the PCG state. */
int ppf_debug_pcg(const float *b, float *x, unsigned max_iter, unsigned *iters, float *resid);
/* The contact line search (contact.cu:2472-2740: vertex, edge and
 * collision-mesh CCD over trees swept from x0 to x1, 3n floats each) on the
 * initialized scene: the fraction of x1 - x0 it admits (its time of impact
 * over line_search_max_t); overlap (may be NULL) is set when a pair starts
 * inside its offset. */
float ppf_debug_contact_line_search(const float *x0, const float *x1, unsigned *overlap);
/* The strain-limit line search of faces and rod edges (strainlimiting.cu:
 * 192-305) on the initialized scene, from positions x0 to x1 (3n floats
 * each): the fraction of x1 - x0 it admits (its time of impact divided by
 * line_search_max_t, as the reference returns it). */
float ppf_debug_strain_line_search(const float *x0, const float *x1);
/* The Schwarz layout of the last solve: sizes[3] = {aggregates, coarse
 * domains, levels} (zeros when no Schwarz solve ran), the aggregate of each
 * vertex (n) and the domain of each aggregate (sizes[0], written when there
 * are domains). Either array may be NULL. */
void ppf_debug_schwarz_layout(unsigned *sizes, unsigned *agg, unsigned *dom);

#ifdef __cplusplus
}
#endif

#endif
