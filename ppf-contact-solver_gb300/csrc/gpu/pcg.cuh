// pcg.cuh -- block-Jacobi preconditioned CG on the assembled Newton system.
//
// Restates crates/ppf-cts-solver/src/cpp/solver/solver.cu:
//   block-Jacobi inverse (floored eigendecomposition)   357-400
//   seeded residual r = b - A x0, L1 norm err0          1014-1035
//   curvature verdict on p^T A p vs 256 eps sum|terms|  66-114, 804-884
//   recurrence, beta = rz1 / rz0, p = z + beta p        431-571, 1099-1169
//   convergence err / err0 < tol, checked at iterations 1, 5, 9, ... and at
//   every iteration once err / err0 < 8 tol             987-988, 1267-1379
// as ONE persistent cooperative launch per solve: every scalar (alpha, beta,
// the check schedule, the verdicts) is computed on the device by every block
// from the same fixed-order reduction, and the host reads the result once.
//
// Operator layout (SELL-32): rows are cut into slices of 32; slice s owns
// slots [off[s], off[s+1]); slot k of lane l holds one 3x3 block of row
// 32 s + l with its column index. Values are stored entry-major per slot,
// val[(slot * 9 + e) * 32 + lane] (e = column-major entry of the block), so
// a warp reads each entry of 32 rows' blocks as one 128-byte line. Both
// triangles are stored: row i carries A(i, j) for every j, so a row's
// product needs no atomics and no transposed gathers. Unused slots hold a
// zero block pointing at the row itself.
#pragma once

#include <vector>

#include <cuda_bf16.h>

#include "radix_sort.cuh"
#include "scene.cuh"

namespace ppf {
namespace gpu {

constexpr unsigned kSliceRows = 32;

struct SellMatrix {
    unsigned n_slices;
    const unsigned *slice_off; // n_slices + 1, in slots
    const unsigned *col;       // 32 per slot
    const float *val;          // 9 x 32 per slot
    // null, or per slice the first slot of its upper segment: each row's
    // blocks left of the diagonal sit in [slice_off, slice_mid), the
    // diagonal block and those right of it in [slice_mid, slice_off + 1)
    const unsigned *slice_mid;
};

// Entries of contact rows longer than the contact slices' cap: one row per
// work item, processed by a whole warp.
struct OverflowRows {
    unsigned count;          // rows with overflow
    const unsigned *row;     // count: vertex of each
    const uint2 *range;      // count: (first entry, entries)
    const unsigned *col;     // entries
    const float *val;        // 9 per entry, column-major block
    const unsigned *index;   // n: overflow row of each vertex, or 0xffffffff
};

// Contact part: only the rows that have contact blocks, in a stable order of
// decreasing block count, cut into SELL-32 slices over that order (lane l of
// slice s is row perm[32 s + l]), so rows of like length share a slice.
struct ContactRows {
    unsigned rows;          // rows with contact blocks (an upper bound when sizes is set)
    SellMatrix sell;        // n_slices = ceil(rows / 32)
    const unsigned *perm;   // sorted position -> row
    const unsigned *index;  // n: row -> sorted position, or 0xffffffff
    // null, or the device's {rows, overflow rows}: the PCG's task kernels
    // read these, so the host fields above need only bound them
    const unsigned *sizes;
};

typedef __nv_bfloat16 bf16_t;

// Factored preconditioner P = G^T G + eps D^{-1} (D^{-1}: the block-Jacobi
// inverse), G block lower-triangular on the operator's own pattern. Its
// slot values are bf16 (both slots of an edge round the same value, so P
// stays symmetric positive definite) in arrays parallel to the operator's
// value arrays: the slot of
// row a, column b holds G(a, b) when b < a and G(b, a)^T when b > a, so
// y = G r walks the slots below the diagonal and z = G^T y the slots above
// it. The diagonal blocks G(a, a) are kept apart, 9 floats per vertex
// (column-major). Slots touching a Dirichlet vertex hold zero blocks.
struct PcgFactor {
    const bf16_t *fixed;   // as SellMatrix::val of the fixed part
    const bf16_t *contact; // as the contact part's SellMatrix::val
    const bf16_t *ovf;     // as OverflowRows::val
    const float *diag;    // 9 per vertex; null: block-Jacobi only
    float eps;
};

constexpr unsigned kSchwarzMaxMembers = 16; // vertices per Schwarz aggregate

// Aggregate additive-Schwarz preconditioner (schwarz.cuh); n_agg == 0 when
// unused. Aggregate g holds members[agg_off[g] .. agg_off[g+1]) and its
// factor G = L^{-1} packed row-major lower-triangular at ainv + ainv_off[g].
// With the coarse level (n_dom > 0) the aggregates are the coarse nodes:
// domain D holds the nodes dom_members[dom_off[D] .. dom_off[D+1]) and the
// packed factor of its Galerkin block at ainv1 + ainv1_off[D]; rc holds the
// restricted residual, one float4 per aggregate; weight damps the coarse
// correction.
struct SchwarzView {
    unsigned n_agg;
    const unsigned *agg_off, *members, *ainv_off;
    const float *ainv;
    unsigned n_dom;
    const unsigned *dom_off, *dom_members, *ainv1_off;
    const float *ainv1;
    float4 *rc;
    float weight;
};

// A = fixed part (elastic + inertia + per-vertex terms, diagonal included)
// + contact part (blocks outside the fixed pattern: sorted contact rows up to
// a width cap, plus overflow rows).
struct PcgOperator {
    unsigned n;
    SellMatrix fixed;
    ContactRows contact;
    OverflowRows ovf;
    const float *inv_diag; // block-Jacobi inverse, (slice * 9 + e) * 32 + lane
    PcgFactor factor;      // factor.diag == null: P = block-Jacobi
    SchwarzView schwarz;   // n_agg > 0: P = aggregate Schwarz (factor unused)
};

struct PcgResult {
    unsigned iter;
    float resid;     // err / err0 at return
    int state;       // 0 converged, 1 truncated (success), 2 failed
    int break_cause; // 0 none, 1 negative curvature, 3 unresolvable curvature
    float err0;
    float break_val;
    unsigned status;
};

struct PcgWorkspace {
    DevBuf<float> R;               // {z, p} record per vertex (8 floats)
    DevBuf<float4> p, Ap;          // one float4 per vertex
    DevBuf<float4> Ap_ovf;         // one per overflow row
    DevBuf<float4> Ap_c;           // one per contact row (sorted position)
    DevBuf<float4> Y;              // G r of the factored preconditioner
    DevBuf<unsigned> task_cost, task_off, task_start, scan_tmp, dyn_ctr;
    DevBuf<float> partials;
    DevBuf<unsigned> barrier;
    DevBuf<PcgResult> result;
    unsigned grid = 0, threads = 0;
    // 0: each solve runs on the whole grid (one block per SM, grid-wide
    // barriers through L2); 2 to max_cluster: on one thread-block cluster of
    // that many CTAs, whose hardware barrier stands for the grid barrier
    unsigned cluster = 0, max_cluster = 0;
    // threads per CTA of a one-cluster block-Jacobi solve (256, 512 or
    // 1024; 0: 1024): smaller CTAs share an SM with other solves'
    unsigned cluster_threads = 0;
    // share of the product work, in sixteenths of its cost, split into the
    // blocks' static ranges (the rest is the common pool); 0: the default 12
    unsigned static_sixteenths = 0;
    void reserve(unsigned n);
};

// ---- SELL layouts ------------------------------------------------------------
// Fixed part: the slot of every (row, block) is static per scene. `src` maps a
// (slot, lane) to the upper-triangle block it copies (bit 31: transposed),
// or 0xffffffff for padding.
struct SellLayout {
    DevBuf<unsigned> slice_off, slice_mid, col, src;
    DevBuf<float> val;
    unsigned n_slices = 0, slots = 0;
};

// Slot source maps (SellLayout::src, DynLayout::ovf_src): the upper block a
// slot copies, with this bit set when the slot holds its transpose (the slot
// lies in the block's column row), or kSlotPad for padding.
constexpr unsigned kSlotTransposed = 0x80000000u;
constexpr unsigned kSlotPad = 0xFFFFFFFFu;

// Contact slices are at most this many slots wide; longer rows continue in
// the overflow rows.
constexpr unsigned kDynSliceCap = 32;

struct DynLayout {
    SellLayout sell; // over the sorted contact rows
    DevBuf<unsigned> key, perm, index, slice_k, row_ovf, row_flag, ovf_off, flag_off;
    DevBuf<unsigned> scan_tmp, counters;
    DevBuf<unsigned> sizes; // {rows, overflow rows, slots, overflow entries}
    DevBuf<unsigned> ovf_row, ovf_col, ovf_index, ovf_src;
    DevBuf<uint2> ovf_range;
    DevBuf<float> ovf_val;
    RadixSortWorkspace sort_ws;
    unsigned rows = 0, n_ovf = 0, ovf_entries = 0;
};

// Host construction of the fixed layout from the upper pattern and its
// transpose table (row, upper slot) per row, in two segments per slice: the
// blocks left of the diagonal (transposed), then the diagonal and the blocks
// right of it, so a triangular product walks one segment only.
void sell_build_fixed(unsigned n, const std::vector<unsigned> &off,
                      const std::vector<unsigned> &col, const std::vector<unsigned> &tr_off,
                      const std::vector<uint2> &tr, SellLayout &out);
// Copies the assembled upper blocks into the fixed layout.
void sell_pack_fixed(SellLayout &L, const float *upper_val, cudaStream_t q);
// Contact part, rebuilt per Newton iteration from the deduplicated upper CSR
// (off, col, val) and its transpose list (tr_off, tr), leaving out the blocks
// of Dirichlet vertices (dof_mask, zero after elimination). Rows are sorted
// by block count with the stable radix sort. The device writes the layout's
// sizes to out.sizes. With block_cap == 0 four totals are read back to the
// host (one synchronization) and the layout is sized to them; otherwise it
// is sized for at most block_cap contact blocks (upper triangle) with no
// read-back, and its host counts are those bounds. A sort time-out or an
// overrun bound empties the layout and sets a bit of *d_status.
void sell_build_dyn(unsigned n, const unsigned *off, const unsigned *col, const float *val,
                    const unsigned *tr_off, const uint2 *tr, const unsigned *dof_mask,
                    DynLayout &out, cudaStream_t q, unsigned block_cap = 0,
                    unsigned *d_status = nullptr);
inline SellMatrix sell_view(const SellLayout &L) {
    return SellMatrix{L.n_slices, L.slice_off.data(), L.col.data(), L.val.data(),
                      L.slice_mid.data()};
}
inline ContactRows contact_view(const DynLayout &D) {
    return ContactRows{D.rows, sell_view(D.sell), D.perm.data(), D.index.data(),
                       D.sizes.data()};
}
inline OverflowRows overflow_view(const DynLayout &D) {
    return OverflowRows{D.n_ovf, D.ovf_row.data(), D.ovf_range.data(), D.ovf_col.data(),
                        D.ovf_val.data(), D.ovf_index.data()};
}

// Diagonal block inverse per row: inv(B(i,i)), written in the slice layout.
void launch_block_jacobi(unsigned n, const float *upper_val, const unsigned *diag_slot,
                         float *inv_diag, unsigned *d_status, cudaStream_t q);

// Solves A x = b starting from x (b in r on entry; r is overwritten).
// Writes the result into ws.result (device) and returns immediately.
// With run_if set, the solve runs only when *run_if is nonzero on the device
// when it starts (otherwise x, r and the result stay as they are).
void launch_pcg(const PcgOperator &A, float *x, float *r, float tol,
                unsigned max_iter, PcgWorkspace &ws, cudaStream_t q,
                const unsigned *run_if = nullptr);

} // namespace gpu
} // namespace ppf
