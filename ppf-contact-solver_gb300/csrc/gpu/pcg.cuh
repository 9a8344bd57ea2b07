// pcg.cuh -- block-Jacobi preconditioned CG on the assembled Newton system.
//
// Restates crates/ppf-cts-solver/src/cpp/solver/solver.cu:
//   block-Jacobi inverse (floored eigendecomposition)   357-400
//   seeded residual r = b - A x0, L1 norm err0          1014-1035
//   curvature verdict on p^T A p vs 256 eps sum|terms|  66-114
//   recurrence, beta = rz1 / rz0, p = z + beta p        431-571, 1099-1169
//   convergence err / err0 < tol, checked at iterations 1, 5, 9, ... and at
//   every iteration once err / err0 < 8 tol             987-988, 1267-1379
// as ONE persistent cooperative launch per solve: every scalar (alpha, beta,
// the check schedule, the verdicts) is computed on the device by every block
// from the same fixed-order reduction, and the host reads the result once.
#pragma once

#include "scene.cuh"

namespace ppf {
namespace gpu {

// A = fixed (upper + transpose table, diagonal blocks already include the
// per-vertex diagonal C) + dynamic contact blocks (upper + transpose table).
struct PcgOperator {
    unsigned n;
    const unsigned *f_off, *f_col;
    const float *f_val;
    const unsigned *f_tr_off;
    const uint2 *f_tr;
    const unsigned *d_off, *d_col;
    const float *d_val;
    const unsigned *d_tr_off;
    const uint2 *d_tr;
    const float *inv_diag; // 9 per row
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
    DevBuf<float> z, p, Ap;
    DevBuf<float> partials;
    DevBuf<unsigned> barrier;
    DevBuf<PcgResult> result;
    unsigned grid = 0, threads = 0;
    void reserve(unsigned n);
};

// Diagonal block inverse per row: inv(B(i,i)) with C already folded in.
void launch_block_jacobi(const PcgOperator &A, const unsigned *diag_slot,
                         float *inv_diag, unsigned *d_status, cudaStream_t q);

// Solves A x = b starting from x (b in r on entry; r is overwritten).
// Writes the result into ws.result (device) and returns immediately.
void launch_pcg(const PcgOperator &A, float *x, float *r, float tol,
                unsigned max_iter, PcgWorkspace &ws, cudaStream_t q);

// y = A x (one SpMV, for checks).
void launch_spmv(const PcgOperator &A, const float *x, float *y, cudaStream_t q);

} // namespace gpu
} // namespace ppf
