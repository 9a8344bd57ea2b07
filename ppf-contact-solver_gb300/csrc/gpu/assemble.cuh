// assemble.cuh -- Newton system assembly stages (launchers).
#pragma once

#include "contact_rules.cuh"

namespace ppf {
namespace gpu {

struct PairLists {
    uint2 *pf = nullptr;  // (vertex, face)
    uint3 *pe = nullptr;  // (vertex, edge, count | friction << 31)
    uint3 *pp = nullptr;  // (vertex, other, count | friction << 31)
    uint2 *ee = nullptr;  // (edge, other edge)
    unsigned cap_pf = 0, cap_pe = 0, cap_pp = 0, cap_ee = 0;
};

struct DynMatrix {
    unsigned long long *hkey = nullptr; // hash table keys (row << 32 | col)
    unsigned *hval = nullptr;           // CSR position of the key's block
    unsigned hcap = 0;                  // power of two
    unsigned *off = nullptr;            // n + 1
    unsigned *col = nullptr;
    float *val = nullptr;               // 9 per block
    unsigned *tr_off = nullptr;         // n + 1
    uint2 *tr = nullptr;                // (row, block index)
    unsigned *cnt = nullptr;            // n scratch
    unsigned *cnt2 = nullptr;           // n scratch
    unsigned cap = 0;
};

struct AssemblyBuffers {
    float *force;       // 3n
    float *diag;        // 9n
    float *fixed_val;   // 9 B_u
    float *fixed_tmp;   // 9 B_u (elastic-only copy, read by stiffness terms)
    const float *x;     // eval_x
    const float *x0;    // vertex.curr (start of step)
    const float *target;
    IterStatus *st;
    const StepParams *params; // device copy of the step's parameters
};

void launch_vertex_energy(const Scene &s, const AssemblyBuffers &b,
                          cudaStream_t q);
void launch_elastic(const Scene &s, const AssemblyBuffers &b,
                    cudaStream_t q);
void launch_strain_limit(const Scene &s, const AssemblyBuffers &b,
                         cudaStream_t q);
// Per-edge piece counts for split edge queries (see contact_rules.cuh).
struct PieceBuffers {
    unsigned *count;    // E
    unsigned *off;      // E + 1
    unsigned *scan_tmp; // scan_tmp_size(E + 1)
};
void launch_edge_pieces(const Scene &s, const BvhView &eb, const float *x, const float *x1,
                        const unsigned *t_bits, float piece_len, PieceBuffers &pb,
                        cudaStream_t q);
// Grid of a launch over edge pieces: one thread per edge plus slack for the
// extra pieces; the kernels loop over any remainder.
unsigned piece_grid(unsigned ne, unsigned block);
void launch_detect(const Scene &s, const BvhView &fb, const BvhView &eb,
                   const BvhView &vb, const AssemblyBuffers &b, PairLists &pl,
                   const PieceBuffers &pb, cudaStream_t q);
// Dedupes the contact blocks outside the fixed pattern, lays them out and
// zeroes their values. The pair counts are read on the device (clamped to
// the lists' capacities); `bound` is an upper bound of each count (the
// counts themselves, or the capacities) that only sizes the grids.
void launch_dyn_build(const Scene &s, const AssemblyBuffers &b, const PairLists &pl,
                      const unsigned bound[4], DynMatrix &dm, unsigned *d_scan_tmp,
                      cudaStream_t q);
// Sets STATUS_PAIR_OVERFLOW when detection found more pairs than a list holds.
void launch_pair_capacity(const PairLists &pl, IterStatus *st, cudaStream_t q);
void launch_contact_assemble(const Scene &s, const AssemblyBuffers &b, const PairLists &pl,
                             const unsigned bound[4], DynMatrix &dm, cudaStream_t q);
void launch_vertex_constraints(const Scene &s, const AssemblyBuffers &b, cudaStream_t q);
// Contacts against the static collision mesh (contact/contact.cu:1834-1947);
// fb is the free faces' tree of this Newton iteration.
void launch_collision_mesh(const Scene &s, const AssemblyBuffers &b,
                           const BvhView &fb, cudaStream_t q);
void launch_dirichlet(const Scene &s, const AssemblyBuffers &b, const DynMatrix &dm,
                      float *dx, cudaStream_t q);
// Exclusive scan of n u32 into out (n + 1 entries, out[n] = total).
void exclusive_scan(const unsigned *in, unsigned *out, unsigned n, unsigned *tmp,
                    cudaStream_t q);
size_t scan_tmp_size(unsigned n);

} // namespace gpu
} // namespace ppf
