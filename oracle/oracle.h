/*
 * oracle.h -- CPU oracle for the per-step contact solve (TEST INFRASTRUCTURE).
 *
 * A serial C++ restatement of the reference's algorithm for this path, used
 * only as the checker: by tests/, by __graft_entry__.smoke() and by bench.py's
 * CPU-baseline arm. The product library never links, loads or calls it.
 *
 * Parity pinning: the element-level formulas the oracle evaluates (barrier,
 * friction, Baraff-Witkin, dihedral bending, distances, additive CCD, eigen
 * solves) are checked against the reference's own header code compiled from
 * its sources (oracle/Makefile -> oracle/_ref/libppfref.so) and frozen as
 * golden vectors in tests/golden/. The pipeline around them (LBVH, stable sort,
 * Karras topology, traversal, pair rules, sparse assembly, block-Jacobi PCG,
 * line search, Newton control) is restated here from the reference sources
 * cited at each function.
 */
#ifndef PPF_ORACLE_H
#define PPF_ORACLE_H

#include "../include/ppf_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

/* LBVH of one primitive set (crates/ppf-cts-solver/src/cpp/lbvh/lbvh.cu).
 * Same argument meaning as ppf_lbvh_build_host in the product library.
 * Returns the root node index. */
unsigned oracle_lbvh_build(int kind, const float *x0, const float *x1,
                           unsigned n_verts, const unsigned *prims,
                           unsigned n_prims, const float *margin,
                           float extrapolate, unsigned *out_node,
                           float *out_box, unsigned *out_keys);

/* Stable sort of (key, value) pairs by the low key_bits bits
 * (kernels/radix_sort.cu:126-159 semantics). */
void oracle_stable_sort(unsigned *keys, unsigned *vals, unsigned n,
                        int key_bits);

#ifdef __cplusplus
}
#endif

#endif
