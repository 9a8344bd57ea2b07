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
 * by the library on first use and kept. */
int ppf_radix_sort_device(unsigned *d_keys, unsigned *d_vals, unsigned n,
                          int key_bits, void *stream);

#ifdef __cplusplus
}
#endif

#endif
