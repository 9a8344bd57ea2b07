// api_components.cu -- C-ABI entry points for single stages of the solve.
//
// These let a host run one stage (the LBVH build, the radix sort) on the GPU
// with plain pointers, for stage-level parity checks and stage benchmarks.
// They allocate their own device scratch per call.
#include "../../../include/ppf_gb300_ext.h"
#include "fatal.cuh"
#include "lbvh.cuh"

#include <vector>

using namespace ppf;
using namespace ppf::gpu;

namespace {

template <class T> struct HostToDev {
    T *d = nullptr;
    HostToDev(const T *h, size_t n) {
        if (n == 0) return;
        PPF_CUDA(cudaMalloc(&d, n * sizeof(T)));
        if (h) PPF_CUDA(cudaMemcpy(d, h, n * sizeof(T), cudaMemcpyHostToDevice));
    }
    ~HostToDev() {
        if (d) cudaFree(d);
    }
};

struct StatusWord {
    unsigned *d = nullptr;
    StatusWord() {
        PPF_CUDA(cudaMalloc(&d, sizeof(unsigned)));
        PPF_CUDA(cudaMemset(d, 0, sizeof(unsigned)));
    }
    unsigned read() {
        unsigned h = 0;
        PPF_CUDA(cudaMemcpy(&h, d, sizeof(unsigned), cudaMemcpyDeviceToHost));
        return h;
    }
    ~StatusWord() { cudaFree(d); }
};

int report(const FatalError &e) {
    set_fatal(e.code, e.detail.c_str());
    fprintf(stderr, "[ppf_gb300] %s\n", e.detail.c_str());
    return -1;
}

} // namespace

extern "C" unsigned ppf_lbvh_build_host(int kind, const float *x0,
                                        const float *x1, unsigned n_verts,
                                        const unsigned *prims, unsigned n_prims,
                                        const float *margin, float extrapolate,
                                        unsigned *out_node, float *out_box,
                                        unsigned *out_keys) {
    try {
        if (n_prims == 0) return 0u;
        HostToDev<float> dx0(x0, 3 * (size_t)n_verts), dx1(x1, 3 * (size_t)n_verts);
        HostToDev<unsigned> dprims(kind == PRIM_VERTEX ? nullptr : prims,
                                   kind == PRIM_VERTEX ? 0 : (size_t)kind * n_prims);
        HostToDev<float> dmargin(margin, n_prims);
        StatusWord status;
        Lbvh bvh;
        RadixSortWorkspace ws;
        PrimSet ps{(PrimKind)kind, n_prims, dprims.d, dmargin.d, nullptr};
        lbvh_build(bvh, ps, dx1.d, dx0.d, dx1.d, extrapolate, ws, status.d, 0);
        PPF_CUDA(cudaDeviceSynchronize());
        unsigned st = status.read();
        unsigned nn = bvh.nodes();
        if (out_node)
            PPF_CUDA(cudaMemcpy(out_node, bvh.node.data(), nn * sizeof(uint2),
                                cudaMemcpyDeviceToHost));
        if (out_box) {
            std::vector<float4> lo(nn), hi(nn);
            PPF_CUDA(cudaMemcpy(lo.data(), bvh.bmin.data(), nn * sizeof(float4),
                                cudaMemcpyDeviceToHost));
            PPF_CUDA(cudaMemcpy(hi.data(), bvh.bmax.data(), nn * sizeof(float4),
                                cudaMemcpyDeviceToHost));
            for (unsigned i = 0; i < nn; ++i) {
                out_box[8 * i + 0] = lo[i].x;
                out_box[8 * i + 1] = lo[i].y;
                out_box[8 * i + 2] = lo[i].z;
                out_box[8 * i + 3] = lo[i].w;
                out_box[8 * i + 4] = hi[i].x;
                out_box[8 * i + 5] = hi[i].y;
                out_box[8 * i + 6] = hi[i].z;
                out_box[8 * i + 7] = 0.0f;
            }
        }
        if (out_keys && n_prims > 1)
            PPF_CUDA(cudaMemcpy(out_keys, bvh.keys.data(),
                                n_prims * sizeof(unsigned),
                                cudaMemcpyDeviceToHost));
        unsigned root = bvh.root;
        bvh.release();
        ws.release();
        if (st) {
            fprintf(stderr, "[ppf_gb300] lbvh status bits 0x%x\n", st);
            return 0xffffffffu;
        }
        return root;
    } catch (const FatalError &e) {
        report(e);
        return 0xffffffffu;
    }
}

extern "C" int ppf_radix_sort_host(unsigned *keys, unsigned *vals, unsigned n,
                                   int key_bits) {
    try {
        if (n == 0) return 0;
        HostToDev<unsigned> dk(keys, n), dv(vals, n);
        StatusWord status;
        RadixSortWorkspace ws;
        radix_sort_pairs(dk.d, dv.d, n, key_bits, ws, status.d, 0);
        PPF_CUDA(cudaDeviceSynchronize());
        PPF_CUDA(cudaMemcpy(keys, dk.d, n * sizeof(unsigned),
                            cudaMemcpyDeviceToHost));
        PPF_CUDA(cudaMemcpy(vals, dv.d, n * sizeof(unsigned),
                            cudaMemcpyDeviceToHost));
        unsigned st = status.read();
        ws.release();
        return (int)st;
    } catch (const FatalError &e) {
        return report(e);
    }
}

static_assert(ppf::gpu::kNoAllocMaxPairs == PPF_NOALLOC_SORT_MAX_PAIRS,
              "static sort scratch and the header limit must agree");

extern "C" int ppf_radix_sort_device_noalloc(unsigned *d_keys, unsigned *d_vals,
                                             unsigned n, int key_bits, void *stream) {
    try {
        int rc = radix_sort_pairs_noalloc(d_keys, d_vals, n, key_bits, (cudaStream_t)stream);
        if (rc == -2)
            fprintf(stderr,
                    "[ppf_gb300] ppf_radix_sort_device_noalloc: %u pairs exceed the static "
                    "scratch capacity of %u pairs; nothing was sorted\n",
                    n, PPF_NOALLOC_SORT_MAX_PAIRS);
        return rc;
    } catch (const FatalError &e) {
        return report(e);
    }
}

namespace {
// Status word of the allocating device-memory sort: reset on the caller's
// stream at the start of every call, read by ppf_radix_sort_device_status.
StatusWord *g_sort_status = nullptr;
RadixSortWorkspace g_sort_ws;
} // namespace

extern "C" int ppf_radix_sort_device(unsigned *d_keys, unsigned *d_vals,
                                     unsigned n, int key_bits, void *stream) {
    try {
        if (!g_sort_status) g_sort_status = new StatusWord();
        PPF_CUDA(cudaMemsetAsync(g_sort_status->d, 0, sizeof(unsigned), (cudaStream_t)stream));
        radix_sort_pairs(d_keys, d_vals, n, key_bits, g_sort_ws, g_sort_status->d,
                         (cudaStream_t)stream);
        return 0;
    } catch (const FatalError &e) {
        return report(e);
    }
}

extern "C" int ppf_radix_sort_device_status(void *stream) {
    try {
        if (!g_sort_status) return 0;
        unsigned h = 0;
        PPF_CUDA(cudaMemcpyAsync(&h, g_sort_status->d, sizeof(unsigned), cudaMemcpyDeviceToHost,
                                 (cudaStream_t)stream));
        PPF_CUDA(cudaStreamSynchronize((cudaStream_t)stream));
        return (int)h;
    } catch (const FatalError &e) {
        return report(e);
    }
}

extern "C" int ppf_radix_sort_noalloc_status(void *stream) {
    try {
        return (int)radix_sort_noalloc_status((cudaStream_t)stream);
    } catch (const FatalError &e) {
        return report(e);
    }
}
