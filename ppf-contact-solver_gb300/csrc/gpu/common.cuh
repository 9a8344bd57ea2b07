// common.cuh -- shared host/device plumbing for the sm_103a kernels.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <atomic>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "../physics/linalg.cuh"

namespace ppf {
namespace gpu {

// Error bits latched by kernels into the device status word instead of
// trapping: the host reads the word at its sync points and turns a set bit
// into a failed step (or a fatal code), so no kernel ever faults or hangs the
// device on a bad input.
enum StatusBits : unsigned {
    STATUS_OK = 0u,
    STATUS_SORT_LOOKBACK_TIMEOUT = 1u << 0,
    STATUS_BVH_STACK_OVERFLOW = 1u << 1,
    STATUS_PAIR_OVERFLOW = 1u << 2,
    STATUS_BLOCK_OVERFLOW = 1u << 3,
    STATUS_REFIT_CYCLE = 1u << 4,
    STATUS_PCG_BREAKDOWN = 1u << 5,
    STATUS_PCG_NONFINITE = 1u << 6,
    STATUS_PRECOND_NONSPD = 1u << 7,
    STATUS_BAD_SLOT = 1u << 8,
};

void check_cuda(cudaError_t err, const char *what, const char *file, int line);
// Kernels launched by this library since it was loaded (every launch site
// ends in PPF_LAUNCH_CHECK or counts itself with count_launches), in all
// host threads, and by the calling thread alone (what a stream capture on
// that thread recorded).
extern std::atomic<unsigned long long> g_kernel_launches;
extern thread_local unsigned long long t_kernel_launches;
inline void count_launches(unsigned long long k = 1) {
    g_kernel_launches += k;
    t_kernel_launches += k;
}
// A capture's launches run when its graph is replayed, not when captured.
inline void uncount_launches(unsigned long long k) {
    g_kernel_launches -= k;
    t_kernel_launches -= k;
}
// Bytes the library has copied host -> device and device -> host since it was
// loaded, counted at the copies of the per-step path (uploads, status reads,
// contact-layout totals, intersection records, fetch).
extern std::atomic<unsigned long long> g_h2d_bytes, g_d2h_bytes;
// Bumped whenever a DevBuf is allocated anew or released: a captured CUDA
// graph holds raw device pointers, so it is valid only while this count is
// the one it was captured under.
extern std::atomic<unsigned long long> g_buffer_epoch;
// Set while this host thread captures a solver's stream into a graph; a
// DevBuf that would have to grow then reports a host error instead of
// allocating (an allocation would end the capture).
extern thread_local bool g_capturing;
void buffer_grow_during_capture();
#define PPF_CUDA(x) ::ppf::gpu::check_cuda((x), #x, __FILE__, __LINE__)
#define PPF_LAUNCH_CHECK()                                                              \
    (::ppf::gpu::count_launches(),                                                      \
     ::ppf::gpu::check_cuda(cudaGetLastError(), "kernel launch", __FILE__, __LINE__))

constexpr unsigned kNumSMs = 152; // GB300: 2 dies x 76 SMs

inline unsigned div_up(unsigned a, unsigned b) { return (a + b - 1) / b; }
inline size_t div_up(size_t a, size_t b) { return (a + b - 1) / b; }

// Monotone float <-> uint32 map (for atomicMin / atomicMax on floats of any
// sign): negative floats flip every bit, non-negative ones flip the sign bit.
__device__ __forceinline__ unsigned float_to_ordered(float f) {
    unsigned u = __float_as_uint(f);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float ordered_to_float(unsigned u) {
    return __uint_as_float((u & 0x80000000u) ? (u & 0x7fffffffu) : ~u);
}
inline unsigned host_float_to_ordered(float f) {
    unsigned u;
    memcpy(&u, &f, 4);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}

__device__ __forceinline__ Vec3 load3(const float *p) {
    return vec3(p[0], p[1], p[2]);
}
__device__ __forceinline__ void store3(float *p, const Vec3 &v) {
    p[0] = v[0];
    p[1] = v[1];
    p[2] = v[2];
}
__device__ __forceinline__ void atomic_add3(float *p, const Vec3 &v) {
    atomicAdd(p + 0, v[0]);
    atomicAdd(p + 1, v[1]);
    atomicAdd(p + 2, v[2]);
}

// Device buffer with a capacity that only grows (the high-water pattern the
// reference's memory pool follows, without per-call frees).
template <class T> struct DevBuf {
    T *ptr = nullptr;
    size_t cap = 0;
    DevBuf() = default;
    DevBuf(const DevBuf &) = delete;
    DevBuf &operator=(const DevBuf &) = delete;
    ~DevBuf() { release(); }
    void reserve(size_t n) {
        if (n <= cap) return;
        if (g_capturing) buffer_grow_during_capture();
        ++g_buffer_epoch;
        if (ptr) PPF_CUDA(cudaFree(ptr));
        size_t c = n < 16 ? 16 : n;
        PPF_CUDA(cudaMalloc(&ptr, c * sizeof(T)));
        cap = c;
    }
    void release() {
        if (ptr) {
            ++g_buffer_epoch;
            cudaFree(ptr);
        }
        ptr = nullptr;
        cap = 0;
    }
    T *data() const { return ptr; }
};

} // namespace gpu
} // namespace ppf
