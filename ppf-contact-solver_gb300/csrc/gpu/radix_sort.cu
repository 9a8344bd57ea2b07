// radix_sort.cu -- onesweep stable LSD radix sort, 8-bit digits.
#include "fatal.cuh"
#include "radix_sort.cuh"

#include <mutex>

namespace ppf {
namespace gpu {

namespace {

constexpr unsigned kRadix = 256;
constexpr unsigned kWarps = kSortThreads / 32;
constexpr unsigned kFlagAggregate = 1u << 30;
constexpr unsigned kFlagPrefix = 2u << 30;
constexpr unsigned kCountMask = (1u << 30) - 1u;
// Upper bound on look-back polls of one predecessor word. A predecessor tile
// always holds a lower tile id, so it is already resident and publishes within
// microseconds; the bound only converts a logic error into a status bit
// instead of a hung device.
constexpr unsigned kMaxSpins = 1u << 21;

// One read of the keys builds the histograms of all passes.
__global__ void k_digit_histograms(const unsigned *__restrict__ keys, unsigned n,
                                   int passes, unsigned *__restrict__ hist) {
    __shared__ unsigned s_hist[4][kRadix];
    for (unsigned i = threadIdx.x; i < 4 * kRadix; i += blockDim.x)
        (&s_hist[0][0])[i] = 0u;
    __syncthreads();
    for (unsigned i = blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += gridDim.x * blockDim.x) {
        unsigned k = keys[i];
        for (int p = 0; p < passes; ++p)
            atomicAdd(&s_hist[p][(k >> (8 * p)) & 0xffu], 1u);
    }
    __syncthreads();
    for (int p = 0; p < passes; ++p)
        for (unsigned d = threadIdx.x; d < kRadix; d += blockDim.x) {
            unsigned c = s_hist[p][d];
            if (c) atomicAdd(&hist[p * kRadix + d], c);
        }
}

// In-place exclusive scan of each pass's 256 digit counts (one block / pass).
__global__ void k_scan_histograms(unsigned *hist) {
    __shared__ unsigned s[kRadix];
    unsigned *h = hist + blockIdx.x * kRadix;
    unsigned t = threadIdx.x;
    unsigned v = h[t];
    s[t] = v;
    __syncthreads();
    for (unsigned off = 1; off < kRadix; off <<= 1) {
        unsigned a = t >= off ? s[t - off] : 0u;
        __syncthreads();
        s[t] += a;
        __syncthreads();
    }
    h[t] = s[t] - v;
}

__device__ __forceinline__ unsigned lanemask_lt() {
    unsigned m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

// One pass. Warp w of a tile owns the contiguous range
// [tile_base + 256 w, tile_base + 256 (w + 1)) and walks it in 8 rounds of 32,
// so (warp, round, lane) order is input order and the ranks are stable.
__global__ void __launch_bounds__(kSortThreads)
    k_onesweep_pass(const unsigned *__restrict__ keys_in,
                    const unsigned *__restrict__ vals_in,
                    unsigned *__restrict__ keys_out,
                    unsigned *__restrict__ vals_out, unsigned n, int shift,
                    const unsigned *__restrict__ digit_offset,
                    unsigned *lookback, unsigned *tile_ctr, unsigned *status) {
    __shared__ unsigned s_tile;
    __shared__ unsigned s_wcnt[kWarps][kRadix];
    __shared__ unsigned s_base[kRadix];

    const unsigned tid = threadIdx.x;
    const unsigned lane = tid & 31u;
    const unsigned warp = tid >> 5;
    if (tid == 0) s_tile = atomicAdd(tile_ctr, 1u);
    for (unsigned w = 0; w < kWarps; ++w) s_wcnt[w][tid] = 0u;
    __syncthreads();
    const unsigned tile = s_tile;
    const unsigned base = tile * kSortTile + warp * (32u * kSortItems);

    unsigned key[kSortItems], val[kSortItems], dig[kSortItems], rank[kSortItems];
#pragma unroll
    for (unsigned r = 0; r < kSortItems; ++r) {
        unsigned idx = base + r * 32u + lane;
        if (idx < n) {
            key[r] = keys_in[idx];
            val[r] = vals_in[idx];
            dig[r] = (key[r] >> shift) & 0xffu;
        } else {
            key[r] = 0u;
            val[r] = 0u;
            dig[r] = 0x100u; // outside every bucket
        }
    }
    const unsigned lt = lanemask_lt();
#pragma unroll
    for (unsigned r = 0; r < kSortItems; ++r) {
        const unsigned d = dig[r];
        const unsigned peers = __match_any_sync(0xffffffffu, d);
        const unsigned leader = __ffs(peers) - 1u;
        unsigned old = 0u;
        if (d < kRadix) old = s_wcnt[warp][d];
        __syncwarp();
        if (d < kRadix && lane == leader) s_wcnt[warp][d] = old + __popc(peers);
        __syncwarp();
        rank[r] = old + __popc(peers & lt);
    }
    __syncthreads();

    // Thread `tid` owns digit `tid`: per-warp exclusive offsets, tile total.
    const unsigned d = tid;
    unsigned acc = 0u;
    for (unsigned w = 0; w < kWarps; ++w) {
        unsigned c = s_wcnt[w][d];
        s_wcnt[w][d] = acc;
        acc += c;
    }
    volatile unsigned *lb = lookback;
    unsigned excl = 0u;
    if (tile == 0) {
        lb[d] = kFlagPrefix | acc;
    } else {
        lb[tile * kRadix + d] = kFlagAggregate | acc;
        int t = (int)tile - 1;
        unsigned spins = 0u;
        while (t >= 0) {
            unsigned s = lb[(unsigned)t * kRadix + d];
            unsigned flag = s & ~kCountMask;
            if (flag == 0u) {
                if (++spins > kMaxSpins) {
                    atomicOr(status, STATUS_SORT_LOOKBACK_TIMEOUT);
                    break;
                }
                __nanosleep(32);
                continue;
            }
            excl += s & kCountMask;
            if (flag == kFlagPrefix) break;
            --t;
        }
        lb[tile * kRadix + d] = kFlagPrefix | (excl + acc);
    }
    s_base[d] = digit_offset[d] + excl;
    __syncthreads();

#pragma unroll
    for (unsigned r = 0; r < kSortItems; ++r) {
        const unsigned dd = dig[r];
        if (dd < kRadix) {
            unsigned pos = s_base[dd] + s_wcnt[warp][dd] + rank[r];
            if (pos < n) {
                keys_out[pos] = key[r];
                vals_out[pos] = val[r];
            }
        }
    }
}

} // namespace

void RadixSortWorkspace::reserve(size_t n) {
    hist.reserve(4 * kRadix);
    tile_ctr.reserve(4);
    size_t tiles = div_up(n, (size_t)kSortTile);
    lookback.reserve(tiles * kRadix);
    keys_alt.reserve(n);
    vals_alt.reserve(n);
}

void RadixSortWorkspace::release() {
    hist.release();
    lookback.release();
    tile_ctr.release();
    keys_alt.release();
    vals_alt.release();
}

void radix_sort_pairs(unsigned *keys, unsigned *vals, unsigned n, int key_bits,
                      RadixSortWorkspace &ws, unsigned *d_status,
                      cudaStream_t stream) {
    if (n <= 1 || key_bits <= 0) return;
    int passes = (key_bits + 7) / 8;
    if (passes > 4) passes = 4;
    ws.reserve(n);
    const unsigned tiles = div_up(n, kSortTile);
    PPF_CUDA(cudaMemsetAsync(ws.hist.data(), 0, 4 * kRadix * sizeof(unsigned),
                             stream));
    PPF_CUDA(cudaMemsetAsync(ws.tile_ctr.data(), 0, 4 * sizeof(unsigned), stream));
    unsigned hgrid = tiles < 4 * kNumSMs ? tiles : 4 * kNumSMs;
    k_digit_histograms<<<hgrid, 256, 0, stream>>>(keys, n, passes,
                                                  ws.hist.data());
    PPF_LAUNCH_CHECK();
    k_scan_histograms<<<passes, kRadix, 0, stream>>>(ws.hist.data());
    PPF_LAUNCH_CHECK();
    unsigned *src_k = keys, *src_v = vals;
    unsigned *dst_k = ws.keys_alt.data(), *dst_v = ws.vals_alt.data();
    for (int p = 0; p < passes; ++p) {
        PPF_CUDA(cudaMemsetAsync(ws.lookback.data(), 0,
                                 (size_t)tiles * kRadix * sizeof(unsigned),
                                 stream));
        k_onesweep_pass<<<tiles, kSortThreads, 0, stream>>>(
            src_k, src_v, dst_k, dst_v, n, 8 * p, ws.hist.data() + p * kRadix,
            ws.lookback.data(), ws.tile_ctr.data() + p, d_status);
        PPF_LAUNCH_CHECK();
        unsigned *tk = src_k, *tv = src_v;
        src_k = dst_k;
        src_v = dst_v;
        dst_k = tk;
        dst_v = tv;
    }
    if (src_k != keys) {
        PPF_CUDA(cudaMemcpyAsync(keys, src_k, n * sizeof(unsigned),
                                 cudaMemcpyDeviceToDevice, stream));
        PPF_CUDA(cudaMemcpyAsync(vals, src_v, n * sizeof(unsigned),
                                 cudaMemcpyDeviceToDevice, stream));
    }
}

} // namespace gpu
} // namespace ppf

// ---- allocation-free variant ------------------------------------------------
// The same sort with its scratch in file-scope device arrays of a fixed
// capacity, so a call allocates nothing. One scratch set exists per device:
// calls that overlap in time on any streams race on it and must be ordered
// by the caller.
namespace ppf {
namespace gpu {

namespace {

constexpr unsigned kNoAllocTiles = (kNoAllocMaxPairs + kSortTile - 1) / kSortTile;

__device__ __align__(256) unsigned g_na_keys[kNoAllocMaxPairs];
__device__ __align__(256) unsigned g_na_vals[kNoAllocMaxPairs];
__device__ __align__(256) unsigned g_na_lookback[kNoAllocTiles * kRadix];
__device__ __align__(256) unsigned g_na_hist[4 * kRadix];
__device__ __align__(256) unsigned g_na_ctr[4];
__device__ __align__(256) unsigned g_na_status[1];

struct NoAllocScratch {
    unsigned *keys = nullptr, *vals = nullptr, *lookback = nullptr;
    unsigned *hist = nullptr, *ctr = nullptr, *status = nullptr;
};
constexpr int kMaxDevices = 64;
NoAllocScratch g_na[kMaxDevices];
std::once_flag g_na_once[kMaxDevices];

template <class T> void symbol_address(unsigned **out, const T &sym) {
    PPF_CUDA(cudaGetSymbolAddress((void **)out, sym));
}

// Device addresses of the scratch arrays for the current device, looked up
// once per device under a once-flag, so two host threads making their first
// call on one device do not race. A lookup that throws leaves the flag unset
// and the next call tries again.
const NoAllocScratch &noalloc_scratch() {
    int dev = 0;
    PPF_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kMaxDevices) throw FatalError(3, "device ordinal out of range");
    std::call_once(g_na_once[dev], [dev] {
        NoAllocScratch s;
        symbol_address(&s.keys, g_na_keys);
        symbol_address(&s.vals, g_na_vals);
        symbol_address(&s.lookback, g_na_lookback);
        symbol_address(&s.hist, g_na_hist);
        symbol_address(&s.ctr, g_na_ctr);
        symbol_address(&s.status, g_na_status);
        g_na[dev] = s;
    });
    return g_na[dev];
}

} // namespace

int radix_sort_pairs_noalloc(unsigned *keys, unsigned *vals, unsigned n, int key_bits,
                             cudaStream_t stream) {
    if (n > kNoAllocMaxPairs) return -2;
    // set-up first, so that a call with n = 0 performs it (a warm-up call)
    const NoAllocScratch &s = noalloc_scratch();
    PPF_CUDA(cudaMemsetAsync(s.status, 0, sizeof(unsigned), stream));
    if (n <= 1 || key_bits <= 0) return 0;
    int passes = (key_bits + 7) / 8;
    if (passes > 4) passes = 4;
    const unsigned tiles = div_up(n, kSortTile);
    // the histograms and tile counters start at zero every call (the status
    // word was cleared above); the look-back words start at zero every pass
    PPF_CUDA(cudaMemsetAsync(s.hist, 0, 4 * kRadix * sizeof(unsigned), stream));
    PPF_CUDA(cudaMemsetAsync(s.ctr, 0, 4 * sizeof(unsigned), stream));
    unsigned hgrid = tiles < 4 * kNumSMs ? tiles : 4 * kNumSMs;
    k_digit_histograms<<<hgrid, 256, 0, stream>>>(keys, n, passes, s.hist);
    PPF_LAUNCH_CHECK();
    k_scan_histograms<<<passes, kRadix, 0, stream>>>(s.hist);
    PPF_LAUNCH_CHECK();
    unsigned *src_k = keys, *src_v = vals, *dst_k = s.keys, *dst_v = s.vals;
    for (int p = 0; p < passes; ++p) {
        PPF_CUDA(cudaMemsetAsync(s.lookback, 0, (size_t)tiles * kRadix * sizeof(unsigned),
                                 stream));
        k_onesweep_pass<<<tiles, kSortThreads, 0, stream>>>(src_k, src_v, dst_k, dst_v, n,
                                                           8 * p, s.hist + p * kRadix,
                                                           s.lookback, s.ctr + p, s.status);
        PPF_LAUNCH_CHECK();
        unsigned *tk = src_k, *tv = src_v;
        src_k = dst_k;
        src_v = dst_v;
        dst_k = tk;
        dst_v = tv;
    }
    if (src_k != keys) {
        PPF_CUDA(cudaMemcpyAsync(keys, src_k, n * sizeof(unsigned), cudaMemcpyDeviceToDevice,
                                 stream));
        PPF_CUDA(cudaMemcpyAsync(vals, src_v, n * sizeof(unsigned), cudaMemcpyDeviceToDevice,
                                 stream));
    }
    return 0;
}

unsigned radix_sort_noalloc_status(cudaStream_t stream) {
    const NoAllocScratch &s = noalloc_scratch();
    unsigned h = 0;
    PPF_CUDA(cudaMemcpyAsync(&h, s.status, sizeof(unsigned), cudaMemcpyDeviceToHost, stream));
    PPF_CUDA(cudaStreamSynchronize(stream));
    return h;
}

} // namespace gpu
} // namespace ppf
