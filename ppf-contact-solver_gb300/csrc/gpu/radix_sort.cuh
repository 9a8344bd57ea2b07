// radix_sort.cuh -- stable LSD radix sort of (u32 key, u32 value) pairs.
//
// Onesweep structure: one pass over the keys builds the digit histograms of
// every pass at once; then each pass is a single kernel that ranks a tile in
// shared memory and obtains its global digit offsets by decoupled look-back
// over the tiles before it. Digits are 8 bits wide, so a 30-bit Morton code
// sorts in 4 passes (the reference's radix_sort.cu uses 8 passes of 4 bits;
// both are stable counting sorts by key, so they produce the same permutation).
#pragma once

#include "common.cuh"

namespace ppf {
namespace gpu {

struct RadixSortWorkspace {
    DevBuf<unsigned> hist;       // passes x 256 digit offsets
    DevBuf<unsigned> lookback;   // tiles x 256 look-back words (one pass)
    DevBuf<unsigned> tile_ctr;   // one dynamic tile counter per pass
    DevBuf<unsigned> keys_alt;
    DevBuf<unsigned> vals_alt;
    void reserve(size_t n);
    void release();
};

constexpr unsigned kSortThreads = 256;
constexpr unsigned kSortItems = 8; // per thread
constexpr unsigned kSortTile = kSortThreads * kSortItems;

// Sorts `n` pairs in place by the low `key_bits` bits of the key. Stable:
// equal keys keep their input order. `d_status` receives
// STATUS_SORT_LOOKBACK_TIMEOUT if a look-back wait ever exceeds its bound.
void radix_sort_pairs(unsigned *keys, unsigned *vals, unsigned n, int key_bits,
                      RadixSortWorkspace &ws, unsigned *d_status,
                      cudaStream_t stream);

// The same sort with fixed-capacity static device scratch: allocates nothing.
// Returns -2 (and touches nothing) when n exceeds kNoAllocMaxPairs.
constexpr unsigned kNoAllocMaxPairs = 1u << 20;
int radix_sort_pairs_noalloc(unsigned *keys, unsigned *vals, unsigned n, int key_bits,
                             cudaStream_t stream);
// Status bits of the last allocation-free sort ordered before this call on
// `stream` (waits for the stream): 0, or STATUS_SORT_LOOKBACK_TIMEOUT.
unsigned radix_sort_noalloc_status(cudaStream_t stream);

} // namespace gpu
} // namespace ppf
