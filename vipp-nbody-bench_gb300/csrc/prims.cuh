// Device-wide primitives: exclusive scan and a stable LSD radix sort.
// Element counts may live in device memory (`const unsigned *d_n`, nullptr
// means the host value `n_cap`), so a whole force evaluation can be queued
// without reading sizes back; grids are sized from the host capacity and
// tiles beyond the device count do nothing.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

namespace gb {

constexpr int kMaxScanArrays = 3;  // arrays one scan launch sequence can take

struct ScanTemp {
    unsigned *tile_sums = nullptr;  // [kMaxScanArrays][max_tiles]
    int max_tiles = 0;              // per array
};

constexpr int kScanTile = 2048;  // 256 threads x 8

// out[i] = sum_{j<i} in[i] for i < n (n from d_n if non-null, else n_cap).
// If d_total != nullptr, *d_total = sum of all n inputs. in == out allowed.
void scan_exclusive_u32(const unsigned *in, unsigned *out, unsigned n_cap, const unsigned *d_n, unsigned *d_total,
                        ScanTemp &tmp, cudaStream_t st, int64_t *launches);

// The same for up to kMaxScanArrays arrays of one length, in one launch
// sequence: out[a] = exclusive scan of in[a], *total[a] (if non-null) = sum.
struct ScanSet {
    const unsigned *in[kMaxScanArrays];
    unsigned *out[kMaxScanArrays];
    unsigned *total[kMaxScanArrays];
};
void scan_exclusive_multi(const ScanSet &s, int count, unsigned n_cap, const unsigned *d_n, ScanTemp &tmp, cudaStream_t st,
                          int64_t *launches);

constexpr int kSortTile = 4096;  // 256 threads x 16 keys
constexpr int kMaxPasses = 8;    // 8-bit digits: up to 64 key bits

struct SortTemp {
    unsigned long long *status = nullptr;  // [kMaxPasses][max_tiles][256] look-back words
    unsigned *ghist = nullptr;             // [kMaxPasses][256] digit counts, then [kMaxPasses] tile tickets
    unsigned *ticket = nullptr;
    int max_tiles = 0;
};

constexpr unsigned kSortSpinMax = 1u << 24;  // look-back polls before a wait gives up

// Stable sort of (key, val) pairs by bits [bit_lo, bit_hi) of the key.
// Ping-pongs between (k0, v0) and (k1, v1); returns 0 if the result is in
// (k0, v0), 1 if in (k1, v1). vals may be nullptr (keys only). A look-back
// wait that gives up after spin_max polls (at once for 0) sets err_bit in
// *d_err (if d_err is not null) and counts the missing tile directly.
// prezeroed: a kernel queued before the sort has run sort_temp_zero over
// the sort's temporaries (saves two memset nodes per sort).
int radix_sort_u64(uint64_t *k0, unsigned *v0, uint64_t *k1, unsigned *v1, unsigned n_cap, const unsigned *d_n,
                   int bit_lo, int bit_hi, SortTemp &tmp, cudaStream_t st, int64_t *launches, int *d_err = nullptr,
                   int err_bit = 0, bool prezeroed = false, unsigned spin_max = kSortSpinMax);

// What a sort of n_cap keys over bits [bit_lo, bit_hi) needs zeroed: the
// histogram and ticket words, and npasses x tiles x 256 look-back words.
struct SortZero {
    unsigned *ghist;
    unsigned long long *status;
    size_t status_words;
};
SortZero sort_zero_plan(const SortTemp &t, unsigned n_cap, int bit_lo, int bit_hi);

#ifdef __CUDACC__
// Zero the sort temporaries from every thread of a grid (any grid shape).
__device__ __forceinline__ void sort_temp_zero(const SortZero &z) {
    const size_t tid = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x;
    const size_t nt = static_cast<size_t>(gridDim.x) * blockDim.x;
    for (size_t k = tid; k < static_cast<size_t>(256 + 1) * kMaxPasses; k += nt) z.ghist[k] = 0u;
    for (size_t k = tid; k < z.status_words; k += nt) z.status[k] = 0ull;
}
#endif

// Allocation helpers for the temporaries (sized for n_cap elements).
cudaError_t scan_temp_alloc(ScanTemp &t, unsigned n_cap);
cudaError_t sort_temp_alloc(SortTemp &t, unsigned n_cap);
void scan_temp_free(ScanTemp &t);
void sort_temp_free(SortTemp &t);

}  // namespace gb
