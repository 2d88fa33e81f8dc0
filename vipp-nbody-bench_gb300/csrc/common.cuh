// Shared definitions of the GB300 gravity FMM library.
#pragma once

#include <cstddef>
#include <cstdint>

#ifdef __CUDACC__
#include <cuda_runtime.h>
#define GB_HD __host__ __device__ __forceinline__
#define GB_D __device__ __forceinline__
#else
#define GB_HD inline
#endif

namespace gb {

// Morton path: 21 levels of 3 bits below the root, level-1 digit in bits 60..62.
// Digit bit a (a = x, y, z) is 1 for the lower half of the parent box, so the
// digit equals the reference's child offset (octree.hpp:164, 173-176).
constexpr int kMaxLevel = 21;
constexpr int kMaxP = 10;                      // largest supported expansion order
constexpr int kMaxK = (kMaxP + 1) * (kMaxP + 1);
constexpr int kM2LSlots = 216;                 // 27 parent neighbours x 8 children
constexpr int kNbrCap = 27;                    // own p2p / colleague entries per cell
constexpr int kNumOffsets = 343;               // 7^3 same-level offsets in [-3,3]^3

GB_HD int path_shift(int level) { return 3 * (kMaxLevel - level); }

// Level of the first differing digit of two keys (1..21), or 22 when equal.
GB_HD int first_diff_level(uint64_t a, uint64_t b) {
    uint64_t d = a ^ b;
    if (d == 0) return kMaxLevel + 1;
#ifdef __CUDA_ARCH__
    int hb = 63 - __clzll(static_cast<long long>(d));
#else
    int hb = 63 - __builtin_clzll(d);
#endif
    return kMaxLevel - hb / 3;
}

// Status word written by device code; checked by the host after a step.
enum DevErr : int {
    kDevOk = 0,
    kDevNonFinite = 1,
    kDevDepth = 2,
    kDevCapacity = 4,
    kDevTimeout = 8,  // a bounded wait in a pipelined kernel gave up
    kDevForestDepth = 16,  // a forest system needs more key levels than its sort word holds
};

// Tree parameters of one force evaluation, produced on the device.
struct TreeInfo {
    double root_min[3];
    double root_max[3];
    double H[3];          // root box extents
    double S;             // max(H): length unit of the level-0 scaling
    double key_scale[3];  // 2^21 / H: root box -> [0, 2^21) key coordinates
    double key_margin;    // distance (key units) from an integer below which
                          // a key is recomputed by exact midpoint bisection
    double key_scale32[3];  // key_scale 2^32 and -root_min key_scale 2^32:
    double key_off32[3];    // fma(x, scale32, off32) = key coordinate 2^32
    unsigned long long key_mfrac;  // ceil(key_margin 2^32) + 1
    double root_c[3];     // (root_min + root_max) / 2
    int nsplit_total;     // non-leaf cells
    int ncells;
    int nleaves;
    int depth;            // deepest level
    int err;              // DevErr bits
    int level_start[kMaxLevel + 2];   // first cell of each level
    int level_count[kMaxLevel + 2];
    int split_start[kMaxLevel + 2];   // first split entry of each level
    int split_count[kMaxLevel + 2];
    int n_targets_m2l;    // cells at level >= 2
    int n_p2p_chunks;
    long long m2l_pairs;
    long long p2p_pairs;
    long long p2p_ranges;
    // Forest of independent systems (the batched form): entry k of the
    // TreeInfo array holds system k's root box and key fields above, and its
    // particle mass m and G m below; the level tables and the counters above
    // are the whole forest's, in entry 0.
    double m, gm;
    int etile_start[kMaxLevel + 2];  // M2M/L2L tiles of each level (one system per tile)
    int etile_end[kMaxLevel + 2];
    int n_otiles;                    // M2L tiles (one system per tile)
    int pad_;
};

// System of cell c in a forest (c_sys null: one tree, system 0).
GB_HD int cell_system(const int *c_sys, int c) { return c_sys ? c_sys[c] : 0; }

// P2P work chunks of one leaf with n targets. Full chunks hold 32 targets; a
// chunk of t < 32 targets runs floor(32/t) lane groups that share its sources,
// so its cost is ~1/floor(32/t) of a full chunk. The remainder r = n mod 32 is
// one chunk, or two halves when that is cheaper (r = 17..21).
GB_HD bool chunk_split_rem(int r) { return r >= 17 && r <= 21; }
GB_HD int chunk_count(int n) {
    const int r = n % 32;
    return n / 32 + (r == 0 ? 0 : (chunk_split_rem(r) ? 2 : 1));
}
GB_HD void chunk_at(int n, int q, int &off, int &len) {
    const int full = n / 32, r = n % 32;
    if (q < full) {
        off = 32 * q, len = 32;
    } else if (!chunk_split_rem(r)) {
        off = 32 * full, len = r;
    } else if (q == full) {
        off = 32 * full, len = (r + 1) / 2;
    } else {
        off = 32 * full + (r + 1) / 2, len = r / 2;
    }
}

// A chunk whose leaf has more than kSliceSources near-field sources runs as
// several work items, each over a slice of the sources; their partial sums
// are added in slice order afterwards. This bounds the longest work item.
constexpr int kSliceSources = 8192;  // default; the tuning may pick another length
constexpr int kMaxSlices = 4095;
GB_HD int slice_count(unsigned long long srcs, unsigned slice = kSliceSources) {
    const unsigned long long s = (srcs + slice - 1) / slice;
    return s < 1 ? 1 : (s > kMaxSlices ? kMaxSlices : static_cast<int>(s));
}
// Work-item field z: targets (6 bits), slice index (12 bits), slices (12 bits).
GB_HD int item_pack(int nt, int s, int ns) { return nt | (s << 6) | (ns << 18); }
GB_HD int item_nt(int z) { return z & 63; }
GB_HD int item_slice(int z) { return (z >> 6) & 4095; }
GB_HD int item_nslices(int z) { return (z >> 18) & 4095; }

// Index of a real-basis coefficient: (n, 0) -> n^2; (n, m >= 1) real part ->
// n^2 + 2m - 1, imaginary part -> n^2 + 2m.
GB_HD int ridx(int n, int m, int im) { return n * n + (m == 0 ? 0 : 2 * m - 1 + im); }

}  // namespace gb
