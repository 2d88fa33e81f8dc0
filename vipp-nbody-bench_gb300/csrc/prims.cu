// Exclusive scan and stable LSD radix sort (8-bit digits).
//
// Radix pass = histogram per 4096-key tile, one exclusive scan of the
// digit-major histogram (giving every (digit, tile) its output base), then a
// scatter in which each warp ranks its keys with __match_any_sync so equal
// digits keep their input order (stability is what preserves the reference's
// ascending-index order among particles with equal keys).
#include "prims.cuh"

namespace gb {

namespace {

constexpr unsigned kFull = 0xffffffffu;

__device__ __forceinline__ unsigned lanemask_lt() {
    unsigned m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

// Exclusive block scan of one value per thread; returns the exclusive prefix
// and writes the block total to *total. blockDim.x must be a multiple of 32.
__device__ unsigned block_exclusive_scan(unsigned v, unsigned *warp_buf /*[32]*/, unsigned *total) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    unsigned x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const unsigned y = __shfl_up_sync(kFull, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) warp_buf[wid] = x;
    __syncthreads();
    if (wid == 0) {
        unsigned w = lane < nw ? warp_buf[lane] : 0u;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const unsigned y = __shfl_up_sync(kFull, w, o);
            if (lane >= o) w += y;
        }
        if (lane < nw) warp_buf[lane] = w;  // inclusive warp totals
    }
    __syncthreads();
    const unsigned before = wid ? warp_buf[wid - 1] : 0u;
    *total = warp_buf[nw - 1];
    __syncthreads();
    return before + x - v;
}

// Whole scan in one block (small inputs): chunks of 4 elements per thread,
// carried from chunk to chunk; in == out is allowed.
constexpr unsigned kSmallScanMax = 1u << 16;
__global__ void __launch_bounds__(1024) k_scan_small(const unsigned *in, unsigned *out, unsigned n_cap, const unsigned *d_n,
                                                     unsigned *d_total) {
    __shared__ unsigned wb[32];
    const unsigned n = d_n ? *d_n : n_cap;
    unsigned carry = 0;
    for (unsigned base = 0; base < n; base += 4 * blockDim.x) {
        const unsigned i0 = base + 4 * threadIdx.x;
        unsigned v[4], s = 0;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            v[j] = i0 + j < n ? in[i0 + j] : 0u;
            s += v[j];
        }
        unsigned tot;
        unsigned ex = carry + block_exclusive_scan(s, wb, &tot);
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            if (i0 + j < n) out[i0 + j] = ex;
            ex += v[j];
        }
        carry += tot;
    }
    if (d_total && threadIdx.x == 0) *d_total = carry;
}

__global__ void k_scan_reduce(const unsigned *__restrict__ in, unsigned n_cap, const unsigned *d_n,
                              unsigned *__restrict__ tile_sums) {
    __shared__ unsigned wb[32];
    const unsigned n = d_n ? *d_n : n_cap;
    const unsigned base = blockIdx.x * kScanTile;
    unsigned s = 0;
    if (base < n) {
        for (int k = 0; k < kScanTile / 256; ++k) {
            const unsigned i = base + k * 256 + threadIdx.x;
            if (i < n) s += in[i];
        }
    }
    unsigned tot;
    block_exclusive_scan(s, wb, &tot);
    if (threadIdx.x == 0) tile_sums[blockIdx.x] = tot;
}

__global__ void k_scan_tiles(unsigned *__restrict__ tile_sums, unsigned n_cap, const unsigned *d_n, unsigned *d_total) {
    __shared__ unsigned wb[32];
    const unsigned n = d_n ? *d_n : n_cap;
    const unsigned ntiles = (n + kScanTile - 1) / kScanTile;
    unsigned carry = 0;
    for (unsigned b = 0; b < ntiles; b += blockDim.x) {
        const unsigned i = b + threadIdx.x;
        const unsigned v = i < ntiles ? tile_sums[i] : 0u;
        unsigned tot;
        const unsigned ex = block_exclusive_scan(v, wb, &tot);
        if (i < ntiles) tile_sums[i] = carry + ex;
        carry += tot;
    }
    if (d_total && threadIdx.x == 0) *d_total = carry;
}

__global__ void k_scan_apply(const unsigned *__restrict__ in, unsigned *__restrict__ out, unsigned n_cap,
                             const unsigned *d_n, const unsigned *__restrict__ tile_sums) {
    __shared__ unsigned buf[kScanTile];
    __shared__ unsigned wb[32];
    const unsigned n = d_n ? *d_n : n_cap;
    const unsigned base = blockIdx.x * kScanTile;
    if (base >= n) return;  // uniform per block
    for (int k = 0; k < kScanTile / 256; ++k) {
        const unsigned i = base + k * 256 + threadIdx.x;
        buf[k * 256 + threadIdx.x] = i < n ? in[i] : 0u;
    }
    __syncthreads();
    constexpr int kPer = kScanTile / 256;
    unsigned loc[kPer];
    unsigned s = 0;
#pragma unroll
    for (int k = 0; k < kPer; ++k) {
        loc[k] = buf[threadIdx.x * kPer + k];
        s += loc[k];
    }
    unsigned tot;
    unsigned ex = block_exclusive_scan(s, wb, &tot) + tile_sums[blockIdx.x];
#pragma unroll
    for (int k = 0; k < kPer; ++k) {
        buf[threadIdx.x * kPer + k] = ex;
        ex += loc[k];
    }
    __syncthreads();
    for (int k = 0; k < kScanTile / 256; ++k) {
        const unsigned i = base + k * 256 + threadIdx.x;
        if (i < n) out[i] = buf[k * 256 + threadIdx.x];
    }
}

__global__ void k_radix_hist(const uint64_t *__restrict__ keys, unsigned n_cap, const unsigned *d_n, int bit,
                             unsigned *__restrict__ hist, unsigned ntiles_cap) {
    __shared__ unsigned cnt[256];
    const unsigned n = d_n ? *d_n : n_cap;
    cnt[threadIdx.x] = 0;
    __syncthreads();
    const unsigned base = blockIdx.x * kSortTile;
    const int lane = threadIdx.x & 31;
    for (int k = 0; k < kSortTile / 256; ++k) {
        const unsigned i = base + k * 256 + threadIdx.x;
        const unsigned d = i < n ? static_cast<unsigned>((keys[i] >> bit) & 0xffu) : 256u;
        const unsigned peers = __match_any_sync(kFull, d);
        if (d < 256u && lane == __ffs(peers) - 1) atomicAdd(&cnt[d], __popc(peers));
    }
    __syncthreads();
    hist[threadIdx.x * ntiles_cap + blockIdx.x] = cnt[threadIdx.x];
}

constexpr size_t kScatterSmem = sizeof(uint64_t) * kSortTile + sizeof(unsigned) * kSortTile;  // 48 KB

__global__ void __launch_bounds__(256) k_radix_scatter(const uint64_t *__restrict__ kin, const unsigned *__restrict__ vin,
                                                       uint64_t *__restrict__ kout, unsigned *__restrict__ vout,
                                                       unsigned n_cap, const unsigned *d_n, int bit,
                                                       const unsigned *__restrict__ hist, unsigned ntiles_cap) {
    constexpr int kRounds = kSortTile / 256;  // 16
    __shared__ unsigned wcnt[8][256];
    __shared__ unsigned dstart[256];  // first tile-local position of each digit
    __shared__ unsigned wsum[8];
    extern __shared__ __align__(16) unsigned char stage_raw[];  // the tile in digit order
    uint64_t *skey = reinterpret_cast<uint64_t *>(stage_raw);
    unsigned *sval = reinterpret_cast<unsigned *>(skey + kSortTile);
    const unsigned n = d_n ? *d_n : n_cap;
    const unsigned base = blockIdx.x * kSortTile;
    if (base >= n) return;  // uniform
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (int d = threadIdx.x; d < 8 * 256; d += 256) (&wcnt[0][0])[d] = 0;
    __syncthreads();
    uint64_t key[kRounds];
    unsigned val[kRounds], rank[kRounds], dig[kRounds];
    const unsigned lt = lanemask_lt();
#pragma unroll
    for (int k = 0; k < kRounds; ++k) {
        const unsigned i = base + w * (kSortTile / 8) + k * 32 + lane;
        const bool ok = i < n;
        key[k] = ok ? kin[i] : 0ull;
        val[k] = (ok && vin) ? vin[i] : 0u;
        const unsigned d = ok ? static_cast<unsigned>((key[k] >> bit) & 0xffu) : 256u;
        dig[k] = d;
        const unsigned peers = __match_any_sync(kFull, d);
        const unsigned before = d < 256u ? wcnt[w][d] : 0u;
        __syncwarp();
        rank[k] = before + __popc(peers & lt);
        if (d < 256u && lane == __ffs(peers) - 1) wcnt[w][d] += __popc(peers);
        __syncwarp();
    }
    __syncthreads();
    {
        const int d = threadIdx.x;
        unsigned run = 0;
#pragma unroll
        for (int ww = 0; ww < 8; ++ww) {
            const unsigned c = wcnt[ww][d];
            wcnt[ww][d] = run;
            run += c;
        }
        // exclusive scan of the tile's digit totals (thread d holds digit d)
        unsigned incl = run;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const unsigned u = __shfl_up_sync(kFull, incl, o);
            if (lane >= o) incl += u;
        }
        if (lane == 31) wsum[w] = incl;
        __syncthreads();
        unsigned wofs = 0;
        for (int ww = 0; ww < w; ++ww) wofs += wsum[ww];
        dstart[d] = wofs + incl - run;
    }
    __syncthreads();
    // tile-local sorted order in shared memory ...
#pragma unroll
    for (int k = 0; k < kRounds; ++k) {
        const unsigned d = dig[k];
        if (d < 256u) {
            const unsigned lp = dstart[d] + wcnt[w][d] + rank[k];
            skey[lp] = key[k];
            sval[lp] = val[k];
        }
    }
    __syncthreads();
    // ... then written out in that order: consecutive threads write
    // consecutive positions of each digit's run
    const unsigned cnt = min(n - base, static_cast<unsigned>(kSortTile));
    for (unsigned lp = threadIdx.x; lp < cnt; lp += blockDim.x) {
        const uint64_t kk = skey[lp];
        const unsigned d = static_cast<unsigned>((kk >> bit) & 0xffu);
        const unsigned pos = hist[d * ntiles_cap + blockIdx.x] + (lp - dstart[d]);
        kout[pos] = kk;
        if (vout) vout[pos] = sval[lp];
    }
}

}  // namespace

cudaError_t scan_temp_alloc(ScanTemp &t, unsigned n_cap) {
    const int tiles = static_cast<int>((static_cast<uint64_t>(n_cap) + kScanTile - 1) / kScanTile) + 1;
    if (tiles <= t.max_tiles) return cudaSuccess;
    if (t.tile_sums) cudaFree(t.tile_sums);
    t.tile_sums = nullptr;
    cudaError_t e = cudaMalloc(&t.tile_sums, sizeof(unsigned) * tiles);
    t.max_tiles = e == cudaSuccess ? tiles : 0;
    return e;
}

void scan_temp_free(ScanTemp &t) {
    if (t.tile_sums) cudaFree(t.tile_sums);
    t.tile_sums = nullptr;
    t.max_tiles = 0;
}

cudaError_t sort_temp_alloc(SortTemp &t, unsigned n_cap) {
    const int tiles = static_cast<int>((static_cast<uint64_t>(n_cap) + kSortTile - 1) / kSortTile) + 1;
    if (tiles > t.max_tiles) {
        if (t.hist) cudaFree(t.hist);
        t.hist = nullptr;
        cudaError_t e = cudaMalloc(&t.hist, sizeof(unsigned) * 256 * static_cast<size_t>(tiles));
        if (e != cudaSuccess) {
            t.max_tiles = 0;
            return e;
        }
        t.max_tiles = tiles;
    }
    return scan_temp_alloc(t.scan, 256u * static_cast<unsigned>(t.max_tiles));
}

void sort_temp_free(SortTemp &t) {
    if (t.hist) cudaFree(t.hist);
    t.hist = nullptr;
    t.max_tiles = 0;
    scan_temp_free(t.scan);
}

void scan_exclusive_u32(const unsigned *in, unsigned *out, unsigned n_cap, const unsigned *d_n, unsigned *d_total,
                        ScanTemp &tmp, cudaStream_t st, int64_t *launches) {
    const unsigned tiles = (n_cap + kScanTile - 1) / kScanTile;
    if (tiles == 0) {
        if (d_total) cudaMemsetAsync(d_total, 0, sizeof(unsigned), st);
        return;
    }
    if (n_cap <= kSmallScanMax) {  // one launch instead of three
        k_scan_small<<<1, 1024, 0, st>>>(in, out, n_cap, d_n, d_total);
        if (launches) *launches += 1;
        return;
    }
    k_scan_reduce<<<tiles, 256, 0, st>>>(in, n_cap, d_n, tmp.tile_sums);
    k_scan_tiles<<<1, 1024, 0, st>>>(tmp.tile_sums, n_cap, d_n, d_total);
    k_scan_apply<<<tiles, 256, 0, st>>>(in, out, n_cap, d_n, tmp.tile_sums);
    if (launches) *launches += 3;
}

int radix_sort_u64(uint64_t *k0, unsigned *v0, uint64_t *k1, unsigned *v1, unsigned n_cap, const unsigned *d_n,
                   int bit_lo, int bit_hi, SortTemp &tmp, cudaStream_t st, int64_t *launches) {
    const unsigned tiles = (n_cap + kSortTile - 1) / kSortTile;
    if (tiles == 0) return 0;
    cudaFuncSetAttribute(k_radix_scatter, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(kScatterSmem));
    int cur = 0;
    for (int bit = bit_lo; bit < bit_hi; bit += 8) {
        uint64_t *ki = cur ? k1 : k0, *ko = cur ? k0 : k1;
        unsigned *vi = cur ? v1 : v0, *vo = cur ? v0 : v1;
        k_radix_hist<<<tiles, 256, 0, st>>>(ki, n_cap, d_n, bit, tmp.hist, tiles);
        scan_exclusive_u32(tmp.hist, tmp.hist, 256u * tiles, nullptr, nullptr, tmp.scan, st, launches);
        k_radix_scatter<<<tiles, 256, kScatterSmem, st>>>(ki, vi, ko, vo, n_cap, d_n, bit, tmp.hist, tiles);
        if (launches) *launches += 2;
        cur ^= 1;
    }
    return cur;
}

}  // namespace gb
