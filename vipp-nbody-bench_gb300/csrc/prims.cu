// Exclusive scan and stable LSD radix sort (8-bit digits).
//
// Radix sort, one launch per pass after one histogram launch for all passes
// (single-sweep LSD sort with decoupled look-back): every block takes the next
// 4096-key tile from an atomic ticket, ranks its keys by digit (each warp finds
// the lanes holding its digit with one ballot per digit bit and ranks a key
// among them by lane, so equal digits keep their input order: stability is what
// preserves the reference's ascending-index order among particles with equal
// keys), publishes its per-digit counts, and finds the keys of its digits in
// all earlier tiles by looking back over their published counts. A tile waits
// only on tiles whose blocks have already started (tickets are taken in
// order) and that publish their counts before they look back themselves, so
// every wait ends; it is bounded all the same (kSortSpinMax polls, then an
// error bit, and the missing count is read from that tile's keys directly, so
// the output stays exact). The tile is then staged in shared memory in
// digit order and written out in coalesced runs.
#include "prims.cuh"

namespace gb {

namespace {

constexpr unsigned kFull = 0xffffffffu;

__device__ __forceinline__ unsigned lanemask_lt() {
    unsigned m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

// Lanes of the (fully active) warp whose v equals this lane's, for v < 512
// (a digit 0..255, or 256 for a lane without a key): one ballot per bit, each
// keeping the lanes that agree with this lane on that bit.
__device__ __forceinline__ unsigned warp_peers9(unsigned v) {
    unsigned m = kFull;
#pragma unroll
    for (int b = 0; b < 9; ++b) {
        const bool bit = (v >> b) & 1u;
        const unsigned bal = __ballot_sync(kFull, bit);
        m &= bit ? bal : ~bal;
    }
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
// carried from chunk to chunk; in == out is allowed. Block a scans array a.
constexpr unsigned kSmallScanMax = 1u << 16;
__global__ void __launch_bounds__(1024) k_scan_small(ScanSet ss, unsigned n_cap, const unsigned *d_n) {
    __shared__ unsigned wb[32];
    const int a = blockIdx.x;
    const unsigned *in = ss.in[a];
    unsigned *out = ss.out[a];
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
    if (ss.total[a] && threadIdx.x == 0) *ss.total[a] = carry;
}

// Three-launch scan of larger inputs: tile sums (grid y = array), their scan
// (block a = array a), then the tiles with their offsets.
__global__ void k_scan_reduce(ScanSet ss, unsigned n_cap, const unsigned *d_n, unsigned *__restrict__ tile_sums,
                              unsigned tstride) {
    __shared__ unsigned wb[32];
    const unsigned *in = ss.in[blockIdx.y];
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
    if (threadIdx.x == 0) tile_sums[blockIdx.y * tstride + blockIdx.x] = tot;
}

__global__ void k_scan_tiles(ScanSet ss, unsigned *__restrict__ tile_sums, unsigned tstride, unsigned n_cap,
                             const unsigned *d_n) {
    __shared__ unsigned wb[32];
    const int a = blockIdx.x;
    unsigned *ts = tile_sums + a * tstride;
    const unsigned n = d_n ? *d_n : n_cap;
    const unsigned ntiles = (n + kScanTile - 1) / kScanTile;
    unsigned carry = 0;
    for (unsigned b = 0; b < ntiles; b += blockDim.x) {
        const unsigned i = b + threadIdx.x;
        const unsigned v = i < ntiles ? ts[i] : 0u;
        unsigned tot;
        const unsigned ex = block_exclusive_scan(v, wb, &tot);
        if (i < ntiles) ts[i] = carry + ex;
        carry += tot;
    }
    if (ss.total[a] && threadIdx.x == 0) *ss.total[a] = carry;
}

__global__ void k_scan_apply(ScanSet ss, unsigned n_cap, const unsigned *d_n, const unsigned *__restrict__ tile_sums,
                             unsigned tstride) {
    __shared__ unsigned buf[kScanTile];
    __shared__ unsigned wb[32];
    const unsigned *in = ss.in[blockIdx.y];
    unsigned *out = ss.out[blockIdx.y];
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
    unsigned ex = block_exclusive_scan(s, wb, &tot) + tile_sums[blockIdx.y * tstride + blockIdx.x];
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

constexpr unsigned long long kAggregate = 1ull << 32;  // status word: count of the tile's own keys
constexpr unsigned long long kInclusive = 2ull << 32;  // count of keys in this and all earlier tiles

// Keys of digit d among tile t's keys, read directly: the look-back's fallback
// when a wait for tile t's published count gives up.
__device__ unsigned tile_digit_count(const uint64_t *__restrict__ kin, unsigned t, unsigned n, int bit, unsigned d) {
    const unsigned b = t * kSortTile, e = min(n, b + kSortTile);
    unsigned c = 0;
    for (unsigned i = b; i < e; ++i) c += static_cast<unsigned>((kin[i] >> bit) & 0xffu) == d;
    return c;
}

// Digit counts of all passes in one read of the keys: ghist[p][d].
__global__ void k_sweep_hist(const uint64_t *__restrict__ keys, unsigned n_cap, const unsigned *d_n, int bit_lo, int npasses,
                             unsigned *__restrict__ ghist) {
    __shared__ unsigned cnt[kMaxPasses][256];
    const unsigned n = d_n ? *d_n : n_cap;
    for (int k = threadIdx.x; k < kMaxPasses * 256; k += blockDim.x) (&cnt[0][0])[k] = 0;
    __syncthreads();
    const int lane = threadIdx.x & 31;
    // whole warps step together so that every lane takes part in the ballots
    for (unsigned i0 = blockIdx.x * blockDim.x; i0 < n; i0 += gridDim.x * blockDim.x) {
        const unsigned i = i0 + threadIdx.x;
        const uint64_t key = i < n ? keys[i] : 0ull;
        for (int p = 0; p < npasses; ++p) {
            const unsigned d = i < n ? static_cast<unsigned>((key >> (bit_lo + 8 * p)) & 0xffu) : 256u;
            const unsigned peers = warp_peers9(d);
            if (d < 256u && lane == __ffs(peers) - 1) atomicAdd(&cnt[p][d], __popc(peers));
        }
    }
    __syncthreads();
    for (int k = threadIdx.x; k < npasses * 256; k += blockDim.x)
        if ((&cnt[0][0])[k]) atomicAdd(&ghist[k], (&cnt[0][0])[k]);
}

constexpr size_t kScatterSmem = sizeof(uint64_t) * kSortTile + sizeof(unsigned) * kSortTile;  // 48 KB

// One pass over bits [bit, bit + 8): ghist = this pass's digit counts, status
// = tiles x 256 zeroed look-back words, ticket = zeroed tile counter.
__global__ void __launch_bounds__(256) k_sweep(const uint64_t *__restrict__ kin, const unsigned *__restrict__ vin,
                                               uint64_t *__restrict__ kout, unsigned *__restrict__ vout, unsigned n_cap,
                                               const unsigned *d_n, int bit, const unsigned *__restrict__ ghist,
                                               unsigned long long *status, unsigned *ticket, int *d_err, int err_bit,
                                               unsigned spin_max) {
    constexpr int kRounds = kSortTile / 256;  // 16
    __shared__ unsigned wcnt[8][256];
    __shared__ unsigned dstart[256];  // first tile-local position of each digit
    __shared__ unsigned dbase[256];   // first output position of the tile's keys of each digit
    __shared__ unsigned wsum[8];
    __shared__ unsigned s_tile;
    extern __shared__ __align__(16) unsigned char stage_raw[];  // the tile in digit order
    uint64_t *skey = reinterpret_cast<uint64_t *>(stage_raw);
    unsigned *sval = reinterpret_cast<unsigned *>(skey + kSortTile);
    const unsigned n = d_n ? *d_n : n_cap;
    if (threadIdx.x == 0) s_tile = atomicAdd(ticket, 1u);
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (int d = threadIdx.x; d < 8 * 256; d += 256) (&wcnt[0][0])[d] = 0;
    __syncthreads();
    const unsigned tile = s_tile;
    const unsigned base = tile * kSortTile;
    if (base >= n) return;  // uniform; no later tile looks back at it
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
        const unsigned peers = warp_peers9(d);
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
        // publish this tile's count of digit d, then add up the earlier tiles'
        volatile unsigned long long *sw = status + static_cast<size_t>(tile) * 256 + d;
        *sw = (tile == 0 ? kInclusive : kAggregate) | run;
        __threadfence();
        unsigned long long before = 0;
        if (tile > 0) {
            unsigned spins = 0;
            for (long long tt = static_cast<long long>(tile) - 1; tt >= 0;) {
                const unsigned long long v = *(volatile unsigned long long *)(status + static_cast<size_t>(tt) * 256 + d);
                // spin_max == 0 (tests only) gives up on every earlier tile at once
                if ((v >> 32) == 0 || spin_max == 0) {
                    if (++spins > spin_max) {
                        // give up waiting: report it, count tile tt's keys of digit d
                        // directly and go on, so the sort's output stays exact
                        if (d_err) atomicOr(d_err, err_bit);
                        before += tile_digit_count(kin, static_cast<unsigned>(tt), n, bit, static_cast<unsigned>(d));
                        spins = 0;
                        --tt;
                    }
                    continue;
                }
                before += v & 0xffffffffull;
                if ((v >> 32) == (kInclusive >> 32)) break;
                --tt;
            }
            *sw = kInclusive | (before + run);
            __threadfence();
        }
        // exclusive scan of the digit totals: the pass's global digit bases
        // (ghist) and the tile's local digit starts (run)
        const unsigned g = ghist[d];
        unsigned gi = g, incl = run;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const unsigned u = __shfl_up_sync(kFull, incl, o), ug = __shfl_up_sync(kFull, gi, o);
            if (lane >= o) incl += u, gi += ug;
        }
        if (lane == 31) wsum[w] = incl, dbase[w] = gi;  // dbase[0..7] as scratch for the warps' ghist totals
        __syncthreads();
        unsigned wofs = 0, gofs = 0;
        for (int ww = 0; ww < w; ++ww) wofs += wsum[ww], gofs += dbase[ww];
        __syncthreads();
        dstart[d] = wofs + incl - run;
        dbase[d] = gofs + gi - g + static_cast<unsigned>(before);
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
        const unsigned pos = dbase[d] + (lp - dstart[d]);
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
    cudaError_t e = cudaMalloc(&t.tile_sums, sizeof(unsigned) * kMaxScanArrays * static_cast<size_t>(tiles));
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
        sort_temp_free(t);
        cudaError_t e = cudaMalloc(&t.status, sizeof(unsigned long long) * 256 * kMaxPasses * static_cast<size_t>(tiles));
        if (e == cudaSuccess) e = cudaMalloc(&t.ghist, sizeof(unsigned) * (256 + 1) * kMaxPasses);
        if (e != cudaSuccess) {
            sort_temp_free(t);
            return e;
        }
        t.ticket = t.ghist + 256 * kMaxPasses;
        t.max_tiles = tiles;
    }
    return cudaSuccess;
}

void sort_temp_free(SortTemp &t) {
    if (t.status) cudaFree(t.status);
    if (t.ghist) cudaFree(t.ghist);
    t.status = nullptr, t.ghist = nullptr, t.ticket = nullptr;
    t.max_tiles = 0;
}

void scan_exclusive_multi(const ScanSet &s, int count, unsigned n_cap, const unsigned *d_n, ScanTemp &tmp, cudaStream_t st,
                          int64_t *launches) {
    const unsigned tiles = (n_cap + kScanTile - 1) / kScanTile;
    if (count <= 0) return;
    if (tiles == 0) {
        for (int a = 0; a < count; ++a)
            if (s.total[a]) cudaMemsetAsync(s.total[a], 0, sizeof(unsigned), st);
        return;
    }
    if (n_cap <= kSmallScanMax) {  // one launch instead of three
        k_scan_small<<<count, 1024, 0, st>>>(s, n_cap, d_n);
        if (launches) *launches += 1;
        return;
    }
    const unsigned tstride = static_cast<unsigned>(tmp.max_tiles);
    k_scan_reduce<<<dim3(tiles, count), 256, 0, st>>>(s, n_cap, d_n, tmp.tile_sums, tstride);
    k_scan_tiles<<<count, 1024, 0, st>>>(s, tmp.tile_sums, tstride, n_cap, d_n);
    k_scan_apply<<<dim3(tiles, count), 256, 0, st>>>(s, n_cap, d_n, tmp.tile_sums, tstride);
    if (launches) *launches += 3;
}

void scan_exclusive_u32(const unsigned *in, unsigned *out, unsigned n_cap, const unsigned *d_n, unsigned *d_total,
                        ScanTemp &tmp, cudaStream_t st, int64_t *launches) {
    ScanSet s{};
    s.in[0] = in, s.out[0] = out, s.total[0] = d_total;
    scan_exclusive_multi(s, 1, n_cap, d_n, tmp, st, launches);
}

SortZero sort_zero_plan(const SortTemp &t, unsigned n_cap, int bit_lo, int bit_hi) {
    const unsigned tiles = (n_cap + kSortTile - 1) / kSortTile;
    const int npasses = (bit_hi - bit_lo + 7) / 8;
    return SortZero{t.ghist, t.status, static_cast<size_t>(256) * static_cast<size_t>(npasses > 0 ? npasses : 0) * tiles};
}

int radix_sort_u64(uint64_t *k0, unsigned *v0, uint64_t *k1, unsigned *v1, unsigned n_cap, const unsigned *d_n,
                   int bit_lo, int bit_hi, SortTemp &tmp, cudaStream_t st, int64_t *launches, int *d_err, int err_bit,
                   bool prezeroed, unsigned spin_max) {
    const unsigned tiles = (n_cap + kSortTile - 1) / kSortTile;
    const int npasses = (bit_hi - bit_lo + 7) / 8;
    if (tiles == 0 || npasses <= 0) return 0;
    if (npasses > kMaxPasses || static_cast<int>(tiles) > tmp.max_tiles) {
        if (d_err) cudaMemsetAsync(d_err, 0xff, sizeof(int), st);  // cannot happen with the allocation helpers
        return 0;
    }
    cudaFuncSetAttribute(k_sweep, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(kScatterSmem));
    if (!prezeroed) {
        cudaMemsetAsync(tmp.ghist, 0, sizeof(unsigned) * (256 + 1) * kMaxPasses, st);  // histograms and tickets
        cudaMemsetAsync(tmp.status, 0, sizeof(unsigned long long) * 256 * static_cast<size_t>(npasses) * tiles, st);
    }
    k_sweep_hist<<<tiles < 1024u ? tiles : 1024u, 256, 0, st>>>(k0, n_cap, d_n, bit_lo, npasses, tmp.ghist);
    int cur = 0;
    for (int p = 0; p < npasses; ++p) {
        uint64_t *ki = cur ? k1 : k0, *ko = cur ? k0 : k1;
        unsigned *vi = cur ? v1 : v0, *vo = cur ? v0 : v1;
        k_sweep<<<tiles, 256, kScatterSmem, st>>>(ki, vi, ko, vo, n_cap, d_n, bit_lo + 8 * p, tmp.ghist + 256 * p,
                                                  tmp.status + static_cast<size_t>(p) * 256 * tiles, tmp.ticket + p, d_err,
                                                  err_bit, spin_max);
        cur ^= 1;
    }
    if (launches) *launches += 1 + npasses;
    return cur;
}

}  // namespace gb
