// M2L on the 5th-generation tensor cores (tcgen05, sm_103a), mixed precision.
//
// Same work as k_m2l in fmm.cu (fmm.hpp:277-304 restated on scaled real-basis
// expansions): every target cell at level >= 2 gathers the expansions of its
// up-to-189 interaction-list sources and applies one K x K operator per
// source offset. Targets sharing an octant share the slot -> offset map, so a
// tile of 128 same-octant targets is, per slot, one GEMM
//     D[128 x N] += A[128 x K] * B[N x K]^T,  A = gathered source rows,
//                                             B = the slot's operator,
// accumulated in TMEM (128 lanes x N FP32 columns).
//
// Precision, two forms of the same three-product split
//     D += Ahi Bhi + Ahi Blo + Alo Bhi,   x = hi + lo,   FP32 accumulation:
//  * TF32 (default): kind::tf32, hi = FP32 with the low 13 mantissa bits
//    cleared, lo = x - hi: ~2^-21 per product; hi and lo rows are two A
//    operands;
//  * BF16 (GB_FLAG_M2L_BF16): kind::f16 with bf16 operands, hi = bf16(x), lo =
//    bf16(x - hi): ~2^-17 relative error per product. A source row is the
//    concatenation [hi | lo] (2K values), so Ahi Bhi + Alo Bhi is one product
//    over the doubled K, and one B operand [Bhi ; Blo] of 2N rows gives
//    Ahi Blo in the second N accumulator columns (zero rows of Blo under the
//    lo half of K: those K steps issue N-wide MMAs on Bhi alone). It halves
//    the gathered bytes and the MMA time; measured at 4M particles, p = 8:
//    M2L 2.32 instead of 2.79 ms per evaluation, force error against the FP64
//    direct sum unchanged (RMS 2.386e-4), energy drift over 10 steps 5e-7
//    instead of 6e-8.
// The expansions are scaled per cell by powers of the cell size, so bf16's
// FP32 exponent range holds them.
//
// Accumulation: the tensor core's FP32 accumulation adds an error that grows
// with the number of MMAs summed into one accumulator (measured: RMS error
// proportional to the chain length, 1.5e-5 relative on the accelerations with
// all MMAs of a tile in one accumulator). Slots are therefore grouped, kGroup
// slots per group, into one of two TMEM accumulators used in turn; the drain
// warps add each finished group into FP32 registers (round-to-nearest
// additions) while the next group accumulates.
//
// Data flow (one CTA per SM, persistent over tiles, warp-specialised):
//  * k_split_m writes every cell's expansion once more, split and zero-padded
//    to whole 128-byte K chunks (bf16: one [hi | lo] row of 64-element chunks;
//    tf32: a hi row and a lo row of 32-element chunks), plus a zero row that
//    stands in for absent sources;
//  * the loader warps gather, per (slot, K chunk) step, the 128 source rows of
//    the tile with TMA tile::gather4 copies (4 rows of 128 bytes per copy) into
//    128B-swizzled K-major A tiles (bf16: 32 copies; tf32: 64, hi and lo), and
//    the slot's pre-split operator chunk with one cp.async.bulk;
//  * the MMA warp (one thread) issues the step's tcgen05.mma (one per 32-byte
//    K step; tf32: two), commits the stage back to the loaders and each
//    finished group to the drain warps;
//  * the drain warps (warps 0-3 own TMEM lanes 32w..32w+31, i.e. tile rows)
//    add the groups and write the tile's local expansions.
// Every tile runs the same static schedule (189 slots x NKC chunks), so the
// three roles agree on it without exchanging control data.
//
// Every mbarrier wait is bounded by the global timer; on a timeout the CTA
// records kDevTimeout in the status word, stops issuing work, waits (bounded)
// for its own copies and MMAs, frees its TMEM and returns.
#include <cuda.h>

#include <algorithm>
#include <cuda_bf16.h>

#include "workspace.cuh"

namespace gb {

namespace {

constexpr int kRows = 128;          // targets per tile (MMA M)
static_assert(kRows == kM2LTileTC, "forest M2L tiles");
constexpr int kKC32 = 32;           // K chunk in 4-byte units: one 128-byte swizzle row
constexpr int kDrainThreads = 128;  // warps 0-3
#ifndef M2L_LOADER_WARPS
#define M2L_LOADER_WARPS 4
#endif
#ifndef M2L_MAX_STAGES
#define M2L_MAX_STAGES 4  // tf32 stages (56 KB each)
#endif
#ifndef M2L_MAX_STAGES_BF16
#define M2L_MAX_STAGES_BF16 5  // bf16 stages (40 KB each)
#endif
#ifndef M2L_MIN_BLOCKS
#define M2L_MIN_BLOCKS 1  // > 1 caps registers so the kernel fits beside P2P blocks
#endif
#ifndef M2L_WIDE_B
#define M2L_WIDE_B 1
#endif
#ifndef M2L_TMEM_TOTAL
#define M2L_TMEM_TOTAL 1  // drain keeps a tile's running sums in free TMEM columns, not registers
#endif
constexpr int kLoaderWarps = M2L_LOADER_WARPS;  // warps 4 .. 3 + kLoaderWarps
constexpr int kMmaWarp = 4 + kLoaderWarps;
constexpr int kThreads = 32 * (kMmaWarp + 1);
constexpr unsigned long long kWaitNs = 2000000000ull;  // 2 s per wait
#ifndef M2L_PREFETCH2
#define M2L_PREFETCH2 1  // source rows of two slots ahead in flight instead of one (~1% faster at 4M)
#endif
#ifndef M2L_GROUP
#define M2L_GROUP 4
#endif
constexpr int kGroup = M2L_GROUP;   // slots per TMEM accumulation group
constexpr int kSlotsPerTile = 189;  // M2L slots of every octant: 216 minus the 27 adjacent ones
constexpr int kGroupsPerTile = (kSlotsPerTile + kGroup - 1) / kGroup;
constexpr int kSmemMax = 232448;    // opt-in shared memory per block

template <int P, bool BF>
struct TcCfg {
    static constexpr int K = (P + 1) * (P + 1);
    static constexpr int KC = BF ? 2 * kKC32 : kKC32;    // K chunk (elements)
    static constexpr int KS = BF ? 16 : 8;               // K per MMA (32 bytes)
    static constexpr int KA = BF ? 2 * K : K;            // K of the A operand: [hi | lo] or one part
    static constexpr int NKC = (KA + KC - 1) / KC;       // K chunks
    static constexpr int KP = NKC * KC;                  // row length of the split expansions (elements)
    static constexpr int NA = BF ? 1 : 2;                // A tiles per stage
    static constexpr int GATHERS = NA * kRows / 4;       // gather4 copies per stage
    static constexpr int N = (K + 15) / 16 * 16;         // MMA N (multiple of 16 for M = 128)
    // An accumulator holds A [Bhi; Blo]^T (2N columns; the two halves are added
    // by the drain), so the hi and lo operator blocks are adjacent in the stage.
    static constexpr int DCOLS = (BF || M2L_WIDE_B) ? 2 * N : N;
    static constexpr int ACOL = DCOLS <= 32 ? 32 : (DCOLS <= 64 ? 64 : (DCOLS <= 128 ? 128 : 256));
    // The tile's running sums (NCH chunks of 32 columns) stay in TMEM when
    // columns are free: after both accumulators, or in the gaps behind them.
    static constexpr int NCH = (N + 31) / 32;
    static constexpr bool TOT_AFTER = 2 * ACOL + 32 * NCH <= 512;
    static constexpr int GAPCH = (ACOL - DCOLS) / 32;
    static constexpr bool TOTAL_TMEM = M2L_TMEM_TOTAL && (TOT_AFTER || 2 * GAPCH >= NCH);
    static constexpr int TMEM_COLS = TOTAL_TMEM ? 512 : 2 * ACOL;
    static constexpr uint32_t tcol(int k) {
        return static_cast<uint32_t>(TOT_AFTER ? 2 * ACOL + 32 * k : (k < GAPCH ? DCOLS + 32 * k : ACOL + DCOLS + 32 * (k - GAPCH)));
    }
    static constexpr int A_BYTES = kRows * 128;          // one A tile: 16 KB
    static constexpr int B_BYTES = N * 128;              // one of Bhi / Blo
    static constexpr int STAGE = NA * A_BYTES + 2 * B_BYTES;
    static constexpr int MAX_STAGES = BF ? M2L_MAX_STAGES_BF16 : M2L_MAX_STAGES;
    static constexpr int STAGES = (kSmemMax - 2048) / STAGE >= MAX_STAGES ? MAX_STAGES : (kSmemMax - 2048) / STAGE;  // ring depth
    static constexpr size_t SMEM = static_cast<size_t>(STAGES) * STAGE + 1024 + 256;
    // instruction descriptor: D f32 (bits 4-5 = 1), A/B bf16 (bits 7-9, 10-12 = 1,
    // kind::f16) or tf32 (= 2, kind::tf32), both K-major, N >> 3 at bits 17-22,
    // M >> 4 at bits 24-28
    static constexpr uint32_t idesc(int n) {
        return (1u << 4) | ((BF ? 1u : 2u) << 7) | ((BF ? 1u : 2u) << 10) | (static_cast<uint32_t>(n >> 3) << 17) |
               (static_cast<uint32_t>(kRows >> 4) << 24);
    }
    static constexpr uint32_t IDESC = idesc(N);
    static constexpr uint32_t IDESC_W = idesc(2 * N);
    static_assert(2 * N <= 256, "MMA N");
    static_assert(STAGES >= 3, "ring depth");
    static_assert(GATHERS % kLoaderWarps == 0, "loader warps");
    static_assert(STAGE % 1024 == 0, "stages must keep the 1024-byte swizzle atoms aligned");
    static_assert(SMEM <= static_cast<size_t>(kSmemMax), "shared memory");
};

// canonical no-swizzle K-major position of element (row, k) of a [rows x KC]
// chunk, in elements: 8-row x 16-byte core matrices (128 B), K-adjacent core
// matrices 128 B apart, 8-row groups 1024 B apart
__host__ __device__ __forceinline__ int canon(int row, int k) { return (row >> 3) * 256 + (k >> 2) * 32 + (row & 7) * 4 + (k & 3); }
__host__ __device__ __forceinline__ int canon16(int row, int k) { return (row >> 3) * 512 + (k >> 3) * 64 + (row & 7) * 8 + (k & 7); }

__device__ __forceinline__ uint32_t saddr(const void *p) { return static_cast<uint32_t>(__cvta_generic_to_shared(p)); }

__device__ __forceinline__ unsigned long long now_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(saddr(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint64_t *bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(saddr(bar)) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(saddr(bar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_test(uint64_t *bar, unsigned parity) {
    unsigned ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(saddr(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

// Bounded wait; false (and the abort flag raised) when it gives up.
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, unsigned parity, volatile int *abort_flag) {
    if (mbar_test(bar, parity)) return true;
    const unsigned long long t0 = now_ns();
    while (true) {
        if (mbar_test(bar, parity)) return true;
        if (*abort_flag) return false;
        if (now_ns() - t0 > kWaitNs) {
            *abort_flag = 1;
            return false;
        }
    }
}

__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, unsigned bytes, uint64_t *bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(saddr(dst)),
                 "l"(src), "r"(bytes), "r"(saddr(bar))
                 : "memory");
}

// Four rows (r0..r3) of a 2-D tensor, columns [x, x + box width), into dst as
// four consecutive swizzled 128-byte rows.
__device__ __forceinline__ void tma_gather4(void *dst, const CUtensorMap *map, int x, int r0, int r1, int r2, int r3,
                                            uint64_t *bar) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.tile::gather4.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, "
        "%5, %6}], [%7];" ::"r"(saddr(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(r0), "r"(r1), "r"(r2), "r"(r3), "r"(saddr(bar))
        : "memory");
}

// Shared-memory matrix descriptors. No swizzle: start address >> 4 (bits 0-13),
// LBO 128 B >> 4 (bits 16-29), SBO 1024 B >> 4 (bits 32-45), version 1 (bit 46).
__device__ __forceinline__ uint64_t sdesc(const void *p) {
    const uint64_t a = (saddr(p) & 0x3FFFFu) >> 4;
    return a | (static_cast<uint64_t>(128 >> 4) << 16) | (static_cast<uint64_t>(1024 >> 4) << 32) | (1ull << 46);
}
// 128-byte swizzle, K-major: 8-row atoms of 1024 B (SBO), layout type 2 at
// bits 61-63; LBO is not used. The start may move by 32 B steps along K
// inside an atom whose base is 1024-byte aligned.
__device__ __forceinline__ uint64_t sdesc_sw128(const void *p) {
    const uint64_t a = (saddr(p) & 0x3FFFFu) >> 4;
    return a | (1ull << 16) | (static_cast<uint64_t>(1024 >> 4) << 32) | (1ull << 46) | (2ull << 61);
}

__device__ __forceinline__ void umma_tf32(uint32_t dtmem, uint64_t ad, uint64_t bd, uint32_t idesc, uint32_t acc) {
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\ttcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}" ::"r"(dtmem),
        "l"(ad), "l"(bd), "r"(idesc), "r"(acc));
}
__device__ __forceinline__ void umma_bf16(uint32_t dtmem, uint64_t ad, uint64_t bd, uint32_t idesc, uint32_t acc) {
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\ttcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(dtmem),
        "l"(ad), "l"(bd), "r"(idesc), "r"(acc));
}
__device__ __forceinline__ void umma_commit(uint64_t *bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(saddr(bar)) : "memory");
}

__device__ __forceinline__ float tf32_hi(float x) { return __uint_as_float(__float_as_uint(x) & 0xFFFFE000u); }

__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float *v) {
    uint32_t r[32];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, "
        "%16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
          "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]),
          "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),
          "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ void tmem_st32(uint32_t taddr, const float *v) {
    asm volatile(
        "tcgen05.st.sync.aligned.32x32b.x32.b32 [%0], {%1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, %16, "
        "%17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31, %32};" ::"r"(taddr),
        "r"(__float_as_uint(v[0])), "r"(__float_as_uint(v[1])), "r"(__float_as_uint(v[2])), "r"(__float_as_uint(v[3])),
        "r"(__float_as_uint(v[4])), "r"(__float_as_uint(v[5])), "r"(__float_as_uint(v[6])), "r"(__float_as_uint(v[7])),
        "r"(__float_as_uint(v[8])), "r"(__float_as_uint(v[9])), "r"(__float_as_uint(v[10])), "r"(__float_as_uint(v[11])),
        "r"(__float_as_uint(v[12])), "r"(__float_as_uint(v[13])), "r"(__float_as_uint(v[14])), "r"(__float_as_uint(v[15])),
        "r"(__float_as_uint(v[16])), "r"(__float_as_uint(v[17])), "r"(__float_as_uint(v[18])), "r"(__float_as_uint(v[19])),
        "r"(__float_as_uint(v[20])), "r"(__float_as_uint(v[21])), "r"(__float_as_uint(v[22])), "r"(__float_as_uint(v[23])),
        "r"(__float_as_uint(v[24])), "r"(__float_as_uint(v[25])), "r"(__float_as_uint(v[26])), "r"(__float_as_uint(v[27])),
        "r"(__float_as_uint(v[28])), "r"(__float_as_uint(v[29])), "r"(__float_as_uint(v[30])), "r"(__float_as_uint(v[31]))
        : "memory");
}

// Slot s of a target with octant cls maps to same-level offset 2d + u(o') - u(cls);
// adjacent offsets are not M2L slots. Returns the operator index or -1.
__host__ __device__ __forceinline__ int slot_operator(int cls, int s) {
    const int dd = s >> 3, o = s & 7;
    const int uc0 = 1 - (cls & 1), uc1 = 1 - ((cls >> 1) & 1), uc2 = 1 - ((cls >> 2) & 1);
    const int o0 = 2 * (dd % 3 - 1) + 1 - (o & 1) - uc0;
    const int o1 = 2 * ((dd / 3) % 3 - 1) + 1 - ((o >> 1) & 1) - uc1;
    const int o2 = 2 * (dd / 9 - 1) + 1 - ((o >> 2) & 1) - uc2;
    if (o0 >= -1 && o0 <= 1 && o1 >= -1 && o1 <= 1 && o2 >= -1 && o2 <= 1) return -1;
    return (o0 + 3) + 7 * (o1 + 3) + 49 * (o2 + 3);
}

__device__ __forceinline__ int next_slot(int cls, int s) {
    while (s < kM2LSlots && slot_operator(cls, s) < 0) ++s;
    return s;
}

// Target cell of row r of tile-job w (octant w % 8, tile w / 8), or -1: one
// tree's tiles take consecutive octets; a forest's take its per-system octet
// lists (tree.cu: forest_tiles).
__device__ __forceinline__ int tc_row_cell(int w, int r, int base, int per_class, const int4 *otile, const int *oct_list) {
    const int cls = w % 8, tile = w / 8;
    if (otile) {
        const int4 ot = otile[tile];
        return r < ot.z ? base + cls + 8 * oct_list[ot.y + r] : -1;
    }
    const int t = tile * kRows + r;
    return t < per_class ? base + cls + 8 * t : -1;
}

template <int P, bool BF>
__global__ void __launch_bounds__(kThreads, M2L_MIN_BLOCKS)
    k_m2l_tc(const __grid_constant__ CUtensorMap tmap, const TreeInfo *__restrict__ info, const int *__restrict__ m2l_src,
             const unsigned char *__restrict__ bimg_all, const int4 *__restrict__ otile, const int *__restrict__ oct_list,
             int rows_cap, float *__restrict__ Lx, TreeInfo *info_rw) {
    using C = TcCfg<P, BF>;
    constexpr int kGW = C::GATHERS / kLoaderWarps;  // gather4 copies per loader warp and step
    extern __shared__ __align__(1024) unsigned char sm_raw[];
    unsigned char *sm = reinterpret_cast<unsigned char *>((reinterpret_cast<uintptr_t>(sm_raw) + 1023) & ~uintptr_t(1023));
    uint64_t *full = reinterpret_cast<uint64_t *>(sm + C::STAGES * C::STAGE);
    uint64_t *empty = full + C::STAGES;
    uint64_t *accum = empty + C::STAGES;  // [2]: group finished in accumulator a
    uint64_t *tfree = accum + 2;        // [2]: accumulator a drained
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(tfree + 2);
    volatile int *abort_flag = reinterpret_cast<volatile int *>(tmem_slot + 1);

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int base = info->level_start[2];
    const int ntgt = info->n_targets_m2l;
    const int per_class = ntgt > 0 ? ntgt / 8 : 0;
    const int tiles_per_class = otile ? info->n_otiles : (per_class + kRows - 1) / kRows;
    const int ntiles = ntgt > 0 ? 8 * tiles_per_class : 0;
    if (ntiles == 0 || static_cast<int>(blockIdx.x) >= ntiles) return;  // uniform: no barrier or TMEM touched yet

    if (tid == 0) {
        for (int s = 0; s < C::STAGES; ++s) mbar_init(full + s, kLoaderWarps), mbar_init(empty + s, 1);
        for (int a = 0; a < 2; ++a) mbar_init(accum + a, 1), mbar_init(tfree + a, kDrainThreads);
        *abort_flag = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(saddr(tmem_slot)),
                     "r"(static_cast<unsigned>(C::TMEM_COLS))
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = *tmem_slot;

    unsigned mma_steps = 0;  // steps whose MMAs the MMA thread issued
    if (warp >= 4 && warp < kMmaWarp) {
        // --------------------------------------------------------------- loaders
        // Copy G = q kGW + l (+ 32 i) of a step moves row quad G mod 32 (tile
        // rows 4(G mod 32) .. +3) of A tile G / 32 (tf32: hi, lo); absent
        // sources read the zero row. Each loader warp's lane 0 arms the stage's
        // barrier with the bytes of its own warp's copies.
        const int q = warp - 4;
        const int g0 = q * kGW + lane;
        const int quad = g0 % 32;
        const bool active = lane < kGW;
        const bool do_hi = active && (kGW >= 64 || g0 < 32);
        const bool do_lo = !BF && active && (kGW >= 64 || g0 >= 32);
        // operator bytes of chunk kc: [Bhi; Blo], or (bf16) Bhi alone for a chunk
        // of lo inputs only, whose MMAs read only the first N rows
        auto b_bytes = [](int kc) { return (BF && kc * C::KC >= C::K) ? 1u * C::B_BYTES : 2u * C::B_BYTES; };
        // absent sources read a zero row, one per row quad so that the copies
        // of many CTAs do not all meet on one L2 line
        const int zrow = rows_cap - kZeroRows + quad;
        unsigned step = 0;
        bool stop = false;
        for (int w = blockIdx.x; w < ntiles && !stop; w += gridDim.x) {
            const int cls = w % 8;
            // a forest tile's operator images are its system's
            const unsigned char *bimg =
                otile ? bimg_all + static_cast<size_t>(otile[w / 8].x) * (kNumOffsets * C::NKC * 2 * C::B_BYTES) : bimg_all;
            // rows past the tile's targets are not copied at all: their stale
            // shared-memory rows only reach accumulator rows that are never stored
            const int rows = otile ? otile[w / 8].z : min(kRows, per_class - (w / 8) * kRows);
            const bool qv = 4 * quad < rows;
            const bool t_hi = do_hi && qv, t_lo = do_lo && qv;
            const unsigned tx_bytes =
                512u * static_cast<unsigned>(__popc(__ballot_sync(0xffffffffu, t_hi)) + __popc(__ballot_sync(0xffffffffu, t_lo)));
            int crow[4];
#pragma unroll
            for (int i = 0; i < 4; ++i) crow[i] = active ? tc_row_cell(w, 4 * quad + i, base, per_class, otile, oct_list) : -1;
            auto rows_of = [&](int s, int *r) {
#pragma unroll
                for (int i = 0; i < 4; ++i) {
                    const int src = crow[i] >= 0 ? m2l_src[static_cast<size_t>(crow[i]) * kM2LSlots + s] : -1;
                    r[i] = src >= 0 ? src : zrow;
                }
            };
            int s = next_slot(cls, 0);
            int cur[4];
            rows_of(s, cur);
#if M2L_PREFETCH2
            // source rows two slots ahead: the loads of slot s + 2 are in flight
            // while slots s and s + 1 are posted
            int sn = s < kM2LSlots ? next_slot(cls, s + 1) : kM2LSlots;
            int nxt[4] = {zrow, zrow, zrow, zrow};
            if (sn < kM2LSlots) rows_of(sn, nxt);
            while (s < kM2LSlots && !stop) {
                const int oi = slot_operator(cls, s);
                const int snn = sn < kM2LSlots ? next_slot(cls, sn + 1) : kM2LSlots;
                int nxt2[4] = {zrow, zrow, zrow, zrow};
                if (snn < kM2LSlots) rows_of(snn, nxt2);
#else
            while (s < kM2LSlots && !stop) {
                const int oi = slot_operator(cls, s);
                const int sn = next_slot(cls, s + 1);
                int nxt[4] = {zrow, zrow, zrow, zrow};
                if (sn < kM2LSlots) rows_of(sn, nxt);  // in flight while this slot's copies are posted
#endif
                for (int kc = 0; kc < C::NKC; ++kc, ++step) {
                    const int st = step % C::STAGES;
                    const unsigned use = step / C::STAGES;
                    int ok = 1;
                    if (lane == 0) {
                        if (use > 0 && !mbar_wait(empty + st, (use - 1) & 1, abort_flag)) ok = 0;
                        if (ok) mbar_expect_tx(full + st, tx_bytes + (q == 0 ? b_bytes(kc) : 0u));
                    }
                    if (!__shfl_sync(0xffffffffu, ok, 0)) {
                        stop = true;
                        break;
                    }
                    unsigned char *stage = sm + st * C::STAGE;
                    if (t_hi)
                        tma_gather4(stage + 512 * quad, &tmap, kc * C::KC, cur[0], cur[1], cur[2], cur[3], full + st);
                    if (t_lo)
                        tma_gather4(stage + C::A_BYTES + 512 * quad, &tmap, kc * C::KC, cur[0] + rows_cap, cur[1] + rows_cap,
                                    cur[2] + rows_cap, cur[3] + rows_cap, full + st);
                    if (q == 0 && lane == 0)
                        bulk_g2s(stage + C::NA * C::A_BYTES, bimg + (static_cast<size_t>(oi) * C::NKC + kc) * (2 * C::B_BYTES),
                                 b_bytes(kc), full + st);
                }
#if M2L_PREFETCH2
#pragma unroll
                for (int i = 0; i < 4; ++i) cur[i] = nxt[i], nxt[i] = nxt2[i];
                s = sn;
                sn = snn;
#else
#pragma unroll
                for (int i = 0; i < 4; ++i) cur[i] = nxt[i];
                s = sn;
#endif
            }
        }
    } else if (warp == kMmaWarp) {
        // ------------------------------------------------------------------- MMA
        if (lane == 0) {
            unsigned groups = 0;
            bool stop = false;
            for (int w = blockIdx.x; w < ntiles && !stop; w += gridDim.x) {
                for (int j = 0; j < kSlotsPerTile && !stop; ++j) {
                    const int in_group = j % kGroup;
                    const unsigned a = groups & 1;
                    // a group reuses accumulator a once group - 2 has been drained
                    if (in_group == 0 && groups >= 2 && !mbar_wait(tfree + a, ((groups - 2) >> 1) & 1, abort_flag)) {
                        stop = true;
                        break;
                    }
                    const uint32_t dt = tmem + a * C::ACOL;
                    for (int kc = 0; kc < C::NKC; ++kc) {
                        const int st = mma_steps % C::STAGES;
                        const unsigned use = mma_steps / C::STAGES;
                        if (!mbar_wait(full + st, use & 1, abort_flag)) {
                            stop = true;
                            break;
                        }
                        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                        const unsigned char *stage = sm + st * C::STAGE;
                        const uint64_t ahi = sdesc_sw128(stage);
                        const unsigned char *Bhi = stage + C::NA * C::A_BYTES;
                        const unsigned char *Blo = Bhi + C::B_BYTES;
                        const int ksteps = min(C::KC / C::KS, (C::KA - kc * C::KC + C::KS - 1) / C::KS);
                        for (int ks = 0; ks < ksteps; ++ks) {
                            // 32 B along K: +2 in the swizzled start field, two
                            // core matrices (256 B) in the plain layout
                            const uint64_t bhi = sdesc(Bhi + ks * 256);
                            const uint32_t first = (in_group == 0 && kc == 0 && ks == 0) ? 0u : 1u;
                            if (BF) {
                                // [hi | lo] row: K steps that reach hi inputs take [Bhi; Blo]
                                // (2N columns), the lo half Bhi alone (N columns)
                                const bool wide = kc * C::KC + ks * C::KS < C::K;
                                umma_bf16(dt, ahi + 2 * ks, bhi, wide ? C::IDESC_W : C::IDESC, first);
                            } else {
                                const uint64_t alo = sdesc_sw128(stage + C::A_BYTES);
                                if (M2L_WIDE_B) {
                                    umma_tf32(dt, ahi + 2 * ks, bhi, C::IDESC_W, first);  // Ahi [Bhi; Blo]^T
                                } else {
                                    umma_tf32(dt, ahi + 2 * ks, bhi, C::IDESC, first);
                                    umma_tf32(dt, ahi + 2 * ks, sdesc(Blo + ks * 256), C::IDESC, 1u);
                                }
                                umma_tf32(dt, alo + 2 * ks, bhi, C::IDESC, 1u);
                            }
                        }
                        umma_commit(empty + st);
                        ++mma_steps;
                    }
                    if (stop) break;
                    if (in_group == kGroup - 1 || j == kSlotsPerTile - 1) {
                        umma_commit(accum + a);
                        ++groups;
                    }
                }
            }
        }
        __syncwarp();
    } else {
        // ----------------------------------------------------------------- drain
        unsigned groups = 0;
        bool stop = false;
        const uint32_t lanes = tmem + (static_cast<uint32_t>(32 * warp) << 16);  // TMEM lanes 32 warp .. + 31
        if (C::TOTAL_TMEM) {
            // running sums in TMEM (columns tcol(k)), added in the same order as
            // the register form below: total, then each half of the group
            for (int w = blockIdx.x; w < ntiles && !stop; w += gridDim.x) {
                for (int gi = 0; gi < kGroupsPerTile; ++gi, ++groups) {
                    if (!__all_sync(0xffffffffu, mbar_wait(accum + (groups & 1), (groups >> 1) & 1, abort_flag))) {
                        stop = true;
                        break;
                    }
                    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                    const uint32_t col = (groups & 1) * C::ACOL;
#pragma unroll 1
                    for (int k = 0; k < C::NCH; ++k) {
                        float sum[32], v[32];
                        if (gi > 0) {
                            tmem_ld32(lanes + C::tcol(k), sum);
                        } else {
#pragma unroll
                            for (int i = 0; i < 32; ++i) sum[i] = 0.f;
                        }
#pragma unroll
                        for (int h = 0; h < C::DCOLS / C::N; ++h) {
                            tmem_ld32(lanes + col + static_cast<uint32_t>(h * C::N + 32 * k), v);
#pragma unroll
                            for (int i = 0; i < 32; ++i) sum[i] += v[i];
                        }
                        tmem_st32(lanes + C::tcol(k), sum);
                    }
                    asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
                    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
                    mbar_arrive(tfree + (groups & 1));
                }
                if (stop) break;
                const int cell = tc_row_cell(w, tid, base, per_class, otile, oct_list);
                float *out = Lx + static_cast<size_t>(cell < 0 ? 0 : cell) * C::K;
#pragma unroll 1
                for (int k = 0; k < C::NCH; ++k) {
                    float sum[32];
                    tmem_ld32(lanes + C::tcol(k), sum);  // all lanes: the load is warp-collective
#pragma unroll
                    for (int i = 0; i < 32; ++i)
                        if (cell >= 0 && 32 * k + i < C::K) out[32 * k + i] = sum[i];
                }
            }
        } else {
        float acc[C::N];
        for (int w = blockIdx.x; w < ntiles && !stop; w += gridDim.x) {
#pragma unroll
            for (int i = 0; i < C::N; ++i) acc[i] = 0.f;
            for (int gi = 0; gi < kGroupsPerTile; ++gi, ++groups) {
                if (!__all_sync(0xffffffffu, mbar_wait(accum + (groups & 1), (groups >> 1) & 1, abort_flag))) {
                    stop = true;
                    break;
                }
                asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                const uint32_t col = (groups & 1) * C::ACOL;
#pragma unroll
                for (int h = 0; h < C::DCOLS / C::N; ++h)
#pragma unroll
                    for (int c0 = 0; c0 < C::N; c0 += 32) {
                        float v[32];
                        tmem_ld32(tmem + (static_cast<uint32_t>(32 * warp) << 16) + col + static_cast<uint32_t>(h * C::N + c0), v);
#pragma unroll
                        for (int i = 0; i < 32; ++i)
                            if (c0 + i < C::N) acc[c0 + i] += v[i];
                    }
                asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
                mbar_arrive(tfree + (groups & 1));
            }
            if (stop) break;
            const int cell = tc_row_cell(w, tid, base, per_class, otile, oct_list);
            if (cell >= 0) {
                float *out = Lx + static_cast<size_t>(cell) * C::K;
                for (int r = 0; r < C::K; ++r) out[r] = acc[r];
            }
        }
        }
    }
    // Orderly exit: every wait above is bounded, so all threads get here.
    if (warp == kMmaWarp && lane == 0 && mma_steps > 0) {
        // outstanding MMAs of this thread finish before the CTA may exit
        uint64_t *last = empty + ((mma_steps - 1) % C::STAGES);
        mbar_wait(last, ((mma_steps - 1) / C::STAGES) & 1, abort_flag);
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (*abort_flag) {
        if (tid == 0) atomicOr(&info_rw->err, kDevTimeout);
        // give any copy still in flight time to land before the smem is released
        const unsigned long long t0 = now_ns();
        while (now_ns() - t0 < 1000000ull) {
        }
    }
    if (warp == 0) {
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(static_cast<unsigned>(C::TMEM_COLS))
                     : "memory");
    }
}

// Split expansions for the gather; the last kZeroRows rows are zero.
// bf16: rows [0, rows_cap) of KP elements [hi(0..K-1) | lo(0..K-1) | 0].
// tf32: rows [0, rows_cap) hold the hi parts, rows [rows_cap, 2 rows_cap) the
// lo parts, KP floats each, zero beyond K.
template <int P, bool BF>
__global__ void k_split_m(const TreeInfo *__restrict__ info, const float *__restrict__ M, void *__restrict__ ms_v, int rows_cap) {
    using C = TcCfg<P, BF>;
    const int nc = min(info->ncells, rows_cap - kZeroRows);
    const size_t total = static_cast<size_t>(nc) * C::KP;
    const size_t zrow = static_cast<size_t>(rows_cap - kZeroRows) * C::KP;
    if (BF) {
        __nv_bfloat16 *ms = static_cast<__nv_bfloat16 *>(ms_v);
        for (size_t i = static_cast<size_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < total;
             i += static_cast<size_t>(gridDim.x) * blockDim.x) {
            const size_t c = i / C::KP;
            const int j = static_cast<int>(i - c * C::KP);
            const int k = j < C::K ? j : j - C::K;
            const float v = j < 2 * C::K ? M[c * C::K + k] : 0.f;
            const __nv_bfloat16 h = __float2bfloat16_rn(v);
            ms[i] = j < C::K ? h : __float2bfloat16_rn(v - __bfloat162float(h));
        }
        if (blockIdx.x == 0)
            for (int k = threadIdx.x; k < kZeroRows * C::KP; k += blockDim.x) ms[zrow + k] = __float2bfloat16_rn(0.f);
    } else {
        float *ms = static_cast<float *>(ms_v);
        float *lo = ms + static_cast<size_t>(rows_cap) * C::KP;
        for (size_t i = static_cast<size_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < total;
             i += static_cast<size_t>(gridDim.x) * blockDim.x) {
            const size_t c = i / C::KP;
            const int k = static_cast<int>(i - c * C::KP);
            const float v = k < C::K ? M[c * C::K + k] : 0.f;
            const float h = tf32_hi(v);
            ms[i] = h;
            lo[i] = v - h;
        }
        if (blockIdx.x == 0)
            for (int k = threadIdx.x; k < kZeroRows * C::KP; k += blockDim.x) ms[zrow + k] = 0.f, lo[zrow + k] = 0.f;
    }
}

// Pre-split operator images: for each same-level offset oi and K chunk kc,
// one block of 2N rows x KC elements in the canonical K-major layout, rows
// r < N the hi part and rows N + r the lo part of output coefficient r
// (zero outside K x K).
// tf32: element k of the chunk is input coefficient KC kc + k.
// bf16: element j = KC kc + k of the [hi | lo] input row is input coefficient
// j (j < K) or j - K (K <= j < 2K, the lo inputs: rows N + r are zero there).
// (A forest: blockIdx.y is the system, with its own operators and images.)
template <int P, bool BF>
__global__ void k_build_bimg(const float *__restrict__ ops_all, unsigned char *__restrict__ bimg_all) {
    using C = TcCfg<P, BF>;
    const int oi = blockIdx.x;
    const float *ops = ops_all + static_cast<size_t>(blockIdx.y) * kNumOps * C::K * C::K;
    unsigned char *bimg = bimg_all + static_cast<size_t>(blockIdx.y) * (kNumOffsets * C::NKC * 2 * C::B_BYTES);
    const int d0 = oi % 7 - 3, d1 = (oi / 7) % 7 - 3, d2 = oi / 49 - 3;
    if (d0 >= -1 && d0 <= 1 && d1 >= -1 && d1 <= 1 && d2 >= -1 && d2 <= 1) return;
    // the operator staged in shared memory by coalesced loads, then one 16-byte
    // store per thread and step: 8 bf16 or 4 tf32 consecutive K elements of a row
    extern __shared__ float op[];  // [K * K]
    for (int i = threadIdx.x; i < C::K * C::K; i += blockDim.x) op[i] = ops[static_cast<size_t>(oi) * C::K * C::K + i];
    __syncthreads();
    constexpr int VE = BF ? 8 : 4;
    constexpr int RUNS = C::KC / VE;
    for (int kc = 0; kc < C::NKC; ++kc) {
        unsigned char *blk = bimg + (static_cast<size_t>(oi) * C::NKC + kc) * (2 * C::B_BYTES);
        // bf16: a chunk of lo inputs only is copied without its Blo rows (they
        // would be zero there), so they are not written either. Rows of output
        // coefficients past K are not written (they only reach accumulator
        // columns the drain never stores); the K columns are all written.
        const int rows = (BF && kc * C::KC >= C::K) ? C::K : 2 * C::K;
        for (int u = threadIdx.x; u < rows * RUNS; u += blockDim.x) {
            const int vr = u / RUNS, k0 = (u % RUNS) * VE;
            const bool lo_row = vr >= C::K;
            const int ro = lo_row ? vr - C::K : vr;
            const int r = lo_row ? C::N + ro : ro;
            float v[VE];
#pragma unroll
            for (int e = 0; e < VE; ++e) {
                const int j = kc * C::KC + k0 + e;
                int ci = j;
                bool use = j < C::K;
                if (BF && j >= C::K && j < 2 * C::K) ci = j - C::K, use = !lo_row;
                v[e] = (use && ro < C::K) ? op[ro * C::K + ci] : 0.f;
            }
            if (BF) {
                __align__(16) __nv_bfloat16 o[8];
#pragma unroll
                for (int e = 0; e < VE; ++e) {
                    const __nv_bfloat16 h = __float2bfloat16_rn(v[e]);
                    o[e] = lo_row ? __float2bfloat16_rn(v[e] - __bfloat162float(h)) : h;
                }
                *reinterpret_cast<uint4 *>(reinterpret_cast<__nv_bfloat16 *>(blk) + canon16(r, k0)) = *reinterpret_cast<const uint4 *>(o);
            } else {
                float4 o;
                float *of = &o.x;
#pragma unroll
                for (int e = 0; e < VE; ++e) {
                    const float h = tf32_hi(v[e]);
                    of[e] = lo_row ? v[e] - h : h;
                }
                float *f = reinterpret_cast<float *>(blk) + (lo_row ? C::N * C::KC : 0);
                *reinterpret_cast<float4 *>(f + canon(ro, k0)) = o;
            }
        }
    }
}

template <int P, bool BF>
void launch(Workspace &ws) {
    using C = TcCfg<P, BF>;
    const bool forest = ws.forest();
    const int op_smem = static_cast<int>(sizeof(float) * C::K * C::K);
    if (op_smem > 48 * 1024)
        cudaFuncSetAttribute(k_build_bimg<P, BF>, cudaFuncAttributeMaxDynamicSharedMemorySize, op_smem);
    k_build_bimg<P, BF><<<dim3(kNumOffsets, forest ? ws.nsys : 1), 256, op_smem, ws.st>>>(ws.ops_f,
                                                                                 reinterpret_cast<unsigned char *>(ws.bimg));
    k_split_m<P, BF><<<4 * ws.num_sms, 256, 0, ws.st>>>(ws.info, static_cast<const float *>(ws.Mexp), ws.ms_tc,
                                                        static_cast<int>(ws.ms_rows));
    cudaFuncSetAttribute(k_m2l_tc<P, BF>, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(C::SMEM));
    const unsigned ctas = std::max(1u, static_cast<unsigned>(ws.num_sms * ws.m2l_ctas_pct / 100));
    const unsigned gs = capped_grid(ctas, 8 * (ceil_div(ceil_div(ws.c_cap, 8), kRows) + (forest ? ws.nsys : 0)));  // tiles
    k_m2l_tc<P, BF><<<gs, kThreads, C::SMEM, ws.st>>>(ws.tmap_ms, ws.info, ws.m2l_src,
                                                      reinterpret_cast<const unsigned char *>(ws.bimg),
                                                      forest ? ws.otile : nullptr, ws.oct_list,
                                                      static_cast<int>(ws.ms_rows), static_cast<float *>(ws.Lexp), ws.info);
    ws.launches += 3;
}

template <int P>
void launch_kind(Workspace &ws) {
    if (ws.m2l_bf16)
        launch<P, true>(ws);
    else
        launch<P, false>(ws);
}

using EncodeTiled = CUresult (*)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                 const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                 CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

}  // namespace

// Both forms: 343 offsets x NKC chunks x 2N rows x 128 B, with NKC =
// ceil(K / 32) (tf32) = ceil(2K / 64) (bf16).
size_t m2l_tc_image_floats(int p) {
    const int K = (p + 1) * (p + 1);
    const int NKC = (K + kKC32 - 1) / kKC32, N = (K + 15) / 16 * 16;
    return static_cast<size_t>(343) * NKC * 2 * N * kKC32;
}

// 4-byte units per split row: tf32 KP floats (hi or lo); bf16 [hi | lo] rows
// of 2 KP bf16 take the same bytes, in one half of the tf32 allocation.
int m2l_tc_row_floats(int p) {
    const int K = (p + 1) * (p + 1);
    return (K + kKC32 - 1) / kKC32 * kKC32;
}

bool m2l_tc_supported(int p) { return p >= 2 && p <= kMaxP; }

const char *m2l_tc_encode(Workspace &ws) {
    static EncodeTiled encode = nullptr;
    if (!encode) {
        void *fn = nullptr;
        cudaDriverEntryPointQueryResult q{};
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) != cudaSuccess ||
            q != cudaDriverEntryPointSuccess || !fn)
            return "cuTensorMapEncodeTiled is not available";
        encode = reinterpret_cast<EncodeTiled>(fn);
    }
    // bf16: ms_rows rows of 2 ms_kp elements; tf32: 2 ms_rows rows (hi, lo) of
    // ms_kp floats. Rows are ms_kp * 4 bytes either way; boxes are one row
    // (gather4) of 128 bytes.
    const bool bf = ws.m2l_bf16;
    const cuuint64_t dims[2] = {static_cast<cuuint64_t>(bf ? 2 * ws.ms_kp : ws.ms_kp), (bf ? 1ull : 2ull) * ws.ms_rows};
    const cuuint64_t strides[1] = {static_cast<cuuint64_t>(ws.ms_kp) * sizeof(float)};
    const cuuint32_t box[2] = {static_cast<cuuint32_t>(bf ? 2 * kKC32 : kKC32), 1u};
    const cuuint32_t estr[2] = {1u, 1u};
    const CUresult r = encode(&ws.tmap_ms, bf ? CU_TENSOR_MAP_DATA_TYPE_BFLOAT16 : CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, ws.ms_tc,
                              dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                              CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return "cuTensorMapEncodeTiled rejected the split-expansion tensor";
    ws.ms_bf16 = bf;
    return nullptr;
}

void m2l_pass_tc(Workspace &ws) {
    timer_begin(ws, kTM2L);
    switch (ws.p) {
        case 2: launch_kind<2>(ws); break;
        case 3: launch_kind<3>(ws); break;
        case 4: launch_kind<4>(ws); break;
        case 5: launch_kind<5>(ws); break;
        case 6: launch_kind<6>(ws); break;
        case 7: launch_kind<7>(ws); break;
        case 8: launch_kind<8>(ws); break;
        case 9: launch_kind<9>(ws); break;
        case 10: launch_kind<10>(ws); break;
        default: break;
    }
    timer_end(ws, kTM2L);
}

}  // namespace gb
