// M2L on the 5th-generation tensor cores (tcgen05, sm_103a), mixed precision.
//
// Same work as k_m2l in fmm.cu (fmm.hpp:277-304 restated on scaled real-basis
// expansions): every target cell at level >= 2 gathers the expansions of its
// up-to-189 interaction-list sources and applies one K x K operator per
// source offset. Targets sharing an octant share the slot -> offset map, so a
// tile of 128 same-octant targets is, per slot, one GEMM
//     D[128 x N] += A[128 x K] * B[N x K]^T,  A = gathered source rows,
//                                             B = the slot's operator,
// accumulated over all slots in TMEM (128 lanes x N FP32 columns).
//
// Precision: kind::tf32 with a three-term split (hi = FP32 with the low 13
// mantissa bits cleared, lo = x - hi):  D += Ahi Bhi + Ahi Blo + Alo Bhi,
// which carries ~2^-21 relative error per product, FP32 accumulation.
//
// Accumulation: the tensor core's FP32 accumulation adds an error that grows
// with the number of MMAs summed into one accumulator (measured: RMS error
// proportional to the chain length, 1.5e-5 relative on the accelerations with
// all ~6000 MMAs of a tile in one accumulator). Slots are therefore grouped,
// kGroup slots per group, into one of two TMEM accumulators used in turn; the
// producer warps drain each finished group into FP32 registers (round-to-
// nearest additions) while the next group accumulates.
//
// Pipeline (one CTA per SM, persistent over tiles): K is cut into 32-wide
// chunks; each (slot, chunk) step goes through one of C::STAGES shared-memory
// stages holding A hi/lo [128 x 32] and B hi/lo [N x 32] in the canonical
// no-swizzle K-major layout (8-row x 16-byte core matrices; LBO = 128 B along
// K, SBO = 1024 B between 8-row groups). B chunks are stored pre-split in that
// exact image in global memory and arrive by one cp.async.bulk; warps 0-3
// gather and split the A rows; warp 4 issues the MMAs (one elected thread)
// and commits each stage back to its producers. Warps 0-3 then read their 32
// TMEM lanes of D (tcgen05.ld) and write the local expansions.
//
// Every mbarrier wait is bounded by the global timer; on a timeout the CTA
// records kDevTimeout in the status word, stops issuing work, waits (bounded)
// for its own bulk copies and MMAs, frees its TMEM and returns.
#include "workspace.cuh"

namespace gb {

namespace {

constexpr int kRows = 128;          // targets per tile (MMA M)
constexpr int kKC = 32;             // K chunk (tf32 elements)
constexpr int kProducers = 128;     // warps 0-3
constexpr int kThreads = 160;       // + issuer warp 4
constexpr unsigned long long kWaitNs = 2000000000ull;  // 2 s per wait
constexpr int kGroup = 4;           // slots per TMEM accumulation group
constexpr int kSmemMax = 232448;    // opt-in shared memory per block

template <int P>
struct TcCfg {
    static constexpr int K = (P + 1) * (P + 1);
    static constexpr int NKC = (K + kKC - 1) / kKC;      // K chunks
    static constexpr int N = (K + 15) / 16 * 16;         // MMA N (multiple of 16 for M = 128)
    static constexpr int ACOL = N <= 32 ? 32 : (N <= 64 ? 64 : 128);  // columns of one accumulator
    static constexpr int TMEM_COLS = 2 * ACOL;
    static constexpr int A_BYTES = kRows * kKC * 4;      // one of hi/lo
    static constexpr int B_BYTES = N * kKC * 4;
    static constexpr int STAGE = 2 * A_BYTES + 2 * B_BYTES;
    static constexpr int STAGES = (kSmemMax - 1280) / STAGE >= 4 ? 4 : 3;  // ring depth
    static constexpr size_t SMEM = static_cast<size_t>(STAGES) * STAGE + 1024 + 256;
    // instruction descriptor: D f32 (bits 4-5 = 1), A/B tf32 (bits 7-9, 10-12 = 2),
    // both K-major, N >> 3 at bits 17-22, M >> 4 at bits 24-28
    static constexpr uint32_t IDESC = (1u << 4) | (2u << 7) | (2u << 10) | (static_cast<uint32_t>(N >> 3) << 17) |
                                      (static_cast<uint32_t>(kRows >> 4) << 24);
};

// canonical no-swizzle K-major position (in floats) of element (row, k) of a [rows x 32] chunk
__host__ __device__ __forceinline__ int canon(int row, int k) { return (row >> 3) * 256 + (k >> 2) * 32 + (row & 7) * 4 + (k & 3); }

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

__device__ __forceinline__ uint64_t sdesc(const void *p) {
    // start address >> 4 (bits 0-13), LBO 128 B >> 4 (bits 16-29), SBO 1024 B >> 4
    // (bits 32-45), descriptor version 1 (bit 46), no swizzle (bits 61-63 = 0)
    const uint64_t a = (saddr(p) & 0x3FFFFu) >> 4;
    return a | (static_cast<uint64_t>(128 >> 4) << 16) | (static_cast<uint64_t>(1024 >> 4) << 32) | (1ull << 46);
}

__device__ __forceinline__ void umma_tf32(uint32_t dtmem, uint64_t ad, uint64_t bd, uint32_t idesc, uint32_t acc) {
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\ttcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}" ::"r"(dtmem),
        "l"(ad), "l"(bd), "r"(idesc), "r"(acc));
}
__device__ __forceinline__ void umma_commit(uint64_t *bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(saddr(bar)) : "memory");
}

// OR of a predicate over the 128 producer threads (named barrier 1).
__device__ __forceinline__ bool bar_or(bool pred) {
    unsigned r;
    asm volatile("{\n\t.reg .pred p, q;\n\tsetp.ne.u32 p, %1, 0;\n\tbar.red.or.pred q, 1, 128, p;\n\tselp.u32 %0, 1, 0, q;\n\t}"
                 : "=r"(r)
                 : "r"(static_cast<unsigned>(pred))
                 : "memory");
    return r != 0;
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

// Slot s of a target with octant cls maps to same-level offset 2d + u(o') - u(cls);
// adjacent offsets are not M2L slots. Returns the operator index or -1.
__device__ __forceinline__ int slot_operator(int cls, int s) {
    const int dd = s >> 3, o = s & 7;
    const int uc0 = 1 - (cls & 1), uc1 = 1 - ((cls >> 1) & 1), uc2 = 1 - ((cls >> 2) & 1);
    const int o0 = 2 * (dd % 3 - 1) + 1 - (o & 1) - uc0;
    const int o1 = 2 * ((dd / 3) % 3 - 1) + 1 - ((o >> 1) & 1) - uc1;
    const int o2 = 2 * (dd / 9 - 1) + 1 - ((o >> 2) & 1) - uc2;
    if (o0 >= -1 && o0 <= 1 && o1 >= -1 && o1 <= 1 && o2 >= -1 && o2 <= 1) return -1;
    return (o0 + 3) + 7 * (o1 + 3) + 49 * (o2 + 3);
}

template <int P>
__global__ void __launch_bounds__(kThreads, 1) k_m2l_tc(const TreeInfo *__restrict__ info, const int *__restrict__ m2l_src,
                                                        const float *__restrict__ bimg, const float *__restrict__ M,
                                                        float *__restrict__ Lx, TreeInfo *info_rw) {
    using C = TcCfg<P>;
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
    const int tiles_per_class = (per_class + kRows - 1) / kRows;
    const int ntiles = 8 * tiles_per_class;
    if (ntiles == 0 || static_cast<int>(blockIdx.x) >= ntiles) return;  // uniform: no barrier or TMEM touched yet

    if (tid == 0) {
        for (int s = 0; s < C::STAGES; ++s) mbar_init(full + s, kProducers + 1), mbar_init(empty + s, 1);
        for (int a = 0; a < 2; ++a) mbar_init(accum + a, 1), mbar_init(tfree + a, kProducers);
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

    unsigned step = 0;     // (slot, chunk) steps of this CTA so far
    unsigned groups = 0;   // accumulation groups of this CTA so far (group g uses accumulator g % 2)
    if (warp < 4) {
        // ------------------------------------------------ producers + epilogue
        // `stop` only changes through bar_or over all 128 producers, so every
        // producer takes the same path through the named barrier.
        bool stop = false;
        unsigned drained = 0;  // groups drained so far
        float acc[C::N];
        // Drain group g: wait for its last MMA, add its accumulator to acc.
        auto drain = [&](unsigned g) -> bool {
            const bool ok = __all_sync(0xffffffffu, mbar_wait(accum + (g & 1), (g >> 1) & 1, abort_flag));
            if (ok) {
                asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                const uint32_t base_col = (g & 1) * C::ACOL;
#pragma unroll
                for (int c0 = 0; c0 < C::N; c0 += 32) {
                    float v[32];
                    tmem_ld32(tmem + (static_cast<uint32_t>(32 * warp) << 16) + base_col + static_cast<uint32_t>(c0), v);
#pragma unroll
                    for (int i = 0; i < 32; ++i)
                        if (c0 + i < C::N) acc[c0 + i] += v[i];
                }
                asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
            }
            mbar_arrive(tfree + (g & 1));
            return ok;
        };
        for (int w = blockIdx.x; w < ntiles && !stop; w += gridDim.x) {
            const int cls = w % 8, t0 = (w / 8) * kRows;
            const int t = t0 + tid;
            const int crow = t < per_class ? base + cls + 8 * t : -1;
#pragma unroll
            for (int i = 0; i < C::N; ++i) acc[i] = 0.f;
            const unsigned tile_groups = groups;
            int in_group = 0;
            for (int s = 0; s < kM2LSlots; ++s) {
                if (slot_operator(cls, s) < 0) continue;
                const int src = crow >= 0 ? m2l_src[static_cast<size_t>(crow) * kM2LSlots + s] : -1;
                const bool any = bar_or(src >= 0);
                stop = bar_or(*abort_flag != 0);
                if (stop) break;
                if (!any) continue;
                for (int kc = 0; kc < C::NKC; ++kc, ++step) {
                    const int st = step % C::STAGES;
                    const unsigned use = step / C::STAGES;
                    if (use > 0 && !mbar_wait(empty + st, (use - 1) & 1, abort_flag)) break;
                    float *Ahi = reinterpret_cast<float *>(sm + st * C::STAGE);
                    float *Alo = Ahi + kRows * kKC;
                    const float *row = src >= 0 ? M + static_cast<size_t>(src) * C::K : nullptr;
#pragma unroll 4
                    for (int k4 = 0; k4 < kKC; k4 += 4) {
                        float v[4];
#pragma unroll
                        for (int e = 0; e < 4; ++e) {
                            const int ci = kc * kKC + k4 + e;
                            v[e] = (row && ci < C::K) ? row[ci] : 0.f;
                        }
                        float4 h, l;
                        h.x = tf32_hi(v[0]), h.y = tf32_hi(v[1]), h.z = tf32_hi(v[2]), h.w = tf32_hi(v[3]);
                        l.x = v[0] - h.x, l.y = v[1] - h.y, l.z = v[2] - h.z, l.w = v[3] - h.w;
                        *reinterpret_cast<float4 *>(Ahi + canon(tid, k4)) = h;
                        *reinterpret_cast<float4 *>(Alo + canon(tid, k4)) = l;
                    }
                    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                    mbar_arrive(full + st);
                }
                // After queueing the first slot of a group, drain the previous
                // group of this tile (its MMAs overlap with the queued ones).
                if (in_group == 0 && groups > tile_groups && drained < groups) {
                    if (!drain(drained)) break;
                    ++drained;
                }
                if (++in_group == kGroup) in_group = 0, ++groups;
            }
            if (in_group > 0) ++groups;  // the tile's last, partial group
            if (!stop) stop = bar_or(*abort_flag != 0);
            if (stop) break;
            bool ok = true;
            while (drained < groups && ok) ok = drain(drained++);
            if (crow >= 0 && ok)
                for (int r = 0; r < C::K; ++r) Lx[static_cast<size_t>(crow) * C::K + r] = groups > tile_groups ? acc[r] : 0.f;
            stop = bar_or(*abort_flag != 0);
        }
    } else {
        // ------------------------------------------------------------ issuer
        // The whole warp scans the tile's sources of a slot; lane 0 alone
        // posts the bulk copies, issues the MMAs and commits.
        bool stop = false;
        for (int w = blockIdx.x; w < ntiles && !stop; w += gridDim.x) {
            const int cls = w % 8, t0 = (w / 8) * kRows;
            int in_group = 0;
            bool acc_on = false;
            for (int s = 0; s < kM2LSlots && !stop; ++s) {
                const int oi = slot_operator(cls, s);
                if (oi < 0) continue;
                bool mine = false;
                for (int r = lane; r < kRows; r += 32) {
                    const int t = t0 + r;
                    if (t < per_class && m2l_src[static_cast<size_t>(base + cls + 8 * t) * kM2LSlots + s] >= 0) mine = true;
                }
                if (!__any_sync(0xffffffffu, mine)) continue;
                int ok = 1;
                if (lane == 0) {
                    const unsigned a = groups & 1;
                    // a new group reuses accumulator a once group - 2 has been drained
                    if (in_group == 0 && groups >= 2 && !mbar_wait(tfree + a, ((groups - 2) >> 1) & 1, abort_flag)) ok = 0;
                    if (in_group == 0) acc_on = false;
                    const uint32_t dt = tmem + a * C::ACOL;
                    for (int kc = 0; kc < C::NKC && ok; ++kc, ++step) {
                        const int st = step % C::STAGES;
                        const unsigned use = step / C::STAGES;
                        if (use > 0 && !mbar_wait(empty + st, (use - 1) & 1, abort_flag)) {
                            ok = 0;
                            break;
                        }
                        unsigned char *stage = sm + st * C::STAGE;
                        float *Bhi = reinterpret_cast<float *>(stage + 2 * C::A_BYTES);
                        mbar_expect_tx(full + st, 2 * C::B_BYTES);
                        bulk_g2s(Bhi, bimg + (static_cast<size_t>(oi) * C::NKC + kc) * (2 * C::N * kKC), 2 * C::B_BYTES,
                                 full + st);
                        if (!mbar_wait(full + st, use & 1, abort_flag)) {
                            ok = 0;
                            break;
                        }
                        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                        const float *Ahi = reinterpret_cast<const float *>(stage);
                        const float *Alo = Ahi + kRows * kKC;
                        const float *Blo = Bhi + C::N * kKC;
                        const int ksteps = min(kKC / 8, (C::K - kc * kKC + 7) / 8);
                        for (int ks = 0; ks < ksteps; ++ks) {
                            const int off = ks * 64;  // 8 tf32 = two core matrices along K = 64 floats
                            umma_tf32(dt, sdesc(Ahi + off), sdesc(Bhi + off), C::IDESC, acc_on ? 1u : 0u);
                            acc_on = true;
                            umma_tf32(dt, sdesc(Ahi + off), sdesc(Blo + off), C::IDESC, 1u);
                            umma_tf32(dt, sdesc(Alo + off), sdesc(Bhi + off), C::IDESC, 1u);
                        }
                        umma_commit(empty + st);
                    }
                    if (*abort_flag) ok = 0;
                    if (ok && in_group + 1 == kGroup) umma_commit(accum + a);
                }
                if (++in_group == kGroup) in_group = 0, ++groups;
                stop = __shfl_sync(0xffffffffu, ok, 0) == 0;
            }
            if (!stop && in_group > 0) {
                if (lane == 0) umma_commit(accum + (groups & 1));
                ++groups;
            }
        }
    }
    // Orderly exit: every wait above is bounded, so all threads get here.
    if (warp == 4 && lane == 0 && step > 0) {
        // outstanding MMAs of this thread finish before the CTA may exit
        uint64_t *last = empty + ((step - 1) % C::STAGES);
        mbar_wait(last, ((step - 1) / C::STAGES) & 1, abort_flag);
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (*abort_flag) {
        if (tid == 0) atomicOr(&info_rw->err, kDevTimeout);
        // give any bulk copy still in flight time to land before the smem is released
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

// Pre-split operator images: for each same-level offset oi and K chunk kc,
// [hi | lo], each N x 32 floats in the canonical K-major layout (rows = output
// coefficient r, k = input coefficient 32 kc + k); zero outside K x K.
template <int P>
__global__ void k_build_bimg(const double *__restrict__ ops_d, float *__restrict__ bimg) {
    using C = TcCfg<P>;
    const int oi = blockIdx.x;
    const int d0 = oi % 7 - 3, d1 = (oi / 7) % 7 - 3, d2 = oi / 49 - 3;
    if (d0 >= -1 && d0 <= 1 && d1 >= -1 && d1 <= 1 && d2 >= -1 && d2 <= 1) return;
    for (int kc = 0; kc < C::NKC; ++kc) {
        float *hi = bimg + (static_cast<size_t>(oi) * C::NKC + kc) * (2 * C::N * kKC);
        float *lo = hi + C::N * kKC;
        for (int i = threadIdx.x; i < C::N * kKC; i += blockDim.x) {
            const int r = i / kKC, k = i % kKC, ci = kc * kKC + k;
            const float v = (r < C::K && ci < C::K) ? static_cast<float>(ops_d[(static_cast<size_t>(oi) * C::K + r) * C::K + ci]) : 0.f;
            const float h = tf32_hi(v);
            hi[canon(r, k)] = h;
            lo[canon(r, k)] = v - h;
        }
    }
}

template <int P>
void launch(Workspace &ws) {
    using C = TcCfg<P>;
    k_build_bimg<P><<<343, 256, 0, ws.st>>>(ws.ops_d, ws.bimg);
    cudaFuncSetAttribute(k_m2l_tc<P>, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(C::SMEM));
    k_m2l_tc<P><<<ws.num_sms, kThreads, C::SMEM, ws.st>>>(ws.info, ws.m2l_src, ws.bimg, static_cast<const float *>(ws.Mexp),
                                                         static_cast<float *>(ws.Lexp), ws.info);
    ws.launches += 2;
}

}  // namespace

size_t m2l_tc_image_floats(int p) {
    const int K = (p + 1) * (p + 1);
    const int NKC = (K + kKC - 1) / kKC, N = (K + 15) / 16 * 16;
    return static_cast<size_t>(343) * NKC * 2 * N * kKC;
}

bool m2l_tc_supported(int p) { return p >= 2 && p <= kMaxP; }

void m2l_pass_tc(Workspace &ws) {
    timer_begin(ws, kTM2L);
    switch (ws.p) {
        case 2: launch<2>(ws); break;
        case 3: launch<3>(ws); break;
        case 4: launch<4>(ws); break;
        case 5: launch<5>(ws); break;
        case 6: launch<6>(ws); break;
        case 7: launch<7>(ws); break;
        case 8: launch<8>(ws); break;
        case 9: launch<9>(ws); break;
        case 10: launch<10>(ws); break;
        default: break;
    }
    timer_end(ws, kTM2L);
}

}  // namespace gb
