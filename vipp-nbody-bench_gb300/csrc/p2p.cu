// Near field (P2P, gravity/include/fmm.hpp:377-385, 513-540) and the FP64
// direct-sum oracle (solver_ref_naive.hpp:103-119) on the GPU.
//
// Work decomposition: every leaf is cut into chunks of 32 targets; a
// persistent grid of warps pulls chunks from a device counter (work queue).
// A warp streams the leaf's near-field source ranges through shared memory
// 32 sources at a time; every lane owns one target and visits the staged
// sources in the same order (broadcast shared-memory reads).
//
// Mixed precision (FP32): positions are kept as hi + lo float pairs relative
// to the root-box centre; targets and staged sources are re-expressed relative
// to the target leaf's centre ((hi - c_hi) + (lo - c_lo)), so FP32 differences
// carry ~1e-7 of the neighbourhood size rather than of the coordinate.
// Pair term: rsqrt, optional Newton step, m r^-3 d; per-batch FP32 partial
// sums folded into a compensated (Kahan) per-target accumulator. The
// reference's factor G multiplies the near field only (fmm.hpp:539).
#include "direct.cuh"
#include "workspace.cuh"

namespace gb {

namespace {

constexpr int kP2PWarps = 4;

struct RootC {
    float hx, hy, hz, lx, ly, lz;
};

__device__ __forceinline__ RootC leaf_centre(const double *c_ctr, int c, const TreeInfo *info) {
    RootC r;
    const double d0 = c_ctr[3 * c] - (info->root_min[0] + info->root_max[0]) / 2;
    const double d1 = c_ctr[3 * c + 1] - (info->root_min[1] + info->root_max[1]) / 2;
    const double d2 = c_ctr[3 * c + 2] - (info->root_min[2] + info->root_max[2]) / 2;
    r.hx = static_cast<float>(d0), r.hy = static_cast<float>(d1), r.hz = static_cast<float>(d2);
    r.lx = static_cast<float>(d0 - r.hx), r.ly = static_cast<float>(d1 - r.hy), r.lz = static_cast<float>(d2 - r.hz);
    return r;
}

template <bool kNewton, bool kSoft>
__global__ void __launch_bounds__(kP2PWarps * 32) k_p2p_f32(const int2 *__restrict__ chunks, const unsigned *counts,
                                                            unsigned *queue, const int *__restrict__ leaves,
                                                            const int *__restrict__ c_end, const double *__restrict__ c_ctr,
                                                            const TreeInfo *__restrict__ info, const unsigned *__restrict__ rng_off,
                                                            const unsigned *__restrict__ rng_len, const uint2 *__restrict__ ranges,
                                                            const float4 *__restrict__ ph, const float4 *__restrict__ pl,
                                                            float G, float eps2, float *__restrict__ nearv, unsigned n) {
    __shared__ float4 src[kP2PWarps][32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const unsigned nch = counts[5];
    while (true) {
        unsigned ci = 0;
        if (lane == 0) ci = atomicAdd(queue, 1u);
        ci = __shfl_sync(0xffffffffu, ci, 0);
        if (ci >= nch) break;
        const int2 ch = chunks[ci];
        const int li = ch.x;
        const int c = leaves[li];
        const int te = c_end[c];
        const int i = ch.y + lane;
        const bool act = i < te;
        const RootC cc = leaf_centre(c_ctr, c, info);
        float tx = 0, ty = 0, tz = 0;
        if (act) {
            const float4 h = ph[i], l = pl[i];
            tx = (h.x - cc.hx) + (l.x - cc.lx);
            ty = (h.y - cc.hy) + (l.y - cc.ly);
            tz = (h.z - cc.hz) + (l.z - cc.lz);
        }
        float sx = 0, sy = 0, sz = 0, kx = 0, ky = 0, kz = 0;  // Kahan sums and compensations
        const unsigned r0 = rng_off[li], nr = rng_len[li];
        for (unsigned r = 0; r < nr; ++r) {
            const uint2 rg = ranges[r0 + r];
            for (unsigned b = rg.x; b < rg.y; b += 32) {
                const unsigned j = b + lane;
                const unsigned cnt = min(32u, rg.y - b);
                if (j < rg.y) {
                    const float4 h = ph[j], l = pl[j];
                    src[w][lane] = make_float4((h.x - cc.hx) + (l.x - cc.lx), (h.y - cc.hy) + (l.y - cc.ly),
                                               (h.z - cc.hz) + (l.z - cc.lz), h.w);
                }
                __syncwarp();
                float bx = 0, by = 0, bz = 0;
#pragma unroll 8
                for (unsigned k = 0; k < cnt; ++k) {
                    const float4 s = src[w][k];
                    const float dx = s.x - tx, dy = s.y - ty, dz = s.z - tz;
                    const float r2 = fmaf(dx, dx, fmaf(dy, dy, fmaf(dz, dz, eps2)));
                    float ri = rsqrtf(r2);
                    if (kNewton) ri = ri * fmaf(-0.5f * r2 * ri, ri, 1.5f);
                    if (!kSoft) ri = r2 > 0.f ? ri : 0.f;
                    const float mr = s.w * ri;
                    const float f = mr * (ri * ri);
                    bx = fmaf(dx, f, bx);
                    by = fmaf(dy, f, by);
                    bz = fmaf(dz, f, bz);
                }
                __syncwarp();
                {
                    float y = bx - kx, t = sx + y;
                    kx = (t - sx) - y, sx = t;
                    y = by - ky, t = sy + y;
                    ky = (t - sy) - y, sy = t;
                    y = bz - kz, t = sz + y;
                    kz = (t - sz) - y, sz = t;
                }
            }
        }
        if (act) {
            nearv[i] = G * sx;
            nearv[n + i] = G * sy;
            nearv[2 * static_cast<size_t>(n) + i] = G * sz;
        }
    }
}

template <bool kSoft>
__global__ void __launch_bounds__(kP2PWarps * 32) k_p2p_f64(const int2 *__restrict__ chunks, const unsigned *counts,
                                                            unsigned *queue, const int *__restrict__ leaves,
                                                            const int *__restrict__ c_end, const unsigned *__restrict__ rng_off,
                                                            const unsigned *__restrict__ rng_len, const uint2 *__restrict__ ranges,
                                                            const double *__restrict__ xs, double Gm, double eps2,
                                                            double *__restrict__ nearv, unsigned n) {
    __shared__ double src[kP2PWarps][3][32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const unsigned nch = counts[5];
    while (true) {
        unsigned ci = 0;
        if (lane == 0) ci = atomicAdd(queue, 1u);
        ci = __shfl_sync(0xffffffffu, ci, 0);
        if (ci >= nch) break;
        const int2 ch = chunks[ci];
        const int li = ch.x;
        const int c = leaves[li];
        const int te = c_end[c];
        const int i = ch.y + lane;
        const bool act = i < te;
        const double tx = act ? xs[i] : 0.0, ty = act ? xs[n + i] : 0.0, tz = act ? xs[2 * static_cast<size_t>(n) + i] : 0.0;
        double ax = 0, ay = 0, az = 0;
        const unsigned r0 = rng_off[li], nr = rng_len[li];
        for (unsigned r = 0; r < nr; ++r) {
            const uint2 rg = ranges[r0 + r];
            for (unsigned b = rg.x; b < rg.y; b += 32) {
                const unsigned j = b + lane;
                const unsigned cnt = min(32u, rg.y - b);
                if (j < rg.y) {
                    src[w][0][lane] = xs[j];
                    src[w][1][lane] = xs[n + j];
                    src[w][2][lane] = xs[2 * static_cast<size_t>(n) + j];
                }
                __syncwarp();
                for (unsigned k = 0; k < cnt; ++k) {
                    const double dx = src[w][0][k] - tx, dy = src[w][1][k] - ty, dz = src[w][2][k] - tz;
                    const double r2 = dx * dx + dy * dy + dz * dz + eps2;
                    double ri = rsqrt(r2);
                    if (!kSoft) ri = r2 > 0.0 ? ri : 0.0;
                    const double f = Gm * ri * ri * ri;
                    ax += f * dx;
                    ay += f * dy;
                    az += f * dz;
                }
                __syncwarp();
            }
        }
        if (act) {
            nearv[i] = ax;
            nearv[n + i] = ay;
            nearv[2 * static_cast<size_t>(n) + i] = az;
        }
    }
}

}  // namespace

bool g_p2p_newton = true;

void p2p_pass(Workspace &ws) {
    timer_begin(ws, kTP2P);
    cudaMemsetAsync(ws.queue, 0, sizeof(unsigned), ws.st);
    const unsigned gs = static_cast<unsigned>(ws.num_sms) * 8;
    const bool soft = ws.eps > 0;
    if (ws.mixed) {
        const float eps2 = static_cast<float>(ws.eps * ws.eps);
        const float G = static_cast<float>(ws.G);
        auto *o = static_cast<float *>(ws.nearf);
#define GB_P2P32(NW, SF)                                                                                                \
    k_p2p_f32<NW, SF><<<gs, kP2PWarps * 32, 0, ws.st>>>(ws.chunks, ws.d_counts, ws.queue, ws.leaves, ws.c_end, ws.c_ctr, \
                                                        ws.info, ws.rng_off, ws.rng_len, ws.ranges, ws.ph, ws.pl, G, eps2, o, ws.n)
        if (g_p2p_newton) {
            if (soft)
                GB_P2P32(true, true);
            else
                GB_P2P32(true, false);
        } else {
            if (soft)
                GB_P2P32(false, true);
            else
                GB_P2P32(false, false);
        }
#undef GB_P2P32
    } else {
        const double Gm = ws.G * ws.m, eps2 = ws.eps * ws.eps;
        auto *o = static_cast<double *>(ws.nearf);
        if (soft)
            k_p2p_f64<true><<<gs, kP2PWarps * 32, 0, ws.st>>>(ws.chunks, ws.d_counts, ws.queue, ws.leaves, ws.c_end, ws.rng_off,
                                                              ws.rng_len, ws.ranges, ws.xs, Gm, eps2, o, ws.n);
        else
            k_p2p_f64<false><<<gs, kP2PWarps * 32, 0, ws.st>>>(ws.chunks, ws.d_counts, ws.queue, ws.leaves, ws.c_end,
                                                               ws.rng_off, ws.rng_len, ws.ranges, ws.xs, Gm, eps2, o, ws.n);
    }
    ws.launches += 1;
    timer_end(ws, kTP2P);
}

void direct_sum(Workspace &ws, const double *x_orig, const long long *targets, unsigned nt, double *out_soa,
                double *part, unsigned nsplit) {
    const dim3 grid((nt + kDirectTB - 1) / kDirectTB, nsplit);
    k_direct_part<SoA><<<grid, kDirectTB, 0, ws.st>>>(SoA{x_orig, ws.n}, ws.n, targets, nt, nsplit, ws.G * ws.m,
                                                     ws.eps * ws.eps, part);
    k_direct_reduce<<<(nt + 255) / 256, 256, 0, ws.st>>>(part, nt, nsplit, out_soa, nullptr);
    ws.launches += 2;
}

}  // namespace gb
