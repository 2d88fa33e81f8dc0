// Near field (P2P, gravity/include/fmm.hpp:377-385, 513-540) and the FP64
// direct-sum oracle (solver_ref_naive.hpp:103-119) on the GPU.
//
// Work decomposition: every leaf is cut into chunks (common.cuh chunk_at):
// full chunks of 32 targets, and remainders of t < 32 targets that run
// floor(32/t) lane groups over disjoint subsets of the same sources (combined
// at the end through shared memory), so small leaves keep most lanes busy. A
// persistent grid of warps pulls chunks from a device counter (work queue).
// A warp streams the leaf's near-field source ranges through shared memory
// 32 sources at a time, prefetching the next batch into registers while it
// works on the current one; lanes read the staged sources with broadcast
// shared-memory loads.
//
// Mixed precision (FP32): positions are kept as hi + lo float pairs relative
// to the root-box centre; targets and staged sources are re-expressed relative
// to the target leaf's centre ((hi - c_hi) + (lo - c_lo)), so FP32 differences
// carry ~1e-7 of the neighbourhood size rather than of the coordinate.
// Pair term: rsqrt.approx.ftz (a Newton step on request: it leaves the RMS
// error unchanged to 1e-10 at 20% of the cost), r^-3 d (equal masses: m
// and the reference's G, fmm.hpp:539, multiply the sum once); per-batch FP32
// partial sums folded into a compensated (Kahan) per-target accumulator.
#include "direct.cuh"
#include "workspace.cuh"

#ifndef GB_P2P_CARVEOUT_MAX
#define GB_P2P_CARVEOUT_MAX 1  // P2P SMs keep full shared memory, so the tensor-core M2L can start beside P2P blocks
#endif

namespace gb {

namespace {

constexpr int kP2PWarps = 4;

__device__ __forceinline__ float rsqrt_ftz(float x) {
    float r;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}

// Source-batch cursor over a slice [v0, v0 + len) of the concatenation of a
// leaf's source ranges; batches never cross a range end.
struct Cursor {
    const uint2 *rng;
    unsigned nr, r, b, end, rem;
    __device__ __forceinline__ void start(const uint2 *ranges, unsigned n, unsigned v0, unsigned len) {
        rng = ranges, nr = n, r = 0, rem = len, b = 0, end = 0;
        for (; r < nr; ++r) {
            const uint2 g = rng[r];
            if (v0 < g.y - g.x) {
                b = g.x + v0, end = g.y;
                break;
            }
            v0 -= g.y - g.x;
        }
        if (rem == 0) r = nr;
    }
    __device__ __forceinline__ bool valid() const { return r < nr; }
    __device__ __forceinline__ unsigned count() const { return min(min(32u, end - b), rem); }
    __device__ __forceinline__ void advance() {
        const unsigned c = count();
        rem -= c, b += c;
        if (rem == 0) {
            r = nr;
        } else if (b >= end && ++r < nr) {
            const uint2 g = rng[r];
            b = g.x, end = g.y;
        }
    }
};

// The same walk in full batches: up to 32 sources taken across range
// boundaries, lane l getting the l-th (a batch is cut only at the slice's end,
// so every batch but the last is full and takes the paired path). The state
// is uniform over the warp; the loop runs once per range the batch touches.
struct BatchCursor {
    const uint2 *rng;
    unsigned nr, r, b, end, rem;
    __device__ __forceinline__ void start(const uint2 *ranges, unsigned n, unsigned v0, unsigned len) {
        Cursor c;
        c.start(ranges, n, v0, len);
        rng = c.rng, nr = c.nr, r = c.r, b = c.b, end = c.end, rem = c.rem;
    }
    // the next batch: its size, and this lane's source index (lane < size)
    __device__ __forceinline__ unsigned next(unsigned lane, unsigned &idx) {
        unsigned filled = 0;
        idx = 0;
        while (filled < 32u && rem > 0 && r < nr) {
            const unsigned take = min(min(32u - filled, end - b), rem);
            if (lane >= filled && lane < filled + take) idx = b + (lane - filled);
            filled += take, rem -= take, b += take;
            if (b >= end && ++r < nr) {
                const uint2 g = rng[r];
                b = g.x, end = g.y;
            }
        }
        return filled;
    }
};

// Work item -> (leaf, first target, targets, slice, slices, partial slot,
// source slice [v0, v0 + len)).
struct Item {
    int li, t0, nt, sl, ns, pslot;
    unsigned v0, len;
    __device__ __forceinline__ Item(const int4 w, const unsigned *src_total) {
        li = w.x, t0 = w.y, nt = item_nt(w.z), sl = item_slice(w.z), ns = item_nslices(w.z), pslot = w.w;
        const unsigned S = src_total[li];
        const unsigned per = (S + ns - 1) / ns;
        v0 = min(S, sl * per);
        len = min(per, S - v0);
    }
};

template <bool kNewton, bool kSoft>
__device__ __forceinline__ void pair_f32(const float4 s, float tx, float ty, float tz, float eps2, float &bx, float &by,
                                         float &bz) {
    const float dx = s.x - tx, dy = s.y - ty, dz = s.z - tz;
    const float r2 = fmaf(dx, dx, fmaf(dy, dy, fmaf(dz, dz, eps2)));
    float ri = rsqrt_ftz(r2);
    if (kNewton) ri = ri * fmaf(-0.5f * r2 * ri, ri, 1.5f);
    if (!kSoft) ri = r2 > 0.f ? ri : 0.f;
    const float f = ri * (ri * ri);
    bx = fmaf(dx, f, bx);
    by = fmaf(dy, f, by);
    bz = fmaf(dz, f, bz);
}

// Register budgets of the mixed-precision kernel (tuning knob p2p_occupancy):
// compiled for 8 resident blocks per SM (64 registers) or for 6 (80
// registers: more pair terms in flight per warp, which pays while P2P shares
// the SMs with the far field on 2 blocks per SM). Both fit beside the far
// field's kernels (a 96-register build kept the cluster M2M from starting
// beside P2P and serialised the two). The same arithmetic either way, so
// the same results bit for bit.
template <bool kNewton, bool kSoft, int kMinBlocks>
__global__ void __launch_bounds__(kP2PWarps * 32, kMinBlocks) k_p2p_f32(const int4 *__restrict__ chunks, const unsigned *counts,
                                                            unsigned *queue, const int *__restrict__ leaves,
                                                            const double *__restrict__ c_ctr,
                                                            const TreeInfo *__restrict__ info, const int *__restrict__ c_sys,
                                                            const unsigned *__restrict__ rng_off,
                                                            const unsigned *__restrict__ rng_len, const uint2 *__restrict__ ranges,
                                                            const float4 *__restrict__ ph, const float4 *__restrict__ pl,
                                                            const unsigned *__restrict__ src_total, float *__restrict__ part,
                                                            float Gm, float eps2, float *__restrict__ nearv, unsigned n) {
    __shared__ float4 src[kP2PWarps][32];
    __shared__ float4 srcxy[kP2PWarps][16];  // sources 2m, 2m+1 as {x, x', y, y'}
    __shared__ float2 srcz[kP2PWarps][16];   // and {z, z'}
    __shared__ float red[kP2PWarps][3][32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const unsigned nch = counts[5];
    float *pxy = reinterpret_cast<float *>(srcxy[w]);
    float *pz = reinterpret_cast<float *>(srcz[w]);
    while (true) {
        unsigned ci = 0;
        if (lane == 0) ci = atomicAdd(queue, 1u);
        ci = __shfl_sync(0xffffffffu, ci, 0);
        if (ci >= nch) break;
        const Item it(chunks[ci], src_total);
        const int nt = it.nt;
        const int g = 32 / nt;
        const int grp = lane / nt;
        const int t = lane - grp * nt;
        const bool tact = grp < g;
        const int i = it.t0 + t;
        const int leaf = leaves[it.li];
        const RootC cc = leaf_centre(c_ctr, leaf, info + cell_system(c_sys, leaf));
        float tx = 0, ty = 0, tz = 0;
        if (tact) {
            const float4 h = ph[i], l = pl[i];
            tx = (h.x - cc.hx) + (l.x - cc.lx);
            ty = (h.y - cc.hy) + (l.y - cc.ly);
            tz = (h.z - cc.hz) + (l.z - cc.lz);
        }
        float sx = 0, sy = 0, sz = 0, kx = 0, ky = 0, kz = 0;  // Kahan sums and compensations
        BatchCursor cur;
        cur.start(ranges + rng_off[it.li], rng_len[it.li], it.v0, it.len);
        float4 h = make_float4(0, 0, 0, 0), l = h;
        unsigned sidx;
        unsigned cnt = cur.next(static_cast<unsigned>(lane), sidx);
        if (static_cast<unsigned>(lane) < cnt) h = ph[sidx], l = pl[sidx];
        const float2 ntx = make_float2(-tx, -tx), nty = make_float2(-ty, -ty), ntz = make_float2(-tz, -tz);
        const float2 e2 = make_float2(eps2, eps2);
        while (cnt) {
            if (static_cast<unsigned>(lane) < cnt) {
                const float qx = (h.x - cc.hx) + (l.x - cc.lx), qy = (h.y - cc.hy) + (l.y - cc.ly),
                            qz = (h.z - cc.hz) + (l.z - cc.lz);
                src[w][lane] = make_float4(qx, qy, qz, 0.f);
                pxy[(lane >> 1) * 4 + (lane & 1)] = qx;
                pxy[(lane >> 1) * 4 + 2 + (lane & 1)] = qy;
                pz[(lane >> 1) * 2 + (lane & 1)] = qz;
            }
            __syncwarp();
            const unsigned now = cnt;
            cnt = cur.next(static_cast<unsigned>(lane), sidx);  // prefetch the next batch while this one is computed
            if (static_cast<unsigned>(lane) < cnt) h = ph[sidx], l = pl[sidx];
            float bx = 0, by = 0, bz = 0;
            if (g == 1 && now == 32) {
                // two sources per step on paired FP32 instructions (.f32x2);
                // each component rounds exactly like the scalar operation
                float2 ax = make_float2(0.f, 0.f), ay = ax, az = ax;
#pragma unroll
                for (int m = 0; m < 16; ++m) {
                    const float4 q = srcxy[w][m];
                    const float2 dx = __fadd2_rn(make_float2(q.x, q.y), ntx);
                    const float2 dy = __fadd2_rn(make_float2(q.z, q.w), nty);
                    const float2 dz = __fadd2_rn(srcz[w][m], ntz);
                    const float2 r2 = __ffma2_rn(dx, dx, __ffma2_rn(dy, dy, __ffma2_rn(dz, dz, e2)));
                    float2 ri = make_float2(rsqrt_ftz(r2.x), rsqrt_ftz(r2.y));
                    if (kNewton) {
                        ri.x = ri.x * fmaf(-0.5f * r2.x * ri.x, ri.x, 1.5f);
                        ri.y = ri.y * fmaf(-0.5f * r2.y * ri.y, ri.y, 1.5f);
                    }
                    if (!kSoft) ri.x = r2.x > 0.f ? ri.x : 0.f, ri.y = r2.y > 0.f ? ri.y : 0.f;
                    const float2 f = __fmul2_rn(ri, __fmul2_rn(ri, ri));
                    ax = __ffma2_rn(dx, f, ax);
                    ay = __ffma2_rn(dy, f, ay);
                    az = __ffma2_rn(dz, f, az);
                }
                bx = ax.x + ax.y, by = ay.x + ay.y, bz = az.x + az.y;
            } else if (tact) {
                for (unsigned k = grp; k < now; k += g) pair_f32<kNewton, kSoft>(src[w][k], tx, ty, tz, eps2, bx, by, bz);
            }
            __syncwarp();
            float y = bx - kx, tt = sx + y;
            kx = (tt - sx) - y, sx = tt;
            y = by - ky, tt = sy + y;
            ky = (tt - sy) - y, sy = tt;
            y = bz - kz, tt = sz + y;
            kz = (tt - sz) - y, sz = tt;
        }
        sx -= kx, sy -= ky, sz -= kz;
        if (g > 1) {
            red[w][0][lane] = sx, red[w][1][lane] = sy, red[w][2][lane] = sz;
            __syncwarp();
            if (grp == 0)
                for (int q = 1; q < g; ++q) sx += red[w][0][t + q * nt], sy += red[w][1][t + q * nt], sz += red[w][2][t + q * nt];
            __syncwarp();
        }
        if (grp == 0) {
            if (it.ns == 1) {
                nearv[i] = Gm * sx;
                nearv[n + i] = Gm * sy;
                nearv[2 * static_cast<size_t>(n) + i] = Gm * sz;
            } else {
                float *o = part + static_cast<size_t>(it.pslot) * 96;
                o[t] = sx, o[32 + t] = sy, o[64 + t] = sz;
            }
        }
    }
}

template <bool kSoft>
__global__ void __launch_bounds__(kP2PWarps * 32) k_p2p_f64(const int4 *__restrict__ chunks, const unsigned *counts,
                                                            unsigned *queue, const unsigned *__restrict__ rng_off,
                                                            const unsigned *__restrict__ rng_len, const uint2 *__restrict__ ranges,
                                                            const double *__restrict__ xs, const unsigned *__restrict__ src_total,
                                                            double *__restrict__ part, double Gm, double eps2,
                                                            double *__restrict__ nearv, unsigned n) {
    __shared__ double src[kP2PWarps][3][32];
    __shared__ double red[kP2PWarps][3][32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const unsigned nch = counts[5];
    while (true) {
        unsigned ci = 0;
        if (lane == 0) ci = atomicAdd(queue, 1u);
        ci = __shfl_sync(0xffffffffu, ci, 0);
        if (ci >= nch) break;
        const Item it(chunks[ci], src_total);
        const int nt = it.nt;
        const int g = 32 / nt;
        const int grp = lane / nt;
        const int t = lane - grp * nt;
        const bool tact = grp < g;
        const int i = it.t0 + t;
        const double tx = tact ? xs[i] : 0.0, ty = tact ? xs[n + i] : 0.0, tz = tact ? xs[2 * static_cast<size_t>(n) + i] : 0.0;
        double ax = 0, ay = 0, az = 0;
        Cursor cur;
        cur.start(ranges + rng_off[it.li], rng_len[it.li], it.v0, it.len);
        while (cur.valid()) {
            const unsigned cnt = cur.count();
            if (static_cast<unsigned>(lane) < cnt) {
                const unsigned j = cur.b + lane;
                src[w][0][lane] = xs[j];
                src[w][1][lane] = xs[n + j];
                src[w][2][lane] = xs[2 * static_cast<size_t>(n) + j];
            }
            __syncwarp();
            if (tact)
                for (unsigned k = grp; k < cnt; k += g) {
                    const double dx = src[w][0][k] - tx, dy = src[w][1][k] - ty, dz = src[w][2][k] - tz;
                    const double r2 = dx * dx + dy * dy + dz * dz + eps2;
                    double ri = rsqrt(r2);
                    if (!kSoft) ri = r2 > 0.0 ? ri : 0.0;
                    const double f = ri * ri * ri;
                    ax += f * dx;
                    ay += f * dy;
                    az += f * dz;
                }
            __syncwarp();
            cur.advance();
        }
        if (g > 1) {
            red[w][0][lane] = ax, red[w][1][lane] = ay, red[w][2][lane] = az;
            __syncwarp();
            if (grp == 0)
                for (int q = 1; q < g; ++q) ax += red[w][0][t + q * nt], ay += red[w][1][t + q * nt], az += red[w][2][t + q * nt];
            __syncwarp();
        }
        if (grp == 0) {
            if (it.ns == 1) {
                nearv[i] = Gm * ax;
                nearv[n + i] = Gm * ay;
                nearv[2 * static_cast<size_t>(n) + i] = Gm * az;
            } else {
                double *o = part + static_cast<size_t>(it.pslot) * 96;
                o[t] = ax, o[32 + t] = ay, o[64 + t] = az;
            }
        }
    }
}

// Sum the slices of every split chunk in slice order (deterministic).
template <typename T>
__global__ void k_p2p_combine(const int4 *__restrict__ chunks, const unsigned *counts, const T *__restrict__ part, T scale,
                              T *__restrict__ nearv, unsigned n) {
    const unsigned nit = counts[5];
    for (unsigned q = blockIdx.x * blockDim.x + threadIdx.x; q < nit * 32u; q += gridDim.x * blockDim.x) {
        const int4 w = chunks[q >> 5];
        const int t = static_cast<int>(q & 31u);
        const int ns = item_nslices(w.z);
        if (ns <= 1 || item_slice(w.z) != 0 || t >= item_nt(w.z)) continue;
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            T s = 0;
            for (int k = 0; k < ns; ++k) s += part[static_cast<size_t>(w.w + k) * 96 + 32 * a + t];
            nearv[static_cast<size_t>(a) * n + w.y + t] = scale * s;
        }
    }
}

// Near-field potential (diagnostic, FP64, after an evaluation): for every
// target i of a work item, sum over its near-field sources j != i (tree
// indices) of (|x_j - x_i|^2 + eps^2)^(-1/2). Split items leave per-slice
// partial sums in part[slot][0..31]; k_p2p_phi_combine adds them in slice order.
__global__ void __launch_bounds__(kP2PWarps * 32) k_p2p_phi(const int4 *__restrict__ chunks, const unsigned *counts,
                                                            unsigned *queue, const unsigned *__restrict__ rng_off,
                                                            const unsigned *__restrict__ rng_len, const uint2 *__restrict__ ranges,
                                                            const double *__restrict__ xs, const unsigned *__restrict__ src_total,
                                                            double *__restrict__ part, double Gm, double eps2,
                                                            double *__restrict__ phiv, unsigned n) {
    __shared__ double src[kP2PWarps][3][32];
    __shared__ double red[kP2PWarps][32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const unsigned nch = counts[5];
    while (true) {
        unsigned ci = 0;
        if (lane == 0) ci = atomicAdd(queue, 1u);
        ci = __shfl_sync(0xffffffffu, ci, 0);
        if (ci >= nch) break;
        const Item it(chunks[ci], src_total);
        const int nt = it.nt;
        const int g = 32 / nt;
        const int grp = lane / nt;
        const int t = lane - grp * nt;
        const bool tact = grp < g;
        const unsigned i = static_cast<unsigned>(it.t0 + t);
        const double tx = tact ? xs[i] : 0.0, ty = tact ? xs[n + i] : 0.0, tz = tact ? xs[2 * static_cast<size_t>(n) + i] : 0.0;
        double pot = 0;
        Cursor cur;
        cur.start(ranges + rng_off[it.li], rng_len[it.li], it.v0, it.len);
        while (cur.valid()) {
            const unsigned cnt = cur.count(), jb = cur.b;
            if (static_cast<unsigned>(lane) < cnt) {
                const unsigned j = jb + lane;
                src[w][0][lane] = xs[j];
                src[w][1][lane] = xs[n + j];
                src[w][2][lane] = xs[2 * static_cast<size_t>(n) + j];
            }
            __syncwarp();
            if (tact)
                for (unsigned k = grp; k < cnt; k += g) {
                    if (jb + k == i) continue;
                    const double dx = src[w][0][k] - tx, dy = src[w][1][k] - ty, dz = src[w][2][k] - tz;
                    pot += 1.0 / sqrt(dx * dx + dy * dy + dz * dz + eps2);
                }
            __syncwarp();
            cur.advance();
        }
        if (g > 1) {
            red[w][lane] = pot;
            __syncwarp();
            if (grp == 0)
                for (int q = 1; q < g; ++q) pot += red[w][t + q * nt];
            __syncwarp();
        }
        if (grp == 0) {
            if (it.ns == 1)
                phiv[i] = Gm * pot;
            else
                part[static_cast<size_t>(it.pslot) * 96 + t] = pot;
        }
    }
}

// Forest: the near field (or potential) of each particle position times its
// system's G m (the P2P kernels ran with G m = 1; one rounding either way).
template <typename T>
__global__ void k_scale_by_system(T *__restrict__ v, unsigned n, int comps, const int *__restrict__ psys,
                                  const TreeInfo *__restrict__ info) {
    for (unsigned j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x) {
        const T g = static_cast<T>(info[psys[j]].gm);
        for (int a = 0; a < comps; ++a) v[static_cast<size_t>(a) * n + j] = g * v[static_cast<size_t>(a) * n + j];
    }
}

__global__ void k_p2p_phi_combine(const int4 *__restrict__ chunks, const unsigned *counts, const double *__restrict__ part,
                                  double Gm, double *__restrict__ phiv) {
    const unsigned nit = counts[5];
    for (unsigned q = blockIdx.x * blockDim.x + threadIdx.x; q < nit * 32u; q += gridDim.x * blockDim.x) {
        const int4 w = chunks[q >> 5];
        const int t = static_cast<int>(q & 31u);
        const int ns = item_nslices(w.z);
        if (ns <= 1 || item_slice(w.z) != 0 || t >= item_nt(w.z)) continue;
        double s = 0;
        for (int k = 0; k < ns; ++k) s += part[static_cast<size_t>(w.w + k) * 96 + t];
        phiv[w.y + t] = Gm * s;
    }
}

}  // namespace

void near_potential(Workspace &ws, double *phiv) {
    cudaMemsetAsync(ws.queue, 0, sizeof(unsigned), ws.st);
    const unsigned gs = static_cast<unsigned>(ws.num_sms) * 8;
    const double Gm = ws.forest() ? 1.0 : ws.G * ws.m;
    k_p2p_phi<<<gs, kP2PWarps * 32, 0, ws.st>>>(ws.chunks, ws.d_counts, ws.queue, ws.rng_off, ws.rng_len, ws.ranges, ws.xs,
                                                ws.src_total, static_cast<double *>(ws.part), Gm, ws.eps * ws.eps, phiv, ws.n);
    k_p2p_phi_combine<<<gs, 256, 0, ws.st>>>(ws.chunks, ws.d_counts, static_cast<const double *>(ws.part), Gm, phiv);
    ws.launches += 2;
    if (ws.forest()) {
        k_scale_by_system<double><<<gs, 256, 0, ws.st>>>(phiv, ws.n, 1, ws.psys, ws.info);
        ws.launches += 1;
    }
}

// Near-field kernel over the work queue, `per_sm` blocks per SM. The queue
// counter is zeroed at the start of every evaluation (build_tree); several
// launches (on any streams) may drain the same queue, each item is taken once.
// p2p_finish adds the slices of split items after all of them.

template <int kMinBlocks>
void p2p_f32_carveout() {
    // keep the SMs that run P2P configured for full shared memory, so far-field
    // kernels (the tensor-core M2L: up to 206 KB) can start beside the P2P blocks
    cudaFuncSetAttribute(k_p2p_f32<false, true, kMinBlocks>, cudaFuncAttributePreferredSharedMemoryCarveout,
                         cudaSharedmemCarveoutMaxShared);
    cudaFuncSetAttribute(k_p2p_f32<false, false, kMinBlocks>, cudaFuncAttributePreferredSharedMemoryCarveout,
                         cudaSharedmemCarveoutMaxShared);
    cudaFuncSetAttribute(k_p2p_f32<true, true, kMinBlocks>, cudaFuncAttributePreferredSharedMemoryCarveout,
                         cudaSharedmemCarveoutMaxShared);
    cudaFuncSetAttribute(k_p2p_f32<true, false, kMinBlocks>, cudaFuncAttributePreferredSharedMemoryCarveout,
                         cudaSharedmemCarveoutMaxShared);
}

void p2p_pass(Workspace &ws, unsigned per_sm) {
    if (per_sm == 0) return;
    timer_begin(ws, kTP2P);
#if GB_P2P_CARVEOUT_MAX
    p2p_f32_carveout<8>();
    p2p_f32_carveout<6>();
#endif
    const unsigned gs = capped_grid(static_cast<unsigned>(ws.num_sms) * per_sm, ceil_div(ws.n, 128));
    const bool soft = ws.eps > 0;
    if (ws.mixed) {
        const float eps2 = static_cast<float>(ws.eps * ws.eps);
        const float Gm = ws.forest() ? 1.0f : static_cast<float>(ws.G * ws.m);  // a forest scales in p2p_finish
        auto *o = static_cast<float *>(ws.nearf);
        auto *pf = static_cast<float *>(ws.part);
#define GB_P2P32_MB(NW, SF, MB)                                                                                  \
    k_p2p_f32<NW, SF, MB><<<gs, kP2PWarps * 32, 0, ws.st>>>(ws.chunks, ws.d_counts, ws.queue, ws.leaves, ws.c_ctr,    \
                                                            ws.info, forest_cells(ws), ws.rng_off, ws.rng_len,        \
                                                            ws.ranges, ws.ph, ws.pl, ws.src_total, pf, Gm, eps2, o, ws.n)
#define GB_P2P32(NW, SF)             \
    do {                             \
        if (ws.p2p_occ == 6)         \
            GB_P2P32_MB(NW, SF, 6);  \
        else                         \
            GB_P2P32_MB(NW, SF, 8);  \
    } while (0)
        if (ws.p2p_newton) {
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
#undef GB_P2P32_MB
    } else {
        const double Gm = ws.forest() ? 1.0 : ws.G * ws.m, eps2 = ws.eps * ws.eps;
        auto *o = static_cast<double *>(ws.nearf);
        auto *pd = static_cast<double *>(ws.part);
        if (soft)
            k_p2p_f64<true><<<gs, kP2PWarps * 32, 0, ws.st>>>(ws.chunks, ws.d_counts, ws.queue, ws.rng_off, ws.rng_len,
                                                              ws.ranges, ws.xs, ws.src_total, pd, Gm, eps2, o, ws.n);
        else
            k_p2p_f64<false><<<gs, kP2PWarps * 32, 0, ws.st>>>(ws.chunks, ws.d_counts, ws.queue, ws.rng_off, ws.rng_len,
                                                               ws.ranges, ws.xs, ws.src_total, pd, Gm, eps2, o, ws.n);
    }
    ws.launches += 1;
    timer_end(ws, kTP2P);
}

void p2p_finish(Workspace &ws) {
    const unsigned gs = capped_grid(static_cast<unsigned>(ws.num_sms) * 8, ceil_div(ws.n, 128));
    const bool forest = ws.forest();
    const double Gm = forest ? 1.0 : ws.G * ws.m;
    if (ws.mixed)
        k_p2p_combine<float><<<gs, 256, 0, ws.st>>>(ws.chunks, ws.d_counts, static_cast<const float *>(ws.part),
                                                    static_cast<float>(Gm), static_cast<float *>(ws.nearf), ws.n);
    else
        k_p2p_combine<double><<<gs, 256, 0, ws.st>>>(ws.chunks, ws.d_counts, static_cast<const double *>(ws.part), Gm,
                                                     static_cast<double *>(ws.nearf), ws.n);
    ws.launches += 1;
    if (forest) {
        if (ws.mixed)
            k_scale_by_system<float><<<gs, 256, 0, ws.st>>>(static_cast<float *>(ws.nearf), ws.n, 3, ws.psys, ws.info);
        else
            k_scale_by_system<double><<<gs, 256, 0, ws.st>>>(static_cast<double *>(ws.nearf), ws.n, 3, ws.psys, ws.info);
        ws.launches += 1;
    }
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
