// Accurate mode: the far field of the softening difference (no counterpart in
// the reference).
//
// The reference's far field expands the unsoftened 1/r (M2L fmm.hpp:277-304,
// L2P fmm.hpp:332-374) while its near field is softened (fmm.hpp:531-540), and
// only the near field carries G; against the softened direct sum its error
// therefore stops near eps^2/r^2 whatever p is. In the accurate mode the far
// field is multiplied by G and the field of the softening difference is added:
// for every leaf and every far source cell S of it (the M2L lists of the leaf
// and of its ancestors at level >= 2),
//   da(x) = G sum_{j in S} m_j F(|x_j - x|^2) (x_j - x),
//   F(u) = (u + eps^2)^{-3/2} - u^{-3/2},
// expanded about S's centre of mass z to second order in the source offsets
// (y_j = x_j - z, Q = sum_j m_j y_j y_j^T; the first order vanishes about z):
//   [M F(u) + F'(u) tr Q + 2 F''(u) d.Qd] d + 2 F'(u) Qd,   d = z - x, u = |d|^2,
//   F' = -3/2 [(u + e)^{-5/2} - u^{-5/2}],   F'' = 15/4 [(u + e)^{-7/2} - u^{-7/2}].
// Evaluation:
//   * k_soft_near: the lists of the leaf and of its parent at every particle;
//     in the leaf's own list a source at offset o (cell units) with exactly one
//     |o_a| = 2 and the others <= 1 (the 54 nearest far cells, where the
//     expansion converges slowest) is taken as its 8 octants: the children of a
//     non-leaf source, or the leaf's particles split at its mid-planes;
//   * k_soft_far: the lists of the ancestors two and more levels up, once per
//     leaf at its centre c (the value above and the first-order change
//     J (x - c) of its monopole term, J = -M (2 F' d d^T + F I)).
// The oracle's softening_correction (oracle/oracle.hpp) states the same
// approximations in FP64; the error of the expansion against the exact sum over
// the source particles is ~3e-6 of |a| (RMS) on the 4M Plummer sphere with
// eps = 0.005, below the p = 10 expansion's own ~7e-6.
//
// Moments are records of 16 values of T per cell (Mom): the centre of mass
// relative to the root-box centre (FP32: a hi + lo pair), the mass, tr Q, and
// the second central moments. Differences d are formed relative to the target
// leaf's centre, as the near field does, so FP32 keeps ~1e-7 of the
// neighbourhood size. F, F', F'' are differences of (u + e)^{-k/2} and u^{-k/2};
// their FP32 rounding is ~1e-7 / (eps^2/u) relative, at most ~1e-3 of a
// correction that is itself ~eps^2/u of the source's field.
#include <climits>

#include "workspace.cuh"

namespace gb {

namespace {

template <typename T>
struct Mom {
    T zh[3], M;   // centre of mass - root-box centre (hi part), mass
    T zl[3], tr;  // lo part (0 in FP64), trace of Q
    T Q[6];       // xx yy zz xy xz yz
    T pad[2];
};
static_assert(sizeof(Mom<float>) == 64 && sizeof(Mom<double>) == 128, "Mom layout");

template <typename T>
__device__ __forceinline__ T rsqrt_t(T x);
template <>
__device__ __forceinline__ float rsqrt_t<float>(float x) {
    float r;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}
template <>
__device__ __forceinline__ double rsqrt_t<double>(double x) {
    return 1.0 / sqrt(x);
}

// A cell's centre relative to the root-box centre, as (hi, lo) in T.
template <typename T>
struct RelC {
    T h[3], l[3];
};
template <typename T>
__device__ __forceinline__ RelC<T> rel_centre(const double *c_ctr, int c, const TreeInfo *info) {
    RelC<T> r;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        const double d = c_ctr[3 * c + a] - info->root_c[a];
        r.h[a] = static_cast<T>(d);
        r.l[a] = static_cast<T>(d - static_cast<double>(r.h[a]));
    }
    return r;
}

// Position of tree-order particle j relative to the centre of cell c.
template <typename T>
__device__ __forceinline__ void rel_pos(int j, const double *xs, unsigned n, const float4 *ph, const float4 *pl,
                                        const double *cd, const RelC<T> &cc, T y[3]) {
    if (sizeof(T) == 4) {
        const float4 h = ph[j], l = pl[j];
        y[0] = static_cast<T>((h.x - static_cast<float>(cc.h[0])) + (l.x - static_cast<float>(cc.l[0])));
        y[1] = static_cast<T>((h.y - static_cast<float>(cc.h[1])) + (l.y - static_cast<float>(cc.l[1])));
        y[2] = static_cast<T>((h.z - static_cast<float>(cc.h[2])) + (l.z - static_cast<float>(cc.l[2])));
    } else {
        y[0] = static_cast<T>(xs[j] - cd[0]);
        y[1] = static_cast<T>(xs[n + j] - cd[1]);
        y[2] = static_cast<T>(xs[2 * static_cast<size_t>(n) + j] - cd[2]);
    }
}

// Record from sums about a cell centre: count, sum y, sum y y^T (xx yy zz xy xz yz).
template <typename T>
__device__ __forceinline__ void make_record(const T *s, T mass, const RelC<T> &cc, Mom<T> &r) {
    const T cnt = s[0];
    if (cnt == T(0)) {
#pragma unroll
        for (int a = 0; a < 3; ++a) r.zh[a] = T(0), r.zl[a] = T(0);
        r.M = T(0), r.tr = T(0);
#pragma unroll
        for (int k = 0; k < 6; ++k) r.Q[k] = T(0);
        r.pad[0] = r.pad[1] = T(0);
        return;
    }
    const T inv = T(1) / cnt;
    const T g[3] = {s[1] * inv, s[2] * inv, s[3] * inv};
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        const T t = cc.l[a] + g[a];
        r.zh[a] = cc.h[a] + t;
        r.zl[a] = t - (r.zh[a] - cc.h[a]);
    }
    r.M = mass * cnt;
    r.Q[0] = mass * (s[4] - cnt * g[0] * g[0]);
    r.Q[1] = mass * (s[5] - cnt * g[1] * g[1]);
    r.Q[2] = mass * (s[6] - cnt * g[2] * g[2]);
    r.Q[3] = mass * (s[7] - cnt * g[0] * g[1]);
    r.Q[4] = mass * (s[8] - cnt * g[0] * g[2]);
    r.Q[5] = mass * (s[9] - cnt * g[1] * g[2]);
    r.tr = r.Q[0] + r.Q[1] + r.Q[2];
    r.pad[0] = r.pad[1] = T(0);
}

template <typename T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
    for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// ------------------------------------------------------------ leaf moments
// One warp per leaf at level >= 2: the moments of the leaf and of its 8
// octants (coordinate < mid-plane -> lower half, octant bit set; the tree's
// tie rule). Sums per octant by masked warp reductions (fixed order).
template <typename T>
__global__ void __launch_bounds__(128) k_mom_leaf(const int *__restrict__ leaves, const unsigned *counts,
                                                  const int *__restrict__ c_begin, const int *__restrict__ c_end,
                                                  const int *__restrict__ c_level, const double *__restrict__ c_ctr,
                                                  const double *__restrict__ xs, const float4 *__restrict__ ph,
                                                  const float4 *__restrict__ pl, unsigned n,
                                                  const TreeInfo *__restrict__ info, T mass, Mom<T> *__restrict__ mom,
                                                  Mom<T> *__restrict__ moct) {
    __shared__ T sums[4][9][10];  // 8 octants + the whole leaf
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const unsigned NL = counts[3];
    const unsigned warps = gridDim.x * (blockDim.x >> 5);
    for (unsigned li = blockIdx.x * (blockDim.x >> 5) + w; li < NL; li += warps) {
        const int c = leaves[li];
        if (c_level[c] < 2) continue;  // warp-uniform
        const RelC<T> cc = rel_centre<T>(c_ctr, c, info);
        const double cd[3] = {c_ctr[3 * c], c_ctr[3 * c + 1], c_ctr[3 * c + 2]};
        for (int k = lane; k < 80; k += 32) sums[w][k / 10][k % 10] = T(0);
        __syncwarp();
        const int b = c_begin[c], e = c_end[c];
        for (int j0 = b; j0 < e; j0 += 32) {
            const int j = j0 + lane;
            T v[10] = {};
            int oct = -1;
            if (j < e) {
                T y[3];
                rel_pos<T>(j, xs, n, ph, pl, cd, cc, y);
                oct = (y[0] < T(0) ? 1 : 0) | (y[1] < T(0) ? 2 : 0) | (y[2] < T(0) ? 4 : 0);
                v[0] = T(1), v[1] = y[0], v[2] = y[1], v[3] = y[2];
                v[4] = y[0] * y[0], v[5] = y[1] * y[1], v[6] = y[2] * y[2];
                v[7] = y[0] * y[1], v[8] = y[0] * y[2], v[9] = y[1] * y[2];
            }
            for (int o = 0; o < 8; ++o) {
                if (!__ballot_sync(0xffffffffu, oct == o)) continue;  // warp-uniform
#pragma unroll
                for (int k = 0; k < 10; ++k) {
                    const T s = warp_sum(oct == o ? v[k] : T(0));
                    if (lane == 0) sums[w][o][k] += s;
                }
            }
            __syncwarp();
        }
        if (lane < 10) {
            T s = T(0);
            for (int o = 0; o < 8; ++o) s += sums[w][o][lane];
            sums[w][8][lane] = s;
        }
        __syncwarp();
        if (lane < 9) {
            Mom<T> r;
            make_record<T>(sums[w][lane], mass, cc, r);
            if (lane < 8)
                moct[static_cast<size_t>(c) * 8 + lane] = r;
            else
                mom[c] = r;
        }
        __syncwarp();
    }
}

// -------------------------------------------------------- non-leaf moments
// Non-leaf cells of level L (>= 2) from their 8 children: M = sum M_c,
// g = sum M_c g_c / M, Q = sum [Q_c + M_c (g_c - g)(g_c - g)^T], with g_c the
// child's centre of mass relative to the parent's centre.
template <typename T>
__global__ void k_mom_up(int L, const TreeInfo *__restrict__ info, const int *__restrict__ split_cell,
                         const int *__restrict__ c_child, const double *__restrict__ c_ctr, Mom<T> *mom) {
    const int e0 = info->split_start[L], cnt = info->split_count[L];
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < cnt; e += gridDim.x * blockDim.x) {
        const int P = split_cell[e0 + e];
        const int fc = c_child[P];
        const RelC<T> cc = rel_centre<T>(c_ctr, P, info);
        T gc[8][3], Mc[8];
        T M = T(0), g[3] = {T(0), T(0), T(0)};
#pragma unroll
        for (int o = 0; o < 8; ++o) {
            const Mom<T> &r = mom[fc + o];
            Mc[o] = r.M;
#pragma unroll
            for (int a = 0; a < 3; ++a) gc[o][a] = (r.zh[a] - cc.h[a]) + (r.zl[a] - cc.l[a]);
            M += Mc[o];
#pragma unroll
            for (int a = 0; a < 3; ++a) g[a] += Mc[o] * gc[o][a];
        }
        Mom<T> out;
        if (M == T(0)) {
            T z[10] = {};
            make_record<T>(z, T(0), cc, out);
            mom[P] = out;
            continue;
        }
#pragma unroll
        for (int a = 0; a < 3; ++a) g[a] /= M;
        T Q[6] = {};
#pragma unroll
        for (int o = 0; o < 8; ++o) {
            const Mom<T> &r = mom[fc + o];
            const T d0 = gc[o][0] - g[0], d1 = gc[o][1] - g[1], d2 = gc[o][2] - g[2];
            Q[0] += r.Q[0] + Mc[o] * d0 * d0;
            Q[1] += r.Q[1] + Mc[o] * d1 * d1;
            Q[2] += r.Q[2] + Mc[o] * d2 * d2;
            Q[3] += r.Q[3] + Mc[o] * d0 * d1;
            Q[4] += r.Q[4] + Mc[o] * d0 * d2;
            Q[5] += r.Q[5] + Mc[o] * d1 * d2;
        }
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            const T t = cc.l[a] + g[a];
            out.zh[a] = cc.h[a] + t;
            out.zl[a] = t - (out.zh[a] - cc.h[a]);
        }
        out.M = M;
#pragma unroll
        for (int k = 0; k < 6; ++k) out.Q[k] = Q[k];
        out.tr = Q[0] + Q[1] + Q[2];
        out.pad[0] = out.pad[1] = T(0);
        mom[P] = out;
    }
}

// Softening-difference field (no G) of record r at offset d = z - x, added to acc.
template <typename T>
__device__ __forceinline__ void soft_term(const Mom<T> &r, T dx, T dy, T dz, T e2, T &ax, T &ay, T &az) {
    const T u = dx * dx + dy * dy + dz * dz;
    const T A = rsqrt_t<T>(u + e2), B = rsqrt_t<T>(u);
    const T A2 = A * A, B2 = B * B;
    const T A3 = A2 * A, B3 = B2 * B;
    const T A5 = A3 * A2, B5 = B3 * B2;
    const T A7 = A5 * A2, B7 = B5 * B2;
    const T F = A3 - B3;
    const T F1 = T(-1.5) * (A5 - B5);
    const T F2 = T(3.75) * (A7 - B7);
    const T qx = r.Q[0] * dx + r.Q[3] * dy + r.Q[4] * dz;
    const T qy = r.Q[3] * dx + r.Q[1] * dy + r.Q[5] * dz;
    const T qz = r.Q[4] * dx + r.Q[5] * dy + r.Q[2] * dz;
    const T dqd = dx * qx + dy * qy + dz * qz;
    const T a = r.M * F + F1 * r.tr + T(2) * F2 * dqd;
    const T b = T(2) * F1;
    ax += a * dx + b * qx;
    ay += a * dy + b * qy;
    az += a * dz + b * qz;
}

// Per-leaf values of the far levels: the correction's field at the leaf
// centre (3), its Jacobian (9, row-major) and its potential there (1).
constexpr int kTaylor = 13;

// Softening-difference potential (no G; the far potential's convention, whose
// gradient is the far field) of record r at offset d = z - x:
//   M P(u) + 2 P''(u) d.Qd + P'(u) tr Q,  P = (u + e)^{-1/2} - u^{-1/2},
//   P' = -F / 2, P'' = -F' / 2.
template <typename T>
__device__ __forceinline__ T soft_phi_term(const Mom<T> &r, T dx, T dy, T dz, T e2) {
    const T u = dx * dx + dy * dy + dz * dz;
    const T A = rsqrt_t<T>(u + e2), B = rsqrt_t<T>(u);
    const T A2 = A * A, B2 = B * B, A3 = A2 * A, B3 = B2 * B;
    const T F = A3 - B3, F1 = T(-1.5) * (A3 * A2 - B3 * B2);
    const T qx = r.Q[0] * dx + r.Q[3] * dy + r.Q[4] * dz;
    const T qy = r.Q[3] * dx + r.Q[1] * dy + r.Q[5] * dz;
    const T qz = r.Q[4] * dx + r.Q[5] * dy + r.Q[2] * dz;
    const T dqd = dx * qx + dy * qy + dz * qz;
    return r.M * (A - B) - F1 * dqd - T(0.5) * F * r.tr;
}

// Offset of the source relative to the target leaf centre: (z - c).
template <typename T>
__device__ __forceinline__ void src_offset(const Mom<T> &r, const RelC<T> &cc, T s[3]) {
#pragma unroll
    for (int a = 0; a < 3; ++a) s[a] = (r.zh[a] - cc.h[a]) + (r.zl[a] - cc.l[a]);
}

// --------------------------------------------------- far levels (k >= 2)
// One warp per leaf: the value and first-order change at the leaf centre of
// the sources in the M2L lists of the ancestors two and more levels up (each
// lane a fixed subset of slots, then a butterfly sum); 12 values per leaf
// (value, J row-major). Leaves above level 4 get zeros.
template <typename T>
__global__ void __launch_bounds__(128) k_soft_far(const int *__restrict__ leaves, const unsigned *counts,
                                                  const int *__restrict__ c_level, const int *__restrict__ c_parent,
                                                  const double *__restrict__ c_ctr, const TreeInfo *__restrict__ info,
                                                  const int *__restrict__ m2l_src, const Mom<T> *__restrict__ mom, T e2,
                                                  T *__restrict__ taylor) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const unsigned NL = counts[3];
    const unsigned warps = gridDim.x * (blockDim.x >> 5);
    for (unsigned li = blockIdx.x * (blockDim.x >> 5) + w; li < NL; li += warps) {
        const int c = leaves[li];
        if (c_level[c] < 2) continue;  // warp-uniform
        const RelC<T> cc = rel_centre<T>(c_ctr, c, info);
        T v[kTaylor] = {};
        int anc = c_level[c] >= 4 ? c_parent[c_parent[c]] : -1;
        while (anc >= 0 && c_level[anc] >= 2) {
            for (int s = lane; s < kM2LSlots; s += 32) {
                const int src = m2l_src[static_cast<size_t>(anc) * kM2LSlots + s];
                if (src < 0) continue;
                const Mom<T> r = mom[src];
                if (r.M == T(0)) continue;
                T d[3];
                src_offset<T>(r, cc, d);
                soft_term<T>(r, d[0], d[1], d[2], e2, v[0], v[1], v[2]);
                v[12] += soft_phi_term<T>(r, d[0], d[1], d[2], e2);
                const T u = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
                const T A = rsqrt_t<T>(u + e2), B = rsqrt_t<T>(u);
                const T A2 = A * A, B2 = B * B, A3 = A2 * A, B3 = B2 * B;
                const T F = A3 - B3, F1 = T(-1.5) * (A3 * A2 - B3 * B2);
#pragma unroll
                for (int a = 0; a < 3; ++a)
#pragma unroll
                    for (int q = 0; q < 3; ++q) v[3 + 3 * a + q] -= r.M * (T(2) * F1 * d[a] * d[q] + (a == q ? F : T(0)));
            }
            anc = c_parent[anc];
        }
#pragma unroll
        for (int k = 0; k < kTaylor; ++k) v[k] = warp_sum(v[k]);
        if (lane < kTaylor) {
            T out = v[0];
#pragma unroll
            for (int k = 1; k < kTaylor; ++k)
                if (lane == k) out = v[k];
            taylor[static_cast<size_t>(c) * kTaylor + lane] = out;
        }
    }
}

// -------------------------------------------- near levels (k = 0, 1) + apply
// One warp per leaf at level >= 2. The warp first lists the moment records of
// its sources (the leaf's M2L slots, face-slab sources as their 8 octant
// records, then the parent's slots) in shared memory, then streams them in
// batches of 32: each lane stages one record as its offset from the leaf
// centre plus M, tr Q and Q (the next batch's records are loaded while the
// current one is computed), and every lane applies the staged batch to up to
// kTPL of the leaf's particles (targets lane, lane + 32, ...). Last, the
// leaf-centre Taylor part is added and far = G (far + correction).
#ifndef GB_SOFT_TPL
#define GB_SOFT_TPL 2  // targets per lane per pass (measured at 4M, p = 10: 2 -> 38.4, 4 -> 40.8, 8 -> 51.7 ms per step)
#endif
#ifndef GB_SOFT_UNROLL
#define GB_SOFT_UNROLL 4  // record pairs per unrolled step of the FP32 loop (4: 37.9 against 38.5 ms per step for 1)
#endif
#ifndef GB_SOFT_MIN_BLOCKS
#define GB_SOFT_MIN_BLOCKS 1
#endif
constexpr int kSoftWarps = 4;
constexpr int kSoftTPL = GB_SOFT_TPL;
constexpr int kSoftUnroll = GB_SOFT_UNROLL;
constexpr int kSoftMaxSrc = 54 * 8 + 135 + 189;  // 756 records at most

template <typename T>
struct SRec {  // staged record: offset from the target leaf centre, M, tr Q, Q
    T dx, dy, dz, M, tr, q0, q1, q2, q3, q4, q5, pad;
};

template <typename T>
__device__ __forceinline__ void stage(const Mom<T> *__restrict__ mom, const Mom<T> *__restrict__ moct, int code,
                                      const RelC<T> &cc, SRec<T> &r) {
    if (code == INT_MIN) {  // padding entry: far away, no mass
        r.dx = T(1e10), r.dy = T(0), r.dz = T(0), r.M = T(0), r.tr = T(0);
        r.q0 = r.q1 = r.q2 = r.q3 = r.q4 = r.q5 = T(0);
        return;
    }
    const Mom<T> &m = code >= 0 ? mom[code] : moct[~code];
    if (m.M == T(0)) {
        r.dx = T(1e10), r.dy = T(0), r.dz = T(0), r.M = T(0), r.tr = T(0);
        r.q0 = r.q1 = r.q2 = r.q3 = r.q4 = r.q5 = T(0);
        return;
    }
    T d[3];
    src_offset<T>(m, cc, d);
    r.dx = d[0], r.dy = d[1], r.dz = d[2], r.M = m.M, r.tr = m.tr;
    r.q0 = m.Q[0], r.q1 = m.Q[1], r.q2 = m.Q[2], r.q3 = m.Q[3], r.q4 = m.Q[4], r.q5 = m.Q[5];
}

template <typename T>
__device__ __forceinline__ void soft_term_s(const SRec<T> &r, T tx, T ty, T tz, T e2, T &ax, T &ay, T &az) {
    const T dx = r.dx - tx, dy = r.dy - ty, dz = r.dz - tz;
    const T u = dx * dx + dy * dy + dz * dz;
    const T A = rsqrt_t<T>(u + e2), B = rsqrt_t<T>(u);
    const T A2 = A * A, B2 = B * B;
    const T A3 = A2 * A, B3 = B2 * B;
    const T A5 = A3 * A2, B5 = B3 * B2;
    const T A7 = A5 * A2, B7 = B5 * B2;
    const T F = A3 - B3;
    const T F1 = T(-1.5) * (A5 - B5);
    const T F2 = T(3.75) * (A7 - B7);
    const T qx = r.q0 * dx + r.q3 * dy + r.q4 * dz;
    const T qy = r.q3 * dx + r.q1 * dy + r.q5 * dz;
    const T qz = r.q4 * dx + r.q5 * dy + r.q2 * dz;
    const T dqd = dx * qx + dy * qy + dz * qz;
    const T a = r.M * F + F1 * r.tr + T(2) * F2 * dqd;
    const T b = T(2) * F1;
    ax += a * dx + b * qx;
    ay += a * dy + b * qy;
    az += a * dz + b * qz;
}

// FP32: two staged records per step on paired FP32 instructions (.f32x2, each
// component rounded as the scalar operation). A batch of 32 records is kept as
// 16 pairs of 24 floats, field-interleaved ((dx0, dx1, dy0, dy1), ...), so a
// pair is six 16-byte shared-memory loads. The records are staged with the
// term's constants folded in (tr' = -3/2 tr, Q' = 15/2 Q), so that
//   a = M F + F1 tr + 2 F2 d.Qd = M (A^3 - B^3) + tr' (A^5 - B^5) + d.Q'd (A^7 - B^7),
//   2 F1 Qd = -2/5 (A^5 - B^5) Q'd,
// three pipe operations per record fewer than soft_term_s.
__device__ __forceinline__ void put_paired(float *pb, int lane, const SRec<float> &r) {
    float *q = pb + 24 * (lane >> 1) + (lane & 1);
    q[0] = r.dx, q[2] = r.dy, q[4] = r.dz, q[6] = r.M, q[8] = -1.5f * r.tr, q[10] = 7.5f * r.q0;
    q[12] = 7.5f * r.q1, q[14] = 7.5f * r.q2, q[16] = 7.5f * r.q3, q[18] = 7.5f * r.q4, q[20] = 7.5f * r.q5, q[22] = 0.f;
}

__device__ __forceinline__ float2 rsqrt2(float2 x) { return make_float2(rsqrt_t<float>(x.x), rsqrt_t<float>(x.y)); }

__device__ __forceinline__ void soft_term_pair(const float4 *P, float2 ntx, float2 nty, float2 ntz, float2 e2, float2 &ax,
                                               float2 &ay, float2 &az) {
    const float4 a = P[0], b = P[1], c = P[2], d = P[3], e = P[4], f = P[5];
    const float2 m1 = make_float2(-1.f, -1.f);
    const float2 dx = __fadd2_rn(make_float2(a.x, a.y), ntx);
    const float2 dy = __fadd2_rn(make_float2(a.z, a.w), nty);
    const float2 dz = __fadd2_rn(make_float2(b.x, b.y), ntz);
    const float2 M = make_float2(b.z, b.w), tr = make_float2(c.x, c.y);
    const float2 q0 = make_float2(c.z, c.w), q1 = make_float2(d.x, d.y), q2 = make_float2(d.z, d.w);
    const float2 q3 = make_float2(e.x, e.y), q4 = make_float2(e.z, e.w), q5 = make_float2(f.x, f.y);
    const float2 u = __ffma2_rn(dx, dx, __ffma2_rn(dy, dy, __fmul2_rn(dz, dz)));
    const float2 A = rsqrt2(__fadd2_rn(u, e2)), B = rsqrt2(u);
    const float2 A2 = __fmul2_rn(A, A), B2 = __fmul2_rn(B, B);
    const float2 A3 = __fmul2_rn(A2, A), B3 = __fmul2_rn(B2, B);
    const float2 A5 = __fmul2_rn(A3, A2), B5 = __fmul2_rn(B3, B2);
    const float2 A7 = __fmul2_rn(A5, A2), B7 = __fmul2_rn(B5, B2);
    const float2 F = __ffma2_rn(B3, m1, A3);
    const float2 G5 = __ffma2_rn(B5, m1, A5);  // A^5 - B^5
    const float2 G7 = __ffma2_rn(B7, m1, A7);  // A^7 - B^7
    const float2 qx = __ffma2_rn(q0, dx, __ffma2_rn(q3, dy, __fmul2_rn(q4, dz)));  // Q'd
    const float2 qy = __ffma2_rn(q3, dx, __ffma2_rn(q1, dy, __fmul2_rn(q5, dz)));
    const float2 qz = __ffma2_rn(q4, dx, __ffma2_rn(q5, dy, __fmul2_rn(q2, dz)));
    const float2 dqd = __ffma2_rn(dx, qx, __ffma2_rn(dy, qy, __fmul2_rn(dz, qz)));
    const float2 sa = __ffma2_rn(G7, dqd, __ffma2_rn(tr, G5, __fmul2_rn(M, F)));
    const float2 sb = __fmul2_rn(make_float2(-0.4f, -0.4f), G5);
    ax = __ffma2_rn(sa, dx, __ffma2_rn(sb, qx, ax));
    ay = __ffma2_rn(sa, dy, __ffma2_rn(sb, qy, ay));
    az = __ffma2_rn(sa, dz, __ffma2_rn(sb, qz, az));
}

// kPhi: the potential's correction instead (after an evaluation, for the
// diagnostics): the scalar path, farphi[j] += correction (the far potential
// is multiplied by G where near and far are added).
template <typename T, bool kPhi = false>
__global__ void __launch_bounds__(kSoftWarps * 32, GB_SOFT_MIN_BLOCKS) k_soft_near(
    const int *__restrict__ leaves, const unsigned *counts, const int *__restrict__ c_begin, const int *__restrict__ c_end,
    const int *__restrict__ c_level, const int *__restrict__ c_parent, const int *__restrict__ c_child,
    const double *__restrict__ c_ctr, const TreeInfo *__restrict__ info, const int *__restrict__ m2l_src,
    const Mom<T> *__restrict__ mom, const Mom<T> *__restrict__ moct, const T *__restrict__ taylor,
    const double *__restrict__ xs, const float4 *__restrict__ ph, const float4 *__restrict__ pl, unsigned n, T e2, T G,
    T *__restrict__ far, double *__restrict__ farphi = nullptr, T *__restrict__ corr = nullptr) {
    __shared__ int list[kSoftWarps][kSoftMaxSrc + 32];
    __shared__ __align__(16) SRec<T> batch[kSoftWarps][32];  // FP32: the paired layout (put_paired)
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const unsigned NL = counts[3];
    const unsigned warps = gridDim.x * (blockDim.x >> 5);
    for (unsigned li = blockIdx.x * (blockDim.x >> 5) + w; li < NL; li += warps) {
        const int c = leaves[li];
        if (c_level[c] < 2) continue;  // warp-uniform
        const RelC<T> cc = rel_centre<T>(c_ctr, c, info);
        const double cd[3] = {c_ctr[3 * c], c_ctr[3 * c + 1], c_ctr[3 * c + 2]};
        const int P = c_parent[c];
        const int oc = c - c_child[P];
        // ---- the source list: codes >= 0 index mom, ~k indexes moct
        int nsrc = 0;
        for (int lev = 0; lev < 2; ++lev) {
            const int tc = lev == 0 ? c : (c_level[P] >= 2 ? P : -1);
            if (tc < 0) break;
            for (int s0 = 0; s0 < kM2LSlots; s0 += 32) {
                const int s = s0 + lane;
                const int src = s < kM2LSlots ? m2l_src[static_cast<size_t>(tc) * kM2LSlots + s] : -1;
                bool slab = false;
                if (lev == 0 && src >= 0) {
                    const int dd = s >> 3, o = s & 7;
                    const int d[3] = {dd % 3 - 1, (dd / 3) % 3 - 1, dd / 9 - 1};
                    int twos = 0, big = 0;
#pragma unroll
                    for (int a = 0; a < 3; ++a) {
                        const int off = 2 * d[a] + (1 - ((o >> a) & 1)) - (1 - ((oc >> a) & 1));
                        twos += (off == 2 || off == -2);
                        big += (off > 2 || off < -2);
                    }
                    slab = twos == 1 && big == 0;
                }
                const int cnt = src < 0 ? 0 : (slab ? 8 : 1);
                int incl = cnt;  // inclusive warp scan
#pragma unroll
                for (int o = 1; o < 32; o <<= 1) {
                    const int t = __shfl_up_sync(0xffffffffu, incl, o);
                    if (lane >= o) incl += t;
                }
                const int at = nsrc + incl - cnt;
                if (cnt == 1) {
                    list[w][at] = src;
                } else if (cnt == 8) {
                    const int ch = c_child[src];
                    for (int o = 0; o < 8; ++o) list[w][at + o] = ch >= 0 ? ch + o : ~(src * 8 + o);
                }
                nsrc += __shfl_sync(0xffffffffu, incl, 31);
            }
        }
        if (lane < 32) list[w][nsrc + lane] = INT_MIN;  // pad the last batch
        __syncwarp();
        T tl[kTaylor];
#pragma unroll
        for (int k = 0; k < kTaylor; ++k) tl[k] = taylor[static_cast<size_t>(c) * kTaylor + k];
        const int b = c_begin[c], e = c_end[c];
        for (int j0 = b; j0 < e; j0 += 32 * kSoftTPL) {
            const int nq = min(kSoftTPL, (e - j0 + 31) / 32);  // warp-uniform
            T ty[kSoftTPL][3], acc[kSoftTPL][3];
#pragma unroll
            for (int q = 0; q < kSoftTPL; ++q) {
                ty[q][0] = ty[q][1] = ty[q][2] = T(0);
                acc[q][0] = acc[q][1] = acc[q][2] = T(0);
                const int j = j0 + 32 * q + lane;
                if (q < nq && j < e) rel_pos<T>(j, xs, n, ph, pl, cd, cc, ty[q]);
            }
            SRec<T> nxt;
            if (nsrc > 0) stage<T>(mom, moct, list[w][lane], cc, nxt);
            if constexpr (sizeof(T) == 4 && !kPhi) {
                float *pb = reinterpret_cast<float *>(batch[w]);
                const float4 *pb4 = reinterpret_cast<const float4 *>(pb);
                const float2 e22 = make_float2(e2, e2);
                float2 nt[kSoftTPL][3], a2[kSoftTPL][3];
#pragma unroll
                for (int q = 0; q < kSoftTPL; ++q)
#pragma unroll
                    for (int a = 0; a < 3; ++a)
                        nt[q][a] = make_float2(-ty[q][a], -ty[q][a]), a2[q][a] = make_float2(0.f, 0.f);
                for (int b0 = 0; b0 < nsrc; b0 += 32) {
                    put_paired(pb, lane, nxt);
                    __syncwarp();
                    if (b0 + 32 < nsrc) stage<T>(mom, moct, list[w][b0 + 32 + lane], cc, nxt);
                    // a padded batch's tail holds massless records whose terms are exactly zero
                    const int npairs = (min(32, nsrc - b0) + 1) >> 1;
#pragma unroll kSoftUnroll
                    for (int k = 0; k < npairs; ++k) {
#pragma unroll
                        for (int q = 0; q < kSoftTPL; ++q)
                            if (q < nq)
                                soft_term_pair(pb4 + 6 * k, nt[q][0], nt[q][1], nt[q][2], e22, a2[q][0], a2[q][1], a2[q][2]);
                    }
                    __syncwarp();
                }
#pragma unroll
                for (int q = 0; q < kSoftTPL; ++q)
#pragma unroll
                    for (int a = 0; a < 3; ++a) acc[q][a] = a2[q][a].x + a2[q][a].y;
            } else {
                for (int b0 = 0; b0 < nsrc; b0 += 32) {
                    batch[w][lane] = nxt;
                    __syncwarp();
                    if (b0 + 32 < nsrc) stage<T>(mom, moct, list[w][b0 + 32 + lane], cc, nxt);
                    const int nb = min(32, nsrc - b0);
                    for (int k = 0; k < nb; ++k) {
                        const SRec<T> r = batch[w][k];
#pragma unroll
                        for (int q = 0; q < kSoftTPL; ++q) {
                            if (q >= nq) continue;
                            if (kPhi) {
                                Mom<T> m{};
                                m.M = r.M, m.tr = r.tr;
                                m.Q[0] = r.q0, m.Q[1] = r.q1, m.Q[2] = r.q2, m.Q[3] = r.q3, m.Q[4] = r.q4, m.Q[5] = r.q5;
                                acc[q][0] += soft_phi_term<T>(m, r.dx - ty[q][0], r.dy - ty[q][1], r.dz - ty[q][2], e2);
                            } else {
                                soft_term_s<T>(r, ty[q][0], ty[q][1], ty[q][2], e2, acc[q][0], acc[q][1], acc[q][2]);
                            }
                        }
                    }
                    __syncwarp();
                }
            }
#pragma unroll
            for (int q = 0; q < kSoftTPL; ++q) {
                const int j = j0 + 32 * q + lane;
                if (kPhi && q < nq && j < e) {
                    const T *y = ty[q];
                    // far levels: the centre's value and gradient (the field: a = grad phi here)
                    farphi[j] += static_cast<double>(acc[q][0] + tl[12] + tl[0] * y[0] + tl[1] * y[1] + tl[2] * y[2]);
                } else if (q < nq && j < e) {
                    const T *y = ty[q];
                    const T ax = acc[q][0] + tl[0] + tl[3] * y[0] + tl[4] * y[1] + tl[5] * y[2];
                    const T ay = acc[q][1] + tl[1] + tl[6] * y[0] + tl[7] * y[1] + tl[8] * y[2];
                    const T az = acc[q][2] + tl[2] + tl[9] * y[0] + tl[10] * y[1] + tl[11] * y[2];
                    if (corr) {  // kept apart; soften_apply folds it into the far field
                        corr[j] = ax, corr[n + j] = ay, corr[2 * static_cast<size_t>(n) + j] = az;
                    } else {
                        far[j] = G * (far[j] + ax);
                        far[n + j] = G * (far[n + j] + ay);
                        far[2 * static_cast<size_t>(n) + j] = G * (far[2 * static_cast<size_t>(n) + j] + az);
                    }
                }
            }
        }
        __syncwarp();
    }
}

// far = G (far + corr) for every particle (tree order): the particles the
// correction kernel skips have corr = 0 and far = 0 (leaves above level 2).
template <typename T>
__global__ void k_soft_apply(T *__restrict__ far, const T *__restrict__ corr, T G, size_t n3) {
    for (size_t e = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; e < n3; e += static_cast<size_t>(gridDim.x) * blockDim.x)
        far[e] = G * (far[e] + corr[e]);
}

// corr: null writes far = G (far + correction) after L2P; non-null writes the
// correction there (zeroed first), independent of the far-field chain.
template <typename T>
void launch_soften(Workspace &ws, T *corr) {
    const unsigned gw = capped_grid(static_cast<unsigned>(ws.num_sms) * 8, ceil_div(ws.c_cap, 4));  // a warp per leaf
    Mom<T> *mom = static_cast<Mom<T> *>(ws.smom);
    Mom<T> *moct = static_cast<Mom<T> *>(ws.smom_oct);
    T *taylor = static_cast<T *>(ws.staylor);
    const T e2 = static_cast<T>(ws.eps * ws.eps);
    if (corr) cudaMemsetAsync(corr, 0, sizeof(T) * 3 * static_cast<size_t>(ws.n), ws.st);
    k_mom_leaf<T><<<gw, 128, 0, ws.st>>>(ws.leaves, ws.d_counts, ws.c_begin, ws.c_end, ws.c_level, ws.c_ctr, ws.xs, ws.ph,
                                         ws.pl, ws.n, ws.info, static_cast<T>(ws.m), mom, moct);
    ws.launches += 1;
    const unsigned gu = capped_grid(static_cast<unsigned>(ws.num_sms) * 4, ceil_div(ws.s_cap, 256));
    for (int L = ws.sort_levels - 1; L >= 2; --L) {  // parents lie at levels < sort_levels (tree.cu)
        k_mom_up<T><<<gu, 256, 0, ws.st>>>(L, ws.info, ws.split_cell, ws.c_child, ws.c_ctr, mom);
        ws.launches += 1;
    }
    k_soft_far<T><<<gw, 128, 0, ws.st>>>(ws.leaves, ws.d_counts, ws.c_level, ws.c_parent, ws.c_ctr, ws.info, ws.m2l_src,
                                         mom, e2, taylor);
    k_soft_near<T><<<gw, kSoftWarps * 32, 0, ws.st>>>(ws.leaves, ws.d_counts, ws.c_begin, ws.c_end, ws.c_level, ws.c_parent,
                                          ws.c_child, ws.c_ctr, ws.info, ws.m2l_src, mom, moct, taylor, ws.xs, ws.ph,
                                          ws.pl, ws.n, e2, static_cast<T>(ws.G), static_cast<T *>(ws.farf), nullptr, corr);
    ws.launches += 2;
}

}  // namespace

template <typename T>
void launch_soften_phi(Workspace &ws, double *farphi) {
    const unsigned gw = capped_grid(static_cast<unsigned>(ws.num_sms) * 8, ceil_div(ws.c_cap, 4));
    k_soft_near<T, true><<<gw, kSoftWarps * 32, 0, ws.st>>>(
        ws.leaves, ws.d_counts, ws.c_begin, ws.c_end, ws.c_level, ws.c_parent, ws.c_child, ws.c_ctr, ws.info, ws.m2l_src,
        static_cast<const Mom<T> *>(ws.smom), static_cast<const Mom<T> *>(ws.smom_oct), static_cast<const T *>(ws.staylor),
        ws.xs, ws.ph, ws.pl, ws.n, static_cast<T>(ws.eps * ws.eps), static_cast<T>(ws.G), nullptr, farphi);
    ws.launches += 1;
}

// Accurate mode, after an evaluation (its moments and leaf-centre terms are
// still those of the current positions): farphi[j] += the potential's
// softening correction (tree order, no G).
void soften_phi(Workspace &ws, double *farphi) {
    if (ws.mixed)
        launch_soften_phi<float>(ws, farphi);
    else
        launch_soften_phi<double>(ws, farphi);
}

size_t soften_taylor_values() { return kTaylor; }

size_t soften_cell_bytes(bool mixed) {
    const size_t t = mixed ? sizeof(float) : sizeof(double);
    return 16 * t;  // one Mom record
}

void soften_pass(Workspace &ws) {
    timer_begin(ws, kTSoft);
    if (ws.mixed)
        launch_soften<float>(ws, nullptr);
    else
        launch_soften<double>(ws, nullptr);
    timer_end(ws, kTSoft);
}

void soften_corr(Workspace &ws) {
    if (ws.mixed)
        launch_soften<float>(ws, static_cast<float *>(ws.soft_corr));
    else
        launch_soften<double>(ws, static_cast<double *>(ws.soft_corr));
}

void soften_apply(Workspace &ws) {
    const size_t n3 = 3 * static_cast<size_t>(ws.n);
    const unsigned gs = capped_grid(static_cast<unsigned>(ws.num_sms) * 8, ceil_div(n3, 256));
    if (ws.mixed)
        k_soft_apply<float><<<gs, 256, 0, ws.st>>>(static_cast<float *>(ws.farf), static_cast<const float *>(ws.soft_corr),
                                                   static_cast<float>(ws.G), n3);
    else
        k_soft_apply<double><<<gs, 256, 0, ws.st>>>(static_cast<double *>(ws.farf), static_cast<const double *>(ws.soft_corr),
                                                    ws.G, n3);
    ws.launches += 1;
}

}  // namespace gb
