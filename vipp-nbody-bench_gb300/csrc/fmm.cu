// Far field of the reference's FMM (gravity/include/fmm.hpp:224-374,
// solver_ref.hpp:180-232) on the GPU: translation-operator construction,
// P2M, M2M, M2L, L2L, L2P, in FP64 or FP32, on scaled real-basis expansions
// (harmonics.cuh). Passes run as in the reference: P2M on leaves at level
// >= 2, M2M into non-leaves at level >= 2, M2L into every cell at level >= 2
// (index > 8), L2L into cells at level >= 3, L2P on leaves at level >= 2.
#include <cstdio>

#include <cooperative_groups.h>

#include "workspace.cuh"

// Far-field kernels that run beside the P2P blocks of the concurrent near
// field: GB_FAR_MIN_BLOCKS > 1 caps their registers (65536 / (threads x
// min blocks) per thread) so that they fit on an SM next to P2P.
#ifndef GB_FAR_MIN_BLOCKS
#define GB_FAR_MIN_BLOCKS 1
#endif
// FP32 P2M and L2P: 4 resident 128-thread blocks per SM (128 registers, no
// spills); uncapped they took ~200-240 registers and 2 blocks per SM, 15%
// slower. The FP64 forms stay uncapped (a cap of 128 spills ~1 KB).
#ifndef GB_P2M_MIN_BLOCKS
#define GB_P2M_MIN_BLOCKS 4
#endif
#ifndef GB_L2P_MIN_BLOCKS
#define GB_L2P_MIN_BLOCKS 4
#endif

namespace gb {

__constant__ HTab<double> c_htd;
__constant__ HTab<float> c_htf;
__constant__ ATab c_at;

template <typename T>
__device__ __forceinline__ const HTab<T> &htab();
template <>
__device__ __forceinline__ const HTab<double> &htab<double>() {
    return c_htd;
}
template <>
__device__ __forceinline__ const HTab<float> &htab<float>() {
    return c_htf;
}

cudaError_t upload_tables() {
    static HTab<double> hd;
    static HTab<float> hf;
    static ATab at;
    fill_tables(hd, at);
    convert_tables(hd, hf);
    cudaError_t e = cudaMemcpyToSymbol(c_htd, &hd, sizeof(hd));
    if (e == cudaSuccess) e = cudaMemcpyToSymbol(c_htf, &hf, sizeof(hf));
    if (e == cudaSuccess) e = cudaMemcpyToSymbol(c_at, &at, sizeof(at));
    return e;
}

namespace {

// Regular solid harmonics R_n^m(x,y,z), n <= D, m >= 0, visited degree by
// degree inside each order with the recurrence of harmonics.cuh, keeping only
// two previous degrees live: f(n, m, re, im).
template <int D, typename T, typename F>
__device__ __forceinline__ void for_each_regular(T x, T y, T z, F &&f) {
    const HTab<T> &t = htab<T>();
    const T r2 = x * x + y * y + z * z;
    T cre = 1, cim = 0;
#pragma unroll
    for (int m = 0; m <= D; ++m) {
        if (m > 0) {
            const T nre = t.mm[m] * (x * cre - y * cim);
            const T nim = t.mm[m] * (x * cim + y * cre);
            cre = nre, cim = nim;
        }
        f(m, m, cre, cim);
        if (m + 1 <= D) {
            T r1 = t.m1[m] * z * cre, i1 = t.m1[m] * z * cim;
            f(m + 1, m, r1, i1);
            T r0 = cre, i0 = cim;
#pragma unroll
            for (int n = m + 2; n <= D; ++n) {
                const T r2n = t.ra[n][m] * z * r1 - t.rb[n][m] * r2 * r0;
                const T i2n = t.ra[n][m] * z * i1 - t.rb[n][m] * r2 * i0;
                f(n, m, r2n, i2n);
                r0 = r1, i0 = i1, r1 = r2n, i1 = i2n;
            }
        }
    }
}

__device__ __forceinline__ double level_scale(const TreeInfo *info, int L) { return ldexp(info->S, -L); }

// ---------------------------------------------------------------- operators
// The same-level M2L entry (j,k,po | n,m,pi) is c(m') (Y or conj Y) with
//   c(m') = [phase(m') a(n,m') a(j,k) ((-1)^n ainv(j+n, m'-k))] rho^-(j+n+1)
// for m' = m and m' = -m. The bracket does not depend on the offset, so it is
// tabulated once per p (in FP64, multiplied in the same order as m2l_coef, so
// every entry keeps its bits) and an evaluation only multiplies by the
// offset's power of rho and harmonics.
struct M2LEnt {
    double t[2];        // bracket of the m' = m and m' = -m terms
    float tf[2];        // the same in FP32 (mixed precision)
    short y[2];         // index of Re Y_{j+n}^{|m'-k|} in yt (Im follows)
    signed char sg[2];  // Y order m' - k: 0 (real), +1, -1 (conjugate)
    unsigned char q;    // j + n
    unsigned char f;    // bit 0: m > 0 (second term), bit 1: input Im part, bit 2: output Im part
};

// Entries [kind K^2 + ro K + ri]: kind 0 M2L (m2l_coef without rho^-(j+n+1)
// and Y), 1 M2M and 2 L2L (m2m_coef / l2l_coef without |t|^deg and Y), so
// that an operator entry is t Z[y] with Z = Y rho^(-deg-1) (M2L) or Y |t|^deg.
__device__ void shift_entry(int kind, int j, int k, int n, int mm, double &t, int &deg, int &order) {
    t = 0, deg = 0, order = 0;
    if (kind == 1) {  // M2M: child (n, mm) into parent (j, k)
        const int nn = j - n, m_ = k - mm;
        if (nn < 0 || iabs(m_) > nn) return;
        deg = nn, order = -m_;
        t = phase_even(iabs(k) - iabs(m_) - iabs(mm)) * aco(c_at, nn, m_) * aco(c_at, n, mm) * aco_inv(c_at, j, k) *
            ldexp(1.0, -n);
    } else {  // L2L: parent (n, mm) into child (j, k)
        if (n < j || iabs(mm - k) > n - j) return;
        deg = n - j, order = mm - k;
        t = phase_even(iabs(mm) - iabs(mm - k) - iabs(k)) * aco(c_at, n - j, mm - k) * aco(c_at, j, k) *
            (((n + j) % 2 ? -1.0 : 1.0) * aco_inv(c_at, n, mm)) * ldexp(1.0, -(j + 1));
    }
}

__global__ void k_m2l_table(int p, M2LEnt *__restrict__ tab) {
    const int K = (p + 1) * (p + 1);
    for (int idx = blockIdx.x * blockDim.x + threadIdx.x; idx < 3 * K * K; idx += gridDim.x * blockDim.x) {
        const int kind = idx / (K * K), ro = (idx % (K * K)) / K, ri = idx % K;
        int j, k, po, n, m, pi;
        rdecode(ro, j, k, po);
        rdecode(ri, n, m, pi);
        M2LEnt e;
        if (kind > 0) {
            for (int s = 0; s < 2; ++s) {
                double t;
                int deg, order;
                shift_entry(kind, j, k, n, s == 0 ? m : -m, t, deg, order);
                if (s == 1 && m == 0) t = 0;
                e.t[s] = t;
                e.tf[s] = static_cast<float>(t);
                e.y[s] = static_cast<short>(ridx(deg, iabs(order), 0));
                e.sg[s] = static_cast<signed char>(order == 0 ? 0 : (order > 0 ? 1 : -1));
            }
            e.q = 0;
            e.f = static_cast<unsigned char>((m > 0 ? 1 : 0) | (pi ? 2 : 0) | (po ? 4 : 0));
            tab[idx] = e;
            continue;
        }
        for (int s = 0; s < 2; ++s) {
            const int mm = s == 0 ? m : -m;
            const int o = mm - k;
            e.t[s] = (s == 1 && m == 0) ? 0.0
                                        : phase_even(iabs(k - mm) - iabs(k) - iabs(mm)) * aco(c_at, n, mm) * aco(c_at, j, k) *
                                              ((n % 2 ? -1.0 : 1.0) * aco_inv(c_at, j + n, o));
            e.tf[s] = static_cast<float>(e.t[s]);
            e.y[s] = static_cast<short>(ridx(j + n, iabs(o), 0));
            e.sg[s] = static_cast<signed char>(o == 0 ? 0 : (o > 0 ? 1 : -1));
        }
        e.q = static_cast<unsigned char>(j + n);
        e.f = static_cast<unsigned char>((m > 0 ? 1 : 0) | (pi ? 2 : 0) | (po ? 4 : 0));
        tab[idx] = e;
    }
}

// One term of an M2L operator entry from a table entry: the bracket t times
// Z = Y_{j+n}^{m'-k} rho^-(j+n+1) (Z precomputed per operator, conjugated for
// negative orders). T = double: FP64 operators; T = float: the FP32 operators
// of the mixed forms (t and Z rounded to FP32, one FP32 product: ~2^-23).
template <typename T>
__device__ __forceinline__ void m2l_term(const M2LEnt &e, int s, const T *Z, T &re, T &im) {
    const T yr = Z[e.y[s]];
    T yi = e.sg[s] == 0 ? T(0) : Z[e.y[s] + 1];
    if (e.sg[s] < 0) yi = -yi;
    const T c = sizeof(T) == 4 ? static_cast<T>(e.tf[s]) : static_cast<T>(e.t[s]);
    re = c * yr;
    im = c * yi;
}

template <typename T>
__device__ __forceinline__ T m2l_entry(const M2LEnt &e, const T *Z) {
    T ar, ai, br = 0, bi = 0;
    m2l_term<T>(e, 0, Z, ar, ai);
    if (e.f & 1) m2l_term<T>(e, 1, Z, br, bi);
    T vr, vi;
    if ((e.f & 2) == 0) {
        vr = ar + br;
        vi = ai + bi;
    } else {
        vr = -(ai - bi);
        vi = ar - br;
    }
    return (e.f & 4) ? vi : vr;
}
// One block per operator: 343 same-level M2L offsets (adjacent ones unused),
// 8 M2M octants, 8 L2L octants. Shifts are the ideal cell-centre offsets of
// the current root box in units of the level's length s:
//   M2L  t = (dx Hx, dy Hy, dz Hz) / S,
//   M2M  t = child - parent = (+-Hx, +-Hy, +-Hz) / (4 S) (minus for a lower half),
//   L2L  t = parent - child.
// A forest's systems each get their own operators (blockIdx.y: system).
// Mixed precision writes the M2L operators in FP32 only (ops_f; the
// tensor-core images are split from them); FP64 writes both.
__global__ void k_build_ops(const TreeInfo *__restrict__ info_all, int p, const M2LEnt *__restrict__ m2l_tab,
                            double *__restrict__ ops_d, float *__restrict__ ops_f, bool mixed, int b0) {
    extern __shared__ double sm[];
    const int K = (p + 1) * (p + 1);
    const int b = b0 + static_cast<int>(blockIdx.x);
    const TreeInfo *info = info_all + blockIdx.y;
    int kind;
    double tv[3];
    if (b < 343) {
        const int d[3] = {b % 7 - 3, (b / 7) % 7 - 3, b / 49 - 3};
        if (abs(d[0]) <= 1 && abs(d[1]) <= 1 && abs(d[2]) <= 1) return;
        kind = 0;
        for (int a = 0; a < 3; ++a) tv[a] = d[a] * info->H[a] / info->S;
    } else {
        const int o = (b - 343) & 7;
        kind = b < kOpL2L ? 1 : 2;
        for (int a = 0; a < 3; ++a) {
            const double s = ((o >> a) & 1) ? -1.0 : 1.0;
            tv[a] = (kind == 1 ? s : -s) * info->H[a] / (4.0 * info->S);
        }
    }
    const int D = kind == 0 ? 2 * p : p;
    double *yt = sm;                   // (D+1)^2
    double *pw = sm + (2 * p + 1) * (2 * p + 1);  // 2p+3
    const double rho = sqrt(tv[0] * tv[0] + tv[1] * tv[1] + tv[2] * tv[2]);
    // solid_regular_rt's recurrences spread over threads, each value by the
    // same operations: thread 0 walks the diagonal (m, m), then thread m the
    // degrees of order m; thread 32 the powers of rho
    {
        const double x = tv[0] / rho, y = tv[1] / rho, z = tv[2] / rho;
        const HTab<double> &t = c_htd;
        if (threadIdx.x == 0) {
            double cre = 1, cim = 0;
            for (int m = 0; m <= D; ++m) {
                if (m > 0) {
                    const double nre = t.mm[m] * (x * cre - y * cim);
                    const double nim = t.mm[m] * (x * cim + y * cre);
                    cre = nre, cim = nim;
                }
                yt[ridx(m, m, 0)] = cre;
                if (m > 0) yt[ridx(m, m, 1)] = cim;
            }
        } else if (threadIdx.x == 32) {
            double a = 1;
            const double f = kind == 0 ? 1.0 / rho : rho;
            for (int i = 0; i < 2 * p + 3; ++i) pw[i] = a, a *= f;
        }
        __syncthreads();
        const int m = threadIdx.x;
        if (m <= D) {
            const double r2 = x * x + y * y + z * z;
            const double cre = yt[ridx(m, m, 0)], cim = m > 0 ? yt[ridx(m, m, 1)] : 0.0;
            if (m + 1 <= D) {
                yt[ridx(m + 1, m, 0)] = t.m1[m] * z * cre;
                if (m > 0) yt[ridx(m + 1, m, 1)] = t.m1[m] * z * cim;
            }
            for (int n = m + 2; n <= D; ++n) {
                yt[ridx(n, m, 0)] = t.ra[n][m] * z * yt[ridx(n - 1, m, 0)] - t.rb[n][m] * r2 * yt[ridx(n - 2, m, 0)];
                if (m > 0) yt[ridx(n, m, 1)] = t.ra[n][m] * z * yt[ridx(n - 1, m, 1)] - t.rb[n][m] * r2 * yt[ridx(n - 2, m, 1)];
            }
        }
        __syncthreads();
    }
    double *od = ops_d + (static_cast<size_t>(blockIdx.y) * kNumOps + b) * K * K;
    float *of = ops_f + (static_cast<size_t>(blockIdx.y) * kNumOps + b) * K * K;
    if (kind == 0) {
        // real_entry's combination of the two terms, from the table, with
        // Z[y] = yt[y] rho^-(deg y + 1) formed once per operator
        const int ny = (D + 1) * (D + 1);
        double *Z = pw + 2 * p + 3;
        float *Zf = reinterpret_cast<float *>(Z + (2 * p + 1) * (2 * p + 1));
        for (int y = threadIdx.x; y < ny; y += blockDim.x) {
            int dg = static_cast<int>(sqrtf(static_cast<float>(y)));
            while (dg * dg > y) --dg;
            while ((dg + 1) * (dg + 1) <= y) ++dg;
            Z[y] = yt[y] * pw[dg + 1];
            Zf[y] = static_cast<float>(Z[y]);
        }
        __syncthreads();
        if (mixed) {
            for (int idx = threadIdx.x; idx < K * K; idx += blockDim.x) of[idx] = m2l_entry<float>(m2l_tab[idx], Zf);
        } else {
            for (int idx = threadIdx.x; idx < K * K; idx += blockDim.x) {
                const double v = m2l_entry<double>(m2l_tab[idx], Z);
                od[idx] = v;
                of[idx] = static_cast<float>(v);
            }
        }
        return;
    }
    for (int idx = threadIdx.x; idx < K * K; idx += blockDim.x) {
        const int ro = idx / K, ri = idx % K;  // output-major storage: [ro][ri]
        int j, k, po, n, m, pi;
        rdecode(ro, j, k, po);
        rdecode(ri, n, m, pi);
        const double v = real_entry(kind, c_at, yt, pw, j, k, po, n, m, pi);
        od[idx] = v;
        of[idx] = static_cast<float>(v);
    }
}

// Z tables of the mixed forms' FP32 operators, one thread per (system,
// operator), or per (system, operator, order m) when there are few systems
// (cols = 2p + 1: shorter serial chains, the prologue repeated per order), so
// that every lane of the FP64 pipe works (spread over a warp's lanes as
// k_build_ops does, most FP64 issue slots went to idle lanes and the tables
// cost ~2 ms per evaluation for 512 systems). The harmonics follow
// k_build_ops's recurrences value by value: the diagonal up to (m, m), then
// column m down with two running values.
// Z[y] = Y(y) rho^-(deg y + 1) (M2L) or Y(y) |t|^deg y (M2M, L2L), stride nmax.
__global__ void k_zf_tables(const TreeInfo *__restrict__ info_all, int nsys, int p, int cols, float *__restrict__ zf) {
    const long long gid = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x;
    if (gid >= static_cast<long long>(nsys) * kNumOps * cols) return;
    const int mcol = static_cast<int>(gid % cols);
    const int sidx = static_cast<int>(gid / cols / kNumOps), b = static_cast<int>((gid / cols) % kNumOps);
    const int nmax = (2 * p + 1) * (2 * p + 1);
    int kind = 0, oct = 0;
    const int dd[3] = {b % 7 - 3, (b / 7) % 7 - 3, b / 49 - 3};
    if (b < kOpM2M) {
        if (abs(dd[0]) <= 1 && abs(dd[1]) <= 1 && abs(dd[2]) <= 1) return;
    } else {
        kind = b < kOpL2L ? 1 : 2;
        oct = (b - kOpM2M) & 7;
    }
    const int D = kind == 0 ? 2 * p : p;
    if (mcol > D) return;
    const int m_end = cols == 1 ? D : mcol;  // orders mcol .. m_end
    const TreeInfo *info = info_all + sidx;
    double tv[3];
    if (kind == 0) {
        for (int a = 0; a < 3; ++a) tv[a] = dd[a] * info->H[a] / info->S;
    } else {
        for (int a = 0; a < 3; ++a) {
            const double sg = ((oct >> a) & 1) ? -1.0 : 1.0;
            tv[a] = (kind == 1 ? sg : -sg) * info->H[a] / (4.0 * info->S);
        }
    }
    const double rho = sqrt(tv[0] * tv[0] + tv[1] * tv[1] + tv[2] * tv[2]);
    const double x = tv[0] / rho, y = tv[1] / rho, z = tv[2] / rho;
    const double r2 = x * x + y * y + z * z;
    double pw[2 * kMaxP + 3];
    {
        double a = 1;
        const double f = kind == 0 ? 1.0 / rho : rho;
        for (int i = 0; i < 2 * p + 3; ++i) pw[i] = a, a *= f;
    }
    const int sh = kind == 0 ? 1 : 0;  // Z's power of rho: deg + 1 (M2L), deg (M2M, L2L)
    float *Z = zf + (static_cast<size_t>(sidx) * kNumOps + b) * nmax;
    const HTab<double> &t = c_htd;
    double cre = 1, cim = 0;  // Y(m, m)
    for (int m = 1; m <= mcol; ++m) {
        const double nre = t.mm[m] * (x * cre - y * cim);
        const double nim = t.mm[m] * (x * cim + y * cre);
        cre = nre, cim = nim;
    }
    for (int m = mcol; m <= m_end; ++m) {
        if (m > mcol) {
            const double nre = t.mm[m] * (x * cre - y * cim);
            const double nim = t.mm[m] * (x * cim + y * cre);
            cre = nre, cim = nim;
        }
        Z[ridx(m, m, 0)] = static_cast<float>(cre * pw[m + sh]);
        if (m > 0) Z[ridx(m, m, 1)] = static_cast<float>(cim * pw[m + sh]);
        if (m + 1 > D) continue;
        double ar = cre, ai = cim;  // Y(n - 2, m)
        double br = t.m1[m] * z * cre, bi = m > 0 ? t.m1[m] * z * cim : 0.0;  // Y(n - 1, m)
        Z[ridx(m + 1, m, 0)] = static_cast<float>(br * pw[m + 1 + sh]);
        if (m > 0) Z[ridx(m + 1, m, 1)] = static_cast<float>(bi * pw[m + 1 + sh]);
        for (int n = m + 2; n <= D; ++n) {
            const double vr = t.ra[n][m] * z * br - t.rb[n][m] * r2 * ar;
            Z[ridx(n, m, 0)] = static_cast<float>(vr * pw[n + sh]);
            ar = br, br = vr;
            if (m > 0) {
                const double vi = t.ra[n][m] * z * bi - t.rb[n][m] * r2 * ai;
                Z[ridx(n, m, 1)] = static_cast<float>(vi * pw[n + sh]);
                ai = bi, bi = vi;
            }
        }
    }
}

// The FP32 operators of the mixed forms for kSysPerBlock systems at once
// (blockIdx.x: operator, as in k_build_ops; blockIdx.y: group of systems),
// from the Z tables of k_zf_tables: every thread reads each table entry once
// for all the group's systems (the entry table is the main traffic: one read
// per operator made a forest's 512 x 359 operators cost ~8 ms per
// evaluation). Entries t Z[y] (M2LEnt tables: M2L, M2M, L2L).
constexpr int kSysPerBlock = 8;

__global__ void __launch_bounds__(32 * kSysPerBlock) k_build_ops_f(int nsys, int p, const M2LEnt *__restrict__ tabs,
                                                               const float *__restrict__ zf, float *__restrict__ ops_f) {
    extern __shared__ float smf[];
    const int K = (p + 1) * (p + 1), nmax = (2 * p + 1) * (2 * p + 1);
    const int b = blockIdx.x;
    int kind = 0;
    const int dd[3] = {b % 7 - 3, (b / 7) % 7 - 3, b / 49 - 3};
    if (b < kOpM2M) {
        if (abs(dd[0]) <= 1 && abs(dd[1]) <= 1 && abs(dd[2]) <= 1) return;
    } else {
        kind = b < kOpL2L ? 1 : 2;
    }
    const int D = kind == 0 ? 2 * p : p, ny = (D + 1) * (D + 1);
    const M2LEnt *tab = tabs + static_cast<size_t>(kind) * K * K;
    const int sys0 = blockIdx.y * kSysPerBlock;
    const int ng = min(kSysPerBlock, nsys - sys0);
    for (int i = threadIdx.x; i < ng * ny; i += blockDim.x) {
        const int q = i / ny, yy = i - q * ny;
        smf[q * nmax + yy] = zf[(static_cast<size_t>(sys0 + q) * kNumOps + b) * nmax + yy];
    }
    __syncthreads();
    for (int idx = threadIdx.x; idx < K * K; idx += blockDim.x) {
        const M2LEnt e = tab[idx];
        for (int q = 0; q < ng; ++q)
            ops_f[((static_cast<size_t>(sys0 + q)) * kNumOps + b) * K * K + idx] = m2l_entry<float>(e, smf + q * nmax);
    }
}

// Particle position relative to cell centre c in units of s: FP64 from xs,
// or (FP32 forms) from the hi/lo pairs re-centred on the cell, which keeps the
// FP64 pipe out of the per-particle work.
template <typename T>
struct CellFrame {
    double cx, cy, cz, inv_s;
    RootC cc;
    float is;
    __device__ __forceinline__ CellFrame(const double *c_ctr, int c, const TreeInfo *info, double inv_s_) {
        cx = c_ctr[3 * c], cy = c_ctr[3 * c + 1], cz = c_ctr[3 * c + 2], inv_s = inv_s_;
        if (sizeof(T) == 4) cc = leaf_centre(c_ctr, c, info), is = static_cast<float>(inv_s_);
    }
    __device__ __forceinline__ void at(int j, const double *xs, unsigned n, const float4 *ph, const float4 *pl, T &ux, T &uy,
                                       T &uz) const {
        if (sizeof(T) == 4) {
            const float4 h = ph[j], l = pl[j];
            ux = static_cast<T>(((h.x - cc.hx) + (l.x - cc.lx)) * is);
            uy = static_cast<T>(((h.y - cc.hy) + (l.y - cc.ly)) * is);
            uz = static_cast<T>(((h.z - cc.hz) + (l.z - cc.lz)) * is);
        } else {
            ux = static_cast<T>((xs[j] - cx) * inv_s);
            uy = static_cast<T>((xs[n + j] - cy) * inv_s);
            uz = static_cast<T>((xs[2 * static_cast<size_t>(n) + j] - cz) * inv_s);
        }
    }
};

// --------------------------------------------------------------------- P2M
// One step of a warp reduce-scatter: each lane keeps one half of its S values
// (the upper half if lane & o) and adds its partner's copy of that half.
template <int S, typename T>
__device__ __forceinline__ void rs_step(T *a, int lane, int o) {
    const bool up = (lane & o) != 0;
#pragma unroll
    for (int i = 0; i < S / 2; ++i) {
        const T send = up ? a[i] : a[i + S / 2];
        const T keep = up ? a[i + S / 2] : a[i];
        a[i] = keep + __shfl_xor_sync(0xffffffffu, send, o);
    }
}

// One warp per leaf at level >= 2: M~_n^m = sum_i m conj(R_n^m((x_i - c)/s)).
// The lanes' partial sums (KR = K rounded up to 32) are combined by a
// five-step reduce-scatter, after which lane l holds coefficients
// [KR/32 l, KR/32 (l+1)): 2 KR shuffles instead of 5 K.
template <int P, typename T>
__global__ void __launch_bounds__(128, sizeof(T) == 4 ? GB_P2M_MIN_BLOCKS : GB_FAR_MIN_BLOCKS) k_p2m(const int *__restrict__ leaves, const unsigned *counts,
                                             const int *__restrict__ c_begin, const int *__restrict__ c_end,
                                             const int *__restrict__ c_level, const double *__restrict__ c_ctr,
                                             const double *__restrict__ xs, const float4 *__restrict__ ph,
                                             const float4 *__restrict__ pl, unsigned n, const TreeInfo *__restrict__ info_all,
                                             const int *__restrict__ c_sys, double mass, T *__restrict__ M) {
    constexpr int K = (P + 1) * (P + 1);
    const int lane = threadIdx.x & 31;
    const unsigned NL = counts[3];
    const unsigned warps = gridDim.x * (blockDim.x >> 5);
    for (unsigned li = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); li < NL; li += warps) {
        const int c = leaves[li];
        const int L = c_level[c];
        if (L < 2) continue;
        const TreeInfo *info = info_all + cell_system(c_sys, c);
        const CellFrame<T> fr(c_ctr, c, info, 1.0 / level_scale(info, L));
        constexpr int KR = (K + 31) / 32 * 32;
        T acc[KR];
#pragma unroll
        for (int r = 0; r < KR; ++r) acc[r] = 0;
        const T q = static_cast<T>(c_sys ? info->m : mass);
        for (int j = c_begin[c] + lane; j < c_end[c]; j += 32) {
            T ux, uy, uz;
            fr.at(j, xs, n, ph, pl, ux, uy, uz);
            for_each_regular<P, T>(ux, uy, uz, [&](int nn, int mm, T re, T im) {
                acc[ridx(nn, mm, 0)] += q * re;
                if (mm > 0) acc[ridx(nn, mm, 1)] -= q * im;
            });
        }
        rs_step<KR>(acc, lane, 16);
        rs_step<KR / 2>(acc, lane, 8);
        rs_step<KR / 4>(acc, lane, 4);
        rs_step<KR / 8>(acc, lane, 2);
        rs_step<KR / 16>(acc, lane, 1);
#pragma unroll
        for (int i = 0; i < KR / 32; ++i) {
            const int r = (KR / 32) * lane + i;
            if (r < K) M[static_cast<size_t>(c) * K + r] = acc[i];
        }
    }
}

// ------------------------------------------------------------ tile GEMM core
// M2M, M2L and L2L are all D[64 targets][K] += A[64][K] x Op^T with a K x K
// operator. Both operands sit in shared memory with the input index
// contiguous and a row stride KS (elements) with KS * sizeof(T) = 16 mod 128
// bytes, so the 16-byte vector loads of 8 consecutive rows fall into distinct
// bank groups. 256 threads: ty = 0..15 owns 4 target rows, tx = 0..15 owns the
// output columns tx + 16 j (j < NJ).
constexpr int kTile = 64;
static_assert(kTile == kM2LTileCC, "forest M2L tiles");

constexpr int tile_stride(int K, int esz) {
    int vw = 16 / esz;
    int s = (K + vw - 1) / vw * vw;
    while ((s * esz) % 128 != 16) s += vw;
    return s;
}

template <int P, typename T>
struct TileCfg {
    static constexpr int K = (P + 1) * (P + 1);
    static constexpr int KS = tile_stride(K, static_cast<int>(sizeof(T)));
    static constexpr int KO = (K + 15) / 16 * 16;
    static constexpr int NJ = KO / 16;
    static constexpr int VW = 16 / static_cast<int>(sizeof(T));
    static constexpr size_t smem = sizeof(T) * static_cast<size_t>(kTile + KO) * KS;
};

template <typename T>
struct Vec16;
template <>
struct Vec16<float> {
    using type = float4;
};
template <>
struct Vec16<double> {
    using type = double2;
};

__device__ __forceinline__ float vget(const float4 &v, int e) { return e == 0 ? v.x : e == 1 ? v.y : e == 2 ? v.z : v.w; }
__device__ __forceinline__ double vget(const double2 &v, int e) { return e == 0 ? v.x : v.y; }

template <int P, typename T>
__device__ __forceinline__ void tile_gemm(const T *__restrict__ A, const T *__restrict__ Op, T (&acc)[4][TileCfg<P, T>::NJ],
                                          int ty, int tx) {
    using C = TileCfg<P, T>;
    using V = typename Vec16<T>::type;
#pragma unroll 2
    for (int ci = 0; ci < C::KS; ci += C::VW) {
        V av[4], ov[C::NJ];
#pragma unroll
        for (int a = 0; a < 4; ++a) av[a] = *reinterpret_cast<const V *>(A + (ty * 4 + a) * C::KS + ci);
#pragma unroll
        for (int j = 0; j < C::NJ; ++j) ov[j] = *reinterpret_cast<const V *>(Op + (tx + 16 * j) * C::KS + ci);
#pragma unroll
        for (int e = 0; e < C::VW; ++e)
#pragma unroll
            for (int a = 0; a < 4; ++a)
#pragma unroll
                for (int j = 0; j < C::NJ; ++j) acc[a][j] += vget(av[a], e) * vget(ov[j], e);
    }
}

// Zero both tiles (padding stays zero: later loads write columns < K only).
template <int P, typename T>
__device__ __forceinline__ void tile_clear(T *sm) {
    using C = TileCfg<P, T>;
    for (int i = threadIdx.x; i < (kTile + C::KO) * C::KS; i += blockDim.x) sm[i] = T(0);
}

// Op tile <- operator oi (global, output-major K x K).
template <int P, typename T>
__device__ __forceinline__ void tile_load_op(T *Op, const T *__restrict__ ops, int oi) {
    using C = TileCfg<P, T>;
    const T *op = ops + static_cast<size_t>(oi) * C::K * C::K;
    for (int i = threadIdx.x; i < C::K * C::K; i += blockDim.x) Op[(i / C::K) * C::KS + i % C::K] = op[i];
}

// A row t <- expansion of cell src[t] (zero when src[t] < 0).
template <int P, typename T>
__device__ __forceinline__ void tile_gather(T *A, const int *srcs, const T *__restrict__ X) {
    using C = TileCfg<P, T>;
    for (int i = threadIdx.x; i < kTile * C::K; i += blockDim.x) {
        const int t = i / C::K, ci = i % C::K;
        const int s = srcs[t];
        A[t * C::KS + ci] = s >= 0 ? X[static_cast<size_t>(s) * C::K + ci] : T(0);
    }
}

// --------------------------------------------------------------------- M2M
// One block per non-leaf cell of level L (>= 2): M~ = sum_o M2M_o M~_child(o).
// --------------------------------------------------------------------- M2L
// Targets: every cell at level >= 2, grouped by octant (cells 1 + 8q + o share
// octant o), so that one tile of 64 targets shares the same 189 source slots
// (parent-neighbour d, child o') and each slot maps to one offset operator.
// Per slot: gather the tile's source expansions, multiply by the operator.
// A forest (otile non-null) takes its tiles from the per-system octet lists
// (tree.cu: forest_tiles), each tile with its system's operators.
template <int P, typename T>
__global__ void __launch_bounds__(256) k_m2l(const TreeInfo *__restrict__ info, const int *__restrict__ m2l_src,
                                             const T *__restrict__ ops_all, const int4 *__restrict__ otile,
                                             const int *__restrict__ oct_list, const T *__restrict__ M, T *__restrict__ Lx) {
    using C = TileCfg<P, T>;
    extern __shared__ __align__(16) unsigned char smraw[];
    T *A = reinterpret_cast<T *>(smraw);  // [64][KS]
    T *Op = A + kTile * C::KS;             // [KO][KS]
    __shared__ int srcs[kTile], trow[kTile];
    const int tid = threadIdx.x, ty = tid >> 4, tx = tid & 15;
    const int base = info->level_start[2];
    const int ntgt = info->n_targets_m2l;
    if (ntgt <= 0) return;
    const int per_class = ntgt / 8;
    const int tiles_per_class = otile ? info->n_otiles : (per_class + kTile - 1) / kTile;
    tile_clear<P, T>(A);
    for (int w = blockIdx.x; w < 8 * tiles_per_class; w += gridDim.x) {
        const int cls = w % 8, tile = w / 8;
        const T *ops = ops_all;
        __syncthreads();  // the previous tile's rows are written out
        int rows;  // targets of the tile (rows past them skip the GEMM)
        if (otile) {
            const int4 ot = otile[tile];
            ops = ops_all + static_cast<size_t>(ot.x) * kNumOps * C::K * C::K;
            rows = ot.z;
            if (tid < kTile) trow[tid] = tid < ot.z ? base + cls + 8 * oct_list[ot.y + tid] : -1;
        } else {
            rows = per_class - tile * kTile;
            if (tid < kTile) {
                const int t = tile * kTile + tid;
                trow[tid] = t < per_class ? base + cls + 8 * t : -1;
            }
        }
        T acc[4][C::NJ];
#pragma unroll
        for (int a = 0; a < 4; ++a)
#pragma unroll
            for (int j = 0; j < C::NJ; ++j) acc[a][j] = 0;
        const int uc[3] = {1 - (cls & 1), 1 - ((cls >> 1) & 1), 1 - ((cls >> 2) & 1)};
        for (int s = 0; s < kM2LSlots; ++s) {
            const int dd = s >> 3, o = s & 7;
            const int off[3] = {2 * (dd % 3 - 1) + 1 - (o & 1) - uc[0], 2 * ((dd / 3) % 3 - 1) + 1 - ((o >> 1) & 1) - uc[1],
                                2 * (dd / 9 - 1) + 1 - ((o >> 2) & 1) - uc[2]};
            if (off[0] >= -1 && off[0] <= 1 && off[1] >= -1 && off[1] <= 1 && off[2] >= -1 && off[2] <= 1) continue;
            int any = 0;
            if (tid < kTile) {
                const int src = trow[tid] >= 0 ? m2l_src[static_cast<size_t>(trow[tid]) * kM2LSlots + s] : -1;
                srcs[tid] = src;
                any = src >= 0;
            }
            if (!__syncthreads_or(any)) continue;
            tile_load_op<P, T>(Op, ops, (off[0] + 3) + 7 * (off[1] + 3) + 49 * (off[2] + 3));
            tile_gather<P, T>(A, srcs, M);
            __syncthreads();
            if (ty * 4 < rows) tile_gemm<P, T>(A, Op, acc, ty, tx);
            __syncthreads();
        }
#pragma unroll
        for (int a = 0; a < 4; ++a) {
            if (trow[ty * 4 + a] < 0) continue;
            const size_t c = static_cast<size_t>(trow[ty * 4 + a]);
#pragma unroll
            for (int j = 0; j < C::NJ; ++j) {
                const int r = tx + 16 * j;
                if (r < C::K) Lx[c * C::K + r] = acc[a][j];
            }
        }
    }
}

// M2M for one level L >= 2 on thread-block clusters of 8 CTAs: a cluster
// takes a tile of 64 non-leaf cells and CTA o of the cluster applies M2M_o to
// the children in octant o. Each CTA leaves its partial tile in its shared
// memory; after a cluster barrier, CTA o adds rows 8o .. 8o+7 of the eight
// partial tiles through distributed shared memory, in octant order 0..7, and
// writes the parents' multipoles. (One CTA doing the 8 octants in turn made a
// level cost ~165 us whatever its size.)
template <int P, typename T>
__global__ void __cluster_dims__(8, 1, 1) __launch_bounds__(256, GB_FAR_MIN_BLOCKS)
    k_m2m(int L, const TreeInfo *__restrict__ info, const int *__restrict__ split_cell, const int *__restrict__ c_child,
          const T *__restrict__ ops_all, const int2 *__restrict__ etile, const int *__restrict__ c_sys, T *M) {
    namespace cg = cooperative_groups;
    using C = TileCfg<P, T>;
    extern __shared__ __align__(16) unsigned char smraw[];
    T *A = reinterpret_cast<T *>(smraw);  // [64][KS]: gathered children, then the partial tile
    T *Op = A + kTile * C::KS;
    __shared__ int par[kTile], srcs[kTile];
    cg::cluster_group cluster = cg::this_cluster();
    const int o = static_cast<int>(cluster.block_rank());
    const int tid = threadIdx.x, ty = tid >> 4, tx = tid & 15;
    const int e0 = info->split_start[L], cnt = info->split_count[L];
    // a forest's tiles: one system each, with that system's operator
    const int et0 = etile ? info->etile_start[L] : 0;
    const int tiles = etile ? info->etile_end[L] - et0 : (cnt + kTile - 1) / kTile;
    // uniform over each cluster (it shares blockIdx.x / 8): a cluster without a
    // tile reaches no cluster barrier and skips loading its operator
    if (static_cast<int>(blockIdx.x) / 8 >= tiles) return;
    tile_clear<P, T>(A);
    int loaded = -1;  // system whose operator is in Op
    const int nclusters = static_cast<int>(gridDim.x) / 8;
    for (int w = static_cast<int>(blockIdx.x) / 8; w < tiles; w += nclusters) {  // same w in all 8 CTAs
        int first = e0 + w * kTile, count = cnt - w * kTile, sys = 0;
        if (etile) {
            const int2 et = etile[et0 + w];
            first = et.x, count = et.y, sys = c_sys[split_cell[first]];
        }
        if (sys != loaded) {  // Op is not read here: the previous tile ended with a cluster barrier
            tile_load_op<P, T>(Op, ops_all + static_cast<size_t>(sys) * kNumOps * C::K * C::K, kOpM2M + o);
            loaded = sys;
        }
        if (tid < kTile) {
            par[tid] = tid < count ? split_cell[first + tid] : -1;
            srcs[tid] = par[tid] >= 0 ? c_child[par[tid]] + o : -1;
        }
        __syncthreads();
        tile_gather<P, T>(A, srcs, M);
        __syncthreads();
        T acc[4][C::NJ];
#pragma unroll
        for (int a = 0; a < 4; ++a)
#pragma unroll
            for (int j = 0; j < C::NJ; ++j) acc[a][j] = 0;
        if (ty * 4 < count) tile_gemm<P, T>(A, Op, acc, ty, tx);  // rows past the tile's parents are not stored
        __syncthreads();
#pragma unroll
        for (int a = 0; a < 4; ++a)
#pragma unroll
            for (int j = 0; j < C::NJ; ++j) {
                const int r = tx + 16 * j;
                if (r < C::K) A[(ty * 4 + a) * C::KS + r] = acc[a][j];
            }
        cluster.sync();  // all eight partial tiles written
        for (int i = tid; i < 8 * C::K; i += blockDim.x) {
            const int row = 8 * o + i / C::K, r = i % C::K;
            const int pc = par[row];
            if (pc < 0) continue;
            T sum = 0;
#pragma unroll
            for (int q = 0; q < 8; ++q) sum += cluster.map_shared_rank(A, q)[row * C::KS + r];
            M[static_cast<size_t>(pc) * C::K + r] = sum;
        }
        cluster.sync();  // no CTA overwrites its partial tile while others read it
    }
}

// L2L into level Lp+1 (Lp >= 2): for each octant o, tiles of 64 non-leaf cells
// of level Lp; child o of each gets L~ += L2L_o L~_parent.
template <int P, typename T>
__global__ void __launch_bounds__(256, GB_FAR_MIN_BLOCKS) k_l2l(int Lp, const TreeInfo *__restrict__ info, const int *__restrict__ split_cell,
                                             const int *__restrict__ c_child, const T *__restrict__ ops_all,
                                             const int2 *__restrict__ etile, const int *__restrict__ c_sys, T *Lx) {
    using C = TileCfg<P, T>;
    extern __shared__ __align__(16) unsigned char smraw[];
    T *A = reinterpret_cast<T *>(smraw);
    T *Op = A + kTile * C::KS;
    __shared__ int par[kTile];
    const int tid = threadIdx.x, ty = tid >> 4, tx = tid & 15;
    const int e0 = info->split_start[Lp], cnt = info->split_count[Lp];
    const int et0 = etile ? info->etile_start[Lp] : 0;
    const int tiles = etile ? info->etile_end[Lp] - et0 : (cnt + kTile - 1) / kTile;
    if (static_cast<int>(blockIdx.x) >= 8 * tiles) return;  // no (tile, octant) for this block
    tile_clear<P, T>(A);
    for (int w = blockIdx.x; w < 8 * tiles; w += gridDim.x) {
        const int o = w % 8, tile = w / 8;
        int first = e0 + tile * kTile, count = cnt - tile * kTile, sys = 0;
        if (etile) {
            const int2 et = etile[et0 + tile];
            first = et.x, count = et.y, sys = c_sys[split_cell[first]];
        }
        __syncthreads();
        if (tid < kTile) par[tid] = tid < count ? split_cell[first + tid] : -1;
        __syncthreads();
        tile_load_op<P, T>(Op, ops_all + static_cast<size_t>(sys) * kNumOps * C::K * C::K, kOpL2L + o);
        tile_gather<P, T>(A, par, Lx);
        __syncthreads();
        T acc[4][C::NJ];
#pragma unroll
        for (int a = 0; a < 4; ++a)
#pragma unroll
            for (int j = 0; j < C::NJ; ++j) acc[a][j] = 0;
        if (ty * 4 < count) tile_gemm<P, T>(A, Op, acc, ty, tx);
#pragma unroll
        for (int a = 0; a < 4; ++a) {
            const int pc = par[ty * 4 + a];
            if (pc < 0) continue;
            const size_t c = static_cast<size_t>(c_child[pc] + o);
#pragma unroll
            for (int j = 0; j < C::NJ; ++j) {
                const int r = tx + 16 * j;
                if (r < C::K) Lx[c * C::K + r] += acc[a][j];
            }
        }
    }
}

// --------------------------------------------------------------------- L2P
// One warp per leaf at level >= 2. With u = (x - c)/s the potential of the
// local expansion is Phi = (1/s) sum_j [L~_j^0 R_j^0(u) + 2 Re sum_k L~_j^k R_j^k(u)];
// the acceleration grad Phi follows from the ladder relations (harmonics.cuh):
//   a_x + i a_y = s^-2 sum_j [ sum_{k>=0} L~_j^k sqrt((j-k)(j-k-1)) R_{j-1}^{k+1}
//                             - sum_{k>=1} conj(L~_j^k) sqrt((j+k)(j+k-1)) conj(R_{j-1}^{k-1}) ]
//   a_z        = s^-2 sum_j [ L~_j^0 j R_{j-1}^0 + 2 Re sum_{k>=1} L~_j^k sqrt((j-k)(j+k)) R_{j-1}^k ]
// so every R_n^q (n <= p-1) meets L~ of degree n+1 and orders q-1, q, q+1.
template <int P, typename T>
__global__ void __launch_bounds__(128, sizeof(T) == 4 ? GB_L2P_MIN_BLOCKS : GB_FAR_MIN_BLOCKS) k_l2p(const int *__restrict__ leaves, const unsigned *counts,
                                             const int *__restrict__ c_begin, const int *__restrict__ c_end,
                                             const int *__restrict__ c_level, const double *__restrict__ c_ctr,
                                             const double *__restrict__ xs, const float4 *__restrict__ ph,
                                             const float4 *__restrict__ pl, unsigned n, const TreeInfo *__restrict__ info_all,
                                             const int *__restrict__ c_sys, const T *__restrict__ Lx, T *__restrict__ far) {
    constexpr int K = (P + 1) * (P + 1);
    __shared__ T Ls[4][K];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const unsigned NL = counts[3];
    const unsigned warps = gridDim.x * (blockDim.x >> 5);
    const HTab<T> &t = htab<T>();
    for (unsigned li = blockIdx.x * (blockDim.x >> 5) + w; li < NL; li += warps) {
        const int c = leaves[li];
        const int L = c_level[c];
        if (L < 2) {  // no local expansion: these particles' far field is zero
            for (int j = c_begin[c] + lane; j < c_end[c]; j += 32)
                far[j] = T(0), far[n + j] = T(0), far[2 * static_cast<size_t>(n) + j] = T(0);
            continue;
        }
        for (int r = lane; r < K; r += 32) Ls[w][r] = Lx[static_cast<size_t>(c) * K + r];
        __syncwarp();
        const TreeInfo *info = info_all + cell_system(c_sys, c);
        const double s = level_scale(info, L), inv_s = 1.0 / s;
        const CellFrame<T> fr(c_ctr, c, info, inv_s);
        const T sc = static_cast<T>(inv_s * inv_s);
        const T *Lc = Ls[w];
        for (int j = c_begin[c] + lane; j < c_end[c]; j += 32) {
            T ux, uy, uz;
            fr.at(j, xs, n, ph, pl, ux, uy, uz);
            T gre = 0, gim = 0, gz = 0;
            for_each_regular<P - 1, T>(ux, uy, uz, [&](int nn, int q, T rr, T ri) {
                const int jj = nn + 1;
                // a_z: L~_{n+1}^q R_n^q
                {
                    const T lr = Lc[ridx(jj, q, 0)], li2 = q ? Lc[ridx(jj, q, 1)] : T(0);
                    const T wz = t.lz[jj][q] * (q ? T(2) : T(1));
                    gz += wz * (lr * rr - li2 * ri);
                }
                // a_x + i a_y, first sum: k = q - 1
                if (q >= 1) {
                    const int k = q - 1;
                    const T lr = Lc[ridx(jj, k, 0)], li2 = k ? Lc[ridx(jj, k, 1)] : T(0);
                    const T cf = t.lp[jj][k];
                    gre += cf * (lr * rr - li2 * ri);
                    gim += cf * (lr * ri + li2 * rr);
                }
                // second sum: k = q + 1, - conj(L) conj(R)
                {
                    const int k = q + 1;
                    const T lr = Lc[ridx(jj, k, 0)], li2 = Lc[ridx(jj, k, 1)];
                    const T cf = t.lm[jj][k];
                    gre -= cf * (lr * rr - li2 * ri);
                    gim += cf * (lr * ri + li2 * rr);
                }
            });
            far[j] = gre * sc;
            far[n + j] = gim * sc;
            far[2 * static_cast<size_t>(n) + j] = gz * sc;
        }
        __syncwarp();
    }
}

// acc[perm[j]] = near[j] + far[j], added in T (FP32 forms: one rounding of
// 2^-24 of the sum, below the error of either part, and no FP64 add). acc is
// [N][3] (AoS): a particle's three components share one scattered 24-byte
// write instead of three 8-byte ones.
template <typename T>
__global__ void k_finalize(const unsigned *__restrict__ perm, unsigned n, const T *__restrict__ nearv,
                           const T *__restrict__ farv, double *__restrict__ acc) {
    const unsigned j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n) return;
    const size_t i = perm[j];
#pragma unroll
    for (int a = 0; a < 3; ++a)
        acc[3 * i + a] = static_cast<double>(nearv[static_cast<size_t>(a) * n + j] + farv[static_cast<size_t>(a) * n + j]);
}

// Far-field potential (diagnostic, after an evaluation): the potential of
// the local expansion at each particle of a leaf at level >= 2,
// Phi = (1/s) sum_j [L~_j^0 R_j^0(u) + 2 Re sum_k L~_j^k R_j^k(u)], u = (x - c)/s,
// whose gradient is the far-field acceleration of k_l2p (no G, as there).
template <int P, typename T>
__global__ void __launch_bounds__(128) k_l2p_phi(const int *__restrict__ leaves, const unsigned *counts,
                                                 const int *__restrict__ c_begin, const int *__restrict__ c_end,
                                                 const int *__restrict__ c_level, const double *__restrict__ c_ctr,
                                                 const double *__restrict__ xs, unsigned n, const TreeInfo *__restrict__ info_all,
                                                 const int *__restrict__ c_sys, const T *__restrict__ Lx, double *__restrict__ farphi) {
    constexpr int K = (P + 1) * (P + 1);
    __shared__ T Ls[4][K];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const unsigned NL = counts[3];
    const unsigned warps = gridDim.x * (blockDim.x >> 5);
    for (unsigned li = blockIdx.x * (blockDim.x >> 5) + w; li < NL; li += warps) {
        const int c = leaves[li];
        const int L = c_level[c];
        if (L < 2) continue;  // warp-uniform
        for (int r = lane; r < K; r += 32) Ls[w][r] = Lx[static_cast<size_t>(c) * K + r];
        __syncwarp();
        const TreeInfo *info = info_all + cell_system(c_sys, c);
        const double s = level_scale(info, L), inv_s = 1.0 / s;
        const double cx = c_ctr[3 * c], cy = c_ctr[3 * c + 1], cz = c_ctr[3 * c + 2];
        const T *Lc = Ls[w];
        for (int j = c_begin[c] + lane; j < c_end[c]; j += 32) {
            const T ux = static_cast<T>((xs[j] - cx) * inv_s);
            const T uy = static_cast<T>((xs[n + j] - cy) * inv_s);
            const T uz = static_cast<T>((xs[2 * static_cast<size_t>(n) + j] - cz) * inv_s);
            T phi = 0;
            for_each_regular<P, T>(ux, uy, uz, [&](int nn, int q, T rr, T ri) {
                const T lr = Lc[ridx(nn, q, 0)], li2 = q ? Lc[ridx(nn, q, 1)] : T(0);
                phi += (q ? T(2) : T(1)) * (lr * rr - li2 * ri);
            });
            farphi[j] = static_cast<double>(phi) * inv_s;
        }
        __syncwarp();
    }
}

template <int P, typename T>
void launch_l2p_phi(Workspace &ws, double *farphi) {
    const unsigned gs = capped_grid(static_cast<unsigned>(ws.num_sms) * 8, ceil_div(ws.c_cap, 4));  // a warp per leaf
    k_l2p_phi<P, T><<<gs, 128, 0, ws.st>>>(ws.leaves, ws.d_counts, ws.c_begin, ws.c_end, ws.c_level, ws.c_ctr, ws.xs, ws.n,
                                           ws.info, forest_cells(ws), static_cast<const T *>(ws.Lexp), farphi);
    ws.launches += 1;
}

template <int P, typename T>
void launch_p2m(Workspace &ws) {
    const unsigned gs = capped_grid(static_cast<unsigned>(ws.num_sms) * 8, ceil_div(ws.c_cap, 4));
    k_p2m<P, T><<<gs, 128, 0, ws.st>>>(ws.leaves, ws.d_counts, ws.c_begin, ws.c_end, ws.c_level, ws.c_ctr, ws.xs, ws.ph,
                                       ws.pl, ws.n, ws.info, forest_cells(ws), ws.m, static_cast<T *>(ws.Mexp));
}

template <int P, typename T>
void launch_l2p(Workspace &ws) {
    const unsigned gs = capped_grid(static_cast<unsigned>(ws.num_sms) * 8, ceil_div(ws.c_cap, 4));
    k_l2p<P, T><<<gs, 128, 0, ws.st>>>(ws.leaves, ws.d_counts, ws.c_begin, ws.c_end, ws.c_level, ws.c_ctr, ws.xs, ws.ph,
                                       ws.pl, ws.n, ws.info, forest_cells(ws), static_cast<const T *>(ws.Lexp),
                                       static_cast<T *>(ws.farf));
}

template <int P, typename T>
const T *ops_of(const Workspace &ws) {
    return static_cast<const T *>(sizeof(T) == 4 ? static_cast<const void *>(ws.ops_f) : static_cast<const void *>(ws.ops_d));
}

template <int P, typename T>
void launch_m2l(Workspace &ws) {
    const size_t smem = TileCfg<P, T>::smem;
    cudaFuncSetAttribute(k_m2l<P, T>, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
    const unsigned gs = capped_grid(static_cast<unsigned>(ws.num_sms) * 2,
                                    8 * (ceil_div(ceil_div(ws.c_cap, 8), kTile) + (ws.forest() ? ws.nsys : 0)));
    k_m2l<P, T><<<gs, 256, smem, ws.st>>>(ws.info, ws.m2l_src, ops_of<P, T>(ws), ws.forest() ? ws.otile : nullptr,
                                          ws.oct_list, static_cast<const T *>(ws.Mexp), static_cast<T *>(ws.Lexp));
    ws.launches += 1;
}

template <int P, typename T>
void launch_m2m_levels(Workspace &ws) {
    const size_t smem = TileCfg<P, T>::smem;
    cudaFuncSetAttribute(k_m2m<P, T>, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
    const unsigned gs = 8 * capped_grid(static_cast<unsigned>(ws.num_sms) / 8 * 2, ceil_div(ws.s_cap, kTile));  // clusters of 8 CTAs
    // no cell is deeper than the key levels the sort ordered (tree.cu), so
    // parents lie at levels < ws.sort_levels
    for (int L = ws.sort_levels - 1; L >= 2; --L) {
        k_m2m<P, T><<<gs, 256, smem, ws.st>>>(L, ws.info, ws.split_cell, ws.c_child, ops_of<P, T>(ws),
                                              ws.forest() ? ws.etile : nullptr, ws.c_sys, static_cast<T *>(ws.Mexp));
        ws.launches += 1;
    }
}

template <int P, typename T>
void launch_l2l_levels(Workspace &ws) {
    const size_t smem = TileCfg<P, T>::smem;
    cudaFuncSetAttribute(k_l2l<P, T>, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
    const unsigned gs = capped_grid(static_cast<unsigned>(ws.num_sms) * 2, 8 * ceil_div(ws.s_cap, kTile));
    for (int Lp = 2; Lp <= ws.sort_levels - 1; ++Lp) {
        k_l2l<P, T><<<gs, 256, smem, ws.st>>>(Lp, ws.info, ws.split_cell, ws.c_child, ops_of<P, T>(ws),
                                              ws.forest() ? ws.etile : nullptr, ws.c_sys, static_cast<T *>(ws.Lexp));
        ws.launches += 1;
    }
}

template <typename T>
void dispatch_p(Workspace &ws, int which, double *farphi = nullptr) {
    switch (ws.p) {
#define GB_CASE(PP)                      \
    case PP:                             \
        if (which == 5) launch_l2p_phi<PP, T>(ws, farphi); \
        if (which == 0) launch_p2m<PP, T>(ws); \
        if (which == 1) launch_m2l<PP, T>(ws); \
        if (which == 2) launch_l2p<PP, T>(ws); \
        if (which == 3) launch_m2m_levels<PP, T>(ws); \
        if (which == 4) launch_l2l_levels<PP, T>(ws); \
        break;
        GB_CASE(1)
        GB_CASE(2)
        GB_CASE(3)
        GB_CASE(4)
        GB_CASE(5)
        GB_CASE(6)
        GB_CASE(7)
        GB_CASE(8)
        GB_CASE(9)
        GB_CASE(10)
#undef GB_CASE
        default:
            break;
    }
}

}  // namespace

size_t m2l_table_bytes(int p) {  // M2L, M2M and L2L tables
    const size_t K = static_cast<size_t>(p + 1) * (p + 1);
    return 3 * sizeof(M2LEnt) * K * K;
}

void build_m2l_table(Workspace &ws) {
    k_m2l_table<<<64, 256, 0, ws.st>>>(ws.p, static_cast<M2LEnt *>(ws.m2l_tab));
    ws.launches += 1;
}

void build_operators(Workspace &ws) {
    timer_begin(ws, kTOps);
    const size_t ny = static_cast<size_t>(2 * ws.p + 1) * (2 * ws.p + 1);  // yt, pw, Z, Zf
    const size_t smem = sizeof(double) * (2 * ny + 2 * ws.p + 3) + sizeof(float) * ny;
    const int nsys = ws.forest() ? ws.nsys : 1;
    if (ws.mixed) {
        // M2L offsets: FP32 operators, kSysPerBlock systems per block; then M2M and L2L
        // few systems: a thread per order (latency); many: a thread per operator (FP64 work)
        const int cols = nsys < 16 ? 2 * ws.p + 1 : 1;
        k_zf_tables<<<static_cast<unsigned>(ceil_div(static_cast<size_t>(nsys) * kNumOps * cols, 128)), 128, 0, ws.st>>>(
            ws.info, nsys, ws.p, cols, ws.zf);
        const size_t smem_f = kSysPerBlock * sizeof(float) * ny;
        k_build_ops_f<<<dim3(kNumOps, (nsys + kSysPerBlock - 1) / kSysPerBlock), 32 * kSysPerBlock, smem_f, ws.st>>>(
            nsys, ws.p, static_cast<const M2LEnt *>(ws.m2l_tab), ws.zf, ws.ops_f);
        ws.launches += 1;
    } else {
        k_build_ops<<<dim3(kNumOps, nsys), 256, smem, ws.st>>>(ws.info, ws.p, static_cast<const M2LEnt *>(ws.m2l_tab), ws.ops_d,
                                                              ws.ops_f, false, 0);
    }
    ws.launches += 1;
    timer_end(ws, kTOps);
}

void upward_pass(Workspace &ws) {
    timer_begin(ws, kTUp);
    if (ws.mixed) {
        dispatch_p<float>(ws, 0);
        dispatch_p<float>(ws, 3);
    } else {
        dispatch_p<double>(ws, 0);
        dispatch_p<double>(ws, 3);
    }
    ws.launches += 1;
    timer_end(ws, kTUp);
}

void m2l_pass(Workspace &ws) {
    timer_begin(ws, kTM2L);
    if (ws.mixed)
        dispatch_p<float>(ws, 1);
    else
        dispatch_p<double>(ws, 1);
    timer_end(ws, kTM2L);
}

void downward_pass(Workspace &ws) {
    timer_begin(ws, kTDown);
    if (ws.mixed) {  // L2P writes every particle's far field (zero above level 2)
        dispatch_p<float>(ws, 4);
        dispatch_p<float>(ws, 2);
    } else {
        dispatch_p<double>(ws, 4);
        dispatch_p<double>(ws, 2);
    }
    ws.launches += 1;
    timer_end(ws, kTDown);
}

void far_potential(Workspace &ws, double *farphi) {
    cudaMemsetAsync(farphi, 0, sizeof(double) * ws.n, ws.st);  // particles of leaves above level 2
    if (ws.mixed)
        dispatch_p<float>(ws, 5, farphi);
    else
        dispatch_p<double>(ws, 5, farphi);
}

void finalize_accel(Workspace &ws, double *acc_orig) {
    const unsigned n = ws.n;
    if (ws.mixed)
        k_finalize<float><<<(n + 255) / 256, 256, 0, ws.st>>>(ws.perm, n, static_cast<const float *>(ws.nearf),
                                                            static_cast<const float *>(ws.farf), acc_orig);
    else
        k_finalize<double><<<(n + 255) / 256, 256, 0, ws.st>>>(ws.perm, n, static_cast<const double *>(ws.nearf),
                                                              static_cast<const double *>(ws.farf), acc_orig);
    ws.launches += 1;
}

}  // namespace gb
