// Solid harmonics and translation operators of the reference's expansion
// (gravity/include/fmm.hpp), written for a real coefficient basis and for
// per-cell length scaling. Host+device: the same functions build the device
// operators and run in the CPU self-check of the operator algebra.
//
// Normalisation (fmm.hpp:169-194): Y_n^m = sqrt((n-|m|)!/(n+|m|)!) P_n^{|m|}(cos t) e^{i m phi}
// with the Condon-Shortley phase inside P, so Y_n^{-m} = conj(Y_n^m).
// Regular solid harmonics R_n^m(u) = |u|^n Y_n^m(u/|u|) follow the
// three-term recurrences
//   R_0^0 = 1,  R_m^m = -sqrt((2m-1)/(2m)) (x + i y) R_{m-1}^{m-1},
//   R_{m+1}^m = sqrt(2m+1) z R_m^m,
//   R_n^m = ((2n-1) z R_{n-1}^m - sqrt((n+m-1)(n-m-1)) |u|^2 R_{n-2}^m) / sqrt((n+m)(n-m)),
// which avoid the angles (and the reference's r = 0 / sin t = 0 divisions in
// L2P, fmm.hpp:370-372). Their derivatives are the ladder relations
//   d/dz R_n^m = sqrt((n-m)(n+m)) R_{n-1}^m,
//   (d/dx + i d/dy) R_n^m = sqrt((n-m)(n-m-1)) R_{n-1}^{m+1},
//   (d/dx - i d/dy) R_n^m = -sqrt((n+m)(n+m-1)) R_{n-1}^{m-1}   (m >= 1).
//
// Scaled expansions: for a cell of level L with length unit s_L = S 2^-L
// (S = largest root-box extent) the library stores
//   M~_n^m = M_n^m / s^n,   L~_j^k = L_j^k s^{j+1},
// which makes every translation operator independent of the level, so one
// set of matrices (M2L per same-level offset, M2M/L2L per octant) serves the
// whole tree. Real basis: for every degree n, Re(n,0), then Re(n,m), Im(n,m)
// for m = 1..n (ridx in common.cuh); negative orders are conjugates.
#pragma once

#include <cmath>

#include "common.cuh"

namespace gb {

constexpr int kTabN = 2 * kMaxP + 1;  // degrees 0..20

template <typename T>
struct HTab {
    T mm[kTabN];           // -sqrt((2m-1)/(2m))
    T m1[kTabN];           // sqrt(2m+1)
    T ra[kTabN][kTabN];    // (2n-1)/sqrt((n+m)(n-m))
    T rb[kTabN][kTabN];    // sqrt((n+m-1)(n-m-1))/sqrt((n+m)(n-m))
    T lz[kTabN][kTabN];    // sqrt((n-m)(n+m))
    T lp[kTabN][kTabN];    // sqrt((n-m)(n-m-1))
    T lm[kTabN][kTabN];    // sqrt((n+m)(n+m-1))
};

// A_n^m = (-1)^n / sqrt((n-m)! (n+m)!)  (fmm.hpp:201-221), m = |m|.
struct ATab {
    double a[kTabN][kTabN];
    double ainv[kTabN][kTabN];  // 1 / a (0 where a is 0): operator entries multiply instead of
                                // divide, FP64 division being costly on this GPU
};

inline void fill_tables(HTab<double> &t, ATab &at) {
    for (int m = 0; m < kTabN; ++m) {
        t.mm[m] = m == 0 ? 0.0 : -std::sqrt((2.0 * m - 1.0) / (2.0 * m));
        t.m1[m] = std::sqrt(2.0 * m + 1.0);
    }
    for (int n = 0; n < kTabN; ++n)
        for (int m = 0; m < kTabN; ++m) {
            const double np = n + m, nm = n - m;
            t.ra[n][m] = (m <= n - 2) ? (2.0 * n - 1.0) / std::sqrt(np * nm) : 0.0;
            t.rb[n][m] = (m <= n - 2) ? std::sqrt((np - 1.0) * (nm - 1.0)) / std::sqrt(np * nm) : 0.0;
            t.lz[n][m] = (m <= n) ? std::sqrt(nm * np) : 0.0;
            t.lp[n][m] = (m <= n) ? std::sqrt(nm * (nm - 1.0 > 0 ? nm - 1.0 : 0.0)) : 0.0;
            t.lm[n][m] = (m <= n) ? std::sqrt(np * (np - 1.0 > 0 ? np - 1.0 : 0.0)) : 0.0;
            double f1 = 1, f2 = 1;
            if (m <= n) {
                for (int i = 2; i <= n - m; ++i) f1 *= i;
                for (int i = 2; i <= n + m; ++i) f2 *= i;
                at.a[n][m] = (n % 2 ? -1.0 : 1.0) / std::sqrt(f1 * f2);
                at.ainv[n][m] = 1.0 / at.a[n][m];
            } else {
                at.a[n][m] = 0.0;
                at.ainv[n][m] = 0.0;
            }
        }
}

template <typename T, typename U>
inline void convert_tables(const HTab<U> &s, HTab<T> &d) {
    for (int i = 0; i < kTabN; ++i) d.mm[i] = static_cast<T>(s.mm[i]), d.m1[i] = static_cast<T>(s.m1[i]);
    for (int i = 0; i < kTabN; ++i)
        for (int j = 0; j < kTabN; ++j) {
            d.ra[i][j] = static_cast<T>(s.ra[i][j]);
            d.rb[i][j] = static_cast<T>(s.rb[i][j]);
            d.lz[i][j] = static_cast<T>(s.lz[i][j]);
            d.lp[i][j] = static_cast<T>(s.lp[i][j]);
            d.lm[i][j] = static_cast<T>(s.lm[i][j]);
        }
}

// Regular solid harmonics R_n^m(x,y,z), n <= D, m >= 0, real basis (ridx).
template <int D, typename T>
GB_HD void solid_regular(T x, T y, T z, const HTab<T> &t, T *out) {
    const T r2 = x * x + y * y + z * z;
    T cre = 1, cim = 0;  // R_m^m
#pragma unroll
    for (int m = 0; m <= D; ++m) {
        if (m > 0) {
            const T nre = t.mm[m] * (x * cre - y * cim);
            const T nim = t.mm[m] * (x * cim + y * cre);
            cre = nre, cim = nim;
        }
        out[ridx(m, m, 0)] = cre;
        if (m > 0) out[ridx(m, m, 1)] = cim;
        if (m + 1 <= D) {
            out[ridx(m + 1, m, 0)] = t.m1[m] * z * cre;
            if (m > 0) out[ridx(m + 1, m, 1)] = t.m1[m] * z * cim;
        }
#pragma unroll
        for (int n = m + 2; n <= D; ++n) {
            out[ridx(n, m, 0)] = t.ra[n][m] * z * out[ridx(n - 1, m, 0)] - t.rb[n][m] * r2 * out[ridx(n - 2, m, 0)];
            if (m > 0) out[ridx(n, m, 1)] = t.ra[n][m] * z * out[ridx(n - 1, m, 1)] - t.rb[n][m] * r2 * out[ridx(n - 2, m, 1)];
        }
    }
}

// Same with a runtime degree (operator construction, host checks).
template <typename T>
GB_HD void solid_regular_rt(int D, T x, T y, T z, const HTab<T> &t, T *out) {
    const T r2 = x * x + y * y + z * z;
    T cre = 1, cim = 0;
    for (int m = 0; m <= D; ++m) {
        if (m > 0) {
            const T nre = t.mm[m] * (x * cre - y * cim);
            const T nim = t.mm[m] * (x * cim + y * cre);
            cre = nre, cim = nim;
        }
        out[ridx(m, m, 0)] = cre;
        if (m > 0) out[ridx(m, m, 1)] = cim;
        if (m + 1 <= D) {
            out[ridx(m + 1, m, 0)] = t.m1[m] * z * cre;
            if (m > 0) out[ridx(m + 1, m, 1)] = t.m1[m] * z * cim;
        }
        for (int n = m + 2; n <= D; ++n) {
            out[ridx(n, m, 0)] = t.ra[n][m] * z * out[ridx(n - 1, m, 0)] - t.rb[n][m] * r2 * out[ridx(n - 2, m, 0)];
            if (m > 0) out[ridx(n, m, 1)] = t.ra[n][m] * z * out[ridx(n - 1, m, 1)] - t.rb[n][m] * r2 * out[ridx(n - 2, m, 1)];
        }
    }
}

// Y_n^m of a direction from a real-basis table of unit-vector solid harmonics,
// any sign of m (negative orders are conjugates).
GB_HD void ydir(const double *yt, int n, int m, double &re, double &im) {
    const int am = m < 0 ? -m : m;
    re = yt[ridx(n, am, 0)];
    im = am == 0 ? 0.0 : yt[ridx(n, am, 1)];
    if (m < 0) im = -im;
}

GB_HD double aco(const ATab &at, int n, int m) { return at.a[n][m < 0 ? -m : m]; }
GB_HD double aco_inv(const ATab &at, int n, int m) { return at.ainv[n][m < 0 ? -m : m]; }
GB_HD double phase_even(int e) { return ((e / 2) % 2 == 0) ? 1.0 : -1.0; }  // i^e, e even
GB_HD int iabs(int v) { return v < 0 ? -v : v; }

// Complex coefficient of M~_n^m (source) in L~_j^k (target) for the scaled
// same-level M2L (fmm.hpp:277-304), shift t = source centre - target centre
// in units of the level's s, rho = |t|, yt = Y(t/|t|) up to degree 2p.
GB_HD void m2l_coef(const ATab &at, const double *yt, const double *rinv_pow, int j, int k, int n, int m, double &re,
                    double &im) {
    double yr, yi;
    ydir(yt, j + n, m - k, yr, yi);
    const double c = phase_even(iabs(k - m) - iabs(k) - iabs(m)) * aco(at, n, m) * aco(at, j, k) *
                     ((n % 2 ? -1.0 : 1.0) * aco_inv(at, j + n, m - k)) * rinv_pow[j + n + 1];
    re = c * yr;
    im = c * yi;
}

// Coefficient of M~'_{n'}^{m'} (child) in M~_j^k (parent) for the scaled M2M
// (fmm.hpp:247-274); t = child centre - parent centre in units of the
// parent's s, rpow[i] = |t|^i.
GB_HD bool m2m_coef(const ATab &at, const double *yt, const double *rpow, int j, int k, int np, int mp, double &re,
                    double &im) {
    const int n = j - np, m = k - mp;
    if (n < 0 || iabs(m) > n) {
        re = im = 0;
        return false;
    }
    double yr, yi;
    ydir(yt, n, -m, yr, yi);
    const double c = phase_even(iabs(k) - iabs(m) - iabs(mp)) * aco(at, n, m) * aco(at, np, mp) * rpow[n] *
                     aco_inv(at, j, k) * ldexp(1.0, -np);
    re = c * yr;
    im = c * yi;
    return true;
}

// Coefficient of L~_n^m (parent) in L~_j^k (child) for the scaled L2L
// (fmm.hpp:307-329); t = parent centre - child centre in units of the
// parent's s, rpow[i] = |t|^i.
GB_HD bool l2l_coef(const ATab &at, const double *yt, const double *rpow, int j, int k, int n, int m, double &re,
                    double &im) {
    if (n < j || iabs(m - k) > n - j) {
        re = im = 0;
        return false;
    }
    double yr, yi;
    ydir(yt, n - j, m - k, yr, yi);
    const double c = phase_even(iabs(m) - iabs(m - k) - iabs(k)) * aco(at, n - j, m - k) * aco(at, j, k) * rpow[n - j] *
                     (((n + j) % 2 ? -1.0 : 1.0) * aco_inv(at, n, m)) * ldexp(1.0, -(j + 1));
    re = c * yr;
    im = c * yi;
    return true;
}

// One entry of a real-basis operator matrix: row (j,k,part_out), column
// (n,m,part_in). kind 0: M2L, 1: M2M, 2: L2L.
GB_HD double real_entry(int kind, const ATab &at, const double *yt, const double *pw, int j, int k, int po, int n, int m,
                        int pi) {
    double ar = 0, ai = 0, br = 0, bi = 0;
    auto coef = [&](int mm, double &re, double &im) {
        if (kind == 0)
            m2l_coef(at, yt, pw, j, k, n, mm, re, im);
        else if (kind == 1)
            m2m_coef(at, yt, pw, j, k, n, mm, re, im);
        else
            l2l_coef(at, yt, pw, j, k, n, mm, re, im);
    };
    coef(m, ar, ai);
    if (m > 0) coef(-m, br, bi);
    double vr, vi;
    if (pi == 0) {  // input Re(n,m): M^m = 1, M^-m = 1
        vr = ar + br;
        vi = ai + bi;
    } else {        // input Im(n,m): M^m = i, M^-m = -i  ->  i (a - b)
        vr = -(ai - bi);
        vi = ar - br;
    }
    return po == 0 ? vr : vi;
}

// Decode a real-basis index into (n, m, part).
GB_HD void rdecode(int r, int &n, int &m, int &part) {
    n = 0;
    while ((n + 1) * (n + 1) <= r) ++n;
    const int q = r - n * n;
    if (q == 0) {
        m = 0, part = 0;
    } else {
        m = (q + 1) / 2;
        part = (q + 1) % 2;
    }
}

}  // namespace gb
