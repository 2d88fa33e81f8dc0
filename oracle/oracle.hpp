// ORACLE — test infrastructure, not product code.
//
// A CPU restatement (C++17, OpenMP) of the reference's gravity FMM path
// (satoshigeyuki/vipp-nbody-bench, gravity/include/*.hpp). It is the checker
// for the CUDA path and the timed CPU baseline ("port") beside it. Only
// tests/, __graft_entry__.smoke() and bench.py's CPU-baseline / reference
// legs may load it. The product library never links or calls it.
//
// Parity pin: every function here is checked against the reference's own
// golden values (gravity/test/*.cpp known-answer tests) and against outputs of
// the reference headers compiled unmodified (oracle/_ref, fixtures under
// tests/golden/).
//
// Each function names the reference lines whose behaviour it restates. The
// arithmetic follows the same formulas in the same association order where the
// result is summed (P2P, RK4), so results agree to rounding.
#pragma once

#include <algorithm>
#include <cmath>
#include <complex>
#include <cstddef>
#include <cstdint>
#include <limits>
#include <random>
#include <stdexcept>
#include <vector>

namespace vipp_oracle {

using cd = std::complex<double>;

struct V3 {
    double x, y, z;
};

inline V3 sub(const V3 &a, const V3 &b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline double norm2(const V3 &a) { return a.x * a.x + a.y * a.y + a.z * a.z; }

// Spherical coordinates of a vector; problem.hpp:113-119. theta is 0 when
// r == 0; phi is 0 on the z axis, sign taken from y.
inline void polar(const V3 &v, double &r, double &theta, double &phi) {
    r = std::sqrt(norm2(v));
    theta = std::fabs(r) < std::numeric_limits<double>::min() ? 0.0 : std::acos(v.z / r);
    const double rxy = std::sqrt(v.x * v.x + v.y * v.y);
    const double s = v.y < 0 ? -1.0 : 1.0;
    phi = s * (rxy < std::numeric_limits<double>::min() ? 0.0 : std::acos(v.x / rxy));
}

// n! as a double; fmm.hpp:9-16.
inline double fact(unsigned n) {
    double r = 1;
    for (unsigned i = 2; i <= n; ++i) r *= i;
    return r;
}

// Associated Legendre functions with the Condon-Shortley phase, from the
// explicit Rodrigues series (fmm.hpp:20-73):
//   P_n^m(x) = (-1)^m (1-x^2)^{m/2} 2^{-n}
//              * sum_{k=0}^{(n-m)/2} (-1)^k (2n-2k)! / (k! (n-k)! (n-2k-m)!) x^{n-2k-m}
struct Legendre {
    unsigned nmax;
    std::vector<double> v;  // [n*(nmax+1)+m]
    Legendre(unsigned nmax_, double x) : nmax(nmax_), v((nmax_ + 1) * (nmax_ + 1), 0.0) {
        const double w = std::sqrt(1 - x * x);
        double wm = 1;  // (1-x^2)^{m/2}
        for (unsigned m = 0; m <= nmax; ++m) {
            for (unsigned n = m; n <= nmax; ++n) {
                double acc = 0;
                for (unsigned k = 0; 2 * k <= n - m; ++k) {
                    const double c = fact(2 * n - 2 * k) / (fact(k) * fact(n - k) * fact(n - 2 * k - m));
                    acc += (k % 2 ? -c : c) * std::pow(x, static_cast<int>(n - 2 * k - m));
                }
                v[n * (nmax + 1) + m] = acc * wm / std::ldexp(1.0, static_cast<int>(n)) * (m % 2 ? -1.0 : 1.0);
            }
            wm *= w;
        }
    }
    double operator()(unsigned n, unsigned m) const { return v[n * (nmax + 1) + m]; }
};

// -sin(theta) dP_n^m/dx at x = cos(theta), i.e. dP_n^m(cos theta)/dtheta, by
// differentiating the same series (fmm.hpp:77-165):
//   -y d/dx [(-1)^m y^m Q(x) / 2^n] = -(-1)^m y^{m-1} 2^{-n} (-m x Q + y^2 Q'),  y = sin(theta)
struct LegendreDTheta {
    unsigned nmax;
    std::vector<double> v;
    LegendreDTheta(unsigned nmax_, double theta) : nmax(nmax_), v((nmax_ + 1) * (nmax_ + 1), 0.0) {
        const double x = std::cos(theta), y = std::sin(theta);
        for (unsigned n = 0; n <= nmax; ++n) {  // m = 0: -y Q'(x) / 2^n
            double acc = 0;
            for (unsigned k = 0; 2 * k <= n; ++k) {
                const unsigned e = n - 2 * k;
                if (e == 0) continue;
                const double c = fact(2 * n - 2 * k) / (fact(k) * fact(n - k) * fact(e));
                acc += (k % 2 ? -c : c) * e * std::pow(x, static_cast<int>(e - 1));
            }
            v[n * (nmax + 1)] = -y * acc / std::ldexp(1.0, static_cast<int>(n));
        }
        double ym1 = 1;  // y^{m-1}
        for (unsigned m = 1; m <= nmax; ++m) {
            for (unsigned n = m; n <= nmax; ++n) {
                double acc = 0;
                for (unsigned k = 0; 2 * k <= n - m; ++k) {
                    const unsigned e = n - 2 * k - m;
                    const double c = fact(2 * n - 2 * k) / (fact(k) * fact(n - k) * fact(e));
                    const double sc = k % 2 ? -c : c;
                    if (e == 0)
                        acc += sc * (-static_cast<double>(m) * x);
                    else
                        acc += sc * std::pow(x, static_cast<int>(e - 1)) * (-static_cast<double>(m) * x * x + y * y * e);
                }
                v[n * (nmax + 1) + m] = -(m % 2 ? -1.0 : 1.0) * ym1 * acc / std::ldexp(1.0, static_cast<int>(n));
            }
            ym1 *= y;
        }
    }
    double operator()(unsigned n, unsigned m) const { return v[n * (nmax + 1) + m]; }
};

// sqrt((n-|m|)! / (n+|m|)!)
inline double ynorm(unsigned n, unsigned am) {
    double c = 1;
    for (unsigned i = n - am + 1; i <= n + am; ++i) c /= i;
    return std::sqrt(c);
}

// Y_n^m(theta, phi) = sqrt((n-|m|)!/(n+|m|)!) P_n^{|m|}(cos theta) e^{i m phi}
// (fmm.hpp:169-194); note Y_n^{-m} = conj(Y_n^m) in this convention.
struct SphHarm {
    Legendre P;
    double phi;
    SphHarm(unsigned nmax, double theta, double phi_) : P(nmax, std::cos(theta)), phi(phi_) {}
    cd operator()(unsigned n, int m) const {
        const unsigned am = static_cast<unsigned>(m < 0 ? -m : m);
        return ynorm(n, am) * P(n, am) * cd{std::cos(m * phi), std::sin(m * phi)};
    }
};

// A_n^m = (-1)^n / sqrt((n-m)! (n+m)!)  (fmm.hpp:201-221).
inline double Acoef(unsigned n, int m) {
    const unsigned am = static_cast<unsigned>(m < 0 ? -m : m);
    if (n < am) throw std::runtime_error("n must be >= |m|");
    double d = 1;
    for (unsigned i = n - am + 1; i <= n + am; ++i) d *= i;
    d = std::sqrt(d);
    for (unsigned i = 1; i <= n - am; ++i) d *= i;
    return n % 2 ? -1.0 / d : 1.0 / d;
}

// i^e for even e, which is all the translation formulas need: (-1)^{e/2}.
inline double ipow_even(int e) { return ((e / 2) % 2 == 0) ? 1.0 : -1.0; }

struct Cell {
    long long parent = -1;
    int level = 0;
    V3 mn{0, 0, 0}, mx{0, 0, 0};
    long long first_child = -1;  // -1: leaf
    std::vector<long long> pts;  // leaf members in insertion (ascending index) order
    std::vector<cd> M, L;        // (p+1) x (2p+1), empty until computed
    bool leaf() const { return first_child < 0; }
    V3 center() const { return {(mn.x + mx.x) / 2, (mn.y + mx.y) / 2, (mn.z + mx.z) / 2}; }
};

// Adaptive octree by serial insertion (octree.hpp:79-191). The root box is the
// bounding box padded by 1e-5 (fmm.hpp:403-405, problem.hpp:167). A leaf that
// already holds floor(sqrt(8) s) points splits when one more arrives; its
// eight children are appended contiguously, child offset bit0/1/2 = 0 meaning
// the upper x/y/z half; boxes are closed and the first child that contains a
// point takes it, so ties on a mid-plane go to the upper half.
struct Tree {
    std::vector<Cell> cells;
    const std::vector<V3> *x = nullptr;
    std::size_t threshold = 0;
    int max_level = 0;

    Tree(const std::vector<V3> &pts, std::size_t s) : x(&pts) {
        threshold = static_cast<std::size_t>(std::floor(std::sqrt(8.0) * static_cast<double>(s)));
        Cell root;
        if (!pts.empty()) {
            V3 lo{std::numeric_limits<double>::max(), std::numeric_limits<double>::max(), std::numeric_limits<double>::max()};
            V3 hi{std::numeric_limits<double>::lowest(), std::numeric_limits<double>::lowest(), std::numeric_limits<double>::lowest()};
            for (const auto &p : pts) {
                lo.x = std::min(lo.x, p.x), lo.y = std::min(lo.y, p.y), lo.z = std::min(lo.z, p.z);
                hi.x = std::max(hi.x, p.x), hi.y = std::max(hi.y, p.y), hi.z = std::max(hi.z, p.z);
            }
            const double pad = 1e-5;
            root.mn = {lo.x - pad, lo.y - pad, lo.z - pad};
            root.mx = {hi.x + pad, hi.y + pad, hi.z + pad};
        }
        cells.push_back(root);
        for (std::size_t i = 0; i < pts.size(); ++i)
            if (!insert(0, static_cast<long long>(i))) throw std::runtime_error("failed to insert point");
    }

    bool contains(const Cell &c, const V3 &p) const {
        return !(p.x < c.mn.x || c.mx.x < p.x || p.y < c.mn.y || c.mx.y < p.y || p.z < c.mn.z || c.mx.z < p.z);
    }

    bool insert(std::size_t ci, long long i) {
        const V3 &p = (*x)[static_cast<std::size_t>(i)];
        if (!contains(cells[ci], p)) return false;
        if (cells[ci].leaf()) {
            if (cells[ci].pts.size() < threshold) {
                cells[ci].pts.push_back(i);
                return true;
            }
            split(ci);
        }
        const long long base = cells[ci].first_child;
        for (long long c = base; c < base + 8; ++c)
            if (insert(static_cast<std::size_t>(c), i)) return true;
        return false;
    }

    void split(std::size_t ci) {
        const V3 lo = cells[ci].mn, hi = cells[ci].mx;
        const V3 mid{(hi.x + lo.x) / 2, (hi.y + lo.y) / 2, (hi.z + lo.z) / 2};
        const long long base = static_cast<long long>(cells.size());
        const int lvl = cells[ci].level + 1;
        max_level = std::max(max_level, lvl);
        for (unsigned o = 0; o < 8; ++o) {
            Cell c;
            c.parent = static_cast<long long>(ci);
            c.level = lvl;
            c.mn = {(o & 1) ? lo.x : mid.x, (o & 2) ? lo.y : mid.y, (o & 4) ? lo.z : mid.z};
            c.mx = {(o & 1) ? mid.x : hi.x, (o & 2) ? mid.y : hi.y, (o & 4) ? mid.z : hi.z};
            cells.push_back(std::move(c));
        }
        std::vector<long long> old;
        old.swap(cells[ci].pts);
        cells[ci].first_child = base;
        for (long long i : old) {
            bool ok = false;
            for (long long c = base; c < base + 8 && !ok; ++c) ok = insert(static_cast<std::size_t>(c), i);
            if (!ok) throw std::runtime_error("failed to insert point");
        }
    }

    // Octant of a cell inside its parent, one bit per axis, 1 = lower half
    // (fmm.hpp:464-471).
    unsigned octant(std::size_t ci) const {
        return static_cast<unsigned>(ci - static_cast<std::size_t>(cells[static_cast<std::size_t>(cells[ci].parent)].first_child));
    }

    // Same-level adjacency (fmm.hpp:475-493): integer coordinates built from
    // the octant bits up to the common ancestor; adjacent or equal iff every
    // coordinate differs by at most one.
    bool adjacent_or_equal(std::size_t a, std::size_t b) const {
        if (cells[a].parent == cells[b].parent) return true;
        long long ia[3], ib[3];
        unsigned oa = octant(a), ob = octant(b);
        for (int d = 0; d < 3; ++d) ia[d] = (oa >> d) & 1, ib[d] = (ob >> d) & 1;
        std::size_t pa = static_cast<std::size_t>(cells[a].parent), pb = static_cast<std::size_t>(cells[b].parent);
        for (int lv = 1;; ++lv) {
            oa = octant(pa), ob = octant(pb);
            for (int d = 0; d < 3; ++d) ia[d] += static_cast<long long>((oa >> d) & 1) << lv, ib[d] += static_cast<long long>((ob >> d) & 1) << lv;
            if (cells[pa].parent == cells[pb].parent) {
                long long s = 0;
                for (int d = 0; d < 3; ++d) s += (ia[d] - ib[d]) * (ia[d] - ib[d]);
                return s <= 3;
            }
            pa = static_cast<std::size_t>(cells[pa].parent), pb = static_cast<std::size_t>(cells[pb].parent);
        }
    }
};

// Interaction lists, top-down (solver_ref.hpp:115-162). For every cell:
//   p2p  = parent's p2p list, then each adjacent cousin where either side is a leaf
//   coll = adjacent cousins when both sides are non-leaves (the cell itself included)
//   m2l  = cousins that are not adjacent
// where cousins are the children of the parent's coll list, in list order and
// child order. The root puts itself in its p2p list (leaf) or coll list.
struct Lists {
    std::vector<std::vector<long long>> m2l, p2p, coll;
    explicit Lists(const Tree &t) : m2l(t.cells.size()), p2p(t.cells.size()), coll(t.cells.size()) {
        build(t, 0);
    }
    void build(const Tree &t, std::size_t ci) {
        const Cell &c = t.cells[ci];
        if (c.parent < 0) {
            (c.leaf() ? p2p[ci] : coll[ci]).push_back(static_cast<long long>(ci));
        } else {
            const std::size_t pi = static_cast<std::size_t>(c.parent);
            p2p[ci] = p2p[pi];
            for (long long q : coll[pi]) {
                const long long base = t.cells[static_cast<std::size_t>(q)].first_child;
                for (long long u = base; u < base + 8; ++u) {
                    const std::size_t ui = static_cast<std::size_t>(u);
                    if (t.adjacent_or_equal(ci, ui)) {
                        if (!c.leaf() && !t.cells[ui].leaf())
                            coll[ci].push_back(u);
                        else
                            p2p[ci].push_back(u);
                    } else {
                        m2l[ci].push_back(u);
                    }
                }
            }
        }
        if (!c.leaf())
            for (long long u = c.first_child; u < c.first_child + 8; ++u) build(t, static_cast<std::size_t>(u));
    }
};

inline std::size_t eidx(unsigned p, unsigned n, int m) { return n * (2 * p + 1) + static_cast<std::size_t>(m + static_cast<int>(p)); }

// P2M (fmm.hpp:224-244): M_k^m = sum_i q rho_i^k Y_k^{-m}(alpha_i, beta_i), k <= p;
// negative orders are the conjugates.
inline void p2m(Cell &c, unsigned p, const std::vector<V3> &x, double q) {
    c.M.assign((p + 1) * (2 * p + 1), cd{0, 0});
    const V3 ctr = c.center();
    for (long long i : c.pts) {
        double r, th, ph;
        polar(sub(x[static_cast<std::size_t>(i)], ctr), r, th, ph);
        const SphHarm Y(p, th, ph);
        double rk = 1;
        for (unsigned k = 0; k <= p; ++k) {
            for (unsigned m = 0; m <= k; ++m) c.M[eidx(p, k, static_cast<int>(m))] += (q * rk) * Y(k, -static_cast<int>(m));
            rk *= r;
        }
    }
    for (unsigned k = 1; k <= p; ++k)
        for (unsigned m = 1; m <= k; ++m) c.M[eidx(p, k, -static_cast<int>(m))] = std::conj(c.M[eidx(p, k, static_cast<int>(m))]);
}

// M2M (fmm.hpp:247-274): shift each child's multipole to the parent centre.
//   M_j^k += O_{j-n}^{k-m} i^{|k|-|m|-|k-m|} A_n^m A_{j-n}^{k-m} rho^n Y_n^{-m} / A_j^k
inline void m2m(Tree &t, std::size_t ci, unsigned p) {
    Cell &c = t.cells[ci];
    c.M.assign((p + 1) * (2 * p + 1), cd{0, 0});
    const V3 ctr = c.center();
    for (long long u = c.first_child; u < c.first_child + 8; ++u) {
        const Cell &ch = t.cells[static_cast<std::size_t>(u)];
        double r, th, ph;
        polar(sub(ch.center(), ctr), r, th, ph);
        const SphHarm Y(p, th, ph);
        for (unsigned j = 0; j <= p; ++j)
            for (int k = -static_cast<int>(j); k <= static_cast<int>(j); ++k) {
                const double ajk = Acoef(j, k);
                double rn = 1;
                for (unsigned n = 0; n <= j; ++n) {
                    const int lo = std::max(-static_cast<int>(n), static_cast<int>(n) + k - static_cast<int>(j));
                    const int hi = std::min(static_cast<int>(j) + k - static_cast<int>(n), static_cast<int>(n));
                    for (int m = lo; m <= hi; ++m) {
                        const cd O = ch.M[eidx(p, j - n, k - m)];
                        const double ph_ = ipow_even(std::abs(k) - std::abs(m) - std::abs(k - m));
                        c.M[eidx(p, j, k)] += (O * ph_ * Acoef(n, m) * Acoef(j - n, k - m) * rn * Y(n, -m)) / ajk;
                    }
                    rn *= r;
                }
            }
    }
}

// M2L (fmm.hpp:277-304): for every cell in the list, with (rho, alpha, beta)
// the source centre minus the target centre,
//   L_j^k += M_n^m i^{|k-m|-|k|-|m|} A_n^m A_j^k Y_{j+n}^{m-k} / ((-1)^n A_{j+n}^{m-k} rho^{j+n+1})
inline void m2l(Tree &t, std::size_t ci, unsigned p, const std::vector<long long> &srcs) {
    Cell &c = t.cells[ci];
    c.L.assign((p + 1) * (2 * p + 1), cd{0, 0});
    const V3 ctr = c.center();
    for (long long s : srcs) {
        const Cell &sc = t.cells[static_cast<std::size_t>(s)];
        double r, th, ph;
        polar(sub(sc.center(), ctr), r, th, ph);
        const SphHarm Y(2 * p, th, ph);
        double rj1 = r;
        for (unsigned j = 0; j <= p; ++j) {
            for (int k = -static_cast<int>(j); k <= static_cast<int>(j); ++k) {
                const double ajk = Acoef(j, k);
                double rn = 1;
                cd acc = c.L[eidx(p, j, k)];
                for (unsigned n = 0; n <= p; ++n) {
                    for (int m = -static_cast<int>(n); m <= static_cast<int>(n); ++m) {
                        const double ph_ = ipow_even(std::abs(k - m) - std::abs(k) - std::abs(m));
                        acc += (sc.M[eidx(p, n, m)] * ph_ * Acoef(n, m) * ajk * Y(j + n, m - k)) /
                               ((n % 2 ? -1.0 : 1.0) * Acoef(j + n, m - k) * rj1 * rn);
                    }
                    rn *= r;
                }
                c.L[eidx(p, j, k)] = acc;
            }
            rj1 *= r;
        }
    }
}

// L2L (fmm.hpp:307-329), with (rho, alpha, beta) the parent centre minus the child centre:
//   L_j^k += L_n^m i^{|m|-|m-k|-|k|} A_{n-j}^{m-k} A_j^k Y_{n-j}^{m-k} rho^{n-j} / ((-1)^{n+j} A_n^m)
inline void l2l(Tree &t, std::size_t ci, unsigned p) {
    Cell &c = t.cells[ci];
    const Cell &par = t.cells[static_cast<std::size_t>(c.parent)];
    double r, th, ph;
    polar(sub(par.center(), c.center()), r, th, ph);
    const SphHarm Y(p, th, ph);
    for (unsigned j = 0; j <= p; ++j)
        for (int k = -static_cast<int>(j); k <= static_cast<int>(j); ++k) {
            const double ajk = Acoef(j, k);
            double rnj = 1;
            for (unsigned n = j; n <= p; ++n) {
                const int lo = std::max(-static_cast<int>(n), k - static_cast<int>(n - j));
                const int hi = std::min(static_cast<int>(n), static_cast<int>(n - j) + k);
                for (int m = lo; m <= hi; ++m) {
                    const double ph_ = ipow_even(std::abs(m) - std::abs(m - k) - std::abs(k));
                    c.L[eidx(p, j, k)] += (par.L[eidx(p, n, m)] * ph_ * Acoef(n - j, m - k) * ajk * Y(n - j, m - k) * rnj) /
                                          (((n + j) % 2 ? -1.0 : 1.0) * Acoef(n, m));
                }
                rnj *= r;
            }
        }
}

// L2P (fmm.hpp:332-374): gradient of sum L_l^m r^l Y_l^m in spherical
// components, converted to Cartesian and added to a[i]. No G factor (the
// reference's); the accurate mode passes g = G.
inline void l2p(const Cell &c, unsigned p, const std::vector<V3> &x, std::vector<V3> &a, double g = 1.0) {
    const V3 ctr = c.center();
    for (long long i : c.pts) {
        double r, th, ph;
        polar(sub(x[static_cast<std::size_t>(i)], ctr), r, th, ph);
        const SphHarm Y(p, th, ph);
        const LegendreDTheta dP(p, th);
        double rl = 1, dr = 0, dth = 0, dph = 0;
        for (unsigned l = 0; l <= p; ++l) {
            for (int m = -static_cast<int>(l); m <= static_cast<int>(l); ++m) {
                const cd Llm = c.L[eidx(p, l, m)];
                const cd ylm = Y(l, m);
                const unsigned am = static_cast<unsigned>(std::abs(m));
                const cd e{std::cos(m * ph), std::sin(m * ph)};
                dr += (Llm * rl * ylm * (l / r)).real();
                dth += (Llm * rl * ynorm(l, am) * dP(l, am) * e).real();
                dph += (Llm * rl * ylm * cd{0, static_cast<double>(m)}).real();
            }
            rl *= r;
        }
        const double ct = std::cos(th), st = std::sin(th), cp = std::cos(ph), sp = std::sin(ph);
        V3 &ai = a[static_cast<std::size_t>(i)];
        ai.x += g * (st * cp * dr + ct * cp / r * dth - sp / (r * st) * dph);
        ai.y += g * (st * sp * dr + ct * sp / r * dth + cp / (r * st) * dph);
        ai.z += g * (ct * dr - st / r * dth);
    }
}

// Softened pair term G m (xj - xi) / (|xj - xi|^2 + eps^2)^{3/2}
// (fmm.hpp:531-540, solver_ref_naive.hpp:361).
inline V3 pair_acc(const V3 &xi, const V3 &xj, double Gm, double eps) {
    const V3 d = sub(xj, xi);
    const double den = std::pow(norm2(d) + eps * eps, 1.5);
    return {Gm * d.x / den, Gm * d.y / den, Gm * d.z / den};
}

// Subtree sum of pair terms for target i, skipping i itself (fmm.hpp:513-528).
inline V3 subtree_acc(const Tree &t, std::size_t ci, std::size_t i, const std::vector<V3> &x, double Gm, double eps) {
    V3 acc{0, 0, 0};
    const Cell &c = t.cells[ci];
    if (c.leaf()) {
        for (long long j : c.pts) {
            if (static_cast<std::size_t>(j) == i) continue;
            const V3 d = pair_acc(x[i], x[static_cast<std::size_t>(j)], Gm, eps);
            acc.x += d.x, acc.y += d.y, acc.z += d.z;
        }
    } else {
        for (long long u = c.first_child; u < c.first_child + 8; ++u) {
            const V3 d = subtree_acc(t, static_cast<std::size_t>(u), i, x, Gm, eps);
            acc.x += d.x, acc.y += d.y, acc.z += d.z;
        }
    }
    return acc;
}

// P2P (fmm.hpp:377-385).
inline void p2p(const Tree &t, std::size_t ci, const std::vector<long long> &nb, const std::vector<V3> &x,
                std::vector<V3> &a, double Gm, double eps) {
    for (long long i : t.cells[ci].pts) {
        V3 &ai = a[static_cast<std::size_t>(i)];
        for (long long q : nb) {
            const V3 d = subtree_acc(t, static_cast<std::size_t>(q), static_cast<std::size_t>(i), x, Gm, eps);
            ai.x += d.x, ai.y += d.y, ai.z += d.z;
        }
    }
}

// ---------------------------------------------------------------------------
// Accurate mode (no counterpart in the reference). The reference's far field
// expands the unsoftened 1/r (M2L fmm.hpp:277-304, L2P fmm.hpp:332-374) while
// its near field is softened (fmm.hpp:531-540) and only the near field carries
// G, so against the softened direct sum its error stops near eps^2/r^2 whatever
// p is. The accurate mode multiplies the far field by G and adds the far field
// of the softening difference: for every leaf and every far source cell S of
// it (the M2L lists of the leaf and of its ancestors at level >= 2),
//   da(x) = G sum_{j in S} m_j F(|x_j - x|^2) (x_j - x),
//   F(u) = (u + eps^2)^{-3/2} - u^{-3/2},
// expanded about S's centre of mass z to second order in the source offsets
// (y_j = x_j - z, Q = sum_j m_j y_j y_j^T; the first order vanishes about z):
//   M F(u) d + [2 F''(u) (d.Qd) + F'(u) tr Q] d + 2 F'(u) Qd,   d = z - x, u = |d|^2.
// Evaluation (the approximations the GPU kernels make too):
//   * the lists of the leaf (k = 0) and of its parent (k = 1) at every
//     particle; in the leaf's own list, a source at offset o (cell units) with
//     exactly one |o_a| = 2 and the others <= 1 (the 54 nearest far cells,
//     where the expansion converges slowest) is taken as its 8 octants, each
//     with its own moments (children of a non-leaf source; the leaf's own
//     particles split at its mid-planes, ties to the upper half, otherwise);
//   * the lists of the ancestors at k >= 2 once at the leaf centre c: the
//     value above plus the first-order change J (x - c) of its monopole term,
//     J = -M (2 F'(u) d d^T + F(u) I).

struct CellMoments {
    double M = 0;          // mass
    V3 z{0, 0, 0};         // centre of mass
    double Q[6] = {};      // central second moments xx, yy, zz, xy, xz, yz
};

// Moments of a point set (equal masses).
inline CellMoments moments_of(const std::vector<V3> &x, const std::vector<long long> &pts, double mass) {
    CellMoments mo;
    if (pts.empty()) return mo;
    V3 s{0, 0, 0};
    for (long long j : pts) {
        const V3 &p = x[static_cast<std::size_t>(j)];
        s.x += p.x, s.y += p.y, s.z += p.z;
    }
    const double c = static_cast<double>(pts.size());
    mo.M = mass * c;
    mo.z = {s.x / c, s.y / c, s.z / c};
    for (long long j : pts) {
        const V3 y = sub(x[static_cast<std::size_t>(j)], mo.z);
        mo.Q[0] += mass * y.x * y.x, mo.Q[1] += mass * y.y * y.y, mo.Q[2] += mass * y.z * y.z;
        mo.Q[3] += mass * y.x * y.y, mo.Q[4] += mass * y.x * y.z, mo.Q[5] += mass * y.y * y.z;
    }
    return mo;
}

// Members of a cell's subtree (tree order within leaves).
inline void subtree_points(const Tree &t, std::size_t ci, std::vector<long long> &out) {
    const Cell &c = t.cells[ci];
    if (c.leaf()) {
        out.insert(out.end(), c.pts.begin(), c.pts.end());
        return;
    }
    for (long long u = c.first_child; u < c.first_child + 8; ++u) subtree_points(t, static_cast<std::size_t>(u), out);
}

// Whole-cell moments of every cell, and the 8 octant moments of every leaf
// (particles split at the leaf's mid-planes, coordinate < mid -> lower half,
// octant bit set; the tree's own tie rule).
struct SoftMoments {
    std::vector<CellMoments> cell;
    std::vector<CellMoments> leaf_oct;  // [8 * cell], filled for leaves
};

inline SoftMoments soft_moments(const Tree &t, const std::vector<V3> &x, double mass) {
    const std::size_t nc = t.cells.size();
    SoftMoments sm;
    sm.cell.resize(nc);
    sm.leaf_oct.resize(8 * nc);
#pragma omp parallel for schedule(dynamic, 8)
    for (std::size_t c = 0; c < nc; ++c) {
        std::vector<long long> pts;
        subtree_points(t, c, pts);
        sm.cell[c] = moments_of(x, pts, mass);
        if (t.cells[c].leaf()) {
            const V3 mid = t.cells[c].center();
            std::vector<long long> part[8];
            for (long long j : pts) {
                const V3 &p = x[static_cast<std::size_t>(j)];
                part[(p.x < mid.x ? 1 : 0) | (p.y < mid.y ? 2 : 0) | (p.z < mid.z ? 4 : 0)].push_back(j);
            }
            for (int o = 0; o < 8; ++o) sm.leaf_oct[8 * c + static_cast<std::size_t>(o)] = moments_of(x, part[o], mass);
        }
    }
    return sm;
}

// F, F', F'' of the softening difference at u = |d|^2 (e = eps^2), written
// without the cancellation of (u + e)^{-k/2} - u^{-k/2}: with w = sqrt(1 + e/u),
// (1 + e/u)^{-k/2} - 1 = -(w^k - 1) / w^k and w - 1 = (e/u) / (w + 1).
inline void soft_diff(double u, double e, double &F, double &F1, double &F2) {
    const double q = e / u, w = std::sqrt(1.0 + q), wm1 = q / (w + 1.0);
    const double w2 = w * w, w3 = w2 * w, w5 = w3 * w2, w7 = w5 * w2;
    const double s3 = wm1 * (w2 + w + 1.0);                                    // w^3 - 1
    const double s5 = wm1 * (w2 * w2 + w3 + w2 + w + 1.0);                     // w^5 - 1
    const double s7 = wm1 * (w5 * w + w5 + w2 * w2 + w3 + w2 + w + 1.0);       // w^7 - 1
    const double ru = 1.0 / std::sqrt(u), ru3 = ru * ru * ru, ru5 = ru3 * ru * ru, ru7 = ru5 * ru * ru;
    F = -ru3 * s3 / w3;
    F1 = 1.5 * ru5 * s5 / w5;
    F2 = -3.75 * ru7 * s7 / w7;
}

// Softening-difference field of S at xi (no G), to second order.
inline V3 soft_far_term(const CellMoments &S, const V3 &xi, double eps) {
    const V3 d = sub(S.z, xi);
    double F, F1, F2;
    soft_diff(norm2(d), eps * eps, F, F1, F2);
    const double *Q = S.Q;
    const V3 Qd{Q[0] * d.x + Q[3] * d.y + Q[4] * d.z, Q[3] * d.x + Q[1] * d.y + Q[5] * d.z,
                Q[4] * d.x + Q[5] * d.y + Q[2] * d.z};
    const double dQd = d.x * Qd.x + d.y * Qd.y + d.z * Qd.z, tr = Q[0] + Q[1] + Q[2];
    const double a = S.M * F + 2.0 * F2 * dQd + F1 * tr;
    return {a * d.x + 2.0 * F1 * Qd.x, a * d.y + 2.0 * F1 * Qd.y, a * d.z + 2.0 * F1 * Qd.z};
}

// Offset (cell units) of same-level cell b from cell a.
inline void level_offset(const Tree &t, std::size_t a, std::size_t b, int off[3]) {
    const V3 ca = t.cells[a].center(), cb = t.cells[b].center();
    const double h[3] = {t.cells[a].mx.x - t.cells[a].mn.x, t.cells[a].mx.y - t.cells[a].mn.y,
                         t.cells[a].mx.z - t.cells[a].mn.z};
    const double d[3] = {cb.x - ca.x, cb.y - ca.y, cb.z - ca.z};
    for (int k = 0; k < 3; ++k) off[k] = static_cast<int>(std::lround(d[k] / h[k]));
}

inline bool face_slab(const int off[3]) {
    int twos = 0, big = 0;
    for (int k = 0; k < 3; ++k) twos += std::abs(off[k]) == 2, big += std::abs(off[k]) > 2;
    return twos == 1 && big == 0;
}

// The softening correction of every particle of the leaves at level >= 2,
// times G, added to a.
inline void softening_correction(const Tree &t, const Lists &ls, const std::vector<V3> &x, double G, double mass,
                                 double eps, std::vector<V3> &a) {
    if (eps == 0) return;
    const SoftMoments sm = soft_moments(t, x, mass);
    const std::size_t nc = t.cells.size();
#pragma omp parallel for schedule(dynamic, 4)
    for (std::size_t leaf = 0; leaf < nc; ++leaf) {
        const Cell &L = t.cells[leaf];
        if (!L.leaf() || L.pts.empty() || L.level < 2) continue;
        const V3 c = L.center();
        V3 fc{0, 0, 0};
        double J[9] = {};
        std::vector<V3> corr(L.pts.size(), V3{0, 0, 0});
        auto at_particles = [&](const CellMoments &S) {
            if (S.M == 0) return;
            for (std::size_t q = 0; q < L.pts.size(); ++q) {
                const V3 f = soft_far_term(S, x[static_cast<std::size_t>(L.pts[q])], eps);
                corr[q].x += f.x, corr[q].y += f.y, corr[q].z += f.z;
            }
        };
        int k = 0;
        for (long long anc = static_cast<long long>(leaf); anc >= 0 && t.cells[static_cast<std::size_t>(anc)].level >= 2;
             anc = t.cells[static_cast<std::size_t>(anc)].parent, ++k) {
            const std::size_t au = static_cast<std::size_t>(anc);
            for (long long sidx : ls.m2l[au]) {
                const std::size_t su = static_cast<std::size_t>(sidx);
                const CellMoments &S = sm.cell[su];
                if (S.M == 0) continue;
                if (k == 0) {
                    int off[3];
                    level_offset(t, au, su, off);
                    if (face_slab(off)) {
                        for (int o = 0; o < 8; ++o)
                            at_particles(t.cells[su].leaf() ? sm.leaf_oct[8 * su + static_cast<std::size_t>(o)]
                                                            : sm.cell[static_cast<std::size_t>(t.cells[su].first_child + o)]);
                        continue;
                    }
                }
                if (k <= 1) {
                    at_particles(S);
                } else {
                    const V3 f = soft_far_term(S, c, eps);
                    fc.x += f.x, fc.y += f.y, fc.z += f.z;
                    const V3 d = sub(S.z, c);
                    double F, F1, F2;
                    soft_diff(norm2(d), eps * eps, F, F1, F2);
                    const double dd[3] = {d.x, d.y, d.z};
                    for (int r = 0; r < 3; ++r)
                        for (int q = 0; q < 3; ++q) J[3 * r + q] -= S.M * (2.0 * F1 * dd[r] * dd[q] + (r == q ? F : 0.0));
                }
            }
        }
        for (std::size_t q = 0; q < L.pts.size(); ++q) {
            const std::size_t i = static_cast<std::size_t>(L.pts[q]);
            const V3 y = sub(x[i], c);
            a[i].x += G * (corr[q].x + fc.x + J[0] * y.x + J[1] * y.y + J[2] * y.z);
            a[i].y += G * (corr[q].y + fc.y + J[3] * y.x + J[4] * y.y + J[5] * y.z);
            a[i].z += G * (corr[q].z + fc.z + J[6] * y.x + J[7] * y.y + J[8] * y.z);
        }
    }
}

// One force evaluation (solver_ref.hpp:164-232): zero, tree, lists, then
// P2M (leaves, level >= 2) / M2M (level >= 2) upward; M2L (index > 8, i.e.
// level >= 2) and P2P (leaves); L2L (level >= 3) / L2P (leaves, level >= 2)
// downward. Level-ordered loops replace the reference's recursion; each cell's
// own arithmetic is unchanged.
struct FmmStats {
    std::size_t ncells = 0, nleaves = 0, m2l_pairs = 0, p2p_pairs = 0;
    int depth = 0;
};

// mode 0: the reference's method; mode 1: the accurate mode (far field times
// G plus the softening correction, see softening_correction).
inline void accel_fmm(const std::vector<V3> &x, std::size_t s, double G, double mass, double eps, unsigned p,
                      std::vector<V3> &a, FmmStats *st = nullptr, int mode = 0) {
    a.assign(x.size(), V3{0, 0, 0});
    Tree t(x, s);
    Lists ls(t);
    const std::size_t nc = t.cells.size();
    std::vector<std::vector<std::size_t>> bylevel(static_cast<std::size_t>(t.max_level) + 1);
    for (std::size_t i = 0; i < nc; ++i) bylevel[static_cast<std::size_t>(t.cells[i].level)].push_back(i);
    for (int lv = t.max_level; lv >= 2; --lv) {
        const auto &cl = bylevel[static_cast<std::size_t>(lv)];
#pragma omp parallel for schedule(dynamic, 16)
        for (std::size_t k = 0; k < cl.size(); ++k) {
            if (t.cells[cl[k]].leaf())
                p2m(t.cells[cl[k]], p, x, mass);
            else
                m2m(t, cl[k], p);
        }
    }
    const double Gm = G * mass;
#pragma omp parallel for schedule(dynamic, 4)
    for (std::size_t i = 0; i < nc; ++i) {
        if (i > 8) m2l(t, i, p, ls.m2l[i]);
        if (t.cells[i].leaf()) p2p(t, i, ls.p2p[i], x, a, Gm, eps);
    }
    for (int lv = 2; lv <= t.max_level; ++lv) {
        const auto &cl = bylevel[static_cast<std::size_t>(lv)];
#pragma omp parallel for schedule(dynamic, 16)
        for (std::size_t k = 0; k < cl.size(); ++k) {
            if (lv >= 3) l2l(t, cl[k], p);
            if (t.cells[cl[k]].leaf()) l2p(t.cells[cl[k]], p, x, a, mode == 1 ? G : 1.0);
        }
    }
    if (mode == 1) softening_correction(t, ls, x, G, mass, eps, a);
    if (st) {
        st->ncells = nc;
        st->depth = t.max_level;
        for (std::size_t i = 0; i < nc; ++i) {
            if (i > 8) st->m2l_pairs += ls.m2l[i].size();
            if (t.cells[i].leaf()) ++st->nleaves;
        }
    }
}

// Direct softened sum for one target (solver_ref_naive.hpp:103-119).
inline V3 direct_one(const std::vector<V3> &x, std::size_t i, double G, double mass, double eps) {
    V3 acc{0, 0, 0};
    for (std::size_t j = 0; j < x.size(); ++j) {
        if (i == j) continue;
        const V3 d = sub(x[j], x[i]);
        const double den = std::pow(norm2(d) + eps * eps, 1.5);
        const double gm = G * mass;
        acc.x += gm * d.x / den, acc.y += gm * d.y / den, acc.z += gm * d.z / den;
    }
    return acc;
}

// Softened potential of the direct sum at target i, phi_i = -G m sum_{j != i}
// (|x_j - x_i|^2 + eps^2)^(-1/2). The reference computes no potential; this is
// the FP64 checker of the GPU potentials (same softening and self exclusion as
// direct_one, solver_ref_naive.hpp:103-119).
inline double direct_phi_one(const std::vector<V3> &x, std::size_t i, double G, double mass, double eps) {
    double s = 0;
    for (std::size_t j = 0; j < x.size(); ++j) {
        if (i == j) continue;
        s += 1.0 / std::sqrt(norm2(sub(x[j], x[i])) + eps * eps);
    }
    return -G * mass * s;
}

// Classical RK4 step (solver_ref.hpp:36-104): stage weights dt/6, dt/3, dt/3,
// dt/6; stage states x0 + c dt v_stage, v0 + c dt a with c = 1/2, 1/2, 1.
template <class AccelFn>
inline void rk4_step(std::vector<V3> &x, std::vector<V3> &v, double dt, AccelFn &&acc) {
    const std::size_t N = x.size();
    const std::vector<V3> x0 = x, v0 = v;
    std::vector<V3> xo = x, vo = v, a;
    const double w[4] = {dt / 6, dt / 3, dt / 3, dt / 6};
    const double c[3] = {dt / 2, dt / 2, dt};
    for (int st = 0; st < 4; ++st) {
        if (st > 0) {
#pragma omp parallel for
            for (std::size_t i = 0; i < N; ++i) {
                x[i] = {x0[i].x + v[i].x * c[st - 1], x0[i].y + v[i].y * c[st - 1], x0[i].z + v[i].z * c[st - 1]};
                v[i] = {v0[i].x + a[i].x * c[st - 1], v0[i].y + a[i].y * c[st - 1], v0[i].z + a[i].z * c[st - 1]};
            }
        }
        acc(x, a);
#pragma omp parallel for
        for (std::size_t i = 0; i < N; ++i) {
            xo[i].x += w[st] * v[i].x, xo[i].y += w[st] * v[i].y, xo[i].z += w[st] * v[i].z;
            vo[i].x += w[st] * a[i].x, vo[i].y += w[st] * a[i].y, vo[i].z += w[st] * a[i].z;
        }
    }
    x = xo;
    v = vo;
}

// Plummer initial conditions exactly as problem.hpp:188-292: mt19937_64(seed);
// x0 ~ U[0, 1-eps); r = x0^{1/3} / sqrt(1 - x0^{2/3}); v_e = sqrt(2) (r^2+1)^{-1/4};
// speed q v_e with q by von Neumann rejection on q^2 (1-q^2)^{7/2} below
// P_MAX = sqrt(7) 686/19683; directions from two uniforms each.
inline void plummer_reference(std::size_t N, double eps, std::uint64_t seed, std::vector<V3> &x, std::vector<V3> &v) {
    std::mt19937_64 eng(seed);
    std::uniform_real_distribution<double> dpos(0, 1.0 - eps), du(0, 1), dv(0, 1);
    const double pmax = std::sqrt(7.0) * 686 / 19683;
    const double PI = 3.141592653589793;
    auto xyz = [&](double norm, double r, double t) {
        const double xx = (1.0 - r * 2) * norm;
        const double yz = std::sqrt(norm * norm - xx * xx);
        return V3{xx, yz * std::cos(PI * 2 * t), yz * std::sin(PI * 2 * t)};
    };
    x.clear();
    v.clear();
    for (std::size_t i = 0; i < N; ++i) {
        const double x0 = dpos(eng);
        const double r = std::pow(x0, 1.0 / 3) / std::pow(1.0 - std::pow(x0, 2.0 / 3), 0.5);
        const double ve = std::sqrt(2.0) * std::pow(r * r + 1, -1.0 / 4);
        double q;
        while (true) {
            const double x1 = dv(eng), x2 = dv(eng);
            if (pmax * x1 < x2 * x2 * std::pow(1.0 - x2 * x2, 3.5)) {
                q = x2;
                break;
            }
        }
        const double x3 = du(eng), x4 = du(eng);
        x.push_back(xyz(r, x3, x4));
        const double x5 = dv(eng), x6 = dv(eng);
        v.push_back(xyz(q * ve, x5, x6));
    }
}

// E(T) = alpha T^c fit by bisection on c (benchmark.hpp:198-242).
inline void curve_fit(const std::vector<double> &e, const std::vector<double> &t, double &alpha, double &c) {
    double cmin = -10, cmax = 10;
    c = (cmin + cmax) / 2;
    const auto iters = static_cast<std::size_t>(std::ceil(std::log2((cmax - cmin) / 1e-10)));
    for (std::size_t it = 0; it < iters; ++it) {
        double s1 = 0, s2 = 0, s3 = 0, s4 = 0;
        for (std::size_t i = 0; i < t.size(); ++i) {
            const double xi = std::pow(t[i], c), lt = std::log(t[i]);
            s1 += e[i] * xi;
            s2 += xi * xi;
            s3 += e[i] * xi * lt;
            s4 += xi * xi * lt;
        }
        if (s1 * s4 - s2 * s3 >= 0)
            cmax = c;
        else
            cmin = c;
        c = (cmin + cmax) / 2;
    }
    double num = 0, den = 0;
    for (std::size_t i = 0; i < t.size(); ++i) {
        const double xi = std::pow(t[i], c);
        num += e[i] * xi;
        den += xi * xi;
    }
    alpha = num / den;
}

}  // namespace vipp_oracle
