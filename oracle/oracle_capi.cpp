// ORACLE — test infrastructure, not product code. C-ABI over oracle.hpp for
// the Python tests and the CPU-baseline legs of bench.py (loaded with ctypes).
#include "oracle.hpp"

#include <chrono>
#include <cstring>
#include <memory>
#ifdef _OPENMP
#include <omp.h>
#endif

using namespace vipp_oracle;

static std::vector<V3> to_v3(const double *aos, std::size_t n) {
    std::vector<V3> v(n);
    for (std::size_t i = 0; i < n; ++i) v[i] = {aos[3 * i], aos[3 * i + 1], aos[3 * i + 2]};
    return v;
}
static void from_v3(const std::vector<V3> &v, double *aos) {
    for (std::size_t i = 0; i < v.size(); ++i) aos[3 * i] = v[i].x, aos[3 * i + 1] = v[i].y, aos[3 * i + 2] = v[i].z;
}

struct OrcTree {
    std::vector<V3> x;
    std::unique_ptr<Tree> t;
    std::unique_ptr<Lists> l;
};
static OrcTree g_tree;

extern "C" {

int orc_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

void orc_set_threads(int n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}

void orc_P(unsigned nmax, double x, double *out) {
    Legendre P(nmax, x);
    for (unsigned n = 0; n <= nmax; ++n)
        for (unsigned m = 0; m <= nmax; ++m) out[n * (nmax + 1) + m] = m <= n ? P(n, m) : 0.0;
}

void orc_DP(unsigned nmax, double theta, double *out) {
    LegendreDTheta D(nmax, theta);
    for (unsigned n = 0; n <= nmax; ++n)
        for (unsigned m = 0; m <= nmax; ++m) out[n * (nmax + 1) + m] = m <= n ? D(n, m) : 0.0;
}

void orc_Y(unsigned nmax, double theta, double phi, double *out) {
    SphHarm Y(nmax, theta, phi);
    const unsigned w = 2 * nmax + 1;
    for (unsigned n = 0; n <= nmax; ++n)
        for (int m = -static_cast<int>(nmax); m <= static_cast<int>(nmax); ++m) {
            cd c{0, 0};
            if (static_cast<unsigned>(std::abs(m)) <= n) c = Y(n, m);
            const std::size_t o = 2 * (n * w + static_cast<unsigned>(m + static_cast<int>(nmax)));
            out[o] = c.real();
            out[o + 1] = c.imag();
        }
}

// Tree + lists, same export layout as the reference shim's dump.
std::size_t orc_tree_build(const double *x_aos, std::size_t n, std::size_t s) {
    g_tree.x = to_v3(x_aos, n);
    g_tree.t.reset(new Tree(g_tree.x, s));
    g_tree.l.reset(new Lists(*g_tree.t));
    return g_tree.t->cells.size();
}

void orc_tree_fetch(long long *parent, int *level, long long *first_child, double *mins, double *maxs, long long *pt_off,
                    long long *pts, long long *list_sizes) {
    const auto &cells = g_tree.t->cells;
    long long off = 0;
    for (std::size_t i = 0; i < cells.size(); ++i) {
        const Cell &c = cells[i];
        parent[i] = c.parent;
        level[i] = c.level;
        first_child[i] = c.first_child;
        mins[3 * i] = c.mn.x, mins[3 * i + 1] = c.mn.y, mins[3 * i + 2] = c.mn.z;
        maxs[3 * i] = c.mx.x, maxs[3 * i + 1] = c.mx.y, maxs[3 * i + 2] = c.mx.z;
        pt_off[i] = off;
        for (long long j : c.pts) pts[off++] = j;
        list_sizes[3 * i] = static_cast<long long>(g_tree.l->m2l[i].size());
        list_sizes[3 * i + 1] = static_cast<long long>(g_tree.l->p2p[i].size());
        list_sizes[3 * i + 2] = static_cast<long long>(g_tree.l->coll[i].size());
    }
    pt_off[cells.size()] = off;
}

void orc_tree_lists(long long *m2l, long long *p2p, long long *coll) {
    std::size_t a = 0, b = 0, c = 0;
    for (std::size_t i = 0; i < g_tree.t->cells.size(); ++i) {
        for (long long j : g_tree.l->m2l[i]) m2l[a++] = j;
        for (long long j : g_tree.l->p2p[i]) p2p[b++] = j;
        for (long long j : g_tree.l->coll[i]) coll[c++] = j;
    }
}

// One FMM force evaluation. stats (may be null): ncells, nleaves, depth, m2l pairs.
int orc_accel_mode(const double *x_aos, std::size_t n, std::size_t s, double G, double m, double eps, unsigned p,
                   int mode, double *a_aos, long long *stats) {
    try {
        auto x = to_v3(x_aos, n);
        std::vector<V3> a;
        FmmStats st;
        accel_fmm(x, s, G, m, eps, p, a, &st, mode);
        from_v3(a, a_aos);
        if (stats) {
            stats[0] = static_cast<long long>(st.ncells);
            stats[1] = static_cast<long long>(st.nleaves);
            stats[2] = st.depth;
            stats[3] = static_cast<long long>(st.m2l_pairs);
        }
        return 0;
    } catch (...) {
        return 1;
    }
}

int orc_accel(const double *x_aos, std::size_t n, std::size_t s, double G, double m, double eps, unsigned p, double *a_aos,
              long long *stats) {
    return orc_accel_mode(x_aos, n, s, G, m, eps, p, 0, a_aos, stats);
}

int orc_rk4_mode(double *x_aos, double *v_aos, std::size_t n, double G, double m, double eps, double dt, std::size_t s,
                 unsigned p, int steps, int mode) {
    try {
        auto x = to_v3(x_aos, n), v = to_v3(v_aos, n);
        for (int k = 0; k < steps; ++k)
            rk4_step(x, v, dt,
                     [&](const std::vector<V3> &xx, std::vector<V3> &aa) { accel_fmm(xx, s, G, m, eps, p, aa, nullptr, mode); });
        from_v3(x, x_aos);
        from_v3(v, v_aos);
        return 0;
    } catch (...) {
        return 1;
    }
}

int orc_rk4(double *x_aos, double *v_aos, std::size_t n, double G, double m, double eps, double dt, std::size_t s, unsigned p,
            int steps) {
    return orc_rk4_mode(x_aos, v_aos, n, G, m, eps, dt, s, p, steps, 0);
}

// Direct sum for the listed targets (all when targets == null).
void orc_direct_accel(const double *x_aos, std::size_t n, double G, double m, double eps, const long long *targets,
                      std::size_t nt, double *a_aos) {
    auto x = to_v3(x_aos, n);
    const std::size_t cnt = targets ? nt : n;
#pragma omp parallel for schedule(dynamic, 64)
    for (std::size_t k = 0; k < cnt; ++k) {
        const std::size_t i = targets ? static_cast<std::size_t>(targets[k]) : k;
        const V3 a = direct_one(x, i, G, m, eps);
        a_aos[3 * k] = a.x, a_aos[3 * k + 1] = a.y, a_aos[3 * k + 2] = a.z;
    }
}

void orc_direct_phi(const double *x_aos, std::size_t n, double G, double m, double eps, const long long *targets,
                    std::size_t nt, double *phi) {
    auto x = to_v3(x_aos, n);
    const std::size_t cnt = targets ? nt : n;
#pragma omp parallel for schedule(dynamic, 64)
    for (std::size_t k = 0; k < cnt; ++k) phi[k] = direct_phi_one(x, targets ? static_cast<std::size_t>(targets[k]) : k, G, m, eps);
}

void orc_direct_rk4(double *x_aos, double *v_aos, std::size_t n, double G, double m, double eps, double dt, int steps) {
    auto x = to_v3(x_aos, n), v = to_v3(v_aos, n);
    for (int k = 0; k < steps; ++k)
        rk4_step(x, v, dt, [&](const std::vector<V3> &xx, std::vector<V3> &aa) {
            aa.resize(xx.size());
#pragma omp parallel for schedule(dynamic, 64)
            for (std::size_t i = 0; i < xx.size(); ++i) aa[i] = direct_one(xx, i, G, m, eps);
        });
    from_v3(x, x_aos);
    from_v3(v, v_aos);
}

void orc_plummer_reference(std::size_t n, double eps, unsigned long long seed, double *x_aos, double *v_aos) {
    std::vector<V3> x, v;
    plummer_reference(n, eps, seed, x, v);
    from_v3(x, x_aos);
    from_v3(v, v_aos);
}

void orc_curve_fit(const double *e, const double *t, std::size_t n, double *alpha, double *c) {
    std::vector<double> ev(e, e + n), tv(t, t + n);
    curve_fit(ev, tv, *alpha, *c);
}

// Known-answer set-ups of gravity/test/test_fmm.cpp, restated. out: complex pairs.
// kat 0: P2M of one particle at (1,1,1), p=2 (test_fmm.cpp:326-338): M00, M10, M11.
// kat 1: M2M after a manual root split, p=2 (:340-355): M00, M10.
// kat 2: L_1^1 of cell 9 for three particles, s=1, p=2 (:357-387).
void orc_kat(int which, double *out) {
    if (which == 0) {
        std::vector<V3> x{{1, 1, 1}};
        Tree t(x, 1);
        p2m(t.cells[0], 2, x, 1.0);
        const cd a = t.cells[0].M[eidx(2, 0, 0)], b = t.cells[0].M[eidx(2, 1, 0)], c = t.cells[0].M[eidx(2, 1, 1)];
        out[0] = a.real(), out[1] = a.imag(), out[2] = b.real(), out[3] = b.imag(), out[4] = c.real(), out[5] = c.imag();
    } else if (which == 1) {
        std::vector<V3> x{{1, 0, 0}};
        Tree t(x, 1);
        t.threshold = 2;
        t.split(0);
        for (long long u = 1; u < 9; ++u) p2m(t.cells[static_cast<std::size_t>(u)], 2, x, 1.0);
        m2m(t, 0, 2);
        const cd a = t.cells[0].M[eidx(2, 0, 0)], b = t.cells[0].M[eidx(2, 1, 0)];
        out[0] = a.real(), out[1] = a.imag(), out[2] = b.real(), out[3] = b.imag();
    } else {
        std::vector<V3> x{{1, 1, 1}, {1, -1, -1}, {-1, -1, -1}};
        const unsigned p = 2;
        Tree t(x, 1);
        t.threshold = 2;
        t.split(1);
        t.split(8);
        Lists ls(t);
        std::vector<std::vector<std::size_t>> bylevel(static_cast<std::size_t>(t.max_level) + 1);
        for (std::size_t i = 0; i < t.cells.size(); ++i) bylevel[static_cast<std::size_t>(t.cells[i].level)].push_back(i);
        for (int lv = t.max_level; lv >= 2; --lv)
            for (std::size_t ci : bylevel[static_cast<std::size_t>(lv)]) {
                if (t.cells[ci].leaf())
                    p2m(t.cells[ci], p, x, 1.0 / 3);
                else
                    m2m(t, ci, p);
            }
        for (std::size_t i = 9; i < t.cells.size(); ++i) m2l(t, i, p, ls.m2l[i]);
        // The test's downward pass shifts into non-leaf cells only (test_fmm.cpp:67-80).
        for (int lv = 3; lv <= t.max_level; ++lv)
            for (std::size_t ci : bylevel[static_cast<std::size_t>(lv)])
                if (!t.cells[ci].leaf()) l2l(t, ci, p);
        const cd l = t.cells[9].L[eidx(p, 1, 1)];
        out[0] = l.real(), out[1] = l.imag();
    }
}

// CPU-baseline sample: the whole tree, lists and upward pass, then the
// per-cell far/near work (M2L, P2P, L2L, L2P) for every `stride`-th cell at
// level >= 2 only. Returns wall times [tree+lists, upward, sampled cells] and
// counts [cells, sampled cells, m2l pairs (all), m2l pairs (sampled),
// p2p pairs (all), p2p pairs (sampled)] so the caller can scale the sampled
// part up to the whole evaluation.
int orc_accel_sampled(const double *x_aos, std::size_t n, std::size_t s, double G, double m, double eps, unsigned p,
                      std::size_t stride, double *times, long long *counts) {
    try {
        using clk = std::chrono::steady_clock;
        auto x = to_v3(x_aos, n);
        std::vector<V3> a(n, V3{0, 0, 0});
        auto t0 = clk::now();
        Tree t(x, s);
        Lists ls(t);
        auto t1 = clk::now();
        const std::size_t nc = t.cells.size();
        std::vector<std::vector<std::size_t>> bylevel(static_cast<std::size_t>(t.max_level) + 1);
        for (std::size_t i = 0; i < nc; ++i) bylevel[static_cast<std::size_t>(t.cells[i].level)].push_back(i);
        for (int lv = t.max_level; lv >= 2; --lv) {
            const auto &cl = bylevel[static_cast<std::size_t>(lv)];
#pragma omp parallel for schedule(dynamic, 16)
            for (std::size_t k = 0; k < cl.size(); ++k) {
                if (t.cells[cl[k]].leaf())
                    p2m(t.cells[cl[k]], p, x, m);
                else
                    m2m(t, cl[k], p);
            }
        }
        auto t2 = clk::now();
        // Pair counts of the whole evaluation (P2P pairs via subtree sizes).
        std::vector<long long> sub(nc, 0);
        for (std::size_t i = nc; i-- > 0;) {
            if (t.cells[i].leaf())
                sub[i] = static_cast<long long>(t.cells[i].pts.size());
            else
                for (long long u = t.cells[i].first_child; u < t.cells[i].first_child + 8; ++u) sub[i] += sub[static_cast<std::size_t>(u)];
        }
        long long m2l_all = 0, p2p_all = 0;
        std::vector<std::size_t> sample;
        for (std::size_t i = 0; i < nc; ++i) {
            if (i > 8) m2l_all += static_cast<long long>(ls.m2l[i].size());
            if (t.cells[i].leaf()) {
                long long srcs = 0;
                for (long long q : ls.p2p[i]) srcs += sub[static_cast<std::size_t>(q)];
                p2p_all += static_cast<long long>(t.cells[i].pts.size()) * srcs;
            }
            if (t.cells[i].level >= 2 && i % stride == 0) sample.push_back(i);
        }
        long long m2l_s = 0, p2p_s = 0;
        for (std::size_t i : sample) {
            m2l_s += static_cast<long long>(ls.m2l[i].size());
            if (t.cells[i].leaf()) {
                long long srcs = 0;
                for (long long q : ls.p2p[i]) srcs += sub[static_cast<std::size_t>(q)];
                p2p_s += static_cast<long long>(t.cells[i].pts.size()) * srcs;
            }
        }
        const double Gm = G * m;
        // Only the cost is sampled: every cell gets a (zero) local expansion
        // so a sampled cell's L2L has a parent local to read.
        for (std::size_t i = 9; i < nc; ++i) t.cells[i].L.assign((p + 1) * (2 * p + 1), cd{0, 0});
        auto t3 = clk::now();
#pragma omp parallel for schedule(dynamic, 1)
        for (std::size_t k = 0; k < sample.size(); ++k) {
            const std::size_t i = sample[k];
            if (i > 8) m2l(t, i, p, ls.m2l[i]);
            if (t.cells[i].leaf()) p2p(t, i, ls.p2p[i], x, a, Gm, eps);
            if (t.cells[i].level >= 3) l2l(t, i, p);
            if (t.cells[i].leaf()) l2p(t.cells[i], p, x, a);
        }
        auto t4 = clk::now();
        times[0] = std::chrono::duration<double>(t1 - t0).count();
        times[1] = std::chrono::duration<double>(t2 - t1).count();
        times[2] = std::chrono::duration<double>(t4 - t3).count();
        counts[0] = static_cast<long long>(nc);
        counts[1] = static_cast<long long>(sample.size());
        counts[2] = m2l_all;
        counts[3] = m2l_s;
        counts[4] = p2p_all;
        counts[5] = p2p_s;
        return 0;
    } catch (...) {
        return 1;
    }
}

}  // extern "C"

extern "C" {
// The accurate mode's softening correction at the listed targets, and the
// exact sum it approximates: over every particle of the far source cells (the
// M2L lists of the target's leaf and of its ancestors at level >= 2) of
// G m F(|d|^2) d, F(u) = (u + eps^2)^-3/2 - u^-3/2.
int orc_soft_correction_check(const double *x_aos, std::size_t n, std::size_t s, double G, double m, double eps,
                              const long long *targets, std::size_t nt, double *exact_aos, double *approx_aos) {
    try {
        auto x = to_v3(x_aos, n);
        Tree t(x, s);
        Lists ls(t);
        std::vector<V3> a(n, V3{0, 0, 0});
        softening_correction(t, ls, x, G, m, eps, a);
        std::vector<long long> leaf_of(n, -1);
        for (std::size_t c = 0; c < t.cells.size(); ++c)
            if (t.cells[c].leaf())
                for (long long i : t.cells[c].pts) leaf_of[static_cast<std::size_t>(i)] = static_cast<long long>(c);
#pragma omp parallel for schedule(dynamic, 1)
        for (std::size_t q = 0; q < nt; ++q) {
            const std::size_t i = static_cast<std::size_t>(targets[q]);
            approx_aos[3 * q] = a[i].x, approx_aos[3 * q + 1] = a[i].y, approx_aos[3 * q + 2] = a[i].z;
            V3 acc{0, 0, 0};
            for (long long anc = leaf_of[i]; anc >= 0 && t.cells[static_cast<std::size_t>(anc)].level >= 2;
                 anc = t.cells[static_cast<std::size_t>(anc)].parent) {
                for (long long sidx : ls.m2l[static_cast<std::size_t>(anc)]) {
                    std::vector<std::size_t> stack{static_cast<std::size_t>(sidx)};
                    while (!stack.empty()) {
                        const std::size_t u = stack.back();
                        stack.pop_back();
                        if (!t.cells[u].leaf()) {
                            for (long long w = t.cells[u].first_child; w < t.cells[u].first_child + 8; ++w)
                                stack.push_back(static_cast<std::size_t>(w));
                            continue;
                        }
                        for (long long j : t.cells[u].pts) {
                            const V3 d = sub(x[static_cast<std::size_t>(j)], x[i]);
                            double F, F1, F2;
                            soft_diff(norm2(d), eps * eps, F, F1, F2);
                            acc.x += G * m * F * d.x, acc.y += G * m * F * d.y, acc.z += G * m * F * d.z;
                        }
                    }
                }
            }
            exact_aos[3 * q] = acc.x, exact_aos[3 * q + 1] = acc.y, exact_aos[3 * q + 2] = acc.z;
        }
        return 0;
    } catch (...) {
        return 1;
    }
}
}
