// Test infrastructure only: a C-ABI shim over the reference's own gravity
// headers (satoshigeyuki/vipp-nbody-bench, gravity/include/*.hpp), compiled
// unmodified from where they lie by oracle/build_ref.sh into oracle/_ref/.
// Only tests/ and the golden-fixture generator load the result; no product
// path does. It reaches the reference's private members through the
// ENABLE_TEST friend hooks the reference itself provides
// (octree.hpp:123-125, fmm.hpp:495-497, solver_ref.hpp:29-32,
// solver_ref_naive.hpp:272-274, problem.hpp:245-247, benchmark.hpp:177-179).
#define ENABLE_TEST
#include <benchmark.hpp>
#include <solver_ref.hpp>
#include <solver_ref_naive.hpp>

#include <cstdint>
#include <cstring>
#include <vector>

namespace gravity {
using R = double;
using RCell = Cell<R, R, R, R, R, R>;
using RTree = Octree<RCell, Vector<R>>;
using RSolver = SolverRef<R, R, R, R, R, R>;
using RNaive = SolverRefNaive<R, R, R, R, R, R>;
using RProblem = Problem<R, R, R, R, R, R>;

struct FMMTest {
    static void calc_link(const RCell &cell, const std::vector<RCell> &cells,
                          std::vector<std::vector<std::size_t>> &a,
                          std::vector<std::vector<std::size_t>> &ni,
                          std::vector<std::vector<std::size_t>> &n, std::size_t level) {
        RSolver::calc_link(cell, cells, a, ni, n, level);
    }
    static std::complex<R> getM(const RCell &c, unsigned p, unsigned k, int m) { return c.multipole(p, k, m); }
    static std::complex<R> getL(const RCell &c, unsigned p, unsigned j, int k) { return c.local(p, j, k); }
    static void divide(RTree &t, std::size_t idx, std::size_t thr) { t.subdivide(idx, thr); }
    static bool has_multipole(const RCell &c) { return !c._multipole.empty(); }
    static bool has_local(const RCell &c) { return !c._local.empty(); }
    // Upward pass exactly as solver_ref.hpp:184-201.
    static void calcM(RTree &tree, unsigned p, R m, const std::vector<Vector<R>> &x) {
        auto &cells = tree.cells();
        tree.apply(RTree::fix([&cells, &p, &m, &x](const auto &f, RCell &cell, std::size_t level) -> void {
                       const auto &content = cell.content();
                       if (content.index() == RCell::INDEX_POINTS) {
                           if (level >= 2) p2m(cell, p, x, m);
                       } else {
                           const auto base = std::get<RCell::INDEX_CELLS>(content);
                           for (auto ci = base; ci < base + 8; ++ci) f(f, cells[ci], level + 1);
                           if (level >= 2) m2m(cell, p, cells);
                       }
                   }),
                   std::size_t{0});
    }
    // M2L for index > 8 then L2L top-down, as gravity/test/test_fmm.cpp:54-81.
    static void calcL(RTree &tree, unsigned p) {
        auto &cells = tree.cells();
        std::vector<std::vector<std::size_t>> a{cells.size()}, ni{cells.size()}, n{cells.size()};
        tree.apply(calc_link, cells, a, ni, n, std::size_t{0});
        for (std::size_t i = 0; i < cells.size(); ++i)
            if (cells[i].index() > 8) m2l(cells[i], p, cells, a[i]);
        tree.apply(RTree::fix([&cells, &p](const auto &f, RCell &cell, std::size_t level) -> void {
                       const auto &content = cell.content();
                       if (content.index() == RCell::INDEX_CELLS) {
                           if (level >= 3) l2l(cell, p, cells);
                           const auto base = std::get<RCell::INDEX_CELLS>(content);
                           for (auto ci = base; ci < base + 8; ++ci) f(f, cells[ci], level + 1);
                       }
                   }),
                   std::size_t{0});
    }
};

struct SolverRefTest {
    static void acceleration(const std::vector<Vector<R>> &x, std::size_t s, R G, R m, R eps,
                             std::vector<Vector<R>> &a, unsigned p) {
        RSolver::acceleration(x, s, G, m, eps, a, p);
    }
    static void runge_kutta(std::vector<Vector<R>> &x, std::vector<Vector<R>> &v, R G, R m, R eps,
                            R dt, std::size_t s, unsigned p) {
        RSolver::runge_kutta(x, v, G, m, eps, dt, s, p);
    }
};

struct SolverRefNaiveTest {
    static Vector<R> acceleration(const std::vector<Vector<R>> &x, R G, R m, R eps, std::size_t i) {
        return RNaive::acceleration(x, G, m, eps, i);
    }
    static void runge_kutta(std::vector<Vector<R>> &x, std::vector<Vector<R>> &v, R G, R m, R eps, R dt) {
        RNaive::runge_kutta(x, v, G, m, eps, dt);
    }
};

struct ProblemTest {
    static R r(R x0) { return RProblem::r(x0); }
    static R v_e(R r) { return RProblem::v_e(r); }
    static R P(R q) { return RProblem::P(q); }
    static Vector<R> calc_xyz(R n, R r, R t) { return RProblem::calc_xyz<R>(n, r, t); }
};

struct BenchmarkTest {
    static std::tuple<R, R> curve_fitting(const std::vector<R> &e, const std::vector<R> &t) {
        return Benchmark<R, R, R, R, R, R>::curve_fitting(e, t);
    }
    static std::vector<R> geometric_sequence(R a, R r, std::size_t n) {
        return Benchmark<R, R, R, R, R, R>::geometric_sequence(a, r, n);
    }
};
}  // namespace gravity

using namespace gravity;

static std::vector<Vector<R>> to_vec(const double *aos, std::size_t n) {
    std::vector<Vector<R>> v;
    v.reserve(n);
    for (std::size_t i = 0; i < n; ++i) v.emplace_back(aos[3 * i], aos[3 * i + 1], aos[3 * i + 2]);
    return v;
}
static void from_vec(const std::vector<Vector<R>> &v, double *aos) {
    for (std::size_t i = 0; i < v.size(); ++i) {
        aos[3 * i] = v[i].x();
        aos[3 * i + 1] = v[i].y();
        aos[3 * i + 2] = v[i].z();
    }
}

extern "C" {

// Problem::initialize (problem.hpp:188-211) with the given constructor arguments.
int ref_initialize(std::size_t n, std::size_t s, double eps, int has_eps, unsigned p, std::uint64_t seed,
                   double *x_aos, double *v_aos, double *eps_out, double *dt_out, double *m_out) {
    try {
        RProblem prob{n, s, has_eps ? std::optional<R>(eps) : std::nullopt, 1, 1, 1, p, seed};
        std::vector<Vector<R>> x, v;
        prob.initialize(x, v);
        from_vec(x, x_aos);
        from_vec(v, v_aos);
        if (eps_out) *eps_out = prob.epsilon();
        if (dt_out) *dt_out = prob.delta_t();
        if (m_out) *m_out = prob.m();
        return 0;
    } catch (...) {
        return 1;
    }
}

void ref_problem_parts(double x0, double q, double *r, double *ve, double *P) {
    *r = ProblemTest::r(x0);
    *ve = ProblemTest::v_e(x0);
    *P = ProblemTest::P(q);
}

void ref_calc_xyz(double norm, double r, double t, double *out3) {
    auto v = ProblemTest::calc_xyz(norm, r, t);
    out3[0] = v.x();
    out3[1] = v.y();
    out3[2] = v.z();
}

// SolverRef::acceleration (solver_ref.hpp:164-177): tree + lists + FMM.
void ref_accel(const double *x_aos, std::size_t n, std::size_t s, double G, double m, double eps, unsigned p,
               double *a_aos) {
    auto x = to_vec(x_aos, n);
    std::vector<Vector<R>> a(n, Vector<R>{});
    SolverRefTest::acceleration(x, s, G, m, eps, a, p);
    from_vec(a, a_aos);
}

// SolverRef::runge_kutta (solver_ref.hpp:36-104), `steps` times.
void ref_rk4(double *x_aos, double *v_aos, std::size_t n, double G, double m, double eps, double dt,
             std::size_t s, unsigned p, int steps) {
    auto x = to_vec(x_aos, n);
    auto v = to_vec(v_aos, n);
    for (int k = 0; k < steps; ++k) SolverRefTest::runge_kutta(x, v, G, m, eps, dt, s, p);
    from_vec(x, x_aos);
    from_vec(v, v_aos);
}

// SolverRefNaive::acceleration (solver_ref_naive.hpp:103-119) for every i.
void ref_naive_accel(const double *x_aos, std::size_t n, double G, double m, double eps, double *a_aos) {
    auto x = to_vec(x_aos, n);
    for (std::size_t i = 0; i < n; ++i) {
        auto a = SolverRefNaiveTest::acceleration(x, G, m, eps, i);
        a_aos[3 * i] = a.x();
        a_aos[3 * i + 1] = a.y();
        a_aos[3 * i + 2] = a.z();
    }
}

void ref_naive_rk4(double *x_aos, double *v_aos, std::size_t n, double G, double m, double eps, double dt,
                   int steps) {
    auto x = to_vec(x_aos, n);
    auto v = to_vec(v_aos, n);
    for (int k = 0; k < steps; ++k) SolverRefNaiveTest::runge_kutta(x, v, G, m, eps, dt);
    from_vec(x, x_aos);
    from_vec(v, v_aos);
}

// Special functions (fmm.hpp:20-194).
void ref_P(unsigned nmax, double x, double *out /*(nmax+1)^2, [n*(nmax+1)+m]*/) {
    P<R> pp{nmax, nmax, x};
    for (unsigned n = 0; n <= nmax; ++n)
        for (unsigned m = 0; m <= nmax; ++m) out[n * (nmax + 1) + m] = m <= n ? pp(n, m) : 0.0;
}
void ref_DP(unsigned nmax, double theta, double *out) {
    DP<R> dp{nmax, nmax, theta};
    for (unsigned n = 0; n <= nmax; ++n)
        for (unsigned m = 0; m <= nmax; ++m) out[n * (nmax + 1) + m] = m <= n ? dp(n, m) : 0.0;
}
void ref_Y(unsigned nmax, double theta, double phi, double *out /*[(n*(2nmax+1)+(m+nmax))*2]*/) {
    Y<R> y{nmax, nmax, theta, phi};
    const unsigned w = 2 * nmax + 1;
    for (unsigned n = 0; n <= nmax; ++n)
        for (int m = -static_cast<int>(nmax); m <= static_cast<int>(nmax); ++m) {
            std::complex<R> c{0, 0};
            if (static_cast<unsigned>(m < 0 ? -m : m) <= n) c = y(n, m);
            out[2 * (n * w + static_cast<unsigned>(m + static_cast<int>(nmax)))] = c.real();
            out[2 * (n * w + static_cast<unsigned>(m + static_cast<int>(nmax))) + 1] = c.imag();
        }
}

// Tree dump. Counts first (cells_out == nullptr) then fills.
// Per cell: parent (-1 root), level, first_child (-1 leaf), min[3], max[3], point range into
// pts_out. Lists from calc_link (solver_ref.hpp:115-162) in CSR form.
struct RefTreeDump {
    std::vector<RCell> cells;
    std::vector<std::vector<std::size_t>> a, ni, n;
};
static RefTreeDump *g_dump = nullptr;

std::size_t ref_tree_build(const double *x_aos, std::size_t npts, std::size_t s) {
    delete g_dump;
    g_dump = new RefTreeDump;
    auto x = to_vec(x_aos, npts);
    RTree tree{x, s};
    g_dump->cells = tree.cells();
    auto &cells = g_dump->cells;
    g_dump->a.assign(cells.size(), {});
    g_dump->ni.assign(cells.size(), {});
    g_dump->n.assign(cells.size(), {});
    FMMTest::calc_link(cells[0], cells, g_dump->a, g_dump->ni, g_dump->n, 0);
    return cells.size();
}

// list_sizes: [ncells*3] sizes of (m2l, p2p, colleague) lists
void ref_tree_fetch(long long *parent, int *level, long long *first_child, double *mins, double *maxs,
                    long long *pt_off, long long *pts, long long *list_sizes) {
    auto &cells = g_dump->cells;
    long long off = 0;
    for (std::size_t i = 0; i < cells.size(); ++i) {
        const auto &c = cells[i];
        parent[i] = c.parent() ? static_cast<long long>(c.parent().value()) : -1;
        int lv = 0;
        auto q = c.parent();
        while (q) {
            ++lv;
            q = cells[q.value()].parent();
        }
        level[i] = lv;
        mins[3 * i] = c.min().x();
        mins[3 * i + 1] = c.min().y();
        mins[3 * i + 2] = c.min().z();
        maxs[3 * i] = c.max().x();
        maxs[3 * i + 1] = c.max().y();
        maxs[3 * i + 2] = c.max().z();
        pt_off[i] = off;
        if (c.is_leaf()) {
            first_child[i] = -1;
            for (auto j : c.points()) pts[off++] = static_cast<long long>(j);
        } else {
            first_child[i] = static_cast<long long>(std::get<RCell::INDEX_CELLS>(c.content()));
        }
        list_sizes[3 * i] = static_cast<long long>(g_dump->a[i].size());
        list_sizes[3 * i + 1] = static_cast<long long>(g_dump->ni[i].size());
        list_sizes[3 * i + 2] = static_cast<long long>(g_dump->n[i].size());
    }
    pt_off[cells.size()] = off;
}

void ref_tree_lists(long long *m2l, long long *p2p, long long *coll) {
    auto &cells = g_dump->cells;
    std::size_t a = 0, b = 0, c = 0;
    for (std::size_t i = 0; i < cells.size(); ++i) {
        for (auto j : g_dump->a[i]) m2l[a++] = static_cast<long long>(j);
        for (auto j : g_dump->ni[i]) p2p[b++] = static_cast<long long>(j);
        for (auto j : g_dump->n[i]) coll[c++] = static_cast<long long>(j);
    }
}

// Multipoles/locals of every cell after calcM/calcL (test_fmm.cpp:32-81) with order p.
// out: [ncells][(p+1)][(2p+1)][2]; has_m/has_l flags per cell.
std::size_t ref_expansions(const double *x_aos, std::size_t npts, std::size_t s, unsigned p, double m,
                           double *mult, double *loc, int *has_m, int *has_l) {
    auto x = to_vec(x_aos, npts);
    RTree tree{x, s};
    FMMTest::calcM(tree, p, m, x);
    FMMTest::calcL(tree, p);
    const auto &cells = tree.cells();
    if (!mult) return cells.size();
    const unsigned w = 2 * p + 1;
    for (std::size_t i = 0; i < cells.size(); ++i) {
        has_m[i] = FMMTest::has_multipole(cells[i]);
        has_l[i] = FMMTest::has_local(cells[i]);
        for (unsigned k = 0; k <= p; ++k)
            for (int mm = -static_cast<int>(k); mm <= static_cast<int>(k); ++mm) {
                const std::size_t o = 2 * ((i * (p + 1) + k) * w + static_cast<unsigned>(mm + static_cast<int>(p)));
                std::complex<R> vm{0, 0}, vl{0, 0};
                if (has_m[i]) vm = FMMTest::getM(cells[i], p, k, mm);
                if (has_l[i]) vl = FMMTest::getL(cells[i], p, k, mm);
                mult[o] = vm.real();
                mult[o + 1] = vm.imag();
                loc[o] = vl.real();
                loc[o + 1] = vl.imag();
            }
    }
    return cells.size();
}

// gravity/test/test_fmm.cpp:357-387 setup: 3 points, s=1, p=2, manual subdivisions of cells 1 and 8.
void ref_kat_L(double *out_l11 /*2*/) {
    const std::vector<Vector<R>> x{{1, 1, 1}, {1, -1, -1}, {-1, -1, -1}};
    const unsigned p = 2;
    RTree tree{x, 1};
    FMMTest::divide(tree, 1, 2);
    FMMTest::divide(tree, 8, 2);
    FMMTest::calcM(tree, p, R{1} / 3, x);
    FMMTest::calcL(tree, p);
    auto l = FMMTest::getL(tree.cells()[9], p, 1, 1);
    out_l11[0] = l.real();
    out_l11[1] = l.imag();
}

void ref_curve_fitting(const double *e, const double *t, std::size_t n, double *alpha, double *c) {
    std::vector<R> ev(e, e + n), tv(t, t + n);
    auto [a, cc] = BenchmarkTest::curve_fitting(ev, tv);
    *alpha = a;
    *c = cc;
}

}  // extern "C"
