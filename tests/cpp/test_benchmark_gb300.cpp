// The validation-included benchmark driver (include/gravity/benchmark_gb300.hpp)
// used the way the reference accepts a solver (gravity/include/benchmark.hpp:91-175):
// the mixed-precision GPU solver against the FP64 GPU pipeline as comparator,
// identical solvers, and a solver with a 1% wrong time step, which must fail.
// Its curve fit is checked against the oracle's restatement of the reference's
// (oracle/oracle.hpp curve_fit). Built and run by tests/test_cpp_adapter.py.
#include <cmath>
#include <cstdio>
#include <vector>

#include <gravity/benchmark_gb300.hpp>
#include <gravity/solver_gb300.hpp>

#include "../../oracle/oracle.hpp"

namespace {

template <class U>
struct VecT {
    U x_ = 0, y_ = 0, z_ = 0;
    U x() const { return x_; }
    U y() const { return y_; }
    U z() const { return z_; }
    U &x() { return x_; }
    U &y() { return y_; }
    U &z() { return z_; }
};
using Vec = VecT<double>;
using VecF = VecT<float>;  // the reference's GRAVITY_FLOAT vectors

// Problem stand-in: the reference's accessors plus initialize() from the
// oracle's bit-identical restatement of Problem::initialize (Plummer sphere).
struct PlummerProblem {
    std::size_t n;
    std::size_t s_;
    double eps;
    unsigned p_;
    unsigned long long seed;
    std::size_t N() const { return n; }
    double epsilon() const { return eps; }
    double get_G() const { return 1.0; }
    double m() const { return 1.0 / static_cast<double>(n); }
    unsigned p() const { return p_; }
    std::size_t s() const { return s_; }
    double delta_t() const { return eps / std::sqrt(2.0); }  // problem.hpp:235-243
    template <class W>
    void initialize(std::vector<W> &x, std::vector<W> &v) const {
        std::vector<vipp_oracle::V3> x3, v3;
        vipp_oracle::plummer_reference(n, eps, seed, x3, v3);
        x.resize(n), v.resize(n);
        using U = decltype(x[0].x_);
        for (std::size_t i = 0; i < n; ++i) {
            x[i].x_ = static_cast<U>(x3[i].x), x[i].y_ = static_cast<U>(x3[i].y), x[i].z_ = static_cast<U>(x3[i].z);
            v[i].x_ = static_cast<U>(v3[i].x), v[i].y_ = static_cast<U>(v3[i].y), v[i].z_ = static_cast<U>(v3[i].z);
        }
    }
};

// A solver whose step is 1% short: solve(problem, t) steps delta_t / (1.01 t).
template <class S>
struct ShortStep {
    S s;
    template <class P, class X, class V>
    void preprocess(const P &p, const X &x, const V &v) { s.preprocess(p, x, v); }
    template <class P, class X, class V>
    void solve(const P &p, double t, X &x, V &v) { s.solve(p, 1.01 * t, x, v); }
    template <class P, class X, class V>
    void postprocess(const P &p, X &x, V &v) { s.postprocess(p, x, v); }
};

int failures = 0;
void expect(bool ok, const char *what) {
    std::printf("%s %s\n", ok ? "PASS" : "FAIL", what);
    if (!ok) ++failures;
}

void show(const char *name, const gravity::BenchmarkResultGB300 &r) {
    std::printf("%s: E(T) =", name);
    for (double e : r.e_t) std::printf(" %.3e", e);
    std::printf("  alpha %.3e (threshold %.3e)  c %.3f  %s  eval %.3f s\n", r.alpha, r.alpha_threshold, r.c,
                r.passed ? "passed" : "failed", r.eval_seconds);
}

}  // namespace

int main() {
    using gravity::BenchmarkGB300;
    {  // curve fit against the oracle's restatement of the reference's
        const auto t = BenchmarkGB300::geometric_sequence(1, 2, 5);
        std::vector<double> e;
        for (std::size_t k = 0; k < t.size(); ++k) e.push_back(3e-4 * std::pow(t[k], -2.5) * (1 + 0.01 * ((k % 2) ? 1 : -1)));
        const auto [a, c] = BenchmarkGB300::curve_fitting(e, t);
        double ao = 0, co = 0;
        vipp_oracle::curve_fit(e, t, ao, co);
        expect(std::fabs(a - ao) <= 1e-12 * std::fabs(ao) && std::fabs(c - co) <= 1e-9, "curve fit equals the oracle's");
        expect(std::fabs(c + 2.5) < 0.05, "curve fit recovers the exponent");
    }
    const PlummerProblem pr{8192, 32, 0.01, 6, 5};
    using Mixed = gravity::SolverGB300<double, double, double, double, double, double, GB_PREC_MIXED>;
    using Fp64 = gravity::SolverGB300<double, double, double, double, double, double>;
    std::vector<Vec> xe, ve, xr, vr;
    {
        Mixed eval;
        Fp64 ref;
        const auto r = BenchmarkGB300::run(eval, ref, pr, pr, xe, ve, xr, vr);
        show("mixed vs FP64", r);
        expect(r.passed, "mixed-precision GPU solver passes against the FP64 pipeline");
        expect(r.e_t[0] > 0 && r.e_t[4] < r.e_t[0], "E(T) decreases with T");
    }
    {
        Fp64 eval, ref;
        const auto r = BenchmarkGB300::run(eval, ref, pr, pr, xe, ve, xr, vr);
        show("FP64 vs FP64", r);
        expect(r.passed && r.e_t[0] == 0.0, "identical solvers: E(T) = 0, passed");
    }
    {
        ShortStep<Fp64> eval;
        Fp64 ref;
        const auto r = BenchmarkGB300::run(eval, ref, pr, pr, xe, ve, xr, vr);
        show("1% short step", r);
        expect(!r.passed && r.c > -1.5, "a solver with a wrong step fails (E ~ T^-1)");
    }
    {  // benchmark_different_precision (benchmark.hpp:33-87): float state, mixed GPU solver, FP64 comparator
        using MixedF = gravity::SolverGB300<float, float, float, float, float, float, GB_PREC_MIXED>;
        MixedF eval;
        Fp64 ref;
        std::vector<VecF> xf, vf;
        const auto r = BenchmarkGB300::run(eval, ref, pr, pr, xf, vf, xr, vr);
        show("float mixed vs FP64", r);
        expect(r.passed, "float-typed mixed solver passes against the FP64 pipeline");
    }
    std::printf(failures ? "%d FAILED\n" : "ALL PASSED\n", failures);
    return failures ? 1 : 0;
}
