// Validation-included benchmark of a Solver, as the reference accepts a
// replacement solver (gravity/include/benchmark.hpp:91-175, curve fit
// :210-243): for every T of a time-step set (1, 2, 4, 8, 16 by default) both
// the evaluated solver and a comparator start from the same initial state and
// take one RK4 step of delta_t / T (the comparator optionally in `subdivide`
// steps of delta_t / (subdivide T)); E(T) = sqrt(sum_i |x_eval,i - x_ref,i|^2)
// is fitted to E(T) = alpha T^c, and the solver passes when
// alpha < 1e-6 sqrt(N) or c < -5 + 1e-2. Only the evaluated solver's solve()
// is timed.
//
// The reference runs SolverRef<double> on the CPU as the comparator; any
// Solver fits here, e.g. gravity::SolverGB300 in FP64, which reproduces
// SolverRef<double>'s RK4 step to ~1e-14 relative.
//
// Problem requirements: N(), and initialize(x, v) filling the initial state
// (the reference's Problem::initialize, problem.hpp:188-211); plus what the
// two solvers read (p, s, epsilon, get_G, m, delta_t).
//
// Built with ENABLE_PRINT, run() writes the evaluated solver's positions as
// the reference's ENABLE_PRINT build does (benchmark.hpp:15-20, 46-58):
// before.csv from the initial state and after<T>.csv after each solve, one
// "x,y,z" line per particle in the stream's default format.
#pragma once

#include <chrono>
#include <cmath>
#include <tuple>
#include <vector>
#ifdef ENABLE_PRINT
#include <fstream>
#include <sstream>
#include <string>
#endif

namespace gravity {

struct BenchmarkResultGB300 {
    std::vector<double> t_set;
    std::vector<double> e_t;  // E(T) for each T
    double alpha = 0, c = 0;
    double alpha_threshold = 0, c_threshold = 0;
    bool passed = false;
    double eval_seconds = 0;  // solve() of the evaluated solver, summed over T
};

struct BenchmarkGB300 {
    static constexpr double ALPHA_THRESHOLD = 1e-6;  // times sqrt(N)
    static constexpr double C_THRESHOLD = 1e-2;      // c < -5 + C_THRESHOLD
    static constexpr double C_MIN = -10, C_MAX = 10, C_EPSILON = 1e-10;

    // {a, a r, a r^2, ..., a r^(n-1)}
    static std::vector<double> geometric_sequence(double a, double r, std::size_t n) {
        std::vector<double> s(n, a);
        for (std::size_t i = 1; i < n; ++i) s[i] = s[i - 1] * r;
        return s;
    }

    // Least-squares fit of E(T) = alpha T^c: for a given c the best alpha is
    // sum E T^c / sum T^2c; the residual's derivative in c changes sign where
    //   (sum E T^c)(sum T^2c ln T) - (sum T^2c)(sum E T^c ln T) = 0,
    // which is found by bisection on [C_MIN, C_MAX] to C_EPSILON.
    static std::tuple<double, double> curve_fitting(const std::vector<double> &e_t, const std::vector<double> &t_set) {
        double lo = C_MIN, hi = C_MAX, c = 0.5 * (lo + hi);
        const int iters = static_cast<int>(std::ceil(std::log2((C_MAX - C_MIN) / C_EPSILON)));
        for (int it = 0; it < iters; ++it) {
            double se = 0, s2 = 0, sel = 0, s2l = 0;
            for (std::size_t k = 0; k < t_set.size(); ++k) {
                const double tc = std::pow(t_set[k], c), lt = std::log(t_set[k]);
                se += e_t[k] * tc;
                s2 += tc * tc;
                sel += e_t[k] * tc * lt;
                s2l += tc * tc * lt;
            }
            if (se * s2l - s2 * sel >= 0)
                hi = c;
            else
                lo = c;
            c = 0.5 * (lo + hi);
        }
        double num = 0, den = 0;
        for (std::size_t k = 0; k < t_set.size(); ++k) {
            const double tc = std::pow(t_set[k], c);
            num += e_t[k] * tc;
            den += tc * tc;
        }
        return {num / den, c};
    }

#ifdef ENABLE_PRINT
    template <class X>
    static void print(const std::string &filename, const std::vector<X> &x) {
        std::ofstream out(filename);
        for (const auto &q : x) out << q.x() << "," << q.y() << "," << q.z() << "\n";
    }
#endif

    // The evaluated and comparator states may use different vector types
    // (the reference's benchmark_different_precision, benchmark.hpp:33-87).
    template <class EvalSolver, class RefSolver, class ProblemEval, class ProblemRef, class XE, class VE, class XR, class VR>
    static BenchmarkResultGB300 run(EvalSolver &eval, RefSolver &ref, const ProblemEval &problem, const ProblemRef &problem_ref,
                                    std::vector<XE> &x_eval, std::vector<VE> &v_eval, std::vector<XR> &x_ref,
                                    std::vector<VR> &v_ref, std::vector<double> t_set = geometric_sequence(1, 2, 5),
                                    std::size_t subdivide = 1) {
        BenchmarkResultGB300 r;
        r.t_set = t_set;
        for (const double t : t_set) {
            problem.initialize(x_eval, v_eval);
#ifdef ENABLE_PRINT
            print("before.csv", x_eval);
#endif
            eval.preprocess(problem, x_eval, v_eval);
            const auto t0 = std::chrono::high_resolution_clock::now();
            eval.solve(problem, t, x_eval, v_eval);
            const auto t1 = std::chrono::high_resolution_clock::now();
            eval.postprocess(problem, x_eval, v_eval);
            r.eval_seconds += std::chrono::duration<double>(t1 - t0).count();
#ifdef ENABLE_PRINT
            std::ostringstream name;
            name << "after" << t << ".csv";
            print(name.str(), x_eval);
#endif

            problem_ref.initialize(x_ref, v_ref);
            ref.preprocess(problem_ref, x_ref, v_ref);
            for (std::size_t k = 0; k < subdivide; ++k) ref.solve(problem_ref, static_cast<double>(subdivide) * t, x_ref, v_ref);
            ref.postprocess(problem_ref, x_ref, v_ref);

            double e2 = 0;
            for (std::size_t i = 0; i < x_eval.size(); ++i) {
                const double dx = static_cast<double>(x_eval[i].x()) - static_cast<double>(x_ref[i].x());
                const double dy = static_cast<double>(x_eval[i].y()) - static_cast<double>(x_ref[i].y());
                const double dz = static_cast<double>(x_eval[i].z()) - static_cast<double>(x_ref[i].z());
                e2 += dx * dx + dy * dy + dz * dz;
            }
            r.e_t.push_back(std::sqrt(e2));
        }
        std::tie(r.alpha, r.c) = curve_fitting(r.e_t, r.t_set);
        r.alpha_threshold = ALPHA_THRESHOLD * std::sqrt(static_cast<double>(problem.N()));
        r.c_threshold = -5 + C_THRESHOLD;
        r.passed = r.alpha < r.alpha_threshold || r.c < r.c_threshold;
        return r;
    }
};

}  // namespace gravity
