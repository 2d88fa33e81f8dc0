// The drop-in adapter instantiated with the reference's own types:
// gravity::Problem and gravity::Vector (gravity/include/problem.hpp:32-302),
// driven exactly as Benchmark::benchmark drives a Solver
// (gravity/include/benchmark.hpp:118-128): initialize -> preprocess ->
// solve(problem, t, x, v) -> postprocess. Compiled and linked by
// tests/test_reference_boundary.py against the reference's headers where they
// are present; it runs only on a GPU host.
#include <cstdio>
#include <optional>
#include <vector>

#include <problem.hpp>
#include <gravity/solver_gb300.hpp>

template <class R, int Precision, int Mode>
int run_one(const char *name) {
    using Problem = gravity::Problem<R, R, R, R, R, R>;
    const Problem problem{2048, 16, std::optional<R>(R(0.01)), R(1), R(1), R(1), 4, 0};
    std::vector<gravity::Vector<R>> x, v;
    problem.initialize(x, v);
    gravity::SolverGB300<R, R, R, R, R, R, Precision, Mode> solver;
    solver.preprocess(problem, x, v);
    solver.solve(problem, R(1), x, v);
    solver.postprocess(problem, x, v);
    std::printf("%s: x[0] = (%g, %g, %g)\n", name, static_cast<double>(x[0].x()), static_cast<double>(x[0].y()),
                static_cast<double>(x[0].z()));
    return 0;
}

int main() {
    run_one<double, GB_PREC_FP64, GB_MODE_REF>("double, fp64");
    run_one<float, GB_PREC_MIXED, GB_MODE_REF>("float, mixed");
    run_one<double, GB_PREC_MIXED, GB_MODE_ACCURATE>("double, mixed, accurate");
    std::printf("ALL PASSED\n");
    return 0;
}
