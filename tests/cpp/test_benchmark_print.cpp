// BenchmarkGB300::run built with ENABLE_PRINT, driven by two host-only stub
// solvers (no GPU): it must write before.csv and after<T>.csv in the working
// directory, as the reference's ENABLE_PRINT build does.
#define ENABLE_PRINT
#include <cstdio>
#include <vector>

#include "gravity/benchmark_gb300.hpp"

struct Vec {
    double a[3];
    double x() const { return a[0]; }
    double y() const { return a[1]; }
    double z() const { return a[2]; }
};

struct StubProblem {
    std::size_t N() const { return 3; }
    void initialize(std::vector<Vec> &x, std::vector<Vec> &v) const {
        x = {{{0.125, -1.5, 2.0}}, {{1.0 / 3.0, 1e-7, -123456.789}}, {{0.0, 2.5e10, -0.0}}};
        v.assign(3, Vec{{0.0, 0.0, 0.0}});
    }
};

// Moves every position by t * shift along x.
struct StubSolver {
    double shift;
    void preprocess(const StubProblem &, std::vector<Vec> &, std::vector<Vec> &) {}
    void solve(const StubProblem &, double t, std::vector<Vec> &x, std::vector<Vec> &) {
        for (auto &q : x) q.a[0] += t * shift;
    }
    void postprocess(const StubProblem &, std::vector<Vec> &, std::vector<Vec> &) {}
};

int main() {
    StubProblem prob;
    StubSolver eval{1e-3}, ref{1e-3 + 1e-9};
    std::vector<Vec> xe, ve, xr, vr;
    const auto r = gravity::BenchmarkGB300::run(eval, ref, prob, prob, xe, ve, xr, vr, {1, 2, 4});
    std::printf("ran %zu T values\n", r.e_t.size());
    return r.e_t.size() == 3 ? 0 : 1;
}
