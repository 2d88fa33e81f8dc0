// The drop-in adapter gravity::SolverGB300 used the way the reference's
// benchmark uses a Solver (gravity/include/benchmark.hpp:118-146):
// preprocess -> solve(problem, t, x, v) -> postprocess, with a problem type
// that has the reference's accessors (p, s, epsilon, get_G, m, delta_t) and
// a 3-vector with x()/y()/z(). Checked against the oracle's restatement of the
// reference (oracle/oracle.hpp) and the closed-form two-body step of
// gravity/test/test_solver_ref_naive.cpp:47-79. Built and run by
// tests/test_cpp_adapter.py on a GPU host.
#include <cmath>
#include <cstdio>
#include <stdexcept>
#include <string>
#include <vector>

#include <gravity/solver_gb300.hpp>

#include "../../oracle/oracle.hpp"

namespace {

struct Vec {
    double x_ = 0, y_ = 0, z_ = 0;
    Vec() = default;
    Vec(double a, double b, double c) : x_(a), y_(b), z_(c) {}
    double x() const { return x_; }
    double y() const { return y_; }
    double z() const { return z_; }
    double &x() { return x_; }
    double &y() { return y_; }
    double &z() { return z_; }
};

// Stand-in with the accessor names SolverRef::solve reads (solver_ref.hpp:21-26).
struct Problem {
    std::size_t N, s_;
    double eps, G_, M_;
    unsigned p_;
    std::size_t N_() const { return N; }
    double epsilon() const { return eps; }
    double get_G() const { return G_; }
    double m() const { return M_ / static_cast<double>(N); }
    unsigned p() const { return p_; }
    std::size_t s() const { return s_; }
    double delta_t() const { return eps / std::sqrt(2.0); }  // problem.hpp:235-243
};

int failures = 0;
void expect(bool ok, const char *what) {
    std::printf("%s %s\n", ok ? "PASS" : "FAIL", what);
    if (!ok) ++failures;
}

}  // namespace

int main(int argc, char **argv) {
    const std::string dir = argc > 1 ? argv[1] : ".";  // where the checkpoint test writes its file
    using Solver = gravity::SolverGB300<double, double, double, double, double, double>;
    {  // two-body RK4 step against its closed form, via the FMM solver (root leaf: direct P2P)
        const double eps = 1e-4, d = 10.0, t = eps / std::sqrt(2.0);  // delta_t()/t == 1
        Problem pr{2, 10, eps, 1.0, 2.0, 4};
        std::vector<Vec> x{{0, 0, 0}, {d, 0, 0}}, v{{0, 0, 0}, {0, 0, 0}};
        Solver s;
        s.preprocess(pr, x, v);
        s.solve(pr, t, x, v);
        s.postprocess(pr, x, v);
        const double d2e2 = d * d + eps * eps;
        const double k1 = d / std::pow(d2e2, 1.5), l2 = k1 / 2, k2 = k1, l3 = l2;
        const double k3 = (d - l2) / std::pow((d - l2) * (d - l2) + eps * eps, 1.5), l4 = k3;
        const double k4 = (d - 2 * l3) / std::pow((d - 2 * l3) * (d - 2 * l3) + eps * eps, 1.5);
        const double xd = (2 * l2 + 2 * l3 + l4) / 6, vd = (k1 + 2 * k2 + 2 * k3 + k4) / 6;
        expect(std::fabs(x[0].x() - xd) < 1e-15 && std::fabs(x[1].x() - (d - xd)) < 1e-14, "two-body positions");
        expect(std::fabs(v[0].x() - vd) < 1e-15 && std::fabs(v[1].x() + vd) < 1e-15, "two-body velocities");
    }
    {  // Plummer sphere: three steps against the oracle's restated reference RK4
        const std::size_t n = 3000;
        Problem pr{n, 16, 0.01, 1.0, 1.0, 5};
        std::vector<vipp_oracle::V3> x3, v3;
        vipp_oracle::plummer_reference(n, pr.eps, 9, x3, v3);
        std::vector<Vec> x(n), v(n);
        for (std::size_t i = 0; i < n; ++i) x[i] = {x3[i].x, x3[i].y, x3[i].z}, v[i] = {v3[i].x, v3[i].y, v3[i].z};
        Solver s;
        s.preprocess(pr, x, v);
        const double t = 10.0;  // dt = delta_t()/10
        for (int k = 0; k < 3; ++k) s.solve(pr, t, x, v);
        s.postprocess(pr, x, v);
        for (int k = 0; k < 3; ++k)
            vipp_oracle::rk4_step(x3, v3, pr.delta_t() / t, [&](const std::vector<vipp_oracle::V3> &xx, std::vector<vipp_oracle::V3> &aa) {
                vipp_oracle::accel_fmm(xx, pr.s_, pr.G_, pr.m(), pr.eps, pr.p_, aa);
            });
        double dx = 0, dv = 0, xs = 0, vs = 0;
        for (std::size_t i = 0; i < n; ++i) {
            dx = std::fmax(dx, std::fabs(x[i].x() - x3[i].x) + std::fabs(x[i].y() - x3[i].y) + std::fabs(x[i].z() - x3[i].z));
            dv = std::fmax(dv, std::fabs(v[i].x() - v3[i].x) + std::fabs(v[i].y() - v3[i].y) + std::fabs(v[i].z() - v3[i].z));
            xs = std::fmax(xs, std::fabs(x3[i].x)), vs = std::fmax(vs, std::fabs(v3[i].x));
        }
        std::printf("plummer3000 max |dx| %.3e |dv| %.3e\n", dx, dv);
        expect(dx <= 1e-13 * xs && dv <= 1e-10 * vs, "Plummer RK4 trajectory vs oracle");
        const auto a = s.acceleration();
        expect(a.size() == 3 * n, "acceleration size");
    }
    {  // checkpoint: a solver restarted from the file written after two steps
       // continues bit-identically to the solver that wrote it
        const std::size_t n = 2000;
        Problem pr{n, 16, 0.01, 1.0, 1.0, 5};
        std::vector<vipp_oracle::V3> x3, v3;
        vipp_oracle::plummer_reference(n, pr.eps, 4, x3, v3);
        std::vector<Vec> x(n), v(n), xb(n), vb(n);
        for (std::size_t i = 0; i < n; ++i) x[i] = {x3[i].x, x3[i].y, x3[i].z}, v[i] = {v3[i].x, v3[i].y, v3[i].z};
        const std::string path = dir + "/solver_gb300.ckpt";
        const double t = 10.0, t_saved = 2 * pr.delta_t() / t;
        Solver a;
        a.preprocess(pr, x, v);
        a.solve(pr, t, x, v);
        a.solve(pr, t, x, v);
        a.save_checkpoint(path, t_saved);
        a.solve(pr, t, x, v);
        a.postprocess(pr, x, v);
        Solver b;
        const double t_loaded = b.load_checkpoint(pr, path);
        b.solve(pr, t, xb, vb);
        b.postprocess(pr, xb, vb);
        bool same = t_loaded == t_saved;
        for (std::size_t i = 0; i < n; ++i)
            same = same && x[i].x() == xb[i].x() && x[i].y() == xb[i].y() && x[i].z() == xb[i].z() &&
                   v[i].x() == vb[i].x() && v[i].y() == vb[i].y() && v[i].z() == vb[i].z();
        expect(same, "checkpoint restart bit-identical");
        std::remove(path.c_str());
    }
    {  // errors surface as std::runtime_error, like the reference's exceptions
        Problem bad{10, 0, 0.01, 1.0, 1.0, 4};  // s = 0 (problem.hpp:182-184)
        std::vector<Vec> x(10), v(10);
        bool threw = false;
        try {
            Solver s;
            s.preprocess(bad, x, v);
        } catch (const std::runtime_error &) {
            threw = true;
        }
        expect(threw, "s = 0 rejected");
        threw = false;
        try {
            Solver s;
            Problem pr{10, 4, 0.01, 1.0, 1.0, 4};
            s.solve(pr, 1.0, x, v);
        } catch (const std::runtime_error &) {
            threw = true;
        }
        expect(threw, "solve before preprocess rejected");
    }
    std::printf("%s\n", failures ? "FAILED" : "ALL PASSED");
    return failures ? 1 : 0;
}
