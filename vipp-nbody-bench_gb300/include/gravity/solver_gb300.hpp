// gravity::SolverGB300 — header-only drop-in for the reference's Solver
// concept (gravity/include/solver.hpp:6-9, solver_ref.hpp:11-27), backed by
// the GB300 C-ABI (include/vipp_gb300.h, libvipp_gb300.so).
//
// Switch a reference build over by changing the alias in solver.hpp:
//
//     #include <gravity/solver_gb300.hpp>
//     template <class M, class T, class X, class V, class A, class G>
//     using Solver = SolverGB300<M, T, X, V, A, G>;
//
// Semantics follow SolverRef:
//   preprocess(problem, x, v)   copies the particles to the GPU (creates the
//                               context on first use; reads p, s, epsilon,
//                               get_G and m from the problem)
//   solve(problem, t, x, v)     one classical RK4 step of size
//                               problem.delta_t() / t on the GPU
//   postprocess(problem, x, v)  copies positions and velocities back into x, v
// Only solve is timed by the reference's benchmark (benchmark.hpp:123-128), so
// the host<->device copies sit in pre/postprocess. Errors are thrown as
// std::runtime_error, as the reference does.
//
// Template parameters are the reference's six types. Arithmetic on the GPU is
// FP64 (GB_PREC_FP64) by default, or the mixed pipeline (GB_PREC_MIXED) via
// the seventh parameter; the eighth selects the method (GB_MODE_REF, the
// reference's, by default; GB_MODE_ACCURATE adds the softened far field).
// Positions and velocities cross the boundary as doubles whatever X and V are.
#ifndef GRAVITY_SOLVER_GB300_HPP
#define GRAVITY_SOLVER_GB300_HPP

#include <cstddef>
#include <stdexcept>
#include <string>
#include <vector>

#include "vipp_gb300.h"

namespace gravity {

template <class M, class T, class X, class V, class A, class G, int Precision = GB_PREC_FP64, int Mode = GB_MODE_REF>
struct SolverGB300 final {
    SolverGB300() = default;
    explicit SolverGB300(int device) : device_(device) {}
    SolverGB300(const SolverGB300 &) = delete;
    SolverGB300 &operator=(const SolverGB300 &) = delete;
    ~SolverGB300() {
        if (ctx_) gb_destroy(ctx_);
    }

    template <class Problem, class PX, class PV>
    void preprocess(const Problem &problem, const std::vector<PX> &x, const std::vector<PV> &v) {
        if (x.size() != v.size()) throw std::runtime_error("x and v differ in length");
        configure(problem);
        n_ = x.size();
        pack(x, bx_);
        pack(v, bv_);
        check(gb_upload(ctx_, bx_.data(), bv_.data(), n_));
    }

    template <class Problem, class PX, class PV>
    void solve(const Problem &problem, const T t, std::vector<PX> &x, std::vector<PV> &v) {
        if (!ctx_ || x.size() != n_ || v.size() != n_) throw std::runtime_error("solve before preprocess");
        configure(problem);
        check(gb_rk4_step(ctx_, static_cast<double>(problem.delta_t() / t)));
    }

    template <class Problem, class PX, class PV>
    void postprocess(const Problem &, std::vector<PX> &x, std::vector<PV> &v) {
        if (!ctx_) throw std::runtime_error("postprocess before preprocess");
        bx_.resize(3 * n_);
        bv_.resize(3 * n_);
        check(gb_download(ctx_, bx_.data(), bv_.data()));
        unpack(bx_, x);
        unpack(bv_, v);
    }

    // One force evaluation at the uploaded positions (SolverRef::acceleration).
    std::vector<double> acceleration() {
        std::vector<double> a(3 * n_);
        check(gb_accel(ctx_, a.data(), nullptr));
        return a;
    }

    // Checkpoint of the current state with simulated time t (gb_checkpoint_save).
    void save_checkpoint(const std::string &path, double t = 0) {
        if (!ctx_) throw std::runtime_error("save_checkpoint before preprocess");
        check(gb_checkpoint_save(ctx_, path.c_str(), t));
    }

    // Restart from a checkpoint: configures the context from problem, as
    // preprocess does, and loads the saved state and step count (the file's
    // configuration must match); returns the saved time. postprocess then
    // gives the saved state.
    template <class Problem>
    double load_checkpoint(const Problem &problem, const std::string &path) {
        configure(problem);
        double t = 0;
        check(gb_checkpoint_load(ctx_, path.c_str(), 0, &t));
        gb_stats st{};
        check(gb_get_stats(ctx_, &st));
        n_ = static_cast<std::size_t>(st.n);
        return t;
    }

    gb_ctx *context() const { return ctx_; }

  private:
    template <class Problem>
    void configure(const Problem &problem) {
        gb_config c{};
        c.p = static_cast<int>(problem.p());
        c.s = static_cast<int>(problem.s());
        c.eps = static_cast<double>(problem.epsilon());
        c.G = static_cast<double>(problem.get_G());
        c.m = static_cast<double>(problem.m());
        c.precision = Precision;
        c.device = device_;
        c.flags = 0;
        c.mode = Mode;
        if (!ctx_) {
            gb_ctx *h = nullptr;
            const int rc = gb_create(&c, &h);
            if (rc != GB_OK) throw std::runtime_error(std::string("gb_create: ") + gb_last_error(nullptr));
            ctx_ = h;
        } else if (c.p != cfg_.p || c.s != cfg_.s || c.eps != cfg_.eps || c.G != cfg_.G || c.m != cfg_.m) {
            check(gb_set_config(ctx_, &c));
        }
        cfg_ = c;
    }

    template <class P>
    static void pack(const std::vector<P> &src, std::vector<double> &dst) {
        dst.resize(3 * src.size());
        for (std::size_t i = 0; i < src.size(); ++i) {
            dst[3 * i] = static_cast<double>(src[i].x());
            dst[3 * i + 1] = static_cast<double>(src[i].y());
            dst[3 * i + 2] = static_cast<double>(src[i].z());
        }
    }

    template <class P>
    static void unpack(const std::vector<double> &src, std::vector<P> &dst) {
        using C = decltype(dst[0].x() + 0);
        for (std::size_t i = 0; i < dst.size(); ++i) {
            dst[i].x() = static_cast<C>(src[3 * i]);
            dst[i].y() = static_cast<C>(src[3 * i + 1]);
            dst[i].z() = static_cast<C>(src[3 * i + 2]);
        }
    }

    void check(int rc) const {
        if (rc != GB_OK) throw std::runtime_error(std::string("vipp_gb300: ") + gb_last_error(ctx_));
    }

    gb_ctx *ctx_ = nullptr;
    gb_config cfg_{};
    int device_ = 0;
    std::size_t n_ = 0;
    std::vector<double> bx_, bv_;
};

}  // namespace gravity

#endif  // GRAVITY_SOLVER_GB300_HPP
