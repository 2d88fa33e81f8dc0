// CPU check of the operator algebra used by the CUDA kernels.
//
// Runs one FMM force evaluation on the CPU with the library's own host+device
// math (csrc/harmonics.cuh: solid-harmonic recurrences, scaled real-basis
// M2M/M2L/L2L matrices, ladder-operator L2P) on the oracle's tree and lists,
// and prints the largest relative difference of the accelerations from the
// oracle's restatement of the reference (oracle/oracle.hpp). Also checks the
// recurrence against the oracle's Y_n^m. Built and run by
// tests/test_operator_algebra.py.
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "../oracle/oracle.hpp"
#include "../vipp-nbody-bench_gb300/csrc/harmonics.cuh"

using namespace vipp_oracle;

int main(int argc, char **argv) {
    const std::size_t N = argc > 1 ? std::strtoul(argv[1], nullptr, 10) : 3000;
    const std::size_t s = argc > 2 ? std::strtoul(argv[2], nullptr, 10) : 8;
    const int p = argc > 3 ? std::atoi(argv[3]) : 4;
    const double eps = 0.01;
    std::vector<V3> x, v;
    plummer_reference(N, eps, 7, x, v);
    const double mass = 1.0 / static_cast<double>(N);

    static gb::HTab<double> H;
    static gb::ATab At;
    gb::fill_tables(H, At);

    // 1. Recurrence vs the oracle's Y_n^m (series form of the reference).
    double yerr = 0;
    {
        const double u[3] = {0.3, -0.7, 0.45};
        double r, th, ph;
        polar(V3{u[0], u[1], u[2]}, r, th, ph);
        SphHarm Y(2 * p, th, ph);
        std::vector<double> R((2 * p + 1) * (2 * p + 1));
        gb::solid_regular_rt<double>(2 * p, u[0], u[1], u[2], H, R.data());
        for (int n = 0; n <= 2 * p; ++n)
            for (int m = 0; m <= n; ++m) {
                const cd ref = Y(static_cast<unsigned>(n), m) * std::pow(r, n);
                const double re = R[gb::ridx(n, m, 0)], im = m ? R[gb::ridx(n, m, 1)] : 0.0;
                yerr = std::max(yerr, std::abs(cd(re, im) - ref) / std::max(1e-300, std::abs(ref) + 1e-3));
            }
    }

    // 2. FMM with the library's operators on the oracle's tree and lists.
    Tree t(x, s);
    Lists ls(t);
    const std::size_t nc = t.cells.size();
    const int K = (p + 1) * (p + 1);
    const double Hx[3] = {t.cells[0].mx.x - t.cells[0].mn.x, t.cells[0].mx.y - t.cells[0].mn.y,
                          t.cells[0].mx.z - t.cells[0].mn.z};
    const double S = std::max(Hx[0], std::max(Hx[1], Hx[2]));
    // integer coordinates (1 = upper half)
    std::vector<std::array<long long, 3>> coord(nc);
    for (std::size_t c = 1; c < nc; ++c) {
        const unsigned o = t.octant(c);
        const auto &pc = coord[static_cast<std::size_t>(t.cells[c].parent)];
        for (int a = 0; a < 3; ++a) coord[c][a] = 2 * pc[a] + (((o >> a) & 1) ? 0 : 1);
    }
    auto build_op = [&](int kind, const double tv[3], std::vector<double> &op) {
        const double rho = std::sqrt(tv[0] * tv[0] + tv[1] * tv[1] + tv[2] * tv[2]);
        const int D = kind == 0 ? 2 * p : p;
        std::vector<double> yt((D + 1) * (D + 1));
        gb::solid_regular_rt<double>(D, tv[0] / rho, tv[1] / rho, tv[2] / rho, H, yt.data());
        std::vector<double> pw(2 * p + 3);
        for (int i = 0; i < 2 * p + 3; ++i) pw[i] = kind == 0 ? std::pow(1.0 / rho, i) : std::pow(rho, i);
        op.assign(K * K, 0.0);
        for (int ro = 0; ro < K; ++ro)
            for (int ri = 0; ri < K; ++ri) {
                int j, k, po, n, m, pi;
                gb::rdecode(ro, j, k, po);
                gb::rdecode(ri, n, m, pi);
                op[ro * K + ri] = gb::real_entry(kind, At, yt.data(), pw.data(), j, k, po, n, m, pi);
            }
    };
    std::vector<std::vector<double>> M(nc, std::vector<double>(K, 0.0)), L(nc, std::vector<double>(K, 0.0));
    std::vector<double> m2m_op[8], l2l_op[8];
    for (unsigned o = 0; o < 8; ++o) {
        double tv[3];
        for (int a = 0; a < 3; ++a) tv[a] = (((o >> a) & 1) ? -1.0 : 1.0) * Hx[a] / S / 4;
        build_op(1, tv, m2m_op[o]);
        double tl[3] = {-tv[0], -tv[1], -tv[2]};
        build_op(2, tl, l2l_op[o]);
    }
    std::vector<std::vector<double>> m2l_op(343);
    std::vector<double> Rb(K);
    // upward
    for (int lv = t.max_level; lv >= 2; --lv)
        for (std::size_t c = 0; c < nc; ++c) {
            if (t.cells[c].level != lv) continue;
            const double sL = S * std::ldexp(1.0, -lv);
            if (t.cells[c].leaf()) {
                const V3 ctr = t.cells[c].center();
                for (long long i : t.cells[c].pts) {
                    const V3 u = sub(x[static_cast<std::size_t>(i)], ctr);
                    gb::solid_regular_rt<double>(p, u.x / sL, u.y / sL, u.z / sL, H, Rb.data());
                    for (int r = 0; r < K; ++r) {
                        int n, m, part;
                        gb::rdecode(r, n, m, part);
                        M[c][r] += mass * (part ? -Rb[r] : Rb[r]);
                    }
                }
            } else {
                for (unsigned o = 0; o < 8; ++o) {
                    const auto &ch = M[static_cast<std::size_t>(t.cells[c].first_child) + o];
                    for (int ro = 0; ro < K; ++ro)
                        for (int ri = 0; ri < K; ++ri) M[c][ro] += m2m_op[o][ro * K + ri] * ch[ri];
                }
            }
        }
    // M2L
    for (std::size_t c = 9; c < nc; ++c)
        for (long long q : ls.m2l[c]) {
            const std::size_t qi = static_cast<std::size_t>(q);
            int d[3];
            for (int a = 0; a < 3; ++a) d[a] = static_cast<int>(coord[qi][a] - coord[c][a]);
            const int oi = (d[0] + 3) + 7 * (d[1] + 3) + 49 * (d[2] + 3);
            if (m2l_op[oi].empty()) {
                double tv[3];
                for (int a = 0; a < 3; ++a) tv[a] = d[a] * Hx[a] / S;
                build_op(0, tv, m2l_op[oi]);
            }
            for (int ro = 0; ro < K; ++ro)
                for (int ri = 0; ri < K; ++ri) L[c][ro] += m2l_op[oi][ro * K + ri] * M[qi][ri];
        }
    // downward + evaluation
    std::vector<V3> a(N, V3{0, 0, 0});
    const double Gm = mass;
    for (std::size_t c = 0; c < nc; ++c)
        if (t.cells[c].leaf()) p2p(t, c, ls.p2p[c], x, a, Gm, eps);
    for (int lv = 2; lv <= t.max_level; ++lv)
        for (std::size_t c = 0; c < nc; ++c) {
            if (t.cells[c].level != lv) continue;
            if (lv >= 3) {
                const unsigned o = t.octant(c);
                const auto &par = L[static_cast<std::size_t>(t.cells[c].parent)];
                for (int ro = 0; ro < K; ++ro)
                    for (int ri = 0; ri < K; ++ri) L[c][ro] += l2l_op[o][ro * K + ri] * par[ri];
            }
            if (!t.cells[c].leaf()) continue;
            const double sL = S * std::ldexp(1.0, -lv);
            const V3 ctr = t.cells[c].center();
            for (long long i : t.cells[c].pts) {
                const V3 u = sub(x[static_cast<std::size_t>(i)], ctr);
                gb::solid_regular_rt<double>(p, u.x / sL, u.y / sL, u.z / sL, H, Rb.data());
                double gre = 0, gim = 0, gz = 0;
                const auto &Lc = L[c];
                for (int j = 1; j <= p; ++j)
                    for (int k = 0; k <= j; ++k) {
                        const double lr = Lc[gb::ridx(j, k, 0)], li = k ? Lc[gb::ridx(j, k, 1)] : 0.0;
                        // d/dz
                        if (k <= j - 1) {
                            const double rr = Rb[gb::ridx(j - 1, k, 0)], ri = k ? Rb[gb::ridx(j - 1, k, 1)] : 0.0;
                            const double w = H.lz[j][k] * (k ? 2.0 : 1.0);
                            gz += w * (lr * rr - li * ri);
                        }
                        // (d/dx + i d/dy): L R_{j-1}^{k+1} term
                        if (k + 1 <= j - 1) {
                            const double rr = Rb[gb::ridx(j - 1, k + 1, 0)], ri = Rb[gb::ridx(j - 1, k + 1, 1)];
                            gre += H.lp[j][k] * (lr * rr - li * ri);
                            gim += H.lp[j][k] * (lr * ri + li * rr);
                        }
                        // - conj(L) conj(R_{j-1}^{k-1}) term
                        if (k >= 1) {
                            const double rr = Rb[gb::ridx(j - 1, k - 1, 0)], ri = (k - 1) ? Rb[gb::ridx(j - 1, k - 1, 1)] : 0.0;
                            gre -= H.lm[j][k] * (lr * rr - li * ri);
                            gim -= H.lm[j][k] * (-(lr * ri + li * rr));
                        }
                    }
                const double sc = 1.0 / (sL * sL);
                V3 &ai = a[static_cast<std::size_t>(i)];
                ai.x += gre * sc, ai.y += gim * sc, ai.z += gz * sc;
            }
        }
    std::vector<V3> aref;
    accel_fmm(x, s, 1.0, mass, eps, static_cast<unsigned>(p), aref);
    double maxrel = 0, rms = 0;
    for (std::size_t i = 0; i < N; ++i) {
        const V3 d = sub(a[i], aref[i]);
        const double rel = std::sqrt(norm2(d) / norm2(aref[i]));
        maxrel = std::max(maxrel, rel);
        rms += rel * rel;
    }
    std::printf("yerr %.3e maxrel %.3e rms %.3e cells %zu depth %d\n", yerr, maxrel, std::sqrt(rms / N), nc, t.max_level);
    return 0;
}
