// Initial conditions on the GPU: the reference's Plummer sphere
// (Problem::initialize, gravity/include/problem.hpp:188-211, 245-292) drawn
// with one counter-based random stream per particle instead of one serial
// mt19937_64, so N particles are generated in parallel. Same model, same
// steps per particle:
//   radius  r = x0^(1/3) / sqrt(1 - x0^(2/3)), x0 uniform on [0, x0_max)
//           (the inverse of the Plummer mass profile r^3 / (1 + r^2)^(3/2));
//           the reference draws x0 on [0, 1 - eps); a radius cap r <= r_max
//           instead redraws x0 on [0, 1) until r <= r_max;
//   speed   q v_e(r), v_e = sqrt(2) (r^2 + 1)^(-1/4), q accepted from uniform
//           pairs (x1, x2) when P_MAX x1 < P(x2), P(q) = q^2 (1 - q^2)^(7/2),
//           P_MAX = sqrt(7) 686 / 19683;
//   direction of both: (1 - 2 u) n, sqrt(n^2 - x^2) (cos 2 pi w, sin 2 pi w).
// Draw k of particle i is u_k = U(mix(mix(seed + i) + k)) with mix the
// SplitMix64 output function (Steele, Lea, Flood 2014; constants as
// published by Vigna) and U the top 53 bits scaled to [0, 1). Distribution
// parity with the reference is checked statistically (its mt19937_64 and
// uniform_real_distribution draws are implementation-defined anyway).
#include "workspace.cuh"

namespace gb {

namespace {

__device__ __forceinline__ uint64_t mix64(uint64_t z) {
    z += 0x9e3779b97f4a7c15ull;
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    return z ^ (z >> 31);
}

struct Stream {
    uint64_t key;
    uint64_t k = 0;
    __device__ explicit Stream(uint64_t seed, uint64_t i) : key(mix64(seed + i)) {}
    __device__ double next() { return static_cast<double>(mix64(key + k++) >> 11) * 0x1.0p-53; }
};

constexpr int kMaxTries = 1 << 12;  // rejection loops: the chance of exhausting them is below 1e-400

__device__ __forceinline__ double plummer_r(double x0) { return cbrt(x0) / sqrt(1.0 - pow(x0, 2.0 / 3.0)); }

__device__ __forceinline__ void xyz(double norm, double u, double w, double *out, size_t stride) {
    const double x = (1.0 - 2.0 * u) * norm;
    const double yz = sqrt(fmax(norm * norm - x * x, 0.0));
    double sw, cw;
    sincospi(2.0 * w, &sw, &cw);
    out[0] = x, out[stride] = yz * cw, out[2 * stride] = yz * sw;
}

__global__ void k_plummer(unsigned n, uint64_t seed, double x0_max, double r_max, double *__restrict__ x,
                          double *__restrict__ v, TreeInfo *info) {
    const unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    Stream s(seed, i);
    double r = 0;
    bool ok = false;
    if (r_max > 0) {
        for (int t = 0; t < kMaxTries && !ok; ++t) {
            r = plummer_r(s.next());
            ok = r <= r_max;
        }
    } else {
        r = plummer_r(s.next() * x0_max);
        ok = true;
    }
    const double p_max = sqrt(7.0) * 686.0 / 19683.0;
    const double ve = sqrt(2.0) * pow(r * r + 1.0, -0.25);
    double q = 0;
    bool okq = false;
    for (int t = 0; t < kMaxTries && !okq; ++t) {
        const double x1 = s.next(), x2 = s.next();
        const double om = 1.0 - x2 * x2;
        okq = p_max * x1 < x2 * x2 * om * om * om * sqrt(om);
        q = x2;
    }
    if (!ok || !okq) atomicOr(&info->err, kDevNonFinite);
    const double u3 = s.next(), u4 = s.next();
    xyz(r, u3, u4, x + i, n);
    const double u5 = s.next(), u6 = s.next();
    xyz(q * ve, u5, u6, v + i, n);
}

}  // namespace

// x, v: SoA [3][n] of the context's state.
void generate_plummer(Workspace &ws, unsigned n, uint64_t seed, double x0_max, double r_max) {
    cudaMemsetAsync(ws.info, 0, sizeof(TreeInfo), ws.st);
    k_plummer<<<(n + 255) / 256, 256, 0, ws.st>>>(n, seed, x0_max, r_max, ws.x, ws.v, ws.info);
    ws.launches += 1;
}

}  // namespace gb
