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
// The same streams draw the benchmark's larger synthetic workloads on the
// device: the adaptive-depth stress workload (8 Plummer clusters and a uniform
// background; no reference counterpart) and the batching form's systems
// (Plummer spheres scaled by their radius).
#include <cmath>

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

// One Plummer particle (G = M = a = 1) from stream s into x[0], x[n], x[2n]
// (and v), scaled: positions x_scale r_hat + x_off, velocities v_scale v_hat +
// v_off. False if a rejection loop ran out.
__device__ bool plummer_particle(Stream &s, double x0_max, double r_max, double x_scale, const double *x_off,
                                 double v_scale, const double *v_off, double *x, double *v, size_t n) {
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
    const double u3 = s.next(), u4 = s.next();
    xyz(r, u3, u4, x, n);
    const double u5 = s.next(), u6 = s.next();
    xyz(q * ve, u5, u6, v, n);
    for (int a = 0; a < 3; ++a) {
        x[a * n] = x_scale * x[a * n] + x_off[a];
        v[a * n] = v_scale * v[a * n] + v_off[a];
    }
    return ok && okq;
}

// The adaptive-depth stress workload: particle i below first[count] belongs
// to the cluster whose index range holds it, the rest to the uniform
// background at rest. Cluster k: a Plummer sphere of scale radius radius[k]
// and mass (its particles) / n (G = 1), radii capped at r_max scale radii,
// centred on centre[k], moving with bulk[k].
struct Clusters {
    int count;
    unsigned first[9];  // first particle of each cluster, first[count] = first background particle
    double centre[8][3], radius[8], bulk[8][3], vscale[8];
};

__global__ void k_clustered(unsigned n, uint64_t seed, double r_max, Clusters cl, double *__restrict__ x,
                            double *__restrict__ v, TreeInfo *info) {
    const unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    Stream s(seed, i);
    if (i >= cl.first[cl.count]) {  // background: uniform in [0, 1)^3, at rest
        for (int a = 0; a < 3; ++a) x[i + static_cast<size_t>(a) * n] = s.next(), v[i + static_cast<size_t>(a) * n] = 0.0;
        return;
    }
    int k = 0;
    while (k + 1 < cl.count && i >= cl.first[k + 1]) ++k;
    if (!plummer_particle(s, 1.0, r_max, cl.radius[k], cl.centre[k], cl.vscale[k], cl.bulk[k], x + i, v + i, n))
        atomicOr(&info->err, kDevNonFinite);
}

__global__ void k_plummer(unsigned n, uint64_t seed, double x0_max, double r_max, double *__restrict__ x,
                          double *__restrict__ v, TreeInfo *info, double x_scale, double v_scale) {
    const unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    Stream s(seed, i);
    const double zero[3] = {0.0, 0.0, 0.0};
    if (!plummer_particle(s, x0_max, r_max, x_scale, zero, v_scale, zero, x + i, v + i, n))
        atomicOr(&info->err, kDevNonFinite);
}

// Forest: every system's Plummer sphere in one launch. Position j of system
// s = psys[j] is particle j - seg[s] of stream family seeds[s], scaled by
// scales[s] (positions, velocities): the draws generate_plummer makes for
// that system alone.
__global__ void k_plummer_forest(unsigned n, const int *__restrict__ psys, const unsigned *__restrict__ seg,
                                 const uint64_t *__restrict__ seeds, const double2 *__restrict__ scales, double x0_max,
                                 double r_max, double *__restrict__ x, double *__restrict__ v, TreeInfo *info) {
    const unsigned j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n) return;
    const int sidx = psys[j];
    Stream s(seeds[sidx], j - seg[sidx]);
    const double zero[3] = {0.0, 0.0, 0.0};
    if (!plummer_particle(s, x0_max, r_max, scales[sidx].x, zero, scales[sidx].y, zero, x + j, v + j, n))
        atomicOr(&info->err, kDevNonFinite);
}

}  // namespace

void generate_plummer_forest(Workspace &ws, const uint64_t *seeds, const double2 *scales, double x0_max, double r_max) {
    cudaMemsetAsync(ws.info, 0, sizeof(TreeInfo), ws.st);
    k_plummer_forest<<<(ws.n + 255) / 256, 256, 0, ws.st>>>(ws.n, ws.psys, ws.seg, seeds, scales, x0_max, r_max, ws.x, ws.v,
                                                            ws.info);
    ws.launches += 1;
}

// x, v: SoA [3][n] of the context's state; positions x x_scale, velocities x v_scale.
void generate_plummer(Workspace &ws, unsigned n, uint64_t seed, double x0_max, double r_max, double x_scale,
                      double v_scale) {
    cudaMemsetAsync(ws.info, 0, sizeof(TreeInfo), ws.st);
    k_plummer<<<(n + 255) / 256, 256, 0, ws.st>>>(n, seed, x0_max, r_max, ws.x, ws.v, ws.info, x_scale, v_scale);
    ws.launches += 1;
}

// Host draws of the cluster parameters: the same SplitMix64 output function on
// a stream family of their own (the seed mixed with a constant).
namespace {
double host_uniform(uint64_t seed, uint64_t i, uint64_t k) {
    auto mix = [](uint64_t z) {
        z += 0x9e3779b97f4a7c15ull;
        z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
        z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
        return z ^ (z >> 31);
    };
    return static_cast<double>(mix(mix(seed + i) + k) >> 11) * 0x1.0p-53;
}
}  // namespace

int generate_clustered(Workspace &ws, unsigned n, uint64_t seed, int clusters, double background, double r_max,
                       double *params) {
    if (clusters < 1 || clusters > 8 || !(background >= 0 && background < 1)) return -1;
    Clusters cl{};
    cl.count = clusters;
    const unsigned n_bg = static_cast<unsigned>(std::llround(background * n));
    const unsigned n_cl = n - n_bg;
    unsigned o = 0;
    const uint64_t pseed = seed ^ 0x5bd1e995c1a5e4a3ull;
    for (int k = 0; k < clusters; ++k) {
        const unsigned m = n_cl / clusters + (static_cast<unsigned>(k) < n_cl % clusters ? 1u : 0u);
        cl.first[k] = o;
        o += m;
        for (int a = 0; a < 3; ++a) cl.centre[k][a] = host_uniform(pseed, k, a);
        cl.radius[k] = 0.01 + 0.09 * host_uniform(pseed, k, 3);
        for (int a = 0; a < 3; ++a) {  // Gaussian bulk velocity, sigma 0.3 (Box-Muller)
            const double u1 = 1.0 - host_uniform(pseed, k, 4 + 2 * a), u2 = host_uniform(pseed, k, 5 + 2 * a);
            cl.bulk[k][a] = 0.3 * std::sqrt(-2.0 * std::log(u1)) * std::cos(2.0 * 3.141592653589793 * u2);
        }
        cl.vscale[k] = std::sqrt((static_cast<double>(m) / n) / cl.radius[k]);  // G = 1, cluster mass m / n
        if (params) {
            double *q = params + 8 * k;
            for (int a = 0; a < 3; ++a) q[a] = cl.centre[k][a], q[4 + a] = cl.bulk[k][a];
            q[3] = cl.radius[k];
            q[7] = static_cast<double>(m);
        }
    }
    cl.first[clusters] = o;
    cudaMemsetAsync(ws.info, 0, sizeof(TreeInfo), ws.st);
    k_clustered<<<(n + 255) / 256, 256, 0, ws.st>>>(n, seed, r_max, cl, ws.x, ws.v, ws.info);
    ws.launches += 1;
    return 0;
}

}  // namespace gb
