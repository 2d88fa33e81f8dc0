// FP64 direct softened sum (the accuracy oracle of the GPU path;
// gravity/include/solver_ref_naive.hpp:103-119), split over sources.
//
// Few targets against many sources (the 65,536-particle error sample of a
// 4M-particle system) leave most SMs idle with one thread per target, so the
// sources are cut into `nsplit` slices: block (bx, sy) sums slice sy for 256
// targets into the scratch buffer part[sy][3][nt], and a second kernel adds
// the slices in slice order (deterministic).
//
// Position and output layouts are policies: SoA planes [3][n] (the solver
// context's own buffers) or AoS triples (caller buffers).
#pragma once

#include <cuda_runtime.h>

namespace gb {

struct SoA {
    const double *p;
    unsigned n;
    __device__ __forceinline__ double x(unsigned i) const { return p[i]; }
    __device__ __forceinline__ double y(unsigned i) const { return p[n + i]; }
    __device__ __forceinline__ double z(unsigned i) const { return p[2 * static_cast<size_t>(n) + i]; }
};

struct AoS {
    const double *p;
    __device__ __forceinline__ double x(unsigned i) const { return p[3 * static_cast<size_t>(i)]; }
    __device__ __forceinline__ double y(unsigned i) const { return p[3 * static_cast<size_t>(i) + 1]; }
    __device__ __forceinline__ double z(unsigned i) const { return p[3 * static_cast<size_t>(i) + 2]; }
};

constexpr int kDirectTB = 256;

// kCheckTargets: target indices come from device memory the host never saw;
// an index outside [0, n) is not dereferenced and its result is NaN.
template <class Pos, bool kCheckTargets = false>
__global__ void __launch_bounds__(kDirectTB) k_direct_part(Pos pos, unsigned n, const long long *__restrict__ targets,
                                                           unsigned nt, unsigned nsplit, double Gm, double eps2,
                                                           double *__restrict__ part) {
    __shared__ double sx[kDirectTB], sy[kDirectTB], sz[kDirectTB];
    const unsigned k = blockIdx.x * kDirectTB + threadIdx.x;
    bool act = k < nt;
    bool bad = false;
    long long ti = act ? (targets ? targets[k] : static_cast<long long>(k)) : 0;
    if (kCheckTargets && act && (ti < 0 || ti >= static_cast<long long>(n))) {
        bad = true;
        act = false;
        ti = 0;
    }
    const unsigned i = static_cast<unsigned>(ti);
    const double tx = act ? pos.x(i) : 0.0, ty = act ? pos.y(i) : 0.0, tz = act ? pos.z(i) : 0.0;
    const unsigned per = (n + nsplit - 1) / nsplit;
    const unsigned lo = blockIdx.y * per;
    const unsigned hi = min(n, lo + per);
    double ax = 0, ay = 0, az = 0;
    for (unsigned b = lo; b < hi; b += kDirectTB) {
        const unsigned j = b + threadIdx.x;
        if (j < hi) {
            sx[threadIdx.x] = pos.x(j);
            sy[threadIdx.x] = pos.y(j);
            sz[threadIdx.x] = pos.z(j);
        }
        __syncthreads();
        const unsigned cnt = min(static_cast<unsigned>(kDirectTB), hi - b);
        for (unsigned q = 0; q < cnt; ++q) {
            if (b + q == i) continue;  // i == j is skipped (solver_ref_naive.hpp:109-111)
            const double dx = sx[q] - tx, dy = sy[q] - ty, dz = sz[q] - tz;
            const double r2 = dx * dx + dy * dy + dz * dz + eps2;
            const double ri = rsqrt(r2);
            const double f = Gm * ri * ri * ri;
            ax += f * dx;
            ay += f * dy;
            az += f * dz;
        }
        __syncthreads();
    }
    if (act || bad) {
        if (bad) ax = ay = az = __longlong_as_double(0x7ff8000000000000LL);
        double *o = part + static_cast<size_t>(blockIdx.y) * 3 * nt;
        o[k] = ax;
        o[nt + k] = ay;
        o[2 * static_cast<size_t>(nt) + k] = az;
    }
}

// out_soa: planes [3][nt]; out_aos: triples. Exactly one of them is non-null.
static __global__ void k_direct_reduce(const double *__restrict__ part, unsigned nt, unsigned nsplit, double *__restrict__ out_soa,
                                double *__restrict__ out_aos) {
    const unsigned k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nt) return;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        double s = 0;
        for (unsigned q = 0; q < nsplit; ++q) s += part[(static_cast<size_t>(q) * 3 + a) * nt + k];
        if (out_soa)
            out_soa[static_cast<size_t>(a) * nt + k] = s;
        else
            out_aos[3 * static_cast<size_t>(k) + a] = s;
    }
}

// Source slices that fill about four waves of blocks, at least 256 sources each.
inline unsigned direct_nsplit(unsigned n, unsigned nt, int num_sms) {
    const unsigned bx = (nt + kDirectTB - 1) / kDirectTB;
    unsigned s = (4u * static_cast<unsigned>(num_sms) + bx - 1) / (bx ? bx : 1);
    const unsigned smax = n / kDirectTB > 0 ? n / kDirectTB : 1;
    if (s > smax) s = smax;
    if (s > 256) s = 256;
    return s ? s : 1;
}

}  // namespace gb
