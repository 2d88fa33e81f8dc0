// Classical RK4 combination in FP64 (gravity/include/solver_ref.hpp:36-112)
// and the AoS <-> SoA layout conversions at the host boundary.
//
// After force evaluation k (k = 0..3) of a step, with v the stage velocity
// and a the stage acceleration:
//   xo += w_k v,  vo += w_k a            (w = dt/6, dt/3, dt/3, dt/6;
//                                         k = 0 starts them: xo = x0 + w_0 v)
//   k < 3: x = x0 + v c_k, v = v0 + a c_k (c = dt/2, dt/2, dt; x uses the old v)
//   k = 3: x = xo, v = vo
// Products and sums are issued as separate round-to-nearest operations
// (__dmul_rn/__dadd_rn) so no FMA contraction changes the reference's
// rounding: given the same accelerations the step is bit-identical.
#include "workspace.cuh"

namespace gb {

namespace {

// The step's start state. The accumulators xo, vo are started by stage 0
// from x0, v0 (not here), so a step repeated after a capacity overflow, which
// restores x, v from x0, v0 and runs all four stages again, does not add its
// stage sums to the failed attempt's.
__global__ void k_rk4_begin(const double *__restrict__ x, const double *__restrict__ v, double *__restrict__ x0,
                            double *__restrict__ v0, size_t n3) {
    for (size_t e = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; e < n3; e += static_cast<size_t>(gridDim.x) * blockDim.x)
        x0[e] = x[e], v0[e] = v[e];
}

// The stage's acceleration is read where the force evaluation left it, in
// tree order, through the inverse permutation: a = near[j] + far[j] with
// j = inv[i], added in T exactly as the accelerations returned to the caller
// are (finalize); the state is SoA in particle order. Small systems read the
// six [3][N] planes directly; large ones read one packed sum per particle
// (near_far_sum: float4, or three doubles), one sector instead of six.
template <typename T, bool kPacked>
__global__ void k_rk4_stage(int stage, double w, double c, double *__restrict__ x, double *__restrict__ v,
                            const double *__restrict__ x0, const double *__restrict__ v0, double *__restrict__ xo,
                            double *__restrict__ vo, const unsigned *__restrict__ inv, const T *__restrict__ nearv,
                            const T *__restrict__ farv, const T *__restrict__ packed, size_t n) {
    constexpr int kStride = sizeof(T) == 4 ? 4 : 3;  // packed layout: float4, or three doubles
    for (size_t i = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; i < n; i += static_cast<size_t>(gridDim.x) * blockDim.x) {
        const size_t j = inv[i];
        T av[3];
        if (kPacked && sizeof(T) == 4) {
            const float4 q = reinterpret_cast<const float4 *>(packed)[j];
            av[0] = q.x, av[1] = q.y, av[2] = q.z;
        } else {
#pragma unroll
            for (int k = 0; k < 3; ++k) av[k] = kPacked ? packed[kStride * j + k] : nearv[k * n + j] + farv[k * n + j];
        }
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            const size_t e = k * n + i;
            const double ve = v[e], ae = static_cast<double>(av[k]);
            const double xoe = __dadd_rn(stage == 0 ? x0[e] : xo[e], __dmul_rn(w, ve));
            const double voe = __dadd_rn(stage == 0 ? v0[e] : vo[e], __dmul_rn(w, ae));
            xo[e] = xoe, vo[e] = voe;
            if (stage < 3) {
                x[e] = __dadd_rn(x0[e], __dmul_rn(ve, c));
                v[e] = __dadd_rn(v0[e], __dmul_rn(ae, c));
            } else {
                x[e] = xoe;
                v[e] = voe;
            }
        }
    }
}

// packed[j] = near[j] + far[j] in tree order (coalesced), for the stage's
// permuted reads of large systems
template <typename T>
__global__ void k_near_far_sum(const T *__restrict__ nearv, const T *__restrict__ farv, T *__restrict__ packed, size_t n) {
    for (size_t j = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; j < n; j += static_cast<size_t>(gridDim.x) * blockDim.x) {
        T a[3];
#pragma unroll
        for (int k = 0; k < 3; ++k) a[k] = nearv[k * n + j] + farv[k * n + j];
        if (sizeof(T) == 4)
            reinterpret_cast<float4 *>(packed)[j] = make_float4(a[0], a[1], a[2], 0.f);
        else
#pragma unroll
            for (int k = 0; k < 3; ++k) packed[3 * j + k] = a[k];
    }
}

__global__ void k_restore(double *__restrict__ x, double *__restrict__ v, const double *__restrict__ x0,
                          const double *__restrict__ v0, size_t n3) {
    for (size_t e = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; e < n3; e += static_cast<size_t>(gridDim.x) * blockDim.x)
        x[e] = x0[e], v[e] = v0[e];
}

__global__ void k_aos_to_soa(const double *__restrict__ aos, double *__restrict__ soa, unsigned n) {
    const unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
#pragma unroll
    for (int a = 0; a < 3; ++a) soa[static_cast<size_t>(a) * n + i] = aos[3 * static_cast<size_t>(i) + a];
}

__global__ void k_soa_to_aos(const double *__restrict__ soa, double *__restrict__ aos, unsigned n) {
    const unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
#pragma unroll
    for (int a = 0; a < 3; ++a) aos[3 * static_cast<size_t>(i) + a] = soa[static_cast<size_t>(a) * n + i];
}

inline unsigned grid_stride_blocks(const Workspace &ws) { return static_cast<unsigned>(ws.num_sms) * 8; }

// From this size on the stage reads packed near + far sums (an extra pass that
// saves the five other sectors each permuted read would touch).
constexpr unsigned kPackedStageMin = 1u << 16;

}  // namespace

void rk4_begin(Workspace &ws) {
    k_rk4_begin<<<grid_stride_blocks(ws), 256, 0, ws.st>>>(ws.x, ws.v, ws.x0, ws.v0, 3 * static_cast<size_t>(ws.n));
    ws.launches += 1;
}

void rk4_stage(Workspace &ws, int stage, double dt) {
    timer_begin(ws, kTRK4);
    // weights and stage offsets exactly as solver_ref.hpp:58, 64, 71, 77, 84, 90, 97
    const double w = (stage == 0 || stage == 3) ? dt / 6 : dt / 3;
    const double c = stage < 2 ? dt / 2 : dt;
    // large systems: the near + far sums packed per particle in the acc buffer
    // (free during steps), then one permuted read per particle
    const bool packed = ws.n >= kPackedStageMin;
    const size_t n = ws.n;
    if (ws.mixed) {
        const float *nf = static_cast<const float *>(ws.nearf), *ff = static_cast<const float *>(ws.farf);
        float *pk = reinterpret_cast<float *>(ws.acc);
        if (packed) {
            k_near_far_sum<float><<<grid_stride_blocks(ws), 256, 0, ws.st>>>(nf, ff, pk, n);
            k_rk4_stage<float, true><<<grid_stride_blocks(ws), 256, 0, ws.st>>>(stage, w, c, ws.x, ws.v, ws.x0, ws.v0, ws.xo, ws.vo,
                                                                               ws.inv, nf, ff, pk, n);
        } else {
            k_rk4_stage<float, false><<<grid_stride_blocks(ws), 256, 0, ws.st>>>(stage, w, c, ws.x, ws.v, ws.x0, ws.v0, ws.xo,
                                                                                ws.vo, ws.inv, nf, ff, pk, n);
        }
    } else {
        const double *nf = static_cast<const double *>(ws.nearf), *ff = static_cast<const double *>(ws.farf);
        double *pk = ws.acc;
        if (packed) {
            k_near_far_sum<double><<<grid_stride_blocks(ws), 256, 0, ws.st>>>(nf, ff, pk, n);
            k_rk4_stage<double, true><<<grid_stride_blocks(ws), 256, 0, ws.st>>>(stage, w, c, ws.x, ws.v, ws.x0, ws.v0, ws.xo,
                                                                                ws.vo, ws.inv, nf, ff, pk, n);
        } else {
            k_rk4_stage<double, false><<<grid_stride_blocks(ws), 256, 0, ws.st>>>(stage, w, c, ws.x, ws.v, ws.x0, ws.v0, ws.xo,
                                                                                 ws.vo, ws.inv, nf, ff, pk, n);
        }
    }
    if (packed) ws.launches += 1;
    ws.launches += 1;
    timer_end(ws, kTRK4);
}

void rk4_restore(Workspace &ws) {
    k_restore<<<grid_stride_blocks(ws), 256, 0, ws.st>>>(ws.x, ws.v, ws.x0, ws.v0, 3 * static_cast<size_t>(ws.n));
    ws.launches += 1;
}

void aos_to_soa(Workspace &ws, const double *aos, double *soa, unsigned n) {
    if (!n) return;
    k_aos_to_soa<<<(n + 255) / 256, 256, 0, ws.st>>>(aos, soa, n);
    ws.launches += 1;
}

void soa_to_aos(Workspace &ws, const double *soa, double *aos, unsigned n) {
    if (!n) return;
    k_soa_to_aos<<<(n + 255) / 256, 256, 0, ws.st>>>(soa, aos, n);
    ws.launches += 1;
}

}  // namespace gb
