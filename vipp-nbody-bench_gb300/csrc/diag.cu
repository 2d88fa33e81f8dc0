// Potentials and conserved quantities of the current state: diagnostics,
// run after a force evaluation and outside the RK4 step. The reference
// computes neither (its Solver has no potential); the FP64 direct sum of the
// oracle is their checker.
//
// Potential per unit mass, in the convention of the accelerations (a = -grad
// phi): phi_i = -(G m sum_near (r^2 + eps^2)^-1/2 + Phi_far,i), where the far
// part is the local expansion's potential without G, as the reference's far
// field carries no G (fmm.hpp's M2L/L2P never multiply it; G = 1 in every
// reference configuration).
#include "workspace.cuh"

namespace gb {

namespace {

constexpr int kRB = 256;      // threads per reduction block
constexpr int kRBlocks = 256;  // reduction blocks (fixed: the sums are deterministic)
constexpr int kSums = 8;

__global__ void k_phi_finalize(const unsigned *__restrict__ perm, unsigned n, const double *__restrict__ phis,
                               double gfar, double *__restrict__ phi_orig) {
    const unsigned j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n) return;
    phi_orig[perm[j]] = -(phis[j] + gfar * phis[static_cast<size_t>(n) + j]);
}

// Per block: sum |v|^2, sum phi, sum v (3), sum x cross v (3) over a fixed
// grid-stride partition, reduced in a fixed order.
__global__ void __launch_bounds__(kRB) k_conserved_partial(const double *__restrict__ x, const double *__restrict__ v,
                                                          const double *__restrict__ phi, unsigned n,
                                                          double *__restrict__ part) {
    double s[kSums] = {};
    for (unsigned i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const double px = x[i], py = x[n + i], pz = x[2 * static_cast<size_t>(n) + i];
        const double vx = v[i], vy = v[n + i], vz = v[2 * static_cast<size_t>(n) + i];
        s[0] += vx * vx + vy * vy + vz * vz;
        s[1] += phi[i];
        s[2] += vx, s[3] += vy, s[4] += vz;
        s[5] += py * vz - pz * vy, s[6] += pz * vx - px * vz, s[7] += px * vy - py * vx;
    }
    __shared__ double red[kSums][kRB / 32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
    for (int q = 0; q < kSums; ++q) {
        for (int o = 16; o; o >>= 1) s[q] += __shfl_xor_sync(0xffffffffu, s[q], o);
        if (lane == 0) red[q][w] = s[q];
    }
    __syncthreads();
    if (threadIdx.x < kSums) {
        double t = 0;
        for (int k = 0; k < kRB / 32; ++k) t += red[threadIdx.x][k];
        part[threadIdx.x * kRBlocks + blockIdx.x] = t;
    }
}

__global__ void k_conserved_final(const double *__restrict__ part, double *__restrict__ out) {
    if (threadIdx.x >= kSums) return;
    double t = 0;
    for (int b = 0; b < kRBlocks; ++b) t += part[threadIdx.x * kRBlocks + b];
    out[threadIdx.x] = t;
}

}  // namespace

size_t diag_scratch_doubles() { return kSums * kRBlocks + kSums; }

void potential_orig(Workspace &ws, double *phi_orig) {
    far_potential(ws, ws.phis + ws.n);
    if (ws.accurate) soften_phi(ws, ws.phis + ws.n);
    near_potential(ws, ws.phis);
    // the far part carries G only in the accurate mode (the reference's far field has none)
    k_phi_finalize<<<(ws.n + 255) / 256, 256, 0, ws.st>>>(ws.perm, ws.n, ws.phis, ws.accurate ? ws.G : 1.0, phi_orig);
    ws.launches += 1;
}

// sums8 (device): sum |v|^2, sum phi, sum v, sum x cross v over the caller's
// particles (original order); uses ws.diag.
void conserved_sums(Workspace &ws, const double *phi_orig, double *sums8) {
    k_conserved_partial<<<kRBlocks, kRB, 0, ws.st>>>(ws.x, ws.v, phi_orig, ws.n, ws.diag);
    k_conserved_final<<<1, 32, 0, ws.st>>>(ws.diag, sums8);
    ws.launches += 2;
}

}  // namespace gb
