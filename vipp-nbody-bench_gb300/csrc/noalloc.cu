// gb_direct_accel_noalloc: the FP64 direct-sum accelerations for callers that
// cannot allocate GPU memory.
//
// Some hosts own every byte of device memory themselves: a simulation code
// with its own pool allocator, a runtime that forbids allocation once it has
// started (CUDA-graph replay loops, real-time pipelines), or a plugin that may
// only touch the buffers its host hands it. Such a caller cannot create a
// solver context (gb_create and gb_direct_accel allocate their buffers with
// cudaMalloc). This entry point takes the caller's device buffers and
// allocates nothing: the per-slice partial sums that the split-source kernel
// needs live in one file-scope device array, g_direct_scratch, of fixed size
// kNoAllocScratchDoubles doubles (16 MiB). Every GPU that loads the library
// reserves that array until the process exits.
//
// Host code cannot use the array's name as a device address (in host code it
// names a host-side stand-in), so the first call on each device looks up the
// real address with cudaGetSymbolAddress while that device is current, and
// caches it; that first call should therefore be made before any stream
// capture begins. The cache is keyed on the device's current CUDA context as
// well: after cudaDeviceReset the device gets a new context with the module
// loaded at a new address, and the next call looks the address up again.
#include <cuda.h>

#include <cmath>
#include <cstddef>
#include <cstdint>
#include <mutex>

#include "../../include/vipp_gb300.h"
#include "direct.cuh"

namespace gb {
namespace {

constexpr size_t kNoAllocScratchDoubles = size_t{1} << 21;  // 16 MiB
constexpr int kMaxDevices = 64;

static __device__ __align__(256) double g_direct_scratch[kNoAllocScratchDoubles];

struct DeviceSlot {
    double *scratch = nullptr;  // device address of g_direct_scratch on this device
    int num_sms = 0;
    CUcontext ctx = nullptr;    // the context that address belongs to
};
DeviceSlot g_slots[kMaxDevices];
std::mutex g_slots_mu;

using CtxGetCurrentFn = CUresult (*)(CUcontext *);

// The calling thread's current CUDA context (the device's primary context once
// the runtime has set it up), or nullptr when it cannot be read.
CUcontext current_context() {
    static CtxGetCurrentFn fn = [] {
        void *f = nullptr;
        cudaDriverEntryPointQueryResult q{};
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) != cudaSuccess ||
            q != cudaDriverEntryPointSuccess)
            f = nullptr;
        return reinterpret_cast<CtxGetCurrentFn>(f);
    }();
    CUcontext c = nullptr;
    if (!fn || fn(&c) != CUDA_SUCCESS) return nullptr;
    return c;
}

// Set-up, once per device and context, with that device current.
int device_slot(int dev, DeviceSlot &out) {
    if (dev < 0 || dev >= kMaxDevices) return GB_ERR_INVALID;
    // null before the runtime has made a context current: then look up (which does that) and read it after
    const CUcontext ctx = current_context();
    std::lock_guard<std::mutex> lock(g_slots_mu);
    DeviceSlot &s = g_slots[dev];
    if (!s.scratch || !ctx || s.ctx != ctx) {
        s.scratch = nullptr;
        void *p = nullptr;
        if (cudaGetSymbolAddress(&p, g_direct_scratch) != cudaSuccess || !p) return GB_ERR_CUDA;
        int sms = 0;
        if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms <= 0)
            return GB_ERR_CUDA;
        s.num_sms = sms;
        s.scratch = static_cast<double *>(p);
        s.ctx = ctx ? ctx : current_context();
    }
    out = s;
    return GB_OK;
}

}  // namespace
}  // namespace gb

extern "C" int gb_direct_accel_noalloc(const double *x_dev, size_t n, const int64_t *targets_dev, size_t ntargets,
                                       double G, double m, double eps, double *a_dev, void *stream) {
    using namespace gb;
    if (n > 0x7fffffffu || ntargets > 0x7fffffffu) return GB_ERR_INVALID;
    if (!(eps >= 0) || !std::isfinite(eps) || !std::isfinite(G) || !std::isfinite(m)) return GB_ERR_INVALID;
    const size_t nt = targets_dev ? ntargets : n;
    if (nt == 0) return GB_OK;
    if (n == 0) return GB_ERR_INVALID;  // listed targets, but no particle they could index
    if (!x_dev || !a_dev) return GB_ERR_INVALID;
    if (3 * nt > kNoAllocScratchDoubles) return GB_ERR_CAPACITY;  // more than 699,050 targets
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess) return GB_ERR_NO_DEVICE;
    // an error the caller left pending stays theirs: report it untouched
    if (cudaPeekAtLastError() != cudaSuccess) return GB_ERR_CUDA;
    DeviceSlot slot;
    const int rc = device_slot(dev, slot);
    if (rc != GB_OK) return rc;
    unsigned nsplit = direct_nsplit(static_cast<unsigned>(n), static_cast<unsigned>(nt), slot.num_sms);
    const size_t fit = kNoAllocScratchDoubles / (3 * nt);
    if (nsplit > fit) nsplit = static_cast<unsigned>(fit);
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const dim3 grid(static_cast<unsigned>((nt + kDirectTB - 1) / kDirectTB), nsplit);
    // every (slice, target) entry of the scratch is written before it is read,
    // so nothing left there by an earlier call needs clearing
    k_direct_part<AoS, true><<<grid, kDirectTB, 0, st>>>(AoS{x_dev}, static_cast<unsigned>(n),
                                                         reinterpret_cast<const long long *>(targets_dev),
                                                         static_cast<unsigned>(nt), nsplit, G * m, eps * eps, slot.scratch);
    k_direct_reduce<<<static_cast<unsigned>((nt + 255) / 256), 256, 0, st>>>(slot.scratch, static_cast<unsigned>(nt), nsplit,
                                                                             nullptr, a_dev);
    if (cudaGetLastError() != cudaSuccess) return GB_ERR_CUDA;
    return GB_OK;
}
