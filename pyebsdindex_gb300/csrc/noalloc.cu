// ebsd_find_bands_static: band detection that allocates no memory.
//
// Who needs this: callers that may not call cudaMalloc themselves or let a library do it --
// an application whose device memory is owned by its framework's pool allocator (raw
// cudaMalloc/cudaFree outside the pool is forbidden, and the pool cannot hand a C library a
// plan-lifetime workspace), and streaming acquisition loops that must keep a fixed device
// footprint after start-up because cudaMalloc/cudaFree can synchronise the device and stall
// the detector.  For them this entry point runs the per-stage FP32 path (EBSD_PLAIN_F32, the
// same kernels as ebsd_find_bands) with its scratch -- the padded Radon image, LoG image,
// theta-dilated image, peak flags and per-pattern statistics -- in a fixed, file-scope
// device array instead of the plan's cudaMalloc'ed workspace.
//
// Limits and rules, stated once here and in include/ebsdgpu.h:
//   * The array is kStaticScratchBytes = 64 MiB.  One call handles at most
//     floor((64 MiB - 1 KiB - 4*ksz_rho*ksz_theta) / bytes_per_pattern) patterns, where
//     bytes_per_pattern = 12 * (nRho + 2*pad_rho) * (nTheta + 2*pad_theta) + nRho*nTheta + 8
//     (80x80 patterns with nRho 120, nTheta 180, padding 11: 366 KB per pattern, at most 183
//     patterns per call); larger requests return EBSD_E_SCRATCH and touch nothing.
//   * Every GPU that loads this library holds the 64 MiB until the process exits.
//   * The device address of the array is looked up with cudaGetSymbolAddress the first time
//     the entry point runs on a device (with that device current) and cached; make that
//     first call on each device before any stream capture.
//   * The caller's current device is left as it was: the call switches to the plan's device
//     for its own work and switches back on every return.
//   * All calls share the one array per device and the kernels overwrite every scratch cell
//     they read before reading it, so nothing needs clearing between calls; two calls whose
//     work overlaps on the GPU (different streams, or different host threads) race on the
//     array and corrupt each other's results.  Serialise them.
#include "ebsd_internal.cuh"

#include <mutex>

namespace {

constexpr size_t kStaticScratchBytes = (size_t)64 << 20;
constexpr int kMaxDevices = 64;

static __device__ __align__(256) unsigned char g_static_scratch[kStaticScratchBytes];

std::mutex g_scratch_mtx;
void* g_scratch_addr[kMaxDevices] = {};

// Device address of g_static_scratch on the current device (set-up once per device).
int scratch_address(int device, void** out) {
    if (device < 0 || device >= kMaxDevices) return EBSD_E_DEVICE;
    std::lock_guard<std::mutex> lk(g_scratch_mtx);
    if (!g_scratch_addr[device]) {
        void* ptr = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&ptr, g_static_scratch);
        if (e != cudaSuccess || ptr == nullptr) return EBSD_E_LAUNCH;
        g_scratch_addr[device] = ptr;
    }
    *out = g_scratch_addr[device];
    return EBSD_OK;
}

// Keeps the caller's current device: switches to the plan's device for the call's lifetime.
struct DeviceGuard {
    int saved = -1;
    bool ok = false;
    explicit DeviceGuard(int device) {
        if (cudaGetDevice(&saved) != cudaSuccess) return;
        ok = saved == device || cudaSetDevice(device) == cudaSuccess;
    }
    ~DeviceGuard() {
        if (saved >= 0) cudaSetDevice(saved);
    }
};

}  // namespace

extern "C" int ebsd_find_bands_static(ebsd_plan_t p, int dtype, const void* d_pats, int64_t n,
                                      const ebsd_bands* d_out, void* stream) {
    if (!p || !d_out || n < 0) return EBSD_E_ARG;
    if (n > 0 && !d_pats) return EBSD_E_ARG;
    if (dtype != EBSD_U8 && dtype != EBSD_U16 && dtype != EBSD_F32) return EBSD_E_DTYPE;
    if (!d_out->max || !d_out->normmax || !d_out->maxloc || !d_out->avemax || !d_out->aveloc ||
        !d_out->width || !d_out->theta || !d_out->rho || !d_out->valid)
        return EBSD_E_ARG;
    if (n == 0) return EBSD_OK;
    if (n > 65535 || ebsd::plain_workspace_bytes(p, EBSD_PLAIN_F32, n) > kStaticScratchBytes)
        return EBSD_E_SCRATCH;
    DeviceGuard guard(p->device);
    if (!guard.ok) return EBSD_E_DEVICE;
    void* scratch = nullptr;
    int rc = scratch_address(p->device, &scratch);
    if (rc != EBSD_OK) return rc;
    int64_t launches = 0;
    return ebsd::plain_run_chunk_ws(p, EBSD_PLAIN_F32, dtype, d_pats, n, d_out, 0,
                                    (cudaStream_t)stream, &launches, scratch);
}
