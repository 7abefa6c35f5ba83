// wrs_noalloc.cu -- an inclusive prefix sum that allocates no device memory.
//
// wrs_prefix_sum needs a wrs_buffers object, i.e. one cudaMalloc, for the lookback state of
// its single-pass scan.  Some callers cannot allocate at all: code that runs inside a host
// application whose memory pool has already reserved all device memory, code on a path where
// the device-wide synchronisation of cudaMalloc/cudaFree is not acceptable, or code called
// from inside another allocator or a driver callback, where calling back into the CUDA
// allocator is not allowed.  wrs_prefix_sum_noalloc serves them: its scratch (the control
// block, the per-tile total-mass partials of the compensated mode and the double-buffered
// lookback states) is a fixed-size array in this library's own device memory, sized for up
// to kNoAllocMaxN weights.  The array is a file-scope __device__ variable, so every GPU that
// loads the library holds it (about 1.2 MiB) until the process exits.
#include <cstring>
#include <mutex>
#include <string>

#include "../../include/wrs.h"
#include "wrs_device.cuh"
#include "wrs_internal.cuh"

using namespace wrs;

namespace {

constexpr uint32_t kNoAllocMaxN = 1u << 26;  // 67,108,864 weights
constexpr uint32_t kNoAllocTiles = (kNoAllocMaxN + kTileItems - 1) / kTileItems + 1;
constexpr size_t kNoAllocPartialsOffset = sizeof(BuildCtrl);
constexpr size_t kNoAllocStatesOffset =
    (kNoAllocPartialsOffset + kNoAllocTiles * sizeof(double) + 255) / 256 * 256;
constexpr size_t kNoAllocBytes = kNoAllocStatesOffset + 2ull * kNoAllocTiles * sizeof(ScanState);

static_assert(kNoAllocStatesOffset % alignof(ScanState) == 0, "state alignment");

// The scratch itself.  In host code this name is only a handle for the runtime; the device
// address is looked up with cudaGetSymbolAddress (below).
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];

constexpr int kMaxDevices = 64;
std::mutex g_mutex;
void* g_scratch_ptr[kMaxDevices] = {};

wrs_status fail(wrs_status s, const char* msg) {
    set_last_error(s, msg);
    return s;
}

// Device address of the scratch on the current device, looked up once per device.
cudaError_t scratch_address(void** out) {
    int dev = -1;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lock(g_mutex);
    if (!g_scratch_ptr[dev]) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) return e;
        g_scratch_ptr[dev] = p;
    }
    *out = g_scratch_ptr[dev];
    return cudaSuccess;
}

}  // namespace

extern "C" wrs_status wrs_prefix_sum_noalloc(void* stream, const float* in, uint32_t n,
                                             float* out, uint32_t scan_precision,
                                             uint32_t* device_status) {
    if (!in || !out) return fail(WRS_ERR_INVALID_ARG, "NULL argument");
    if (n == 0) return fail(WRS_ERR_INVALID_ARG, "n must be >= 1");
    if (n > kNoAllocMaxN)
        return fail(WRS_ERR_CAPACITY,
                              "n exceeds the 67108864 (2^26) weights the no-allocation scratch "
                              "holds; use wrs_prefix_sum with a wrs_buffers object");
    if (scan_precision > WRS_SCAN_FLOAT_FLOAT)
        return fail(WRS_ERR_INVALID_ARG, "unknown scan precision");
    const cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    void* base = nullptr;
    if (scratch_address(&base) != cudaSuccess)
        return fail(WRS_ERR_CUDA, "cudaGetSymbolAddress of the scratch failed");
    BuildCtrl* ctrl = static_cast<BuildCtrl*>(base);
    double* partials =
        reinterpret_cast<double*>(static_cast<unsigned char*>(base) + kNoAllocPartialsOffset);
    ScanState* states =
        reinterpret_cast<ScanState*>(static_cast<unsigned char*>(base) + kNoAllocStatesOffset);
    // The array keeps whatever the previous call left.  Zero the control block (tickets,
    // epoch, mass counter, status) and the half of the states this launch uses (epoch 0 ->
    // first half); the partials need no clearing.
    if (cudaMemsetAsync(base, 0, sizeof(BuildCtrl), st) != cudaSuccess ||
        cudaMemsetAsync(states, 0, kNoAllocTiles * sizeof(ScanState), st) != cudaSuccess)
        return fail(WRS_ERR_CUDA, "clearing the scratch failed");
    if (launch_scan(st, scan_precision != WRS_SCAN_FP32, in, n, out, ctrl, states, kNoAllocTiles,
                    partials, kSpinLimit) != cudaSuccess)
        return fail(WRS_ERR_CUDA, "scan launch failed");
    if (device_status &&
        cudaMemcpyAsync(device_status, &ctrl->status, sizeof(uint32_t), cudaMemcpyDeviceToDevice,
                        st) != cudaSuccess)
        return fail(WRS_ERR_CUDA, "status copy failed");
    return WRS_OK;
}
