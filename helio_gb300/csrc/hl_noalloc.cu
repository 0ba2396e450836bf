// hl_noalloc.cu — froxel light clustering for callers that cannot allocate device
// memory.
//
// hl_bin_froxels needs scratch space on the device (each light's view-space record and
// the per-froxel counts before their prefix sum). It takes that space from the context,
// which grows it with cudaMalloc. Some callers cannot call cudaMalloc: a renderer whose
// frame code runs inside a CUDA stream capture (allocation is not allowed while a
// stream is being captured), an engine whose device memory is all owned by its own pool
// allocator under a fixed budget, or a real-time thread that must not take the driver
// paths that allocation can block on. For them, hl_bin_froxels_noalloc runs the same
// kernels with their scratch in one file-scope device array, so a call allocates nothing:
// the caller passes inputs and outputs only.
//
// The array lives on every GPU that loads this library until the process exits. Its
// device address is looked up once per device with cudaGetSymbolAddress, on the first
// call made on that device (with the device current); that first call should come before
// any stream capture. The cached address belongs to the device's primary context: a
// cudaDeviceReset destroys that context and the address with it, so a process that
// resets a device must not call this entry point on that device again (the next call
// would launch on a stale address). Every call shares the array: the kernels write every scratch word
// they read within the call, so nothing has to start at zero, but calls that overlap on
// the GPU (on different streams, or from different host threads) race on the array and
// must be serialised by the caller.
#include <mutex>

#include "hl_common.cuh"
#include "hl_internal.h"

namespace {

constexpr uint32_t kMaxLights = HL_NOALLOC_MAX_LIGHTS;
constexpr uint32_t kMaxFroxels = HL_NOALLOC_MAX_FROXELS;
constexpr size_t kLightBytes = size_t(kMaxLights) * sizeof(hl::BinLight);
constexpr size_t kCountBytes = size_t(kMaxFroxels) * sizeof(uint32_t);
constexpr size_t kScratchBytes = kLightBytes + kCountBytes;  // 192 KiB + 128 KiB

// The scratch of every hl_bin_froxels_noalloc call on a device.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_setup_mutex;
void* g_scratch_ptr[kMaxDevices] = {};  // device address of g_noalloc_scratch per device

// Device address of the scratch array on the current device (set-up on first use).
hl_status scratch_address(void** out) {
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return HL_ERR_CUDA;
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (!g_scratch_ptr[dev]) {
        void* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p) {
            (void)cudaGetLastError();  // the lookup's error is not left for the caller's next check
            return HL_ERR_CUDA;
        }
        g_scratch_ptr[dev] = p;
    }
    *out = g_scratch_ptr[dev];
    return HL_OK;
}

inline bool aligned16(const void* p) { return (reinterpret_cast<uintptr_t>(p) & 15u) == 0; }

}  // namespace

extern "C" hl_status hl_bin_froxels_noalloc(const void* camera, const void* lights, uint32_t n_lights,
                                            const hl_froxel_params* params, const hl_froxel_lists* out,
                                            void* stream) {
    if (!camera || !params || !out || !out->offsets) return HL_ERR_INVALID_ARGUMENT;
    if (n_lights > 0 && !lights) return HL_ERR_INVALID_ARGUMENT;
    if (out->capacity > 0 && !out->indices) return HL_ERR_INVALID_ARGUMENT;
    if (!aligned16(camera) || (lights && !aligned16(lights))) return HL_ERR_LAYOUT;
    hl::SliceTable tab;
    // validates the grid (hl_froxel_slice_table rejects zero or oversized grids)
    const hl_status ps = hl_froxel_slice_table(params, tab.z);
    if (ps != HL_OK) return ps;
    const uint64_t F = uint64_t(params->grid_x) * params->grid_y * params->grid_z;
    if (n_lights > kMaxLights || F > kMaxFroxels) return HL_ERR_SIZE;
    void* base = nullptr;
    const hl_status ss = scratch_address(&base);
    if (ss != HL_OK) return ss;
    hl::BinLight* bl = static_cast<hl::BinLight*>(base);
    uint32_t* counts = reinterpret_cast<uint32_t*>(static_cast<unsigned char*>(base) + kLightBytes);
    const cudaStream_t st = static_cast<cudaStream_t>(stream);
    cudaError_t e = hl::launch_prep_bin_lights(camera, lights, n_lights, true, bl, st);
    if (e == cudaSuccess)
        e = hl::launch_bin_froxels(camera, bl, n_lights, *params, tab, counts, out->offsets, out->indices,
                                   out->capacity, nullptr, st);
    return e == cudaSuccess ? HL_OK : HL_ERR_CUDA;
}
