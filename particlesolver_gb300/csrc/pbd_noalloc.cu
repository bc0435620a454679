// Neighbour-grid build for callers that must not allocate device memory.
//
// Some hosts of this step cannot call cudaMalloc at the point where they
// need a grid: code running inside a CUDA graph capture or a caller-owned
// stream-ordered region, embedders whose device memory is handed out by
// their own allocator (a renderer or engine that owns every buffer), and
// callers that forbid allocation in a real-time step loop.  For them,
// pbd_build_grid_noalloc takes its scratch -- cell hashes, arrival slots,
// the unordered bucket, the per-cell counts / offsets and the scan partial
// sums -- from one file-scope device array of fixed size instead of
// per-system buffers.  That array exists once per device in every process
// that loads the library and stays allocated until the process exits.
//
// Limits: at most kNoAllocMaxParticles particles and kNoAllocMaxCells grid
// cells per call; larger requests are rejected with PBD_ERR_INVALID_ARGUMENT.
// The array is shared by every call on a device and keeps the previous
// call's contents: each call clears the counts it needs first, and calls
// whose work overlaps on the GPU (different streams, or different host
// threads without ordering) race on it.
#include <cstdio>
#include <mutex>

#include "pbd_system.h"

namespace {

constexpr uint32_t kNoAllocMaxParticles = PBD_NOALLOC_MAX_PARTICLES;
constexpr uint32_t kNoAllocMaxCells = PBD_NOALLOC_MAX_CELLS;
constexpr uint32_t kScanTileWords = 4096u;  // k_scan_* tile size
constexpr size_t kPartials = (kNoAllocMaxCells + 1u + kScanTileWords - 1u) / kScanTileWords;
// hash, slot, bucket: one word per particle each; offsets: cells + 1 words
constexpr size_t kOffHash = 0;
constexpr size_t kOffSlot = kOffHash + kNoAllocMaxParticles;
constexpr size_t kOffTmp = kOffSlot + kNoAllocMaxParticles;
constexpr size_t kOffCells = kOffTmp + kNoAllocMaxParticles;
constexpr size_t kOffPartials = kOffCells + kNoAllocMaxCells + 1u;
constexpr size_t kScratchWords = kOffPartials + kPartials;

// ~7 MiB per device, for the life of the process.
static __device__ __align__(256) uint32_t g_grid_scratch[kScratchWords];

// Device address of g_grid_scratch per device.  The host symbol itself is
// only a stand-in and must never reach a kernel.  The address is looked up
// (cudaGetSymbolAddress, with that device current) on every call made
// outside stream capture, so a context torn down and recreated in between
// (cudaDeviceReset reloads the module at a new address) never leaves a
// stale pointer behind; a call on a capturing stream uses the address of
// the last call outside capture, so the first call on a device must come
// before any capture.
constexpr int kMaxDevices = 64;
std::mutex g_setup_mutex;
uint32_t *g_scratch_ptr[kMaxDevices] = {};

int scratch_for_current_device(cudaStream_t stream, uint32_t **out, std::string &why) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) {
        why = std::string("cudaGetDevice failed: ") + cudaGetErrorString(e);
        return PBD_ERR_CUDA;
    }
    if (dev < 0 || dev >= kMaxDevices) {
        why = "device index out of range for the no-allocation scratch table";
        return PBD_ERR_CUDA;
    }
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    e = cudaStreamIsCapturing(stream, &cap);
    if (e != cudaSuccess) {
        why = std::string("cudaStreamIsCapturing failed: ") + cudaGetErrorString(e);
        return PBD_ERR_CUDA;
    }
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (cap == cudaStreamCaptureStatusNone) {
        void *p = nullptr;
        e = cudaGetSymbolAddress(&p, g_grid_scratch);
        if (e != cudaSuccess || !p) {
            why = std::string("cudaGetSymbolAddress failed: ") + cudaGetErrorString(e);
            return PBD_ERR_CUDA;
        }
        g_scratch_ptr[dev] = static_cast<uint32_t *>(p);
    } else if (!g_scratch_ptr[dev]) {
        why = "pbd_build_grid_noalloc: the first call on a device must come before any stream capture";
        return PBD_ERR_INVALID_ARGUMENT;
    }
    *out = g_scratch_ptr[dev];
    return PBD_OK;
}

int fail(int code, const std::string &msg) {
    pbd_internal_set_thread_error(msg);
    return code;
}

}  // namespace

extern "C" int pbd_build_grid_noalloc(const pbd_params *params, const float *positions, uint32_t n,
                                      uint32_t *sorted_index, uint32_t *cell_start, uint32_t *cell_end,
                                      void *stream) {
    std::string why;
    pbd::DevParams P;
    if (int rc = pbd_internal_device_params(params, &P, &why)) return fail(rc, why);
    if (n > kNoAllocMaxParticles) {
        char msg[160];
        snprintf(msg, sizeof msg, "pbd_build_grid_noalloc: %u particles exceed the limit of %u", n,
                 kNoAllocMaxParticles);
        return fail(PBD_ERR_INVALID_ARGUMENT, msg);
    }
    if (P.num_cells > kNoAllocMaxCells) {
        char msg[160];
        snprintf(msg, sizeof msg, "pbd_build_grid_noalloc: %u grid cells exceed the limit of %u", P.num_cells,
                 kNoAllocMaxCells);
        return fail(PBD_ERR_INVALID_ARGUMENT, msg);
    }
    if ((n && (!positions || !sorted_index)) || !cell_start || !cell_end)
        return fail(PBD_ERR_INVALID_ARGUMENT, "pbd_build_grid_noalloc: NULL buffer");
    if (pbd::scan_partial_count(P.num_cells + 1u) > kPartials)
        return fail(PBD_ERR_INVALID_ARGUMENT, "pbd_build_grid_noalloc: scan scratch too small for the grid");
    uint32_t *scratch = nullptr;
    if (int rc = scratch_for_current_device(static_cast<cudaStream_t>(stream), &scratch, why))
        return fail(rc, why);
    const cudaError_t e = pbd::launch_sort_into_cells(
        P, n, reinterpret_cast<const float4 *>(positions), scratch + kOffHash, scratch + kOffSlot,
        scratch + kOffCells, scratch + kOffPartials, scratch + kOffTmp, sorted_index, cell_start, cell_end,
        static_cast<cudaStream_t>(stream));
    if (e != cudaSuccess)
        return fail(PBD_ERR_CUDA, std::string("pbd_build_grid_noalloc: launch failed: ") + cudaGetErrorString(e));
    return PBD_OK;
}
