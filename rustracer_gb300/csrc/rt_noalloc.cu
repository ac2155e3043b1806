// The photon-grid build for callers that cannot allocate device memory.
//
// rt_stage_photon_grid allocates its device buffers on every call.  Some callers cannot do that: frame
// loops with a hard no-allocation rule (cudaMalloc / cudaFree can synchronise the device and stall a
// frame), hosts whose device memory is handed out by their own allocator (an engine's or a
// framework's pool that owns every byte the process may touch), and processes running close to the
// memory limit, where an allocation could fail in the middle of a frame.  For them,
// rt_stage_photon_grid_noalloc takes device pointers for its input and outputs and keeps its scratch
// -- per-slot cell keys and slot order, per-cell cursors, the scan's tile sums and the binned total --
// in one file-scope __device__ array of fixed size.  Every GPU that loads this library holds that
// array (RT_NOALLOC_SCRATCH_BYTES, 9,438,208 bytes) until the process exits.
#include <cuda_runtime.h>

#include "rt_internal.h"
#include "rt_kernels.h"

using rt::set_error;

namespace {

constexpr size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }
constexpr size_t kKeysOff = 0;
constexpr size_t kOrderOff = align256(kKeysOff + 4 * (size_t)RT_NOALLOC_MAX_SLOTS);
constexpr size_t kCursorOff = align256(kOrderOff + 4 * (size_t)RT_NOALLOC_MAX_SLOTS);
constexpr size_t kPartialsOff = align256(kCursorOff + 4 * (size_t)RT_NOALLOC_MAX_CELLS);
constexpr size_t kPartialsMax = RT_NOALLOC_MAX_CELLS / 2048 + 2;  // the scan's tile sums (+ grand total)
constexpr size_t kTotalOff = align256(kPartialsOff + 4 * kPartialsMax);
constexpr size_t kScratchBytes = align256(kTotalOff + 16);
static_assert(kScratchBytes <= RT_NOALLOC_SCRATCH_BYTES, "scratch layout exceeds the declared size");

}  // namespace

// Shared by every call on a device.  In host code the name is only a handle: the array's device
// address comes from cudaGetSymbolAddress with the device current.
static __device__ __align__(256) unsigned char g_grid_scratch[RT_NOALLOC_SCRATCH_BYTES];

extern "C" int rt_stage_photon_grid_noalloc(const rt_photon *d_photons, const rt_grid_params *gp, uint32_t *d_counts,
                                            uint32_t *d_meta, rt_photon *d_sorted, void *stream) {
    rt::clear_error();
    (void)cudaGetLastError();  // a non-sticky error left by earlier, unrelated work is not this call's
    if (!gp || !d_counts || !d_meta || !d_sorted || (gp->photon_slots && !d_photons)) {
        set_error("rt_stage_photon_grid_noalloc: null argument");
        return RT_ERR_INVALID_ARGUMENT;
    }
    if ((reinterpret_cast<uintptr_t>(d_photons) | reinterpret_cast<uintptr_t>(d_sorted)) % 16u != 0u ||
        (reinterpret_cast<uintptr_t>(d_counts) | reinterpret_cast<uintptr_t>(d_meta)) % 4u != 0u) {
        set_error("rt_stage_photon_grid_noalloc: d_photons / d_sorted must be 16-byte aligned, d_counts / d_meta 4-byte");
        return RT_ERR_INVALID_ARGUMENT;
    }
    if (gp->num_cells == 0 || gp->num_cells > RT_NOALLOC_MAX_CELLS || gp->photon_slots > RT_NOALLOC_MAX_SLOTS) {
        set_error("rt_stage_photon_grid_noalloc: %u slots and %u cells requested; this entry point handles at most "
                  "%u slots and %u cells (use rt_stage_photon_grid beyond that)",
                  gp->photon_slots, gp->num_cells, (unsigned)RT_NOALLOC_MAX_SLOTS, (unsigned)RT_NOALLOC_MAX_CELLS);
        return RT_ERR_INVALID_ARGUMENT;
    }
    if (rtd::grid_scan_partials(gp->num_cells) > kPartialsMax) {
        set_error("rt_stage_photon_grid_noalloc: scan tile sums exceed the scratch layout");
        return RT_ERR_INVALID_ARGUMENT;
    }
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) {
        set_error("rt_stage_photon_grid_noalloc: no usable current device (%s)", cudaGetErrorString(e));
        return RT_ERR_CUDA;
    }
    // The array's address on the current device, looked up on every call: a lookup allocates nothing
    // once the module is loaded, and a fresh one stays right after cudaDeviceReset reloads it.  The
    // first call on a device may load the module (lazy loading), which creates the array.
    void *base = nullptr;
    e = cudaGetSymbolAddress(&base, g_grid_scratch);
    if (e != cudaSuccess || !base) {
        set_error("rt_stage_photon_grid_noalloc: cudaGetSymbolAddress failed on device %d: %s", dev,
                  cudaGetErrorString(e));
        return RT_ERR_CUDA;
    }
    unsigned char *b = static_cast<unsigned char *>(base);
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    uint32_t *keys = reinterpret_cast<uint32_t *>(b + kKeysOff);
    rtd::GridBuffers g;
    g.photons = reinterpret_cast<const float4 *>(d_photons);
    g.keys = keys;
    g.slot_count = gp->photon_slots;
    g.num_cells = gp->num_cells;
    g.counts = d_counts;  // cleared by the build (with the cursors); the scan totals are written whole
    g.meta = reinterpret_cast<uint2 *>(d_meta);
    g.cursor = reinterpret_cast<uint32_t *>(b + kCursorOff);
    g.order = reinterpret_cast<uint32_t *>(b + kOrderOff);
    g.sorted = reinterpret_cast<float4 *>(d_sorted);
    g.sorted_pos = nullptr;
    g.rank = nullptr;  // the scratch holds no rank array: count, atomic scatter, multi-photon cell pass
    g.scan_partials = reinterpret_cast<uint32_t *>(b + kPartialsOff);
    g.total = reinterpret_cast<uint32_t *>(b + kTotalOff);
    if ((e = rtd::launch_photon_keys(g.photons, g.slot_count, *gp, keys, st)) != cudaSuccess ||
        (e = rtd::launch_grid_build(g, st)) != cudaSuccess) {
        set_error("rt_stage_photon_grid_noalloc: launch failed: %s", cudaGetErrorString(e));
        return RT_ERR_CUDA;
    }
    return RT_OK;
}
