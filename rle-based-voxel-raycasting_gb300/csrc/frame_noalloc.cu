// Whole-frame render that allocates no device memory.
//
// rle_render_frame needs a ray buffer between the raycast and the resolve;
// there the caller passes it in.  Some callers cannot provide one: a render
// loop with a hard frame budget must not call cudaMalloc once it runs (the
// call can synchronise the device and stall the frame), and a plug-in hosted
// by an application that owns the GPU memory budget may not allocate at all.
// For them this entry point keeps the ray buffer in a fixed array compiled
// into the library.  Device code is loaded lazily (the CUDA default since
// 12.2), so the array is reserved on a device by the first call there, which
// also looks up its address; it stays reserved until the process exits, and
// later calls allocate nothing.  The cached address does not survive a
// cudaDeviceReset of the device.
#include <cuda_runtime.h>

#include <mutex>

#include "rle_internal.h"

namespace {

// Ray buffer of one frame: the packed words of the rays it casts, then their
// depths (256-byte aligned).  64 MiB holds e.g. 4000 rays x 1920 samples.
constexpr size_t kScratchBytes = static_cast<size_t>(64) << 20;
__device__ __align__(256) unsigned char g_frame_scratch[kScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_scratch_mutex;
void* g_scratch_addr[kMaxDevices] = {};

// Device address of the scratch array on `dev` (which must be current),
// looked up on the first call for that device.
rle_status scratch_address(int dev, void** out) {
    std::lock_guard<std::mutex> lock(g_scratch_mutex);
    if (dev < 0 || dev >= kMaxDevices) {
        rle::set_error("rle_render_frame_noalloc: device %d out of range", dev);
        return RLE_ERR_INVALID_ARG;
    }
    if (!g_scratch_addr[dev]) {
        void* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_frame_scratch);
        if (e != cudaSuccess || !p) {
            rle::set_error("rle_render_frame_noalloc: cudaGetSymbolAddress: %s", cudaGetErrorString(e));
            return RLE_ERR_CUDA;
        }
        g_scratch_addr[dev] = p;
    }
    *out = g_scratch_addr[dev];
    return RLE_OK;
}

}  // namespace

extern "C" size_t rle_render_frame_noalloc_limit(void) { return kScratchBytes; }

extern "C" rle_status rle_render_frame_noalloc(const rle_scene* scene, const rle_camera* cam,
                                               const rle_view_params* view, uint32_t* d_colour, float* d_depth,
                                               void* stream) {
    if (!scene || !cam || !view || !d_colour || !d_depth) {
        rle::set_error("rle_render_frame_noalloc: null argument");
        return RLE_ERR_INVALID_ARG;
    }
    rle_raymap rm;
    rle_status st = rle_raymap_build(cam, view, &rm);
    if (st != RLE_OK) return st;
    // only the rows of the rays cast are stored: the raycast writes every
    // word of them, and the resolve reads no other row
    const size_t words = static_cast<size_t>(rm.rays) * static_cast<size_t>(rm.samples);
    const size_t raybuf_bytes = (words * 4 + 255) & ~static_cast<size_t>(255);
    const size_t need = raybuf_bytes + words * 4;
    if (need > kScratchBytes) {
        rle::set_error("rle_render_frame_noalloc: this frame needs %zu bytes of ray buffer (%d rays x %d samples); "
                       "the built-in buffer holds %zu -- use rle_render_frame with a workspace",
                       need, rm.rays, rm.samples, kScratchBytes);
        return RLE_ERR_CAPACITY;
    }
    int prev = -1;
    cudaGetDevice(&prev);
    if (prev != scene->device && cudaSetDevice(scene->device) != cudaSuccess) {
        rle::set_error("rle_render_frame_noalloc: cannot select device %d", scene->device);
        return RLE_ERR_CUDA;
    }
    void* base = nullptr;
    st = scratch_address(scene->device, &base);
    if (st == RLE_OK) {
        uint32_t* raybuf = static_cast<uint32_t*>(base);
        float* raydepth = reinterpret_cast<float*>(static_cast<unsigned char*>(base) + raybuf_bytes);
        st = rle_render_rays(scene, &rm, raybuf, raydepth, nullptr, nullptr, stream);
        if (st == RLE_OK) st = rle_resolve(&rm, raybuf, raydepth, nullptr, d_colour, d_depth, nullptr, stream);
    }
    if (prev >= 0 && prev != scene->device) cudaSetDevice(prev);
    return st;
}
