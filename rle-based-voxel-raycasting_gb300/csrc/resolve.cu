// Ray buffer -> screen resolve on sm_103a.
//
// The reference warps its ray buffer onto the screen in a GLSL fragment
// shader (bin/shader/colorize_buddha_soft.frag:12-80): per pixel it finds
// the fan (up/down/left/right of the vanishing point) the pixel lies in, the
// column ray through it and the sample along that ray, then fetches the
// texel with GL_NEAREST / GL_CLAMP_TO_EDGE (src/GL_Main.cpp:152-157).  This
// kernel does the same arithmetic, one thread per pixel, as IEEE single
// operations in the shader's order (compiled with -fmad=false), and decodes
// the sample: sky, no data, or an RGB565 colour with its float depth.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>

#include "rle_internal.h"

namespace rle {
namespace {

#ifdef RLE_BOUNDS_CHECK
__device__ unsigned int g_bounds[4];
__device__ __forceinline__ bool in_bounds(bool ok, unsigned code, unsigned long long idx) {
    if (!ok) {
        const unsigned prev = atomicOr(&g_bounds[0], code);
        if (prev == 0) {
            g_bounds[1] = static_cast<unsigned>(idx);
            g_bounds[2] = static_cast<unsigned>(idx >> 32);
        }
    }
    return ok;
}
#else
__device__ __forceinline__ bool in_bounds(bool, unsigned, unsigned long long) { return true; }
#endif

__device__ __forceinline__ float step_f(float edge, float x) { return x < edge ? 0.0f : 1.0f; }

__device__ __forceinline__ int texel(float t, int size) {
    int i = static_cast<int>(floorf(t * static_cast<float>(size)));
    return min(max(i, 0), size - 1);
}

__device__ __forceinline__ uint32_t rgb565_to_rgba8(uint32_t c) {
    uint32_t r = (c >> 11) & 31u, g = (c >> 5) & 63u, b = c & 31u;
    r = (r << 3) | (r >> 2);
    g = (g << 2) | (g >> 4);
    b = (b << 3) | (b >> 2);
    return r | (g << 8) | (b << 16) | 0xff000000u;
}

template <bool kHits>
__device__ __forceinline__ void resolve_pixel(const ResolveParams& P, int col, int row) {
    const float RESX = P.resx, RESY = P.resy;
    const float fx = static_cast<float>(col) + 0.5f;
    const float fy = static_cast<float>(P.height - 1 - row) + 0.5f;  // GL rows count from the bottom
    const float scx = fx / RESX, scy = fy / RESY;
    const float border = (RESX - RESY) / (RESX * 2);
    const float scx1 = scx - P.vanish_x, scy1 = scy - P.vanish_y;
    const float upper = step_f(scy1, 0.0f);
    const float left = step_f(scx1, 0.0f);
    const float ostep = step_f(fabsf(scy1) - fabsf(scx1) * RESX / RESY, 0.0f);
    const float seg_up = (1 - upper) * (1 - ostep);
    const float seg_dn = upper * (1 - ostep);
    const float seg_rt = (1 - left) * ostep;
    const float seg_lt = left * ostep;
    const float o2 = (ostep * fx + (1 - ostep) * fy) / RESX;
    const float ang2 = scx1 * fabsf(1 - step_f(scy1, 0.0f) - P.vanish_y) / scy1 +
                       step_f(scy1, 0.0f) * (1 - P.vanish_x) + (1 - step_f(scy1, 0.0f)) * P.vanish_x;
    float ang3 = scy1 * fabsf(1 - step_f(scx1, 0.0f) - P.vanish_x) / scx1 +
                 step_f(scx1, 0.0f) * (1 - P.vanish_y) + (1 - step_f(scx1, 0.0f)) * P.vanish_y;
    ang3 = ang3 * RESY / RESX + border;
    const float x_pre = ostep * ang3 + ang2 * (1 - ostep);
    float ty = seg_dn * (P.ofs_y + x_pre) + seg_up * (P.ofs_x + 1.0f - x_pre) + seg_lt * (P.ofs_w + x_pre) +
               seg_rt * (P.ofs_z + 1.0f - x_pre);
    ty = ty * P.ratio * 0.25f;
    const float r = P.rxg0;
    const float seg_up_x = r * seg_up + (1.0f - r) * seg_dn;
    const float seg_dn_x = r * seg_dn + (1.0f - r) * seg_up;
    const float seg_rt_x = r * seg_rt + (1.0f - r) * seg_lt;
    const float seg_lt_x = r * seg_lt + (1.0f - r) * seg_rt;
    const float tx = seg_up_x * (o2 + border) + seg_dn_x * (1.0f - (o2 + border)) + seg_rt_x * o2 +
                     seg_lt_x * (1.0f - o2);
    const int s = texel(tx, P.S);
    const int rr = texel(ty, P.rows);
    const size_t si = static_cast<size_t>(rr) * P.S + s;
    const size_t pi = static_cast<size_t>(row) * P.width + col;
    // rows past the rays cast hold no data (the reference's pixel buffer
    // keeps whatever an earlier frame left there)
    const bool cast = rr < P.rays && in_bounds(si < static_cast<size_t>(P.rows) * P.S, kBoundsResolve, si);
    const uint32_t w = cast ? __ldg(&P.raybuf[si]) : 0u;
    const float d = cast ? __ldg(&P.raydepth[si]) : 0.0f;
    uint32_t c;
    float dep;
    if (((w >> 16) & 0xffu) == 0xffu) {  // sky: the shader's c.z == 1.0
        c = 0xffffccb2u;
        dep = INFINITY;
    } else if (d == 0.0f) {  // outside the ray's clip range
        c = 0u;
        dep = 0.0f;
    } else {
        c = rgb565_to_rgba8(w & 0xffffu);
        dep = d;
    }
    P.colour[pi] = c;
    P.depth[pi] = dep;
    if (kHits) {
        rle_hit h = {0, 0, 0, 0, 0};
        if (P.rayhit && cast) h = P.rayhit[si];
        P.hit[pi] = h;
    }
}

template <bool kHits>
__global__ void resolve_kernel(const __grid_constant__ ResolveParams P) {
    const int col = blockIdx.x * blockDim.x + threadIdx.x;
    const int row = blockIdx.y;
    if (col >= P.width || row >= P.height) return;
    resolve_pixel<kHits>(P, col, row);
}

// All frames of a batch: block b belongs to the frame f with
// block_start[f] <= b < block_start[f+1] and covers 256 of its pixels.
constexpr int kResolveBlock = 256;

// Persistent: block i takes pixel blocks i, i + gridDim.x, ... of the batch.
__global__ void __launch_bounds__(kResolveBlock) resolve_batch_kernel(const BatchHeader* __restrict__ hdr,
                                                                      const int* __restrict__ block_start,
                                                                      const ResolveParams* __restrict__ frames) {
    const int nframes = hdr->nframes;
    const int total = block_start[nframes];
    int f = 0;
    for (int b = blockIdx.x; b < total; b += gridDim.x) {
        if (b < block_start[f] || b >= block_start[f + 1]) {
            int lo = 0, hi = nframes - 1;  // last frame with block_start <= b
            while (lo < hi) {
                const int mid = (lo + hi + 1) >> 1;
                if (block_start[mid] <= b) lo = mid;
                else hi = mid - 1;
            }
            f = lo;
        }
        const ResolveParams& P = frames[f];
        const long long pix = static_cast<long long>(b - block_start[f]) * kResolveBlock + threadIdx.x;
        if (pix >= static_cast<long long>(P.width) * P.height) continue;
        const int row = static_cast<int>(pix / P.width), col = static_cast<int>(pix % P.width);
        if (P.hit) resolve_pixel<true>(P, col, row);
        else resolve_pixel<false>(P, col, row);
    }
}

}  // namespace

int resolve_batch_blocks(int width, int height) {
    return static_cast<int>((static_cast<long long>(width) * height + kResolveBlock - 1) / kResolveBlock);
}

bool bounds_resolve(unsigned* out4, bool clear) {
#ifdef RLE_BOUNDS_CHECK
    if (cudaMemcpyFromSymbol(out4, g_bounds, sizeof(unsigned) * 4) != cudaSuccess) return false;
    if (clear) {
        const unsigned z[4] = {0, 0, 0, 0};
        if (cudaMemcpyToSymbol(g_bounds, z, sizeof(z)) != cudaSuccess) return false;
    }
    return true;
#else
    (void)out4;
    (void)clear;
    return false;
#endif
}

rle_status launch_resolve_batch(const BatchResolve& b, void* stream) {
    if (b.blocks <= 0) return RLE_OK;
    resolve_batch_kernel<<<b.blocks, kResolveBlock, 0, static_cast<cudaStream_t>(stream)>>>(b.header, b.block_start,
                                                                                            b.frames);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        set_error("batch resolve launch: %s", cudaGetErrorString(e));
        return RLE_ERR_CUDA;
    }
    return RLE_OK;
}

rle_status launch_resolve(const ResolveParams& p, void* stream) {
    const dim3 block(128, 1, 1);
    const dim3 grid((p.width + 127) / 128, p.height, 1);
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    if (p.hit) resolve_kernel<true><<<grid, block, 0, s>>>(p);
    else resolve_kernel<false><<<grid, block, 0, s>>>(p);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        set_error("resolve launch: %s", cudaGetErrorString(e));
        return RLE_ERR_CUDA;
    }
    return RLE_OK;
}

}  // namespace rle
