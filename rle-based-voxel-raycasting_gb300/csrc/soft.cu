// Soft post-filter on sm_103a: the reference's second display pass
// (bin/shader/soft.frag, drawn by src/main.cpp:627-653 over the frame
// buffer object the colorize pass filled).
//
// The colorize pass leaves, per pixel, an RGBA8 texel whose alpha is
// 0.001/z clamped to [0, 1] (z = the ray sample's depth16 as the shader reads
// it: low byte/255/256 + high byte/255; sky has alpha 0,
// colorize_buddha_soft.frag:86-136).  The soft pass then, per pixel:
//   1. takes the largest alpha among the pixel and 7 bilinear samples on a
//      circle of radius 0.005 (texture units of the 2048^2 frame buffer);
//   2. if 0.0023 * that maximum exceeds 0.00008, averages the pixel with the
//      samples of a 5x5 grid of radius 0.0023 * max whose alpha is at least
//      0.7 * max, provided more than 6 contribute; otherwise keeps the pixel.
// The frame buffer texture is RGBA8 with GL_LINEAR filtering and clamp to
// edge (src/GL_Main.h:150-165); here the bilinear weights are computed in
// single precision (a GPU's texture unit quantizes them to 8 bits, which no
// restatement reproduces) and the clamp is to the frame, not the 2048^2
// buffer.  Circle offsets and grid steps are the shader's float loops,
// evaluated once on the host.
//
// Tiling: a block filters a 32x8 tile; the texels of the tile and its apron
// (12 texels: circle radius 10.24 plus the bilinear neighbour) are built
// once into shared memory, then every tap reads shared memory.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>

#include "rle_internal.h"

namespace rle {
namespace {

constexpr int kTileX = 32, kTileY = 8, kApron = 12;
constexpr int kSmemX = kTileX + 2 * kApron, kSmemY = kTileY + 2 * kApron;

struct SoftParams {
    int width, height;
    int ncircle, ngrid;
    float circle[8][2];
    float grid[6];
};

// Frame-buffer texel of pixel (x, row-from-top) as the colorize pass leaves it.
__device__ __forceinline__ uint32_t fbo_texel(const uint32_t* colour, const float* depth, int width, int x, int row) {
    const size_t i = static_cast<size_t>(row) * width + x;
    const uint32_t c = colour[i];
    const float d = depth[i];
    uint32_t w8;
    if (isinf(d)) {
        w8 = 0;  // sky: the colorize pass leaves fragz = 0
    } else {
        const uint32_t d16 = static_cast<uint32_t>(static_cast<int>(d) & 0xfffe);
        const float z = (static_cast<float>(d16 & 255u) / 255.0f) * (1.0f / 256.0f) +
                        static_cast<float>(d16 >> 8) / 255.0f;
        const float fragz = 0.001f / z;
        const float f = fminf(fmaxf(fragz, 0.0f), 1.0f);
        w8 = static_cast<uint32_t>(static_cast<int>(f * 255.0f + 0.5f));
    }
    return (c & 0x00ffffffu) | (w8 << 24);
}

struct F4 {
    float x, y, z, w;
};

__device__ __forceinline__ F4 unpack(uint32_t t) {
    return F4{static_cast<float>(t & 255u) / 255.0f, static_cast<float>((t >> 8) & 255u) / 255.0f,
              static_cast<float>((t >> 16) & 255u) / 255.0f, static_cast<float>(t >> 24) / 255.0f};
}

// GL_LINEAR sample at texture coordinate (u, v) of the 2048^2 buffer; texel
// rows count from the bottom of the frame.
__device__ __forceinline__ F4 sample(const uint32_t (*tile)[kSmemX], int tx0, int ty0, int width, int height,
                                     float u, float v) {
    const float uu = u * 2048.0f - 0.5f, vv = v * 2048.0f - 0.5f;
    const float fx0 = floorf(uu), fy0 = floorf(vv);
    const float a = uu - fx0, b = vv - fy0;
    const int i0 = min(max(static_cast<int>(fx0), 0), width - 1);
    const int i1 = min(max(static_cast<int>(fx0) + 1, 0), width - 1);
    const int j0 = min(max(static_cast<int>(fy0), 0), height - 1);
    const int j1 = min(max(static_cast<int>(fy0) + 1, 0), height - 1);
    const F4 t00 = unpack(tile[j0 - ty0][i0 - tx0]), t10 = unpack(tile[j0 - ty0][i1 - tx0]);
    const F4 t01 = unpack(tile[j1 - ty0][i0 - tx0]), t11 = unpack(tile[j1 - ty0][i1 - tx0]);
    const float w00 = (1.0f - a) * (1.0f - b), w10 = a * (1.0f - b), w01 = (1.0f - a) * b, w11 = a * b;
    F4 r;
    r.x = w00 * t00.x + w10 * t10.x + w01 * t01.x + w11 * t11.x;
    r.y = w00 * t00.y + w10 * t10.y + w01 * t01.y + w11 * t11.y;
    r.z = w00 * t00.z + w10 * t10.z + w01 * t01.z + w11 * t11.z;
    r.w = w00 * t00.w + w10 * t10.w + w01 * t01.w + w11 * t11.w;
    return r;
}

__device__ __forceinline__ uint32_t to_byte(float v) {
    const float f = fminf(fmaxf(v, 0.0f), 1.0f);
    return static_cast<uint32_t>(static_cast<int>(f * 255.0f + 0.5f));
}

__global__ void __launch_bounds__(kTileX * kTileY) soft_kernel(const __grid_constant__ SoftParams P,
                                                               const uint32_t* __restrict__ colour,
                                                               const float* __restrict__ depth,
                                                               uint32_t* __restrict__ out) {
    __shared__ uint32_t tile[kSmemY][kSmemX];
    // tile origin in GL texel coordinates (rows from the bottom)
    const int gx0 = blockIdx.x * kTileX - kApron, gy0 = blockIdx.y * kTileY - kApron;
    const int tid = threadIdx.y * kTileX + threadIdx.x;
    for (int i = tid; i < kSmemX * kSmemY; i += kTileX * kTileY) {
        const int sx = i % kSmemX, sy = i / kSmemX;
        const int x = min(max(gx0 + sx, 0), P.width - 1);
        const int y = min(max(gy0 + sy, 0), P.height - 1);
        tile[sy][sx] = fbo_texel(colour, depth, P.width, x, P.height - 1 - y);
    }
    __syncthreads();
    const int x = blockIdx.x * kTileX + threadIdx.x, y = blockIdx.y * kTileY + threadIdx.y;
    if (x >= P.width || y >= P.height) return;
    const float u = (static_cast<float>(x) + 0.5f) / 2048.0f, v = (static_cast<float>(y) + 0.5f) / 2048.0f;
    F4 col = unpack(tile[y - gy0][x - gx0]);
    float radmax = col.w;
    for (int i = 0; i < P.ncircle; i++) {
        const float w = sample(tile, gx0, gy0, P.width, P.height, P.circle[i][0] + u, P.circle[i][1] + v).w;
        radmax = fmaxf(radmax, w);
    }
    const float rad = 0.0023f * radmax;
    if (rad > 0.00008f) {
        F4 avg = col;
        float n = 1.0f;
        const float thresh = radmax * 0.7f;
        for (int ia = 0; ia < P.ngrid; ia++) {
            for (int ib = 0; ib < P.ngrid; ib++) {
                const float cu = u + P.grid[ia] * rad, cv = v + P.grid[ib] * rad;
                const F4 c = sample(tile, gx0, gy0, P.width, P.height, cu, cv);
                if (c.w >= thresh) {
                    avg.x = avg.x + c.x;
                    avg.y = avg.y + c.y;
                    avg.z = avg.z + c.z;
                    avg.w = avg.w + c.w;
                    n = n + 1.0f;
                }
            }
        }
        if (n > 6.0f) {
            const float inv = 1.0f / n;
            col.x = avg.x * inv;
            col.y = avg.y * inv;
            col.z = avg.z * inv;
            col.w = avg.w * inv;
        }
    }
    out[static_cast<size_t>(P.height - 1 - y) * P.width + x] =
        to_byte(col.x) | (to_byte(col.y) << 8) | (to_byte(col.z) << 16) | (to_byte(col.w) << 24);
}

}  // namespace
}  // namespace rle

extern "C" rle_status rle_soft_filter(const uint32_t* d_colour, const float* d_depth, int width, int height,
                                      uint32_t* d_out, void* stream) {
    if (!d_colour || !d_depth || !d_out || width < 1 || height < 1 || width > 2048 || height > 2048 ||
        d_out == d_colour) {
        rle::set_error("rle_soft_filter: colour, depth and a separate output of 1..2048 x 1..2048 pixels required");
        return RLE_ERR_INVALID_ARG;
    }
    rle::SoftParams P;
    P.width = width;
    P.height = height;
    // the shader's loops, in float: circle angles 0, step 3.1415*1.9/6
    // while below 2*3.1415; grid -1 + k*(2/5) while below 1
    P.ncircle = 0;
    const float step = 3.1415f * 1.9f / 6.0f;
    for (float a = 0.0f; a < 3.1415f * 2.0f && P.ncircle < 8; a += step) {
        P.circle[P.ncircle][0] = std::sin(a) * 0.005f;
        P.circle[P.ncircle][1] = std::cos(a) * 0.005f;
        P.ncircle++;
    }
    P.ngrid = 0;
    for (float a = -1.0f; a < 1.0f && P.ngrid < 6; a += 2.0f / 5.0f) P.grid[P.ngrid++] = a;
    const dim3 block(rle::kTileX, rle::kTileY);
    const dim3 grid((width + rle::kTileX - 1) / rle::kTileX, (height + rle::kTileY - 1) / rle::kTileY);
    rle::soft_kernel<<<grid, block, 0, static_cast<cudaStream_t>(stream)>>>(P, d_colour, d_depth, d_out);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        rle::set_error("rle_soft_filter: %s", cudaGetErrorString(e));
        return RLE_ERR_CUDA;
    }
    return RLE_OK;
}
