// Arithmetic of the seeded scene generator, shared by the host generator
// (scenegen.cpp, g++ with -ffp-contract=off) and the device generator
// (encode.cu, nvcc with -fmad=false and IEEE division): every function is
// integer or single-precision float arithmetic without libm calls, written
// once, so both compilers evaluate the same operations in the same order and
// produce the same bits.
#pragma once

#include <cstdint>

#ifdef __CUDACC__
#define RLE_HD __host__ __device__ __forceinline__
#else
#define RLE_HD inline
#endif

namespace rle {
namespace gen {

RLE_HD uint32_t hash32(uint32_t a, uint32_t b, uint32_t c, uint32_t seed) {
    uint32_t h = seed ^ 0x9E3779B9u;
    h ^= a * 0x85EBCA6Bu; h = (h << 13) | (h >> 19); h *= 0xC2B2AE35u;
    h ^= b * 0x27D4EB2Fu; h = (h << 11) | (h >> 21); h *= 0x165667B1u;
    h ^= c * 0x9E3779B1u; h = (h << 7) | (h >> 25); h *= 0x85EBCA6Bu;
    h ^= h >> 16; h *= 0x7FEB352Du; h ^= h >> 15; h *= 0x846CA68Bu; h ^= h >> 16;
    return h;
}

RLE_HD int ifloor(float v) {
    int i = static_cast<int>(v);
    return (v < static_cast<float>(i)) ? i - 1 : i;
}

// Value noise on a periodic lattice (period lx x lz cells of `cell` voxels).
RLE_HD float value_noise2(int x, int z, int cell, int lx, int lz, uint32_t seed) {
    const int ix = x / cell, iz = z / cell;
    const float fx = static_cast<float>(x - ix * cell) / static_cast<float>(cell);
    const float fz = static_cast<float>(z - iz * cell) / static_cast<float>(cell);
    const int x0 = ix % lx, z0 = iz % lz, x1 = (ix + 1) % lx, z1 = (iz + 1) % lz;
    const float inv = 1.0f / 16777216.0f;
    const float v00 = static_cast<float>(hash32(x0, z0, cell, seed) >> 8) * inv;
    const float v10 = static_cast<float>(hash32(x1, z0, cell, seed) >> 8) * inv;
    const float v01 = static_cast<float>(hash32(x0, z1, cell, seed) >> 8) * inv;
    const float v11 = static_cast<float>(hash32(x1, z1, cell, seed) >> 8) * inv;
    const float sx = fx * fx * (3.0f - 2.0f * fx);
    const float sz = fz * fz * (3.0f - 2.0f * fz);
    const float a = v00 + (v10 - v00) * sx;
    const float b = v01 + (v11 - v01) * sx;
    return a + (b - a) * sz;
}

// Dot product with gradient h % 12, one of the 12 edge directions of a cube
// {(+-1,+-1,0), (+-1,0,+-1), (0,+-1,+-1)} in the order x-y, x-z, y-z pairs.
RLE_HD float grad_dot(int h, float x, float y, float z) {
    const int e = h % 12;
    const int pair = e >> 2;                     // 0: x,y  1: x,z  2: y,z
    const int s0 = (e & 1) ? -1 : 1, s1 = (e & 2) ? -1 : 1;
    const int d0 = pair == 2 ? 0 : s0;
    const int d1 = pair == 0 ? s1 : (pair == 2 ? s0 : 0);
    const int d2 = pair == 0 ? 0 : s1;
    return static_cast<float>(d0) * x + static_cast<float>(d1) * y + static_cast<float>(d2) * z;
}

// 3D simplex noise (Gustavson's formulation of Perlin's simplex noise) over a
// 512-entry permutation table (a shuffled 0..255 repeated twice).
RLE_HD float simplex3(const uint8_t* perm, float x, float y, float z) {
    const float F = 1.0f / 3.0f, G = 1.0f / 6.0f;
    const float s = (x + y + z) * F;
    const int i = ifloor(x + s), j = ifloor(y + s), k = ifloor(z + s);
    const float t = static_cast<float>(i + j + k) * G;
    const float x0 = x - (static_cast<float>(i) - t);
    const float y0 = y - (static_cast<float>(j) - t);
    const float z0 = z - (static_cast<float>(k) - t);
    int i1, j1, k1, i2, j2, k2;
    if (x0 >= y0) {
        if (y0 >= z0) { i1 = 1; j1 = 0; k1 = 0; i2 = 1; j2 = 1; k2 = 0; }
        else if (x0 >= z0) { i1 = 1; j1 = 0; k1 = 0; i2 = 1; j2 = 0; k2 = 1; }
        else { i1 = 0; j1 = 0; k1 = 1; i2 = 1; j2 = 0; k2 = 1; }
    } else {
        if (y0 < z0) { i1 = 0; j1 = 0; k1 = 1; i2 = 0; j2 = 1; k2 = 1; }
        else if (x0 < z0) { i1 = 0; j1 = 1; k1 = 0; i2 = 0; j2 = 1; k2 = 1; }
        else { i1 = 0; j1 = 1; k1 = 0; i2 = 1; j2 = 1; k2 = 0; }
    }
    const int ii = i & 255, jj = j & 255, kk = k & 255;
    float n = 0.0f;
    for (int c = 0; c < 4; c++) {
        const int oi = c == 0 ? 0 : (c == 1 ? i1 : (c == 2 ? i2 : 1));
        const int oj = c == 0 ? 0 : (c == 1 ? j1 : (c == 2 ? j2 : 1));
        const int ok = c == 0 ? 0 : (c == 1 ? k1 : (c == 2 ? k2 : 1));
        float xc, yc, zc;
        if (c == 0) { xc = x0; yc = y0; zc = z0; }
        else if (c == 3) { xc = x0 - 1.0f + 3.0f * G; yc = y0 - 1.0f + 3.0f * G; zc = z0 - 1.0f + 3.0f * G; }
        else {
            const float g = c == 1 ? G : 2.0f * G;
            xc = x0 - static_cast<float>(oi) + g;
            yc = y0 - static_cast<float>(oj) + g;
            zc = z0 - static_cast<float>(ok) + g;
        }
        const int h = perm[ii + oi + perm[jj + oj + perm[kk + ok]]];
        float w = 0.6f - xc * xc - yc * yc - zc * zc;
        if (w > 0.0f) {
            w *= w;
            n += w * w * grad_dot(h, xc, yc, zc);
        }
    }
    return 32.0f * n;
}

// Generator constants (from rle_scenegen_params).
struct Consts {
    int sx, sy, sz, octaves, base_period, caves;
    float height_min, height_max, cave_y0, cave_y1, cave_threshold, cave_period;
    uint32_t seed32;
};

// Ground height (voxels above the bottom, 1..sy) of column (x, z): toroidally
// tiling fBm value noise.
RLE_HD int ground_height(const Consts& p, int x, int z) {
    float sum = 0.0f, amp = 1.0f, norm = 0.0f;
    int cell = p.base_period;
    for (int o = 0; o < p.octaves && cell >= 1; o++) {
        sum += amp * value_noise2(x, z, cell, p.sx / cell, p.sz / cell, p.seed32 + 101u * static_cast<uint32_t>(o));
        norm += amp;
        amp *= 0.5f;
        cell >>= 1;
    }
    const float f = sum / norm;
    // stretch the fBm's central concentration over the height range
    float g = (f - 0.5f) * 1.8f + 0.5f;
    if (g < 0.0f) g = 0.0f;
    if (g > 1.0f) g = 1.0f;
    int h = static_cast<int>(p.height_min + (p.height_max - p.height_min) * g);
    if (h < 1) h = 1;
    if (h > p.sy) h = p.sy;
    return h;
}

// Cave test at height y: two octaves of simplex noise, squashed 4x in y.
RLE_HD bool carved(const Consts& p, const uint8_t* perm, int x, int y, int z) {
    const float inv = 1.0f / p.cave_period;
    const float fx = static_cast<float>(x) * inv, fy = static_cast<float>(y) * inv * 4.0f,
                fz = static_cast<float>(z) * inv;
    const float d = simplex3(perm, fx, fy, fz) + 0.5f * simplex3(perm, 2.0f * fx + 17.0f, 2.0f * fy, 2.0f * fz + 31.0f);
    return d > p.cave_threshold;
}

// Colour tint of column (x, z) at level 0 (the part of the colour that does
// not depend on the height).
RLE_HD int tint(const Consts& p, int x, int z) {
    const int cell = 64 < p.sx && 64 < p.sz ? 64 : (p.sx < p.sz ? p.sx : p.sz);
    return static_cast<int>(value_noise2(x & (p.sx - 1), z & (p.sz - 1), cell, p.sx / cell, p.sz / cell,
                                         p.seed32 ^ 0xC0105EEDu) * 96.0f);
}

// RGB565 colour of level-0 voxel (x, j, z), j counted down from the top,
// given the column's tint: a height-band palette scaled by tint + jitter.
RLE_HD uint16_t colour(const Consts& p, int tint_xz, int x, int j, int z) {
    // palette bands, bottom to top: 0x5C4E42, 0x96825A, 0xC4B478, 0x609646,
    // 0x467C3A, 0x767064, 0x96928C, 0xECECF0 (0xRRGGBB), held as one byte per
    // band in each channel's constant (band b in bits 8b..8b+7), so that no
    // thread builds a table in local memory
    const uint64_t kPalR = 0xEC96764660C4965Cull, kPalG = 0xEC92707C96B4824Eull, kPalB = 0xF08C643A46785A42ull;
    const int y = p.sy - 1 - j;
    int band = y * 8 / p.sy;
    if (band > 7) band = 7;
    if (band < 0) band = 0;
    const int jitter = static_cast<int>(hash32(x, y, z, p.seed32) & 31);
    const int f = 176 + tint_xz + jitter;  // 176..303, /256
    const int sh = 8 * band;
    int r = static_cast<int>((kPalR >> sh) & 255u) * f >> 8, g = static_cast<int>((kPalG >> sh) & 255u) * f >> 8,
        b = static_cast<int>((kPalB >> sh) & 255u) * f >> 8;
    if (r > 255) r = 255;
    if (g > 255) g = 255;
    if (b > 255) b = 255;
    return static_cast<uint16_t>(((r >> 3) << 11) | ((g >> 2) << 5) | (b >> 3));
}

}  // namespace gen
}  // namespace rle
