// Scene building on the GPU: the seeded generator, Tree::get_mipmap's
// >= 3-of-8 rule, RLE4::compress's surface rule and run-length encoding,
// and RLE4::load's column table, as kernels over column bitsets in HBM.
//
// Working layout: one level as column bitsets, cols[(z*sx + x)*W + w] with
// W = ceil(sy/64) u64 words per column, bit j&63 of word j>>6 being voxel j
// of the column counted from the top (the reference's j,
// src/Rle4.cpp:83-88).  A level is encoded in four launches:
//   surface_kernel  surface bits (solid with < 27 solid in-bounds
//                   neighbours, src/Rle4.cpp:100-132) + words per column
//   scan            exclusive prefix of the words -> slab offsets (u64)
//   write_kernel    headers and colours of every column + its table entry
// All of it is integer/bit work bound by HBM traffic; the generator kernel
// (noise) is the only arithmetic-heavy part.
#include <cuda_runtime.h>

#include <cstring>
#include <vector>

#include "rle_internal.h"
#include "scenegen_math.h"

namespace {

using rle::gen::Consts;

constexpr int kThreads = 256;
constexpr int kMaxWords = 16;  // sy <= 1024

rle_status cuda_fail(cudaError_t e, const char* what) {
    rle::set_error("%s: %s", what, cudaGetErrorString(e));
    return e == cudaErrorMemoryAllocation ? RLE_ERR_NO_MEMORY : RLE_ERR_CUDA;
}

inline unsigned grid_for(long long n, int threads = kThreads) {
    return static_cast<unsigned>((n + threads - 1) / threads);
}

// ---------------------------------------------------------------- level 0

struct GenArgs {
    Consts c;
    uint8_t perm[512];
    int W;
};

// One thread per column: ground fill from the fBm height, then the caves.
__global__ void __launch_bounds__(kThreads) gen_columns_kernel(const __grid_constant__ GenArgs a,
                                                               uint64_t* __restrict__ cols) {
    __shared__ uint8_t perm[512];
    for (int i = threadIdx.x; i < 512; i += blockDim.x) perm[i] = a.perm[i];
    __syncthreads();
    const Consts& c = a.c;
    const long long q = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (q >= static_cast<long long>(c.sx) * c.sz) return;
    const int x = static_cast<int>(q & (c.sx - 1));
    const int z = static_cast<int>(q / c.sx);
    const int h = rle::gen::ground_height(c, x, z);
    int y0 = static_cast<int>(c.cave_y0), y1 = static_cast<int>(c.cave_y1);
    if (y0 < 1) y0 = 1;
    if (y1 > h) y1 = h;
    const int ground_j = c.sy - h;  // storage indices >= ground_j are solid
    uint64_t* out = cols + q * a.W;
    for (int w = 0; w < a.W; w++) {
        const int j0 = w * 64;
        uint64_t word;
        if (ground_j <= j0) word = ~0ull;
        else if (ground_j >= j0 + 64) word = 0;
        else word = ~0ull << (ground_j - j0);
        if (c.caves && word) {
            // heights y0 <= y < y1 <-> storage j in (sy-1-y1, sy-1-y0]
            const int jlo = max(j0, c.sy - y1), jhi = min(j0 + 63, c.sy - 1 - y0);
            for (int j = jlo; j <= jhi; j++)
                if (((word >> (j - j0)) & 1) && rle::gen::carved(c, perm, x, c.sy - 1 - j, z))
                    word &= ~(1ull << (j - j0));
        }
        out[w] = word;
    }
}

// Reference Tree layout (bit i&7 of byte (i + j*sx + k*sx*sy) >> 3) ->
// column bitsets.  A warp covers 32 consecutive columns of one row of
// words, so each j reads 4 adjacent bytes.
__global__ void __launch_bounds__(kThreads) transpose_kernel(const uint8_t* __restrict__ bits, int sx, int sy, int sz,
                                                             int W, uint64_t* __restrict__ cols) {
    const long long t = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x;
    const long long n = static_cast<long long>(sx) * sz * W;
    if (t >= n) return;
    const int x = static_cast<int>(t % sx);
    const long long r = t / sx;
    const int w = static_cast<int>(r % W);
    const int z = static_cast<int>(r / W);
    const long long sxy = static_cast<long long>(sx) * sy;
    uint64_t word = 0;
    const int jend = min(sy, w * 64 + 64);
    for (int j = w * 64; j < jend; j++) {
        const long long idx = x + static_cast<long long>(j) * sx + z * sxy;
        word |= static_cast<uint64_t>((bits[idx >> 3] >> (x & 7)) & 1) << (j & 63);
    }
    cols[(static_cast<long long>(z) * sx + x) * W + w] = word;
}

// ----------------------------------------------------------------- mips

__device__ __forceinline__ uint32_t compact_nibble_lsbs(uint64_t v) {
    v &= 0x1111111111111111ull;
    v = (v | (v >> 3)) & 0x0303030303030303ull;
    v = (v | (v >> 6)) & 0x000F000F000F000Full;
    v = (v | (v >> 12)) & 0x000000FF000000FFull;
    v = (v | (v >> 24)) & 0x000000000000FFFFull;
    return static_cast<uint32_t>(v);
}

__device__ __forceinline__ uint32_t spread16(uint32_t v) {
    v &= 0xFFFF;
    v = (v | (v << 8)) & 0x00FF00FFu;
    v = (v | (v << 4)) & 0x0F0F0F0Fu;
    v = (v | (v << 2)) & 0x33333333u;
    v = (v | (v << 1)) & 0x55555555u;
    return v;
}

// Level m+1 from level m (Tree::get_mipmap, src/tree.h:23-85): a voxel is
// solid when >= 3 of its 8 children are.  One thread per output column;
// each input word gives 32 output bits (pairs of rows of 4 columns).
__global__ void __launch_bounds__(kThreads) halve_kernel(const uint64_t* __restrict__ a, int asx, int aW,
                                                         uint64_t* __restrict__ b, int bsx, int bsz, int bsy, int bW) {
    const long long q = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (q >= static_cast<long long>(bsx) * bsz) return;
    const int i = static_cast<int>(q % bsx), k = static_cast<int>(q / bsx);
    const uint64_t* c0 = a + (static_cast<long long>(2 * k) * asx + 2 * i) * aW;
    const uint64_t* c1 = c0 + aW;
    const uint64_t* c2 = a + (static_cast<long long>(2 * k + 1) * asx + 2 * i) * aW;
    const uint64_t* c3 = c2 + aW;
    const uint64_t m55 = 0x5555555555555555ull, m33 = 0x3333333333333333ull;
    uint64_t* dst = b + q * bW;
    uint64_t acc = 0;
    int written = 0;
    for (int w = 0; w < aW; w++) {
        const int j0 = 32 * w;
        if (j0 >= bsy) break;
        uint64_t sa = 0, sb = 0;
        const uint64_t v4[4] = {c0[w], c1[w], c2[w], c3[w]};
#pragma unroll
        for (int t = 0; t < 4; t++) {
            const uint64_t pc = (v4[t] & m55) + ((v4[t] >> 1) & m55);  // 2-bit pair counts
            sa += pc & m33;                                          // even pairs, 4-bit fields
            sb += (pc >> 2) & m33;                                   // odd pairs
        }
        const uint64_t ga = (sa + 0x5555555555555555ull) >> 3;  // nibble >= 3 -> bit 0 of nibble
        const uint64_t gb = (sb + 0x5555555555555555ull) >> 3;
        const uint32_t bits = spread16(compact_nibble_lsbs(ga)) | (spread16(compact_nibble_lsbs(gb)) << 1);
        acc |= static_cast<uint64_t>(bits) << (j0 & 63);
        if ((j0 & 63) == 32 || w == aW - 1 || 32 * (w + 1) >= bsy) {
            dst[j0 >> 6] = acc;
            written = (j0 >> 6) + 1;
            acc = 0;
        }
    }
    for (int w = written; w < bW; w++) dst[w] = 0;
    if (bsy & 63) dst[bW - 1] &= (1ull << (bsy & 63)) - 1;
}

// ------------------------------------------------------- surface + count

// Headers RLE4::compress emits for one finished run after `skip` empty
// voxels: 1023-skip headers, 63-solid headers, then the run's own
// (src/Rle4.cpp:166-182).
__device__ __forceinline__ int run_headers(int skip, int solid) {
    return (skip > 0 ? (skip - 1) / 1023 : 0) + (solid - 1) / 63 + 1;
}

// First index >= p whose bit equals `want` (bits past the words read as 0).
__device__ __forceinline__ int next_bit(const uint64_t* s, int W, int p, bool want) {
    int w = p >> 6;
    if (w >= W) return want ? W * 64 : p;
    uint64_t word = (want ? s[w] : ~s[w]) & (~0ull << (p & 63));
    while (!word) {
        if (++w >= W) return want ? W * 64 : W * 64;
        word = want ? s[w] : ~s[w];
    }
    return w * 64 + __ffsll(static_cast<long long>(word)) - 1;
}

struct LevelStats {
    unsigned long long heads, voxels;
    unsigned int top;  // smallest stored j, 0xffffffff if none
};

__global__ void __launch_bounds__(kThreads) surface_kernel(const uint64_t* __restrict__ cols, int sx, int sy, int sz,
                                                           int W, uint64_t* __restrict__ surf,
                                                           uint32_t* __restrict__ nwords,
                                                           uint16_t* __restrict__ nhead, LevelStats* stats) {
    const long long q = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x;
    unsigned long long heads = 0, voxels = 0;
    unsigned int top = 0xffffffffu;
    if (q < static_cast<long long>(sx) * sz) {
        const int x = static_cast<int>(q % sx), z = static_cast<int>(q / sx);
        const bool edge = x == 0 || z == 0 || x == sx - 1 || z == sz - 1;
        const uint64_t* self = cols + q * W;
        uint64_t s[kMaxWords];
        for (int w = 0; w < W; w++) {
            uint64_t v = self[w];
            if (!edge) {
                uint64_t inner = ~0ull;
                for (int dz = -1; dz <= 1; dz++)
                    for (int dx = -1; dx <= 1; dx++) {
                        const uint64_t* n = cols + ((static_cast<long long>(z) + dz) * sx + x + dx) * W;
                        const uint64_t below = (n[w] << 1) | (w > 0 ? n[w - 1] >> 63 : 0);      // bit j = n[j-1]
                        const uint64_t above = (n[w] >> 1) | (w + 1 < W ? n[w + 1] << 63 : 0);  // bit j = n[j+1]
                        inner &= n[w] & below & above;
                    }
                // j = 0 and j = sy-1 have an out-of-bounds neighbour: never interior
                if (w == 0) inner &= ~1ull;
                if (w == ((sy - 1) >> 6)) inner &= ~(1ull << ((sy - 1) & 63));
                v &= ~inner;
            }
            s[w] = v;
            surf[q * W + w] = v;
            voxels += __popcll(v);
        }
        int nh = 0, end = 0;
        for (int a = next_bit(s, W, 0, true); a < sy; a = next_bit(s, W, end, true)) {
            const int b = next_bit(s, W, a, false);
            if (top == 0xffffffffu) top = static_cast<unsigned>(a);
            nh += run_headers(a - end, b - a);
            end = b;
        }
        heads = static_cast<unsigned long long>(nh);
        nwords[q] = static_cast<uint32_t>(2 + nh + voxels);
        nhead[q] = static_cast<uint16_t>(nh);
    }
    // warp reduction, one atomic per warp
    for (int o = 16; o; o >>= 1) {
        heads += __shfl_down_sync(0xffffffffu, heads, o);
        voxels += __shfl_down_sync(0xffffffffu, voxels, o);
        top = min(top, __shfl_down_sync(0xffffffffu, top, o));
    }
    if ((threadIdx.x & 31) == 0) {
        if (heads) atomicAdd(&stats->heads, heads);
        if (voxels) atomicAdd(&stats->voxels, voxels);
        if (top != 0xffffffffu) atomicMin(&stats->top, top);
    }
}

// ------------------------------------------------------------------ scan

constexpr int kScanThreads = 1024;
constexpr int kScanItems = 4;
constexpr int kScanChunk = kScanThreads * kScanItems;

__device__ __forceinline__ unsigned long long block_exclusive_scan(unsigned long long v,
                                                                   unsigned long long* warp_sums,
                                                                   unsigned long long* total) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    unsigned long long x = v;
    for (int o = 1; o < 32; o <<= 1) {
        const unsigned long long y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) warp_sums[warp] = x;
    __syncthreads();
    if (warp == 0) {
        unsigned long long s = lane < (blockDim.x >> 5) ? warp_sums[lane] : 0;
        for (int o = 1; o < 32; o <<= 1) {
            const unsigned long long y = __shfl_up_sync(0xffffffffu, s, o);
            if (lane >= o) s += y;
        }
        warp_sums[lane] = s;  // inclusive
    }
    __syncthreads();
    const unsigned long long base = warp > 0 ? warp_sums[warp - 1] : 0;
    if (total) *total = warp_sums[(blockDim.x >> 5) - 1];
    return base + x - v;
}

// Block sums of kScanChunk-element chunks.
__global__ void __launch_bounds__(kScanThreads) scan_reduce_kernel(const uint32_t* __restrict__ v, long long n,
                                                                   unsigned long long* __restrict__ sums) {
    __shared__ unsigned long long ws[32];
    const long long base = static_cast<long long>(blockIdx.x) * kScanChunk + threadIdx.x * kScanItems;
    unsigned long long s = 0;
    for (int i = 0; i < kScanItems; i++)
        if (base + i < n) s += v[base + i];
    for (int o = 16; o; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x < 32) {
        unsigned long long t = threadIdx.x < (blockDim.x >> 5) ? ws[threadIdx.x] : 0;
        for (int o = 16; o; o >>= 1) t += __shfl_down_sync(0xffffffffu, t, o);
        if (threadIdx.x == 0) sums[blockIdx.x] = t;
    }
}

// Exclusive scan of the block sums in place (one block, any count); the
// grand total goes to *total.
__global__ void __launch_bounds__(kScanThreads) scan_sums_kernel(unsigned long long* sums, long long nb,
                                                                 unsigned long long* total) {
    __shared__ unsigned long long ws[32];
    __shared__ unsigned long long chunk_total;
    unsigned long long carry = 0;
    for (long long b0 = 0; b0 < nb; b0 += kScanThreads) {
        const long long i = b0 + threadIdx.x;
        const unsigned long long v = i < nb ? sums[i] : 0;
        const unsigned long long ex = block_exclusive_scan(v, ws, &chunk_total);
        if (i < nb) sums[i] = carry + ex;
        __syncthreads();
        carry += chunk_total;
        __syncthreads();
    }
    if (threadIdx.x == 0) *total = carry;
}

__global__ void __launch_bounds__(kScanThreads) scan_down_kernel(const uint32_t* __restrict__ v, long long n,
                                                                 const unsigned long long* __restrict__ sums,
                                                                 unsigned long long* __restrict__ out) {
    __shared__ unsigned long long ws[32];
    const long long base = static_cast<long long>(blockIdx.x) * kScanChunk + threadIdx.x * kScanItems;
    uint32_t item[kScanItems];
    unsigned long long s = 0;
    for (int i = 0; i < kScanItems; i++) {
        item[i] = base + i < n ? v[base + i] : 0u;
        s += item[i];
    }
    unsigned long long ex = block_exclusive_scan(s, ws, nullptr) + sums[blockIdx.x];
    for (int i = 0; i < kScanItems; i++) {
        if (base + i < n) out[base + i] = ex;
        ex += item[i];
    }
}

// ----------------------------------------------------------------- write

enum ColourMode { kColourGen = 0, kColourNormal = 1, kColourVolume = 2 };

struct WriteArgs {
    Consts c;                  // generator constants (kColourGen)
    const uint64_t* cols;      // this level's solid bits (kColourNormal)
    const uint16_t* volume;    // level-0 colours, Tree layout (kColourVolume)
    int sx0, sy0;              // level-0 size (kColourVolume)
    int mode, mip;
    int sx, sy, sz, W;
    unsigned long long words;  // slab words of the level
};

// The reference's normal-derived colour word without material bits
// (src/Rle4.cpp:134-161 with col1 == NULL): the negated centroid of the
// solid in-bounds 3x3x3 neighbours, normalised as vec3f::normalize, its y
// mapped to 0..255 and modulated by the (i ^ k) stripe pattern.
__device__ uint16_t normal_word(const WriteArgs& a, int x, int j, int z) {
    int mx = 0, my = 0, mz = 0;
    for (int dz = -1; dz <= 1; dz++) {
        const int zz = z + dz;
        if (zz < 0 || zz >= a.sz) continue;
        for (int dx = -1; dx <= 1; dx++) {
            const int xx = x + dx;
            if (xx < 0 || xx >= a.sx) continue;
            const uint64_t* n = a.cols + (static_cast<long long>(zz) * a.sx + xx) * a.W;
            for (int dy = -1; dy <= 1; dy++) {
                const int jj = j + dy;
                if (jj < 0 || jj >= a.sy) continue;
                if ((n[jj >> 6] >> (jj & 63)) & 1) {
                    mx += dx;
                    my += dy;
                    mz += dz;
                }
            }
        }
    }
    float cx = static_cast<float>(-mx), cy = static_cast<float>(my), cz = static_cast<float>(-mz);
    const float square = cx * cx + cy * cy + cz * cz;
    if (square <= 0.00001f) {
        cy = 0.0f;
    } else {
        const float len = 1.0f / sqrtf(square);
        cy *= len;
    }
    int ny = static_cast<int>(127.0f * cy + 128.0f);
    if (ny > 255) ny = 255;
    if (ny < 0) ny = 0;
    const int scale = 1 << a.mip;
    ny = (ny * (((((x * scale) ^ (z * scale)) >> 4) & 15) + 15)) >> 5;
    if (ny > 255) ny = 255;
    if (ny < 0) ny = 0;
    return static_cast<uint16_t>(ny);
}

// One column's words -- [run count][colour count][headers][colours] -- at
// dst (shared or global memory).  Returns the first header (valid when the
// column has runs).
__device__ __forceinline__ uint32_t write_column(const WriteArgs& a, const uint64_t* s, int x, int z, int nh,
                                                 int ncol, uint16_t* dst, bool* have_first_out) {
    dst[0] = static_cast<uint16_t>(nh);
    dst[1] = static_cast<uint16_t>(ncol);
    uint16_t* hp = dst + 2;
    uint16_t* cp = dst + 2 + nh;
    uint32_t first = 0;
    bool have_first = false;
    int tint = 0;
    if (a.mode == kColourGen) tint = rle::gen::tint(a.c, x << a.mip, z << a.mip);
    int end = 0;
    for (int r0 = next_bit(s, a.W, 0, true); r0 < a.sy; r0 = next_bit(s, a.W, end, true)) {
        const int r1 = next_bit(s, a.W, r0, false);
        // headers (src/Rle4.cpp:166-182)
        int skip = r0 - end, solid = r1 - r0;
        while (skip > 1023) {
            if (!have_first) { first = 1023; have_first = true; }
            *hp++ = 1023;
            skip -= 1023;
        }
        while (solid > 63) {
            const uint16_t h = static_cast<uint16_t>(63 * 1024 + (skip & 1023));
            if (!have_first) { first = h; have_first = true; }
            *hp++ = h;
            solid -= 63;
            skip = 0;
        }
        const uint16_t h = static_cast<uint16_t>((solid & 63) * 1024 + (skip & 1023));
        if (!have_first) { first = h; have_first = true; }
        *hp++ = h;
        // colours of the run's voxels, top down
        for (int j = r0; j < r1; j++) {
            uint16_t col;
            if (a.mode == kColourGen) {
                col = rle::gen::colour(a.c, tint, x << a.mip, j << a.mip, z << a.mip);
            } else if (a.mode == kColourNormal) {
                col = normal_word(a, x, j, z);
            } else {
                const long long idx = (static_cast<long long>(x) << a.mip) +
                                      (static_cast<long long>(j) << a.mip) * a.sx0 +
                                      (static_cast<long long>(z) << a.mip) * a.sx0 * a.sy0;
                col = a.volume[idx];
            }
            *cp++ = col;
        }
        end = r1;
    }
    *have_first_out = have_first;
    return first;
}

// u16 words a warp stages in shared memory before one coalesced copy.
constexpr int kStageWords = 2048;

// One thread per column.  The 32 columns of a warp are consecutive, so their
// words form one contiguous range of the slab array: the lanes write their
// columns into a shared-memory stage and the warp copies the range out with
// 4-byte stores (2-byte ones at its two ends, which may share a word with the
// neighbouring warps' ranges).  A warp whose range exceeds the stage writes
// its columns directly.
__global__ void __launch_bounds__(kThreads) write_kernel(const __grid_constant__ WriteArgs a,
                                                         const uint64_t* __restrict__ surf,
                                                         const unsigned long long* __restrict__ offsets,
                                                         const uint16_t* __restrict__ nhead,
                                                         uint16_t* __restrict__ slabs, uint2* __restrict__ table) {
    __shared__ uint16_t stage_all[kThreads / 32][kStageWords];
    uint16_t* stage = stage_all[threadIdx.x >> 5];
    const int lane = threadIdx.x & 31;
    const long long q = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x;
    const long long ncols = static_cast<long long>(a.sx) * a.sz;
    const bool valid = q < ncols;
    int x = 0, z = 0, nh = 0, ncol = 0;
    uint64_t s[kMaxWords];
    unsigned long long ofs = 0;
    if (valid) {
        x = static_cast<int>(q % a.sx);
        z = static_cast<int>(q / a.sx);
        for (int w = 0; w < a.W; w++) {
            s[w] = surf[q * a.W + w];
            ncol += __popcll(s[w]);
        }
        ofs = offsets[q];
        nh = nhead[q];
    }
    const unsigned long long col_end = ofs + 2u + static_cast<unsigned long long>(nh + ncol);
    // the warp's range: from lane 0's offset to the end of its last valid column
    const unsigned valid_mask = __ballot_sync(0xffffffffu, valid);
    if (valid_mask == 0) return;  // a warp past the level's last column
    const int last = 31 - __clz(valid_mask);
    const unsigned long long base = __shfl_sync(0xffffffffu, ofs, 0);
    const unsigned long long stop = __shfl_sync(0xffffffffu, col_end, last);
    const bool staged = stop - base <= static_cast<unsigned long long>(kStageWords);
    bool have_first = false;
    uint32_t first = 0;
    if (valid) {
        uint16_t* dst = staged ? stage + (ofs - base) : slabs + ofs;
        first = write_column(a, s, x, z, nh, ncol, dst, &have_first);
    }
    if (staged) {
        __syncwarp();
        const int n = static_cast<int>(stop - base);
        uint16_t* g = slabs + base;
        int start = 0;
        if ((reinterpret_cast<uintptr_t>(g) & 2u) && n > 0) {
            if (lane == 0) g[0] = stage[0];
            start = 1;
        }
        const int pairs = (n - start) >> 1;
        uint32_t* g32 = reinterpret_cast<uint32_t*>(g + start);
        for (int i = lane; i < pairs; i += 32)
            g32[i] = static_cast<uint32_t>(stage[start + 2 * i]) | (static_cast<uint32_t>(stage[start + 2 * i + 1]) << 16);
        if (((n - start) & 1) && lane == 0) g[n - 1] = stage[n - 1];
    }
    if (!valid) return;
    // RLE4::load's table entry (src/Rle4.cpp:285-314): the word after the
    // two counts is read as the first header even for an empty column, where
    // it is the next column's run count (or nothing past the level's end).
    if (!have_first) first = (ofs + 2 < a.words && q + 1 < ncols) ? nhead[q + 1] : 0u;
    table[q] = make_uint2(static_cast<uint32_t>(ofs), static_cast<uint32_t>(nh) + (first << 16));
}

// ---------------------------------------------------------------- driver

struct DevLevel {
    int sx = 0, sy = 0, sz = 0, W = 0;
    uint64_t* cols = nullptr;
};

struct Scratch {
    uint64_t* surf = nullptr;
    uint32_t* nwords = nullptr;
    uint16_t* nhead = nullptr;
    unsigned long long* offsets = nullptr;
    unsigned long long* sums = nullptr;
    LevelStats* stats = nullptr;  // device, one per level
    unsigned long long* total = nullptr;
    void release() {
        cudaFree(surf);
        cudaFree(nwords);
        cudaFree(nhead);
        cudaFree(offsets);
        cudaFree(sums);
        cudaFree(stats);
        cudaFree(total);
    }
};

struct Build {
    int device = 0;
    cudaStream_t stream = nullptr;
    std::vector<DevLevel> lv;
    Scratch sc;
    ~Build() {
        for (DevLevel& l : lv) cudaFree(l.cols);
        sc.release();
        if (stream) cudaStreamDestroy(stream);
    }
};

rle_status launch_check(const char* what) {
    const cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? RLE_OK : cuda_fail(e, what);
}

rle_status alloc_levels(Build& B, int sx, int sy, int sz, int nummaps) {
    B.lv.resize(nummaps);
    for (int m = 0; m < nummaps; m++) {
        DevLevel& L = B.lv[m];
        L.sx = sx >> m;
        L.sz = sz >> m;
        L.sy = m == 0 ? sy : B.lv[m - 1].sy / 2;
        L.W = (L.sy + 63) / 64;
        const size_t bytes = static_cast<size_t>(L.sx) * L.sz * L.W * 8;
        const cudaError_t e = cudaMalloc(&L.cols, bytes);
        if (e != cudaSuccess) return cuda_fail(e, "scene build: cudaMalloc(level bits)");
    }
    const long long n0 = static_cast<long long>(sx) * sz;
    const long long nb = (n0 + kScanChunk - 1) / kScanChunk;
    cudaError_t e;
    if ((e = cudaMalloc(&B.sc.surf, static_cast<size_t>(n0) * B.lv[0].W * 8)) != cudaSuccess ||
        (e = cudaMalloc(&B.sc.nwords, static_cast<size_t>(n0) * 4)) != cudaSuccess ||
        (e = cudaMalloc(&B.sc.nhead, static_cast<size_t>(n0) * 2)) != cudaSuccess ||
        (e = cudaMalloc(&B.sc.offsets, static_cast<size_t>(n0) * 8)) != cudaSuccess ||
        (e = cudaMalloc(&B.sc.sums, static_cast<size_t>(nb) * 8)) != cudaSuccess ||
        (e = cudaMalloc(&B.sc.stats, sizeof(LevelStats) * RLE_MAX_MIPS)) != cudaSuccess ||
        (e = cudaMalloc(&B.sc.total, 8)) != cudaSuccess)
        return cuda_fail(e, "scene build: cudaMalloc(scratch)");
    return RLE_OK;
}

rle_status build_mips(Build& B) {
    for (size_t m = 1; m < B.lv.size(); m++) {
        const DevLevel& A = B.lv[m - 1];
        const DevLevel& L = B.lv[m];
        halve_kernel<<<grid_for(static_cast<long long>(L.sx) * L.sz), kThreads, 0, B.stream>>>(
            A.cols, A.sx, A.W, L.cols, L.sx, L.sz, L.sy, L.W);
        const rle_status st = launch_check("halve_kernel");
        if (st != RLE_OK) return st;
    }
    return RLE_OK;
}

// Encodes every level into a new scene.
rle_status encode_levels(Build& B, WriteArgs base, rle_scene** out) {
    const int nummaps = static_cast<int>(B.lv.size());
    cudaError_t e = cudaMemsetAsync(B.sc.stats, 0, sizeof(LevelStats) * RLE_MAX_MIPS, B.stream);
    if (e != cudaSuccess) return cuda_fail(e, "scene build: cudaMemsetAsync");
    std::vector<LevelStats> init(RLE_MAX_MIPS);
    for (auto& s : init) s = LevelStats{0, 0, 0xffffffffu};
    e = cudaMemcpyAsync(B.sc.stats, init.data(), sizeof(LevelStats) * RLE_MAX_MIPS, cudaMemcpyHostToDevice, B.stream);
    if (e != cudaSuccess) return cuda_fail(e, "scene build: stats upload");
    e = cudaStreamSynchronize(B.stream);
    if (e != cudaSuccess) return cuda_fail(e, "scene build");

    rle_scene* s = new (std::nothrow) rle_scene();
    if (!s) return RLE_ERR_NO_MEMORY;
    s->device = B.device;
    s->nummaps = nummaps;
    s->height = B.lv[0].sy;
    long long top_all = 0x7fffffffLL;
    rle_status st = RLE_OK;
    for (int m = 0; m < nummaps && st == RLE_OK; m++) {
        const DevLevel& L = B.lv[m];
        const long long n = static_cast<long long>(L.sx) * L.sz;
        const long long nb = (n + kScanChunk - 1) / kScanChunk;
        surface_kernel<<<grid_for(n), kThreads, 0, B.stream>>>(L.cols, L.sx, L.sy, L.sz, L.W, B.sc.surf,
                                                                B.sc.nwords, B.sc.nhead, B.sc.stats + m);
        if ((st = launch_check("surface_kernel")) != RLE_OK) break;
        scan_reduce_kernel<<<static_cast<unsigned>(nb), kScanThreads, 0, B.stream>>>(B.sc.nwords, n, B.sc.sums);
        if ((st = launch_check("scan_reduce_kernel")) != RLE_OK) break;
        scan_sums_kernel<<<1, kScanThreads, 0, B.stream>>>(B.sc.sums, nb, B.sc.total);
        if ((st = launch_check("scan_sums_kernel")) != RLE_OK) break;
        scan_down_kernel<<<static_cast<unsigned>(nb), kScanThreads, 0, B.stream>>>(B.sc.nwords, n, B.sc.sums,
                                                                                    B.sc.offsets);
        if ((st = launch_check("scan_down_kernel")) != RLE_OK) break;
        unsigned long long words = 0;
        LevelStats ls;
        if ((e = cudaMemcpyAsync(&words, B.sc.total, 8, cudaMemcpyDeviceToHost, B.stream)) != cudaSuccess ||
            (e = cudaMemcpyAsync(&ls, B.sc.stats + m, sizeof(ls), cudaMemcpyDeviceToHost, B.stream)) != cudaSuccess ||
            (e = cudaStreamSynchronize(B.stream)) != cudaSuccess) {
            st = cuda_fail(e, "scene build: level totals");
            break;
        }
        if (words > 0xffffffffull) {
            rle::set_error("scene build: level %d needs %llu slab words (the column table holds 32-bit offsets)", m,
                           words);
            st = RLE_ERR_CAPACITY;
            break;
        }
        rle::Level& D = s->lv[m];
        D.sx = L.sx;
        D.sy = L.sy;
        D.sz = L.sz;
        D.words = words;
        const size_t tbytes = static_cast<size_t>(n) * 8;
        const size_t sbytes = static_cast<size_t>(words) * 2 + rle::kSlabPadBytes;
        if ((e = cudaMalloc(&D.d_table, tbytes)) != cudaSuccess) { st = cuda_fail(e, "scene build: cudaMalloc(table)"); break; }
        if ((e = cudaMalloc(&D.d_slabs, sbytes)) != cudaSuccess) { st = cuda_fail(e, "scene build: cudaMalloc(slabs)"); break; }
        // zero padding after the words (the writer covers every word)
        if ((e = cudaMemsetAsync(reinterpret_cast<char*>(D.d_slabs) + words * 2, 0, rle::kSlabPadBytes, B.stream)) !=
            cudaSuccess) {
            st = cuda_fail(e, "scene build: cudaMemsetAsync(padding)");
            break;
        }
        s->device_bytes += tbytes + sbytes;
        WriteArgs a = base;
        a.cols = L.cols;
        a.mip = m;
        a.sx = L.sx;
        a.sy = L.sy;
        a.sz = L.sz;
        a.W = L.W;
        a.words = words;
        write_kernel<<<grid_for(n), kThreads, 0, B.stream>>>(a, B.sc.surf, B.sc.offsets, B.sc.nhead, D.d_slabs,
                                                             reinterpret_cast<uint2*>(D.d_table));
        if ((st = launch_check("write_kernel")) != RLE_OK) break;
        if (m == 0) {
            s->run_headers = ls.heads;
            s->surface_voxels = ls.voxels;
        }
        // same clamp as the loader: an empty level reports INT_MAX
        const int top = ls.top > 0x7fffffffu ? 0x7fffffff : static_cast<int>(ls.top);
        const long long top0 = static_cast<long long>(top) << m;
        if (top0 < top_all) top_all = top0;
    }
    if (st == RLE_OK && (e = cudaStreamSynchronize(B.stream)) != cudaSuccess) st = cuda_fail(e, "scene build");
    if (st != RLE_OK) {
        rle_scene_free(s);
        return st;
    }
    s->top_index = static_cast<int>(top_all);
    *out = s;
    return RLE_OK;
}

struct DeviceGuard {
    int prev = -1;
    explicit DeviceGuard() { cudaGetDevice(&prev); }
    ~DeviceGuard() {
        if (prev >= 0) cudaSetDevice(prev);
    }
};

rle_status begin(Build& B, int device) {
    int ndev = 0;
    cudaError_t e = cudaGetDeviceCount(&ndev);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGetDeviceCount");
    if (device < 0 || device >= ndev) {
        rle::set_error("scene build: device %d of %d", device, ndev);
        return RLE_ERR_INVALID_ARG;
    }
    B.device = device;
    if ((e = cudaSetDevice(device)) != cudaSuccess) return cuda_fail(e, "cudaSetDevice");
    if ((e = cudaStreamCreateWithFlags(&B.stream, cudaStreamNonBlocking)) != cudaSuccess)
        return cuda_fail(e, "cudaStreamCreate");
    return RLE_OK;
}

}  // namespace

extern "C" rle_status rle_scenegen_device(const rle_scenegen_params* p, int device, rle_scene** out) {
    if (!out) return RLE_ERR_INVALID_ARG;
    *out = nullptr;
    rle_status st = rle::scenegen_check(p);
    if (st != RLE_OK) return st;
    DeviceGuard guard;
    Build B;
    if ((st = begin(B, device)) != RLE_OK) return st;
    if ((st = alloc_levels(B, p->sx, p->sy, p->sz, p->nummaps)) != RLE_OK) return st;
    GenArgs g;
    g.c = rle::scenegen_consts(*p);
    rle::scenegen_perm(p->seed, g.perm);
    g.W = B.lv[0].W;
    gen_columns_kernel<<<grid_for(static_cast<long long>(p->sx) * p->sz), kThreads, 0, B.stream>>>(g, B.lv[0].cols);
    if ((st = launch_check("gen_columns_kernel")) != RLE_OK) return st;
    if ((st = build_mips(B)) != RLE_OK) return st;
    WriteArgs a;
    std::memset(&a, 0, sizeof(a));
    a.c = g.c;
    a.mode = kColourGen;
    return encode_levels(B, a, out);
}

extern "C" rle_status rle_encode_device(const uint8_t* d_bits, const uint16_t* d_colours, int sx, int sy, int sz,
                                        int nummaps, int device, rle_scene** out) {
    if (!out) return RLE_ERR_INVALID_ARG;
    *out = nullptr;
    auto pow2 = [](int v) { return v >= 8 && (v & (v - 1)) == 0; };
    if (!d_bits || !pow2(sx) || !pow2(sz) || sx > 65536 || sz > 65536 || sy < 1 || sy > 1024 || nummaps < 1 ||
        nummaps > RLE_MAX_MIPS || (sx >> (nummaps - 1)) < 1 || (sz >> (nummaps - 1)) < 1 ||
        (sy >> (nummaps - 1)) < 1) {
        rle::set_error("rle_encode_device: bits required; sx, sz powers of two in 8..65536, sy in 1..1024, "
                       "1..%d levels that keep every dimension >= 1",
                       RLE_MAX_MIPS);
        return RLE_ERR_INVALID_ARG;
    }
    DeviceGuard guard;
    Build B;
    rle_status st = begin(B, device);
    if (st != RLE_OK) return st;
    if ((st = alloc_levels(B, sx, sy, sz, nummaps)) != RLE_OK) return st;
    const long long n = static_cast<long long>(sx) * sz * B.lv[0].W;
    transpose_kernel<<<grid_for(n), kThreads, 0, B.stream>>>(d_bits, sx, sy, sz, B.lv[0].W, B.lv[0].cols);
    if ((st = launch_check("transpose_kernel")) != RLE_OK) return st;
    if ((st = build_mips(B)) != RLE_OK) return st;
    WriteArgs a;
    std::memset(&a, 0, sizeof(a));
    a.mode = d_colours ? kColourVolume : kColourNormal;
    a.volume = d_colours;
    a.sx0 = sx;
    a.sy0 = sy;
    return encode_levels(B, a, out);
}
