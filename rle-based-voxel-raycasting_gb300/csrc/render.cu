// Column-ray traversal on sm_103a.
//
// One thread casts one column ray through the 2D grid of RLE columns with
// the reference's 2D DDA, picks the mip level by distance, walks each
// visited column's run headers, projects solid runs to screen spans and
// fills them with perspective-correct colour and depth, culling with a
// floating horizon and a per-ray occupancy bitmask in shared memory
// (Render::render_line, src/Cuda_Render.h:96-737, with the switches
// FLOATING_HORIZON, XFLOATING_HORIZON and SHAREMEMCLIP of src/core.h:24-32).
//
// Arithmetic: compiled with -fmad=false and IEEE division/square root, every
// float operation is the single IEEE operation the reference performs, in
// its order, so results match the reference's host build bit for bit.  The
// per-frame sines and cosines arrive precomputed from the host (the
// reference evaluates the same host-side values per ray).
//
// Output, per ray row (ray-major, `S` samples): every sample is written
// exactly once -- coloured samples when they are drawn, the rest at the end
// (sky 0x00ff8844 inside the ray's clip range, 0 outside).  The occupancy
// bitmask (1 bit per sample) says which is which.  The reference instead
// clears the clip range to sky first and never touches samples outside it.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>

#include "rle_internal.h"

namespace rle {
namespace {

constexpr uint32_t kSky = 0x00ff8844u;

struct Counts {
    unsigned long long cells = 0, fetched = 0, headers = 0, runs = 0, spans = 0, pixels = 0;
};

// Occupancy bitmask of one ray: word w of thread t at smem[w * stride + t],
// so lanes touching the same word index hit distinct banks.
struct Mask {
    uint32_t* base;
    int stride;
    __device__ __forceinline__ bool get(int y) const { return (base[(y >> 5) * stride] >> (y & 31)) & 1u; }
    __device__ __forceinline__ void set(int y) const { base[(y >> 5) * stride] |= 1u << (y & 31); }
    __device__ __forceinline__ uint32_t word(int w) const { return base[w * stride]; }
    // first y in [y, end) whose bit is clear, or end
    __device__ __forceinline__ int first_clear(int y, int end) const {
        while (y < end) {
            const uint32_t free_bits = ~word(y >> 5) >> (y & 31);
            if (free_bits) {
                const int r = y + (__ffs(free_bits) - 1);
                return r < end ? r : end;
            }
            y = (y | 31) + 1;
        }
        return end;
    }
};

struct F3 {
    float x, y, z;
};
__device__ __forceinline__ F3 f3(float x, float y, float z) { return F3{x, y, z}; }
__device__ __forceinline__ F3 add(F3 a, F3 b) { return f3(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ F3 sub(F3 a, F3 b) { return f3(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ F3 mul(F3 a, float s) { return f3(a.x * s, a.y * s, a.z * s); }

// Render::LineScale (src/Cuda_Render.h:39-52)
__device__ __forceinline__ float line_scale(F3 in, F3 c, float cmax, float cmin) {
    float sx = 1, sy = 1;
    if (c.x > 1) sx = (1 - in.x) / (c.x - in.x);
    if (c.x < 0) sx = in.x / (in.x - c.x);
    if (c.y > cmax) sy = (cmax - in.y) / (c.y - in.y);
    if (c.y < cmin) sy = (-cmin + in.y) / (in.y - c.y);
    return (sx < sy) ? sx : sy;
}

__device__ __forceinline__ F3 to3d(const RayParams& P, F3 v) {
    return f3(P.to3d[0][0] * v.x + P.to3d[1][0] * v.y + P.to3d[2][0] * v.z + P.to3d[3][0],
              P.to3d[0][1] * v.x + P.to3d[1][1] * v.y + P.to3d[2][1] * v.z + P.to3d[3][1],
              P.to3d[0][2] * v.x + P.to3d[1][2] * v.y + P.to3d[2][2] * v.z + P.to3d[3][2]);
}

// Casts ray x.  Writes coloured samples; returns the clip range through
// ymin/ymax (ymax < ymin: the ray covers no samples).
template <bool kHits, bool kCount>
__device__ __forceinline__ void cast(const RayParams& P, int x, const Mask& mask, uint32_t* row, float* drow,
                                     rle_hit* hrow, int& ymin_out, int& ymax_out, Counts& cnt) {
    const int S = P.S;
    const float res_x2 = static_cast<float>(S / 2);
    const float res_y2 = res_x2;

    // ---- 2D line of this ray in its fan, and its horizontal direction ----
    const int r0 = P.res[0], r1 = P.res[1] + r0, r2 = P.res[2] + r1;
    int q = 0;
    if (x >= r2) q = 3;
    else if (x >= r1) q = 2;
    else if (x >= r0) q = 1;
    float qofs = static_cast<float>(x);
    if (q == 1) qofs -= static_cast<float>(r0);
    if (q == 2) qofs -= static_cast<float>(r1);
    if (q == 3) qofs -= static_cast<float>(r2);
    const float a = qofs / static_cast<float>(P.res[q]);
    F3 p1 = f3(P.p5x, P.p5y, P.p5z);
    const F3 n0 = f3(P.p_no[2 * q][0], P.p_no[2 * q][1], P.p_no[2 * q][2]);
    const F3 n1 = f3(P.p_no[2 * q + 1][0], P.p_no[2 * q + 1][1], P.p_no[2 * q + 1][2]);
    F3 p2 = add(n0, mul(sub(n1, n0), a));
    {  // ClipLine (src/Cuda_Render.h:54-65)
        float s = line_scale(p1, p2, P.clip_max, P.clip_min);
        const F3 c2 = add(p1, mul(sub(p2, p1), s));
        s = line_scale(p2, p1, P.clip_max, P.clip_min);
        const F3 c1 = add(p2, mul(sub(p1, p2), s));
        p1 = c1;
        p2 = c2;
    }
    const F3 p1_3d = to3d(P, mul(p1, 4.0f));
    const F3 p2_3d = to3d(P, mul(p2, 4.0f));
    F3 d = sub(mul(add(p1_3d, p2_3d), 0.5f), f3(P.p4[0], P.p4[1], P.p4[2]));
    d.y = 0;
    {
        const float inv = 1.0f / sqrtf(d.x * d.x + d.y * d.y + d.z * d.z);
        d = mul(d, inv);
    }
    {
        const float xx = P.cos_ny * d.x + P.sin_ny * d.z;
        const float zz = P.cos_ny * d.z - P.sin_ny * d.x;
        d.x = xx;
        d.z = zz;
    }
    const float ray_x = d.x, ray_z = d.z;
    const bool vertical = q < 2;
    const float sin_x = P.sin_x, cos_x = P.cos_x;

    // ---- reverse texturing and the ray's sample range (:203-250) ----
    bool reverse = false;
    if (vertical && ray_z <= 0) reverse = true;
    if (!vertical && ray_x <= 0 && sin_x > 0) reverse = true;
    if (!vertical && ray_x > 0 && sin_x < 0) reverse = true;
    float rmul = reverse ? -P.focal : P.focal;
    if (vertical) rmul = -rmul;
    const int p_add = reverse ? 1 : -2;
    int a1x = static_cast<int>(static_cast<float>(S) * p1.x) + p_add;
    int a1y = static_cast<int>(static_cast<float>(S) * p1.y) + p_add;
    int a2x = static_cast<int>(static_cast<float>(S) * p2.x) - p_add;
    int a2y = static_cast<int>(static_cast<float>(S) * p2.y) - p_add;
    a1x = min(max(a1x, 0), S - 1);
    a1y = min(max(a1y, 0), S - 1);
    a2x = min(max(a2x, 0), S - 1);
    a2y = min(max(a2y, 0), S - 1);
    if (a1y == a2y) return;
    int ymin = vertical ? S - 1 - a1y : S - 1 - a1x;
    int ymax = vertical ? S - 1 - a2y : S - 1 - a2x;
    if (reverse) {
        ymin = S - 1 - ymin;
        ymax = S - 1 - ymax;
    }
    if (ymin > ymax) {
        const int t = ymin;
        ymin = ymax;
        ymax = t;
    }
    if (ymin >= ymax) return;
    ymin_out = ymin;
    ymax_out = ymax;

    // ---- DDA set-up (:270-304) ----
    const float dir_x = ray_x * P.cos_y + ray_z * P.sin_y;
    const float dir_y = ray_x * P.sin_y - ray_z * P.cos_y;
    float fix_x = -1, fix_y = -1, sign_x = -1, sign_y = -1;
    float frac_x = P.posx - static_cast<float>(static_cast<int>(P.posx));
    float frac_y = P.posz - static_cast<float>(static_cast<int>(P.posz));
    if (dir_x >= 0) { fix_x = 0; sign_x = 1; frac_x = 1 - frac_x; }
    if (dir_y >= 0) { fix_y = 0; sign_y = 1; frac_y = 1 - frac_y; }
    float g0y = dir_y / fabsf(dir_x), g0x = sign_x;
    float g1x = dir_x / fabsf(dir_y), g1y = sign_y;
    float i0x = g0x * frac_x, i0y = g0y * frac_x;
    float i1x = g1x * frac_y, i1y = g1y * frac_y;
    float gd0 = sqrtf(g0x * g0x + g0y * g0y);
    float gd1 = sqrtf(g1x * g1x + g1y * g1y);
    float dd0 = sqrtf(i0x * i0x + i0y * i0y);
    float dd1 = sqrtf(i1x * i1x + i1y * i1y);
    float pbx = 0, pby = 0, dd_before = 0;
    float pnx = 0, pny = 0, dd_now = 0;
    int index = 0, index_before = 0;

    int mip = 0;
    int gridx = P.gridx0, gridz = P.gridz0;
    const uint2* table = P.table[0];
    const uint16_t* slab_base = P.slabs[0];
    const float pos3d_z_add = sin_x;
    const float pos3d_y_add = (vertical ? cos_x : 0.0f) * rmul;
    const float mountain = P.posy;
    float z = 0, dz = 1;
    float y_map_switch = P.posy;
    int mapswitch = P.mapswitch0;
    const float zfar = static_cast<float>(P.z_far);

    for (;;) {
        while (z > static_cast<float>(mapswitch) || y_map_switch > 512.0f) {
            y_map_switch = y_map_switch * 0.5f;
            if (mip < P.nummaps - 1) {
                mip++;
                gridx >>= 1;
                gridz >>= 1;
                table = P.table[mip];
                slab_base = P.slabs[mip];
            }
            g0x *= 2; g0y *= 2; g1x *= 2; g1y *= 2;
            gd0 *= 2; gd1 *= 2;
            mapswitch *= 2;
            dz *= 2;
        }
        z += dz;
        if (z > zfar) return;
        if (ymin >= ymax) return;

        dd_before = dd_now;
        pbx = pnx;
        pby = pny;
        index_before = index;
        if (dd1 < dd0) {
            dd_now = dd1;
            index = 1;
            dd1 += gd1;
            pnx = i1x; pny = i1y;
            i1x += g1x;
            i1y += g1y;
        } else {
            dd_now = dd0;
            index = 0;
            pnx = i0x; pny = i0y;
            dd0 += gd0;
            i0x += g0x;
            i0y += g0y;
        }
        if (kCount) cnt.cells++;
        const int fxi = static_cast<int>(static_cast<float>(1 - index_before) * fix_x);
        const int fzi = static_cast<int>(static_cast<float>(index_before) * fix_y);
        const float dd_delta = dd_now - dd_before;
        const float vs_x = ray_x * dd_before;
        const float vs_z = ray_z * dd_before;
        const int voxel_x = static_cast<int>(P.posx + pbx) + fxi;
        const int voxel_z = static_cast<int>(P.posz + pby) + fzi;
        const int vx = (voxel_x >> mip) & (gridx - 1);
        const int vz = (voxel_z >> mip) & (gridz - 1);
        const float corr_x = ray_x * dd_delta;
        const float corr_z = ray_z * dd_delta;
        const float pz = cos_x * vs_z + sin_x * mountain;
        float py = vertical ? cos_x * mountain - sin_x * vs_z : vs_x;
        py *= rmul;

        // clip top (:467)
        if (pz * res_y2 + py <= pz * static_cast<float>(ymin)) continue;

        const uint2 entry = __ldg(&table[static_cast<size_t>(vx) + static_cast<size_t>(vz) * gridx]);
        if (kCount) cnt.fetched++;
        const float czz = cos_x * corr_z;
        float cyy = vertical ? -sin_x * corr_z : corr_x;
        cyy *= rmul;

        const uint16_t* hdr = slab_base + 2 + entry.x;
        const int nruns = entry.y & 0xffffu;
        const uint16_t* colours = hdr + nruns;
        uint32_t sti = entry.y >> 16;
        int sg = 0;       // sti_general: height below the next run, level-0 units
        float tex = 0;    // colour index of the next run's first voxel

        for (int r = 0; r < nruns; r++) {
            if (r > 0) {
                sti = __ldg(&hdr[r]);
                if (kCount) cnt.headers++;
            }
            int solid = static_cast<int>(sti >> 10);
            sg += static_cast<int>(sti & 1023u) << mip;
            if (solid == 0) continue;
            const int texture = static_cast<int>(tex);
            tex += static_cast<float>(solid);
            solid <<= mip;
            const float sgs = static_cast<float>(sg);  // run bottom
            sg += solid;
            const float sgf = static_cast<float>(sg);  // run top
            if (kCount) cnt.runs++;

            float czz1 = pz, cyy1 = py;
            if (mountain + sgs >= 0) { czz1 += czz; cyy1 += cyy; }
            const float pz1 = czz1 + pos3d_z_add * sgs;
            if (pz1 <= 0) continue;
            const float py1 = cyy1 + pos3d_y_add * sgs;
            int scr_y2 = static_cast<int>(res_y2 + py1 / pz1);
            if (scr_y2 <= ymin) break;

            float czz2 = pz, cyy2 = py;
            if (mountain + sgf < 0) { czz2 += czz; cyy2 += cyy; }
            const float pz2 = czz2 + pos3d_z_add * sgf;
            if (pz2 <= 0) continue;
            const float py2 = cyy2 + pos3d_y_add * sgf;
            int scr_y1 = static_cast<int>(res_y2 + py2 / pz2 - 1);
            if (scr_y1 >= ymax) continue;

            // floating horizon (:563-580)
            if (scr_y2 >= ymax) {
                scr_y2 = ymax;
                ymax = scr_y1;
            }
            if (scr_y1 <= ymin) {
                scr_y1 = ymin;
                ymin = scr_y2;
                ymin = mask.first_clear(ymin, ymax > ymin ? ymax : ymin);
            }
            int y = mask.first_clear(scr_y1, scr_y2);
            if (y >= scr_y2) continue;

            // perspective-correct interpolation (:645-680)
            const float pz1r = pz + pos3d_z_add * sgs;
            const float py1r = py + pos3d_y_add * sgs;
            const float pz2r = pz + pos3d_z_add * sgf;
            const float py2r = py + pos3d_y_add * sgf;
            const float scr_y2r = res_y2 + py1r / pz1r;
            const float scr_y1r = res_y2 + py2r / pz2r;
            const float u1z = tex / pz2r;
            float u2dz = static_cast<float>(texture) / pz1r - u1z;
            const float onez1 = 1 / pz2r;
            float onedz2 = 1 / pz1r - onez1;
            u2dz /= scr_y2r - scr_y1r;
            onedz2 /= scr_y2r - scr_y1r;
            if (kCount) cnt.spans++;
            const float mult = static_cast<float>(y + 1) - scr_y1r;
            float uz = u1z + u2dz * mult;
            float onez = onez1 + onedz2 * mult;
            const float umin = static_cast<float>(texture);
            const float umax = static_cast<float>(static_cast<double>(tex) - 1.0);
            for (; y < scr_y2; ++y, uz += u2dz, onez += onedz2) {
                if (mask.get(y)) continue;
                const uint32_t u = static_cast<uint32_t>(fminf(fmaxf(uz / onez, umin), umax));
                const float depth = 1 / onez;
                const uint32_t real_z = static_cast<uint32_t>(static_cast<int>(depth) & 0xfffe);
                const uint32_t c16 = __ldg(&colours[u]);
                row[y] = c16 + (real_z << 16);
                drow[y] = depth;
                if (kHits) {
                    rle_hit h;
                    h.x = static_cast<uint16_t>(vx);
                    h.z = static_cast<uint16_t>(vz);
                    h.y = static_cast<uint16_t>((static_cast<int>(sgs) >> mip) + static_cast<int>(u - static_cast<uint32_t>(texture)));
                    h.mip = static_cast<uint8_t>(mip);
                    h.flags = 1;
                    hrow[y] = h;
                }
                if (kCount) cnt.pixels++;
                mask.set(y);
            }
        }
    }
}

template <bool kHits, bool kCount>
__global__ void raycast_kernel(const __grid_constant__ RayParams P) {
    extern __shared__ uint32_t smem[];
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    Counts cnt;
    if (x < P.rays) {
        const int S = P.S;
        const int words = (S + 31) >> 5;
        const Mask mask{smem + threadIdx.x, static_cast<int>(blockDim.x)};
        for (int w = 0; w < words; w++) mask.base[w * mask.stride] = 0;
        uint32_t* row = P.raybuf + static_cast<size_t>(x) * S;
        float* drow = P.raydepth + static_cast<size_t>(x) * S;
        rle_hit* hrow = kHits ? P.rayhit + static_cast<size_t>(x) * S : nullptr;
        int ymin = 0, ymax = -1;
        cast<kHits, kCount>(P, x, mask, row, drow, hrow, ymin, ymax, cnt);
        // every sample not coloured: sky inside the clip range, none outside
        for (int y = 0; y < S; y++) {
            if (mask.get(y)) continue;
            const bool in = y >= ymin && y <= ymax;
            row[y] = in ? kSky : 0u;
            drow[y] = in ? INFINITY : 0.0f;
            if (kHits) {
                rle_hit h = {0, 0, 0, 0, static_cast<uint8_t>(in ? 2 : 0)};
                hrow[y] = h;
            }
        }
    }
    if (kCount) {
        unsigned long long v[6] = {cnt.cells, cnt.fetched, cnt.headers, cnt.runs, cnt.spans, cnt.pixels};
        for (int i = 0; i < 6; i++) {
            unsigned long long s = v[i];
            for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
            if ((threadIdx.x & 31) == 0 && s) atomicAdd(&reinterpret_cast<unsigned long long*>(P.counters)[i], s);
        }
    }
}

template <bool kHits, bool kCount>
rle_status launch_variant(const RayParams& p, cudaStream_t stream) {
    const int words = (p.S + 31) >> 5;
    // 128 threads per block while their bitmasks fit in 200 KB of shared memory
    int threads = 128;
    while (threads > 32 && static_cast<size_t>(threads) * words * 4 > 200 * 1024) threads -= 32;
    const size_t smem = static_cast<size_t>(threads) * words * 4;
    if (smem > 227 * 1024) {
        set_error("rle_render_rays: %d samples per ray exceed the shared-memory bitmask", p.S);
        return RLE_ERR_CAPACITY;
    }
    cudaError_t e = cudaFuncSetAttribute(raycast_kernel<kHits, kCount>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         static_cast<int>(smem));
    if (e != cudaSuccess) {
        set_error("cudaFuncSetAttribute: %s", cudaGetErrorString(e));
        return RLE_ERR_CUDA;
    }
    const int blocks = (p.rays + threads - 1) / threads;
    raycast_kernel<kHits, kCount><<<blocks, threads, smem, stream>>>(p);
    e = cudaGetLastError();
    if (e != cudaSuccess) {
        set_error("raycast launch: %s", cudaGetErrorString(e));
        return RLE_ERR_CUDA;
    }
    return RLE_OK;
}

}  // namespace

rle_status launch_raycast(const RayParams& p, void* stream) {
    if (p.rays <= 0) return RLE_OK;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const bool hits = p.rayhit != nullptr, count = p.counters != nullptr;
    if (hits && count) return launch_variant<true, true>(p, s);
    if (hits) return launch_variant<true, false>(p, s);
    if (count) return launch_variant<false, true>(p, s);
    return launch_variant<false, false>(p, s);
}

}  // namespace rle
