// Column-ray traversal on sm_103a.
//
// Algorithm (Render::render_line, src/Cuda_Render.h:96-737, with the
// switches FLOATING_HORIZON, XFLOATING_HORIZON and SHAREMEMCLIP of
// src/core.h:24-32): a column ray marches the 2D grid of RLE columns with a
// 2D DDA, picks the mip level by distance, walks each visited column's run
// headers, projects solid runs to screen spans and fills them with
// perspective-correct colour and depth, culling with a floating horizon and
// an occupancy bitmask.
//
// Parallel decomposition: a group of G lanes (G = 8, 16 or 32; 32/G rays
// per warp) owns one ray.  The ray is processed in chunks of G DDA steps,
// the next chunk's DDA and table fetches issued before this chunk's merge:
//   1. all lanes step the DDA in lockstep (the DDA is a chain of IEEE
//      additions, so every lane repeats the same operations) and lane k
//      keeps the state of step k; the state before it comes from lane k-1;
//   2. each lane, in parallel, derives its cell, pre-culls it against the
//      horizon at the start of the chunk, fetches the column-table entry,
//      scans the column's runs and records in shared memory the runs the
//      walk could still draw, with their span constants; a __ballot_sync
//      gives the cells that may draw;
//   3. the group walks those cells in order (values broadcast with
//      __shfl_sync) and applies the exact sequential horizon logic to the
//      recorded runs; span pixels are interpolated and written by all G
//      lanes at once, or, for short spans, claimed in the bitmask and
//      coloured later G samples at a time.
// The pre-cull is conservative: the horizon only closes (ymin grows, ymax
// shrinks), so a cell or run culled at the chunk start would be culled at
// its turn too.  The result is the sequential algorithm's, bit for bit.
//
// Arithmetic: compiled with -fmad=false and IEEE division/square root, each
// float operation is the single IEEE operation the reference performs, in
// its order.  Per-frame sines/cosines come precomputed from the host.
//
// Output, per ray row (ray-major, S samples): every sample is written once
// -- coloured samples when drawn, the rest in a final coalesced pass (sky
// 0x00ff8844 inside the ray's clip range, 0 outside), guided by the bitmask.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>

#include "rle_internal.h"

namespace rle {
namespace {

constexpr uint32_t kSky = 0x00ff8844u;

// Debug builds with RLE_BOUNDS_CHECK range-check every column-table, slab
// and ray-buffer index: a failed check records its code (and the first
// index) in g_bounds and skips the access (reads return 0) instead of
// touching memory outside the scene or the frame.
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

struct Counts {
    unsigned long long cells = 0, fetched = 0, headers = 0, runs = 0, spans = 0, pixels = 0;
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

// Device-wide nanosecond clock and the SM a thread runs on (profiling).
__device__ __forceinline__ uint64_t global_ns() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}
__device__ __forceinline__ uint32_t sm_id() {
    uint32_t s;
    asm volatile("mov.u32 %0, %%smid;" : "=r"(s));
    return s;
}

// Run-header staging (staging depth 2 or 3; the variants built with kStage):
// 2 stages a cell's header line in L2, 3 in L1, ahead of the scan that reads
// it.  Depth 1 variants carry none of this code: a runtime test in the chunk
// loop measured 1% slower single frames and 4% slower batches at depth 1.
__device__ __forceinline__ void stage_headers(const uint16_t* h, int staging) {
    if (staging == 2) asm volatile("prefetch.global.L2 [%0];" ::"l"(h));
    else if (staging >= 3) asm volatile("prefetch.global.L1 [%0];" ::"l"(h));
}

// First lane of the group a lane mask describes.
__device__ __forceinline__ int lane_base(unsigned gmask) { return __ffs(gmask) - 1; }

// Occupancy bitmask of one ray in shared memory (1 bit per sample).
struct Mask {
    uint32_t* w;
    __device__ __forceinline__ bool get(int y) const { return (w[y >> 5] >> (y & 31)) & 1u; }
    // first y in [y, end) whose bit is clear, or end
    __device__ __forceinline__ int first_clear(int y, int end) const {
        while (y < end) {
            const uint32_t free_bits = ~w[y >> 5] >> (y & 31);
            if (free_bits) {
                const int r = y + (__ffs(free_bits) - 1);
                return r < end ? r : end;
            }
            y = (y | 31) + 1;
        }
        return end;
    }
};

// Per-ray constants after set-up.
struct Ray {
    float ray_x, ray_z;
    float rmul;          // res_x2_mul_reverse (with the field-of-view focal length)
    float pos3d_z_add, pos3d_y_add;
    float fix_x, fix_y;
    bool vertical;
    int ymin, ymax;      // clip range at the start (ymax < ymin: the ray is empty)
};

// Ray set-up: fan, 2D line, 3D direction, sample range, DDA start
// (src/Cuda_Render.h:129-304).  Returns false if the ray covers no samples.
struct Dda {
    float g0x, g0y, g1x, g1y, gd0, gd1;
    float i0x, i0y, i1x, i1y, dd0, dd1;
    float dd_now, pnx, pny;
    int index;
};

__device__ __forceinline__ bool setup_ray(const RayParams& P, int x, Ray& R, Dda& D) {
    const int S = P.S;
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
    R.ray_x = d.x;
    R.ray_z = d.z;
    R.vertical = q < 2;
    const float sin_x = P.sin_x, cos_x = P.cos_x;

    bool reverse = false;
    if (R.vertical && R.ray_z <= 0) reverse = true;
    if (!R.vertical && R.ray_x <= 0 && sin_x > 0) reverse = true;
    if (!R.vertical && R.ray_x > 0 && sin_x < 0) reverse = true;
    float rmul = reverse ? -P.focal : P.focal;
    if (R.vertical) rmul = -rmul;
    R.rmul = rmul;
    R.pos3d_z_add = sin_x;
    R.pos3d_y_add = (R.vertical ? cos_x : 0.0f) * rmul;
    R.ymin = 0;
    R.ymax = -1;
    const int p_add = reverse ? 1 : -2;
    int a1x = static_cast<int>(static_cast<float>(S) * p1.x) + p_add;
    int a1y = static_cast<int>(static_cast<float>(S) * p1.y) + p_add;
    int a2x = static_cast<int>(static_cast<float>(S) * p2.x) - p_add;
    int a2y = static_cast<int>(static_cast<float>(S) * p2.y) - p_add;
    a1x = min(max(a1x, 0), S - 1);
    a1y = min(max(a1y, 0), S - 1);
    a2x = min(max(a2x, 0), S - 1);
    a2y = min(max(a2y, 0), S - 1);
    if (a1y == a2y) return false;
    int ymin = R.vertical ? S - 1 - a1y : S - 1 - a1x;
    int ymax = R.vertical ? S - 1 - a2y : S - 1 - a2x;
    if (reverse) {
        ymin = S - 1 - ymin;
        ymax = S - 1 - ymax;
    }
    if (ymin > ymax) {
        const int t = ymin;
        ymin = ymax;
        ymax = t;
    }
    if (ymin >= ymax) return false;
    R.ymin = ymin;
    R.ymax = ymax;

    const float dir_x = R.ray_x * P.cos_y + R.ray_z * P.sin_y;
    const float dir_y = R.ray_x * P.sin_y - R.ray_z * P.cos_y;
    float sign_x = -1, sign_y = -1;
    R.fix_x = -1;
    R.fix_y = -1;
    float frac_x = P.posx - static_cast<float>(static_cast<int>(P.posx));
    float frac_y = P.posz - static_cast<float>(static_cast<int>(P.posz));
    if (dir_x >= 0) { R.fix_x = 0; sign_x = 1; frac_x = 1 - frac_x; }
    if (dir_y >= 0) { R.fix_y = 0; sign_y = 1; frac_y = 1 - frac_y; }
    D.g0y = dir_y / fabsf(dir_x);
    D.g0x = sign_x;
    D.g1x = dir_x / fabsf(dir_y);
    D.g1y = sign_y;
    D.i0x = D.g0x * frac_x;
    D.i0y = D.g0y * frac_x;
    D.i1x = D.g1x * frac_y;
    D.i1y = D.g1y * frac_y;
    D.gd0 = sqrtf(D.g0x * D.g0x + D.g0y * D.g0y);
    D.gd1 = sqrtf(D.g1x * D.g1x + D.g1y * D.g1y);
    D.dd0 = sqrtf(D.i0x * D.i0x + D.i0y * D.i0y);
    D.dd1 = sqrtf(D.i1x * D.i1x + D.i1y * D.i1y);
    D.dd_now = 0;
    D.pnx = 0;
    D.pny = 0;
    D.index = 0;
    return true;
}

// One DDA cell as the merge needs it.
struct Cell {
    float pz, py, czz, cyy;
    uint32_t ex, ey;  // column-table entry
    int mip;
    int vx, vz;
    bool loaded;
    int nrec;    // candidate runs recorded by scan_runs; -1: too many, walk the runs
    int guard0;  // guard of the first recorded run (the cell is a no-op once ymin reaches it)
};

// Candidate runs a lane records per cell for the merge (shared memory,
// 3 x float4 per run).  Six: since the scan drops runs whose samples are all
// taken, cells rarely have more candidates, and the 12 KB per block this
// saves over eight go to L1 (the shared-memory carve-out of four blocks per
// SM drops a step), which frames rendered concurrently use: the end-to-end
// loop 5-6% faster, single frames and batches unchanged (4 and 5 slots:
// single frames 5% / 1.2% slower; 7: no L1 gain).
constexpr int kRecs = 6;

// A lane's last coloured sample, stored one pass late: the colour gather
// (a dependent load) then overlaps the following work instead of stalling
// the group at the store.  Every sample is written once, so the order of
// the stores does not matter.
struct Pending {
    uint32_t* at = nullptr;
    uint32_t colour = 0, z = 0;
    __device__ __forceinline__ void flush() {
        if (at) *at = colour + z;
        at = nullptr;
    }
};

// Per-span constants of the perspective-correct fill (:642-700): screen
// position of the span's far end, texture and 1/z gradients along the span.
struct Span {
    float scr_y1r, u1z, u2dz, onez1, onedz2, umax;
    int texture, sg0;
};

__device__ __forceinline__ Span span_setup(float res_y2, const Ray& R, float pz, float py, float sgs, float sgf,
                                           float tex, int texture) {
    Span sp;
    const float pz1r = pz + R.pos3d_z_add * sgs;
    const float py1r = py + R.pos3d_y_add * sgs;
    const float pz2r = pz + R.pos3d_z_add * sgf;
    const float py2r = py + R.pos3d_y_add * sgf;
    const float scr_y2r = res_y2 + py1r / pz1r;
    const float scr_y1r = res_y2 + py2r / pz2r;
    const float u1z = tex / pz2r;
    float u2dz = static_cast<float>(texture) / pz1r - u1z;
    const float onez1 = 1 / pz2r;
    float onedz2 = 1 / pz1r - onez1;
    u2dz /= scr_y2r - scr_y1r;
    onedz2 /= scr_y2r - scr_y1r;
    sp.scr_y1r = scr_y1r;
    sp.u1z = u1z;
    sp.u2dz = u2dz;
    sp.onez1 = onez1;
    sp.onedz2 = onedz2;
    sp.umax = static_cast<float>(static_cast<double>(tex) - 1.0);
    sp.texture = texture;
    sp.sg0 = static_cast<int>(sgs);
    return sp;
}

// Fills samples y .. scr_y2-1 of a span that the occupancy mask leaves open.
template <int G, bool kCount>
__device__ __forceinline__ void draw_span(const Mask& mask, unsigned gmask, int k, uint32_t* row, float* drow,
                                          rle_hit* hrow, const uint16_t* colours, uint64_t colour_room, int S, int y,
                                          int scr_y2, const Span& sp, int mip, int vx, int vz, Pending& pend,
                                          Counts& cnt) {
    const float u2dz = sp.u2dz, onedz2 = sp.onedz2;
    if constexpr (kCount) cnt.spans++;
    const float mult = static_cast<float>(y + 1) - sp.scr_y1r;
    float uz = sp.u1z + u2dz * mult;
    float onez = sp.onez1 + onedz2 * mult;
    const float umin = static_cast<float>(sp.texture);
    const float umax = sp.umax;
    // G pixels per pass: the accumulation runs in lockstep in every lane (it
    // is a chain of IEEE additions, one per sample, masked or not); lane k
    // keeps the values of sample y + k and does its divisions in parallel.
    for (int y0 = y; y0 < scr_y2; y0 += G) {
        const int n = min(G, scr_y2 - y0);
        // lane k needs the accumulators after k more additions
        float my_uz = uz, my_onez = onez;
        for (int j = 0; j < k && j < n; j++) {
            my_uz += u2dz;
            my_onez += onedz2;
        }
        if (n == G) {  // start of the next pass: G additions from this one
            uz = __shfl_sync(gmask, my_uz, (lane_base(gmask)) + G - 1) + u2dz;
            onez = __shfl_sync(gmask, my_onez, (lane_base(gmask)) + G - 1) + onedz2;
        }
        const int yy = y0 + k;
        bool wrote = false;
        if (yy < scr_y2 && !mask.get(yy) && in_bounds(yy < S, kBoundsRay, static_cast<unsigned long long>(yy))) {
            const uint32_t u = static_cast<uint32_t>(fminf(fmaxf(my_uz / my_onez, umin), umax));
            const float depth = 1 / my_onez;
            const uint32_t real_z = static_cast<uint32_t>(static_cast<int>(depth) & 0xfffe);
            pend.flush();
            pend.at = &row[yy];
            pend.colour = in_bounds(u < colour_room, kBoundsColour, u) ? __ldg(&colours[u]) : 0u;
            pend.z = real_z << 16;
            drow[yy] = depth;
            if (hrow) {
                rle_hit h;
                h.x = static_cast<uint16_t>(vx);
                h.z = static_cast<uint16_t>(vz);
                h.y = static_cast<uint16_t>((sp.sg0 >> mip) + static_cast<int>(u - static_cast<uint32_t>(sp.texture)));
                h.mip = static_cast<uint8_t>(mip);
                h.flags = 1;
                hrow[yy] = h;
            }
            atomicOr(&mask.w[yy >> 5], 1u << (yy & 31));
            wrote = true;
        }
        if constexpr (kCount) cnt.pixels += __popc(__ballot_sync(gmask, wrote));
        __syncwarp(gmask);
    }
}

// Exact sequential processing of one cell (the body of the reference's main
// loop after the DDA step).  Uniform across the G lanes of the group.
template <int G, bool kCount>
__device__ __forceinline__ void merge_cell(const RayParams& P, const Ray& R, const Mask& mask, unsigned gmask, int k,
                                           uint32_t* row, float* drow, rle_hit* hrow, Cell c, int& ymin, int& ymax,
                                           Pending& pend, Counts& cnt) {
    const float res_y2 = static_cast<float>(P.S / 2);
    // clip top (:467)
    if (c.pz * res_y2 + c.py <= c.pz * static_cast<float>(ymin)) return;
    if (!c.loaded) {
        const size_t ti = static_cast<size_t>(c.vx) + static_cast<size_t>(c.vz) * (P.gridx0 >> c.mip);
        const uint2 e = in_bounds(ti < P.table_cols[c.mip], kBoundsTable, ti) ? __ldg(&P.table[c.mip][ti])
                                                                               : make_uint2(0u, 0u);
        c.ex = e.x;
        c.ey = e.y;
    }
    if constexpr (kCount) cnt.fetched++;
    const uint16_t* hdr = P.slabs[c.mip] + 2 + c.ex;
    const int nruns = c.ey & 0xffffu;
    const uint16_t* colours = hdr + nruns;
    const float mountain = P.posy;
    uint32_t sti = c.ey >> 16;
    int sg = 0;
    float tex = 0;
    for (int r = 0; r < nruns; r++) {
        if (r > 0) {
            const uint64_t hi = static_cast<uint64_t>(c.ex) + 2u + static_cast<uint64_t>(r);
            sti = in_bounds(hi < P.slab_words[c.mip], kBoundsHeader, hi) ? __ldg(&hdr[r]) : 0u;
            if constexpr (kCount) cnt.headers++;
        }
        int solid = static_cast<int>(sti >> 10);
        sg += static_cast<int>(sti & 1023u) << c.mip;
        if (solid == 0) continue;
        const int texture = static_cast<int>(tex);
        tex += static_cast<float>(solid);
        solid <<= c.mip;
        const float sgs = static_cast<float>(sg);
        sg += solid;
        const float sgf = static_cast<float>(sg);
        if constexpr (kCount) cnt.runs++;
        float czz1 = c.pz, cyy1 = c.py;
        if (mountain + sgs >= 0) { czz1 += c.czz; cyy1 += c.cyy; }
        const float pz1 = czz1 + R.pos3d_z_add * sgs;
        if (pz1 <= 0) continue;
        const float py1 = cyy1 + R.pos3d_y_add * sgs;
        int scr_y2 = static_cast<int>(res_y2 + py1 / pz1);
        if (scr_y2 <= ymin) break;
        float czz2 = c.pz, cyy2 = c.py;
        if (mountain + sgf < 0) { czz2 += c.czz; cyy2 += c.cyy; }
        const float pz2 = czz2 + R.pos3d_z_add * sgf;
        if (pz2 <= 0) continue;
        const float py2 = cyy2 + R.pos3d_y_add * sgf;
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
        const int y = mask.first_clear(scr_y1, scr_y2);
        if (y >= scr_y2) continue;
        const Span sp = span_setup(res_y2, R, c.pz, c.py, sgs, sgf, tex, texture);
        const uint64_t cofs = static_cast<uint64_t>(c.ex) + 2u + static_cast<uint64_t>(nruns);
        const uint64_t room = cofs <= P.slab_words[c.mip] ? P.slab_words[c.mip] - cofs : 0u;
        draw_span<G, kCount>(mask, gmask, k, row, drow, hrow, colours, room, P.S, y, scr_y2, sp, c.mip, c.vx, c.vz,
                             pend, cnt);
    }
}


// Where the DDA of one ray stands between chunks (uniform in its group).
struct Walk {
    Dda d;
    float z, dz, zswitch;
    int mapswitch, mip;
};

// One DDA step (:376-414), written with selects: the chain from one step to
// the next is a compare and a select (the additions for both axes are issued
// beside the compare), shorter than a branch on the compare.
__device__ __forceinline__ void dda_step(Dda& d) {
    const bool c1 = d.dd1 < d.dd0;
    d.dd_now = c1 ? d.dd1 : d.dd0;
    d.index = c1 ? 1 : 0;
    d.pnx = c1 ? d.i1x : d.i0x;
    d.pny = c1 ? d.i1y : d.i0y;
    const float n1 = d.dd1 + d.gd1, n0 = d.dd0 + d.gd0;
    const float a1x = d.i1x + d.g1x, a1y = d.i1y + d.g1y;
    const float a0x = d.i0x + d.g0x, a0y = d.i0y + d.g0y;
    d.dd1 = c1 ? n1 : d.dd1;
    d.i1x = c1 ? a1x : d.i1x;
    d.i1y = c1 ? a1y : d.i1y;
    d.dd0 = c1 ? d.dd0 : n0;
    d.i0x = c1 ? d.i0x : a0x;
    d.i0y = c1 ? d.i0y : a0y;
}

// The update half of dda_step (c1: the step's compare): the state after the
// step.  The step's own values (dd_now, pnx, pny, index) are selects on the
// state before it, which dda_chunk forms only where a lane captures them.
__device__ __forceinline__ void dda_advance(Dda& d, bool c1) {
    const float n1 = d.dd1 + d.gd1, n0 = d.dd0 + d.gd0;
    const float a1x = d.i1x + d.g1x, a1y = d.i1y + d.g1y;
    const float a0x = d.i0x + d.g0x, a0y = d.i0y + d.g0y;
    d.dd1 = c1 ? n1 : d.dd1;
    d.i1x = c1 ? a1x : d.i1x;
    d.i1y = c1 ? a1y : d.i1y;
    d.dd0 = c1 ? d.dd0 : n0;
    d.i0x = c1 ? d.i0x : a0x;
    d.i0y = c1 ? d.i0y : a0y;
}

// Level-of-detail switch at the top of a step (:343-365): past the switch
// distance the ray moves to the next mip level and doubles its step.
__device__ __forceinline__ void lod_switch(Walk& w, int nummaps) {
    while (w.z > w.zswitch) {
        if (w.mip < nummaps - 1) w.mip++;
        w.d.g0x *= 2; w.d.g0y *= 2; w.d.g1x *= 2; w.d.g1y *= 2;
        w.d.gd0 *= 2; w.d.gd1 *= 2;
        w.mapswitch *= 2;
        w.zswitch = static_cast<float>(w.mapswitch);
        w.dz *= 2;
    }
}

// Derives the cell of one DDA step and, unless the horizon known now culls
// it, starts the fetch of its column-table entry (the value is first used by
// scan_runs, one chunk later in the pipeline).
__device__ __forceinline__ void cell_geometry(const RayParams& P, const Ray& R, bool valid, float before, float delta,
                                              float pbx, float pby, int ib, int mip, int ymin, Cell& c) {
    const float res_y2 = static_cast<float>(P.S / 2);
    const float sin_x = P.sin_x, cos_x = P.cos_x;
    const float mountain = P.posy;
    const int fxi = ib ? 0 : static_cast<int>(R.fix_x);
    const int fzi = ib ? static_cast<int>(R.fix_y) : 0;
    const float vs_x = R.ray_x * before;
    const float vs_z = R.ray_z * before;
    const int voxel_x = static_cast<int>(P.posx + pbx) + fxi;
    const int voxel_z = static_cast<int>(P.posz + pby) + fzi;
    c.mip = mip;
    c.vx = (voxel_x >> mip) & ((P.gridx0 >> mip) - 1);
    c.vz = (voxel_z >> mip) & ((P.gridz0 >> mip) - 1);
    const float corr_x = R.ray_x * delta;
    const float corr_z = R.ray_z * delta;
    c.pz = cos_x * vs_z + sin_x * mountain;
    const float py = R.vertical ? cos_x * mountain - sin_x * vs_z : vs_x;
    c.py = py * R.rmul;
    c.czz = cos_x * corr_z;
    const float cyy = R.vertical ? -sin_x * corr_z : corr_x;
    c.cyy = cyy * R.rmul;
    c.ex = 0;
    c.ey = 0;
    c.nrec = 0;
    // clip top at the horizon known now; for pz >= 0 it only gets truer as ymin grows
    const bool culled = c.pz >= 0.0f && c.pz * res_y2 + c.py <= c.pz * static_cast<float>(ymin);
    c.loaded = valid && !culled;
    if (c.loaded) {
        const size_t ti = static_cast<size_t>(c.vx) + static_cast<size_t>(c.vz) * (P.gridx0 >> mip);
        const uint2 e =
            in_bounds(ti < P.table_cols[mip], kBoundsTable, ti) ? __ldg(&P.table[mip][ti]) : make_uint2(0u, 0u);
        c.ex = e.x;
        c.ey = e.y;
    }
}

// Pre-culls a cell against the horizon at the start of its merge and scans
// its runs.  Returns whether the exact walk could draw from it.
//
// The scan also records, in `rec` (this lane's kRecs slots), every run the
// exact walk could still draw, with its projection and span constants, so
// that the sequential merge needs no per-run arithmetic.  A run is recorded
// unless, at the chunk's horizon, the walk would skip it for good (`pz1 <= 0`,
// `pz2 <= 0`, `scr_y1 >= ymax`); the walk's break test (`scr_y2 <= ymin`) of
// the skipped runs before a recorded run is folded into that run's guard (the
// smallest scr_y2 among them and its own), since nothing changes between
// those tests.  The scan ends where the walk would already break at the
// chunk's horizon.  More than kRecs such runs: c.nrec = -1, and the merge
// walks the runs itself.
//
// A run none of whose samples in the open range [ymin, ymax) is still free
// in the occupancy mask is dropped the same way (its scr_y2 folded into the
// next record's guard).  Its turn in the walk could not colour a sample
// either: the mask only gains bits and the range only closes.  Nor can it
// move the horizon in a way that matters: ymin always names a free sample
// (or the range is closed), so a span with no free sample never reaches
// ymin, and the ymax it would set only cuts off samples that are all taken
// -- ymin, the only horizon value the walk's other tests read, evolves the
// same with or without it.
__device__ __forceinline__ bool scan_runs(const RayParams& P, const Ray& R, const Mask& mask, int ymin, int ymax,
                                          Cell& c, float4* rec) {
    const float res_y2 = static_cast<float>(P.S / 2);
    const float mountain = P.posy;
    const int mip = c.mip;
    c.nrec = 0;
    c.guard0 = 0x7fffffff;
    if (!c.loaded) return false;
    // clip top at the current horizon
    if (c.pz >= 0.0f && c.pz * res_y2 + c.py <= c.pz * static_cast<float>(ymin)) return false;
    const uint16_t* hdr = P.slabs[mip] + 2 + c.ex;
    const int nruns = c.ey & 0xffffu;
    const uint32_t colour_ofs = c.ex + 2u + static_cast<uint32_t>(nruns);
    uint32_t sti = c.ey >> 16;
    int sg = 0, texi = 0, n = 0;
    int guard = 0x7fffffff;
    for (int r = 0; r < nruns; r++) {
        if (r > 0) {
            const uint64_t hi = static_cast<uint64_t>(c.ex) + 2u + static_cast<uint64_t>(r);
            sti = in_bounds(hi < P.slab_words[mip], kBoundsHeader, hi) ? __ldg(&hdr[r]) : 0u;
        }
        int solid = static_cast<int>(sti >> 10);
        sg += static_cast<int>(sti & 1023u) << mip;
        if (solid == 0) continue;
        const int texture = texi;
        texi += solid;
        solid <<= mip;
        const float sgs = static_cast<float>(sg);
        sg += solid;
        const float sgf = static_cast<float>(sg);
        float czz1 = c.pz, cyy1 = c.py;
        if (mountain + sgs >= 0) { czz1 += c.czz; cyy1 += c.cyy; }
        const float pz1 = czz1 + R.pos3d_z_add * sgs;
        if (pz1 <= 0) continue;
        const float py1 = cyy1 + R.pos3d_y_add * sgs;
        const int scr_y2 = static_cast<int>(res_y2 + py1 / pz1);
        if (scr_y2 <= ymin) break;  // the walk breaks here or earlier
        guard = min(guard, scr_y2);
        float czz2 = c.pz, cyy2 = c.py;
        if (mountain + sgf < 0) { czz2 += c.czz; cyy2 += c.cyy; }
        const float pz2 = czz2 + R.pos3d_z_add * sgf;
        if (pz2 <= 0) continue;
        const float py2 = cyy2 + R.pos3d_y_add * sgf;
        const int scr_y1 = static_cast<int>(res_y2 + py2 / pz2 - 1);
        if (scr_y1 >= ymax) continue;
        {  // every sample it could colour is taken already
            const int lo = scr_y1 > ymin ? scr_y1 : ymin;
            const int hi = scr_y2 < ymax ? scr_y2 : ymax;
            if (mask.first_clear(lo, hi) >= hi) continue;
        }
        if (n == kRecs) {
            n = -1;
            break;
        }
        // tex counts colours in float in the walk; integers this small are exact
        const Span sp = span_setup(res_y2, R, c.pz, c.py, sgs, sgf, static_cast<float>(texi), texture);
        rec[3 * n + 0] = make_float4(__int_as_float(guard), __int_as_float(scr_y2), __int_as_float(scr_y1),
                                     __uint_as_float(colour_ofs));
        rec[3 * n + 1] = make_float4(sp.scr_y1r, sp.u1z, sp.u2dz, sp.onez1);
        rec[3 * n + 2] = make_float4(sp.onedz2, sp.umax, __int_as_float(sp.texture), __int_as_float(sp.sg0));
        if (n == 0) c.guard0 = guard;
        guard = 0x7fffffff;
        n++;
    }
    c.nrec = n;
    return n != 0;
}

// Short spans are not filled when the merge reaches them: the merge claims
// their samples in the occupancy mask (the samples still free at that
// moment, exactly those the fill would colour) and queues the span; a
// flush then colours the queued samples of up to G spans G at a time, one
// sample per lane.  A span of at most kShortSpan samples lies in two mask
// words, and a sample m places into its span needs m accumulation steps,
// which the lane replays from the span's start.  Longer spans are filled at
// once by draw_span.  Queue entry: 3 x float4 in shared memory,
//   {first free sample | level << 16, claimed bits of the span's two mask
//    words, colour offset of the column},
//   {scr_y1r, u1z, u2dz, onez1},
//   {onedz2, texture | colours of the run << 16, sg0, vx | vz << 16}
// (the sample index is below 2^14, a column holds fewer than 2^16 colours
// and a run at most 63, so the fields fit; the clamp bound umax is the
// float of texture + colours - 1, exactly as the walk computes it).
constexpr int kQueueVecs = 3;
constexpr int kShortSpan = 32;

// The packed fill of short spans pays at up to 2048 samples per ray (1080p
// frames -2%, 480p -5%, batches of up to 1080p -3%); at 4096 it costs more
// than it saves (4K frames +4%, batches of 4K frames +17%).
constexpr int kDeferMaxSamples = 2048;

struct SpanQueue {
    float4* e;  // G entries of this ray
    int n;
};

template <int G>
__device__ __forceinline__ void flush_spans(const RayParams& P, SpanQueue& q, unsigned gmask, int k, uint32_t* row,
                                            float* drow, rle_hit* hrow, Pending& pend) {
    if (q.n == 0) return;
    const int lb = lane_base(gmask);
    // samples per queued span, inclusive prefix over the group's lanes
    int cnt = 0;
    if (k < q.n) {
        const float4 e0 = q.e[kQueueVecs * k];
        cnt = __popc(__float_as_uint(e0.y)) + __popc(__float_as_uint(e0.z));
    }
    int incl = cnt;
#pragma unroll
    for (int o = 1; o < G; o <<= 1) {
        const int v = __shfl_up_sync(gmask, incl, o);
        if (k >= o) incl += v;
    }
    const int total = __shfl_sync(gmask, incl, lb + q.n - 1);
    for (int b = 0; b < total; b += G) {
        const int t = b + k;
        // span of sample t: entries start at strictly increasing sample
        // numbers (every queued span owns at least one sample); those that
        // start at or before b, plus those starting in (b, b + k], count
        // the spans at or before t
        const int start = incl - cnt;
        const bool entry = k < q.n;
        unsigned le = __ballot_sync(gmask, entry && start <= b) >> lb;
        if constexpr (G < 32) le &= (1u << G) - 1u;
        const unsigned marks =
            __reduce_or_sync(gmask, (entry && start > b && start < b + G) ? (1u << (start - b)) : 0u);
        const unsigned upto = k >= 31 ? 0xffffffffu : ((2u << k) - 1u);
        const int lo = __popc(le) - 1 + __popc(marks & upto);
        const int before = __shfl_sync(gmask, start, lb + lo);
        if (t < total) {
            const float4 e0 = q.e[kQueueVecs * lo], e1 = q.e[kQueueVecs * lo + 1], e2 = q.e[kQueueVecs * lo + 2];
            const uint32_t own0 = __float_as_uint(e0.y), own1 = __float_as_uint(e0.z);
            const int r = t - before, c0 = __popc(own0);
            const int bit = r < c0 ? static_cast<int>(__fns(own0, 0, r + 1)) : 32 + static_cast<int>(__fns(own1, 0, r - c0 + 1));
            const int y = static_cast<int>(__float_as_uint(e0.x) & 0xffffu);
            const int mip = static_cast<int>(__float_as_uint(e0.x) >> 16);
            const int p = (y & ~31) + bit;  // the span's first mask word + bit
            const float u2dz = e1.z, onedz2 = e2.x;
            const float mult = static_cast<float>(y + 1) - e1.x;
            float uz = e1.y + u2dz * mult;
            float onez = e1.w + onedz2 * mult;
            for (int j = y; j < p; j++) {
                uz += u2dz;
                onez += onedz2;
            }
            const int texture = static_cast<int>(__float_as_uint(e2.y) & 0xffffu);
            const float umax = static_cast<float>(texture + static_cast<int>(__float_as_uint(e2.y) >> 16) - 1);
            const uint32_t u = static_cast<uint32_t>(fminf(fmaxf(uz / onez, static_cast<float>(texture)), umax));
            const float depth = 1 / onez;
            const uint32_t real_z = static_cast<uint32_t>(static_cast<int>(depth) & 0xfffe);
            const uint64_t ci = static_cast<uint64_t>(__float_as_uint(e0.w)) + u;
            if (in_bounds(p < P.S, kBoundsRay, static_cast<unsigned long long>(p))) {
                pend.flush();
                pend.at = &row[p];
                pend.colour = in_bounds(ci < P.slab_words[mip], kBoundsColour, ci) ? __ldg(&P.slabs[mip][ci]) : 0u;
                pend.z = real_z << 16;
                drow[p] = depth;
            }
            if (hrow && p < P.S) {
                const uint32_t vxz = __float_as_uint(e2.w);
                rle_hit h;
                h.x = static_cast<uint16_t>(vxz & 0xffffu);
                h.z = static_cast<uint16_t>(vxz >> 16);
                h.y = static_cast<uint16_t>((__float_as_int(e2.z) >> mip) + static_cast<int>(u - static_cast<uint32_t>(texture)));
                h.mip = static_cast<uint8_t>(mip);
                h.flags = 1;
                hrow[p] = h;
            }
        }
    }
    __syncwarp(gmask);  // the entries are rewritten by the next spans
    q.n = 0;
}

// The exact walk over the runs scan_runs recorded for one cell (same tests,
// same order, same horizon updates as merge_cell).  a0: the first record when
// the caller loaded it already (G < 32).
template <int G, bool kDefer>
__device__ __forceinline__ void merge_recorded(const RayParams& P, const Mask& mask, unsigned gmask, int k,
                                               uint32_t* row, float* drow, rle_hit* hrow, const float4* rec, float4 a0,
                                               int nrec,
                                               float pz, float py, int mip, int vx, int vz, int& ymin, int& ymax,
                                               Pending& pend, SpanQueue& q, Counts& cnt) {
    const float res_y2 = static_cast<float>(P.S / 2);
    // clip top (:467)
    if (pz * res_y2 + py <= pz * static_cast<float>(ymin)) return;
    for (int r = 0; r < nrec; r++) {
        const float4 a = (G < 32 && r == 0) ? a0 : rec[3 * r];
        if (__float_as_int(a.x) <= ymin) break;
        int scr_y2 = __float_as_int(a.y), scr_y1 = __float_as_int(a.z);
        if (scr_y1 >= ymax) continue;
        // floating horizon (:563-580)
        if (scr_y2 >= ymax) {
            scr_y2 = ymax;
            ymax = scr_y1;
        }
        // the first free sample of the span: a span reaching ymin starts there,
        // since ymin always names a free sample (or the range is closed, and
        // then y >= scr_y2 as in the walk), so only the other spans scan the mask
        int y;
        if (scr_y1 <= ymin) {
            y = ymin;
            ymin = mask.first_clear(scr_y2, ymax > scr_y2 ? ymax : scr_y2);
        } else {
            y = mask.first_clear(scr_y1, scr_y2);
        }
        if (y >= scr_y2) continue;
        const float4 b = rec[3 * r + 1], d = rec[3 * r + 2];
        Span sp;
        sp.scr_y1r = b.x;
        sp.u1z = b.y;
        sp.u2dz = b.z;
        sp.onez1 = b.w;
        sp.onedz2 = d.x;
        sp.umax = d.y;
        sp.texture = __float_as_int(d.z);
        sp.sg0 = __float_as_int(d.w);
        if (kDefer && scr_y2 - y <= kShortSpan) {
            // claim the free samples of [y, scr_y2) now, colour them later
            if (q.n == G) flush_spans<G>(P, q, gmask, k, row, drow, hrow, pend);
            const int base = y & ~31, wi = base >> 5;
            const int hi_bits = scr_y2 - base - 32;  // samples in the second word (<= 31)
            const uint32_t r0 = (hi_bits >= 0 ? 0xffffffffu : ((1u << (scr_y2 - base)) - 1u)) & (0xffffffffu << (y - base));
            const uint32_t r1 = hi_bits > 0 ? ((1u << hi_bits) - 1u) : 0u;
            const uint32_t m0 = mask.w[wi], m1 = r1 ? mask.w[wi + 1] : 0u;
            const uint32_t own0 = r0 & ~m0, own1 = r1 & ~m1;
            __syncwarp(gmask);  // every lane has read m0, m1 before any lane stores
            {
                // Every lane stores the same words (the merge is uniform over the
                // group), so each lane later reads back its own stores: no branch
                // to one lane and no second barrier.
                mask.w[wi] = m0 | r0;
                if (r1) mask.w[wi + 1] = m1 | r1;
                float4* e = q.e + kQueueVecs * q.n;
                const int colours_in_run = static_cast<int>(d.y) + 1 - sp.texture;  // d.y = texture + colours - 1
                e[0] = make_float4(__uint_as_float(static_cast<uint32_t>(y) | (static_cast<uint32_t>(mip) << 16)),
                                   __uint_as_float(own0), __uint_as_float(own1), a.w);
                e[1] = b;
                e[2] = make_float4(d.x, __uint_as_float(static_cast<uint32_t>(sp.texture) |
                                                        (static_cast<uint32_t>(colours_in_run) << 16)),
                                   d.w, __uint_as_float(static_cast<uint32_t>(vx) | (static_cast<uint32_t>(vz) << 16)));
            }
            q.n++;
            continue;
        }
        const uint16_t* colours = P.slabs[mip] + __float_as_uint(a.w);
        const uint64_t cofs = __float_as_uint(a.w);
        const uint64_t room = cofs <= P.slab_words[mip] ? P.slab_words[mip] - cofs : 0u;
        draw_span<G, false>(mask, gmask, k, row, drow, hrow, colours, room, P.S, y, scr_y2, sp, mip, vx, vz, pend,
                            cnt);
    }
}

// One chunk of the DDA: G steps in lockstep, lane k keeping the state after
// step k; the state before step k is the state after step k-1 (a shuffle
// from lane k-1; lane 0 takes the chunk start).  Advances W past the chunk
// and returns how many of its steps are valid (fewer than G: the ray ends).
struct ChunkStep {
    float before, delta, pbx, pby;
    int ib, mip;
};

template <int G>
__device__ __forceinline__ int dda_chunk(const RayParams& P, Walk& W, int k, unsigned gmask, ChunkStep& st) {
    const float zfar = static_cast<float>(P.z_far);
    // ---- 1. G DDA steps in lockstep; lane k keeps the state after step k ----
    // the state before step k is the state after step k-1 (a shuffle
    // from lane k-1; lane 0 takes the chunk start)
    const float start_dd = W.d.dd_now, start_px = W.d.pnx, start_py = W.d.pny;
    const int start_ix = W.d.index;
    float c_dd = 0, c_px = 0, c_py = 0;
    int c_ix = 0, smip = W.mip;
    int nvalid = G;
    // z, dz and the switch distances are integers held exactly in
    // floats: when neither a LOD switch nor the end of the ray can
    // fall inside the chunk, the steps need no checks
    const int zi = static_cast<int>(W.z), dzi = static_cast<int>(W.dz);
    // every step's z stays at or below the switch distance and the chunk's
    // last z at or below z_far (dz > 0; the products stay far below 2^31)
    const bool plain = W.mapswitch - zi >= (G - 1) * dzi && P.z_far - zi >= G * dzi;
    if (plain) {
#pragma unroll
        for (int s = 0; s < G; s++) {
            if (s == G - 1) {
                dda_step(W.d);
                if (s == k) {
                    c_dd = W.d.dd_now;
                    c_px = W.d.pnx;
                    c_py = W.d.pny;
                    c_ix = W.d.index;
                }
            } else {
                const bool c1 = W.d.dd1 < W.d.dd0;
                if (s == k) {
                    c_dd = c1 ? W.d.dd1 : W.d.dd0;
                    c_px = c1 ? W.d.i1x : W.d.i0x;
                    c_py = c1 ? W.d.i1y : W.d.i0y;
                    c_ix = c1 ? 1 : 0;
                }
                dda_advance(W.d, c1);
            }
        }
        W.z += W.dz * static_cast<float>(G);
    } else {
        bool ended_here = false;
#pragma unroll 1
        for (int s = 0; s < G; s++) {
            if (W.z > W.zswitch) {
                lod_switch(W, P.nummaps);
                if (k >= s) smip = W.mip;  // cells from step s on use the new level
            }
            W.z += W.dz;
            if (W.z > zfar) {
                nvalid = s;
                ended_here = true;
                break;
            }
            dda_step(W.d);
            if (s == k) {
                c_dd = W.d.dd_now;
                c_px = W.d.pnx;
                c_py = W.d.pny;
                c_ix = W.d.index;
            }
        }
        (void)ended_here;
    }
    float before = __shfl_up_sync(gmask, c_dd, 1);
    float pbx = __shfl_up_sync(gmask, c_px, 1);
    float pby = __shfl_up_sync(gmask, c_py, 1);
    int ib = __shfl_up_sync(gmask, c_ix, 1);
    if (k == 0) {
        before = start_dd;
        pbx = start_px;
        pby = start_py;
        ib = start_ix;
    }
    const float delta = c_dd - before;
    st.before = before;
    st.delta = delta;
    st.pbx = pbx;
    st.pby = pby;
    st.ib = ib;
    st.mip = smip;
    return nvalid;
}

// Whether no cell at or beyond DDA distance t0 can draw a span.
//
// A run whose top lies h below the eye (h = position.y + its column index,
// level-0 units, h grows downwards) seen at distance t projects with
// pz1 = c*t + d*h and py1 = py_t*t + py_h*h (c = cos_x*ray_z, d = sin_x;
// py_t = -rmul*sin_x*ray_z, py_h = rmul*cos_x for rays of the up/down fans,
// py_t = rmul*ray_x, py_h = 0 for the left/right fans; :483-559).  The run is
// dropped at its turn (`scr_y2 <= ymin`, or `pz1 <= 0`) whenever
// f = K*pz1 + py1 < 0 with K = res_y2 - ymin - 1.  f is linear in (t, h), so
// it stays negative for every t >= t0 and every h >= h0 (h0: the scene's
// topmost voxel) if its slopes in t and h are not positive and f(t0, h0) < 0.
// A margin of 1e-4 of the magnitudes of the terms covers the float rounding
// of the kernel's evaluation (about 1e-6 relative); ymin only grows later,
// which only lowers f where pz1 > 0.
__device__ __forceinline__ bool ray_is_done(const RayParams& P, const Ray& R, float t0, int ymin) {
    const float eps = 1e-4f;
    const float res_y2 = static_cast<float>(P.S / 2);
    const float K = res_y2 - static_cast<float>(ymin) - 1.0f;
    const float c = P.cos_x * R.ray_z, d = P.sin_x;
    const float py_t = R.vertical ? -R.rmul * P.sin_x * R.ray_z : R.rmul * R.ray_x;
    const float py_h = R.vertical ? R.rmul * P.cos_x : 0.0f;
    const float a = K * c + py_t, b = K * d + py_h;
    const float scale = res_y2 + fabsf(K) + 1.0f;
    const float ma = fabsf(c) * scale + fabsf(py_t), mb = fabsf(d) * scale + fabsf(py_h);
    const float h0 = P.posy + static_cast<float>(P.top_index);
    return a + eps * ma <= 0.0f && b + eps * mb <= 0.0f &&
           a * t0 + b * h0 + eps * (ma * t0 + mb * fabsf(h0)) < 0.0f;
}

// Casts ray x of frame P with the G lanes of one group (lane k, lane mask
// gmask), using mask_words (S/32 words of shared memory) as its bitmask.
// active = false: the lanes only take part in the group's collectives.
// chunks of G DDA steps, lane k taking step k of each.
template <int G, bool kCount, bool kHits, bool kDefer, bool kStage>
__device__ __forceinline__ void cast_ray(const RayParams& P, int x, bool active, uint32_t* mask_words, float4* recs,
                                         float4* spans, int k, unsigned gmask, int staging, Counts& cnt) {
    const int S = P.S;
    const int words = (S + 31) >> 5;
    Mask mask{mask_words};

    float4* my_recs = recs + static_cast<size_t>(threadIdx.x) * (3 * kRecs);
    Pending pend;
    SpanQueue q{spans, 0};
    Ray R;
    Walk W;
    bool live = false;
    if (active) {
        for (int w = k; w < words; w += G) mask.w[w] = 0;
        live = setup_ray(P, x, R, W.d);
    } else {
        R.ymin = 0;
        R.ymax = -1;
    }
    // A whole-warp barrier, also with several rays per warp: every lane that
    // has not exited passes one at the start and one at the end of each ray
    // (a group with no ray left exits, and exited lanes do not count), so it
    // always completes -- and it brings a warp's groups back into step at
    // their ray boundaries, where they then issue together (a barrier over
    // the group alone measured 6% slower for 4K batches at 16 lanes).
    __syncwarp();
    uint32_t* row = active ? P.raybuf + static_cast<size_t>(x) * S : nullptr;
    float* drow = active ? P.raydepth + static_cast<size_t>(x) * S : nullptr;
    rle_hit* hrow = nullptr;
    if constexpr (kHits) hrow = (active && P.rayhit) ? P.rayhit + static_cast<size_t>(x) * S : nullptr;
    const int ymin0 = R.ymin, ymax0 = R.ymax;

    if (live) {
        int ymin = R.ymin, ymax = R.ymax;
        W.mip = 0;
        W.z = 0;
        W.dz = 1;
        W.mapswitch = P.mapswitch0;
        W.zswitch = static_cast<float>(W.mapswitch);
        {
            // first step's switch test, the only one the camera height can
            // trigger: y_map_switch starts at position.y and only halves
            float y_map_switch = P.posy;
            while (W.z > W.zswitch || y_map_switch > 512.0f) {
                y_map_switch = y_map_switch * 0.5f;
                if (W.mip < P.nummaps - 1) W.mip++;
                W.d.g0x *= 2; W.d.g0y *= 2; W.d.g1x *= 2; W.d.g1y *= 2;
                W.d.gd0 *= 2; W.d.gd1 *= 2;
                W.mapswitch *= 2;
                W.zswitch = static_cast<float>(W.mapswitch);
                W.dz *= 2;
            }
        }
        ChunkStep st;
        int nvalid = dda_chunk<G>(P, W, k, gmask, st);
        Cell c;
        cell_geometry(P, R, k < nvalid, st.before, st.delta, st.pbx, st.pby, st.ib, st.mip, ymin, c);
        for (;;) {
            if (nvalid == 0) break;
            const bool ended = nvalid < G;
            const bool valid = k < nvalid;
            const float t_end = W.d.dd_now;  // DDA distance at the end of this chunk
            // whether the ray can end after this chunk, tested at the horizon
            // before the merge: ymin only grows, so a test that passes now
            // passes after the merge too, and its latency hides under the DDA
            const bool done_next = !kCount && ray_is_done(P, R, t_end, ymin);
            // ---- 1. the next chunk's DDA steps and column-table fetches are
            // issued now; their loads complete while this chunk is merged ----
            int nvalid_next = 0;
            Cell c_next;
            if (!ended) {
                ChunkStep st_next;
                nvalid_next = dda_chunk<G>(P, W, k, gmask, st_next);
                cell_geometry(P, R, k < nvalid_next, st_next.before, st_next.delta, st_next.pbx, st_next.pby,
                              st_next.ib, st_next.mip, ymin, c_next);
            }

            // ---- 2. each lane: its cell -- pre-cull at the current horizon, run scan ----
            const bool drawable = scan_runs(P, R, mask, ymin, ymax, c, my_recs);
            // with counters every valid cell goes through the exact walk
            unsigned todo = __ballot_sync(gmask, kCount ? valid : drawable) >> lane_base(gmask);
            if constexpr (G < 32) todo &= (1u << G) - 1u;
            __syncwarp(gmask);  // the records are read by the whole group

            // ---- 3. exact sequential merge of the cells that may draw ----
            bool stop = false;
            while (todo) {
                const int s = __ffs(todo) - 1;
                todo &= todo - 1;
                const int src = lane_base(gmask) + s;
                const float4* rec = recs + static_cast<size_t>((threadIdx.x & ~31u) + src) * (3 * kRecs);
                // with several rays per warp, the cell's first record is loaded
                // beside the shuffles that fetch its values (measured: batches
                // -4%; single frames at 32 lanes +1.6%, so not there)
                float4 a0 = make_float4(0.f, 0.f, 0.f, 0.f);
                if constexpr (G < 32) a0 = rec[0];
                const float pz = __shfl_sync(gmask, c.pz, src);
                const float py = __shfl_sync(gmask, c.py, src);
                const int packed = __shfl_sync(gmask, (c.nrec + 1) | (c.mip << 8), src);
                const int nrec = (packed & 0xff) - 1, mip = packed >> 8;
                int vx = 0, vz = 0;
                if (kHits && hrow) {
                    vx = __shfl_sync(gmask, c.vx, src);
                    vz = __shfl_sync(gmask, c.vz, src);
                }
                // the reference ends the ray when its horizon closes, checked
                // at every step before the cell (:370)
                if (ymin >= ymax) {
                    stop = true;
                    break;
                }
                if constexpr (kCount) cnt.cells++;  // with counters every valid step is visited
                if (kCount || nrec < 0) {
                    Cell cs;
                    cs.pz = pz;
                    cs.py = py;
                    cs.czz = __shfl_sync(gmask, c.czz, src);
                    cs.cyy = __shfl_sync(gmask, c.cyy, src);
                    cs.ex = __shfl_sync(gmask, c.ex, src);
                    cs.ey = __shfl_sync(gmask, c.ey, src);
                    cs.mip = mip;
                    cs.vx = __shfl_sync(gmask, c.vx, src);
                    cs.vz = __shfl_sync(gmask, c.vz, src);
                    cs.loaded = __shfl_sync(gmask, static_cast<int>(c.loaded), src) != 0;
                    merge_cell<G, kCount>(P, R, mask, gmask, k, row, drow, hrow, cs, ymin, ymax, pend, cnt);
                } else {
                    const int ymin_before = ymin;
                    merge_recorded<G, kDefer>(P, mask, gmask, k, row, drow, hrow, rec, a0, nrec, pz, py, mip, vx, vz,
                                              ymin, ymax, pend, q, cnt);
                    if (ymin != ymin_before) {
                        // cells whose first recorded run now breaks the walk
                        // at once are no-ops: drop them all in one vote
                        unsigned keep = __ballot_sync(gmask, c.nrec < 0 || c.guard0 > ymin) >> lane_base(gmask);
                        if constexpr (G < 32) keep &= (1u << G) - 1u;
                        todo &= keep;
                    }
                }
            }
            __syncwarp(gmask);  // records are rewritten by the next chunk
            if (stop || ymin >= ymax || ended) break;
            // Nothing further along this ray can be drawn once every run of
            // every later cell projects below the floating horizon (the
            // reference walks on to z_far without drawing).  Exact counters
            // need the full walk, so they keep it.
            if (done_next) break;
            // staging depth >= 2: the next chunk's table entries have arrived
            // under the merge; stage each cell's header line (second header
            // on; the first travels in the table entry) for its scan, which
            // follows the next DDA chunk
            if (kStage && c_next.loaded && (c_next.ey & 0xffffu) > 1u)
                stage_headers(P.slabs[c_next.mip] + 3 + c_next.ex, staging);
            c = c_next;
            nvalid = nvalid_next;
        }
    }
    flush_spans<G>(P, q, gmask, k, row, drow, hrow, pend);
    pend.flush();
    __syncwarp();  // whole warp, as at the start of the ray

    // ---- coalesced fill of the samples no span coloured ----
    if (active) {
        for (int y = k; y < S; y += G) {
            if (mask.get(y)) continue;
            const bool in = y >= ymin0 && y <= ymax0;
            row[y] = in ? kSky : 0u;
            drow[y] = in ? INFINITY : 0.0f;
            if (hrow) {
                rle_hit h = {0, 0, 0, 0, static_cast<uint8_t>(in ? 2 : 0)};
                hrow[y] = h;
            }
        }
    }
    if (kCount && active && k == 0) {
        // the lanes of a group hold the same counts; lane 0 adds the ray's
        unsigned long long* c = reinterpret_cast<unsigned long long*>(P.counters);
        const unsigned long long v[6] = {cnt.cells, cnt.fetched, cnt.headers, cnt.runs, cnt.spans, cnt.pixels};
        for (int i = 0; i < 6; i++)
            if (v[i]) atomicAdd(&c[i], v[i]);
    }
    cnt = Counts();
}

// Shared memory of a raycast block: the rays' occupancy masks (`words` per
// ray slot), then, 16-byte aligned, kRecs run records per thread.
__host__ __device__ __forceinline__ int mask_region_words(int slots, int words) {
    return (slots * words + 3) & ~3;
}
__host__ __device__ __forceinline__ size_t raycast_smem_bytes(int threads, int slots, int words, bool queues) {
    // masks | run records (kRecs per thread) | span queues, in the variants that
    // defer short spans (32 / slots-per-warp entries per ray, i.e. one per
    // lane of the group: as many entries per block as threads)
    return static_cast<size_t>(mask_region_words(slots, words)) * 4 +
           static_cast<size_t>(threads) * kRecs * 3 * sizeof(float4) +
           (queues ? static_cast<size_t>(threads) * kQueueVecs * sizeof(float4) : 0u);
}

// Lane layout of a group of G lanes within a block.
template <int G>
struct Lanes {
    int lane, g, k, slot;
    unsigned gmask;
    __device__ __forceinline__ Lanes() {
        constexpr int kGroups = 32 / G;
        lane = threadIdx.x & 31;
        g = lane / G;  // ray group within the warp
        k = lane % G;  // lane within the group
        gmask = (G == 32) ? 0xffffffffu : (((1u << G) - 1u) << (g * G));
        slot = (threadIdx.x >> 5) * kGroups + g;  // ray slot within the block
    }
};

// One frame: ray slot s of block b casts ray b * slots + s.  kCount: the
// DETAIL_BENCH counters (exact walk of every cell); kHits: hit records;
// kDefer: packed fill of short spans; kStage: run-header staging (depth 2/3).
template <int G, bool kCount, bool kHits, bool kDefer, bool kStage>
__global__ void __launch_bounds__(128) raycast_kernel(const __grid_constant__ RayParams P) {
    extern __shared__ uint32_t smem[];
    const Lanes<G> L;
    const int rays_per_block = (blockDim.x >> 5) * (32 / G);
    const int x = blockIdx.x * rays_per_block + L.slot;
    const int words = (P.S + 31) >> 5;
    float4* recs = reinterpret_cast<float4*>(smem + mask_region_words(rays_per_block, words));
    float4* spans =
        kDefer ? recs + static_cast<size_t>(blockDim.x) * (3 * kRecs) + static_cast<size_t>(L.slot) * (kQueueVecs * G)
               : nullptr;
    Counts cnt;
    // per-ray timing (rle_render_rays_timed): the first lane of the group
    // stamps the ray's start and end; nothing else changes
    if (P.ray_time && L.k == 0 && x < P.rays) {
        rle_ray_time* t = P.ray_time + x;
        t->start_ns = global_ns();
        t->start_clock = static_cast<uint64_t>(clock64());
    }
    cast_ray<G, kCount, kHits, kDefer, kStage>(P, x, x < P.rays, smem + L.slot * words, recs, spans, L.k, L.gmask,
                                               P.staging, cnt);
    if (P.ray_time && L.k == 0 && x < P.rays) {
        rle_ray_time* t = P.ray_time + x;
        t->end_clock = static_cast<uint64_t>(clock64());
        t->end_ns = global_ns();
        t->sm = sm_id();
        t->reserved = 0;
    }
}

// Many frames in one persistent launch.  The rays of all frames form one
// index space (ray_start[f] = first global ray of frame f); each group takes
// `tile` consecutive rays at a time from a global counter until none are
// left, so long and short rays of every frame balance across the GPU.
template <int G, bool kHits, bool kDefer, bool kStage>
__global__ void __launch_bounds__(128) raycast_batch_kernel(BatchHeader* hdr, const int* __restrict__ ray_start,
                                                            const RayParams* __restrict__ frames, int tile,
                                                            int staging, int max_words) {
    extern __shared__ uint32_t smem[];
    const Lanes<G> L;
    const int nframes = hdr->nframes;
    const int total = ray_start[nframes];
    uint32_t* mask_words = smem + L.slot * max_words;
    float4* recs = reinterpret_cast<float4*>(
        smem + mask_region_words((static_cast<int>(blockDim.x) >> 5) * (32 / G), max_words));
    float4* spans =
        kDefer ? recs + static_cast<size_t>(blockDim.x) * (3 * kRecs) + static_cast<size_t>(L.slot) * (kQueueVecs * G)
               : nullptr;
    Counts cnt;
    int f = 0;  // frame of the current ray (rays are taken in increasing order)
    // Guided self-scheduling: a group claims up to `tile` adjacent rays, but
    // never more than half its fair share of what is left, so the last rays
    // go out one at a time and no group is left with a long private tail.
    const int grab = tile;
    const int groups = static_cast<int>(gridDim.x) * (static_cast<int>(blockDim.x) / G);
    for (;;) {
        unsigned int t0 = 0, n = 1;
        if (L.k == 0) {
            const int seen = static_cast<int>(*reinterpret_cast<volatile unsigned int*>(&hdr->next_ray));
            n = static_cast<unsigned int>(max(1, min(grab, (total - seen) / (2 * groups))));
            t0 = atomicAdd(&hdr->next_ray, n);
        }
        t0 = __shfl_sync(L.gmask, t0, lane_base(L.gmask));
        n = __shfl_sync(L.gmask, n, lane_base(L.gmask));
        if (static_cast<int>(t0) >= total) break;
        const int t1 = min(static_cast<int>(t0) + static_cast<int>(n), total);
        for (int r = static_cast<int>(t0); r < t1; r++) {
            if (r < ray_start[f] || r >= ray_start[f + 1]) {
                int lo = 0, hi = nframes - 1;  // last frame with ray_start <= r
                while (lo < hi) {
                    const int mid = (lo + hi + 1) >> 1;
                    if (ray_start[mid] <= r) lo = mid;
                    else hi = mid - 1;
                }
                f = lo;
            }
            cast_ray<G, false, kHits, kDefer, kStage>(frames[f], r - ray_start[f], true, mask_words, recs, spans, L.k,
                                                     L.gmask, staging, cnt);
        }
    }
}

template <int G, bool kCount, bool kHits, bool kDefer, bool kStage>
rle_status launch_variant(const RayParams& p, int threads, cudaStream_t stream) {
    const int words = (p.S + 31) >> 5;
    const int rays_per_block = threads / 32 * (32 / G);
    const size_t smem = raycast_smem_bytes(threads, rays_per_block, words, kDefer);
    if (smem > 227 * 1024) {
        set_error("rle_render_rays: %d samples per ray exceed shared memory at this launch shape", p.S);
        return RLE_ERR_CAPACITY;
    }
    cudaError_t e = cudaFuncSetAttribute(raycast_kernel<G, kCount, kHits, kDefer, kStage>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
    if (e != cudaSuccess) {
        set_error("cudaFuncSetAttribute: %s", cudaGetErrorString(e));
        return RLE_ERR_CUDA;
    }
    const int blocks = (p.rays + rays_per_block - 1) / rays_per_block;
    raycast_kernel<G, kCount, kHits, kDefer, kStage><<<blocks, threads, smem, stream>>>(p);
    e = cudaGetLastError();
    if (e != cudaSuccess) {
        set_error("raycast launch: %s", cudaGetErrorString(e));
        return RLE_ERR_CUDA;
    }
    return RLE_OK;
}

template <int G, bool kStage>
rle_status launch_output(const RayParams& p, int threads, cudaStream_t stream) {
    if (p.S <= kDeferMaxSamples) {
        return p.rayhit ? launch_variant<G, false, true, true, kStage>(p, threads, stream)
                        : launch_variant<G, false, false, true, kStage>(p, threads, stream);
    }
    return p.rayhit ? launch_variant<G, false, true, false, kStage>(p, threads, stream)
                    : launch_variant<G, false, false, false, kStage>(p, threads, stream);
}

template <int G>
rle_status launch_shape(const RayParams& p, int threads, cudaStream_t stream) {
    if (p.counters) {  // the counts do not depend on the staging depth
        return p.rayhit ? launch_variant<G, true, true, false, false>(p, threads, stream)
                        : launch_variant<G, true, false, false, false>(p, threads, stream);
    }
    return p.staging >= 2 ? launch_output<G, true>(p, threads, stream) : launch_output<G, false>(p, threads, stream);
}

template <int G, bool kDefer>
size_t batch_smem(int threads, int max_samples) {
    return raycast_smem_bytes(threads, threads / 32 * (32 / G), (max_samples + 31) >> 5, kDefer);
}

template <int G, bool kHits, bool kDefer, bool kStage>
rle_status batch_blocks(int threads, int max_samples, int* blocks) {
    const size_t smem = batch_smem<G, kDefer>(threads, max_samples);
    if (smem > 227 * 1024) {
        set_error("batch: %d samples per ray exceed shared memory at this launch shape", max_samples);
        return RLE_ERR_CAPACITY;
    }
    cudaError_t e = cudaFuncSetAttribute(raycast_batch_kernel<G, kHits, kDefer, kStage>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
    int dev = 0, sms = 0, per_sm = 0;
    if (e == cudaSuccess) e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e == cudaSuccess)
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, raycast_batch_kernel<G, kHits, kDefer, kStage>,
                                                          threads, smem);
    if (e != cudaSuccess) {
        set_error("batch launch set-up: %s", cudaGetErrorString(e));
        return RLE_ERR_CUDA;
    }
    *blocks = sms * (per_sm > 0 ? per_sm : 1);
    return RLE_OK;
}

template <int G, bool kHits, bool kDefer, bool kStage>
rle_status batch_launch(const BatchRaycast& b, cudaStream_t stream) {
    const size_t smem = batch_smem<G, kDefer>(b.threads, b.max_samples);
    int blocks = b.blocks;
    if (blocks <= 0) {
        const rle_status st = batch_blocks<G, kHits, kDefer, kStage>(b.threads, b.max_samples, &blocks);
        if (st != RLE_OK) return st;
    }
    raycast_batch_kernel<G, kHits, kDefer, kStage><<<blocks, b.threads, smem, stream>>>(
        b.header, b.ray_start, b.frames, b.tile, b.staging, (b.max_samples + 31) >> 5);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        set_error("batch raycast launch: %s", cudaGetErrorString(e));
        return RLE_ERR_CUDA;
    }
    return RLE_OK;
}

template <int G, bool kDefer>
rle_status batch_blocks_for(int threads, int max_samples, bool hits, bool stage, int* blocks) {
    if (stage)
        return hits ? batch_blocks<G, true, kDefer, true>(threads, max_samples, blocks)
                    : batch_blocks<G, false, kDefer, true>(threads, max_samples, blocks);
    return hits ? batch_blocks<G, true, kDefer, false>(threads, max_samples, blocks)
                : batch_blocks<G, false, kDefer, false>(threads, max_samples, blocks);
}

template <int G, bool kDefer>
rle_status batch_launch_for(const BatchRaycast& b, cudaStream_t s) {
    if (b.staging >= 2)
        return b.hits ? batch_launch<G, true, kDefer, true>(b, s) : batch_launch<G, false, kDefer, true>(b, s);
    return b.hits ? batch_launch<G, true, kDefer, false>(b, s) : batch_launch<G, false, kDefer, false>(b, s);
}

}  // namespace

rle_status batch_grid_blocks(int lanes, int threads, int max_samples, bool hits, int staging, int* blocks) {
    const bool defer = max_samples <= kDeferMaxSamples;
    const bool stage = staging >= 2;
    switch (lanes) {
        case 8: return defer ? batch_blocks_for<8, true>(threads, max_samples, hits, stage, blocks)
                             : batch_blocks_for<8, false>(threads, max_samples, hits, stage, blocks);
        case 16: return defer ? batch_blocks_for<16, true>(threads, max_samples, hits, stage, blocks)
                              : batch_blocks_for<16, false>(threads, max_samples, hits, stage, blocks);
        case 32: return defer ? batch_blocks_for<32, true>(threads, max_samples, hits, stage, blocks)
                              : batch_blocks_for<32, false>(threads, max_samples, hits, stage, blocks);
        default:
            set_error("batch: lanes per ray must be 8, 16 or 32");
            return RLE_ERR_INVALID_ARG;
    }
}

rle_status launch_raycast_batch(const BatchRaycast& b, void* stream) {
    if (b.threads % 32 != 0 || b.threads <= 0 || b.threads > 128 || b.tile < 1 || b.staging < 1 || b.staging > 3) {
        set_error("batch: threads per block a multiple of 32 up to 128, tile >= 1, staging 1..3");
        return RLE_ERR_INVALID_ARG;
    }
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const bool defer = b.max_samples <= kDeferMaxSamples;
    switch (b.lanes) {
        case 8: return defer ? batch_launch_for<8, true>(b, s) : batch_launch_for<8, false>(b, s);
        case 16: return defer ? batch_launch_for<16, true>(b, s) : batch_launch_for<16, false>(b, s);
        case 32: return defer ? batch_launch_for<32, true>(b, s) : batch_launch_for<32, false>(b, s);
        default:
            set_error("batch: lanes per ray must be 8, 16 or 32");
            return RLE_ERR_INVALID_ARG;
    }
}

bool bounds_render(unsigned* out4, bool clear) {
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

rle_status launch_raycast(const RayParams& p, void* stream) {
    if (p.rays <= 0) return RLE_OK;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const int lanes = p.lanes_per_ray > 0 ? p.lanes_per_ray : 32;
    const int threads = p.threads_per_block > 0 ? p.threads_per_block : 128;
    if (threads % 32 != 0 || threads > 128) {
        set_error("raycast: threads per block must be a multiple of 32, at most 128");
        return RLE_ERR_INVALID_ARG;
    }
    if (p.staging < 0 || p.staging > 3) {
        set_error("raycast: staging depth 1..3 (0 = default)");
        return RLE_ERR_INVALID_ARG;
    }
    switch (lanes) {
        case 8: return launch_shape<8>(p, threads, s);
        case 16: return launch_shape<16>(p, threads, s);
        case 32: return launch_shape<32>(p, threads, s);
        default:
            set_error("raycast: lanes per ray must be 8, 16 or 32");
            return RLE_ERR_INVALID_ARG;
    }
}

}  // namespace rle
