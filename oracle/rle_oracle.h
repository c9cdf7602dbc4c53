/* CPU oracle for the RLE column raycaster (test infrastructure only).
 *
 * A plain-C restatement of the reference's algorithm for the render path:
 *   - RLE4 encoder, mip builder and column-table loader (src/Rle4.cpp, src/tree.h)
 *   - per-camera ray map (src/RayMap.h:98-402)
 *   - per-column-ray raycast (src/Cuda_Render.h:96-737)
 *   - ray buffer -> screen resolve (bin/shader/colorize_buddha_soft.frag:12-80)
 * Only the test suite, the smoke check and the CPU-baseline leg of the
 * benchmark may load this library; the renderer never does.
 *
 * Parity is pinned against the reference's own sources compiled for the host
 * (oracle/ref, producing oracle/_ref/libref.so) and against the golden
 * fixtures under tests/golden that library generated.  The resolve is pinned
 * only against this restatement: the GLSL cannot run without a graphics stack.
 */
#ifndef RLE_ORACLE_H
#define RLE_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct { float x, y, z; } orc_v3;

/* Field-for-field the per-frame part of RayMap_GPU (src/RayMap.h:16-54),
 * plus the render parameters that src/core.h fixes at compile time. */
typedef struct orc_raymap {
    orc_v3 vanishing_point_2d;
    int map_line_count;
    orc_v3 rotation;
    orc_v3 position;
    float border, clip_min, clip_max;
    int maxres;
    int res[4];
    orc_v3 p4;
    orc_v3 p_2d[8];
    orc_v3 p_no[8];
    float to3d[4][4];
    float p_ofs_min[4], p_ofs_max[4];
    /* render parameters (src/core.h:3-10 as runtime values) */
    int samples;       /* RENDER_SIZE: samples per column ray (res_x = res_y) */
    int mip_distance;  /* MIP_DISTANCE */
    int z_far;         /* RAYS_DISTANCE */
    float fov_scale;   /* tan(fov/2); 1 reproduces the fixed +-1 frustum */
} orc_raymap;

typedef struct orc_mip {
    int sx, sy, sz;
    const uint32_t* table;  /* uint2 {slab_ofs, count | first_header << 16} */
    const uint16_t* slabs;
    long long slabs_words;
} orc_mip;

/* Per-ray counters with the meaning of DETAIL_BENCH (src/Cuda_Render.h:14-22). */
typedef struct orc_counters {
    long long cells;      /* DDA cells stepped */
    long long fetched;    /* column-table entries read (8 B each) */
    long long headers;    /* run headers read from the slab array (2 B each) */
    long long runs;       /* solid runs examined */
    long long spans;      /* spans that reached the pixel loop */
    long long pixels;     /* ray-buffer samples written with a colour (2 B colour read each) */
} orc_counters;

/* Hit record of one ray-buffer sample: the voxel that coloured it. */
typedef struct orc_hit {
    uint16_t x, z, y;  /* cell and height at level `mip` */
    uint8_t mip;
    uint8_t flags;     /* 1 = hit, 2 = sky, 0 = no data */
} orc_hit;

/* ---- scene format ------------------------------------------------------ */

/* RLE4::compress (src/Rle4.cpp:52-198) on a bit volume (bit i&7 of byte
 * (i + j*sx + k*sx*sy) >> 3).  colours: optional u16 per voxel, same index
 * without the >>3; NULL selects the reference's normal-derived colour word.
 * Writes the per-column start offsets (sx*sz) and returns the slab words in
 * *slabs (malloc'd) and their count in *nwords. */
int orc_encode_mip(const uint8_t* bits, const uint16_t* colours, int sx, int sy, int sz,
                   int mip, uint32_t* column_start, uint16_t** slabs, long long* nwords);

/* Tree::get_mipmap (src/tree.h:23-85): a voxel of the half-size volume is
 * solid when at least 3 of its 8 children are. */
int orc_mipmap(const uint8_t* bits, int sx, int sy, int sz, uint8_t* out);

/* RLE4::load's column walk (src/Rle4.cpp:285-314): slab words -> uint2
 * table of 2*sx*sz words.  Returns 0, or -1 if the walk leaves the array. */
int orc_build_table(const uint16_t* slabs, long long nwords, int sx, int sz, uint32_t* table);

/* ---- ray map ------------------------------------------------------------ */

/* RayMap::get_ray_map (src/RayMap.h:98-402) with set_border(border) and
 * RAYS_CASTED_RES = 4*maxres.  fov_scale scales the frustum corners
 * (src/RayMap.h:107-114); 1 is the reference frustum. */
void orc_raymap_build(orc_raymap* rm, float px, float py, float pz, float rx, float ry, float rz,
                      float border, int maxres, float fov_scale, int samples, int mip_distance,
                      int z_far);

/* ---- raycast ------------------------------------------------------------ */

/* Render::render_line (src/Cuda_Render.h:96-737) for rays [0, nrays).
 * out: nrays*samples packed words (colour16 | depth16 << 16); every word is
 * written: 0 outside the ray's clip range, 0x00ff8844 for sky.
 * depth (optional): float 1/onez of each written sample, +inf for sky, 0 else.
 * hits (optional), counters (optional, per ray). nthreads <= 0: OpenMP default. */
int orc_render_rays(const orc_raymap* rm, const orc_mip* mips, int nummaps, int nrays,
                    uint32_t* out, float* depth, orc_hit* hits, orc_counters* counters,
                    int nthreads);

/* ---- resolve ------------------------------------------------------------ */

/* colorize_buddha_soft.frag:12-80 texcoord maths with a nearest fetch
 * (GL_NEAREST + GL_CLAMP_TO_EDGE, src/GL_Main.cpp:152-157) from a ray buffer
 * of `rows` rows.  Output row 0 is the top of the screen.
 * raydepth is required: a sample whose depth is 0 was outside its ray's clip
 * range (no data); byte 2 == 0xff marks sky, as the shader's c.z == 1.0 test.
 * colour: RGBA8 from RGB565 for hits, 0xFFFFCCB2 for sky, 0 for no data.
 * depth: the sample's float depth, +inf for sky, 0 for no data.
 * Rows at or past orc_rays_to_render(rm) were not cast and read as no data.
 * sample_index (optional): the ray-buffer word index each pixel fetched (-1: none). */
void orc_resolve(const orc_raymap* rm, int width, int height, int rows, const uint32_t* raybuf,
                 const float* raydepth, const orc_hit* rayhit, uint32_t* colour, float* depth,
                 orc_hit* hit, int64_t* sample_index);

/* bin/shader/soft.frag over the colorize pass's frame buffer, one resolved
 * frame (RGBA8 colour + float depth as orc_resolve writes them) in, RGBA8
 * out; bilinear taps in single precision, clamped to the frame. */
void orc_soft_filter(const uint32_t* colour, const float* depth, int width, int height, uint32_t* out);

/* Rows the reference's ray buffer has (RAYS_CASTED = 4*maxres, src/main.cpp:459)
 * and the rays a frame renders into it: min(sum res, rows). */
int orc_raybuf_rows(const orc_raymap* rm);
int orc_rays_to_render(const orc_raymap* rm);

#ifdef __cplusplus
}
#endif
#endif
