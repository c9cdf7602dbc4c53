// Internal declarations shared by the host C++ and the CUDA translation units.
#pragma once

#include <cuda_runtime_api.h>
#include <vector_types.h>

#include "scenegen_math.h"

#include <cstddef>
#include <cstdint>
#include <string>

#include "rle_gb300.h"

namespace rle {

// Per-thread last-error message behind rle_last_error().
void set_error(const char* fmt, ...);
void clear_error();

// One mip level resident on the device.  The table is the uint2 column
// directory {slab_offset, run_count | first_header << 16}, x fastest
// (RLE4::load, src/Rle4.cpp:285-314); slabs are the u16 words.
struct Level {
    int sx = 0, sy = 0, sz = 0;
    uint64_t words = 0;
    uint32_t* d_table = nullptr;  // 2 * sx * sz words
    uint16_t* d_slabs = nullptr;  // words (+ 8 words of zero padding)
};

}  // namespace rle

struct rle_scene {
    int device = 0;
    int nummaps = 0;
    rle::Level lv[RLE_MAX_MIPS];
    uint64_t device_bytes = 0;
    uint64_t run_headers = 0;
    uint64_t surface_voxels = 0;
    // smallest column-axis index (level-0 units) of any stored voxel on any
    // level: nothing in the scene lies above it
    int top_index = 0;
    int height = 0;  // sy of level 0
};

namespace rle {

// Zero padding after each level's slab words: keeps a column's last 16-byte
// header group inside the allocation.  The bounds-checked build pads 64 KB,
// so that reads its checks refuse would still land in zeros.
#ifdef RLE_BOUNDS_CHECK
constexpr size_t kSlabPadBytes = 65536;
#else
constexpr size_t kSlabPadBytes = 16;
#endif

// Bounds-check word codes (RLE_BOUNDS_CHECK builds).
enum BoundsCode : unsigned {
    kBoundsTable = 1u,    // column-table index past the level
    kBoundsHeader = 2u,   // run-header index past the level's words
    kBoundsColour = 4u,   // colour-word index past the level's words
    kBoundsRay = 8u,      // ray-buffer row or sample index out of range
    kBoundsResolve = 16u  // resolve fetch outside the ray buffer
};

// Host-side .rle4 parse + column-table build (no device work).
struct HostLevel {
    int sx = 0, sy = 0, sz = 0;
    const uint16_t* slabs = nullptr;  // points into the caller's bytes
    uint64_t words = 0;
};
rle_status parse_rle4(const void* bytes, size_t nbytes, HostLevel* levels, int* nummaps);
rle_status build_table(const HostLevel& lv, uint32_t* table, uint64_t* run_headers,
                       uint64_t* surface_voxels, int* top_index = nullptr);

// Kernel parameters of one ray map bound to one scene.  Everything the
// device needs per frame, passed by value as a __grid_constant__.
struct RayParams {
    float p5x, p5y, p5z;          // p_2d[5] (z cleared as src/RayMap.h:206)
    float p_no[8][3];
    float to3d[4][4];
    float p4[3];
    float clip_min, clip_max;
    int res[4];
    float sin_x, cos_x, sin_y, cos_y, sin_ny, cos_ny;
    float posx, posy, posz;
    float rotx;
    float focal;                  // (S/2) / fov_scale
    int S;                        // samples per ray
    int rays;                     // rays to cast
    int mapswitch0;               // MIP_DISTANCE * (0.25*(4-|rot.x|)), src/Cuda_Render.h:335
    int z_far;
    int nummaps;
    int gridx0, gridz0;
    int top_index;                // scene's topmost voxel index (level-0 units)
    int height;                   // scene height (level 0)
    const uint2* table[RLE_MAX_MIPS];
    const uint16_t* slabs[RLE_MAX_MIPS];
    uint64_t slab_words[RLE_MAX_MIPS];  // words per level (bounds checks)
    uint32_t table_cols[RLE_MAX_MIPS];  // columns per level (bounds checks)
    uint32_t* raybuf;
    float* raydepth;
    rle_hit* rayhit;
    rle_counters* counters;
    rle_ray_time* ray_time;       // per-ray start/end times (single-frame kernel), or null
    // launch shape (0 = default): lanes cooperating on one ray, DDA steps
    // each lane claims per chunk, block size
    int lanes_per_ray;
    int cells_per_lane;
    int threads_per_block;
    int staging;                  // staging depth of the column data (1..3; 0 = default)
};

// Per-frame constants of the resolve (uniforms of colorize_buddha_soft.frag).
struct ResolveParams {
    float resx, resy;
    float vanish_x, vanish_y;
    float ofs_x, ofs_y, ofs_z, ofs_w;
    float ratio;
    float rxg0;
    int width, height;
    int S, rows;
    int rays;                     // rows >= rays were not cast: no data
    const uint32_t* raybuf;
    const float* raydepth;
    const rle_hit* rayhit;
    uint32_t* colour;
    float* depth;
    rle_hit* hit;
};

rle_status fill_ray_params(const rle_scene* scene, const rle_raymap* rm, RayParams* p);
rle_status fill_resolve_params(const rle_raymap* rm, ResolveParams* p);

// Kernel launchers (render.cu, resolve.cu).
rle_status launch_raycast(const RayParams& p, void* stream);
rle_status launch_resolve(const ResolveParams& p, void* stream);

// Many frames in one launch each (batch.cpp drives these).  The frame count
// and the work counter live in device memory, so one captured graph serves
// every batch size.
struct BatchHeader {
    int nframes;
    unsigned int next_ray;     // work counter, zero before the launch
    int pad[2];
};
struct BatchRaycast {
    BatchHeader* header;       // device
    const int* ray_start;      // device array [nframes + 1], prefix of rays
    const RayParams* frames;   // device array [nframes]
    int tile;                  // most adjacent rays a lane group claims at once
    int staging;               // staging depth of the column data (1..3)
    int lanes;                 // lanes per ray: 8, 16, 32
    int threads;               // block size
    int max_samples;           // largest S of the frames the launch may see
    int blocks;                // grid size (0: fill the GPU)
    int hits;                  // frames may carry hit buffers
};
struct BatchResolve {
    const BatchHeader* header;    // device
    const int* block_start;       // device array [nframes + 1], prefix of 256-pixel blocks
    const ResolveParams* frames;  // device array [nframes]
    int blocks;                   // persistent grid size
};
rle_status launch_raycast_batch(const BatchRaycast& b, void* stream);
rle_status launch_resolve_batch(const BatchResolve& b, void* stream);
int resolve_batch_blocks(int width, int height);  // 256-pixel blocks of one frame

// A batch whose frames may come from different scenes (one per frame).
// frame_done (optional, n events): event i is recorded once frame i's outputs
// are written (per-frame mode: behind its own launches; persistent: behind
// the batch).
rle_status batch_render_scenes(rle_batch* b, const rle_scene* const* scenes, const rle_frame_request* frames, int n,
                               void* stream, cudaEvent_t* frame_done = nullptr);
size_t batch_capacity_words(const rle_batch* b);
int batch_max_frames(const rle_batch* b);
rle_status batch_grid_blocks(int lanes, int threads, int max_samples, bool hits, int staging, int* blocks);

// Bounds-check words of the device code (zeros when none fired); false in
// builds without RLE_BOUNDS_CHECK.  read: flags, first index hit; clear
// resets them.
bool bounds_render(unsigned* out4, bool clear);
bool bounds_resolve(unsigned* out4, bool clear);

// Scene generator pieces shared by the host and device generators.
rle_status scenegen_check(const rle_scenegen_params* p);
void scenegen_perm(uint64_t seed, uint8_t* perm512);
gen::Consts scenegen_consts(const rle_scenegen_params& p);

}  // namespace rle
