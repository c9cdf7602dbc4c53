/* rle_gb300: GB300-native (sm_103a) renderer for scenes stored as
 * run-length-encoded voxel columns (.rle4).
 *
 * C ABI.  Every entry point returns an rle_status; device buffers are owned by
 * the caller unless an entry point says otherwise; work is ordered on the
 * CUDA stream the caller passes (a cudaStream_t passed as void*, NULL = the
 * legacy default stream).  Handles are safe to use from several host threads
 * as long as one handle is not freed while in use.
 *
 * The render path replaces the reference's
 *   extern "C" void cuda_main_render2(int pbo_out, int width, int height,
 *                                     RayMap_GPU* raymap)
 * (RLE-Raycaster/src/Cuda_Main.cu:124,183-271) and the code around it:
 *   RayMap::get_ray_map      src/RayMap.h:98-402      -> rle_raymap_build
 *   Render::render_line      src/Cuda_Render.h:96-737 -> rle_render_rays
 *   colorize_*.frag resolve  bin/shader/colorize_buddha_soft.frag:12-80
 *                                                     -> rle_resolve
 *   RLE4::load/all_to_gpu    src/Rle4.cpp:244-448     -> rle_scene_load_*
 * The GL pixel-buffer output of the reference becomes caller-owned device
 * buffers.
 */
#ifndef RLE_GB300_H
#define RLE_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum rle_status {
    RLE_OK = 0,
    RLE_ERR_INVALID_ARG = -1, /* null pointer, bad size, non-finite camera, ... */
    RLE_ERR_IO = -2,          /* file could not be opened or read */
    RLE_ERR_FORMAT = -3,      /* .rle4 bytes inconsistent with their headers */
    RLE_ERR_CUDA = -4,        /* a CUDA runtime call failed */
    RLE_ERR_NO_MEMORY = -5,   /* host or device allocation failed / budget exceeded */
    RLE_ERR_CAPACITY = -6,    /* output or work buffer too small, limit exceeded */
    RLE_ERR_TIMEOUT = -7,     /* a bounded wait gave up */
    RLE_ERR_CANCELLED = -8,   /* request cancelled before it ran */
    RLE_ERR_UNSUPPORTED = -9  /* feature not available on this device/build */
} rle_status;

#define RLE_MAX_MIPS 8

/* Printable name of a status. */
const char* rle_status_string(rle_status s);
/* Build identification, e.g. "rle_gb300 1.0 sm_103a". */
const char* rle_version(void);
/* Message of the last error on the calling host thread (may be empty). */
const char* rle_last_error(void);

/* ---------------------------------------------------------------------- */
/* Scenes                                                                 */
/* ---------------------------------------------------------------------- */

/* A scene resident on one device: per mip level the column table
 * (uint2 {slab_offset, run_count | first_header << 16}, one per column,
 * x fastest) and the slab words (u16 run headers then u16 colours per
 * column), exactly the layout RLE4::load builds (src/Rle4.cpp:285-314),
 * with 32-bit offsets widened to unsigned (up to 2^32 words per level). */
typedef struct rle_scene rle_scene;

typedef struct rle_scene_info {
    int device;
    int nummaps;
    int sx[RLE_MAX_MIPS], sy[RLE_MAX_MIPS], sz[RLE_MAX_MIPS];
    uint64_t slab_words[RLE_MAX_MIPS];
    uint64_t device_bytes;   /* table + slab bytes held on the device */
    uint64_t run_headers;    /* run headers over all columns of level 0 */
    uint64_t surface_voxels; /* colour words of level 0 */
} rle_scene_info;

/* .rle4 file or bytes (src/Rle4.cpp:220-242 format: int nummaps, then per
 * level int sx, sy, sz, slabs_size and u16 slabs[slabs_size]).  Builds the
 * column tables on the host and uploads to `device`.  sx and sz must be
 * powers of two (the renderer wraps the map toroidally). */
rle_status rle_scene_load_file(const char* path, int device, rle_scene** out);
rle_status rle_scene_load_memory(const void* bytes, size_t nbytes, int device, rle_scene** out);
rle_status rle_scene_free(rle_scene* scene);
rle_status rle_scene_get_info(const rle_scene* scene, rle_scene_info* out);
/* Host copy of one level's column table (2*sx*sz u32) and/or slab words. */
rle_status rle_scene_copy_level(const rle_scene* scene, int mip, uint32_t* table, uint16_t* slabs);

/* ---------------------------------------------------------------------- */
/* Synthetic scenes (seeded, deterministic on every host)                 */
/* ---------------------------------------------------------------------- */

typedef struct rle_scenegen_params {
    int sx, sy, sz;          /* grid; sx, sz powers of two >= 8; sy multiple of 64, <= 1024 */
    uint64_t seed;
    int nummaps;             /* mip levels, each halving x, y and z (>= 1) */
    float height_min;        /* fBm ground height range, voxels */
    float height_max;
    int octaves;             /* fBm value-noise octaves */
    int base_period;         /* lattice period of the lowest octave, voxels */
    int caves;               /* carve 3D simplex-noise caves/overhangs */
    float cave_y0, cave_y1;  /* height band the caves live in */
    float cave_threshold;    /* density above which a voxel is carved */
    float cave_period;       /* wavelength of the cave noise, voxels */
} rle_scenegen_params;

/* Defaults for a scene of the given size and seed: heights 32..224 scaled
 * by sy/256, 6 octaves; caves (when asked) in the band 64..200 scaled. */
rle_status rle_scenegen_default(int sx, int sy, int sz, uint64_t seed, int caves,
                                rle_scenegen_params* out);
/* Generates the scene and returns it as .rle4 bytes (free with rle_host_free). */
rle_status rle_scenegen_rle4(const rle_scenegen_params* p, void** bytes, size_t* nbytes);
/* Dense view of one mip level for small scenes: solid bits in the
 * reference's Tree layout (bit i&7 of byte (i + j*sx + k*sx*sy) >> 3) and the
 * RGB565 colour the generator gives every voxel (same index, no >> 3). */
rle_status rle_scenegen_dense(const rle_scenegen_params* p, int mip, uint8_t* bits,
                              uint16_t* colours);
void rle_host_free(void* p);

/* Range-checked debug build (build.py --bounds-check ->
 * librle_gb300_checked.so): every column-table, slab and ray-buffer index
 * the kernels use is checked; a failed check is recorded and the access
 * skipped.  Reads (and with clear != 0 resets) the record of `device`:
 * out4[0] = OR of the failed checks (1 column table, 2 run header, 4 colour
 * word, 8 ray-buffer sample, 16 resolve fetch), out4[1..2] = low and high
 * words of the first failing index.  RLE_ERR_UNSUPPORTED in the regular
 * build.  No reference counterpart (the reference has no such mode). */
rle_status rle_bounds_check_read(int device, uint32_t* out4, int clear);
/* Debug build only: device pointers of one level's column table and slab
 * words and the level's word count, for tests that corrupt a resident scene
 * on purpose (the checked build then has to refuse the bad indices).  The
 * checked build pads every level's words with 64 KB of zeros.
 * RLE_ERR_UNSUPPORTED in the regular build. */
rle_status rle_debug_level_pointers(const rle_scene* scene, int mip, void** table, void** slabs,
                                    uint64_t* words);

/* ---------------------------------------------------------------------- */
/* Soft post-filter                                                       */
/* ---------------------------------------------------------------------- */
/* The reference's second display pass, bin/shader/soft.frag, drawn by
 * src/main.cpp:627-653 over the frame the colorize pass left: per pixel,
 * a box filter over the neighbours near the front depth (an edge-aware
 * blur whose radius grows with 1/z).  Input is one resolved frame as
 * rle_resolve / rle_render_frame write it (RGBA8 colour, float depth; sky
 * and no-data pixels as documented there); output is RGBA8 (alpha: the
 * filtered 0.001/z term of the frame buffer).  width, height <= 2048 (the
 * reference's frame buffer); d_out must not alias d_colour.  Bilinear taps
 * are computed in single precision and clamp to the frame.  Stream-ordered,
 * no synchronisation, no allocation. */
rle_status rle_soft_filter(const uint32_t* d_colour, const float* d_depth, int width, int height,
                           uint32_t* d_out, void* stream);

/* ---------------------------------------------------------------------- */
/* Scene building on the GPU                                              */
/* ---------------------------------------------------------------------- */
/* Both calls build a device-resident scene with kernels only: mip levels,
 * surface extraction, run-length encoding and the column tables are
 * computed in device memory and nothing passes through the host.  A level
 * may hold up to 2^32 - 1 slab words (the .rle4 file stores a signed 32-bit
 * count, src/Rle4.cpp:279,297).  They block until the scene is ready and
 * use temporary device memory of about 2 x the level-0 bit volume plus
 * 16 bytes per level-0 column.  The result is freed with rle_scene_free. */

/* The generator of rle_scenegen_rle4 run on the GPU.  The scene equals,
 * bit for bit, rle_scenegen_rle4 + rle_scene_load_memory for the same
 * parameters (tables, slab words, statistics).
 * Replaces RLE4::compress_all (src/Rle4.cpp:14-48) -> Tree::get_mipmap
 * (src/tree.h:23-85) -> RLE4::compress (src/Rle4.cpp:52-198) ->
 * RLE4::all_to_gpu (src/Rle4.cpp:432-448) for generated scenes. */
rle_status rle_scenegen_device(const rle_scenegen_params* p, int device, rle_scene** out);

/* RLE4::compress_all for a caller's voxel volume already on the device:
 * d_bits is level 0 in the reference's Tree layout (bit i&7 of byte
 * (i + j*sx + k*sx*sy) >> 3, j = 0 the top of the column), sx and sz powers
 * of two >= 8, 1 <= sy <= 1024.  Levels 1..nummaps-1 are Tree::get_mipmap's
 * >= 3-of-8 rule.  Colour word of a stored voxel (i, j, k) of level m:
 * d_colours[(i<<m) + (j<<m)*sx + (k<<m)*sx*sy] when d_colours is not NULL
 * (u16 per level-0 voxel, same index as the bits), else the reference's
 * normal-derived word without material bits (src/Rle4.cpp:134-161, col1 ==
 * NULL).  Reads the inputs on `device`; does not modify them. */
rle_status rle_encode_device(const uint8_t* d_bits, const uint16_t* d_colours, int sx, int sy, int sz,
                             int nummaps, int device, rle_scene** out);

/* ---------------------------------------------------------------------- */
/* Cameras and ray maps                                                   */
/* ---------------------------------------------------------------------- */

typedef struct rle_camera {
    float pos[3];   /* RayMap_GPU.position: x, z on the column grid; y is
                       minus the eye height (a voxel of height h sits at
                       pos[1] + h relative to the eye) */
    float rot[3];   /* RayMap_GPU.rotation: x = pitch in radians (positive
                       looks down), y = yaw in radians, z unused */
    float fov_deg;  /* horizontal field of view; 90 is the reference frustum */
} rle_camera;

typedef struct rle_view_params {
    int width, height;  /* screen in pixels */
    int samples;        /* samples per column ray (RENDER_SIZE); 0 = width */
    int maxres;         /* column rays per unit of fan (RAYS_CASTED_RES/4); 0 = width */
    float border;       /* vertical border of the square ray-map plane; <= 0 = (W-H)/(2W) */
    int mip_distance;   /* distance of the first LOD switch (MIP_DISTANCE); 0 = width */
    int z_far;          /* ray length in DDA steps (RAYS_DISTANCE); 0 = 80000 */
} rle_view_params;

/* Per-frame state of one camera: the fields of RayMap_GPU
 * (src/RayMap.h:16-54) without the scene pointers, plus the render
 * parameters the reference fixes at compile time and the per-frame sines
 * and cosines the device would otherwise compute. */
typedef struct rle_raymap {
    float vanishing_point_2d[3];
    int map_line_count;        /* sum of res[] */
    float rotation[3];
    float position[3];
    float border, clip_min, clip_max;
    int maxres;
    int res[4];                /* column rays of the up, down, left, right fans */
    float p4[3];
    float p_2d[8][3];
    float p_no[8][3];
    float to3d[4][4];
    float p_ofs_min[4], p_ofs_max[4];
    int samples;               /* samples per ray (S) */
    int mip_distance;
    int z_far;
    float fov_scale;           /* tan(fov/2) */
    /* derived, filled by rle_raymap_build */
    float sin_x, cos_x, sin_y, cos_y;    /* of rotation.x / rotation.y */
    float sin_neg_y, cos_neg_y;          /* of -rotation.y */
    int width, height;         /* screen */
    int rows;                  /* ray-buffer rows (RAYS_CASTED = 4*maxres) */
    int rays;                  /* rays rendered: min(map_line_count, rows) */
} rle_raymap;

/* RayMap::get_ray_map for one camera (host, microseconds). */
rle_status rle_raymap_build(const rle_camera* cam, const rle_view_params* view, rle_raymap* out);

/* ---------------------------------------------------------------------- */
/* Rendering                                                              */
/* ---------------------------------------------------------------------- */

/* The voxel that coloured a sample or pixel. */
typedef struct rle_hit {
    uint16_t x, z, y;   /* cell and height at level `mip` */
    uint8_t mip;
    uint8_t flags;      /* 1 = voxel, 2 = sky, 0 = no data */
} rle_hit;

/* Per-ray work counters (the reference's DETAIL_BENCH counters,
 * src/Cuda_Render.h:14-22), summed over a frame. */
typedef struct rle_counters {
    unsigned long long cells;    /* DDA cells stepped */
    unsigned long long fetched;  /* column-table entries read (8 B) */
    unsigned long long headers;  /* run headers read from slabs (2 B) */
    unsigned long long runs;     /* solid runs examined */
    unsigned long long spans;    /* spans drawn */
    unsigned long long pixels;   /* samples coloured (2 B colour read each) */
} rle_counters;

/* Launch shape of the raycast kernel (process-wide; 0 = built-in default).
 *   lanes_per_ray      lanes of a warp cooperating on one column ray: 8, 16
 *                      or 32 (4, 2 or 1 rays per warp); default 32
 *   cells_per_lane     DDA steps each lane takes per chunk: 1 (reserved)
 *   threads_per_block  32, 64, 96 or 128; default 128
 *   staging            staging depth of the column data a ray reads: 1 the
 *                      column-table entries of the next chunk of cells load
 *                      while the current chunk is merged; 2 also each of
 *                      those cells' run-header line is staged in L2 before
 *                      its scan; 3 the same into L1; default 1 */
typedef struct rle_tuning {
    int lanes_per_ray;
    int cells_per_lane;
    int threads_per_block;
    int staging;
} rle_tuning;
rle_status rle_tuning_set(const rle_tuning* t);
rle_status rle_tuning_get(rle_tuning* t);

/* Words of the ray buffer of a ray map: rows * samples. */
size_t rle_raybuf_words(const rle_raymap* rm);

/* Drop-in for cuda_main_render2: casts every column ray of the ray map into
 * the ray buffer, row r = ray r, `samples` words per row.
 *   d_raybuf   (required) colour16 | depth16 << 16 per sample, as the PBO of
 *              the reference; 0x00ff8844 = sky; 0 = outside the ray's range
 *   d_raydepth (required) float depth (1/onez) per sample; +inf sky; 0 none
 *   d_rayhit   (optional) rle_hit per sample
 *   d_counters (optional) one rle_counters, accumulated (atomically)
 * Rows >= rm->rays are left untouched. */
rle_status rle_render_rays(const rle_scene* scene, const rle_raymap* rm, uint32_t* d_raybuf,
                           float* d_raydepth, rle_hit* d_rayhit, rle_counters* d_counters,
                           void* stream);

/* When each column ray of one launch ran: the timing counterpart of the
 * reference's per-ray DETAIL_BENCH records (src/Cuda_Render.h:14-22, summed
 * at src/Cuda_Main.cu:244-267), for profiling.  A frame cannot end before
 * its slowest ray: end_clock - start_clock of that ray, at the SM clock,
 * bounds the launch from below. */
typedef struct rle_ray_time {
    uint64_t start_ns, end_ns;        /* %globaltimer (ns, the same clock on every SM) */
    uint64_t start_clock, end_clock;  /* clock64() of the SM that cast the ray */
    uint32_t sm;                      /* that SM (%smid) */
    uint32_t reserved;
} rle_ray_time;

/* rle_render_rays without hit records or counters (the production kernel the
 * benchmark times) that also writes d_times[r] for every cast ray
 * r < rm->rays.  The two timestamps per ray are the only extra work. */
rle_status rle_render_rays_timed(const rle_scene* scene, const rle_raymap* rm, uint32_t* d_raybuf,
                                 float* d_raydepth, rle_ray_time* d_times, void* stream);

/* The colorize shader's resolve as a kernel: per screen pixel (row 0 at the
 * top), the ray-buffer sample its fan geometry selects.
 *   d_colour RGBA8 (R in the low byte): RGB565 expanded, sky 0xFFFFCCB2, none 0
 *   d_depth  float depth, +inf sky, 0 none
 *   d_hit    (optional) the sample's rle_hit
 * Ray-buffer rows >= rm->rays were not cast and read as no data. */
rle_status rle_resolve(const rle_raymap* rm, const uint32_t* d_raybuf, const float* d_raydepth,
                       const rle_hit* d_rayhit, uint32_t* d_colour, float* d_depth,
                       rle_hit* d_hit, void* stream);

/* Camera to screen in one call: ray map on the host, raycast and resolve on
 * the device.  The ray buffer lives in d_workspace, which must hold
 * rle_frame_workspace_bytes(view) bytes (256-byte aligned). */
size_t rle_frame_workspace_bytes(const rle_view_params* view);
rle_status rle_render_frame(const rle_scene* scene, const rle_camera* cam,
                            const rle_view_params* view, void* d_workspace,
                            size_t workspace_bytes, uint32_t* d_colour, float* d_depth,
                            rle_hit* d_hit, void* stream);

/* ---------------------------------------------------------------------- */
/* Batched rendering                                                      */
/* ---------------------------------------------------------------------- */

/* Many cameras -- any mix of resolutions -- in one call, in one of two
 * launch modes (rle_batch_tuning.per_frame):
 *   per-frame (default): one raycast + resolve launch pair per frame, the
 *     frames forked over eight worker streams of the batch and joined back
 *     on the caller's stream, so up to eight frames are in flight and one
 *     frame's slowest column rays overlap the next frames';
 *   persistent: one raycast launch and one resolve launch for the whole
 *     batch -- the column rays of all frames form one work queue that lane
 *     groups drain tile by tile -- captured once (with the upload of the
 *     per-frame parameters) into a CUDA graph and replayed for every batch.
 * rle_batch_autotune times both over its launch shapes.  No counterpart in
 * the reference, which renders one camera per launch
 * (src/Cuda_Main.cu:183-271). */
typedef struct rle_batch rle_batch;

typedef struct rle_frame_request {
    rle_camera cam;
    rle_view_params view;
    uint32_t* d_colour;  /* width*height RGBA8, as rle_resolve */
    float* d_depth;      /* width*height */
    rle_hit* d_hit;      /* optional; needs a batch created with hits */
} rle_frame_request;

typedef struct rle_batch_tuning {
    int tile_rays;          /* tile width: most adjacent column rays a lane group claims at
                               once, 1..256 (default 1; claims shrink as the queue drains) */
    int lanes_per_ray;      /* lanes cooperating on one column ray: 8, 16, 32 */
    int staging;            /* staging depth of the column data, 1..3, as rle_tuning.staging */
    int threads_per_block;  /* 32, 64, 96 or 128 */
    int use_graph;          /* 1: capture once and replay (default); 0: plain launches */
    int per_frame;          /* 1 (default): one plain raycast + resolve launch pair per frame,
                               the frames forked over eight worker streams of the batch (up
                               to eight in flight) and joined back on the caller's stream;
                               0: the persistent pair */
} rle_batch_tuning;

/* max_frames per batch; raybuf_words: ray-buffer capacity shared by the
 * frames of one batch (a frame needs rays * samples words, see
 * rle_batch_words_needed); max_samples: largest samples-per-ray accepted. */
rle_status rle_batch_create(int device, int max_frames, size_t raybuf_words, int max_samples, int with_hits,
                            rle_batch** out);
rle_status rle_batch_free(rle_batch* b);
rle_status rle_batch_set_tuning(rle_batch* b, const rle_batch_tuning* t);
rle_status rle_batch_get_tuning(const rle_batch* b, rle_batch_tuning* t);
/* Ray-buffer words a set of frames needs (0 if a camera or view is invalid). */
size_t rle_batch_words_needed(const rle_frame_request* frames, int n);
/* Renders n frames; outputs as rle_render_frame.  Asynchronous on `stream`;
 * one batch object renders one batch at a time: calls are serialised on the
 * host, and a call's device work waits for the previous call's (which shares
 * the batch's ray buffer and parameter block), whatever streams they use. */
rle_status rle_batch_render(rle_batch* b, const rle_scene* scene, const rle_frame_request* frames, int n,
                            void* stream);
/* Times every tile_rays x lanes_per_ray x staging combination
 * ({1,2,4,8,16,32,64} x {8,16,32} x {1,2,3}: tile width, 4/2/1 rays per
 * warp, staging depth -- three independent axes) and the per-frame launches
 * (lanes {8,16,32} x staging {1,2,3}) on these frames (median of `repeats`
 * runs each), keeps the fastest as the batch's tuning and returns it. */
rle_status rle_batch_autotune(rle_batch* b, const rle_scene* scene, const rle_frame_request* frames, int n,
                              int repeats, rle_batch_tuning* best, float* best_ms);

/* ---------------------------------------------------------------------- */
/* Serving                                                                */
/* ---------------------------------------------------------------------- */

/* A render server: scenes stay resident on one device, requests queue on the
 * host and a scheduler thread turns the queue into batched launches as soon
 * as a batch slot and ray-buffer memory are free (continuous batching: work
 * that arrives while other batches run joins the next launch, and up to
 * max_inflight batches overlap on the device).  A request's outputs go to
 * device buffers its submitter owns.  No counterpart in the reference,
 * which renders one camera per call in its display loop. */
typedef struct rle_server rle_server;

typedef struct rle_server_config {
    int device;
    size_t hbm_budget_bytes;      /* scenes + the server's ray buffers must fit */
    int max_frames_per_batch;     /* frames one launch may carry */
    int max_inflight;             /* batches on the device at once (>= 1) */
    size_t raybuf_words;          /* ray-buffer words of each batch slot */
    int max_samples;              /* widest samples-per-ray accepted */
    int plain;                    /* 1: one request per launch, one at a time (for comparison) */
    rle_batch_tuning batch_tuning; /* launch shape of the batch slots (rle_batch_set_tuning);
                                      all zero: the batch default (per-frame, 32 lanes) */
} rle_server_config;

typedef struct rle_request {
    int scene_id;
    rle_camera cam;
    rle_view_params view;
    uint32_t* d_colour;
    float* d_depth;
} rle_request;

typedef struct rle_completion {
    uint64_t ticket;
    rle_status status;
    double submit_s, launch_s, done_s;  /* host monotonic clock, seconds */
    double gpu_ms;  /* device time from the start of the batch that carried the request to
                       the end of its frame (CUDA events: one on the slot's stream before
                       the batch, one behind the frame's launches); 0 if it never ran */
} rle_completion;

typedef struct rle_server_stats {
    uint64_t submitted, completed, failed, cancelled, batches;
    double p50_ms, p99_ms, mean_ms, max_ms;  /* submit -> done, over completed requests */
    double pixels;                           /* primary rays rendered */
    double busy_s;                           /* first submit -> last completion */
    double mrays_per_s;                      /* pixels / busy_s / 1e6 */
    uint64_t device_bytes;                   /* scenes + ray buffers held */
} rle_server_stats;

rle_status rle_server_create(const rle_server_config* cfg, rle_server** out);
/* Registers a loaded scene (on the server's device); its device bytes count
 * against the budget (RLE_ERR_NO_MEMORY if it does not fit). */
rle_status rle_server_add_scene(rle_server* s, const rle_scene* scene, int* scene_id);
/* Queues a request (non-blocking).  RLE_ERR_CAPACITY if it could never fit
 * one batch slot; RLE_ERR_INVALID_ARG for a bad scene id, camera or view. */
rle_status rle_server_submit(rle_server* s, const rle_request* r, uint64_t* ticket);
/* Cancels a request still waiting in the queue (RLE_ERR_INVALID_ARG if it
 * already launched or is unknown); it completes with RLE_ERR_CANCELLED. */
rle_status rle_server_cancel(rle_server* s, uint64_t ticket);
/* Waits up to timeout_ms for one request (RLE_ERR_TIMEOUT if it has not
 * completed); on completion fills *out if given. */
rle_status rle_server_wait(rle_server* s, uint64_t ticket, int timeout_ms, rle_completion* out);
/* Waits up to timeout_ms until nothing is queued or running. */
rle_status rle_server_drain(rle_server* s, int timeout_ms);
/* Completions not yet taken, oldest first (up to max). */
rle_status rle_server_poll(rle_server* s, rle_completion* out, int max, int* n);
rle_status rle_server_get_stats(rle_server* s, rle_server_stats* out);
/* Clears the latency record and counters (not the queue). */
rle_status rle_server_reset_stats(rle_server* s);
/* Test hook: the next `count` batch launches fail on the host as a failed
 * CUDA launch would; their requests complete with RLE_ERR_CUDA and the
 * server keeps serving.  No device fault is involved. */
rle_status rle_server_inject_launch_failures(rle_server* s, int count);
/* Holds (1) or resumes (0) launching; queued requests wait meanwhile. */
rle_status rle_server_pause(rle_server* s, int paused);
rle_status rle_server_destroy(rle_server* s);

/* Camera to screen without any device allocation (no counterpart in the
 * reference).  For callers that may not allocate device memory while they
 * run -- a render loop with a hard frame budget (cudaMalloc can synchronise
 * the device), or a plug-in whose host application owns the GPU memory
 * budget.  Same result as rle_render_frame without hit records.
 * The ray buffer lives in a fixed array built into the library:
 * rle_render_frame_noalloc_limit() bytes (64 MiB) per device, held until the
 * process exits.  A frame needs 8 x rays x samples bytes of it (e.g. 1080p
 * with up to ~4300 column rays); larger frames return RLE_ERR_CAPACITY.
 * When the array is reserved: CUDA loads a library's device code lazily by
 * default (CUDA 12.2 and later), so the array is reserved on a device by the
 * first call on that device, which also looks up its device address (with
 * that device current).  That first call can therefore allocate, wait for
 * the device or fail with RLE_ERR_CUDA if the device has no room: make it at
 * start-up, before the frame loop and before any stream capture.  Later calls
 * allocate nothing.  With CUDA_MODULE_LOADING=EAGER in the environment the
 * array is reserved when the library loads instead.
 * The looked-up address is kept for the life of the process: after a
 * cudaDeviceReset of that device it is stale, so do not call this entry
 * point on a device that was reset.
 * All calls share the one array: calls whose work can overlap on the GPU
 * (different streams, or host threads without ordering) race -- issue them on
 * one stream.  Nothing in the array needs clearing: every word a frame reads
 * is written by that frame first. */
size_t rle_render_frame_noalloc_limit(void);
rle_status rle_render_frame_noalloc(const rle_scene* scene, const rle_camera* cam,
                                    const rle_view_params* view, uint32_t* d_colour, float* d_depth,
                                    void* stream);

#ifdef __cplusplus
}
#endif
#endif
