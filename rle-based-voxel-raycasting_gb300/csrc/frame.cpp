// C entry points of the render path: ray map + scene -> kernel parameters,
// argument validation, and the one-call frame (raycast + resolve).
//
// rle_render_rays is the drop-in for cuda_main_render2 (src/Cuda_Main.cu:183-271):
// the reference maps a GL pixel buffer, copies an ~82 KB Render struct to the
// device, launches cudaRender and synchronises; here the caller's device
// buffers are written, the per-frame constants travel as a kernel parameter
// and nothing synchronises the host.
#include <cuda_runtime.h>

#include <atomic>
#include <cmath>
#include <cstring>

#include "rle_internal.h"

namespace rle {

rle_status fill_ray_params(const rle_scene* scene, const rle_raymap* rm, RayParams* p) {
    std::memset(p, 0, sizeof(*p));
    if (rm->samples < 8 || rm->samples > 16384 || rm->rays < 0 || rm->rays > rm->rows || rm->maxres < 1 ||
        rm->rows != 4 * rm->maxres || !(rm->fov_scale > 0.0f) || !std::isfinite(rm->fov_scale)) {
        set_error("ray map: inconsistent sizes (build it with rle_raymap_build)");
        return RLE_ERR_INVALID_ARG;
    }
    for (int i = 0; i < 4; i++) {
        if (rm->res[i] < 0) {
            set_error("ray map: negative ray count");
            return RLE_ERR_INVALID_ARG;
        }
    }
    for (int i = 0; i < 3; i++) {
        if (!std::isfinite(rm->position[i]) || std::fabs(rm->position[i]) > 1.0e6f || !std::isfinite(rm->rotation[i])) {
            set_error("ray map: camera position/rotation must be finite, |pos| <= 1e6");
            return RLE_ERR_INVALID_ARG;
        }
    }
    p->p5x = rm->p_2d[5][0];
    p->p5y = rm->p_2d[5][1];
    p->p5z = rm->p_2d[5][2];
    std::memcpy(p->p_no, rm->p_no, sizeof(p->p_no));
    std::memcpy(p->to3d, rm->to3d, sizeof(p->to3d));
    std::memcpy(p->p4, rm->p4, sizeof(p->p4));
    p->clip_min = rm->clip_min;
    p->clip_max = rm->clip_max;
    std::memcpy(p->res, rm->res, sizeof(p->res));
    p->sin_x = rm->sin_x;
    p->cos_x = rm->cos_x;
    p->sin_y = rm->sin_y;
    p->cos_y = rm->cos_y;
    p->sin_ny = rm->sin_neg_y;
    p->cos_ny = rm->cos_neg_y;
    p->posx = rm->position[0];
    p->posy = rm->position[1];
    p->posz = rm->position[2];
    p->rotx = rm->rotation[0];
    p->S = rm->samples;
    p->focal = static_cast<float>(rm->samples / 2) / rm->fov_scale;
    p->rays = rm->rays;
    // mapswitch * (0.25*(4-abs(viewrot.x))): float subtraction, double
    // product, truncation to int (src/Cuda_Render.h:335)
    p->mapswitch0 = static_cast<int>(static_cast<double>(rm->mip_distance) *
                                     (0.25 * static_cast<double>(4.0f - std::fabs(rm->rotation[0]))));
    p->z_far = rm->z_far;
    p->nummaps = scene->nummaps;
    p->gridx0 = scene->lv[0].sx;
    p->gridz0 = scene->lv[0].sz;
    p->top_index = scene->top_index;
    p->height = scene->height;
    for (int m = 0; m < scene->nummaps; m++) {
        p->table[m] = reinterpret_cast<const uint2*>(scene->lv[m].d_table);
        p->slabs[m] = scene->lv[m].d_slabs;
        p->slab_words[m] = scene->lv[m].words;
        p->table_cols[m] = static_cast<uint32_t>(static_cast<uint64_t>(scene->lv[m].sx) * scene->lv[m].sz);
    }
    return RLE_OK;
}

rle_status fill_resolve_params(const rle_raymap* rm, ResolveParams* p) {
    std::memset(p, 0, sizeof(*p));
    if (rm->width < 1 || rm->height < 1 || rm->samples < 1 || rm->rows < 1 || rm->maxres < 1) {
        set_error("ray map: inconsistent sizes (build it with rle_raymap_build)");
        return RLE_ERR_INVALID_ARG;
    }
    const float resx = static_cast<float>(rm->width), resy = static_cast<float>(rm->height);
    const float rcr = static_cast<float>(4 * rm->maxres);  // RAYS_CASTED_RES
    p->resx = resx;
    p->resy = resy;
    // uniforms of the colorize shader (src/main.cpp:575-603)
    p->vanish_x = 1 - rm->vanishing_point_2d[0];
    p->vanish_y = (1 - rm->vanishing_point_2d[1] - rm->border) * resx / resy;
    const float ofs1 = 4 * static_cast<float>(rm->res[0]) / rcr;
    const float ofs2 = 4 * static_cast<float>(rm->res[1]) / rcr + ofs1;
    const float ofs3 = 4 * static_cast<float>(rm->res[2]) / rcr + ofs2;
    p->ofs_x = -rm->p_ofs_min[0];
    p->ofs_y = -rm->p_ofs_min[1] + ofs1;
    p->ofs_z = -rm->p_ofs_min[2] + ofs2;
    p->ofs_w = -rm->p_ofs_min[3] + ofs3;
    p->ratio = rcr / static_cast<float>(rm->rows);
    p->rxg0 = rm->rotation[0] > 0 ? 1.0f : 0.0f;
    p->width = rm->width;
    p->height = rm->height;
    p->S = rm->samples;
    p->rows = rm->rows;
    p->rays = rm->rays;
    return RLE_OK;
}

namespace {

struct DeviceGuard {
    int prev = -1;
    bool ok = true;
    explicit DeviceGuard(int dev) {
        cudaGetDevice(&prev);
        if (prev != dev) ok = cudaSetDevice(dev) == cudaSuccess;
    }
    ~DeviceGuard() {
        int cur = -1;
        cudaGetDevice(&cur);
        if (prev >= 0 && cur != prev) cudaSetDevice(prev);
    }
};

}  // namespace
}  // namespace rle

namespace {
std::atomic<int> g_lanes_per_ray{0};
std::atomic<int> g_cells_per_lane{0};
std::atomic<int> g_threads_per_block{0};
std::atomic<int> g_staging{0};

bool shape_built(int lanes, int cells) {
    return (lanes == 0 || lanes == 8 || lanes == 16 || lanes == 32) && (cells == 0 || cells == 1);
}
}  // namespace

extern "C" rle_status rle_tuning_set(const rle_tuning* t) {
    if (!t) return RLE_ERR_INVALID_ARG;
    const int l = t->lanes_per_ray, c = t->cells_per_lane, b = t->threads_per_block, st = t->staging;
    if (!shape_built(l, c) || b < 0 || b > 128 || b % 32 != 0 || st < 0 || st > 3) {
        rle::set_error("rle_tuning_set: lanes_per_ray in {0,8,16,32}, cells_per_lane in {0,1}, threads_per_block in "
                       "{0,32,..,128}, staging in {0,1,2,3}");
        return RLE_ERR_INVALID_ARG;
    }
    g_lanes_per_ray = l;
    g_cells_per_lane = c;
    g_threads_per_block = b;
    g_staging = st;
    return RLE_OK;
}

extern "C" rle_status rle_tuning_get(rle_tuning* t) {
    if (!t) return RLE_ERR_INVALID_ARG;
    t->lanes_per_ray = g_lanes_per_ray;
    t->cells_per_lane = g_cells_per_lane;
    t->threads_per_block = g_threads_per_block;
    t->staging = g_staging;
    return RLE_OK;
}

extern "C" size_t rle_raybuf_words(const rle_raymap* rm) {
    if (!rm || rm->rows < 0 || rm->samples < 0) return 0;
    return static_cast<size_t>(rm->rows) * static_cast<size_t>(rm->samples);
}

extern "C" rle_status rle_render_rays(const rle_scene* scene, const rle_raymap* rm, uint32_t* d_raybuf,
                                      float* d_raydepth, rle_hit* d_rayhit, rle_counters* d_counters,
                                      void* stream) {
    if (!scene || !rm || !d_raybuf || !d_raydepth) {
        rle::set_error("rle_render_rays: scene, ray map, ray buffer and depth buffer are required");
        return RLE_ERR_INVALID_ARG;
    }
    rle::RayParams p;
    rle_status st = rle::fill_ray_params(scene, rm, &p);
    if (st != RLE_OK) return st;
    p.raybuf = d_raybuf;
    p.raydepth = d_raydepth;
    p.rayhit = d_rayhit;
    p.counters = d_counters;
    p.lanes_per_ray = g_lanes_per_ray;
    p.cells_per_lane = g_cells_per_lane;
    p.threads_per_block = g_threads_per_block;
    p.staging = g_staging;
    rle::DeviceGuard g(scene->device);
    if (!g.ok) {
        rle::set_error("rle_render_rays: cannot select device %d", scene->device);
        return RLE_ERR_CUDA;
    }
    return rle::launch_raycast(p, stream);
}

extern "C" rle_status rle_render_rays_timed(const rle_scene* scene, const rle_raymap* rm, uint32_t* d_raybuf,
                                            float* d_raydepth, rle_ray_time* d_times, void* stream) {
    if (!scene || !rm || !d_raybuf || !d_raydepth || !d_times) {
        rle::set_error("rle_render_rays_timed: scene, ray map, ray/depth buffers and the time records are required");
        return RLE_ERR_INVALID_ARG;
    }
    rle::RayParams p;
    rle_status st = rle::fill_ray_params(scene, rm, &p);
    if (st != RLE_OK) return st;
    p.raybuf = d_raybuf;
    p.raydepth = d_raydepth;
    p.ray_time = d_times;
    p.lanes_per_ray = g_lanes_per_ray;
    p.cells_per_lane = g_cells_per_lane;
    p.threads_per_block = g_threads_per_block;
    p.staging = g_staging;
    rle::DeviceGuard g(scene->device);
    if (!g.ok) {
        rle::set_error("rle_render_rays_timed: cannot select device %d", scene->device);
        return RLE_ERR_CUDA;
    }
    return rle::launch_raycast(p, stream);
}

extern "C" rle_status rle_resolve(const rle_raymap* rm, const uint32_t* d_raybuf, const float* d_raydepth,
                                  const rle_hit* d_rayhit, uint32_t* d_colour, float* d_depth, rle_hit* d_hit,
                                  void* stream) {
    if (!rm || !d_raybuf || !d_raydepth || !d_colour || !d_depth) {
        rle::set_error("rle_resolve: ray map, ray/depth buffers and colour/depth outputs are required");
        return RLE_ERR_INVALID_ARG;
    }
    rle::ResolveParams p;
    rle_status st = rle::fill_resolve_params(rm, &p);
    if (st != RLE_OK) return st;
    p.raybuf = d_raybuf;
    p.raydepth = d_raydepth;
    p.rayhit = d_rayhit;
    p.colour = d_colour;
    p.depth = d_depth;
    p.hit = d_hit;
    return rle::launch_resolve(p, stream);
}

namespace {

// Workspace layout of one frame: ray buffer, depth buffer, hit buffer,
// each 256-byte aligned.
struct FrameLayout {
    size_t raybuf = 0, raydepth = 0, rayhit = 0, total = 0;
};

FrameLayout frame_layout(size_t words) {
    auto up = [](size_t v) { return (v + 255) & ~static_cast<size_t>(255); };
    FrameLayout l;
    l.raybuf = 0;
    l.raydepth = up(words * 4);
    l.rayhit = l.raydepth + up(words * 4);
    l.total = l.rayhit + up(words * sizeof(rle_hit));
    return l;
}

size_t view_words(const rle_view_params* v) {
    const int S = v->samples > 0 ? v->samples : v->width;
    const int maxres = v->maxres > 0 ? v->maxres : v->width;
    return static_cast<size_t>(4 * maxres) * static_cast<size_t>(S);
}

}  // namespace

extern "C" size_t rle_frame_workspace_bytes(const rle_view_params* view) {
    if (!view || view->width <= 0) return 0;
    return frame_layout(view_words(view)).total;
}

extern "C" rle_status rle_render_frame(const rle_scene* scene, const rle_camera* cam, const rle_view_params* view,
                                       void* d_workspace, size_t workspace_bytes, uint32_t* d_colour,
                                       float* d_depth, rle_hit* d_hit, void* stream) {
    if (!scene || !cam || !view || !d_workspace || !d_colour || !d_depth) {
        rle::set_error("rle_render_frame: null argument");
        return RLE_ERR_INVALID_ARG;
    }
    if ((reinterpret_cast<uintptr_t>(d_workspace) & 255) != 0) {
        rle::set_error("rle_render_frame: workspace must be 256-byte aligned");
        return RLE_ERR_INVALID_ARG;
    }
    rle_raymap rm;
    rle_status st = rle_raymap_build(cam, view, &rm);
    if (st != RLE_OK) return st;
    const FrameLayout l = frame_layout(rle_raybuf_words(&rm));
    if (workspace_bytes < l.total) {
        rle::set_error("rle_render_frame: workspace %zu bytes, %zu needed", workspace_bytes, l.total);
        return RLE_ERR_CAPACITY;
    }
    char* ws = static_cast<char*>(d_workspace);
    uint32_t* raybuf = reinterpret_cast<uint32_t*>(ws + l.raybuf);
    float* raydepth = reinterpret_cast<float*>(ws + l.raydepth);
    rle_hit* rayhit = d_hit ? reinterpret_cast<rle_hit*>(ws + l.rayhit) : nullptr;
    st = rle_render_rays(scene, &rm, raybuf, raydepth, rayhit, nullptr, stream);
    if (st != RLE_OK) return st;
    rle::DeviceGuard g(scene->device);
    return rle_resolve(&rm, raybuf, raydepth, rayhit, d_colour, d_depth, d_hit, stream);
}

extern "C" rle_status rle_bounds_check_read(int device, uint32_t* out4, int clear) {
    if (!out4) return RLE_ERR_INVALID_ARG;
    int prev = -1;
    cudaGetDevice(&prev);
    if (cudaSetDevice(device) != cudaSuccess) {
        rle::set_error("rle_bounds_check_read: device %d", device);
        return RLE_ERR_INVALID_ARG;
    }
    unsigned a[4] = {0, 0, 0, 0}, b[4] = {0, 0, 0, 0};
    const bool ok = rle::bounds_render(a, clear != 0) && rle::bounds_resolve(b, clear != 0);
    if (prev >= 0) cudaSetDevice(prev);
    if (!ok) {
        rle::set_error("rle_bounds_check_read: this library was built without RLE_BOUNDS_CHECK");
        return RLE_ERR_UNSUPPORTED;
    }
    out4[0] = a[0] | b[0];
    out4[1] = a[0] ? a[1] : b[1];
    out4[2] = a[0] ? a[2] : b[2];
    out4[3] = 0;
    return RLE_OK;
}

extern "C" rle_status rle_debug_level_pointers(const rle_scene* scene, int mip, void** table, void** slabs,
                                               uint64_t* words) {
#ifdef RLE_BOUNDS_CHECK
    if (!scene || mip < 0 || mip >= scene->nummaps || !table || !slabs || !words) return RLE_ERR_INVALID_ARG;
    *table = scene->lv[mip].d_table;
    *slabs = scene->lv[mip].d_slabs;
    *words = scene->lv[mip].words;
    return RLE_OK;
#else
    (void)scene;
    (void)mip;
    (void)table;
    (void)slabs;
    (void)words;
    rle::set_error("rle_debug_level_pointers: this library was built without RLE_BOUNDS_CHECK");
    return RLE_ERR_UNSUPPORTED;
#endif
}
