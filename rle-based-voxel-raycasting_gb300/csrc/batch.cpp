// Batched rendering: many cameras per call, either as one plain launch pair
// per frame forked over worker streams (the default) or as one persistent
// raycast launch and one persistent resolve launch, captured once into a
// CUDA graph.
//
// Per batch the host builds every frame's ray map, packs the per-frame
// kernel parameters, the ray and pixel-block prefix sums and the frame count
// into a pinned staging block and the graph copies it to the device before
// the two kernels run.  Two staging blocks alternate, each guarded by an
// event, so the host prepares batch n+1 while batch n is on the GPU.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <mutex>
#include <new>
#include <vector>

#include "rle_internal.h"

namespace {

size_t align_up(size_t v, size_t a) { return (v + a - 1) / a * a; }

struct Layout {
    size_t header = 0, ray_start = 0, block_start = 0, ray_params = 0, resolve_params = 0, total = 0;
    explicit Layout(int max_frames) {
        header = 0;
        ray_start = align_up(sizeof(rle::BatchHeader), 256);
        block_start = align_up(ray_start + sizeof(int) * (max_frames + 1), 256);
        ray_params = align_up(block_start + sizeof(int) * (max_frames + 1), 256);
        resolve_params = align_up(ray_params + sizeof(rle::RayParams) * max_frames, 256);
        total = align_up(resolve_params + sizeof(rle::ResolveParams) * max_frames, 256);
    }
};

bool valid_tuning(const rle_batch_tuning& t) {
    return t.tile_rays >= 1 && t.tile_rays <= 256 && (t.lanes_per_ray == 8 || t.lanes_per_ray == 16 ||
                                                      t.lanes_per_ray == 32) &&
           t.staging >= 1 && t.staging <= 3 && t.threads_per_block >= 32 && t.threads_per_block <= 128 &&
           t.threads_per_block % 32 == 0 && (t.use_graph == 0 || t.use_graph == 1) &&
           (t.per_frame == 0 || t.per_frame == 1);
}

rle_status cuda_fail(cudaError_t e, const char* what) {
    rle::set_error("%s: %s", what, cudaGetErrorString(e));
    return e == cudaErrorMemoryAllocation ? RLE_ERR_NO_MEMORY : RLE_ERR_CUDA;
}

}  // namespace

struct rle_batch {
    int device = 0;
    int max_frames = 0;
    size_t raybuf_words = 0;
    int max_samples = 0;
    bool with_hits = false;
    Layout layout{1};
    uint32_t* d_raybuf = nullptr;
    float* d_raydepth = nullptr;
    rle_hit* d_rayhit = nullptr;
    unsigned char* d_params = nullptr;
    unsigned char* h_params[2] = {nullptr, nullptr};
    cudaEvent_t staged[2] = {nullptr, nullptr};
    bool staged_used[2] = {false, false};
    int parity = 0;
    cudaStream_t capture = nullptr;
    cudaGraphExec_t graph[2] = {nullptr, nullptr};
    // per-frame mode: the frames' launch pairs fork over these streams and
    // join back on the caller's stream
    static constexpr int kWorkers = 8;
    cudaStream_t workers[kWorkers] = {};
    cudaEvent_t fork = nullptr;
    cudaEvent_t joins[kWorkers] = {};
    // per-frame launches at 32 lanes: measured ahead of the persistent pair
    // on batches of 1080p frames, on the config-3 mix and in the config-4
    // server (lower latency and higher saturated throughput)
    rle_batch_tuning tuning{1, 32, 1, 128, 1, 1};
    int raycast_blocks = 0;
    int resolve_blocks = 0;
    std::mutex mu;
};

namespace {

void drop_graphs(rle_batch* b) {
    for (auto& g : b->graph) {
        if (g) cudaGraphExecDestroy(g);
        g = nullptr;
    }
}

void release(rle_batch* b) {
    if (!b) return;
    int prev = -1;
    cudaGetDevice(&prev);
    cudaSetDevice(b->device);
    drop_graphs(b);
    for (int i = 0; i < 2; i++) {
        if (b->staged[i]) {
            cudaEventSynchronize(b->staged[i]);
            cudaEventDestroy(b->staged[i]);
        }
        if (b->h_params[i]) cudaFreeHost(b->h_params[i]);
    }
    if (b->capture) cudaStreamDestroy(b->capture);
    for (int w = 0; w < rle_batch::kWorkers; w++) {
        if (b->workers[w]) {
            cudaStreamSynchronize(b->workers[w]);
            cudaStreamDestroy(b->workers[w]);
        }
        if (b->joins[w]) cudaEventDestroy(b->joins[w]);
    }
    if (b->fork) cudaEventDestroy(b->fork);
    if (b->d_raybuf) cudaFree(b->d_raybuf);
    if (b->d_raydepth) cudaFree(b->d_raydepth);
    if (b->d_rayhit) cudaFree(b->d_rayhit);
    if (b->d_params) cudaFree(b->d_params);
    if (prev >= 0) cudaSetDevice(prev);
    delete b;
}

rle_status prepare_grid(rle_batch* b) {
    rle_status st = rle::batch_grid_blocks(b->tuning.lanes_per_ray, b->tuning.threads_per_block, b->max_samples,
                                           b->with_hits, b->tuning.staging, &b->raycast_blocks);
    if (st != RLE_OK) return st;
    int sms = 0;
    const cudaError_t e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, b->device);
    if (e != cudaSuccess) return cuda_fail(e, "cudaDeviceGetAttribute");
    b->resolve_blocks = sms * 8;
    return RLE_OK;
}

// Fills the staging block `h` for these frames; returns the frame count.
rle_status stage_frames(rle_batch* b, const rle_scene* scene, const rle_scene* const* scenes,
                        const rle_frame_request* frames, int n, unsigned char* h) {
    const Layout& L = b->layout;
    auto* hdr = reinterpret_cast<rle::BatchHeader*>(h + L.header);
    auto* ray_start = reinterpret_cast<int*>(h + L.ray_start);
    auto* block_start = reinterpret_cast<int*>(h + L.block_start);
    auto* rp = reinterpret_cast<rle::RayParams*>(h + L.ray_params);
    auto* sp = reinterpret_cast<rle::ResolveParams*>(h + L.resolve_params);
    size_t words = 0;
    long long rays = 0, blocks = 0;
    for (int i = 0; i < n; i++) {
        const rle_frame_request& fr = frames[i];
        if (!fr.d_colour || !fr.d_depth || (fr.d_hit && !b->with_hits)) {
            rle::set_error("rle_batch_render: frame %d: colour and depth outputs required%s", i,
                           fr.d_hit && !b->with_hits ? "; hits need a batch created with hits" : "");
            return RLE_ERR_INVALID_ARG;
        }
        rle_raymap rm;
        rle_status st = rle_raymap_build(&fr.cam, &fr.view, &rm);
        if (st != RLE_OK) return st;
        if (rm.samples > b->max_samples) {
            rle::set_error("rle_batch_render: frame %d has %d samples per ray, the batch accepts %d", i, rm.samples,
                           b->max_samples);
            return RLE_ERR_CAPACITY;
        }
        const rle_scene* sc = scenes ? scenes[i] : scene;
        if (!sc || sc->device != b->device) {
            rle::set_error("rle_batch_render: frame %d: scene missing or on another device", i);
            return RLE_ERR_INVALID_ARG;
        }
        st = rle::fill_ray_params(sc, &rm, &rp[i]);
        if (st != RLE_OK) return st;
        st = rle::fill_resolve_params(&rm, &sp[i]);
        if (st != RLE_OK) return st;
        const size_t need = align_up(static_cast<size_t>(rm.rays) * rm.samples, 32);
        if (words + need > b->raybuf_words) {
            rle::set_error("rle_batch_render: frames need more than the batch's %zu ray-buffer words",
                           b->raybuf_words);
            return RLE_ERR_CAPACITY;
        }
        // only the rows of the rays cast are stored (the resolve reads no other)
        rp[i].raybuf = b->d_raybuf + words;
        rp[i].raydepth = b->d_raydepth + words;
        rp[i].rayhit = fr.d_hit ? b->d_rayhit + words : nullptr;
        rp[i].counters = nullptr;
        sp[i].raybuf = rp[i].raybuf;
        sp[i].raydepth = rp[i].raydepth;
        sp[i].rayhit = rp[i].rayhit;
        sp[i].colour = fr.d_colour;
        sp[i].depth = fr.d_depth;
        sp[i].hit = fr.d_hit;
        words += need;
        ray_start[i] = static_cast<int>(rays);
        block_start[i] = static_cast<int>(blocks);
        rays += rm.rays;
        blocks += rle::resolve_batch_blocks(rm.width, rm.height);
        if (rays > 0x7fffffffLL || blocks > 0x7fffffffLL) {
            rle::set_error("rle_batch_render: batch too large");
            return RLE_ERR_CAPACITY;
        }
    }
    ray_start[n] = static_cast<int>(rays);
    block_start[n] = static_cast<int>(blocks);
    std::memset(hdr, 0, sizeof(*hdr));
    hdr->nframes = n;
    hdr->next_ray = 0;
    return RLE_OK;
}

rle_status enqueue(rle_batch* b, int parity, cudaStream_t s) {
    const Layout& L = b->layout;
    cudaError_t e = cudaMemcpyAsync(b->d_params, b->h_params[parity], L.total, cudaMemcpyHostToDevice, s);
    if (e != cudaSuccess) return cuda_fail(e, "rle_batch_render: parameter upload");
    rle::BatchRaycast rc;
    rc.header = reinterpret_cast<rle::BatchHeader*>(b->d_params + L.header);
    rc.ray_start = reinterpret_cast<const int*>(b->d_params + L.ray_start);
    rc.frames = reinterpret_cast<const rle::RayParams*>(b->d_params + L.ray_params);
    rc.tile = b->tuning.tile_rays;
    rc.staging = b->tuning.staging;
    rc.lanes = b->tuning.lanes_per_ray;
    rc.threads = b->tuning.threads_per_block;
    rc.max_samples = b->max_samples;
    rc.blocks = b->raycast_blocks;
    rc.hits = b->with_hits ? 1 : 0;
    rle_status st = rle::launch_raycast_batch(rc, s);
    if (st != RLE_OK) return st;
    rle::BatchResolve rs;
    rs.header = rc.header;
    rs.block_start = reinterpret_cast<const int*>(b->d_params + L.block_start);
    rs.frames = reinterpret_cast<const rle::ResolveParams*>(b->d_params + L.resolve_params);
    rs.blocks = b->resolve_blocks;
    return rle::launch_resolve_batch(rs, s);
}

// frame_done (optional, n events): event i is recorded once frame i's
// outputs are written -- behind the frame's own launches in per-frame mode,
// behind the whole batch in persistent mode.
rle_status render_locked(rle_batch* b, const rle_scene* scene, const rle_scene* const* scenes,
                         const rle_frame_request* frames, int n, cudaStream_t stream,
                         cudaEvent_t* frame_done = nullptr) {
    const int par = b->parity;
    if (b->staged_used[par]) {
        const cudaError_t e = cudaEventSynchronize(b->staged[par]);
        if (e != cudaSuccess) return cuda_fail(e, "rle_batch_render: waiting for the staging block");
    }
    rle_status st = stage_frames(b, scene, scenes, frames, n, b->h_params[par]);
    if (st != RLE_OK) return st;
    // The previous call's launches use the same device parameter block and
    // ray buffer; on another stream they may still be running, so this
    // call's device work waits for them (a no-op on the same stream).
    if (b->staged_used[par ^ 1]) {
        const cudaError_t e = cudaStreamWaitEvent(stream, b->staged[par ^ 1], 0);
        if (e != cudaSuccess) return cuda_fail(e, "rle_batch_render: ordering after the previous batch");
    }
    if (!b->raycast_blocks) {
        st = prepare_grid(b);
        if (st != RLE_OK) return st;
    }
    if (b->tuning.per_frame) {
        // one plain launch pair per frame, parameters by value from the
        // staging block; frame i goes to worker stream i % k, so up to k
        // frames are in flight and one frame's slowest rays overlap the next
        // frames' (each frame has its own rows of the ray buffer); the
        // workers fork from and join back onto the caller's stream
        const Layout& L = b->layout;
        auto* rp = reinterpret_cast<rle::RayParams*>(b->h_params[par] + L.ray_params);
        auto* sp = reinterpret_cast<rle::ResolveParams*>(b->h_params[par] + L.resolve_params);
        const int k = std::min(n, rle_batch::kWorkers);
        cudaError_t e = cudaEventRecord(b->fork, stream);
        for (int w = 0; w < k && e == cudaSuccess; w++) e = cudaStreamWaitEvent(b->workers[w], b->fork, 0);
        if (e != cudaSuccess) return cuda_fail(e, "rle_batch_render: fork to the worker streams");
        for (int i = 0; i < n && st == RLE_OK; i++) {
            rp[i].lanes_per_ray = b->tuning.lanes_per_ray;
            rp[i].threads_per_block = b->tuning.threads_per_block;
            rp[i].staging = b->tuning.staging;
            st = rle::launch_raycast(rp[i], b->workers[i % k]);
            if (st == RLE_OK) st = rle::launch_resolve(sp[i], b->workers[i % k]);
            if (st == RLE_OK && frame_done && cudaEventRecord(frame_done[i], b->workers[i % k]) != cudaSuccess)
                st = cuda_fail(cudaGetLastError(), "rle_batch_render: frame event");
        }
        // joined even after a failed launch: the caller's stream never runs
        // ahead of work already queued, and the next call waits for it below
        for (int w = 0; w < k; w++) {
            const cudaError_t ej = cudaEventRecord(b->joins[w], b->workers[w]);
            const cudaError_t ew = ej == cudaSuccess ? cudaStreamWaitEvent(stream, b->joins[w], 0) : ej;
            if (ew != cudaSuccess && st == RLE_OK) st = cuda_fail(ew, "rle_batch_render: join of the worker streams");
        }
    } else if (b->tuning.use_graph) {
        if (!b->graph[par]) {
            cudaGraph_t g = nullptr;
            cudaError_t e = cudaStreamBeginCapture(b->capture, cudaStreamCaptureModeThreadLocal);
            if (e != cudaSuccess) return cuda_fail(e, "cudaStreamBeginCapture");
            st = enqueue(b, par, b->capture);
            e = cudaStreamEndCapture(b->capture, &g);
            if (st != RLE_OK) {
                if (g) cudaGraphDestroy(g);
                return st;
            }
            if (e != cudaSuccess) return cuda_fail(e, "cudaStreamEndCapture");
            e = cudaGraphInstantiate(&b->graph[par], g, 0);
            cudaGraphDestroy(g);
            if (e != cudaSuccess) return cuda_fail(e, "cudaGraphInstantiate");
        }
        const cudaError_t e = cudaGraphLaunch(b->graph[par], stream);
        if (e != cudaSuccess) return cuda_fail(e, "cudaGraphLaunch");
    } else {
        st = enqueue(b, par, stream);
    }
    if (!b->tuning.per_frame && st == RLE_OK && frame_done) {
        for (int i = 0; i < n && st == RLE_OK; i++)
            if (cudaEventRecord(frame_done[i], stream) != cudaSuccess)
                st = cuda_fail(cudaGetLastError(), "rle_batch_render: frame event");
    }
    // recorded also after a failed launch, whose earlier launches may still
    // use the ray buffer: the next call's device work waits for them
    const cudaError_t e = cudaEventRecord(b->staged[par], stream);
    if (e != cudaSuccess) return st != RLE_OK ? st : cuda_fail(e, "cudaEventRecord");
    b->staged_used[par] = true;
    b->parity ^= 1;
    return st;
}

struct DeviceScope {
    int prev = -1;
    bool ok = true;
    explicit DeviceScope(int dev) {
        cudaGetDevice(&prev);
        if (prev != dev) ok = cudaSetDevice(dev) == cudaSuccess;
    }
    ~DeviceScope() {
        int cur = -1;
        cudaGetDevice(&cur);
        if (prev >= 0 && cur != prev) cudaSetDevice(prev);
    }
};

}  // namespace

extern "C" rle_status rle_batch_create(int device, int max_frames, size_t raybuf_words, int max_samples,
                                       int with_hits, rle_batch** out) {
    if (!out || max_frames < 1 || max_frames > 65536 || raybuf_words < 32 || max_samples < 8 ||
        max_samples > 16384) {
        rle::set_error("rle_batch_create: max_frames 1..65536, raybuf_words >= 32, max_samples 8..16384");
        return RLE_ERR_INVALID_ARG;
    }
    *out = nullptr;
    rle_batch* b = new (std::nothrow) rle_batch();
    if (!b) return RLE_ERR_NO_MEMORY;
    b->device = device;
    b->max_frames = max_frames;
    b->raybuf_words = raybuf_words;
    b->max_samples = max_samples;
    b->with_hits = with_hits != 0;
    b->layout = Layout(max_frames);
    DeviceScope ds(device);
    if (!ds.ok) {
        delete b;
        rle::set_error("rle_batch_create: cannot select device %d", device);
        return RLE_ERR_INVALID_ARG;
    }
    cudaError_t e = cudaSuccess;
    rle_status st = RLE_OK;
    if ((e = cudaMalloc(&b->d_raybuf, raybuf_words * 4)) != cudaSuccess) st = cuda_fail(e, "cudaMalloc(raybuf)");
    if (st == RLE_OK && (e = cudaMalloc(&b->d_raydepth, raybuf_words * 4)) != cudaSuccess)
        st = cuda_fail(e, "cudaMalloc(raydepth)");
    if (st == RLE_OK && b->with_hits && (e = cudaMalloc(&b->d_rayhit, raybuf_words * sizeof(rle_hit))) != cudaSuccess)
        st = cuda_fail(e, "cudaMalloc(rayhit)");
    if (st == RLE_OK && (e = cudaMalloc(&b->d_params, b->layout.total)) != cudaSuccess)
        st = cuda_fail(e, "cudaMalloc(params)");
    for (int i = 0; i < 2 && st == RLE_OK; i++) {
        if ((e = cudaHostAlloc(&b->h_params[i], b->layout.total, cudaHostAllocDefault)) != cudaSuccess)
            st = cuda_fail(e, "cudaHostAlloc(params)");
        else if ((e = cudaEventCreateWithFlags(&b->staged[i], cudaEventDisableTiming)) != cudaSuccess)
            st = cuda_fail(e, "cudaEventCreate");
        else
            std::memset(b->h_params[i], 0, b->layout.total);
    }
    if (st == RLE_OK && (e = cudaStreamCreateWithFlags(&b->capture, cudaStreamNonBlocking)) != cudaSuccess)
        st = cuda_fail(e, "cudaStreamCreate");
    if (st == RLE_OK && (e = cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming)) != cudaSuccess)
        st = cuda_fail(e, "cudaEventCreate");
    for (int w = 0; w < rle_batch::kWorkers && st == RLE_OK; w++) {
        if ((e = cudaStreamCreateWithFlags(&b->workers[w], cudaStreamNonBlocking)) != cudaSuccess)
            st = cuda_fail(e, "cudaStreamCreate");
        else if ((e = cudaEventCreateWithFlags(&b->joins[w], cudaEventDisableTiming)) != cudaSuccess)
            st = cuda_fail(e, "cudaEventCreate");
    }
    if (st != RLE_OK) {
        release(b);
        return st;
    }
    *out = b;
    return RLE_OK;
}

extern "C" rle_status rle_batch_free(rle_batch* b) {
    if (!b) return RLE_ERR_INVALID_ARG;
    release(b);
    return RLE_OK;
}

extern "C" rle_status rle_batch_set_tuning(rle_batch* b, const rle_batch_tuning* t) {
    if (!b || !t || !valid_tuning(*t)) {
        rle::set_error("rle_batch_set_tuning: tile 1..256, lanes 8/16/32, staging 1..3, threads 32..128 step 32");
        return RLE_ERR_INVALID_ARG;
    }
    std::lock_guard<std::mutex> lock(b->mu);
    DeviceScope ds(b->device);
    for (int i = 0; i < 2; i++)
        if (b->staged_used[i]) cudaEventSynchronize(b->staged[i]);
    drop_graphs(b);
    b->tuning = *t;
    b->raycast_blocks = 0;
    return RLE_OK;
}

extern "C" rle_status rle_batch_get_tuning(const rle_batch* b, rle_batch_tuning* t) {
    if (!b || !t) return RLE_ERR_INVALID_ARG;
    *t = b->tuning;
    return RLE_OK;
}

extern "C" size_t rle_batch_words_needed(const rle_frame_request* frames, int n) {
    if (!frames || n < 0) return 0;
    size_t words = 0;
    for (int i = 0; i < n; i++) {
        rle_raymap rm;
        if (rle_raymap_build(&frames[i].cam, &frames[i].view, &rm) != RLE_OK) return 0;
        words += align_up(static_cast<size_t>(rm.rays) * rm.samples, 32);
    }
    return words;
}

extern "C" rle_status rle_batch_render(rle_batch* b, const rle_scene* scene, const rle_frame_request* frames, int n,
                                       void* stream) {
    if (!b || !scene || (n > 0 && !frames) || n < 0 || n > b->max_frames) {
        rle::set_error("rle_batch_render: batch, scene and 0..max_frames frames required");
        return RLE_ERR_INVALID_ARG;
    }
    if (scene->device != b->device) {
        rle::set_error("rle_batch_render: scene on device %d, batch on device %d", scene->device, b->device);
        return RLE_ERR_INVALID_ARG;
    }
    if (n == 0) return RLE_OK;
    std::lock_guard<std::mutex> lock(b->mu);
    DeviceScope ds(b->device);
    return render_locked(b, scene, nullptr, frames, n, static_cast<cudaStream_t>(stream));
}

namespace rle {

rle_status batch_render_scenes(rle_batch* b, const rle_scene* const* scenes, const rle_frame_request* frames, int n,
                               void* stream, cudaEvent_t* frame_done) {
    if (!b || !scenes || (n > 0 && !frames) || n < 0 || n > b->max_frames) {
        set_error("rle_batch_render: batch, scenes and 0..max_frames frames required");
        return RLE_ERR_INVALID_ARG;
    }
    if (n == 0) return RLE_OK;
    std::lock_guard<std::mutex> lock(b->mu);
    DeviceScope ds(b->device);
    return render_locked(b, nullptr, scenes, frames, n, static_cast<cudaStream_t>(stream), frame_done);
}

size_t batch_capacity_words(const rle_batch* b) { return b ? b->raybuf_words : 0; }
int batch_max_frames(const rle_batch* b) { return b ? b->max_frames : 0; }

}  // namespace rle

extern "C" rle_status rle_batch_autotune(rle_batch* b, const rle_scene* scene, const rle_frame_request* frames,
                                         int n, int repeats, rle_batch_tuning* best, float* best_ms) {
    if (!b || !scene || !frames || n < 1 || repeats < 1) return RLE_ERR_INVALID_ARG;
    DeviceScope ds(b->device);
    cudaStream_t s = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    cudaError_t e = cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreate(&e0);
    if (e == cudaSuccess) e = cudaEventCreate(&e1);
    if (e != cudaSuccess) return cuda_fail(e, "rle_batch_autotune: set-up");
    const rle_batch_tuning start = b->tuning;
    rle_batch_tuning win = start;
    float win_ms = 1e30f;
    rle_status st = RLE_OK;
    const int lanes[] = {8, 16, 32}, stagings[] = {1, 2, 3};
    for (int lv : lanes) {
        // the persistent launch over tile x staging, then the per-frame launches (tile -1)
        for (int tv : {1, 2, 4, 8, 16, 32, 64, -1}) {
            for (int sv : stagings) {
                rle_batch_tuning t = start;
                t.per_frame = tv < 0 ? 1 : 0;
                t.tile_rays = tv < 0 ? start.tile_rays : tv;
                t.lanes_per_ray = lv;
                t.staging = sv;
                if ((st = rle_batch_set_tuning(b, &t)) != RLE_OK) break;
                if ((st = rle_batch_render(b, scene, frames, n, s)) != RLE_OK) break;  // warm-up / capture
                std::vector<float> ms;
                for (int r = 0; r < repeats && st == RLE_OK; r++) {
                    cudaEventRecord(e0, s);
                    st = rle_batch_render(b, scene, frames, n, s);
                    cudaEventRecord(e1, s);
                    cudaEventSynchronize(e1);
                    float v = 0;
                    cudaEventElapsedTime(&v, e0, e1);
                    ms.push_back(v);
                }
                if (st != RLE_OK) break;
                std::nth_element(ms.begin(), ms.begin() + ms.size() / 2, ms.end());
                const float med = ms[ms.size() / 2];
                if (med < win_ms) {
                    win_ms = med;
                    win = t;
                }
            }
            if (st != RLE_OK) break;
        }
        if (st != RLE_OK) break;
    }
    cudaStreamSynchronize(s);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaStreamDestroy(s);
    const rle_status st2 = rle_batch_set_tuning(b, st == RLE_OK ? &win : &start);
    if (st != RLE_OK) return st;
    if (best) *best = win;
    if (best_ms) *best_ms = win_ms;
    return st2;
}
