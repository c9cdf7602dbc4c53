// Render server: resident scenes, a host request queue and a scheduler
// thread doing continuous batching.
//
// The scheduler keeps up to max_inflight batch slots busy.  Whenever a slot
// is free it takes queued requests in arrival order, as many as fit the
// slot's frame count and ray-buffer words, and launches them as one batch
// (rle_batch) on the slot's stream.  Each request completes when its own
// frame's event does (in the batch's default per-frame mode a frame is done
// behind its own two launches, before the rest of its batch), and the slot
// is free again once the whole batch is; both are observed by polling
// events, so no host thread blocks on the device.  Requests that arrive while batches run
// simply wait for the next free slot, and batches in different slots overlap
// on the device.  In `plain` mode each request is its own launch
// (rle_render_frame) and runs alone, the baseline the batching is measured
// against.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <mutex>
#include <new>
#include <thread>
#include <unordered_map>
#include <vector>

#include "rle_internal.h"

namespace {

double now_s() {
    using clk = std::chrono::steady_clock;
    return std::chrono::duration<double>(clk::now().time_since_epoch()).count();
}

enum ReqState { kQueued = 0, kRunning = 1, kDone = 2 };

struct Req {
    rle_request r;
    uint64_t ticket = 0;
    size_t words = 0;
    double pixels = 0;
    double submit_s = 0, launch_s = 0, done_s = 0;
    double gpu_ms = 0;  // device time from its batch's start to the end of its frame (events)
    rle_status status = RLE_OK;
    int state = kQueued;
};

struct Slot {
    rle_batch* batch = nullptr;
    cudaStream_t stream = nullptr;
    cudaEvent_t start = nullptr;  // recorded before a batch's launches
    cudaEvent_t done = nullptr;   // and after them
    std::vector<cudaEvent_t> frame_done;  // per frame of the batch (batched mode)
    std::vector<char> finished;           // per ticket: its completion is out
    bool busy = false;
    std::vector<uint64_t> tickets;
    void* workspace = nullptr;  // plain mode
    size_t workspace_bytes = 0;
};

}  // namespace

struct rle_server {
    rle_server_config cfg{};
    std::vector<const rle_scene*> scenes;
    uint64_t scene_bytes = 0, buffer_bytes = 0;
    std::vector<Slot> slots;

    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::deque<uint64_t> queue;
    std::unordered_map<uint64_t, Req> reqs;
    std::deque<rle_completion> completions;
    uint64_t next_ticket = 1;
    int inject = 0;
    bool paused = false;
    bool stop = false;
    std::thread worker;

    // statistics
    std::vector<double> lat_ms;
    uint64_t submitted = 0, completed = 0, failed = 0, cancelled = 0, batches = 0;
    double pixels = 0, first_submit = -1, last_done = 0;
};

namespace {

void finish(rle_server* s, Req& q, rle_status st, double t) {
    q.state = kDone;
    q.status = st;
    q.done_s = t;
    rle_completion c;
    c.ticket = q.ticket;
    c.status = st;
    c.submit_s = q.submit_s;
    c.launch_s = q.launch_s;
    c.done_s = t;
    c.gpu_ms = q.gpu_ms;
    s->completions.push_back(c);
    if (st == RLE_OK) {
        s->completed++;
        s->lat_ms.push_back((t - q.submit_s) * 1e3);
        s->pixels += q.pixels;
        s->last_done = std::max(s->last_done, t);
    } else if (st == RLE_ERR_CANCELLED) {
        s->cancelled++;
    } else {
        s->failed++;
    }
}

// Completes one request of a slot (lock held).
void finish_ticket(rle_server* s, Slot& sl, size_t i, cudaEvent_t end, cudaError_t e, double t) {
    sl.finished[i] = 1;
    auto it = s->reqs.find(sl.tickets[i]);
    if (it == s->reqs.end()) return;
    if (e != cudaSuccess) rle::set_error("server: batch failed on the device: %s", cudaGetErrorString(e));
    float gpu_ms = 0;
    if (e == cudaSuccess && cudaEventElapsedTime(&gpu_ms, sl.start, end) != cudaSuccess) gpu_ms = 0;
    it->second.gpu_ms = gpu_ms;
    finish(s, it->second, e == cudaSuccess ? RLE_OK : RLE_ERR_CUDA, t);
}

// Marks done the requests whose frames are finished, and frees the slots
// whose batches are.  Called with the lock held.  A slot's frames finish
// roughly in order (frame i runs on the batch's worker stream i mod 8), so
// the scan of a slot stops after eight frames that are not ready yet.
bool retire(rle_server* s) {
    bool any = false;
    for (Slot& sl : s->slots) {
        if (!sl.busy) continue;
        if (!sl.frame_done.empty()) {
            int pending = 0;
            for (size_t i = 0; i < sl.tickets.size() && pending < 8; i++) {
                if (sl.finished[i]) continue;
                const cudaError_t e = cudaEventQuery(sl.frame_done[i]);
                if (e == cudaErrorNotReady) {
                    pending++;
                    continue;
                }
                finish_ticket(s, sl, i, sl.frame_done[i], e, now_s());
                any = true;
            }
        }
        const cudaError_t e = cudaEventQuery(sl.done);
        if (e == cudaErrorNotReady) continue;
        const double t = now_s();
        for (size_t i = 0; i < sl.tickets.size(); i++)
            if (!sl.finished[i]) finish_ticket(s, sl, i, sl.done, e, t);
        sl.tickets.clear();
        sl.finished.clear();
        sl.busy = false;
        any = true;
    }
    return any;
}

// Launches the queue head on a free slot.  Called with the lock held; drops
// it around the host-side launch work.
bool launch_one(rle_server* s, std::unique_lock<std::mutex>& lk) {
    if (s->paused && !s->stop) return false;
    Slot* slot = nullptr;
    for (Slot& sl : s->slots)
        if (!sl.busy) {
            slot = &sl;
            break;
        }
    if (!slot) return false;
    // requests for this launch, in arrival order
    std::vector<uint64_t> take;
    size_t words = 0;
    const size_t cap = s->cfg.plain ? SIZE_MAX : rle::batch_capacity_words(slot->batch);
    const size_t max_frames = s->cfg.plain ? 1 : static_cast<size_t>(s->cfg.max_frames_per_batch);
    while (!s->queue.empty() && take.size() < max_frames) {
        const uint64_t tk = s->queue.front();
        auto it = s->reqs.find(tk);
        if (it == s->reqs.end() || it->second.state != kQueued) {
            s->queue.pop_front();
            continue;
        }
        if (!take.empty() && words + it->second.words > cap) break;
        words += it->second.words;
        take.push_back(tk);
        s->queue.pop_front();
    }
    if (take.empty()) return false;
    const double t = now_s();
    std::vector<rle_frame_request> frames(take.size());
    std::vector<const rle_scene*> scenes(take.size());
    std::vector<double> px(take.size());
    for (size_t i = 0; i < take.size(); i++) {
        Req& q = s->reqs[take[i]];
        q.state = kRunning;
        q.launch_s = t;
        frames[i].cam = q.r.cam;
        frames[i].view = q.r.view;
        frames[i].d_colour = q.r.d_colour;
        frames[i].d_depth = q.r.d_depth;
        frames[i].d_hit = nullptr;
        scenes[i] = s->scenes[q.r.scene_id];
    }
    const bool inject = s->inject > 0;
    if (inject) s->inject--;
    slot->busy = true;  // reserve the slot while the lock is dropped
    slot->tickets = take;
    slot->finished.assign(take.size(), 0);
    s->batches++;
    lk.unlock();
    rle_status st = RLE_OK;
    if (!inject && cudaEventRecord(slot->start, slot->stream) != cudaSuccess) st = RLE_ERR_CUDA;
    if (st != RLE_OK) {
        rle::set_error("server: cudaEventRecord failed");
    } else if (inject) {
        rle::set_error("server: injected launch failure");
        st = RLE_ERR_CUDA;
    } else if (s->cfg.plain) {
        st = rle_render_frame(scenes[0], &frames[0].cam, &frames[0].view, slot->workspace, slot->workspace_bytes,
                              frames[0].d_colour, frames[0].d_depth, nullptr, slot->stream);
    } else {
        st = rle::batch_render_scenes(slot->batch, scenes.data(), frames.data(), static_cast<int>(frames.size()),
                                      slot->stream, slot->frame_done.data());
    }
    if (st == RLE_OK && cudaEventRecord(slot->done, slot->stream) != cudaSuccess) st = RLE_ERR_CUDA;
    lk.lock();
    if (st != RLE_OK) {
        const double tf = now_s();
        for (uint64_t tk : slot->tickets) finish(s, s->reqs[tk], st, tf);
        slot->tickets.clear();
        slot->finished.clear();
        slot->busy = false;
        s->cv_done.notify_all();
    }
    return true;
}

void run(rle_server* s) {
    cudaSetDevice(s->cfg.device);
    std::unique_lock<std::mutex> lk(s->mu);
    for (;;) {
        bool progress = retire(s);
        while (launch_one(s, lk)) progress = true;
        if (progress) s->cv_done.notify_all();
        bool busy = false;
        for (const Slot& sl : s->slots) busy = busy || sl.busy;
        if (s->stop && !busy && s->queue.empty()) break;
        if (!busy && (s->queue.empty() || (s->paused && !s->stop)))
            s->cv_work.wait(lk, [s] { return s->stop || (!s->queue.empty() && !s->paused); });
        else if (!progress)
            s->cv_work.wait_for(lk, std::chrono::microseconds(20));
    }
}

void release(rle_server* s) {
    if (!s) return;
    if (s->worker.joinable()) {
        {
            std::lock_guard<std::mutex> lk(s->mu);
            s->stop = true;
            for (uint64_t tk : s->queue) {
                auto it = s->reqs.find(tk);
                if (it != s->reqs.end() && it->second.state == kQueued) finish(s, it->second, RLE_ERR_CANCELLED, now_s());
            }
            s->queue.clear();
        }
        s->cv_work.notify_all();
        s->worker.join();
    }
    int prev = -1;
    cudaGetDevice(&prev);
    cudaSetDevice(s->cfg.device);
    for (Slot& sl : s->slots) {
        if (sl.stream) cudaStreamSynchronize(sl.stream);
        if (sl.batch) rle_batch_free(sl.batch);
        if (sl.done) cudaEventDestroy(sl.done);
        for (cudaEvent_t ev : sl.frame_done) cudaEventDestroy(ev);
        if (sl.start) cudaEventDestroy(sl.start);
        if (sl.stream) cudaStreamDestroy(sl.stream);
        if (sl.workspace) cudaFree(sl.workspace);
    }
    if (prev >= 0) cudaSetDevice(prev);
    delete s;
}

}  // namespace

extern "C" rle_status rle_server_create(const rle_server_config* cfg, rle_server** out) {
    if (!cfg || !out || cfg->max_inflight < 1 || cfg->max_inflight > 16 || cfg->max_frames_per_batch < 1 ||
        cfg->raybuf_words < 32 || cfg->max_samples < 8 || cfg->max_samples > 16384) {
        rle::set_error("rle_server_create: max_inflight 1..16, max_frames_per_batch >= 1, raybuf_words >= 32, "
                       "max_samples 8..16384");
        return RLE_ERR_INVALID_ARG;
    }
    *out = nullptr;
    rle_server* s = new (std::nothrow) rle_server();
    if (!s) return RLE_ERR_NO_MEMORY;
    s->cfg = *cfg;
    if (cfg->plain) s->cfg.max_inflight = 1;
    int prev = -1;
    cudaGetDevice(&prev);
    if (cudaSetDevice(cfg->device) != cudaSuccess) {
        delete s;
        rle::set_error("rle_server_create: cannot select device %d", cfg->device);
        return RLE_ERR_INVALID_ARG;
    }
    // device memory this server holds besides scenes
    size_t per_slot;
    size_t plain_ws = 0;
    if (cfg->plain) {
        rle_view_params v = {cfg->max_samples, 8, cfg->max_samples, cfg->max_samples, 0.0f, 0, 0};
        plain_ws = rle_frame_workspace_bytes(&v);
        per_slot = plain_ws;
    } else {
        per_slot = cfg->raybuf_words * 8 + 65536;
    }
    s->buffer_bytes = per_slot * static_cast<size_t>(s->cfg.max_inflight);
    rle_status st = RLE_OK;
    if (s->buffer_bytes > cfg->hbm_budget_bytes) {
        rle::set_error("rle_server_create: %zu bytes of ray buffers exceed the %zu-byte budget",
                       static_cast<size_t>(s->buffer_bytes), cfg->hbm_budget_bytes);
        st = RLE_ERR_NO_MEMORY;
    }
    s->slots.resize(s->cfg.max_inflight);
    for (Slot& sl : s->slots) {
        if (st != RLE_OK) break;
        if (cudaStreamCreateWithFlags(&sl.stream, cudaStreamNonBlocking) != cudaSuccess ||
            cudaEventCreate(&sl.start) != cudaSuccess || cudaEventCreate(&sl.done) != cudaSuccess) {
            st = RLE_ERR_CUDA;
            break;
        }
        if (cfg->plain) {
            if (cudaMalloc(&sl.workspace, plain_ws) != cudaSuccess) st = RLE_ERR_NO_MEMORY;
            sl.workspace_bytes = plain_ws;
        } else {
            st = rle_batch_create(cfg->device, cfg->max_frames_per_batch, cfg->raybuf_words, cfg->max_samples, 0,
                                  &sl.batch);
            if (st == RLE_OK && cfg->batch_tuning.lanes_per_ray != 0)
                st = rle_batch_set_tuning(sl.batch, &cfg->batch_tuning);
            for (int i = 0; i < cfg->max_frames_per_batch && st == RLE_OK; i++) {
                cudaEvent_t ev = nullptr;
                if (cudaEventCreate(&ev) != cudaSuccess) {
                    rle::set_error("rle_server_create: cudaEventCreate failed for the per-frame events");
                    st = RLE_ERR_CUDA;
                } else {
                    sl.frame_done.push_back(ev);
                }
            }
        }
    }
    if (prev >= 0) cudaSetDevice(prev);
    if (st != RLE_OK) {
        release(s);
        return st;
    }
    s->worker = std::thread(run, s);
    *out = s;
    return RLE_OK;
}

extern "C" rle_status rle_server_add_scene(rle_server* s, const rle_scene* scene, int* scene_id) {
    if (!s || !scene || !scene_id) return RLE_ERR_INVALID_ARG;
    std::lock_guard<std::mutex> lk(s->mu);
    if (scene->device != s->cfg.device) {
        rle::set_error("rle_server_add_scene: scene on device %d, server on device %d", scene->device,
                       s->cfg.device);
        return RLE_ERR_INVALID_ARG;
    }
    if (s->scene_bytes + scene->device_bytes + s->buffer_bytes > s->cfg.hbm_budget_bytes) {
        rle::set_error("rle_server_add_scene: scene of %llu bytes exceeds the HBM budget",
                       static_cast<unsigned long long>(scene->device_bytes));
        return RLE_ERR_NO_MEMORY;
    }
    s->scene_bytes += scene->device_bytes;
    s->scenes.push_back(scene);
    *scene_id = static_cast<int>(s->scenes.size()) - 1;
    return RLE_OK;
}

extern "C" rle_status rle_server_submit(rle_server* s, const rle_request* r, uint64_t* ticket) {
    if (!s || !r || !ticket || !r->d_colour || !r->d_depth) return RLE_ERR_INVALID_ARG;
    rle_raymap rm;
    rle_status st = rle_raymap_build(&r->cam, &r->view, &rm);
    if (st != RLE_OK) return st;
    Req q;
    q.r = *r;
    q.words = (static_cast<size_t>(rm.rays) * rm.samples + 31) / 32 * 32;
    q.pixels = static_cast<double>(rm.width) * rm.height;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        if (r->scene_id < 0 || r->scene_id >= static_cast<int>(s->scenes.size())) {
            rle::set_error("rle_server_submit: unknown scene id %d", r->scene_id);
            return RLE_ERR_INVALID_ARG;
        }
        if (rm.samples > s->cfg.max_samples ||
            (!s->cfg.plain && q.words > rle::batch_capacity_words(s->slots[0].batch))) {
            rle::set_error("rle_server_submit: request needs %zu ray-buffer words / %d samples; a slot holds %zu / %d",
                           q.words, rm.samples, s->cfg.plain ? 0 : rle::batch_capacity_words(s->slots[0].batch),
                           s->cfg.max_samples);
            return RLE_ERR_CAPACITY;
        }
        if (s->stop) return RLE_ERR_CANCELLED;
        q.ticket = s->next_ticket++;
        q.submit_s = now_s();
        if (s->first_submit < 0) s->first_submit = q.submit_s;
        s->submitted++;
        *ticket = q.ticket;
        s->reqs.emplace(q.ticket, q);
        s->queue.push_back(q.ticket);
    }
    s->cv_work.notify_one();
    return RLE_OK;
}

extern "C" rle_status rle_server_cancel(rle_server* s, uint64_t ticket) {
    if (!s) return RLE_ERR_INVALID_ARG;
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->reqs.find(ticket);
    if (it == s->reqs.end() || it->second.state != kQueued) return RLE_ERR_INVALID_ARG;
    finish(s, it->second, RLE_ERR_CANCELLED, now_s());
    s->cv_done.notify_all();
    return RLE_OK;
}

extern "C" rle_status rle_server_wait(rle_server* s, uint64_t ticket, int timeout_ms, rle_completion* out) {
    if (!s) return RLE_ERR_INVALID_ARG;
    std::unique_lock<std::mutex> lk(s->mu);
    auto done = [&] {
        auto it = s->reqs.find(ticket);
        return it == s->reqs.end() || it->second.state == kDone;
    };
    if (!s->cv_done.wait_for(lk, std::chrono::milliseconds(timeout_ms < 0 ? 0 : timeout_ms), done))
        return RLE_ERR_TIMEOUT;
    auto it = s->reqs.find(ticket);
    if (it == s->reqs.end()) return RLE_ERR_INVALID_ARG;
    if (out) {
        out->ticket = ticket;
        out->status = it->second.status;
        out->submit_s = it->second.submit_s;
        out->launch_s = it->second.launch_s;
        out->done_s = it->second.done_s;
        out->gpu_ms = it->second.gpu_ms;
    }
    return RLE_OK;
}

extern "C" rle_status rle_server_drain(rle_server* s, int timeout_ms) {
    if (!s) return RLE_ERR_INVALID_ARG;
    std::unique_lock<std::mutex> lk(s->mu);
    auto idle = [&] {
        if (!s->queue.empty()) return false;
        for (const Slot& sl : s->slots)
            if (sl.busy) return false;
        return true;
    };
    if (!s->cv_done.wait_for(lk, std::chrono::milliseconds(timeout_ms < 0 ? 0 : timeout_ms), idle))
        return RLE_ERR_TIMEOUT;
    return RLE_OK;
}

extern "C" rle_status rle_server_poll(rle_server* s, rle_completion* out, int max, int* n) {
    if (!s || !n || (max > 0 && !out)) return RLE_ERR_INVALID_ARG;
    std::lock_guard<std::mutex> lk(s->mu);
    int k = 0;
    while (k < max && !s->completions.empty()) {
        out[k++] = s->completions.front();
        s->reqs.erase(s->completions.front().ticket);
        s->completions.pop_front();
    }
    *n = k;
    return RLE_OK;
}

extern "C" rle_status rle_server_get_stats(rle_server* s, rle_server_stats* out) {
    if (!s || !out) return RLE_ERR_INVALID_ARG;
    std::lock_guard<std::mutex> lk(s->mu);
    *out = rle_server_stats{};
    out->submitted = s->submitted;
    out->completed = s->completed;
    out->failed = s->failed;
    out->cancelled = s->cancelled;
    out->batches = s->batches;
    out->pixels = s->pixels;
    out->device_bytes = s->scene_bytes + s->buffer_bytes;
    if (!s->lat_ms.empty()) {
        std::vector<double> v = s->lat_ms;
        std::sort(v.begin(), v.end());
        auto pct = [&](double p) { return v[std::min(v.size() - 1, static_cast<size_t>(p * (v.size() - 1) + 0.5))]; };
        out->p50_ms = pct(0.50);
        out->p99_ms = pct(0.99);
        out->max_ms = v.back();
        double sum = 0;
        for (double x : v) sum += x;
        out->mean_ms = sum / static_cast<double>(v.size());
    }
    if (s->first_submit >= 0 && s->last_done > s->first_submit) {
        out->busy_s = s->last_done - s->first_submit;
        out->mrays_per_s = s->pixels / out->busy_s / 1e6;
    }
    return RLE_OK;
}

extern "C" rle_status rle_server_reset_stats(rle_server* s) {
    if (!s) return RLE_ERR_INVALID_ARG;
    std::lock_guard<std::mutex> lk(s->mu);
    s->lat_ms.clear();
    s->submitted = s->completed = s->failed = s->cancelled = s->batches = 0;
    s->pixels = 0;
    s->first_submit = -1;
    s->last_done = 0;
    return RLE_OK;
}

extern "C" rle_status rle_server_inject_launch_failures(rle_server* s, int count) {
    if (!s || count < 0) return RLE_ERR_INVALID_ARG;
    std::lock_guard<std::mutex> lk(s->mu);
    s->inject = count;
    return RLE_OK;
}

extern "C" rle_status rle_server_pause(rle_server* s, int paused) {
    if (!s) return RLE_ERR_INVALID_ARG;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->paused = paused != 0;
    }
    s->cv_work.notify_all();
    return RLE_OK;
}

extern "C" rle_status rle_server_destroy(rle_server* s) {
    if (!s) return RLE_ERR_INVALID_ARG;
    release(s);
    return RLE_OK;
}
