// Serving loop: a persistent scheduler thread that admits interactive render requests of
// different scenes and resolutions onto the GPU as slots and memory free up (continuous
// batching), keeps the scenes' BVHs resident, and records each request's queueing, rendering and
// total latency.
//
// Scenes are agb_contexts uploaded by the caller and registered with their HBM footprint; the
// server refuses scenes beyond its HBM budget.  Admitted requests are merged into batches: every
// batch is one agb_batch_render, a wavefront whose every stage is a single kernel launch over the
// paths of all of its requests, whatever their scenes and resolutions.  Two batches are in flight
// at once, so requests that arrive while one renders form the next, which starts at once and
// overlaps it on the device.  Each request keeps its own render state in a view of its scene
// (agb_view_create: frame, accumulation, AOVs), pooled per scene and reused; idle views are
// destroyed when a new request needs their memory.  A request's render state is reserved against
// the budget before it is admitted; requests are admitted in arrival order.  A batch the batched
// renderer refuses (a scene with a ground plane) renders request by request on the views' own
// streams instead.
//
// Threads: the scheduler thread is the only one that calls the render entry points on views;
// callers submit and wait from any thread.  Scenes must not change while the server runs.
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include <cuda_runtime.h>

#include "agb.h"

namespace
{

using Clock = std::chrono::steady_clock;

double msSince(Clock::time_point t0, Clock::time_point t1)
{
    return std::chrono::duration<double, std::milli>(t1 - t0).count();
}

// Paths in flight per request wave of a request rendered alone; bounds its wave buffers
// (agb_bytes_per_path each).
constexpr uint64_t kServeWavePaths = 1u << 21;
// Paths in flight per batch wave (each of the two batches holds wave buffers for this many): a
// quarter of the HBM budget over the two batches, between 4096 and 2^24 paths.
constexpr uint64_t kBatchWavePathsMax = 1u << 24;
constexpr uint64_t kBatchWavePathsMin = 4096;
constexpr int kBatches                = 2;
// Per pixel: running mean, Kahan sum and compensation, last sample (16 B each), moments (8 B),
// AOVs (52 B), temporal history (32 B).
constexpr uint64_t kBytesPerPixel = 4 * 16 + 8 + 52 + 32;

struct Request
{
    uint64_t id = 0;
    agb_serve_request req{};
    Clock::time_point tSubmit, tStart, tDone;
    uint64_t reserved   = 0;
    agb_context* view   = nullptr;
    bool finished       = false;
    agb_status status   = AGB_OK;
    std::string error;
    std::vector<float> rgba;
};

struct Scene
{
    agb_context* ctx = nullptr;
    uint64_t bytes   = 0;
    std::vector<agb_context*> idle;
};

// A request's own render state (its batch's wave buffers are reserved with the batch).
uint64_t estimateBytes(const agb_serve_request& r)
{
    uint64_t pixels = uint64_t(r.width) * r.height;
    return pixels * kBytesPerPixel + (1u << 20);
}

struct Batch
{
    agb_batch* handle = nullptr;
    std::vector<Request*> requests;
    bool busy = false;
};

} // namespace

struct agb_server
{
    int device       = 0;
    uint64_t budget  = 0;
    int maxSlots     = 1;
    agb_denoiser* denoiser = nullptr;

    std::mutex mu;
    std::condition_variable wake, doneCv;
    std::map<int32_t, Scene> scenes;
    std::deque<Request*> queue;
    std::vector<Request*> running; // rendered alone on their views' streams
    Batch batches[kBatches];
    uint64_t batchBytes = 0;       // wave buffers of the batches
    std::map<uint64_t, std::unique_ptr<Request>> all;
    uint64_t nextId     = 1;
    uint64_t sceneBytes = 0, reserved = 0, pooled = 0;
    bool stop           = false;
    std::thread worker;
    // Denoiser buffers (device), grown on demand by the scheduler thread.
    uint16_t* features = nullptr;
    float* denoised    = nullptr;
    uint64_t denoiseCapacity = 0;

    void run();
    bool admit(Request* r, std::unique_lock<std::mutex>& lk);
    agb_status renderAlone(Request* r);
    void launch(Batch& b);
    void finish(Request* r);
    void release(Request* r);
    void failRequest(Request* r, agb_status st, const std::string& msg);
    void evictIdle(uint64_t need);
};

void agb_server::failRequest(Request* r, agb_status st, const std::string& msg)
{
    r->status   = st;
    r->error    = msg;
    r->finished = true;
    r->tDone    = Clock::now();
    doneCv.notify_all();
}

void agb_server::evictIdle(uint64_t need)
{
    for (auto& kv : scenes)
    {
        Scene& sc = kv.second;
        while (!sc.idle.empty() && sceneBytes + batchBytes + reserved + pooled + need > budget)
        {
            agb_context* v = sc.idle.back();
            sc.idle.pop_back();
            uint64_t b = 0;
            agb_context_memory(v, &b);
            agb_context_destroy(v);
            pooled -= std::min(pooled, b);
        }
    }
}

// Reserves a request's memory and gives it a view with its frame set (lock held).  Returns false
// when it must wait for memory.
bool agb_server::admit(Request* r, std::unique_lock<std::mutex>&)
{
    auto it = scenes.find(r->req.scene);
    if (it == scenes.end())
    {
        failRequest(r, AGB_ERR_INVALID_ARG, "unknown scene");
        return true;
    }
    Scene& sc     = it->second;
    uint64_t need = estimateBytes(r->req);
    agb_context* view = nullptr;
    uint64_t viewBytes = 0;
    if (!sc.idle.empty())
    {
        view = sc.idle.back();
        agb_context_memory(view, &viewBytes);
    }
    // A pooled view's memory is already counted; reserve only what it may still need to grow.
    uint64_t extra = need > viewBytes ? need - viewBytes : 0;
    if (sceneBytes + batchBytes + reserved + pooled + extra > budget)
        evictIdle(extra);
    if (sceneBytes + batchBytes + reserved + pooled + extra > budget)
    {
        bool idle = running.empty();
        for (const Batch& b : batches)
            idle = idle && !b.busy;
        if (idle)
        {
            failRequest(r, AGB_ERR_OOM, "request does not fit the HBM budget");
            return true;
        }
        return false;
    }
    if (view)
    {
        sc.idle.pop_back();
        pooled -= std::min(pooled, viewBytes);
    }
    else if (agb_view_create(sc.ctx, nullptr, &view) != AGB_OK)
    {
        failRequest(r, AGB_ERR_CUDA, agb_last_error());
        return true;
    }
    r->view     = view;
    r->reserved = std::max(need, viewBytes);
    reserved += r->reserved;
    r->tStart = Clock::now();
    agb_frame_data f = r->req.frame;
    if ((r->req.flags & AGB_SERVE_DENOISE) && denoiser)
        f.is_denoising_aovs_enabled = 1;
    agb_status st = agb_frame_set(view, &f);
    if (st)
    {
        std::string msg = agb_last_error();
        release(r);
        failRequest(r, st, msg);
    }
    return true;
}

agb_render_options requestOptions(const Request* r, bool denoise)
{
    agb_render_options opt{};
    opt.width               = r->req.width;
    opt.height              = r->req.height;
    opt.accumulation        = AGB_ACCUM_RUNNING_MEAN | (denoise ? AGB_ACCUM_MOMENTS : 0u);
    opt.max_paths_in_flight = uint32_t(kServeWavePaths);
    opt.seed_offset         = r->req.seed_offset;
    return opt;
}

// Renders a request on its view's own stream (requests of scenes the batched renderer refuses).
agb_status agb_server::renderAlone(Request* r)
{
    bool denoise = (r->req.flags & AGB_SERVE_DENOISE) && denoiser;
    agb_render_options opt = requestOptions(r, denoise);
    return agb_render(r->view, &opt, 0, r->req.spp, nullptr);
}

// Starts a batch over its admitted requests (lock held).
void agb_server::launch(Batch& b)
{
    std::vector<agb_context*> views;
    std::vector<agb_render_options> opts;
    std::vector<uint32_t> counts;
    for (Request* r : b.requests)
    {
        views.push_back(r->view);
        opts.push_back(requestOptions(r, (r->req.flags & AGB_SERVE_DENOISE) && denoiser));
        counts.push_back(r->req.spp);
    }
    agb_status st = agb_batch_render(b.handle, views.data(), opts.data(), nullptr, counts.data(),
        uint32_t(views.size()), nullptr);
    if (st == AGB_OK)
    {
        b.busy = true;
        return;
    }
    // Not batchable: each request renders alone.
    for (Request* r : b.requests)
    {
        st = renderAlone(r);
        if (st)
        {
            std::string msg = agb_last_error();
            release(r);
            failRequest(r, st, msg);
        }
        else
            running.push_back(r);
    }
    b.requests.clear();
}

// Returns a request's view to its scene's pool and its reservation to the budget.
void agb_server::release(Request* r)
{
    if (!r->view)
        return;
    Scene& sc = scenes[r->req.scene];
    reserved -= std::min(reserved, r->reserved);
    uint64_t b = 0;
    agb_context_memory(r->view, &b);
    pooled += b;
    sc.idle.push_back(r->view);
    r->view = nullptr;
}

void agb_server::finish(Request* r)
{
    uint64_t pixels = uint64_t(r->req.width) * r->req.height;
    r->rgba.resize(pixels * 4);
    agb_status st = AGB_OK;
    bool denoise  = (r->req.flags & AGB_SERVE_DENOISE) && denoiser;
    if (denoise)
    {
        if (denoiseCapacity < pixels)
        {
            cudaFree(features);
            cudaFree(denoised);
            features = nullptr;
            denoised = nullptr;
            denoiseCapacity = 0;
            if (cudaMalloc(&features, pixels * 16 * 2) == cudaSuccess &&
                cudaMalloc(&denoised, pixels * 16) == cudaSuccess)
                denoiseCapacity = pixels;
        }
        st = denoiseCapacity >= pixels ? agb_denoiser_features(r->view, features) : AGB_ERR_OOM;
        if (!st)
            st = agb_denoiser_forward(denoiser, features, 1, int32_t(r->req.height), int32_t(r->req.width), denoised);
        if (!st && cudaMemcpy(r->rgba.data(), denoised, pixels * 16, cudaMemcpyDeviceToHost) != cudaSuccess)
            st = AGB_ERR_CUDA;
    }
    else
        st = agb_accum_read(r->view, AGB_ACCUM_RUNNING_MEAN, r->rgba.data(), pixels * 4);
    r->status = st;
    if (st)
        r->error = agb_last_error();
    r->tDone = Clock::now();
    release(r);
    r->finished = true;
    doneCv.notify_all();
}

void agb_server::run()
{
    cudaSetDevice(device);
    std::unique_lock<std::mutex> lk(mu);
    for (;;)
    {
        bool busy = !running.empty();
        for (const Batch& b : batches)
            busy = busy || b.busy;
        if (stop && queue.empty() && !busy)
            break;
        // Completions: a batch is done when its wavefront has drained; a request rendered alone
        // when its view's work has.
        for (Batch& b : batches)
            if (b.busy && agb_batch_poll(b.handle) != AGB_ERR_NOT_READY)
            {
                for (Request* r : b.requests)
                    finish(r);
                b.requests.clear();
                b.busy = false;
            }
        for (size_t i = 0; i < running.size();)
        {
            Request* r = running[i];
            if (agb_wait_poll(r->view) == AGB_OK)
            {
                running.erase(running.begin() + long(i));
                finish(r);
            }
            else
                i++;
        }
        // Admissions in arrival order into a free batch while slots are free; the batch starts
        // at once with what has arrived (continuous batching).
        int inFlight = int(running.size());
        for (const Batch& b : batches)
            inFlight += int(b.requests.size());
        for (Batch& b : batches)
        {
            if (b.busy || queue.empty() || inFlight >= maxSlots)
                continue;
            while (!queue.empty() && inFlight < maxSlots)
            {
                Request* r = queue.front();
                if (!admit(r, lk))
                    break;
                queue.pop_front();
                if (r->view)
                {
                    b.requests.push_back(r);
                    inFlight++;
                }
            }
            if (!b.requests.empty())
                launch(b);
        }
        busy = !running.empty();
        for (const Batch& b : batches)
            busy = busy || b.busy;
        if (!busy && queue.empty())
        {
            wake.wait(lk);
            continue;
        }
        lk.unlock();
        std::this_thread::sleep_for(std::chrono::microseconds(50));
        lk.lock();
    }
}

AGB_API agb_status agb_server_create(int32_t device, uint64_t hbm_budget_bytes, int32_t max_slots,
    agb_server** out)
{
    if (!out || max_slots <= 0 || max_slots > 64 || hbm_budget_bytes == 0)
        return AGB_ERR_INVALID_ARG;
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || device < 0 || device >= count)
        return AGB_ERR_INVALID_ARG;
    std::unique_ptr<agb_server> s(new agb_server());
    s->device   = device;
    s->budget   = hbm_budget_bytes;
    s->maxSlots = max_slots;
    // The batches' wave buffers are reserved up front.
    uint64_t batchPaths = hbm_budget_bytes / 4 / (uint64_t(kBatches) * agb_bytes_per_path());
    batchPaths          = std::min(kBatchWavePathsMax, std::max(kBatchWavePathsMin, batchPaths));
    s->batchBytes       = uint64_t(kBatches) * batchPaths * agb_bytes_per_path();
    if (s->batchBytes > hbm_budget_bytes / 2)
        return AGB_ERR_INVALID_ARG;
    for (Batch& b : s->batches)
        if (agb_batch_create(device, nullptr, batchPaths, &b.handle) != AGB_OK)
        {
            for (Batch& c : s->batches)
                agb_batch_destroy(c.handle);
            return AGB_ERR_CUDA;
        }
    agb_server* p = s.get();
    s->worker     = std::thread([p] { p->run(); });
    *out          = s.release();
    return AGB_OK;
}

AGB_API agb_status agb_server_destroy(agb_server* srv)
{
    if (!srv)
        return AGB_OK;
    {
        std::lock_guard<std::mutex> g(srv->mu);
        srv->stop = true;
    }
    srv->wake.notify_all();
    srv->worker.join();
    cudaSetDevice(srv->device);
    for (Batch& b : srv->batches)
        agb_batch_destroy(b.handle);
    for (auto& kv : srv->scenes)
        for (agb_context* v : kv.second.idle)
            agb_context_destroy(v);
    cudaFree(srv->features);
    cudaFree(srv->denoised);
    delete srv;
    return AGB_OK;
}

AGB_API agb_status agb_server_add_scene(agb_server* srv, int32_t scene_id, agb_context* ctx)
{
    if (!srv || !ctx)
        return AGB_ERR_INVALID_ARG;
    uint64_t bytes = 0;
    agb_status st  = agb_context_memory(ctx, &bytes);
    if (st)
        return st;
    std::lock_guard<std::mutex> g(srv->mu);
    if (srv->scenes.count(scene_id))
        return AGB_ERR_INVALID_ARG;
    if (srv->sceneBytes + srv->batchBytes + bytes > srv->budget)
        return AGB_ERR_OOM;
    srv->scenes[scene_id] = Scene{ ctx, bytes, {} };
    srv->sceneBytes += bytes;
    // The batches' shared namespace holds every registered scene, so batches of any mix of them
    // reuse it.
    std::vector<agb_context*> all;
    for (auto& kv : srv->scenes)
        all.push_back(kv.second.ctx);
    for (Batch& b : srv->batches)
        if (!b.busy)
            agb_batch_set_scenes(b.handle, all.data(), uint32_t(all.size()));
    return AGB_OK;
}

AGB_API agb_status agb_server_set_denoiser(agb_server* srv, agb_denoiser* dn)
{
    if (!srv)
        return AGB_ERR_INVALID_ARG;
    std::lock_guard<std::mutex> g(srv->mu);
    srv->denoiser = dn;
    return AGB_OK;
}

AGB_API agb_status agb_server_submit(agb_server* srv, const agb_serve_request* req, uint64_t* id)
{
    if (!srv || !req || !id || req->width == 0 || req->height == 0 || req->spp == 0)
        return AGB_ERR_INVALID_ARG;
    if ((req->flags & AGB_SERVE_DENOISE) && (req->width % 8 || req->height % 8))
        return AGB_ERR_INVALID_ARG;
    std::unique_ptr<Request> r(new Request());
    r->req     = *req;
    r->tSubmit = Clock::now();
    {
        std::lock_guard<std::mutex> g(srv->mu);
        r->id = srv->nextId++;
        *id   = r->id;
        srv->queue.push_back(r.get());
        srv->all[r->id] = std::move(r);
    }
    srv->wake.notify_all();
    return AGB_OK;
}

AGB_API agb_status agb_server_wait(agb_server* srv, uint64_t id, int32_t timeout_ms,
    agb_serve_result* result, float* host_rgba, uint64_t capacity)
{
    if (!srv)
        return AGB_ERR_INVALID_ARG;
    std::unique_lock<std::mutex> lk(srv->mu);
    auto it = srv->all.find(id);
    if (it == srv->all.end())
        return AGB_ERR_INVALID_ARG;
    Request* r = it->second.get();
    auto ready = [r] { return r->finished; };
    if (timeout_ms < 0)
        srv->doneCv.wait(lk, ready);
    else if (!srv->doneCv.wait_for(lk, std::chrono::milliseconds(timeout_ms), ready))
        return AGB_ERR_TIMEOUT;
    if (result)
    {
        result->id         = r->id;
        result->status     = r->status;
        result->width      = r->req.width;
        result->height     = r->req.height;
        bool started       = r->tStart.time_since_epoch().count() != 0;
        result->queue_ms   = started ? msSince(r->tSubmit, r->tStart) : msSince(r->tSubmit, r->tDone);
        result->render_ms  = started ? msSince(r->tStart, r->tDone) : 0.0;
        result->latency_ms = msSince(r->tSubmit, r->tDone);
    }
    agb_status st = r->status;
    if (!st && host_rgba)
    {
        if (capacity < r->rgba.size())
            return AGB_ERR_INVALID_ARG;
        memcpy(host_rgba, r->rgba.data(), r->rgba.size() * sizeof(float));
    }
    srv->all.erase(it);
    return st;
}

AGB_API agb_status agb_server_memory(agb_server* srv, uint64_t* scene_bytes, uint64_t* render_bytes)
{
    if (!srv)
        return AGB_ERR_INVALID_ARG;
    std::lock_guard<std::mutex> g(srv->mu);
    if (scene_bytes)
        *scene_bytes = srv->sceneBytes;
    if (render_bytes)
        *render_bytes = srv->batchBytes + srv->reserved + srv->pooled;
    return AGB_OK;
}
