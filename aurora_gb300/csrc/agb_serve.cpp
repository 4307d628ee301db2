// Serving loop: a persistent scheduler thread that admits interactive render requests of
// different scenes and resolutions onto the GPU as slots and memory free up (continuous
// batching), keeps the scenes' BVHs resident, and records each request's queueing, rendering and
// total latency.
//
// Scenes are agb_contexts uploaded by the caller and registered with their HBM footprint; the
// server refuses scenes beyond its HBM budget.  Each running request renders through a view of its
// scene (agb_view_create: own stream, frame, accumulation) so requests overlap on the device;
// views are pooled per scene and reused, and idle views are destroyed when a new request needs
// their memory.  A request's render state (wave buffers, accumulation, AOVs) is reserved against
// the budget before it is admitted; requests are admitted in arrival order.
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

// Paths in flight per request wave; bounds a slot's wave buffers (agb_bytes_per_path each).
constexpr uint64_t kServeWavePaths = 1u << 21;
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

uint64_t estimateBytes(const agb_serve_request& r)
{
    uint64_t pixels = uint64_t(r.width) * r.height;
    uint64_t spw    = std::max<uint64_t>(1, kServeWavePaths / std::max<uint64_t>(1, pixels));
    uint64_t paths  = std::min<uint64_t>(r.spp, spw) * pixels;
    return pixels * kBytesPerPixel + paths * agb_bytes_per_path() + (1u << 20);
}

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
    std::vector<Request*> running;
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
    void finish(Request* r);
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
        while (!sc.idle.empty() && sceneBytes + reserved + pooled + need > budget)
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

// Starts a request (lock held).  Returns false when it must wait for memory.
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
    if (sceneBytes + reserved + pooled + extra > budget)
        evictIdle(extra);
    if (sceneBytes + reserved + pooled + extra > budget)
    {
        if (running.empty())
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
    bool denoise     = (r->req.flags & AGB_SERVE_DENOISE) && denoiser;
    if (denoise)
        f.is_denoising_aovs_enabled = 1;
    agb_render_options opt{};
    opt.width               = r->req.width;
    opt.height              = r->req.height;
    opt.accumulation        = AGB_ACCUM_RUNNING_MEAN | (denoise ? AGB_ACCUM_MOMENTS : 0u);
    opt.max_paths_in_flight = uint32_t(kServeWavePaths);
    opt.seed_offset         = r->req.seed_offset;
    agb_status st = agb_frame_set(view, &f);
    if (!st)
        st = agb_render(view, &opt, 0, r->req.spp, nullptr);
    if (st)
    {
        std::string msg = agb_last_error();
        reserved -= r->reserved;
        sc.idle.push_back(view);
        uint64_t b = 0;
        agb_context_memory(view, &b);
        pooled += b;
        r->view = nullptr;
        failRequest(r, st, msg);
        return true;
    }
    running.push_back(r);
    return true;
}

void agb_server::finish(Request* r)
{
    Scene& sc = scenes[r->req.scene];
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
    reserved -= std::min(reserved, r->reserved);
    uint64_t b = 0;
    agb_context_memory(r->view, &b);
    pooled += b;
    sc.idle.push_back(r->view);
    r->view     = nullptr;
    r->finished = true;
    doneCv.notify_all();
}

void agb_server::run()
{
    cudaSetDevice(device);
    std::unique_lock<std::mutex> lk(mu);
    for (;;)
    {
        if (stop && queue.empty() && running.empty())
            break;
        // Completions: a request is done when its view's work has drained.
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
        // Admissions in arrival order while slots are free.
        while (!queue.empty() && int(running.size()) < maxSlots)
        {
            Request* r = queue.front();
            if (!admit(r, lk))
                break;
            queue.pop_front();
        }
        if (running.empty() && queue.empty())
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
    if (srv->sceneBytes + bytes > srv->budget)
        return AGB_ERR_OOM;
    srv->scenes[scene_id] = Scene{ ctx, bytes, {} };
    srv->sceneBytes += bytes;
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
        *render_bytes = srv->reserved + srv->pooled;
    return AGB_OK;
}
