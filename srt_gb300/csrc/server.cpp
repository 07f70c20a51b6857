// server.cpp — render serving: jobs of different scenes, resolutions and
// sample counts are admitted against an HBM budget and share one
// wavefront engine; their rays are packed into the same queues and the
// captured iteration graph advances all of them at once.  Jobs that arrive
// while others are on the GPU are admitted between steps as soon as a
// slot, queue capacity and memory free up (continuous batching).
#include <algorithm>
#include <chrono>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <set>
#include <string>
#include <vector>

#include "cache.cuh"
#include "common.h"
#include "mlp.cuh"
#include "scene.h"
#include "wavefront.cuh"

using namespace srt;

namespace {

struct Job {
    int64_t id = 0;
    srt_job_desc desc{};
    int32_t npix = 0;
    int32_t state = SRT_JOB_QUEUED;
    int slot = -1;
    int64_t bytes = 0;          // job state + server-owned film
    void* state_buf = nullptr;  // lpath | frame_done
    float* film = nullptr;
    bool own_film = false;
    double submit_s = 0, admit_s = -1, first_frame_s = -1, done_s = -1;
    std::vector<double> frame_times;
    size_t frames_off = 0;  // byte offset of the frame counters in state_buf
    bool trained = false;   // online training done (cache_train jobs)
};

// online training: training pixels per job (one pixel in `stride`)
constexpr int64_t kServeTrainPaths = 16384;
constexpr int kServeTrainSteps = 4;
constexpr float kServeTrainLr = 1e-2f;
int64_t train_stride(int64_t npix) { return 1 + npix / kServeTrainPaths; }
int64_t train_pixels(int64_t npix) { return (npix + train_stride(npix) - 1) / train_stride(npix); }

size_t frames_bytes(int spp) { return ((size_t)std::max(spp, 1) * 4 + 255) & ~(size_t)255; }

size_t state_bytes(int64_t npix, int spp, bool cache, bool train)
{
    // lpath 16 per pixel (rounded), frame counters, and for a cached job its
    // query records (64 B), throughputs (16 B) and counters, or, when it
    // trains online, the cache module's query and training buffers
    size_t b = (((size_t)npix * 16 + 255) & ~(size_t)255) + frames_bytes(spp);
    if (cache && train) b += cache_job_bytes(npix, train_pixels(npix));
    else if (cache) b += (size_t)npix * 80 + 256;
    return b;
}

bool trains(const srt_job_desc& d) { return d.cache != nullptr && d.cache_train != 0; }

}  // namespace

struct srt_server {
    srt_server_config cfg{};
    Engine engine;
    cudaStream_t stream = nullptr;
    std::chrono::steady_clock::time_point t0;
    int64_t next_id = 1;
    std::map<int64_t, std::unique_ptr<Job>> jobs;
    std::deque<int64_t> queued;
    std::vector<int64_t> slots;  // job id per slot, 0 = free
    int64_t paths_used = 0;
    int64_t bytes_used = 0;
    std::map<const srt_scene*, int> scene_refs;
    // pinned mirrors of the device progress counters
    int32_t* h_pixels_done = nullptr;
    int32_t* h_frames = nullptr;
    size_t h_frames_cap = 0;

    double now() const { return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count(); }

    int64_t scene_bytes(const srt_scene* sc) const { return sc->info.device_bytes; }

    int64_t need_bytes(const Job& j) const
    {
        int64_t b = j.bytes;
        if (!scene_refs.count(j.desc.scene)) b += scene_bytes(j.desc.scene);
        return b;
    }

    srt_status admit(Job& j, int slot)
    {
        const int spp = j.desc.params.samples_per_pixel;
        const bool cached = j.desc.cache != nullptr;
        size_t sb = state_bytes(j.npix, spp, cached, trains(j.desc));
        cudaError_t e = cudaMallocAsync(&j.state_buf, sb, stream);
        if (e != cudaSuccess) return cuda_error(e, "job state allocation");
        if (!j.desc.film) {
            e = cudaMallocAsync(reinterpret_cast<void**>(&j.film), (size_t)j.npix * 16, stream);
            if (e != cudaSuccess) {
                cudaFreeAsync(j.state_buf, stream);
                j.state_buf = nullptr;
                return cuda_error(e, "job film allocation");
            }
            j.own_film = true;
        } else {
            j.film = j.desc.film;
        }
        char* b = reinterpret_cast<char*>(j.state_buf);
        const size_t n = (size_t)j.npix;
        const size_t px_bytes = ((size_t)n * 16 + 255) & ~(size_t)255;
        int32_t* frame_done = reinterpret_cast<int32_t*>(b + px_bytes);
        SRT_CUDA_TRY(cudaMemsetAsync(frame_done, 0, frames_bytes(spp), stream));
        j.frames_off = px_bytes;
        JobRec J{};
        const srt_scene* sc = j.desc.scene;
        J.scene = sc->view;
        J.cam = sc->camera;
        J.cam.nw = J.cam.nh * ((float)j.desc.width / (float)j.desc.height);
        J.film = reinterpret_cast<float4*>(j.film);
        J.lpath = reinterpret_cast<float4*>(b);
        J.pixels_done = engine.pixels_done_slot(slot);
        J.frame_done = frame_done;
        J.width = j.desc.width;
        J.height = j.desc.height;
        J.npix = j.npix;
        J.spp = spp;
        J.max_depth = j.desc.params.max_depth;
        J.rr_depth = j.desc.params.rr_depth;
        J.use_nee = (j.desc.params.use_nee && sc->view.num_lights > 0) ? 1 : 0;
        J.use_mis = j.desc.params.use_mis ? 1 : 0;
        J.seed = j.desc.params.seed;
        J.flags = j.desc.params.flags;
        J.rng_mode = j.desc.params.rng_mode;
        if (cached) {
            // every pixel that is not a training pixel ends at its second
            // vertex with a query (no per-cell fallback while serving)
            char* cb = b + px_bytes + frames_bytes(spp);
            CacheRec& C = J.cache;
            C.w = j.desc.cache->wb;
            C.wpack = j.desc.cache->wpack;
            C.box = j.desc.cache->box;
            C.region_off = nullptr;
            C.region_res = 1;
            if (trains(j.desc)) {
                // online: one pixel in `stride` traces full paths and records
                // its first sample's vertices for the network's next steps
                cache_job_carve(cb, j.npix, train_pixels(j.npix), C);
                C.train_stride = (int32_t)train_stride(j.npix);
                C.train_phase = 0;
            } else {
                C.q_rec = reinterpret_cast<float4*>(cb);
                C.q_beta = reinterpret_cast<float4*>(cb + n * 64);
                C.q_count = reinterpret_cast<int32_t*>(cb + n * 80);
                C.train_stride = j.npix + 1;  // no training pixels
                C.train_phase = -1;
            }
            SRT_CUDA_TRY(cudaMemsetAsync(C.q_count, 0, 64, stream));
            engine.enable_cache();
        }
        SRT_TRY(engine.set_job(slot, J, stream));
        SRT_TRY(engine.start_job(slot, J, stream));
        j.slot = slot;
        j.state = SRT_JOB_RUNNING;
        j.admit_s = now();
        slots[slot] = j.id;
        paths_used += j.npix;
        bytes_used += need_bytes(j);
        scene_refs[j.desc.scene] += 1;
        return SRT_OK;
    }

    srt_status retire(Job& j, double t)
    {
        j.state = SRT_JOB_DONE;
        j.done_s = t;
        // Empty the slot's device record before its state is freed: the cache
        // kernels walk every slot and would otherwise reach the freed (and
        // soon reused) query counters and records of a cached job.
        srt_status st = engine.set_job(j.slot, JobRec{}, stream);
        if (j.state_buf) cudaFreeAsync(j.state_buf, stream);
        j.state_buf = nullptr;
        slots[j.slot] = 0;
        paths_used -= j.npix;
        bytes_used -= (int64_t)state_bytes(j.npix, j.desc.params.samples_per_pixel, j.desc.cache != nullptr,
                                           trains(j.desc));
        if (--scene_refs[j.desc.scene] == 0) {
            scene_refs.erase(j.desc.scene);
            bytes_used -= scene_bytes(j.desc.scene);
        }
        return st;
    }
};

extern "C" srt_status srt_server_create(const srt_server_config* cfg, srt_server** out)
{
    clear_error();
    if (!cfg || !out) return set_error(SRT_ERR_ARG, "NULL argument");
    *out = nullptr;
    if (cfg->max_jobs <= 0 || cfg->max_jobs > 65535 || cfg->max_paths <= 0 || cfg->hbm_budget_bytes <= 0 ||
        cfg->iterations_per_step <= 0)
        return set_error(SRT_ERR_ARG, "server config out of range");
    auto s = std::make_unique<srt_server>();
    s->cfg = *cfg;
    s->cfg.iterations_per_step = std::max(2, cfg->iterations_per_step + (cfg->iterations_per_step & 1));
    s->t0 = std::chrono::steady_clock::now();
    SRT_TRY(s->engine.init(cfg->max_paths, cfg->max_jobs));
    s->bytes_used = (int64_t)s->engine.device_bytes();
    if (s->bytes_used > cfg->hbm_budget_bytes) return set_error(SRT_ERR_BUDGET, "engine queues exceed the HBM budget");
    SRT_CUDA_TRY(cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking));
    s->slots.assign(cfg->max_jobs, 0);
    SRT_CUDA_TRY(cudaMallocHost(reinterpret_cast<void**>(&s->h_pixels_done), 4 * (size_t)cfg->max_jobs));
    SRT_TRY(s->engine.reset_counters(s->stream));
    *out = s.release();
    return SRT_OK;
}

extern "C" srt_status srt_server_submit(srt_server* s, const srt_job_desc* d, int64_t* job_id)
{
    clear_error();
    if (!s || !d || !job_id || !d->scene) return set_error(SRT_ERR_ARG, "NULL argument");
    const srt_pt_params& p = d->params;
    if (d->width <= 0 || d->height <= 0 || p.samples_per_pixel <= 0 || p.max_depth <= 0 || p.max_depth > 255 ||
        p.rng_mode != SRT_RNG_CURAND)
        return set_error(SRT_ERR_ARG, "job parameters out of range");
    if (d->film && reinterpret_cast<uintptr_t>(d->film) % 16) return set_error(SRT_ERR_ARG, "film must be 16-byte aligned");
    auto j = std::make_unique<Job>();
    j->id = s->next_id++;
    j->desc = *d;
    j->npix = d->width * d->height;
    j->bytes = (int64_t)state_bytes(j->npix, p.samples_per_pixel, d->cache != nullptr, trains(*d)) +
               (d->film ? 0 : (int64_t)j->npix * 16);
    if (d->cache && p.max_depth < 2) return set_error(SRT_ERR_ARG, "cached jobs need max_depth >= 2");
    j->submit_s = s->now();
    int64_t fixed = (int64_t)s->engine.device_bytes();
    if (j->npix > s->cfg.max_paths || fixed + j->bytes + d->scene->info.device_bytes > s->cfg.hbm_budget_bytes)
        return set_error(SRT_ERR_BUDGET, "job can never fit the server's paths or HBM budget");
    *job_id = j->id;
    s->queued.push_back(j->id);
    s->jobs.emplace(j->id, std::move(j));
    return SRT_OK;
}

extern "C" srt_status srt_server_step(srt_server* s, int32_t* running, int32_t* queued)
{
    clear_error();
    if (!s) return set_error(SRT_ERR_ARG, "NULL argument");
    // admission: first fit in arrival order
    for (auto it = s->queued.begin(); it != s->queued.end();) {
        Job& j = *s->jobs[*it];
        int slot = -1;
        for (int k = 0; k < (int)s->slots.size(); ++k)
            if (s->slots[k] == 0) {
                slot = k;
                break;
            }
        if (slot < 0) break;
        if (s->paths_used + j.npix <= s->cfg.max_paths && s->bytes_used + s->need_bytes(j) <= s->cfg.hbm_budget_bytes) {
            srt_status st = s->admit(j, slot);
            if (st != SRT_OK) {
                if (st == SRT_ERR_OOM) {  // device allocator full: keep queued
                    ++it;
                    continue;
                }
                j.state = SRT_JOB_FAILED;
                it = s->queued.erase(it);
                return st;
            }
            it = s->queued.erase(it);
        } else {
            ++it;
        }
    }
    int nrun = 0;
    for (int64_t id : s->slots) nrun += id != 0;
    if (nrun > 0) {
        SRT_TRY(s->engine.run(s->stream, 0, false, s->cfg.iterations_per_step));
        // progress counters of the running jobs
        size_t nf = 0;
        for (int64_t id : s->slots)
            if (id) nf += (size_t)s->jobs[id]->desc.params.samples_per_pixel;
        if (nf > s->h_frames_cap) {
            if (s->h_frames) cudaFreeHost(s->h_frames);
            SRT_CUDA_TRY(cudaMallocHost(reinterpret_cast<void**>(&s->h_frames), nf * 4));
            s->h_frames_cap = nf;
        }
        SRT_CUDA_TRY(cudaMemcpyAsync(s->h_pixels_done, s->engine.pixels_done_all(), 4 * s->slots.size(),
                                     cudaMemcpyDeviceToHost, s->stream));
        size_t off = 0;
        for (int64_t id : s->slots) {
            if (!id) continue;
            Job& j = *s->jobs[id];
            const char* b = reinterpret_cast<const char*>(j.state_buf) + j.frames_off;
            SRT_CUDA_TRY(cudaMemcpyAsync(s->h_frames + off, b, 4 * (size_t)j.desc.params.samples_per_pixel,
                                         cudaMemcpyDeviceToHost, s->stream));
            off += (size_t)j.desc.params.samples_per_pixel;
        }
        SRT_CUDA_TRY(cudaStreamSynchronize(s->stream));
        const double t = s->now();
        off = 0;
        for (size_t k = 0; k < s->slots.size(); ++k) {
            int64_t id = s->slots[k];
            if (!id) continue;
            Job& j = *s->jobs[id];
            const int spp = j.desc.params.samples_per_pixel;
            while ((int)j.frame_times.size() < spp && s->h_frames[off + j.frame_times.size()] >= j.npix) {
                if (j.frame_times.empty()) j.first_frame_s = t;
                j.frame_times.push_back(t);
            }
            off += (size_t)spp;
            if (trains(j.desc) && !j.trained && !j.frame_times.empty()) {
                // every training pixel has finished the sample that recorded its vertices
                char* cb = reinterpret_cast<char*>(j.state_buf) + j.frames_off + frames_bytes(spp);
                int64_t nv = 0;
                SRT_TRY(cache_job_train(cb, j.npix, train_pixels(j.npix), j.desc.cache, kServeTrainSteps,
                                        kServeTrainLr, s->stream, &nv));
                j.trained = true;
            }
            if (s->h_pixels_done[k] >= j.npix) SRT_TRY(s->retire(j, t));
        }
    }
    if (running) {
        int n = 0;
        for (int64_t id : s->slots) n += id != 0;
        *running = n;
    }
    if (queued) *queued = (int32_t)s->queued.size();
    return SRT_OK;
}

extern "C" srt_status srt_server_drain(srt_server* s, double timeout_s)
{
    clear_error();
    if (!s) return set_error(SRT_ERR_ARG, "NULL argument");
    double t_end = s->now() + timeout_s;
    for (;;) {
        int32_t r = 0, q = 0;
        SRT_TRY(srt_server_step(s, &r, &q));
        if (r == 0 && q == 0) return SRT_OK;
        if (s->now() > t_end) return set_error(SRT_ERR_TIMEOUT, "server did not drain in time");
    }
}

extern "C" srt_status srt_server_job_info(const srt_server* s, int64_t id, srt_job_info* info)
{
    clear_error();
    if (!s || !info) return set_error(SRT_ERR_ARG, "NULL argument");
    auto it = s->jobs.find(id);
    if (it == s->jobs.end()) return set_error(SRT_ERR_NOT_FOUND, "unknown job id");
    const Job& j = *it->second;
    info->state = j.state;
    info->frames_done = (int32_t)j.frame_times.size();
    info->submit_s = j.submit_s;
    info->admit_s = j.admit_s;
    info->first_frame_s = j.first_frame_s;
    info->done_s = j.done_s;
    info->device_bytes = j.bytes;
    return SRT_OK;
}

extern "C" srt_status srt_server_frame_times(const srt_server* s, int64_t id, double* times, int32_t max, int32_t* n)
{
    clear_error();
    if (!s || !n || (max > 0 && !times)) return set_error(SRT_ERR_ARG, "NULL argument");
    auto it = s->jobs.find(id);
    if (it == s->jobs.end()) return set_error(SRT_ERR_NOT_FOUND, "unknown job id");
    const Job& j = *it->second;
    int32_t k = (int32_t)std::min<size_t>(j.frame_times.size(), (size_t)std::max(max, 0));
    for (int32_t i = 0; i < k; ++i) times[i] = j.frame_times[i];
    *n = (int32_t)j.frame_times.size();
    return SRT_OK;
}

extern "C" srt_status srt_server_film(const srt_server* s, int64_t id, float** film)
{
    clear_error();
    if (!s || !film) return set_error(SRT_ERR_ARG, "NULL argument");
    auto it = s->jobs.find(id);
    if (it == s->jobs.end()) return set_error(SRT_ERR_NOT_FOUND, "unknown job id");
    *film = it->second->film ? it->second->film : it->second->desc.film;
    return SRT_OK;
}

extern "C" srt_status srt_server_release(srt_server* s, int64_t id)
{
    clear_error();
    if (!s) return set_error(SRT_ERR_ARG, "NULL argument");
    auto it = s->jobs.find(id);
    if (it == s->jobs.end()) return set_error(SRT_ERR_NOT_FOUND, "unknown job id");
    Job& j = *it->second;
    if (j.state == SRT_JOB_RUNNING) return set_error(SRT_ERR_ARG, "job is still running");
    if (j.state == SRT_JOB_QUEUED) s->queued.erase(std::find(s->queued.begin(), s->queued.end(), id));
    if (j.own_film && j.film) {
        cudaFreeAsync(j.film, s->stream);
        if (j.state == SRT_JOB_DONE) s->bytes_used -= (int64_t)j.npix * 16;
    }
    s->jobs.erase(it);
    return SRT_OK;
}

extern "C" double srt_server_now(const srt_server* s) { return s ? s->now() : 0.0; }

extern "C" void srt_server_destroy(srt_server* s)
{
    if (!s) return;
    if (s->stream) cudaStreamSynchronize(s->stream);
    for (auto& kv : s->jobs) {
        Job& j = *kv.second;
        if (j.state_buf) cudaFree(j.state_buf);
        if (j.own_film && j.film) cudaFree(j.film);
    }
    if (s->h_pixels_done) cudaFreeHost(s->h_pixels_done);
    if (s->h_frames) cudaFreeHost(s->h_frames);
    if (s->stream) cudaStreamDestroy(s->stream);
    delete s;
}
