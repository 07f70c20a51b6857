// wavefront.cuh — the streaming wavefront path tracer shared by the
// PathTracer pass (srt_pt_*) and the render-serving loop.
//
// One iteration = closest-hit kernel -> shade kernel -> shadow kernel ->
// regenerate kernel -> advance.  Paths of any number of jobs (scenes,
// resolutions, spp) share the queues; each path carries its job id.  In
// SRT_RNG_CURAND mode a pixel has at most one path in flight and its curand
// stream continues across its samples exactly as the megakernel's per-pixel
// loop (src/shader/integrator/path_tracer.cu:56-166) consumes it; a pixel
// whose path ends gets its next sample's camera ray in the same iteration.
#pragma once

#include <vector>

#include "common.h"
#include "device_types.h"
#include "mlp.cuh"

namespace srt {

// Radiance-cache state of a job (all null: a plain job).  Non-training
// pixels end their paths at the second vertex with a network query; one
// pixel in `train_stride` (offset `train_phase`) traces a full path and
// records up to 8 vertices whose targets are computed when it ends.
struct CacheRec {
    const __nv_bfloat16* w;   // network weights (bf16); null = plain job
    const __nv_bfloat16* wpack;  // the same weights in the tensor cores' canonical layout
    MlpBox box;
    float4* q_rec;            // [npix * 4] query records
    float4* q_beta;           // [npix] throughput (rgb), pixel (int bits)
    int32_t* q_count;         // queries this iteration; [1] fallback queries (total)
    const uint8_t* region_off;  // [res^3]: 1 = cache disabled in the cell (plain fallback)
    int32_t region_res;
    int32_t train_stride, train_phase, n_train;
    float4* t_rec;            // [n_train * 8 * 4] records of training vertices
    float4* t_aux;            // [n_train * 8 * 2]: (beta, -), (radiance before -> target, valid)
    int32_t* t_len;           // [n_train] recorded vertices
};
constexpr int kTrainVertices = 8;

// Per-job record read by every kernel (one per admitted render).
struct JobRec {
    SceneView scene;
    CameraRec cam;
    float4* film;        // caller film, float4[w*h], row-major idx = iy*w + ix
    float4* lpath;       // per pixel: radiance of the sample in flight (xyz) and
                         // the pixel's finished samples (w, int bits)
    int32_t* pixels_done;  // pixels that finished every sample (one int)
    int32_t* frame_done;   // [spp]: pixels that finished sample k (progressive frames), or null
    int32_t width, height, npix;
    int32_t spp, max_depth, rr_depth, use_nee, use_mis, seed, flags, rng_mode;
    CacheRec cache;
};

struct PathQueue {
    float4* o;     // origin, pixel (int bits)
    float4* d;     // direction, scatter pdf
    float4* beta;  // throughput, flags: depth bits 0-7, specular bit 8, job bits 16-31
    uint4* ra;     // rng state
    uint2* rb;
};

// A sample that ended in this iteration: its job and pixel, from k_shade to
// k_regen, which adds it to the film.
struct DoneQueue {
    uint2* rec;  // job, pixel
};

struct ShadowQueue {
    float4* o;  // origin, pixel (int bits)
    float4* d;  // direction, tmax
    float4* c;  // contribution, job (int bits)
};

struct Counters {
    // the path queue fills from both ends: paths that continue from the front
    // (n_next), next samples' camera rays from the back (n_cam), so that
    // camera rays, which traverse coherently, share warps; one 64-bit atomic
    // counts both (n_next the low word); the current queue's entries
    // [0, nf_cur) sit at slots 0.., the rest at capacity-1..
    alignas(8) int32_t n_next;
    int32_t n_cam;
    int32_t n_cur, nf_cur;
    alignas(8) int32_t n_shadow;  // with n_done: one 64-bit word, one atomic per warp
    int32_t n_done;
    // the previous iteration's shadow rays and ended samples, which this
    // iteration's k_trace and k_regen take
    int32_t n_sp, n_dp;
    alignas(8) int32_t n_hit;  // closest-hit results of the iteration, by kind (one 64-bit word)
    int32_t n_miss;
    unsigned long long fetch_closest, fetch_shadow;
    long long closest_total, shadow_total, iterations, started;
    long long c_nodes, c_tris, s_nodes, s_tris;  // traversal work (profiling kernels)
    int32_t overflow_stack, overflow_queue;
    long long run_iters, run_limit;  // iterations of the current graph launch and its bound
    // end of a frame: at or below tail_below paths in flight (0: never) the
    // iterations stop (tail_go) and k_finish carries the rest to the end
    int32_t tail_below, tail_go;
    unsigned long long fetch_tail;  // k_finish's next queue entry
    long long tail_paths;           // queue entries k_finish took
};

// Queue counts of one wavefront iteration (written by k_advance for the
// first kIterHistory iterations of a run).
struct IterCount {
    int32_t closest;   // rays through the closest-hit kernel
    int32_t hits;      // of those, rays that hit a triangle
    int32_t misses;    // of those, rays that left the scene
    int32_t shadow;    // rays through the shadow kernel
    int32_t done;      // samples that ended in the iteration
    int32_t pad[3];
};
constexpr int kIterHistory = 4096;

// Per-kernel device time gathered in profiling mode.
struct KernelTimes {
    double ms[5] = {0, 0, 0, 0, 0};  // closest, shade, shadow, regen, advance
    double tail_ms = 0;              // k_finish
    long long launches = 0;          // every kernel the engine launched
};

// Launches the radiance-cache query kernel over every job's queries (mlp.cu).
void launch_cache_queries(const JobRec* jobs, int max_jobs, cudaStream_t st);

// Device state of one wavefront engine (queues sized for `capacity` paths).
class Engine {
public:
    ~Engine();
    srt_status init(int64_t capacity, int max_jobs);
    int64_t capacity() const { return capacity_; }
    size_t device_bytes() const { return bytes_; }

    // Uploads a job record to slot `job` (stream-ordered).
    srt_status set_job(int job, const JobRec& rec, cudaStream_t st);
    // Seeds every pixel of `job`: film cleared, rng initialised, sample-0
    // camera rays appended to the current queue.
    srt_status start_job(int job, const JobRec& rec, cudaStream_t st);
    // Runs graph-captured iteration pairs until no path is in flight,
    // or (when `budget_iters` > 0) at most that many iterations.
    srt_status run(cudaStream_t st, long long max_iters, bool until_idle, long long budget_iters);
    srt_status reset_counters(cudaStream_t st);
    srt_status read_counters(Counters& c, cudaStream_t st);
    // Copies the first n recorded iterations' counts to host memory.
    srt_status read_history(IterCount* host, int n);
    int32_t* pixels_done_slot(int job) const { return pixels_done_ + job; }
    const int32_t* pixels_done_all() const { return pixels_done_; }
    // mode 0: off; 1: timestamps between the kernels and traversal work
    // counters (counting kernel variants); 2: timestamps only, the kernels
    // identical to the unprofiled ones
    void set_profiling(int mode)
    {
        const bool count = mode == 1;
        if (count != count_) drop_graphs();
        profile_ = mode != 0;
        count_ = count;
    }
    // adds the radiance-cache query kernel to the iteration (re-captures the graph)
    void enable_cache()
    {
        if (!cache_) {
            cache_ = true;
            drop_graphs();
        }
    }
    bool profiling() const { return profile_; }
    // direct = true: every iteration's kernels are launched one by one from
    // the host instead of through the captured graph (same kernels, same
    // results)
    void set_direct(bool direct) { direct_ = direct; }
    bool direct() const { return direct_; }
    // paths in flight at or below which a run's remaining samples are
    // finished by k_finish (plain jobs only; 0: the iterations run to the end)
    void set_tail(int32_t below)
    {
        if ((below > 0) != (tail_below_ > 0)) drop_graphs();  // k_finish joins or leaves the graphs
        tail_below_ = below;
    }
    int32_t tail() const { return tail_below_; }
    bool tail_on() const { return tail_below_ > 0 && !cache_; }
    KernelTimes& times() { return times_; }

private:
    srt_status capture(bool profile);
    void drop_graphs();
    // cond: the while-loop handle whose value k_advance sets, or null when
    // the host relaunches the iteration (profiling graph, direct launches)
    void launch_iteration(int parity, cudaStream_t st, bool profile, const cudaGraphConditionalHandle* cond);
    // after the loop: the flush of the last iteration's shadow rays and ended
    // samples, then k_finish and its counter update (no work unless the loop
    // stopped for it)
    void launch_post(cudaStream_t st, bool profile);

    int64_t capacity_ = 0;
    int max_jobs_ = 0;
    size_t bytes_ = 0;
    DeviceBuffer buf_;
    PathQueue q_[2]{};
    ShadowQueue sq_{};
    float4* hits_ = nullptr;
    int32_t* order_ = nullptr;  // queue indices in shading order (hits, then misses)
    DoneQueue done_{};
    Counters* counters_ = nullptr;
    IterCount* history_ = nullptr;  // [kIterHistory]
    JobRec* jobs_ = nullptr;
    int32_t* pixels_done_ = nullptr;
    Counters* host_counters_ = nullptr;
    cudaGraphExec_t graph_ = nullptr, graph_prof_ = nullptr;
    cudaStream_t graph_stream_ = nullptr;
    cudaStream_t side_stream_ = nullptr;        // k_regen beside k_order
    cudaEvent_t fork_ev_ = nullptr, join_ev_ = nullptr;
    cudaEvent_t ev_[2][5][2] = {};
    cudaEvent_t ev_tail_[2] = {};
    bool profile_ = false;
    bool count_ = true;
    bool cache_ = false;
    bool direct_ = false;
    KernelTimes times_;
    int grid_trace_ = 0, grid_stride_ = 0, grid_regen_ = 0, grid_shade_ = 0, grid_order_ = 0, grid_finish_ = 0;
    int32_t tail_below_ = 0;
};

}  // namespace srt

// The PathTracer pass: one engine, one job (srt_pt_* in wavefront.cu; the
// cached variant in cache.cu).
struct srt_pt {
    srt_scene* scene = nullptr;
    int width = 0, height = 0;
    srt::Engine engine;
    srt::DeviceBuffer job_buf;
    float4* lpath = nullptr;
    srt_pt_stats stats{};
    srt::DeviceBuffer cache_buf;  // radiance-cache buffers, sized on first cached render
    int64_t cache_train = 0;
    int cache_res = 0;
    int64_t frame = 0;
};
