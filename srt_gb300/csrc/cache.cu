// cache.cu — the PathTracer pass with a radiance cache (srt_pt_render_cached).
//
// Per frame: most pixels end their paths at the second vertex, where the
// network's outgoing radiance times the path throughput replaces the rest
// of the path; one pixel in `stride` traces a full path (up to 8 recorded
// vertices) whose radiance after each vertex, divided by the throughput
// that reached it, is that vertex's training target (the estimator of the
// NeuralRadiosity RHS pass, src/shader/npr/nr_rhs.cu:50-157, trained online
// instead of offline).  After the frame the targets are gathered, the
// network's relative bias is measured per cell of a coarse grid (cells not
// yet measured, or whose bias is shown to exceed the threshold, fall back
// to plain tracing for the next frame) and the network takes a few Adam
// steps.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>

#include "cache.cuh"
#include "common.h"
#include "mlp.cuh"
#include "scene.h"
#include "wavefront.cuh"

using namespace srt;

namespace {

struct CacheBuffers {
    float4* q_rec;
    float4* q_beta;
    int32_t* q_count;  // [0] queries this iteration, [1] fallback total, [2] batch size,
                       // [3] disabled cells, [4] query total
    uint8_t* region_off;
    float4* region_stat;  // per cell: ema predicted luminance, ema target luminance, ema count, -
    float4* region_new;   // per cell: this frame's sums
    float4* t_rec;
    float4* t_aux;
    int32_t* t_len;
    float4* b_rec;
    float4* b_tgt;
    float4* b_pred;
    float* loss_hist;  // loss of each Adam step of the frame
    int32_t* g_block;  // valid training vertices per gather block
};

constexpr int kMaxTrainSteps = 64;
constexpr int kGatherThreads = 256;  // training-vertex slots per gather block

size_t a256(size_t x) { return (x + 255) & ~(size_t)255; }

CacheBuffers carve(char* base, int64_t npix, int64_t n_train, int res)
{
    CacheBuffers b;
    size_t o = 0;
    auto take = [&](size_t bytes) {
        char* p = base + o;
        o += a256(bytes);
        return p;
    };
    const size_t cells = (size_t)res * res * res;
    const size_t nv = (size_t)n_train * kTrainVertices;
    b.q_rec = (float4*)take((size_t)npix * 64);
    b.q_beta = (float4*)take((size_t)npix * 16);
    b.q_count = (int32_t*)take(64);
    b.region_off = (uint8_t*)take(cells);
    b.region_stat = (float4*)take(cells * 16);
    b.region_new = (float4*)take(cells * 16);
    b.t_rec = (float4*)take(nv * 64);
    b.t_aux = (float4*)take(nv * 32);
    b.t_len = (int32_t*)take((size_t)n_train * 4);
    b.b_rec = (float4*)take(nv * 64);
    b.b_tgt = (float4*)take(nv * 16);
    b.b_pred = (float4*)take(nv * 16);
    b.loss_hist = (float*)take(kMaxTrainSteps * 4);
    b.g_block = (int32_t*)take((nv / kGatherThreads + 1) * 4);
    return b;
}

size_t carve_bytes(int64_t npix, int64_t n_train, int res)
{
    const size_t cells = (size_t)res * res * res;
    const size_t nv = (size_t)n_train * kTrainVertices;
    return a256((size_t)npix * 64) + a256((size_t)npix * 16) + a256(64) + a256(cells) + 2 * a256(cells * 16) +
           a256(nv * 64) + a256(nv * 32) + a256((size_t)n_train * 4) + a256(nv * 64) + 2 * a256(nv * 16) +
           a256(kMaxTrainSteps * 4) + a256((nv / kGatherThreads + 1) * 4) + 256;
}

// Valid training vertices -> contiguous (record, target) batch, in vertex
// order (a stable compaction, so the batch and hence the training steps are
// the same on every run): k_gather_count counts each block's valid slots,
// k_gather_scatter places them after the earlier blocks' ones.
__device__ __forceinline__ bool train_vertex_valid(const CacheBuffers& b, int n_train, int i)
{
    if (i >= n_train * kTrainVertices) return false;
    const int ts = i / kTrainVertices, k = i % kTrainVertices;
    return k < b.t_len[ts] && b.t_aux[2 * (size_t)i + 1].w > 0.0f;
}

__global__ void __launch_bounds__(kGatherThreads) k_gather_count(CacheBuffers b, int n_train)
{
    const int i = blockIdx.x * kGatherThreads + threadIdx.x;
    const int c = __syncthreads_count(train_vertex_valid(b, n_train, i));
    if (threadIdx.x == 0) b.g_block[blockIdx.x] = c;
}

__global__ void __launch_bounds__(kGatherThreads) k_gather_scatter(CacheBuffers b, int n_train, int32_t* count)
{
    __shared__ int32_t part[kGatherThreads / 32];
    __shared__ int32_t warp_valid[kGatherThreads / 32];
    const int t = threadIdx.x, lane = t & 31, w = t >> 5;
    // valid slots of the earlier blocks
    int before = 0;
    for (int k = t; k < (int)blockIdx.x; k += kGatherThreads) before += b.g_block[k];
    for (int o = 16; o > 0; o >>= 1) before += __shfl_xor_sync(0xffffffffu, before, o);
    const int i = blockIdx.x * kGatherThreads + t;
    const bool valid = train_vertex_valid(b, n_train, i);
    const uint32_t vb = __ballot_sync(0xffffffffu, valid);
    if (lane == 0) {
        part[w] = before;
        warp_valid[w] = __popc(vb);
    }
    __syncthreads();
    int offset = 0, in_block = 0;
    for (int k = 0; k < kGatherThreads / 32; ++k) {
        offset += part[k];
        if (k < w) in_block += warp_valid[k];
    }
    if (valid) {
        const int slot = offset + in_block + __popc(vb & ((1u << lane) - 1u));
        for (int j = 0; j < 4; ++j) b.b_rec[4 * (size_t)slot + j] = b.t_rec[4 * (size_t)i + j];
        b.b_tgt[slot] = b.t_aux[2 * (size_t)i + 1];
    }
    if (blockIdx.x == gridDim.x - 1 && t == 0) {
        int total = 0;
        for (int k = 0; k < kGatherThreads / 32; ++k) total += warp_valid[k];
        *count = offset + total;
    }
}

__device__ __forceinline__ int cell_of(float4 p, MlpBox box, int r)
{
    int x = min(max((int)((p.x - box.lo.x) * box.inv_extent.x * r), 0), r - 1);
    int y = min(max((int)((p.y - box.lo.y) * box.inv_extent.y * r), 0), r - 1);
    int z = min(max((int)((p.z - box.lo.z) * box.inv_extent.z * r), 0), r - 1);
    return (z * r + y) * r + x;
}

__device__ __forceinline__ float lum(float4 c) { return 0.2126f * c.x + 0.7152f * c.y + 0.0722f * c.z; }

// per-cell sums of predicted luminance, target luminance, count and squared
// target luminance over this frame's batch
__global__ void k_region_sums(CacheBuffers b, const int32_t* count, MlpBox box, int res)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= *count) return;
    int c = cell_of(b.b_rec[4 * (size_t)i], box, res);
    float t = lum(b.b_tgt[i]);
    atomicAdd(&b.region_new[c].x, lum(b.b_pred[i]));
    atomicAdd(&b.region_new[c].y, t);
    atomicAdd(&b.region_new[c].z, 1.0f);
    atomicAdd(&b.region_new[c].w, t * t);
}

// Exponential moving averages per cell.  A cell is served by the network
// only once it holds 16 (weighted) samples and its measured relative bias
// is not shown to exceed the threshold: |mean pred - mean target| minus two
// standard errors of the target mean must stay below threshold * mean
// target.  Unmeasured cells, including every cell before the first
// training frame, are traced plainly.
__global__ void k_region_update(CacheBuffers b, int cells, float threshold, float decay, int32_t* disabled)
{
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= cells) return;
    float4 s = b.region_stat[c], n = b.region_new[c];
    s.x = decay * s.x + n.x;
    s.y = decay * s.y + n.y;
    s.z = decay * s.z + n.z;
    s.w = decay * s.w + n.w;
    b.region_stat[c] = s;
    b.region_new[c] = make_float4(0.f, 0.f, 0.f, 0.f);
    bool off = true;
    if (s.z >= 16.0f) {
        float mp = s.x / s.z, mt = s.y / s.z;
        float se = sqrtf(fmaxf(s.w / s.z - mt * mt, 0.0f) / s.z);
        off = fabsf(mp - mt) - 2.0f * se > threshold * (mt + 1e-3f);
    }
    b.region_off[c] = off ? 1 : 0;
    if (off) atomicAdd(disabled, 1);
}

}  // namespace

namespace srt {

size_t cache_job_bytes(int64_t npix, int64_t n_train) { return carve_bytes(npix, n_train, 1); }

void cache_job_carve(char* base, int64_t npix, int64_t n_train, CacheRec& C)
{
    CacheBuffers b = carve(base, npix, n_train, 1);
    C.q_rec = b.q_rec;
    C.q_beta = b.q_beta;
    C.q_count = b.q_count;
    C.t_rec = b.t_rec;
    C.t_aux = b.t_aux;
    C.t_len = b.t_len;
    C.n_train = (int32_t)n_train;
}

srt_status cache_job_train(char* base, int64_t npix, int64_t n_train, srt_mlp* mlp, int steps, float lr,
                           cudaStream_t st, int64_t* vertices)
{
    CacheBuffers b = carve(base, npix, n_train, 1);
    const int gblocks = (int)((n_train * kTrainVertices + kGatherThreads - 1) / kGatherThreads);
    k_gather_count<<<gblocks, kGatherThreads, 0, st>>>(b, (int)n_train);
    k_gather_scatter<<<gblocks, kGatherThreads, 0, st>>>(b, (int)n_train, b.q_count + 2);
    SRT_CUDA_TRY(cudaGetLastError());
    int32_t nb32 = 0;
    SRT_CUDA_TRY(cudaMemcpyAsync(&nb32, b.q_count + 2, 4, cudaMemcpyDeviceToHost, st));
    SRT_CUDA_TRY(cudaStreamSynchronize(st));
    const int64_t nb = nb32;
    steps = std::max(1, std::min(steps, kMaxTrainSteps));
    const int64_t slice = (nb + steps - 1) / steps;
    for (int s = 0; s < steps && nb > 0; ++s) {
        const int64_t b0 = s * slice, n = std::min(slice, nb - b0);
        if (n <= 0) break;
        SRT_TRY(mlp_train_launch(mlp, b.b_rec + 4 * b0, b.b_tgt + b0, n, lr, true, st));
    }
    SRT_CUDA_TRY(cudaMemsetAsync(b.q_count + 2, 0, 4, st));
    if (vertices) *vertices = nb;
    return SRT_OK;
}

}  // namespace srt

extern "C" srt_status srt_pt_render_cached(srt_pt* p, float* film, const srt_pt_params* prm, srt_mlp* mlp,
                                           const srt_cache_params* cp, srt_cache_stats* stats, void* stream)
{
    clear_error();
    if (!p || !film || !prm || !mlp || !cp) return set_error(SRT_ERR_ARG, "NULL argument");
    if (prm->samples_per_pixel <= 0 || prm->max_depth < 2 || prm->max_depth > 255 || prm->rng_mode != SRT_RNG_CURAND)
        return set_error(SRT_ERR_ARG, "cached rendering needs spp >= 1, 2 <= max_depth <= 255, curand streams");
    if (cp->train_paths <= 0 || cp->region_res <= 0 || cp->region_res > 64 || cp->train_steps < 0 ||
        cp->train_steps > kMaxTrainSteps ||
        !(cp->learning_rate >= 0.0f))
        return set_error(SRT_ERR_ARG, "cache parameters out of range");
    if (reinterpret_cast<uintptr_t>(film) % 16) return set_error(SRT_ERR_ARG, "film must be 16-byte aligned");
    cudaStream_t st = as_stream(stream);
    const int npix = p->width * p->height;
    const int stride = std::max(1, npix / cp->train_paths);
    const int n_train = (npix + stride - 1) / stride;
    const int res = cp->region_res;
    const int cells = res * res * res;
    if (p->cache_train != n_train || p->cache_res != res) {
        SRT_TRY(p->cache_buf.alloc(carve_bytes(npix, n_train, res), "radiance-cache buffers"));
        SRT_CUDA_TRY(cudaMemset(p->cache_buf.get(), 0, p->cache_buf.bytes()));
        p->cache_train = n_train;
        p->cache_res = res;
        // no cell has been measured: all trace plainly until the first training frame
        CacheBuffers b0 = carve(p->cache_buf.as<char>(), npix, n_train, res);
        SRT_CUDA_TRY(cudaMemset(b0.region_off, 1, (size_t)cells));
    }
    CacheBuffers b = carve(p->cache_buf.as<char>(), npix, n_train, res);
    srt_scene* sc = p->scene;
    JobRec J{};
    J.scene = sc->view;
    J.cam = sc->camera;
    J.film = reinterpret_cast<float4*>(film);
    J.lpath = p->lpath;
    J.pixels_done = p->engine.pixels_done_slot(0);
    J.width = p->width;
    J.height = p->height;
    J.npix = npix;
    J.spp = prm->samples_per_pixel;
    J.max_depth = prm->max_depth;
    J.rr_depth = prm->rr_depth;
    J.use_nee = (prm->use_nee && sc->view.num_lights > 0) ? 1 : 0;
    J.use_mis = prm->use_mis ? 1 : 0;
    J.seed = prm->seed;
    J.flags = prm->flags;
    J.rng_mode = prm->rng_mode;
    CacheRec& C = J.cache;
    C.w = mlp->wb;
    C.wpack = mlp->wpack;
    C.box = mlp->box;
    C.q_rec = b.q_rec;
    C.q_beta = b.q_beta;
    C.q_count = b.q_count;
    C.region_off = b.region_off;
    C.region_res = res;
    C.train_stride = stride;
    C.train_phase = (int)(p->frame % stride);
    C.n_train = n_train;
    C.t_rec = b.t_rec;
    C.t_aux = b.t_aux;
    C.t_len = b.t_len;
    p->frame += 1;

    p->engine.enable_cache();
    p->engine.times() = KernelTimes();
    SRT_TRY(p->engine.reset_counters(st));
    SRT_CUDA_TRY(cudaMemsetAsync(b.q_count, 0, 32, st));
    SRT_TRY(p->engine.set_job(0, J, st));
    SRT_TRY(p->engine.start_job(0, J, st));
    long long bound = (long long)prm->samples_per_pixel * (prm->max_depth + 1) + 16;
    auto t0 = std::chrono::steady_clock::now();
    SRT_TRY(p->engine.run(st, 2 * bound, true, 0));
    Counters cnt;
    SRT_TRY(p->engine.read_counters(cnt, st));
    auto t1 = std::chrono::steady_clock::now();

    srt_cache_stats out{};
    int32_t host_counts[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    if (cp->train) {
        const int gblocks = (n_train * kTrainVertices + kGatherThreads - 1) / kGatherThreads;
        k_gather_count<<<gblocks, kGatherThreads, 0, st>>>(b, n_train);
        k_gather_scatter<<<gblocks, kGatherThreads, 0, st>>>(b, n_train, b.q_count + 2);
        SRT_CUDA_TRY(cudaGetLastError());
        SRT_CUDA_TRY(cudaMemcpyAsync(host_counts, b.q_count, 32, cudaMemcpyDeviceToHost, st));
        SRT_CUDA_TRY(cudaStreamSynchronize(st));
        const int64_t nb = host_counts[2];
        if (nb > 0) {
            // network error per cell before this frame's update decides the fallback mask
            SRT_TRY(mlp_infer_launch(mlp, b.b_rec, nb, b.b_pred, st));
            k_region_sums<<<(int)((nb + 255) / 256), 256, 0, st>>>(b, b.q_count + 2, mlp->box, res);
            SRT_CUDA_TRY(cudaMemsetAsync(b.q_count + 3, 0, 4, st));
            k_region_update<<<(cells + 255) / 256, 256, 0, st>>>(b, cells, cp->region_threshold, 0.9f,
                                                                  b.q_count + 3);
            SRT_CUDA_TRY(cudaGetLastError());
            const int steps = std::max(1, cp->train_steps);
            const int64_t slice = (nb + steps - 1) / steps;
            int used = 0;
            for (int s = 0; s < steps; ++s) {
                int64_t b0 = s * slice, n = std::min(slice, nb - b0);
                if (n <= 0) break;
                SRT_TRY(mlp_train_launch(mlp, b.b_rec + 4 * b0, b.b_tgt + b0, n, cp->learning_rate, true, st));
                SRT_CUDA_TRY(cudaMemcpyAsync(b.loss_hist + s, mlp->loss, 4, cudaMemcpyDeviceToDevice, st));
                ++used;
            }
            float losses[kMaxTrainSteps];
            if (used) {
                SRT_CUDA_TRY(cudaMemcpyAsync(losses, b.loss_hist, 4 * (size_t)used, cudaMemcpyDeviceToHost, st));
                SRT_CUDA_TRY(cudaStreamSynchronize(st));
            }
            float loss_sum = 0.0f;
            for (int s = 0; s < used; ++s) loss_sum += losses[s];
            out.loss = used ? loss_sum / (float)used : 0.0f;
            out.train_vertices = nb;
        }
        SRT_CUDA_TRY(cudaMemcpyAsync(host_counts, b.q_count, 32, cudaMemcpyDeviceToHost, st));
        SRT_CUDA_TRY(cudaMemsetAsync(b.q_count + 2, 0, 8, st));
    } else {
        SRT_CUDA_TRY(cudaMemcpyAsync(host_counts, b.q_count, 32, cudaMemcpyDeviceToHost, st));
    }
    SRT_CUDA_TRY(cudaStreamSynchronize(st));
    auto t2 = std::chrono::steady_clock::now();
    out.trace_ms = (float)std::chrono::duration<double, std::milli>(t1 - t0).count();
    out.train_ms = (float)std::chrono::duration<double, std::milli>(t2 - t1).count();
    out.fallback_queries = host_counts[1];
    out.disabled_cells = host_counts[3];
    out.queries = host_counts[4];
    p->stats.samples = cnt.started;
    p->stats.closest_rays = cnt.closest_total;
    p->stats.shadow_rays = cnt.shadow_total;
    p->stats.iterations = cnt.iterations;
    p->stats.stack_overflows = cnt.overflow_stack;
    p->stats.kernel_launches = p->engine.times().launches;
    SRT_CUDA_TRY(cudaMemsetAsync(b.q_count + 1, 0, 4, st));
    if (stats) *stats = out;
    return SRT_OK;
}
