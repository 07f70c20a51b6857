// trace_kernels.cu — batch ray queries against a resident scene
// (srt_trace_closest / srt_trace_shadow).  Warps fetch 32 rays at a time
// from a global counter so long rays do not hold a whole block.
#include "scene.h"
#include "trace.cuh"

using namespace srt;

namespace {

constexpr int kTraceThreads = 128;

__global__ void __launch_bounds__(kTraceThreads, SRT_TRACE_MIN_BLOCKS) k_trace_closest(SceneView S, const float4* __restrict__ rays,
                                                                    int64_t n, float4* __restrict__ hits,
                                                                    unsigned long long* counter, int* overflow_flag)
{
    __shared__ uint2 stack_mem[kStackEntries * kTraceThreads];
    Stack st{stack_mem + threadIdx.x, kTraceThreads, 0};
    int overflow = 0;
    TraceCount cnt;
    trace_persistent<false, false>(
        n, counter, st, overflow, cnt,
        [&](int64_t i, TravState& s, Stack& stk) {
            float4 a = __ldg(rays + 2 * i), b = __ldg(rays + 2 * i + 1);
            trav_init(s, S.nodes, S.tris, f3(a), f3(b), a.w, b.w, stk);
        },
        [&](int64_t i, const TravState& s, bool fin) {
            if (!fin) return;
            int32_t prim = s.tri >= 0 ? __ldg(S.tri_prim + s.tri) : -1;
            const float2 uv = hit_barycentrics(s);
            hits[i] = make_float4(s.tmax, uv.x, uv.y, __int_as_float(prim));
        });
    if (overflow) atomicAdd(overflow_flag, 1);
}

__global__ void __launch_bounds__(kTraceThreads, SRT_TRACE_MIN_BLOCKS) k_trace_shadow(SceneView S, const float4* __restrict__ rays,
                                                                   int64_t n, int32_t* __restrict__ visible,
                                                                   unsigned long long* counter, int* overflow_flag)
{
    __shared__ uint2 stack_mem[kStackEntries * kTraceThreads];
    Stack st{stack_mem + threadIdx.x, kTraceThreads, 0};
    int overflow = 0;
    TraceCount cnt;
    trace_persistent<true, false>(
        n, counter, st, overflow, cnt,
        [&](int64_t i, TravState& s, Stack& stk) {
            float4 a = __ldg(rays + 2 * i), b = __ldg(rays + 2 * i + 1);
            trav_init(s, S.nodes, S.tris, f3(a), f3(b), a.w, b.w, stk, SRT_SHADOW_FAR_FIRST != 0);
        },
        [&](int64_t i, const TravState& s, bool fin) {
            if (fin) visible[i] = s.tri >= 0 ? 0 : 1;
        });
    if (overflow) atomicAdd(overflow_flag, 1);
}

// tex2D of one of the scene's textures at n normalised coordinates
__global__ void __launch_bounds__(256) k_texture_lookup(cudaTextureObject_t tex, const float2* __restrict__ uv,
                                                             int64_t n, float4* __restrict__ out)
{
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        const float2 c = __ldg(uv + i);
        out[i] = tex2D<float4>(tex, c.x, c.y);
    }
}

struct QueryScratch {
    unsigned long long counter;
    int overflow;
    int pad;
};

srt_status run_query(const srt_scene* s, const float* rays, int64_t n, void* out, bool shadow, void* stream)
{
    clear_error();
    if (!s || (n > 0 && (!rays || !out))) return set_error(SRT_ERR_ARG, "NULL argument");
    if (n < 0) return set_error(SRT_ERR_ARG, "negative ray count");
    if (reinterpret_cast<uintptr_t>(rays) % 16 != 0) return set_error(SRT_ERR_ARG, "rays must be 16-byte aligned");
    if (!shadow && reinterpret_cast<uintptr_t>(out) % 16 != 0)
        return set_error(SRT_ERR_ARG, "hits must be 16-byte aligned");
    if (n == 0) return SRT_OK;
    cudaStream_t st = as_stream(stream);
    QueryScratch* scratch = nullptr;
    SRT_CUDA_TRY(cudaMallocAsync(reinterpret_cast<void**>(&scratch), sizeof(QueryScratch), st));
    cudaError_t e = cudaMemsetAsync(scratch, 0, sizeof(QueryScratch), st);
    int blocks = device_sm_count() * 8;
    if (e == cudaSuccess) {
        if (shadow)
            k_trace_shadow<<<blocks, kTraceThreads, 0, st>>>(s->view, reinterpret_cast<const float4*>(rays), n,
                                                              reinterpret_cast<int32_t*>(out), &scratch->counter,
                                                              &scratch->overflow);
        else
            k_trace_closest<<<blocks, kTraceThreads, 0, st>>>(s->view, reinterpret_cast<const float4*>(rays), n,
                                                               reinterpret_cast<float4*>(out), &scratch->counter,
                                                               &scratch->overflow);
        e = cudaGetLastError();
    }
    int overflow = 0;
    if (e == cudaSuccess) e = cudaMemcpyAsync(&overflow, &scratch->overflow, sizeof(int), cudaMemcpyDeviceToHost, st);
    cudaFreeAsync(scratch, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return cuda_error(e, shadow ? "srt_trace_shadow" : "srt_trace_closest");
    if (overflow) return set_error(SRT_ERR_STACK, "traversal stack overflow");
    return SRT_OK;
}

}  // namespace

extern "C" srt_status srt_trace_closest(const srt_scene* s, const float* rays, int64_t n, float* hits, void* stream)
{
    return run_query(s, rays, n, hits, false, stream);
}

extern "C" srt_status srt_trace_shadow(const srt_scene* s, const float* rays, int64_t n, int32_t* visible,
                                       void* stream)
{
    return run_query(s, rays, n, visible, true, stream);
}

extern "C" srt_status srt_scene_texture_lookup(const srt_scene* s, int32_t texture, const float* uv, int64_t n,
                                               float* out, void* stream)
{
    clear_error();
    if (!s || (n > 0 && (!uv || !out))) return set_error(SRT_ERR_ARG, "NULL argument");
    if (n < 0 || texture < 0 || texture >= (int32_t)s->tex_objects.size())
        return set_error(SRT_ERR_ARG, "bad texture index or count");
    if (reinterpret_cast<uintptr_t>(uv) % 8 || reinterpret_cast<uintptr_t>(out) % 16)
        return set_error(SRT_ERR_ARG, "uv must be 8-byte and out 16-byte aligned");
    if (n == 0) return SRT_OK;
    const int blocks = (int)std::min<int64_t>((n + 255) / 256, (int64_t)device_sm_count() * 8);
    k_texture_lookup<<<blocks, 256, 0, as_stream(stream)>>>(s->tex_objects[texture],
                                                                 reinterpret_cast<const float2*>(uv), n,
                                                                 reinterpret_cast<float4*>(out));
    SRT_CUDA_TRY(cudaGetLastError());
    return SRT_OK;
}
