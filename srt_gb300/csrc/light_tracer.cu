// light_tracer.cu — the LightTracer pass (src/passes/integrator/light_tracer.cu,
// src/shader/integrator/light_tracer.cu:57-175) on this library's BVH.
//
// Particle tracing from the area lights: each of the w*h launch indices
// runs `samples_per_pixel` light paths from its own curand stream
// (curand_init(seed + idx, 0, 0)); a path starts at a light sample with a
// cosine-distributed direction, and at every non-specular vertex it is
// connected to the pinhole camera through a shadow ray, splatting into the
// film pixel the connection lands on (atomic adds, as the reference does).
// One thread per launch index walks its paths with the single-ray
// traversal of trace.cuh (stack in shared memory): light paths do not
// share a camera-side structure worth a wavefront, and the pass is not a
// throughput path of the reference.
#include <cuda_runtime.h>

#include <algorithm>

#include "scene.h"
#include "shading.cuh"
#include "trace.cuh"

namespace srt {

namespace {

constexpr int kLtThreads = 128;

// Camera::get_xy (camera.h:142-148): film coordinates of the ray through the
// camera centre whose direction is `dir` reversed.  Like the reference, a
// point behind the camera is not rejected here.
__device__ __forceinline__ float2 camera_xy(const CameraRec& c, float3 dir)
{
    const float3 l = make_float3(dot(-dir, c.x), dot(-dir, c.y), dot(-dir, c.z));
    const float px = l.x / l.z, py = l.y / l.z;
    return make_float2(px / c.nw + 0.5f, py / c.nh + 0.5f);
}

__device__ __forceinline__ void splat(float4* film, int w, int h, float2 xy, float3 v)
{
    const int idx = (int)(xy.x * (float)w) + (int)(xy.y * (float)h) * w;
    atomicAdd(&film[idx].x, v.x);
    atomicAdd(&film[idx].y, v.y);
    atomicAdd(&film[idx].z, v.z);
}

__global__ void __launch_bounds__(kLtThreads) k_lt_clear(float4* film, int64_t n)
{
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride)
        film[i] = make_float4(0.0f, 0.0f, 0.0f, 1.0f);
}

struct LtArgs {
    int32_t w, h, spp, max_depth, rr_depth, seed;
    bool fixed;
};

__global__ void __launch_bounds__(kLtThreads) k_light_trace(SceneView S, CameraRec cam, LtArgs a, float4* film,
                                                            unsigned long long* counts, int* overflow_flag)
{
    __shared__ uint2 stack_mem[kStackEntries * kLtThreads];
    Stack st{stack_mem + threadIdx.x, kLtThreads, 0};
    int overflow = 0;
    unsigned long long n_closest = 0, n_shadow = 0;
    const int64_t n = (int64_t)a.w * a.h;
    const float aspect = (float)a.w / (float)a.h;
    const float inv_spp = 1.0f / (float)a.spp;
    for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < n;
         idx += (int64_t)gridDim.x * blockDim.x) {
        Rng rng;
        curand_init(pixel_seed(a.seed, (int32_t)idx), 0ull, 0ull, &rng.s);
        for (int i = 0; i < a.spp; ++i) {
            // light->sample(rng.random_float2()), then a cosine-distributed direction
            const float l1 = rng.next();
            const float l2 = rng.next();
            const LightSample ls = sample_light(S, l1, l2, a.fixed);
            const float s1 = rng.next();
            const float s2 = rng.next();
            const float sz = 1.0f - 2.0f * s1;  // uniform_sample_sphere (basic.h:83-89)
            const float sr = sqrtf(1.0f - sz * sz);
            const float phi = 2.0f * (float)M_PI * s2;
            const float3 wi = normalize(ls.normal + make_float3(sr * cosf(phi), sr * sinf(phi), sz));
            float3 ro = ls.pos, rd = wi;
            const float cos_theta = dot(wi, ls.normal);
            float pw = cos_theta * (float)M_1_PI;  // cosine_hemisphere_pdf
            float3 beta = ls.emission * cos_theta / ls.pdf;
            bool specular = true;
            for (int depth = 0; depth < a.max_depth; ++depth) {
                const Hit h = trace_closest(S, ro, rd, 1e-3f, 1e16f, st, overflow);
                ++n_closest;
                const bool hit = h.tri >= 0;
                if (hit) {
                    float3 base_color;
                    float4 em;
                    int mflags;
                    // get_hitinfo (hit_info.h:27-64), as the shading kernel computes it
                    const float4* tp = S.tris + 3 * (size_t)h.tri;
                    const float4 ta = __ldg(tp), tb = __ldg(tp + 1), tc = __ldg(tp + 2);
                    const float3 v0 = f3(ta), v1 = f3(tb), v2 = f3(tc);
                    const InstanceRec ir = S.insts[__float_as_int(ta.w)];
                    const Bxdf bx = unpack_bxdf(S.mats, ir.material, base_color, em, mflags);
                    const float3 pos = v0 * (1.0f - h.u - h.v) + v1 * h.u + v2 * h.v;
                    float3 ng = normalize(cross(v1 - v0, v2 - v0));
                    float3 sn = ng;
                    if (ir.attr & kAttrNormals) {
                        const float4* np = S.normals + 3 * (size_t)h.tri;
                        sn = normalize(f3(__ldg(np)) * (1.0f - h.u - h.v) + f3(__ldg(np + 1)) * h.u +
                                       f3(__ldg(np + 2)) * h.v);
                    }
                    if (mflags & kMatTextured)
                        apply_material_textures(S, ir.attr, ir.material, __float_as_int(ta.w), h.tri, h.u, h.v,
                                                base_color, em, sn);
                    if (dot(ng, sn) < 0.0f) ng = -ng;
                    float3 tan = (fabsf(sn.x) > fabsf(sn.y)) ? make_float3(0.f, 1.f, 0.f) : make_float3(1.f, 0.f, 0.f);
                    if (ir.attr & kAttrTangents) {
                        const float4* gp = S.tangents + 3 * (size_t)h.tri;
                        tan = f3(__ldg(gp)) * (1.0f - h.u - h.v) + f3(__ldg(gp + 1)) * h.u + f3(__ldg(gp + 2)) * h.v;
                    }
                    const Frame fr0 = Frame::from_normal_tangent(sn, tan);
                    // a specular segment that passes the camera centre (light_tracer.cu:97-110)
                    if (specular) {
                        float3 to_cam = cam.pos - ro;
                        const float t = length(to_cam);
                        to_cam = to_cam / t;
                        if (t < length(pos - ro) && dot(to_cam, rd) > 1.0f - 1e-6f) {
                            const float2 xy = camera_xy(cam, rd);
                            if (xy.x >= 0.0f && xy.x < 1.0f && xy.y >= 0.0f && xy.y < 1.0f)
                                splat(film, a.w, a.h, xy, beta / pw * inv_spp);
                        }
                    }
                    if (mflags & kMatEmissive) break;
                    float cos_i = dot(-rd, ng);
                    if (cos_i < 0.0f) ng = -ng;
                    // connection to the camera (light_tracer.cu:120-141)
                    if (!(mflags & kMatSpecular)) {
                        const float3 sd = normalize(cam.pos - pos);
                        const float2 xy = camera_xy(cam, sd);
                        if (xy.x >= 0.0f && xy.x < 1.0f && xy.y >= 0.0f && xy.y < 1.0f) {
                            const float t = length(cam.pos - pos);
                            ++n_shadow;
                            if (!trace_any(S, pos, sd, 1e-3f, t - 1e-3f, st, overflow)) {
                                const float3 fv = material_eval(bx, fr0, -rd, sd, base_color);
                                const float3 L = aspect * beta * fv * dot(sd, ng) / t / t / pw;
                                splat(film, a.w, a.h, xy, L * inv_spp);
                            }
                        }
                    }
                    // next direction (light_tracer.cu:143-153)
                    const float u1 = rng.next();
                    const float u2 = rng.next();
                    const BxdfSample ms = material_sample(bx, fr0, -rd, make_float2(u1, u2), base_color);
                    if (ms.pdf <= 1e-5f) break;
                    beta *= material_eval(bx, fr0, -rd, ms.wi, base_color) * fabsf(dot(ms.wi, ng)) / pw;
                    pw = ms.pdf;
                    specular = (mflags & kMatSpecular) != 0;
                    ro = pos;
                    rd = ms.wi;
                    // Russian roulette (light_tracer.cu:156-162)
                    if (depth >= a.rr_depth) {
                        const float p = fminf(fmaxf(beta.x, fmaxf(beta.y, beta.z)), 0.95f);
                        if (rng.next() > p) break;
                        beta /= p;
                    }
                } else {
                    if (specular) {
                        float3 to_cam = cam.pos - ro;
                        const float t = length(to_cam);
                        to_cam = to_cam / t;
                        if (dot(to_cam, rd) > 1.0f - 1e-6f) {
                            const float2 xy = camera_xy(cam, rd);
                            if (xy.x >= 0.0f && xy.x < 1.0f && xy.y >= 0.0f && xy.y < 1.0f)
                                splat(film, a.w, a.h, xy, beta / pw * inv_spp);
                        }
                    }
                    break;
                }
            }
        }
    }
    if (overflow) atomicExch(overflow_flag, 1);
    atomicAdd(counts, n_closest);
    atomicAdd(counts + 1, n_shadow);
}

}  // namespace

}  // namespace srt

using namespace srt;

extern "C" srt_status srt_lt_render(const srt_scene* s, int32_t width, int32_t height, float* film,
                                    const srt_pt_params* p, srt_pt_stats* stats, void* stream)
{
    clear_error();
    if (!s || !film || !p) return set_error(SRT_ERR_ARG, "NULL argument");
    if (width <= 0 || height <= 0 || p->samples_per_pixel < 0 || p->max_depth < 0)
        return set_error(SRT_ERR_ARG, "bad size or parameters");
    if (reinterpret_cast<uintptr_t>(film) % 16) return set_error(SRT_ERR_ARG, "film must be 16-byte aligned");
    if ((s->camera.type & 0xff) != SRT_CAMERA_PERSPECTIVE)
        return set_error(SRT_ERR_UNSUPPORTED, "the light tracer needs a perspective camera (Camera::get_xy)");
    cudaStream_t st = as_stream(stream);
    const int64_t n = (int64_t)width * height;
    float4* f4 = reinterpret_cast<float4*>(film);
    const int blocks = (int)std::min<int64_t>((n + kLtThreads - 1) / kLtThreads, (int64_t)device_sm_count() * 16);
    k_lt_clear<<<blocks, kLtThreads, 0, st>>>(f4, n);
    SRT_CUDA_TRY(cudaGetLastError());
    if (s->view.num_lights == 0 || p->samples_per_pixel == 0 || p->max_depth == 0) {
        if (stats) *stats = srt_pt_stats{};
        return SRT_OK;
    }
    struct Scratch {
        unsigned long long counts[2];
        int overflow;
        int pad;
    };
    Scratch* sc = nullptr;
    SRT_CUDA_TRY(cudaMallocAsync(reinterpret_cast<void**>(&sc), sizeof(Scratch), st));
    cudaError_t e = cudaMemsetAsync(sc, 0, sizeof(Scratch), st);
    LtArgs a{width, height, p->samples_per_pixel, p->max_depth, p->rr_depth, p->seed,
             (p->flags & SRT_PT_FIXED_CDF_REMAP) != 0};
    if (e == cudaSuccess) {
        k_light_trace<<<blocks, kLtThreads, 0, st>>>(s->view, s->camera, a, f4, sc->counts, &sc->overflow);
        e = cudaGetLastError();
    }
    Scratch host{};
    if (e == cudaSuccess) e = cudaMemcpyAsync(&host, sc, sizeof(Scratch), cudaMemcpyDeviceToHost, st);
    cudaFreeAsync(sc, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return cuda_error(e, "srt_lt_render");
    if (stats) {
        *stats = srt_pt_stats{};
        stats->samples = n * p->samples_per_pixel;
        stats->closest_rays = (int64_t)host.counts[0];
        stats->shadow_rays = (int64_t)host.counts[1];
        stats->stack_overflows = host.overflow;
        stats->kernel_launches = 2;
    }
    if (host.overflow) return set_error(SRT_ERR_STACK, "traversal stack overflow");
    return SRT_OK;
}
