// bxdf_batch.cu — GMaterial::sample / eval / sample_pdf over a batch of
// independent shading points (the Disney BRDF batch workload), plus the
// in-HBM generator of that workload's inputs.
#include "bxdf.h"
#include "common.h"

using namespace srt;

namespace {

__device__ __forceinline__ float3 ld3(const float* p, int64_t i)
{
    return make_float3(p[3 * i], p[3 * i + 1], p[3 * i + 2]);
}
__device__ __forceinline__ void st3(float* p, int64_t i, float3 v)
{
    p[3 * i] = v.x;
    p[3 * i + 1] = v.y;
    p[3 * i + 2] = v.z;
}
__device__ __forceinline__ Bxdf ld_bxdf(int type, const float* params, int64_t i)
{
    const float4* p = reinterpret_cast<const float4*>(params + 12 * i);
    float4 a = __ldg(p), b = __ldg(p + 1), c = __ldg(p + 2);
    return Bxdf{type, a.x, a.y, a.z, a.w, b.x, b.y, b.z, b.w, c.x, c.y, c.z, c.w};
}

__global__ void __launch_bounds__(256) k_bxdf_sample(srt_bxdf_batch B)
{
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < B.n; i += stride) {
        Frame fr = Frame::from_normal(ld3(B.normal, i));
        Bxdf b = ld_bxdf(B.type, B.params, i);
        float2 u = make_float2(B.rnd[2 * i], B.rnd[2 * i + 1]);
        BxdfSample s = material_sample(b, fr, ld3(B.wo, i), u, ld3(B.color, i));
        if (s.pdf == 0.0f && !s.delta) {
            s.f = f3(0.0f);
            s.wi = f3(0.0f);
        }
        st3(B.wi, i, s.wi);
        st3(B.f, i, s.f);
        B.pdf[i] = s.pdf;
        B.delta[i] = s.delta ? 1 : 0;
    }
}

__global__ void __launch_bounds__(256) k_bxdf_eval(srt_bxdf_batch B)
{
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < B.n; i += stride) {
        Frame fr = Frame::from_normal(ld3(B.normal, i));
        Bxdf b = ld_bxdf(B.type, B.params, i);
        float3 wi = ld3(B.wi, i), wo = ld3(B.wo, i), c = ld3(B.color, i);
        st3(B.f, i, material_eval(b, fr, wi, wo, c));
        B.pdf[i] = material_pdf(b, fr, wi, wo, c);
    }
}

// PCG32 (O'Neill, pcg-random.org minimal C generator).
struct Pcg32 {
    uint64_t state, inc;
    __device__ uint32_t next()
    {
        uint64_t old = state;
        state = old * 6364136223846793005ULL + inc;
        uint32_t xs = (uint32_t)(((old >> 18u) ^ old) >> 27u);
        uint32_t rot = (uint32_t)(old >> 59u);
        return (xs >> rot) | (xs << ((32u - rot) & 31u));
    }
    __device__ void seed(uint64_t initstate, uint64_t initseq)
    {
        state = 0u;
        inc = (initseq << 1u) | 1u;
        next();
        state += initstate;
        next();
    }
    __device__ float uniform() { return (float)(next() >> 8) * (1.0f / 16777216.0f); }
};

// Point i draws 21 uniforms from PCG32(initstate = i, initseq = 0): normal
// on the sphere (2), wo on the hemisphere about it (2), colour (3), metallic,
// subsurface, specular, specularTint, anisotropic, sheen, sheenTint,
// clearcoat, clearcoatGloss (9), roughness in [0.05, 1) (1), rnd (4; the
// first two feed sample()).  ior = 1.5, specTrans = 0.
__global__ void __launch_bounds__(256) k_bxdf_generate(int64_t first, srt_bxdf_batch B)
{
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < B.n; i += stride) {
        Pcg32 g;
        g.seed((uint64_t)(first + i), 0u);
        float u[21];
#pragma unroll
        for (int j = 0; j < 21; ++j) u[j] = g.uniform();
        float z = 1.0f - 2.0f * u[0];
        float r = sqrtf(fmaxf(0.0f, 1.0f - z * z));
        float s, c;
        sincosf((2.0f * SRT_PI) * u[1], &s, &c);
        float3 n = make_float3(r * c, r * s, z);
        float hz = u[2];
        float hr = sqrtf(fmaxf(0.0f, 1.0f - hz * hz));
        sincosf((2.0f * SRT_PI) * u[3], &s, &c);
        Frame fr = Frame::from_normal(n);
        float3 wo = fr.to_world(make_float3(hr * c, hr * s, hz));
        // the generator fills the batch's input arrays
        st3(const_cast<float*>(B.normal), i, n);
        st3(const_cast<float*>(B.wo), i, wo);
        st3(const_cast<float*>(B.color), i, make_float3(u[4], u[5], u[6]));
        float4* p = reinterpret_cast<float4*>(const_cast<float*>(B.params) + 12 * i);
        p[0] = make_float4(1.5f, u[7], u[8], 0.05f + 0.95f * u[16]);
        p[1] = make_float4(u[9], u[10], u[11], u[12]);
        p[2] = make_float4(u[13], u[14], u[15], 0.0f);
        float* rnd = const_cast<float*>(B.rnd);
        rnd[2 * i] = u[17];
        rnd[2 * i + 1] = u[18];
    }
}

srt_status check_batch(const srt_bxdf_batch* b, bool need_out)
{
    if (!b) return set_error(SRT_ERR_ARG, "batch is NULL");
    if (b->n < 0) return set_error(SRT_ERR_ARG, "negative batch size");
    if (b->type < SRT_BXDF_DIFFUSE || b->type > SRT_BXDF_DISNEY) return set_error(SRT_ERR_ARG, "unknown bxdf type");
    if (b->n == 0) return SRT_OK;
    if (!b->normal || !b->wo || !b->color || !b->params || !b->rnd || !b->wi || !b->f || !b->pdf ||
        (need_out && !b->delta))
        return set_error(SRT_ERR_ARG, "NULL array in batch");
    if (reinterpret_cast<uintptr_t>(b->params) % 16 != 0)
        return set_error(SRT_ERR_ARG, "params must be 16-byte aligned");
    return SRT_OK;
}

int grid_for(int64_t n)
{
    int64_t blocks = (n + 255) / 256;
    int64_t cap = (int64_t)device_sm_count() * 8;
    return (int)std::max<int64_t>(1, std::min(blocks, cap));
}

}  // namespace

extern "C" srt_status srt_bxdf_sample(const srt_bxdf_batch* b, void* stream)
{
    clear_error();
    SRT_TRY(check_batch(b, true));
    if (b->n == 0) return SRT_OK;
    k_bxdf_sample<<<grid_for(b->n), 256, 0, as_stream(stream)>>>(*b);
    SRT_CUDA_TRY(cudaGetLastError());
    return SRT_OK;
}

extern "C" srt_status srt_bxdf_eval(const srt_bxdf_batch* b, void* stream)
{
    clear_error();
    SRT_TRY(check_batch(b, false));
    if (b->n == 0) return SRT_OK;
    k_bxdf_eval<<<grid_for(b->n), 256, 0, as_stream(stream)>>>(*b);
    SRT_CUDA_TRY(cudaGetLastError());
    return SRT_OK;
}

extern "C" srt_status srt_bxdf_generate(int64_t first, const srt_bxdf_batch* b, void* stream)
{
    clear_error();
    SRT_TRY(check_batch(b, false));
    if (first < 0) return set_error(SRT_ERR_ARG, "negative first index");
    if (b->n == 0) return SRT_OK;
    k_bxdf_generate<<<grid_for(b->n), 256, 0, as_stream(stream)>>>(first, *b);
    SRT_CUDA_TRY(cudaGetLastError());
    return SRT_OK;
}
