// shading.cuh — device pieces the camera-path (wavefront.cu) and the
// light-path (light_tracer.cu) kernels share: the per-pixel curand stream,
// camera rays, light sampling, material unpacking and texture lookups.
#pragma once

#include <curand_kernel.h>

#include "bxdf.h"
#include "device_types.h"
#include "vmath.h"

namespace srt {

namespace {

// ---------------------------------------------------------------------------
// RNG: the reference's per-pixel curand XORWOW stream (random.h:14-31).
// Only the generator words (d, v[5]) are carried; the Box-Muller fields are
// unused by curand_uniform.
// ---------------------------------------------------------------------------
struct Rng {
    curandStateXORWOW s;
    __device__ __forceinline__ void load(uint4 a, uint2 b)
    {
        s.v[0] = a.x;
        s.v[1] = a.y;
        s.v[2] = a.z;
        s.v[3] = a.w;
        s.v[4] = b.x;
        s.d = b.y;
        s.boxmuller_flag = 0;
        s.boxmuller_flag_double = 0;
        s.boxmuller_extra = 0.0f;
        s.boxmuller_extra_double = 0.0;
    }
    __device__ __forceinline__ void store(uint4& a, uint2& b) const
    {
        a = make_uint4(s.v[0], s.v[1], s.v[2], s.v[3]);
        b = make_uint2(s.v[4], s.d);
    }
    __device__ __forceinline__ float next() { return 1.0f - curand_uniform(&s); }
};

__device__ __forceinline__ unsigned long long pixel_seed(int32_t seed, int32_t idx)
{
    // `params.seed + idx` is an int sum widened to unsigned long long (path_tracer.cu:56)
    int32_t si = (int32_t)((uint32_t)seed + (uint32_t)idx);
    return (unsigned long long)(long long)si;
}

// Camera::get_ray, perspective / orthographic (camera.h:107-122).
__device__ __forceinline__ void camera_ray(const CameraRec& c, float x, float y, float3& o, float3& d)
{
    float px = (x - 0.5f) * c.nw, py = (y - 0.5f) * c.nh;
    if (c.type == SRT_CAMERA_ORTHOGRAPHIC) {
        float3 lo = make_float3(px * c.radius, py * c.radius, 1.0f);
        o = lo.x * c.x + lo.y * c.y + lo.z * c.z + c.pos;
        d = 0.0f * c.x + 0.0f * c.y + 1.0f * c.z;
    } else {
        float3 ld = normalize(make_float3(px, py, 1.0f));
        o = c.pos;
        d = ld.x * c.x + ld.y * c.y + ld.z * c.z;
    }
}

__device__ __forceinline__ int cdf_search(const float* __restrict__ cdf, int num, float x)
{
    int lf = 0, rg = num - 1;
    while (lf <= rg) {
        int mid = (lf + rg) >> 1;
        if (__ldg(cdf + mid) <= x)
            lf = mid + 1;
        else
            rg = mid - 1;
    }
    return min(rg + 1, num - 1);
}

// The reference keeps cdf[idx-1] in an int (light.h:65, gmesh.h:49).
__device__ __forceinline__ float cdf_remap(const float* __restrict__ cdf, int idx, float u, bool fixed)
{
    if (fixed) {
        float lower = (idx == 0) ? 0.0f : __ldg(cdf + idx - 1);
        return (u - lower) / (__ldg(cdf + idx) - lower);
    }
    int lower = (idx == 0) ? 0 : (int)__ldg(cdf + idx - 1);
    return (u - (float)lower) / (__ldg(cdf + idx) - (float)lower);
}

struct LightSample {
    float3 pos, normal, emission;
    float pdf;
};

// texture coordinate of a hit (hit_info.h:36-38): the mesh's interpolated
// texcoords, or the barycentric (u, v) when it has none
__device__ __forceinline__ float2 hit_texcoord(const SceneView& S, int32_t attr, size_t tri, float u, float v)
{
    if (!(attr & kAttrTexcoords)) return make_float2(u, v);
    const float2* t = S.texcoords + 3 * tri;
    const float2 a = __ldg(t), b = __ldg(t + 1), c = __ldg(t + 2);
    const float w = 1.0f - u - v;
    return make_float2(a.x * w + b.x * u + c.x * v, a.y * w + b.y * u + c.y * v);
}

// EnvironmentLight::emission (light.h:27-41) of a "uvmap" environment: the
// texture looked up by direction (world y up, math-space z up).
__device__ __forceinline__ float3 env_map_radiance(unsigned long long tex, float3 d)
{
    const float3 m = make_float3(-d.x, d.z, d.y);
    const float phi = atan2f(m.y, m.x), theta = acosf(m.z);  // cartesian_to_spherical_uv (basic.h:41-46)
    const float u = phi * 0.5f * (float)M_1_PI + 0.5f, v = theta * (float)M_1_PI;
    return f3(tex2D<float4>(tex, u, v));
}

__device__ __forceinline__ float3 env_radiance(const SceneView& S, float3 d)
{
    return S.env_tex ? env_map_radiance(S.env_tex, d) : S.env;
}

// GMaterial::surface_color / emission / shading_normal (gmaterial.h:35-56)
// at a hit's texture coordinate: the colour texture replaces the base
// colour (and the emission colour), the normal map's object-space normal,
// turned by the instance (apply_onb), replaces the shading normal.
__device__ __forceinline__ void apply_material_textures(const SceneView& S, int32_t attr, int32_t material, int32_t inst,
                                                     int tri, float u, float v, float3& base_color, float4& em,
                                                     float3& sn)
{
    const float2 tc = hit_texcoord(S, attr, (size_t)tri, u, v);
    const unsigned long long ctex = __ldg(S.mat_tex + 2 * material);
    const unsigned long long ntex = __ldg(S.mat_tex + 2 * material + 1);
    if (ctex) {
        base_color = f3(tex2D<float4>(ctex, tc.x, tc.y));
        em = make_float4(base_color.x * em.w, base_color.y * em.w, base_color.z * em.w, em.w);
    }
    if (ntex) {
        const float3 no = normalize(f3(tex2D<float4>(ntex, tc.x, tc.y)));
        const float4* xr = S.inst_xf + 3 * (size_t)inst;
        const float4 r0 = __ldg(xr), r1 = __ldg(xr + 1), r2 = __ldg(xr + 2);
        sn = make_float3(r0.x * no.x + r0.y * no.y + r0.z * no.z, r1.x * no.x + r1.y * no.y + r1.z * no.z,
                         r2.x * no.x + r2.y * no.y + r2.z * no.z);
    }
}

// GMaterial::emission(texcoord) (gmaterial.h:35-41) of a light sample: the
// colour texture times the intensity
__device__ __forceinline__ float3 light_texture_emission(const SceneView& S, int32_t attr, int32_t material, int32_t t,
                                                      float bu, float bv, float intensity)
{
    const float2 tc = hit_texcoord(S, attr, (size_t)t, bu, bv);
    return f3(tex2D<float4>(__ldg(S.mat_tex + 2 * material), tc.x, tc.y)) * intensity;
}

// Light::sample + GInstance::sample (light.h:61-76, gmesh.h:45-85).
__device__ __forceinline__ LightSample sample_light(const SceneView& S, float u1, float u2, bool fixed)
{
    int li = cdf_search(S.light_cdf, S.num_lights, u1);
    u1 = cdf_remap(S.light_cdf, li, u1, fixed);
    LightRec L = S.lights[li];
    const float* fcdf = S.face_cdf + L.face_begin;
    int fi = cdf_search(fcdf, L.num_faces, u1);
    u1 = cdf_remap(fcdf, fi, u1, fixed);
    float sx = sqrtf(u1);
    float bu = 1.0f - sx, bv = u2 * sx;  // uniform_sample_triangle (basic.h:139-143)
    int32_t t = __ldg(S.light_tri + L.face_begin + fi);
    const float4* tp = S.tris + 3 * (size_t)t;
    float4 a = __ldg(tp), b = __ldg(tp + 1), c = __ldg(tp + 2);
    float3 v0 = f3(a), v1 = f3(b), v2 = f3(c);
    LightSample ls;
    ls.pos = v0 * (1.0f - bu - bv) + v1 * bu + v2 * bv;
    float3 n = normalize(cross(v1 - v0, v2 - v0));
    int32_t inst = __float_as_int(a.w);
    InstanceRec ir = S.insts[inst];
    if (ir.attr & kAttrNormals) {
        const float4* np = S.normals + 3 * (size_t)t;
        float3 sn = f3(__ldg(np)) * (1.0f - bu - bv) + f3(__ldg(np + 1)) * bu + f3(__ldg(np + 2)) * bv;
        if (dot(n, sn) < 0.0f) n = -n;
    }
    ls.normal = n;
    float4 em = __ldg(&S.mats[ir.material].m[4]);
    ls.emission = f3(em);
    if (L.textured) ls.emission = light_texture_emission(S, ir.attr, ir.material, t, bu, bv, em.w);
    ls.pdf = L.pdf;
    return ls;
}

__device__ __forceinline__ Bxdf unpack_bxdf(const MaterialRec* __restrict__ m, int id, float3& base, float4& em,
                                            int& mflags)
{
    const float4* p = &m[id].m[0];
    float4 a = __ldg(p), b = __ldg(p + 1), c = __ldg(p + 2), d = __ldg(p + 3);
    em = __ldg(p + 4);
    base = f3(a);
    mflags = __float_as_int(a.w);
    return Bxdf{mflags & 0xff, b.x, b.y, b.z, b.w, c.x, c.y, c.z, c.w, d.x, d.y, d.z, d.w};
}

constexpr int kMatSpecular = 1 << 8;
constexpr int kMatTransmissive = 1 << 9;
constexpr int kMatEmissive = 1 << 10;
constexpr int kMatTextured = 1 << 11;

}  // namespace

}  // namespace srt
