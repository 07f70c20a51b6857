// vmath.h — small float3 algebra for host and device code of the tracer.
//
// Semantics follow the reference's vector helpers where results must match:
// lerp(a, b, t) = a + t * (b - a), clamp(f, lo, hi) = max(lo, min(f, hi)),
// normalize(v) = v * (1 / sqrt(dot(v, v))).
#pragma once

#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#if defined(__CUDACC__)
#define SRT_HD __host__ __device__ __forceinline__
#else
#define SRT_HD inline
#endif

#define SRT_PI 3.14159265358979323846f
#define SRT_INV_PI 0.318309886183790671538f

namespace srt {

SRT_HD float3 f3(float a) { return make_float3(a, a, a); }
SRT_HD float3 f3(float x, float y, float z) { return make_float3(x, y, z); }
SRT_HD float3 f3(float4 v) { return make_float3(v.x, v.y, v.z); }

SRT_HD float3 operator+(float3 a, float3 b) { return make_float3(a.x + b.x, a.y + b.y, a.z + b.z); }
SRT_HD float3 operator-(float3 a, float3 b) { return make_float3(a.x - b.x, a.y - b.y, a.z - b.z); }
SRT_HD float3 operator-(float3 a) { return make_float3(-a.x, -a.y, -a.z); }
SRT_HD float3 operator*(float3 a, float3 b) { return make_float3(a.x * b.x, a.y * b.y, a.z * b.z); }
SRT_HD float3 operator*(float3 a, float s) { return make_float3(a.x * s, a.y * s, a.z * s); }
SRT_HD float3 operator*(float s, float3 a) { return make_float3(a.x * s, a.y * s, a.z * s); }
SRT_HD float3 operator/(float3 a, float3 b) { return make_float3(a.x / b.x, a.y / b.y, a.z / b.z); }
SRT_HD float3 operator/(float3 a, float s) { return make_float3(a.x / s, a.y / s, a.z / s); }
SRT_HD void operator+=(float3& a, float3 b) { a.x += b.x; a.y += b.y; a.z += b.z; }
SRT_HD void operator*=(float3& a, float3 b) { a.x *= b.x; a.y *= b.y; a.z *= b.z; }
SRT_HD void operator*=(float3& a, float s) { a.x *= s; a.y *= s; a.z *= s; }
SRT_HD void operator/=(float3& a, float s) { a.x /= s; a.y /= s; a.z /= s; }

SRT_HD float dot(float3 a, float3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
SRT_HD float3 cross(float3 a, float3 b)
{
    return make_float3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
// correctly rounded 1/sqrt(x) (IEEE sqrt and division on host and device)
SRT_HD float rsqrt_(float x) { return 1.0f / sqrtf(x); }
SRT_HD float3 normalize(float3 v) { return v * rsqrt_(dot(v, v)); }
SRT_HD float length(float3 v) { return sqrtf(dot(v, v)); }
SRT_HD float lerp(float a, float b, float t) { return a + t * (b - a); }
SRT_HD float3 lerp(float3 a, float3 b, float t) { return a + t * (b - a); }
SRT_HD float clampf(float f, float lo, float hi) { return fmaxf(lo, fminf(f, hi)); }
SRT_HD float max3(float3 v) { return fmaxf(v.x, fmaxf(v.y, v.z)); }
SRT_HD float luminance(float3 c) { return dot(c, make_float3(0.2126f, 0.7152f, 0.0722f)); }
SRT_HD float3 reflect(float3 i, float3 n) { return i - 2.0f * n * dot(n, i); }
SRT_HD bool finite3(float3 v) { return isfinite(v.x) && isfinite(v.y) && isfinite(v.z); }

// Orthonormal frame: z is the (shading) normal.  Built like Onb(n) and
// Onb(n, t) of the reference (src/device_include/math/onb.h:11-23).
struct Frame {
    float3 z, x, y;

    SRT_HD static Frame from_normal(float3 n)
    {
        Frame f;
        f.z = n;
        float3 t = (fabsf(n.x) > fabsf(n.y)) ? make_float3(0.f, 1.f, 0.f) : make_float3(1.f, 0.f, 0.f);
        f.x = normalize(cross(t, n));
        f.y = cross(n, f.x);
        return f;
    }
    SRT_HD static Frame from_normal_tangent(float3 n, float3 t)
    {
        Frame f;
        f.z = n;
        f.x = normalize(t - n * dot(t, n));
        f.y = cross(n, f.x);
        return f;
    }
    SRT_HD float3 to_local(float3 v) const { return make_float3(dot(v, x), dot(v, y), dot(v, z)); }
    SRT_HD float3 to_world(float3 v) const { return v.x * x + v.y * y + v.z * z; }
};

}  // namespace srt
