// bxdf.h — Lambert / diffuse-transmission / thin-dielectric / Disney BxDF in
// FP32, evaluated in the local shading frame (z = shading normal).
//
// Follows the formulas of the reference BxDF (src/device_include/scene/bxdf.h:79-387)
// and its helpers (src/device_include/math/basic.h:103-258): the same lobe
// weights, gates, samplers and mixture pdf, so that values and pdfs agree
// with an FP64 evaluation of those formulas.  Unlike the reference, the
// lobe set-up shared by sample() and pdf() (both use the Fresnel mix at
// wo.z) is computed once per shading point (DisneyLobes) and reused for the
// BSDF sample and the NEE pdf of the same vertex.
#pragma once

#include "vmath.h"

namespace srt {

enum BxdfType : int { BXDF_DIFFUSE = 0, BXDF_DIFFUSE_TRANSMISSION = 1, BXDF_DIELECTRIC = 2, BXDF_DISNEY = 3 };

struct Bxdf {
    int type;
    float ior, metallic, subsurface, roughness, specular, specularTint,
          anisotropic, sheen, sheenTint, clearcoat, clearcoatGloss, specTrans;
};

struct BxdfSample {
    float3 f;
    float3 wi;
    float pdf;
    bool delta;
};

// ---- scalar helpers (basic.h:147-201) --------------------------------------

SRT_HD float schlick(float cos_theta, float eta)
{
    float r0 = (eta - 1.0f) / (eta + 1.0f);
    r0 = r0 * r0;
    float m = clampf(1.0f - cos_theta, 0.0f, 1.0f);
    float m2 = m * m;
    return r0 + (1.0f - r0) * (m2 * m2 * m);
}
SRT_HD float schlick1(float cos_theta)
{
    float m = clampf(1.0f - cos_theta, 0.0f, 1.0f);
    float m2 = m * m;
    return m2 * m2 * m;
}
SRT_HD float fresnel_mix(float metallic, float eta, float c)
{
    return lerp(schlick(c, eta), schlick1(c), metallic);
}
SRT_HD float gtr1(float nh, float a)
{
    if (a >= 1.0f) return SRT_INV_PI;
    float a2 = a * a;
    float t = 1.0f + (a2 - 1.0f) * nh * nh;
    return (a2 - 1.0f) * SRT_INV_PI / (logf(a2) * t);
}
SRT_HD float gtr2(float nh, float a)
{
    float a2 = a * a;
    float t = 1.0f + (a2 - 1.0f) * nh * nh;
    return a2 * SRT_INV_PI / (t * t);
}
SRT_HD float gtr2_aniso(float nh, float hx, float hy, float ax, float ay)
{
    float a = hx / ax, b = hy / ay;
    float t = a * a + b * b + nh * nh;
    return SRT_INV_PI / (ax * ay * t * t);
}
SRT_HD float smith_ggx(float nv, float alpha)
{
    float a = alpha * alpha;
    float b = nv * nv;
    return (2.0f * nv) / (nv + sqrtf(a + b - a * b));
}

// ---- direction samplers (basic.h:103-258) ----------------------------------

SRT_HD float3 cosine_hemisphere(float2 u)
{
    float ox = 2.0f * u.x - 1.0f, oy = 2.0f * u.y - 1.0f;
    float dx = 0.0f, dy = 0.0f;
    if (!(ox == 0.0f && oy == 0.0f)) {
        float r, theta;
        if (fabsf(ox) > fabsf(oy)) {
            r = ox;
            theta = (0.25f * SRT_PI) * (oy / ox);
        } else {
            r = oy;
            theta = (0.5f * SRT_PI) - (0.25f * SRT_PI) * (ox / oy);
        }
        float s, c;
        sincosf(theta, &s, &c);
        dx = r * c;
        dy = r * s;
    }
    return make_float3(dx, dy, sqrtf(fmaxf(0.0f, 1.0f - dx * dx - dy * dy)));
}

SRT_HD float3 sample_gtr1_h(float a, float2 u)
{
    if (a >= 1.0f) return cosine_hemisphere(u);
    float a2 = a * a;
    float phi = (2.0f * SRT_PI) * u.x;
    float cos_t = sqrtf((1.0f - powf(a2, 1.0f - u.y)) / (1.0f - a2));
    float sin_t = clampf(sqrtf(1.0f - cos_t * cos_t), 0.0f, 1.0f);
    float s, c;
    sincosf(phi, &s, &c);
    return make_float3(c * sin_t, s * sin_t, cos_t);
}

SRT_HD float3 sample_gtr2_aniso_h(float ax, float ay, float2 u)
{
    float phi = (2.0f * SRT_PI) * u.x;
    float s, c;
    sincosf(phi, &s, &c);
    float tan_t = sqrtf(u.y / (1.0f - u.y));
    return normalize(make_float3(tan_t * (ax * c), tan_t * (ay * s), 1.0f));
}

SRT_HD float3 sample_ggx_vndf_h(float3 V, float a, float2 u)
{
    float3 vh = normalize(make_float3(a * V.x, a * V.y, V.z));
    float lensq = vh.x * vh.x + vh.y * vh.y;
    float3 t1v = (lensq > 0.0f) ? make_float3(-vh.y, vh.x, 0.0f) * rsqrt_(lensq) : make_float3(1.0f, 0.0f, 0.0f);
    float3 t2v = cross(vh, t1v);
    float r = sqrtf(u.x);
    float phi = (2.0f * SRT_PI) * u.y;
    float s, c;
    sincosf(phi, &s, &c);
    float t1 = r * c;
    float t2 = r * s;
    float sv = 0.5f * (1.0f + vh.z);
    t2 = (1.0f - sv) * sqrtf(1.0f - t1 * t1) + sv * t2;
    float3 nh = t1 * t1v + t2 * t2v + sqrtf(fmaxf(0.0f, 1.0f - t1 * t1 - t2 * t2)) * vh;
    return normalize(make_float3(a * nh.x, a * nh.y, fmaxf(0.0f, nh.z)));
}

SRT_HD float3 refract_dir(float3 i, float3 n, float eta)
{
    float ni = dot(n, -i);
    float k = 1.0f - eta * eta * (1.0f - ni * ni);
    if (k < 0.0f) return make_float3(0.0f, 0.0f, 0.0f);
    return eta * i + (eta * ni - sqrtf(k)) * n;
}

// ---- Disney ----------------------------------------------------------------

// Colour terms and roughness shape that do not depend on directions.
struct DisneyColors {
    float lum;
    float3 spec_color;
    float3 sheen_color;
    float ax, ay;
};

SRT_HD DisneyColors disney_colors(const Bxdf& b, float3 color)
{
    DisneyColors d;
    d.lum = luminance(color);
    float3 ctint = (d.lum > 0.0f) ? color / d.lum : f3(1.0f);
    d.spec_color = lerp(b.specular * 0.08f * lerp(f3(1.0f), ctint, b.specularTint), color, b.metallic);
    d.sheen_color = lerp(f3(1.0f), ctint, b.sheenTint);
    float aspect = sqrtf(1.0f - b.anisotropic * 0.9f);
    float a2 = b.roughness * b.roughness;
    d.ax = fmaxf(0.001f, a2 / aspect);
    d.ay = fmaxf(0.001f, a2 * aspect);
    return d;
}

// Normalised lobe-selection weights with the Fresnel mix at wo.z
// (bxdf.h:242-252 and :353-363).
struct DisneyLobes {
    float dw, srw, stw, ccw;
};

SRT_HD DisneyLobes disney_lobes(const Bxdf& b, const DisneyColors& d, float eta, float vz)
{
    float fm = fresnel_mix(b.metallic, eta, vz);
    DisneyLobes w;
    w.dw = d.lum * (1.0f - b.metallic) * (1.0f - b.specTrans);
    w.srw = luminance(lerp(d.spec_color, f3(1.0f), fm));
    w.stw = (1.0f - fm) * (1.0f - b.metallic) * b.specTrans * d.lum;
    w.ccw = b.clearcoat * (1.0f - b.metallic);
    float total = w.dw + w.srw + w.stw + w.ccw;
    w.dw /= total;
    w.srw /= total;
    w.stw /= total;
    w.ccw /= total;
    return w;
}

SRT_HD float3 disney_eval(const Bxdf& b, const DisneyColors& d, float3 L, float3 V, float3 color, float eta)
{
    float3 H = (L.z > 0.0f) ? normalize(L + V) : normalize(L + V * eta);
    if (H.z <= 0.0f) H = -H;
    float vh = dot(V, H), lh = dot(L, H);

    // gates use the Fresnel mix at dot(V, H) (bxdf.h:108-112)
    float fm = fresnel_mix(b.metallic, eta, vh);
    float one_m = 1.0f - b.metallic;
    float diffuse_w = d.lum * one_m * (1.0f - b.specTrans);
    float spec_reflect_w = luminance(lerp(d.spec_color, f3(1.0f), fm));
    float spec_refract_w = (1.0f - fm) * one_m * b.specTrans * d.lum;
    float clearcoat_w = b.clearcoat * one_m;

    float3 f = f3(0.0f);
    if (diffuse_w > 0.0f && L.z > 0.0f) {
        float fl = schlick1(L.z), fv = schlick1(V.z), fh = schlick1(lh);
        float fd90 = 0.5f + 2.0f * lh * lh * b.roughness;
        float fd = lerp(1.0f, fd90, fl) * lerp(1.0f, fd90, fv);
        float fss90 = lh * lh * b.roughness;
        float fss = lerp(1.0f, fss90, fl) * lerp(1.0f, fss90, fv);
        float ss = 1.25f * (fss * (1.0f / (L.z + V.z) - 0.5f) + 0.5f);
        float3 fsheen = fh * b.sheen * d.sheen_color;
        f += (SRT_INV_PI * lerp(fd, ss, b.subsurface) * color + fsheen) * one_m * (1.0f - b.specTrans);
    }
    if (spec_reflect_w > 0.0f && L.z > 0.0f && V.z > 0.0f) {
        float fm_l = fresnel_mix(b.metallic, eta, lh);
        float3 F = lerp(d.spec_color, f3(1.0f), fm_l);
        float D = gtr2_aniso(H.z, H.x, H.y, d.ax, d.ay);
        float G = smith_ggx(fabsf(L.z), b.roughness) * smith_ggx(fabsf(V.z), b.roughness);
        f += F * D * G / (4.0f * L.z * V.z);
    }
    if (spec_refract_w > 0.0f && L.z < 0.0f) {
        float F = schlick(fabsf(vh), eta);
        float D = gtr2(H.z, b.roughness);
        float den = (lh + vh * eta) * (lh + vh * eta);
        float G = smith_ggx(fabsf(L.z), b.roughness) * smith_ggx(fabsf(V.z), b.roughness) *
                  fabsf(lh) * fabsf(vh) * eta * eta / den;
        float3 rc = make_float3(sqrtf(color.x), sqrtf(color.y), sqrtf(color.z));
        f += rc * one_m * b.specTrans * (1.0f - F) * D * G / (fabsf(L.z) * fabsf(V.z));
    }
    if (clearcoat_w > 0.0f && L.z > 0.0f && V.z > 0.0f) {
        float fh = schlick(lh, 1.0f / 1.5f);
        float F = lerp(0.04f, 1.0f, fh);
        float D = gtr1(H.z, b.clearcoatGloss);
        float G = smith_ggx(L.z, 0.25f) * smith_ggx(V.z, 0.25f);
        f += f3(0.25f * b.clearcoat * F * D * G / (4.0f * L.z * V.z));
    }
    return f;
}

// Mixture pdf of the four lobes at L (bxdf.h:289-310, :365-380).
SRT_HD float disney_pdf(const Bxdf& b, const DisneyColors& d, const DisneyLobes& w, float3 L, float3 V, float eta)
{
    float3 hr = normalize(L + V);
    if (hr.z < 0.0f) hr = -hr;
    float3 ht = normalize(L + V * eta);
    if (ht.z < 0.0f) ht = -ht;
    float vhr = dot(V, hr);

    float pdf = 0.0f;
    if (w.dw > 0.0f && L.z > 0.0f) pdf += w.dw * (L.z * SRT_INV_PI);
    if (w.srw > 0.0f && vhr > 0.0f)
        pdf += w.srw * gtr2_aniso(hr.z, hr.x, hr.y, d.ax, d.ay) * hr.z / (4.0f * vhr);
    float vht = dot(V, ht), lht = dot(L, ht);
    if (w.stw > 0.0f && vht > 0.0f && lht < 0.0f) {
        float den = lht + vht * eta;
        pdf += w.stw * gtr2(ht.z, b.roughness) * smith_ggx(V.z, b.roughness) * fmaxf(vht, 0.0f) / V.z *
               fabsf(lht) / (den * den);
    }
    if (w.ccw > 0.0f && vhr > 0.0f) pdf += w.ccw * gtr1(hr.z, b.clearcoatGloss) * hr.z / (4.0f * vhr);
    return pdf;
}

// ---- generic BxDF interface (local frame; V.z > 0 guaranteed by caller) ----

SRT_HD float3 bxdf_eval(const Bxdf& b, float3 L, float3 V, float3 color, bool inner)
{
    switch (b.type) {
    case BXDF_DIFFUSE: return (L.z <= 0.0f) ? f3(0.0f) : color * SRT_INV_PI;
    case BXDF_DIFFUSE_TRANSMISSION: return color * SRT_INV_PI;
    case BXDF_DISNEY: {
        float eta = inner ? b.ior : 1.0f / b.ior;
        DisneyColors d = disney_colors(b, color);
        return disney_eval(b, d, L, V, color, eta);
    }
    default: return f3(0.0f);
    }
}

SRT_HD float bxdf_pdf(const Bxdf& b, float3 L, float3 V, float3 color, bool inner)
{
    switch (b.type) {
    case BXDF_DIFFUSE: return (L.z <= 0.0f) ? 0.0f : L.z * SRT_INV_PI;
    case BXDF_DIFFUSE_TRANSMISSION: return 0.5f * (fabsf(L.z) * SRT_INV_PI);
    case BXDF_DISNEY: {
        float eta = inner ? b.ior : 1.0f / b.ior;
        DisneyColors d = disney_colors(b, color);
        DisneyLobes w = disney_lobes(b, d, eta, V.z);
        return disney_pdf(b, d, w, L, V, eta);
    }
    default: return 0.0f;
    }
}

SRT_HD BxdfSample bxdf_none()
{
    BxdfSample s;
    s.f = f3(0.0f);
    s.wi = f3(0.0f);
    s.pdf = 0.0f;
    s.delta = false;
    return s;
}

SRT_HD BxdfSample bxdf_sample(const Bxdf& b, float3 V, float2 u, float3 color, bool inner)
{
    BxdfSample s = bxdf_none();
    switch (b.type) {
    case BXDF_DIFFUSE: {
        float3 wi = cosine_hemisphere(u);
        s.f = bxdf_eval(b, wi, V, color, inner);
        s.wi = wi;
        s.pdf = wi.z * SRT_INV_PI;
        return s;
    }
    case BXDF_DIFFUSE_TRANSMISSION: {
        bool front = u.x < 0.5f;
        u.x = front ? u.x * 2.0f : (u.x - 0.5f) * 2.0f;
        float3 wi = cosine_hemisphere(u);
        float pdf = wi.z * SRT_INV_PI;
        if (!front) wi = -wi;
        s.f = bxdf_eval(b, wi, V, color, inner);
        s.wi = wi;
        s.pdf = 0.5f * pdf;
        return s;
    }
    case BXDF_DIELECTRIC: {
        float eta = inner ? b.ior : 1.0f / b.ior;
        float3 n = make_float3(0.0f, 0.0f, 1.0f);
        float3 wi = refract_dir(-V, n, eta);
        float rr = (dot(wi, wi) == 0.0f) ? 1.0f : schlick(V.z, eta);
        if (u.x <= rr) wi = reflect(-V, n);
        s.f = color;
        s.wi = normalize(wi);
        s.pdf = 1.0f;
        s.delta = true;
        return s;
    }
    case BXDF_DISNEY: {
        float eta = inner ? b.ior : 1.0f / b.ior;
        DisneyColors d = disney_colors(b, color);
        DisneyLobes w = disney_lobes(b, d, eta, V.z);
        float3 L;
        if (u.x < w.dw) {
            u.x /= w.dw;
            L = cosine_hemisphere(u);
        } else if (u.x < w.dw + w.srw) {
            u.x = (u.x - w.dw) / w.srw;
            float3 H = sample_gtr2_aniso_h(d.ax, d.ay, u);
            if (dot(V, H) <= 0.0f) return s;
            L = normalize(reflect(-V, H));
        } else if (u.x < w.dw + w.srw + w.stw) {
            u.x = (u.x - w.dw - w.srw) / w.stw;
            float3 H = sample_ggx_vndf_h(V, b.roughness, u);
            L = refract_dir(-V, H, eta);
            if (dot(V, H) <= 0.0f || dot(L, L) == 0.0f) return s;
            L = normalize(L);
        } else {
            u.x = (u.x - w.dw - w.srw - w.stw) / w.ccw;
            float3 H = sample_gtr1_h(b.clearcoatGloss, u);
            if (dot(V, H) <= 0.0f) return s;
            L = normalize(reflect(-V, H));
        }
        s.pdf = disney_pdf(b, d, w, L, V, eta);
        s.f = disney_eval(b, d, L, V, color, eta);
        s.wi = L;
        return s;
    }
    default: return s;
    }
}

// ---- material-level wrappers (gmaterial.h:20-32, 59-103) --------------------

SRT_HD bool bxdf_is_specular(const Bxdf& b)
{
    return b.type == BXDF_DIELECTRIC ||
           (b.type == BXDF_DISNEY && b.metallic >= 0.99f && b.roughness <= 0.01f) ||
           (b.type == BXDF_DISNEY && b.specTrans >= 0.99f && b.roughness <= 0.01f && b.clearcoatGloss <= 0.01f);
}
SRT_HD bool bxdf_is_transmissive(const Bxdf& b)
{
    return b.type == BXDF_DIELECTRIC || b.type == BXDF_DIFFUSE_TRANSMISSION ||
           (b.type == BXDF_DISNEY && b.metallic < 1.0f && b.specTrans > 0.0f);
}

// World-space sample: wo below the shading frame flips both directions and
// sets `inner` (the reference reverses the three axes of the frame).
SRT_HD BxdfSample material_sample(const Bxdf& b, const Frame& fr, float3 wo, float2 u, float3 color)
{
    float3 wol = fr.to_local(wo);
    bool inner = false;
    if (wol.z <= 0.0f) {
        wol = -wol;
        inner = true;
    }
    BxdfSample s = bxdf_sample(b, wol, u, color, inner);
    if (inner) s.wi = -s.wi;
    s.wi = fr.to_world(s.wi);
    return s;
}

SRT_HD float3 material_eval(const Bxdf& b, const Frame& fr, float3 wi, float3 wo, float3 color)
{
    float3 wil = fr.to_local(wi), wol = fr.to_local(wo);
    bool inner = false;
    if (wol.z <= 0.0f) {
        wol = -wol;
        wil = -wil;
        inner = true;
    }
    return bxdf_eval(b, wil, wol, color, inner);
}

SRT_HD float material_pdf(const Bxdf& b, const Frame& fr, float3 wi, float3 wo, float3 color)
{
    float3 wil = fr.to_local(wi), wol = fr.to_local(wo);
    bool inner = false;
    if (wol.z <= 0.0f) {
        wol = -wol;
        wil = -wil;
        inner = true;
    }
    return bxdf_pdf(b, wil, wol, color, inner);
}

}  // namespace srt
