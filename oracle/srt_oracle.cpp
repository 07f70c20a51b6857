// ORACLE — CPU restatement of the reference path-tracing hot path.
//
// Test infrastructure only (tests/, __graft_entry__.smoke(), bench.py's
// cpu_baseline and reference arm).  The product never links or calls it.
// Each function cites the reference file:line it restates (paths relative
// to the woAIxuexiSR/SRT source tree).  Built with -ffp-contract=off so
// FP32 results are the same on x86-64 and aarch64 hosts.
#include "srt_oracle.h"

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <thread>
#include <vector>

extern "C" {
int oracle_curand_state_bytes(void);
void oracle_curand_init(unsigned long long seed, void* state);
float oracle_curand_uniform01(void* state);
}

namespace {

// ---------------------------------------------------------------------------
// small vector type, templated on the real type (float: FP32 restatement,
// double: FP64 evaluation of the same formulas)
// ---------------------------------------------------------------------------
template <class T>
struct V3 {
    T x, y, z;
    V3() : x(0), y(0), z(0) {}
    V3(T a) : x(a), y(a), z(a) {}
    V3(T a, T b, T c) : x(a), y(b), z(c) {}
};
template <class T> V3<T> operator+(V3<T> a, V3<T> b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
template <class T> V3<T> operator-(V3<T> a, V3<T> b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
template <class T> V3<T> operator-(V3<T> a) { return {-a.x, -a.y, -a.z}; }
template <class T> V3<T> operator*(V3<T> a, V3<T> b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
template <class T> V3<T> operator*(V3<T> a, T s) { return {a.x * s, a.y * s, a.z * s}; }
template <class T> V3<T> operator*(T s, V3<T> a) { return {s * a.x, s * a.y, s * a.z}; }
template <class T> V3<T> operator/(V3<T> a, T s) { return {a.x / s, a.y / s, a.z / s}; }
template <class T> V3<T> operator/(V3<T> a, V3<T> b) { return {a.x / b.x, a.y / b.y, a.z / b.z}; }
template <class T> T dot(V3<T> a, V3<T> b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
template <class T> V3<T> cross(V3<T> a, V3<T> b)
{
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
template <class T> T rsq(T v) { return T(1) / std::sqrt(v); }
template <class T> V3<T> normalize(V3<T> v) { return v * rsq(dot(v, v)); }
template <class T> T length(V3<T> v) { return std::sqrt(dot(v, v)); }
template <class T> T lerp(T a, T b, T t) { return a + t * (b - a); }
template <class T> V3<T> lerp(V3<T> a, V3<T> b, T t) { return a + t * (b - a); }
template <class T> T clampv(T f, T lo, T hi) { return std::max(lo, std::min(f, hi)); }
template <class T> T lum(V3<T> c) { return dot(c, V3<T>(T(0.2126f), T(0.7152f), T(0.0722f))); }
template <class T> V3<T> reflect(V3<T> i, V3<T> n) { return i - T(2) * n * dot(n, i); }
template <class T> V3<T> cvt(const float* p) { return V3<T>(T(p[0]), T(p[1]), T(p[2])); }

template <class T> T PI_() { return T(3.14159265358979323846); }
template <class T> T INV_PI_() { return T(0.318309886183790671538); }

// Onb (src/device_include/math/onb.h:6-38)
template <class T>
struct Onb {
    V3<T> z, x, y;
    static Onb from_n(V3<T> n)
    {
        Onb o;
        o.z = n;
        V3<T> t = (std::fabs(n.x) > std::fabs(n.y)) ? V3<T>(0, 1, 0) : V3<T>(1, 0, 0);
        o.x = normalize(cross(t, n));
        o.y = cross(n, o.x);
        return o;
    }
    static Onb from_nt(V3<T> n, V3<T> t)
    {
        Onb o;
        o.z = n;
        o.x = normalize(t - n * dot(t, n));
        o.y = cross(n, o.x);
        return o;
    }
    V3<T> to_world(V3<T> p) const { return p.x * x + p.y * y + p.z * z; }
    V3<T> to_local(V3<T> p) const { return {dot(p, x), dot(p, y), dot(p, z)}; }
};

// ---------------------------------------------------------------------------
// BxDF (src/device_include/scene/bxdf.h:59-388, math/basic.h:103-258)
// ---------------------------------------------------------------------------
template <class T>
struct Bx {
    int type;
    T ior, metallic, subsurface, roughness, specular, specularTint, anisotropic, sheen, sheenTint,
        clearcoat, clearcoatGloss, specTrans;
};
template <class T>
Bx<T> bx_from(int type, const float* p)
{
    Bx<T> b;
    b.type = type;
    b.ior = p[0];
    b.metallic = p[1];
    b.subsurface = p[2];
    b.roughness = p[3];
    b.specular = p[4];
    b.specularTint = p[5];
    b.anisotropic = p[6];
    b.sheen = p[7];
    b.sheenTint = p[8];
    b.clearcoat = p[9];
    b.clearcoatGloss = p[10];
    b.specTrans = p[11];
    return b;
}
template <class T>
struct BSample {
    V3<T> f, wi;
    T pdf = 0;
    bool delta = false;
};

template <class T> T schlick(T c, T eta = T(1))
{
    T r0 = (eta - T(1)) / (eta + T(1));
    r0 = r0 * r0;
    T m = clampv(T(1) - c, T(0), T(1));
    return r0 + (T(1) - r0) * m * m * m * m * m;
}
template <class T> T fmix(T metal, T eta, T c) { return lerp(schlick(c, eta), schlick(c), metal); }
template <class T> T GTR1(T nh, T a)
{
    if (a >= T(1)) return INV_PI_<T>();
    T a2 = a * a;
    T t = T(1) + (a2 - T(1)) * nh * nh;
    return (a2 - T(1)) * INV_PI_<T>() / (std::log(a2) * t);
}
template <class T> T GTR2(T nh, T a)
{
    T a2 = a * a;
    T t = T(1) + (a2 - T(1)) * nh * nh;
    return a2 * INV_PI_<T>() / (t * t);
}
template <class T> T GTR2a(T nh, T hx, T hy, T ax, T ay)
{
    T a = hx / ax, b = hy / ay;
    T t = a * a + b * b + nh * nh;
    return INV_PI_<T>() / (ax * ay * t * t);
}
template <class T> T smithG(T nv, T alpha)
{
    T a = alpha * alpha;
    T b = nv * nv;
    return (T(2) * nv) / (nv + std::sqrt(a + b - a * b));
}
template <class T> V3<T> cos_hemi(T ux, T uy)
{
    T ox = T(2) * ux - T(1), oy = T(2) * uy - T(1);
    T dx = 0, dy = 0;
    if (!(ox == 0 && oy == 0)) {
        T r, th;
        if (std::fabs(ox) > std::fabs(oy)) {
            r = ox;
            th = (PI_<T>() / T(4)) * (oy / ox);
        } else {
            r = oy;
            th = (PI_<T>() / T(2)) - (PI_<T>() / T(4)) * (ox / oy);
        }
        dx = r * std::cos(th);
        dy = r * std::sin(th);
    }
    return {dx, dy, std::sqrt(std::max(T(0), T(1) - dx * dx - dy * dy))};
}
template <class T> V3<T> s_gtr1(T a, T ux, T uy)
{
    if (a >= T(1)) return cos_hemi(ux, uy);
    T a2 = a * a;
    T phi = T(2) * PI_<T>() * ux;
    T ct = std::sqrt((T(1) - std::pow(a2, T(1) - uy)) / (T(1) - a2));
    T st = clampv(std::sqrt(T(1) - ct * ct), T(0), T(1));
    return {std::cos(phi) * st, std::sin(phi) * st, ct};
}
template <class T> V3<T> s_gtr2a(T ax, T ay, T ux, T uy)
{
    T phi = T(2) * PI_<T>() * ux;
    T sp = ay * std::sin(phi), cp = ax * std::cos(phi);
    T tt = std::sqrt(uy / (T(1) - uy));
    return normalize(V3<T>(tt * cp, tt * sp, T(1)));
}
template <class T> V3<T> s_vndf(V3<T> V, T a, T ux, T uy)
{
    V3<T> vh = normalize(V3<T>(a * V.x, a * V.y, V.z));
    T lensq = vh.x * vh.x + vh.y * vh.y;
    V3<T> T1 = (lensq > 0) ? V3<T>(-vh.y, vh.x, T(0)) * rsq(lensq) : V3<T>(1, 0, 0);
    V3<T> T2 = cross(vh, T1);
    T r = std::sqrt(ux);
    T phi = T(2) * PI_<T>() * uy;
    T t1 = r * std::cos(phi), t2 = r * std::sin(phi);
    T s = T(0.5) * (T(1) + vh.z);
    t2 = (T(1) - s) * std::sqrt(T(1) - t1 * t1) + s * t2;
    V3<T> nh = t1 * T1 + t2 * T2 + std::sqrt(std::max(T(0), T(1) - t1 * t1 - t2 * t2)) * vh;
    return normalize(V3<T>(a * nh.x, a * nh.y, std::max(T(0), nh.z)));
}
template <class T> V3<T> refr(V3<T> i, V3<T> n, T eta)
{
    T ni = dot(n, -i);
    T k = T(1) - eta * eta * (T(1) - ni * ni);
    if (k < 0) return V3<T>(0);
    return eta * i + (eta * ni - std::sqrt(k)) * n;
}

template <class T>
struct DisneySetup {
    T lum_;
    V3<T> spec_color, sheen_color;
    T ax, ay;
};
template <class T> DisneySetup<T> dsetup(const Bx<T>& b, V3<T> color)
{
    DisneySetup<T> d;
    d.lum_ = lum(color);
    V3<T> ctint = (d.lum_ > 0) ? color / d.lum_ : V3<T>(1);
    d.spec_color = lerp(b.specular * T(0.08f) * lerp(V3<T>(1), ctint, b.specularTint), color, b.metallic);
    d.sheen_color = lerp(V3<T>(1), ctint, b.sheenTint);
    T aspect = std::sqrt(T(1) - b.anisotropic * T(0.9f));
    T a2 = b.roughness * b.roughness;
    d.ax = std::max(T(0.001f), a2 / aspect);
    d.ay = std::max(T(0.001f), a2 * aspect);
    return d;
}

// BxDF::eval (bxdf.h:79-180)
template <class T> V3<T> bx_eval(const Bx<T>& b, V3<T> L, V3<T> V, V3<T> color, bool inner)
{
    if (b.type == SRT_BXDF_DIFFUSE) return (L.z <= 0) ? V3<T>(0) : color * INV_PI_<T>();
    if (b.type == SRT_BXDF_DIFFUSE_TRANSMISSION) return color * INV_PI_<T>();
    if (b.type != SRT_BXDF_DISNEY) return V3<T>(0);
    T eta = inner ? b.ior : T(1) / b.ior;
    V3<T> H = (L.z > 0) ? normalize(L + V) : normalize(L + V * eta);
    if (H.z <= 0) H = -H;
    T VH = dot(V, H), LH = dot(L, H);
    DisneySetup<T> d = dsetup(b, color);
    T FM = fmix(b.metallic, eta, VH);
    T dw = d.lum_ * (T(1) - b.metallic) * (T(1) - b.specTrans);
    T srw = lum(lerp(d.spec_color, V3<T>(1), FM));
    T stw = (T(1) - FM) * (T(1) - b.metallic) * b.specTrans * d.lum_;
    T ccw = b.clearcoat * (T(1) - b.metallic);

    V3<T> fd(0), fr(0), ft(0), fc(0);
    if (dw > 0 && L.z > 0) {
        T FL = schlick(L.z), FV = schlick(V.z), FH = schlick(LH);
        T Fd90 = T(0.5) + T(2) * LH * LH * b.roughness;
        T Fd = lerp(T(1), Fd90, FL) * lerp(T(1), Fd90, FV);
        T Fss90 = LH * LH * b.roughness;
        T Fss = lerp(T(1), Fss90, FL) * lerp(T(1), Fss90, FV);
        T ss = T(1.25) * (Fss * (T(1) / (L.z + V.z) - T(0.5)) + T(0.5));
        V3<T> Fsheen = FH * b.sheen * d.sheen_color;
        fd = (INV_PI_<T>() * lerp(Fd, ss, b.subsurface) * color + Fsheen) * (T(1) - b.metallic) * (T(1) - b.specTrans);
    }
    if (srw > 0 && L.z > 0 && V.z > 0) {
        T fm2 = fmix(b.metallic, eta, LH);
        V3<T> F = lerp(d.spec_color, V3<T>(1), fm2);
        T D = GTR2a(H.z, H.x, H.y, d.ax, d.ay);
        T G = smithG(std::fabs(L.z), b.roughness) * smithG(std::fabs(V.z), b.roughness);
        fr = F * D * G / (T(4) * L.z * V.z);
    }
    if (stw > 0 && L.z < 0) {
        T F = schlick(std::fabs(VH), eta);
        T D = GTR2(H.z, b.roughness);
        T den = (LH + VH * eta) * (LH + VH * eta);
        T G = smithG(std::fabs(L.z), b.roughness) * smithG(std::fabs(V.z), b.roughness) * std::fabs(LH) *
              std::fabs(VH) * eta * eta / den;
        V3<T> rc(std::sqrt(color.x), std::sqrt(color.y), std::sqrt(color.z));
        ft = rc * (T(1) - b.metallic) * b.specTrans * (T(1) - F) * D * G / (std::fabs(L.z) * std::fabs(V.z));
    }
    if (ccw > 0 && L.z > 0 && V.z > 0) {
        T FH = schlick(LH, T(1) / T(1.5));
        T F = lerp(T(0.04f), T(1), FH);
        T D = GTR1(H.z, b.clearcoatGloss);
        T G = smithG(L.z, T(0.25)) * smithG(V.z, T(0.25));
        fc = V3<T>(T(0.25)) * b.clearcoat * F * D * G / (T(4) * L.z * V.z);
    }
    return fd + fr + ft + fc;
}

template <class T>
void dweights(const Bx<T>& b, const DisneySetup<T>& d, T eta, T vz, T& dw, T& srw, T& stw, T& ccw)
{
    T FM = fmix(b.metallic, eta, vz);
    dw = d.lum_ * (T(1) - b.metallic) * (T(1) - b.specTrans);
    srw = lum(lerp(d.spec_color, V3<T>(1), FM));
    stw = (T(1) - FM) * (T(1) - b.metallic) * b.specTrans * d.lum_;
    ccw = b.clearcoat * (T(1) - b.metallic);
    T tot = dw + srw + stw + ccw;
    dw /= tot;
    srw /= tot;
    stw /= tot;
    ccw /= tot;
}

// mixture pdf (bxdf.h:289-310, 365-380)
template <class T>
T dpdf(const Bx<T>& b, const DisneySetup<T>& d, T dw, T srw, T stw, T ccw, V3<T> L, V3<T> V, T eta)
{
    V3<T> hr = normalize(L + V);
    if (hr.z < 0) hr = -hr;
    V3<T> ht = normalize(L + V * eta);
    if (ht.z < 0) ht = -ht;
    T pdf = 0;
    if (dw > 0 && L.z > 0) pdf += dw * (L.z * INV_PI_<T>());
    if (srw > 0 && dot(V, hr) > 0) pdf += srw * GTR2a(hr.z, hr.x, hr.y, d.ax, d.ay) * hr.z / (T(4) * dot(V, hr));
    if (stw > 0 && dot(V, ht) > 0 && dot(L, ht) < 0) {
        T VH = dot(V, ht), LH = dot(L, ht);
        T den = LH + VH * eta;
        pdf += stw * GTR2(ht.z, b.roughness) * smithG(V.z, b.roughness) * std::max(VH, T(0)) / V.z *
               std::fabs(LH) / (den * den);
    }
    if (ccw > 0 && dot(V, hr) > 0) pdf += ccw * GTR1(hr.z, b.clearcoatGloss) * hr.z / (T(4) * dot(V, hr));
    return pdf;
}

// BxDF::sample_pdf (bxdf.h:321-387)
template <class T> T bx_pdf(const Bx<T>& b, V3<T> L, V3<T> V, V3<T> color, bool inner)
{
    if (b.type == SRT_BXDF_DIFFUSE) return (L.z <= 0) ? T(0) : L.z * INV_PI_<T>();
    if (b.type == SRT_BXDF_DIFFUSE_TRANSMISSION) return T(0.5) * (std::fabs(L.z) * INV_PI_<T>());
    if (b.type != SRT_BXDF_DISNEY) return T(0);
    T eta = inner ? b.ior : T(1) / b.ior;
    DisneySetup<T> d = dsetup(b, color);
    T dw, srw, stw, ccw;
    dweights(b, d, eta, V.z, dw, srw, stw, ccw);
    return dpdf(b, d, dw, srw, stw, ccw, L, V, eta);
}

// BxDF::sample (bxdf.h:182-319)
template <class T> BSample<T> bx_sample(const Bx<T>& b, V3<T> V, T ux, T uy, V3<T> color, bool inner)
{
    BSample<T> s;
    if (b.type == SRT_BXDF_DIFFUSE) {
        V3<T> wi = cos_hemi(ux, uy);
        s.f = bx_eval(b, wi, V, color, inner);
        s.wi = wi;
        s.pdf = wi.z * INV_PI_<T>();
        return s;
    }
    if (b.type == SRT_BXDF_DIFFUSE_TRANSMISSION) {
        if (ux < T(0.5)) {
            V3<T> wi = cos_hemi(ux * T(2), uy);
            s.f = bx_eval(b, wi, V, color, inner);
            s.wi = wi;
            s.pdf = T(0.5) * (wi.z * INV_PI_<T>());
        } else {
            V3<T> wi = cos_hemi((ux - T(0.5)) * T(2), uy);
            s.f = bx_eval(b, -wi, V, color, inner);
            s.wi = -wi;
            s.pdf = T(0.5) * (wi.z * INV_PI_<T>());
        }
        return s;
    }
    if (b.type == SRT_BXDF_DIELECTRIC) {
        T eta = inner ? b.ior : T(1) / b.ior;
        V3<T> n(0, 0, 1);
        V3<T> wi = refr(-V, n, eta);
        T rr = (dot(wi, wi) == 0) ? T(1) : schlick(V.z, eta);
        if (ux <= rr) wi = reflect(-V, n);
        s.f = color;
        s.wi = normalize(wi);
        s.pdf = 1;
        s.delta = true;
        return s;
    }
    if (b.type != SRT_BXDF_DISNEY) return s;
    T eta = inner ? b.ior : T(1) / b.ior;
    DisneySetup<T> d = dsetup(b, color);
    T dw, srw, stw, ccw;
    dweights(b, d, eta, V.z, dw, srw, stw, ccw);
    V3<T> L;
    if (ux < dw) {
        L = cos_hemi(ux / dw, uy);
    } else if (ux < dw + srw) {
        V3<T> H = s_gtr2a(d.ax, d.ay, (ux - dw) / srw, uy);
        if (dot(V, H) <= 0) return BSample<T>();
        L = normalize(reflect(-V, H));
    } else if (ux < dw + srw + stw) {
        V3<T> H = s_vndf(V, b.roughness, (ux - dw - srw) / stw, uy);
        L = refr(-V, H, eta);
        if (dot(V, H) <= 0 || dot(L, L) == 0) return BSample<T>();
        L = normalize(L);
    } else {
        V3<T> H = s_gtr1(b.clearcoatGloss, (ux - dw - srw - stw) / ccw, uy);
        if (dot(V, H) <= 0) return BSample<T>();
        L = normalize(reflect(-V, H));
    }
    s.pdf = dpdf(b, d, dw, srw, stw, ccw, L, V, eta);
    s.f = bx_eval(b, L, V, color, inner);
    s.wi = L;
    return s;
}

// GMaterial wrappers (gmaterial.h:59-103)
template <class T> BSample<T> mat_sample(const Bx<T>& b, const Onb<T>& o, V3<T> wo, T ux, T uy, V3<T> color)
{
    V3<T> wol = o.to_local(wo);
    bool inner = false;
    if (wol.z <= 0) {
        wol = -wol;
        inner = true;
    }
    BSample<T> s = bx_sample(b, wol, ux, uy, color, inner);
    if (inner) s.wi = -s.wi;
    s.wi = o.to_world(s.wi);
    return s;
}
template <class T> V3<T> mat_eval(const Bx<T>& b, const Onb<T>& o, V3<T> wi, V3<T> wo, V3<T> color)
{
    V3<T> wil = o.to_local(wi), wol = o.to_local(wo);
    bool inner = false;
    if (wol.z <= 0) {
        wol = -wol;
        wil = -wil;
        inner = true;
    }
    return bx_eval(b, wil, wol, color, inner);
}
template <class T> T mat_pdf(const Bx<T>& b, const Onb<T>& o, V3<T> wi, V3<T> wo, V3<T> color)
{
    V3<T> wil = o.to_local(wi), wol = o.to_local(wo);
    bool inner = false;
    if (wol.z <= 0) {
        wol = -wol;
        wil = -wil;
        inner = true;
    }
    return bx_pdf(b, wil, wol, color, inner);
}
static bool is_specular(const srt_bxdf& b)
{
    return b.type == SRT_BXDF_DIELECTRIC || (b.type == SRT_BXDF_DISNEY && b.metallic >= 0.99f && b.roughness <= 0.01f) ||
           (b.type == SRT_BXDF_DISNEY && b.specTrans >= 0.99f && b.roughness <= 0.01f && b.clearcoatGloss <= 0.01f);
}
static bool is_transmissive(const srt_bxdf& b)
{
    return b.type == SRT_BXDF_DIELECTRIC || b.type == SRT_BXDF_DIFFUSE_TRANSMISSION ||
           (b.type == SRT_BXDF_DISNEY && b.metallic < 1.0f && b.specTrans > 0.0f);
}
static Bx<float> bx_of(const srt_bxdf& m)
{
    Bx<float> b;
    b.type = m.type;
    b.ior = m.ior;
    b.metallic = m.metallic;
    b.subsurface = m.subsurface;
    b.roughness = m.roughness;
    b.specular = m.specular;
    b.specularTint = m.specularTint;
    b.anisotropic = m.anisotropic;
    b.sheen = m.sheen;
    b.sheenTint = m.sheenTint;
    b.clearcoat = m.clearcoat;
    b.clearcoatGloss = m.clearcoatGloss;
    b.specTrans = m.specTrans;
    return b;
}

// ---------------------------------------------------------------------------
// PCG32 (O'Neill, "PCG: A Family of Simple Fast Space-Efficient Statistically
// Good Algorithms for Random Number Generation", minimal C implementation)
// ---------------------------------------------------------------------------
struct Pcg32 {
    uint64_t state, inc;
    uint32_t next()
    {
        uint64_t old = state;
        state = old * 6364136223846793005ULL + inc;
        uint32_t xs = (uint32_t)(((old >> 18u) ^ old) >> 27u);
        uint32_t rot = (uint32_t)(old >> 59u);
        return (xs >> rot) | (xs << ((-rot) & 31));
    }
    void seed(uint64_t initstate, uint64_t initseq)
    {
        state = 0U;
        inc = (initseq << 1u) | 1u;
        next();
        state += initstate;
        next();
    }
    float uniform() { return (float)(next() >> 8) * (1.0f / 16777216.0f); }
};

// hash RNG of SRT_RNG_HASH (PCG output permutation used as an integer hash)
static inline uint32_t pcg_hash(uint32_t v)
{
    uint32_t s = v * 747796405u + 2891336453u;
    uint32_t w = ((s >> ((s >> 28u) + 4u)) ^ s) * 277803737u;
    return (w >> 22u) ^ w;
}
static inline uint32_t hash_key(uint32_t seed, uint32_t pixel, uint32_t sample)
{
    return pcg_hash(pcg_hash(pcg_hash(seed) ^ pixel) ^ sample);
}
static inline float hash_u(uint32_t key, uint32_t dim)
{
    return (float)(pcg_hash(key ^ pcg_hash(dim)) >> 8) * (1.0f / 16777216.0f);
}

// ---------------------------------------------------------------------------
// scene (object-space meshes + instances, like Scene / GScene)
// ---------------------------------------------------------------------------
typedef V3<float> F3;

struct Xf {  // row-major 3x4 (Transform, math/transform.h:208-240)
    float m[12];
    F3 point(F3 p) const
    {
        return {m[0] * p.x + m[1] * p.y + m[2] * p.z + m[3], m[4] * p.x + m[5] * p.y + m[6] * p.z + m[7],
                m[8] * p.x + m[9] * p.y + m[10] * p.z + m[11]};
    }
    F3 vec(F3 v) const
    {
        return {m[0] * v.x + m[1] * v.y + m[2] * v.z, m[4] * v.x + m[5] * v.y + m[6] * v.z,
                m[8] * v.x + m[9] * v.y + m[10] * v.z};
    }
};

struct OMesh {
    std::vector<F3> v, n, tg;
    std::vector<float> tc;  // 2 per vertex when the mesh has texture coordinates
    std::vector<uint32_t> idx;
    int material;
    float area = 0.0f;
    std::vector<float> area_cdf;
};
struct OInst {
    int mesh;
    Xf xf;
    int light_id;
    int64_t prim_base;
};
struct BNode {
    float bmin[3], bmax[3];
    int32_t left;   // first child (internal) or first prim (leaf)
    int32_t count;  // 0 internal, >0 leaf
};

struct Camera {
    int type;
    F3 pos, x, y, z;
    float radius, nw, nh, aperture, focal;
};

}  // namespace

// A texture read as a CUDA texture object with linear filtering, wrap
// addressing and normalised coordinates (scene.cu:92-139), computed
// exactly: texel centres at (i + 0.5) / size, bilinear weights without the
// hardware's 8-bit fixed-point quantisation, and 8-bit texels decoded with
// the sRGB transfer function of IEC 61966-2-1 (the hardware's decode is a
// coarser table), alpha linear.  Comparisons with the GPU carry a tolerance.
struct OTex {
    int w = 0, h = 0;
    std::vector<double> lin;  // RGBA per texel, decoded
    F3 rgb(float x, float y) const
    {
        double fx = (double)x - std::floor((double)x), fy = (double)y - std::floor((double)y);
        double xb = fx * w - 0.5, yb = fy * h - 0.5;
        double i0 = std::floor(xb), j0 = std::floor(yb);
        double a = xb - i0, b = yb - j0;
        int i = ((int)i0 % w + w) % w, j = ((int)j0 % h + h) % h;
        int i1 = (i + 1) % w, j1 = (j + 1) % h;
        double r[3];
        for (int c = 0; c < 3; ++c)
            r[c] = (1 - a) * (1 - b) * lin[4 * ((size_t)j * w + i) + c] + a * (1 - b) * lin[4 * ((size_t)j * w + i1) + c] +
                   (1 - a) * b * lin[4 * ((size_t)j1 * w + i) + c] + a * b * lin[4 * ((size_t)j1 * w + i1) + c];
        return F3((float)r[0], (float)r[1], (float)r[2]);
    }
    void fetch4(float x, float y, float* out) const
    {
        double fx = (double)x - std::floor((double)x), fy = (double)y - std::floor((double)y);
        double xb = fx * w - 0.5, yb = fy * h - 0.5;
        double i0 = std::floor(xb), j0 = std::floor(yb);
        double a = xb - i0, b = yb - j0;
        int i = ((int)i0 % w + w) % w, j = ((int)j0 % h + h) % h;
        int i1 = (i + 1) % w, j1 = (j + 1) % h;
        for (int c = 0; c < 4; ++c)
            out[c] = (float)((1 - a) * (1 - b) * lin[4 * ((size_t)j * w + i) + c] +
                             a * (1 - b) * lin[4 * ((size_t)j * w + i1) + c] +
                             (1 - a) * b * lin[4 * ((size_t)j1 * w + i) + c] + a * b * lin[4 * ((size_t)j1 * w + i1) + c]);
    }
};

struct oracle_scene {
    std::vector<OTex> tex;
    std::vector<int> mat_tex;  // 2 per material (colour, normal), -1 none
    int env_map = -1;
    std::vector<OMesh> meshes;
    std::vector<OInst> inst;
    std::vector<srt_material> mats;
    // flattened world-space triangles (for intersection)
    std::vector<F3> w0, w1, w2;
    std::vector<int32_t> tri_inst, tri_face;
    // lights (scene.cu:370-417)
    std::vector<int> light_inst;
    std::vector<float> weight_cdf;
    float weight_sum = 0.0f;
    F3 env;
    Camera cam;
    // BVH
    std::vector<BNode> nodes;
    std::vector<int32_t> prim;
};

namespace {

// CameraController(LookAt) + Camera::reset (camera.h:41-53, 165-170;
// transform.h:136-145)
Camera make_camera(const srt_camera_desc& c)
{
    Camera k;
    k.type = c.type & ~SRT_CAMERA_MIRROR_X;
    F3 pos(c.position[0], c.position[1], c.position[2]);
    F3 tgt(c.target[0], c.target[1], c.target[2]);
    F3 up(c.up[0], c.up[1], c.up[2]);
    F3 z = normalize(tgt - pos);
    F3 x = normalize(cross(up, z));
    F3 y = cross(z, x);
    k.pos = pos;
    k.x = normalize(x);
    if (c.type & SRT_CAMERA_MIRROR_X) k.x = k.x * -1.0f;
    k.y = normalize(y);
    k.z = normalize(z);
    k.radius = length(pos - tgt);
    float rad = (c.fov * 0.5f) * (float)M_PI / 180.0f;
    k.nh = 2.0f * std::tan(rad);
    k.nw = k.nh * c.aspect;
    k.aperture = c.aperture;
    k.focal = c.focal;
    return k;
}

// Camera::get_ray, perspective / orthographic (camera.h:107-122)
void camera_ray(const Camera& k, float x, float y, F3& o, F3& d)
{
    float px = (x - 0.5f) * k.nw, py = (y - 0.5f) * k.nh;
    F3 lo, ld;
    if (k.type == SRT_CAMERA_ORTHOGRAPHIC) {
        lo = F3(px * k.radius, py * k.radius, 1.0f);
        ld = F3(0.0f, 0.0f, 1.0f);
    } else {
        lo = F3(0.0f);
        ld = normalize(F3(px, py, 1.0f));
    }
    o = lo.x * k.x + lo.y * k.y + lo.z * k.z + k.pos;
    d = ld.x * k.x + ld.y * k.y + ld.z * k.z;
}

// basic.h:26-38
int bsearch_cdf(const float* cdf, int num, float x)
{
    int lf = 0, rg = num - 1;
    while (lf <= rg) {
        int mid = (lf + rg) / 2;
        if (cdf[mid] <= x)
            lf = mid + 1;
        else
            rg = mid - 1;
    }
    return std::min(rg + 1, num - 1);
}

// remap of a uniform into the chosen CDF bucket; the reference stores
// cdf[idx-1] in an int (light.h:65, gmesh.h:49), which truncates it
float cdf_remap(const float* cdf, int idx, float u, bool fixed)
{
    if (fixed) {
        float lower = (idx == 0) ? 0.0f : cdf[idx - 1];
        return (u - lower) / (cdf[idx] - lower);
    }
    int lower = (idx == 0) ? 0 : (int)cdf[idx - 1];
    return (u - lower) / (cdf[idx] - lower);
}

struct LSample {
    F3 pos, normal, emission;
    float pdf;
};

// Light::sample + GInstance::sample (light.h:61-76, gmesh.h:45-85)
LSample light_sample(const oracle_scene& s, float ux, float uy, bool fixed)
{
    int num = (int)s.light_inst.size();
    int li = bsearch_cdf(s.weight_cdf.data(), num, ux);
    ux = cdf_remap(s.weight_cdf.data(), li, ux, fixed);
    const OInst& in = s.inst[s.light_inst[li]];
    const OMesh& m = s.meshes[in.mesh];
    int nf = (int)m.area_cdf.size();
    int fi = bsearch_cdf(m.area_cdf.data(), nf, ux);
    ux = cdf_remap(m.area_cdf.data(), fi, ux, fixed);
    float sx = std::sqrt(ux);
    float bu = 1.0f - sx, bv = uy * sx;  // uniform_sample_triangle (basic.h:139-143)
    uint32_t i0 = m.idx[3 * fi], i1 = m.idx[3 * fi + 1], i2 = m.idx[3 * fi + 2];
    F3 v0 = m.v[i0], v1 = m.v[i1], v2 = m.v[i2];
    F3 pos = v0 * (1.0f - bu - bv) + v1 * bu + v2 * bv;
    F3 nrm = normalize(cross(v1 - v0, v2 - v0));
    if (!m.n.empty()) {
        F3 sn = m.n[i0] * (1.0f - bu - bv) + m.n[i1] * bu + m.n[i2] * bv;
        if (dot(nrm, sn) < 0.0f) nrm = -nrm;
    }
    const srt_material& mat = s.mats[m.material];
    LSample ls;
    ls.pos = in.xf.point(pos);
    ls.normal = in.xf.vec(nrm);
    ls.emission = cvt<float>(mat.emission_color) * mat.intensity;
    const int ct = s.mat_tex.empty() ? -1 : s.mat_tex[2 * m.material];
    if (ct >= 0) {
        // GMaterial::emission(texcoord) (gmaterial.h:35-41)
        float tu = bu, tv = bv;
        if (!m.tc.empty()) {
            tu = m.tc[2 * i0] * (1.0f - bu - bv) + m.tc[2 * i1] * bu + m.tc[2 * i2] * bv;
            tv = m.tc[2 * i0 + 1] * (1.0f - bu - bv) + m.tc[2 * i1 + 1] * bu + m.tc[2 * i2 + 1] * bv;
        }
        ls.emission = s.tex[ct].rgb(tu, tv) * mat.intensity;
    }
    ls.pdf = mat.intensity / s.weight_sum;
    return ls;
}

float light_pdf_of(const oracle_scene& s, int light_id)
{
    const OInst& in = s.inst[s.light_inst[light_id]];
    return s.mats[s.meshes[in.mesh].material].intensity / s.weight_sum;
}

struct Hit {
    float t, u, v;
    int64_t prim;  // -1 miss
};

// watertight ray/triangle test (Woop, Benthin, Wald, JCGT 2013)
struct RayPre {
    F3 o, d;
    int kx, ky, kz;
    float Sx, Sy, Sz;
};
RayPre ray_pre(F3 o, F3 d)
{
    RayPre r;
    r.o = o;
    r.d = d;
    float ad[3] = {std::fabs(d.x), std::fabs(d.y), std::fabs(d.z)};
    int kz = 0;
    if (ad[1] > ad[kz]) kz = 1;
    if (ad[2] > ad[kz]) kz = 2;
    int kx = (kz + 1) % 3, ky = (kx + 1) % 3;
    float dd[3] = {d.x, d.y, d.z};
    if (dd[kz] < 0.0f) std::swap(kx, ky);
    r.kx = kx;
    r.ky = ky;
    r.kz = kz;
    r.Sx = dd[kx] / dd[kz];
    r.Sy = dd[ky] / dd[kz];
    r.Sz = 1.0f / dd[kz];
    return r;
}
inline float comp(const F3& v, int k) { return k == 0 ? v.x : (k == 1 ? v.y : v.z); }

// returns true on a hit in (tmin, tmax); t, b1, b2 (barycentrics of v1, v2)
bool tri_hit(const RayPre& r, F3 v0, F3 v1, F3 v2, float tmin, float tmax, float& t, float& b1, float& b2)
{
    F3 A = v0 - r.o, B = v1 - r.o, C = v2 - r.o;
    float Ax = comp(A, r.kx) - r.Sx * comp(A, r.kz), Ay = comp(A, r.ky) - r.Sy * comp(A, r.kz);
    float Bx = comp(B, r.kx) - r.Sx * comp(B, r.kz), By = comp(B, r.ky) - r.Sy * comp(B, r.kz);
    float Cx = comp(C, r.kx) - r.Sx * comp(C, r.kz), Cy = comp(C, r.ky) - r.Sy * comp(C, r.kz);
    float U = Cx * By - Cy * Bx;
    float V = Ax * Cy - Ay * Cx;
    float W = Bx * Ay - By * Ax;
    if ((U < 0.0f || V < 0.0f || W < 0.0f) && (U > 0.0f || V > 0.0f || W > 0.0f)) return false;
    float det = U + V + W;
    if (det == 0.0f) return false;
    float Az = r.Sz * comp(A, r.kz), Bz = r.Sz * comp(B, r.kz), Cz = r.Sz * comp(C, r.kz);
    float Tt = U * Az + V * Bz + W * Cz;
    float inv = 1.0f / det;
    float tt = Tt * inv;
    if (!(tt > tmin && tt < tmax)) return false;
    t = tt;
    b1 = V * inv;
    b2 = W * inv;
    return true;
}

// ---- oracle BVH (binary, binned SAH) --------------------------------------
struct BuildRef {
    float bmin[3], bmax[3], c[3];
};
void build_rec(oracle_scene& s, std::vector<BuildRef>& refs, int node, int begin, int end)
{
    BNode& nd = s.nodes[node];
    float bmin[3] = {1e30f, 1e30f, 1e30f}, bmax[3] = {-1e30f, -1e30f, -1e30f};
    float cmin[3] = {1e30f, 1e30f, 1e30f}, cmax[3] = {-1e30f, -1e30f, -1e30f};
    for (int i = begin; i < end; ++i) {
        const BuildRef& r = refs[s.prim[i]];
        for (int k = 0; k < 3; ++k) {
            bmin[k] = std::min(bmin[k], r.bmin[k]);
            bmax[k] = std::max(bmax[k], r.bmax[k]);
            cmin[k] = std::min(cmin[k], r.c[k]);
            cmax[k] = std::max(cmax[k], r.c[k]);
        }
    }
    for (int k = 0; k < 3; ++k) {
        nd.bmin[k] = bmin[k];
        nd.bmax[k] = bmax[k];
    }
    int n = end - begin;
    if (n <= 4) {
        nd.left = begin;
        nd.count = n;
        return;
    }
    const int NB = 16;
    float best = 1e38f;
    int bax = -1, bsplit = -1;
    for (int ax = 0; ax < 3; ++ax) {
        float ext = cmax[ax] - cmin[ax];
        if (!(ext > 0.0f)) continue;
        int cnt[NB] = {0};
        float lo[NB][3], hi[NB][3];
        for (int b = 0; b < NB; ++b)
            for (int k = 0; k < 3; ++k) {
                lo[b][k] = 1e30f;
                hi[b][k] = -1e30f;
            }
        for (int i = begin; i < end; ++i) {
            const BuildRef& r = refs[s.prim[i]];
            int b = std::min(NB - 1, (int)((r.c[ax] - cmin[ax]) / ext * NB));
            cnt[b]++;
            for (int k = 0; k < 3; ++k) {
                lo[b][k] = std::min(lo[b][k], r.bmin[k]);
                hi[b][k] = std::max(hi[b][k], r.bmax[k]);
            }
        }
        float ra[NB], rc[NB];
        float alo[3] = {1e30f, 1e30f, 1e30f}, ahi[3] = {-1e30f, -1e30f, -1e30f};
        int acc = 0;
        for (int b = NB - 1; b > 0; --b) {
            acc += cnt[b];
            for (int k = 0; k < 3; ++k) {
                alo[k] = std::min(alo[k], lo[b][k]);
                ahi[k] = std::max(ahi[k], hi[b][k]);
            }
            float dx = ahi[0] - alo[0], dy = ahi[1] - alo[1], dz = ahi[2] - alo[2];
            ra[b] = acc ? (dx * dy + dy * dz + dz * dx) : 0.0f;
            rc[b] = (float)acc;
        }
        float llo[3] = {1e30f, 1e30f, 1e30f}, lhi[3] = {-1e30f, -1e30f, -1e30f};
        int lacc = 0;
        for (int b = 0; b < NB - 1; ++b) {
            lacc += cnt[b];
            for (int k = 0; k < 3; ++k) {
                llo[k] = std::min(llo[k], lo[b][k]);
                lhi[k] = std::max(lhi[k], hi[b][k]);
            }
            float dx = lhi[0] - llo[0], dy = lhi[1] - llo[1], dz = lhi[2] - llo[2];
            float la = lacc ? (dx * dy + dy * dz + dz * dx) : 0.0f;
            float cost = la * lacc + ra[b + 1] * rc[b + 1];
            if (lacc > 0 && rc[b + 1] > 0 && cost < best) {
                best = cost;
                bax = ax;
                bsplit = b;
            }
        }
    }
    int mid;
    if (bax < 0) {
        mid = begin + n / 2;
    } else {
        float ext = cmax[bax] - cmin[bax];
        auto it = std::partition(s.prim.begin() + begin, s.prim.begin() + end, [&](int32_t p) {
            int b = std::min(NB - 1, (int)((refs[p].c[bax] - cmin[bax]) / ext * NB));
            return b <= bsplit;
        });
        mid = (int)(it - s.prim.begin());
        if (mid == begin || mid == end) mid = begin + n / 2;
    }
    int l = (int)s.nodes.size();
    s.nodes.push_back(BNode());
    s.nodes.push_back(BNode());
    s.nodes[node].left = l;
    s.nodes[node].count = 0;
    build_rec(s, refs, l, begin, mid);
    build_rec(s, refs, l + 1, mid, end);
}

inline bool box_hit(const BNode& b, const F3& o, const F3& inv, float tmin, float tmax, float& tnear)
{
    float t0x = (b.bmin[0] - o.x) * inv.x, t1x = (b.bmax[0] - o.x) * inv.x;
    float t0y = (b.bmin[1] - o.y) * inv.y, t1y = (b.bmax[1] - o.y) * inv.y;
    float t0z = (b.bmin[2] - o.z) * inv.z, t1z = (b.bmax[2] - o.z) * inv.z;
    float tn = std::max(std::max(std::min(t0x, t1x), std::min(t0y, t1y)), std::max(std::min(t0z, t1z), tmin));
    float tf = std::min(std::min(std::max(t0x, t1x), std::max(t0y, t1y)), std::min(std::max(t0z, t1z), tmax));
    tnear = tn;
    return tn <= tf * 1.00000024f;
}

// closest hit (any_hit = true: stop at the first hit)
Hit trace(const oracle_scene& s, F3 o, F3 d, float tmin, float tmax, bool any_hit, bool use_bvh)
{
    Hit h{tmax, 0.0f, 0.0f, -1};
    RayPre r = ray_pre(o, d);
    float t, b1, b2;
    if (!use_bvh || s.nodes.empty()) {
        int64_t nt = (int64_t)s.w0.size();
        for (int64_t i = 0; i < nt; ++i) {
            if (tri_hit(r, s.w0[i], s.w1[i], s.w2[i], tmin, h.t, t, b1, b2)) {
                h.t = t;
                h.u = b1;
                h.v = b2;
                h.prim = i;
                if (any_hit) return h;
            }
        }
        return h;
    }
    F3 inv(1.0f / d.x, 1.0f / d.y, 1.0f / d.z);
    int stack[128];
    int sp = 0;
    stack[sp++] = 0;
    while (sp) {
        const BNode& nd = s.nodes[stack[--sp]];
        float tn;
        if (!box_hit(nd, o, inv, tmin, h.t, tn)) continue;
        if (nd.count > 0) {
            for (int i = nd.left; i < nd.left + nd.count; ++i) {
                int p = s.prim[i];
                if (tri_hit(r, s.w0[p], s.w1[p], s.w2[p], tmin, h.t, t, b1, b2)) {
                    // ties keep the lower primitive id, like the brute-force order
                    if (t < h.t || h.prim < 0 || p < h.prim) {
                        h.t = t;
                        h.u = b1;
                        h.v = b2;
                        h.prim = p;
                    }
                    if (any_hit) return h;
                }
            }
        } else {
            float ta, tb;
            bool ha = box_hit(s.nodes[nd.left], o, inv, tmin, h.t, ta);
            bool hb = box_hit(s.nodes[nd.left + 1], o, inv, tmin, h.t, tb);
            if (ha && hb) {
                if (ta < tb) {
                    stack[sp++] = nd.left + 1;
                    stack[sp++] = nd.left;
                } else {
                    stack[sp++] = nd.left;
                    stack[sp++] = nd.left + 1;
                }
            } else if (ha) {
                stack[sp++] = nd.left;
            } else if (hb) {
                stack[sp++] = nd.left + 1;
            }
        }
    }
    return h;
}

struct HitInfo {
    F3 pos, normal, color, emission;
    Onb<float> onb;
    int mat;
    int light_id;
};

// get_hitinfo (params/hit_info.h:27-64), object space then instance transform
HitInfo hit_info(const oracle_scene& s, int64_t prim, float u, float v)
{
    const OInst& in = s.inst[s.tri_inst[prim]];
    const OMesh& m = s.meshes[in.mesh];
    int f = s.tri_face[prim];
    uint32_t i0 = m.idx[3 * f], i1 = m.idx[3 * f + 1], i2 = m.idx[3 * f + 2];
    F3 v0 = m.v[i0], v1 = m.v[i1], v2 = m.v[i2];
    F3 pos = v0 * (1.0f - u - v) + v1 * u + v2 * v;
    float tu = u, tv = v;
    if (!m.tc.empty()) {
        tu = m.tc[2 * i0] * (1.0f - u - v) + m.tc[2 * i1] * u + m.tc[2 * i2] * v;
        tv = m.tc[2 * i0 + 1] * (1.0f - u - v) + m.tc[2 * i1 + 1] * u + m.tc[2 * i2 + 1] * v;
    }
    const int ct = s.mat_tex.empty() ? -1 : s.mat_tex[2 * m.material];
    const int nt = s.mat_tex.empty() ? -1 : s.mat_tex[2 * m.material + 1];
    F3 nrm = normalize(cross(v1 - v0, v2 - v0));
    F3 sn = nrm;
    if (!m.n.empty()) sn = normalize(m.n[i0] * (1.0f - u - v) + m.n[i1] * u + m.n[i2] * v);
    if (nt >= 0) sn = normalize(s.tex[nt].rgb(tu, tv));  // GMaterial::shading_normal (gmaterial.h:43-48)
    if (dot(nrm, sn) < 0.0f) nrm = -nrm;
    F3 tan = (std::fabs(sn.x) > std::fabs(sn.y)) ? F3(0, 1, 0) : F3(1, 0, 0);
    if (!m.tg.empty()) tan = m.tg[i0] * (1.0f - u - v) + m.tg[i1] * u + m.tg[i2] * v;
    Onb<float> ob = Onb<float>::from_nt(sn, tan);
    HitInfo h;
    h.pos = in.xf.point(pos);
    h.normal = in.xf.vec(nrm);
    h.color = ct >= 0 ? s.tex[ct].rgb(tu, tv) : cvt<float>(s.mats[m.material].base_color);
    h.emission = cvt<float>(s.mats[m.material].emission_color) * s.mats[m.material].intensity;
    if (ct >= 0) h.emission = h.color * s.mats[m.material].intensity;  // GMaterial::emission (gmaterial.h:35-41)
    h.onb.z = in.xf.vec(ob.z);
    h.onb.x = in.xf.vec(ob.x);
    h.onb.y = in.xf.vec(ob.y);
    h.mat = m.material;
    h.light_id = in.light_id;
    return h;
}

struct Rng {
    int mode;
    unsigned char st[128];
    uint32_t key, dim;
    void init_curand(int seed, int idx)
    {
        int si = (int)((unsigned)seed + (unsigned)idx);
        oracle_curand_init((unsigned long long)(long long)si, st);
    }
    void init_hash(int seed, int pixel, int sample)
    {
        key = hash_key((uint32_t)seed, (uint32_t)pixel, (uint32_t)sample);
        dim = 0;
    }
    float next()
    {
        if (mode == SRT_RNG_CURAND) return oracle_curand_uniform01(st);
        return hash_u(key, dim++);
    }
};

// EnvironmentLight::emission (light.h:27-41): constant, or the "uvmap"
// texture at the direction's spherical coordinates (world y up)
F3 env_radiance(const oracle_scene& s, F3 d)
{
    if (s.env_map < 0) return s.env;
    const float mx = -d.x, my = d.z, mz = d.y;
    const float phi = std::atan2(my, mx), theta = std::acos(mz);  // cartesian_to_spherical_uv (basic.h:41-46)
    const float u = phi * 0.5f * (float)M_1_PI + 0.5f, v = theta * (float)M_1_PI;
    return s.tex[s.env_map].rgb(u, v);
}

// Megakernel raygen loop (src/shader/integrator/path_tracer.cu:50-169).
// ev (optional, ev_max bytes): one byte per traced path segment of the
// pixel, in order across its samples: bit 0 traced, bit 1 the ray hit a
// triangle, bit 2 a shadow ray was traced, bit 3 the sample ended there.
// A wavefront that keeps one path per pixel in flight and starts the next
// sample in the iteration the previous one ends traces segment k of every
// pixel in its iteration k, so these bytes give its per-iteration counts.
void render_pixel(const oracle_scene& s, int w, int h, int ix, int iy, const srt_pt_params& p, bool use_bvh,
                  float* film, double* sum, double* sumsq, int64_t* cnt, uint8_t* ev = nullptr, int ev_max = 0)
{
    int seg = 0;
    auto mark = [&](int k, uint8_t bits) {
        if (ev && k >= 0 && k < ev_max) ev[k] |= bits;
    };
    const int idx = iy * w + ix;
    const bool fixed = (p.flags & SRT_PT_FIXED_CDF_REMAP) != 0;
    Rng rng;
    rng.mode = p.rng_mode;
    if (p.rng_mode == SRT_RNG_CURAND) rng.init_curand(p.seed, idx);
    F3 result(0.0f);
    double s1[3] = {0, 0, 0}, s2[3] = {0, 0, 0};
    for (int i = 0; i < p.samples_per_pixel; ++i) {
        if (p.rng_mode == SRT_RNG_HASH) rng.init_hash(p.seed, idx, i);
        cnt[0]++;
        float xx = ((float)ix + rng.next()) / (float)w;
        float yy = ((float)iy + rng.next()) / (float)h;
        F3 ro, rd;
        camera_ray(s.cam, xx, yy, ro, rd);
        bool specular = true;
        float scatter_pdf = 1.0f;
        F3 L(0.0f), beta(1.0f);
        for (int depth = 0; depth < p.max_depth; ++depth) {
            cnt[1]++;
            cnt[3]++;
            Hit hit = trace(s, ro, rd, 1e-3f, 1e16f, false, use_bvh);
            mark(seg++, hit.prim < 0 ? 1 : 3);
            if (hit.prim < 0) {
                L = L + beta * env_radiance(s, rd);
                break;
            }
            HitInfo hi = hit_info(s, hit.prim, hit.u, hit.v);
            const srt_material& mat = s.mats[hi.mat];
            Bx<float> bx = bx_of(mat.bxdf);
            if (mat.intensity > 0.0f) {
                float cos_i = dot(hi.normal, -rd);
                if (cos_i <= 1e-4f) break;
                float mis = 1.0f;
                if (p.use_nee && !specular) {
                    mis = 0.0f;
                    if (p.use_mis) {
                        float t2 = dot(hi.pos - ro, hi.pos - ro);
                        float lpdf = light_pdf_of(s, hi.light_id) * t2 / cos_i;
                        mis = scatter_pdf / (lpdf + scatter_pdf);
                    }
                }
                L = L + beta * hi.emission * mis;
                break;
            }
            float cos_i = dot(hi.normal, -rd);
            if (cos_i < 0.0f) hi.normal = -hi.normal;
            if (p.use_nee && !is_specular(mat.bxdf) && !(depth > 0 && (p.flags & SRT_PT_NEE_FIRST_VERTEX_ONLY))) {
                float lu = rng.next();
                float lv = rng.next();
                LSample ls = light_sample(s, lu, lv, fixed);
                F3 sd = normalize(ls.pos - hi.pos);
                float cos_o = dot(hi.normal, sd);
                float cos_l = dot(ls.normal, -sd);
                float t = length(ls.pos - hi.pos);
                if (cos_l > 1e-4f && ls.pdf > 1e-4f && t > 1e-3f && (cos_o > 0.0f || is_transmissive(mat.bxdf))) {
                    cnt[2]++;
                    mark(seg - 1, 4);
                    Hit sh = trace(s, hi.pos, sd, 1e-3f, t - 1e-3f, true, use_bvh);
                    if (sh.prim < 0) {
                        float mis = 1.0f;
                        float lpdf = ls.pdf * t * t / cos_l;
                        if (p.use_mis) {
                            float mpdf = mat_pdf(bx, hi.onb, sd, -rd, hi.color);
                            mis = lpdf / (lpdf + mpdf);
                        }
                        F3 fv = mat_eval(bx, hi.onb, sd, -rd, hi.color);
                        L = L + beta * fv * std::fabs(cos_o) * ls.emission * mis / lpdf;
                    }
                }
            }
            float bu = rng.next();
            float bv = rng.next();
            BSample<float> ms = mat_sample(bx, hi.onb, -rd, bu, bv, hi.color);
            if (ms.pdf <= 1e-4f) break;
            if (dot(ms.wi, hi.normal) < 0.0f && !is_transmissive(mat.bxdf)) break;
            beta = beta * (ms.f / ms.pdf);
            if (!ms.delta) beta = beta * std::fabs(dot(ms.wi, hi.normal));
            specular = is_specular(mat.bxdf);
            ro = hi.pos;
            rd = ms.wi;
            scatter_pdf = ms.pdf;
            if (depth >= p.rr_depth) {
                float q = std::max(std::max(beta.x, std::max(beta.y, beta.z)), 0.05f);
                if (rng.next() > q) break;
                beta = beta / q;
            }
        }
        mark(seg - 1, 8);
        if (std::isfinite(L.x) && std::isfinite(L.y) && std::isfinite(L.z)) {
            result = result + L / (float)p.samples_per_pixel;
            s1[0] += L.x;
            s1[1] += L.y;
            s1[2] += L.z;
            s2[0] += (double)L.x * L.x;
            s2[1] += (double)L.y * L.y;
            s2[2] += (double)L.z * L.z;
        }
    }
    film[0] = result.x;
    film[1] = result.y;
    film[2] = result.z;
    film[3] = 1.0f;
    for (int k = 0; k < 3; ++k) {
        sum[k] = s1[k];
        sumsq[k] = s2[k];
    }
}

template <class F>
void parallel_for(int64_t n, int threads, F fn)
{
    if (threads <= 1 || n < 2) {
        for (int64_t i = 0; i < n; ++i) fn(i);
        return;
    }
    std::atomic<int64_t> next(0);
    std::vector<std::thread> pool;
    for (int t = 0; t < threads; ++t)
        pool.emplace_back([&]() {
            for (;;) {
                int64_t i = next.fetch_add(1);
                if (i >= n) break;
                fn(i);
            }
        });
    for (auto& th : pool) th.join();
}

}  // namespace

extern "C" {

void oracle_pcg_uniforms(uint64_t initstate, uint64_t initseq, int n, float* out)
{
    Pcg32 g;
    g.seed(initstate, initseq);
    for (int i = 0; i < n; ++i) out[i] = g.uniform();
}

float oracle_hash_uniform(uint32_t seed, uint32_t pixel, uint32_t sample, uint32_t dim)
{
    return hash_u(hash_key(seed, pixel, sample), dim);
}

// Disney batch inputs: PCG32(initstate = point index, initseq = 0), draw order
// normal(2) wo(2) color(3) metallic subsurface specular specularTint
// anisotropic sheen sheenTint clearcoat clearcoatGloss roughness rnd(4).
void oracle_bxdf_generate(int64_t first, int64_t n, float* normal, float* wo, float* color, float* params,
                          float* rnd4)
{
    for (int64_t k = 0; k < n; ++k) {
        Pcg32 g;
        g.seed((uint64_t)(first + k), 0);
        float u[21];
        for (int j = 0; j < 21; ++j) u[j] = g.uniform();
        // uniform direction on the sphere (basic.h:83-89)
        float z = 1.0f - 2.0f * u[0];
        float r = std::sqrt(std::max(0.0f, 1.0f - z * z));
        float phi = 2.0f * (float)M_PI * u[1];
        F3 nn(r * std::cos(phi), r * std::sin(phi), z);
        // uniform hemisphere about n (basic.h:70-76) in Onb(n)
        float hz = u[2];
        float hr = std::sqrt(std::max(0.0f, 1.0f - hz * hz));
        float hphi = 2.0f * (float)M_PI * u[3];
        F3 wl(hr * std::cos(hphi), hr * std::sin(hphi), hz);
        Onb<float> ob = Onb<float>::from_n(nn);
        F3 ww = ob.to_world(wl);
        normal[3 * k] = nn.x;
        normal[3 * k + 1] = nn.y;
        normal[3 * k + 2] = nn.z;
        wo[3 * k] = ww.x;
        wo[3 * k + 1] = ww.y;
        wo[3 * k + 2] = ww.z;
        color[3 * k] = u[4];
        color[3 * k + 1] = u[5];
        color[3 * k + 2] = u[6];
        float* P = params + 12 * k;
        P[0] = 1.5f;           // ior
        P[1] = u[7];           // metallic
        P[2] = u[8];           // subsurface
        P[4] = u[9];           // specular
        P[5] = u[10];          // specularTint
        P[6] = u[11];          // anisotropic
        P[7] = u[12];          // sheen
        P[8] = u[13];          // sheenTint
        P[9] = u[14];          // clearcoat
        P[10] = u[15];         // clearcoatGloss
        P[3] = 0.05f + 0.95f * u[16];  // roughness
        P[11] = 0.0f;          // specTrans
        for (int j = 0; j < 4; ++j) rnd4[4 * k + j] = u[17 + j];
    }
}

void oracle_bxdf_sample(int precision, int type, int64_t n, const float* normal, const float* wo, const float* color,
                        const float* params, const float* rnd, double* wi, double* f, double* pdf, int32_t* delta)
{
    oracle_bxdf_sample_mt(precision, type, n, normal, wo, color, params, rnd, wi, f, pdf, delta, 1);
}

// The same, points split over `threads` host threads (chunks of 4096).
void oracle_bxdf_sample_mt(int precision, int type, int64_t n, const float* normal, const float* wo,
                           const float* color, const float* params, const float* rnd, double* wi, double* f,
                           double* pdf, int32_t* delta, int threads)
{
    const int64_t chunk = 4096;
    parallel_for((n + chunk - 1) / chunk, threads, [&](int64_t c) {
    for (int64_t k = c * chunk; k < std::min(n, (c + 1) * chunk); ++k) {
        if (precision == 64) {
            Bx<double> b = bx_from<double>(type, params + 12 * k);
            Onb<double> ob = Onb<double>::from_n(cvt<double>(normal + 3 * k));
            BSample<double> s = mat_sample(b, ob, cvt<double>(wo + 3 * k), (double)rnd[2 * k], (double)rnd[2 * k + 1],
                                           cvt<double>(color + 3 * k));
            wi[3 * k] = s.wi.x; wi[3 * k + 1] = s.wi.y; wi[3 * k + 2] = s.wi.z;
            f[3 * k] = s.f.x; f[3 * k + 1] = s.f.y; f[3 * k + 2] = s.f.z;
            pdf[k] = s.pdf;
            delta[k] = s.delta;
        } else {
            Bx<float> b = bx_from<float>(type, params + 12 * k);
            Onb<float> ob = Onb<float>::from_n(cvt<float>(normal + 3 * k));
            BSample<float> s = mat_sample(b, ob, cvt<float>(wo + 3 * k), rnd[2 * k], rnd[2 * k + 1],
                                          cvt<float>(color + 3 * k));
            wi[3 * k] = s.wi.x; wi[3 * k + 1] = s.wi.y; wi[3 * k + 2] = s.wi.z;
            f[3 * k] = s.f.x; f[3 * k + 1] = s.f.y; f[3 * k + 2] = s.f.z;
            pdf[k] = s.pdf;
            delta[k] = s.delta;
        }
    }
    });
}

void oracle_bxdf_eval_pdf(int precision, int type, int64_t n, const float* normal, const float* wo, const float* color,
                          const float* params, const double* wi, double* f, double* pdf)
{
    for (int64_t k = 0; k < n; ++k) {
        if (precision == 64) {
            Bx<double> b = bx_from<double>(type, params + 12 * k);
            Onb<double> ob = Onb<double>::from_n(cvt<double>(normal + 3 * k));
            V3<double> w(wi[3 * k], wi[3 * k + 1], wi[3 * k + 2]);
            V3<double> o = cvt<double>(wo + 3 * k), c = cvt<double>(color + 3 * k);
            V3<double> fv = mat_eval(b, ob, w, o, c);
            f[3 * k] = fv.x; f[3 * k + 1] = fv.y; f[3 * k + 2] = fv.z;
            pdf[k] = mat_pdf(b, ob, w, o, c);
        } else {
            Bx<float> b = bx_from<float>(type, params + 12 * k);
            Onb<float> ob = Onb<float>::from_n(cvt<float>(normal + 3 * k));
            V3<float> w((float)wi[3 * k], (float)wi[3 * k + 1], (float)wi[3 * k + 2]);
            V3<float> o = cvt<float>(wo + 3 * k), c = cvt<float>(color + 3 * k);
            V3<float> fv = mat_eval(b, ob, w, o, c);
            f[3 * k] = fv.x; f[3 * k + 1] = fv.y; f[3 * k + 2] = fv.z;
            pdf[k] = mat_pdf(b, ob, w, o, c);
        }
    }
}

oracle_scene* oracle_scene_create(const srt_scene_desc* d)
{
    if (!d || d->num_instances < 0 || d->num_meshes < 0) return nullptr;
    oracle_scene* s = new oracle_scene();
    s->mats.assign(d->materials, d->materials + d->num_materials);
    for (int i = 0; i < d->num_meshes; ++i) {
        const srt_mesh& m = d->meshes[i];
        OMesh om;
        om.material = m.material_id;
        for (int k = 0; k < m.num_vertices; ++k) {
            om.v.push_back(cvt<float>(m.vertices + 3 * k));
            if (m.normals) om.n.push_back(cvt<float>(m.normals + 3 * k));
            if (m.tangents) om.tg.push_back(cvt<float>(m.tangents + 3 * k));
        }
        if (m.texcoords) om.tc.assign(m.texcoords, m.texcoords + 2 * (size_t)m.num_vertices);
        om.idx.assign(m.indices, m.indices + 3 * (size_t)m.num_faces);
        // TriangleMesh::compute_area (src/scene/mesh.cpp:3-18)
        om.area_cdf.resize(m.num_faces);
        for (int f = 0; f < m.num_faces; ++f) {
            F3 v0 = om.v[om.idx[3 * f]], v1 = om.v[om.idx[3 * f + 1]], v2 = om.v[om.idx[3 * f + 2]];
            float A = 0.5f * length(cross(v1 - v0, v2 - v0));
            om.area += A;
            om.area_cdf[f] = om.area;
        }
        for (int f = 0; f < m.num_faces; ++f) om.area_cdf[f] /= om.area;
        s->meshes.push_back(std::move(om));
    }
    int64_t base = 0;
    for (int i = 0; i < d->num_instances; ++i) {
        OInst in;
        in.mesh = d->instances[i].mesh_id;
        std::memcpy(in.xf.m, d->instances[i].transform, sizeof(in.xf.m));
        in.light_id = -1;
        in.prim_base = base;
        const OMesh& m = s->meshes[in.mesh];
        int nf = (int)m.area_cdf.size();
        for (int f = 0; f < nf; ++f) {
            s->w0.push_back(in.xf.point(m.v[m.idx[3 * f]]));
            s->w1.push_back(in.xf.point(m.v[m.idx[3 * f + 1]]));
            s->w2.push_back(in.xf.point(m.v[m.idx[3 * f + 2]]));
            s->tri_inst.push_back(i);
            s->tri_face.push_back(f);
        }
        base += nf;
        s->inst.push_back(in);
    }
    // light table (Scene::build_gscene_instances, scene.cu:370-417)
    float wsum = 0.0f;
    for (int i = 0; i < (int)s->inst.size(); ++i) {
        const OMesh& m = s->meshes[s->inst[i].mesh];
        const srt_material& mat = s->mats[m.material];
        if (mat.intensity <= 0.0f) continue;
        s->inst[i].light_id = (int)s->light_inst.size();
        s->light_inst.push_back(i);
        wsum += mat.intensity * m.area;
        s->weight_cdf.push_back(wsum);
    }
    for (float& c : s->weight_cdf) c /= wsum;
    s->weight_sum = wsum;
    s->env = cvt<float>(d->env_color);
    s->cam = make_camera(d->camera);
    for (int i = 0; i < d->num_textures; ++i) {
        const srt_texture& t = d->textures[i];
        OTex o;
        o.w = t.width;
        o.h = t.height;
        o.lin.resize(4 * (size_t)t.width * t.height);
        for (size_t k = 0; k < o.lin.size(); ++k) {
            if (t.format == SRT_TEXTURE_RGBA8) {
                const double c = static_cast<const uint8_t*>(t.pixels)[k] / 255.0;
                o.lin[k] = (k % 4 == 3) ? c : (c <= 0.04045 ? c / 12.92 : std::pow((c + 0.055) / 1.055, 2.4));
            } else {
                o.lin[k] = static_cast<const float*>(t.pixels)[k];
            }
        }
        s->tex.push_back(std::move(o));
    }
    if (d->material_textures) s->mat_tex.assign(d->material_textures, d->material_textures + 2 * d->num_materials);
    s->env_map = d->env_map - 1;
    return s;
}

void oracle_texture_lookup(const oracle_scene* s, int texture, int64_t n, const float* uv, float* out)
{
    for (int64_t i = 0; i < n; ++i) s->tex[texture].fetch4(uv[2 * i], uv[2 * i + 1], out + 4 * i);
}

void oracle_scene_destroy(oracle_scene* s) { delete s; }
int64_t oracle_scene_num_triangles(const oracle_scene* s) { return (int64_t)s->w0.size(); }
float oracle_scene_light_weight_sum(const oracle_scene* s) { return s->weight_sum; }

void oracle_scene_build_bvh(oracle_scene* s)
{
    int64_t n = (int64_t)s->w0.size();
    std::vector<BuildRef> refs(n);
    for (int64_t i = 0; i < n; ++i) {
        F3 a = s->w0[i], b = s->w1[i], c = s->w2[i];
        BuildRef& r = refs[i];
        r.bmin[0] = std::min(a.x, std::min(b.x, c.x));
        r.bmin[1] = std::min(a.y, std::min(b.y, c.y));
        r.bmin[2] = std::min(a.z, std::min(b.z, c.z));
        r.bmax[0] = std::max(a.x, std::max(b.x, c.x));
        r.bmax[1] = std::max(a.y, std::max(b.y, c.y));
        r.bmax[2] = std::max(a.z, std::max(b.z, c.z));
        for (int k = 0; k < 3; ++k) r.c[k] = 0.5f * (r.bmin[k] + r.bmax[k]);
    }
    s->prim.resize(n);
    for (int64_t i = 0; i < n; ++i) s->prim[i] = (int32_t)i;
    s->nodes.clear();
    s->nodes.reserve(2 * n / 3 + 4);
    s->nodes.push_back(BNode());
    if (n > 0) build_rec(*s, refs, 0, 0, (int)n);
}

void oracle_trace_closest(const oracle_scene* s, const float* rays, int64_t n, float* hits, float* edge, int use_bvh,
                          int threads)
{
    parallel_for(n, threads, [&](int64_t i) {
        const float* r = rays + 8 * i;
        Hit h = trace(*s, F3(r[0], r[1], r[2]), F3(r[4], r[5], r[6]), r[3], r[7], false, use_bvh != 0);
        float* o = hits + 4 * i;
        int32_t pid = (int32_t)h.prim;
        o[0] = h.prim < 0 ? r[7] : h.t;
        o[1] = h.u;
        o[2] = h.v;
        std::memcpy(&o[3], &pid, 4);
        if (edge) edge[i] = h.prim < 0 ? 1.0f : std::min(std::min(h.u, h.v), 1.0f - h.u - h.v);
    });
}

void oracle_trace_shadow(const oracle_scene* s, const float* rays, int64_t n, int32_t* visible, int use_bvh,
                         int threads)
{
    parallel_for(n, threads, [&](int64_t i) {
        const float* r = rays + 8 * i;
        Hit h = trace(*s, F3(r[0], r[1], r[2]), F3(r[4], r[5], r[6]), r[3], r[7], true, use_bvh != 0);
        visible[i] = h.prim < 0 ? 1 : 0;
    });
}

void oracle_camera_rays(const srt_camera_desc* cam, int64_t n, const float* xy, float* rays)
{
    Camera k = make_camera(*cam);
    for (int64_t i = 0; i < n; ++i) {
        F3 o, d;
        camera_ray(k, xy[2 * i], xy[2 * i + 1], o, d);
        float* r = rays + 8 * i;
        r[0] = o.x; r[1] = o.y; r[2] = o.z; r[3] = 0.0f;
        r[4] = d.x; r[5] = d.y; r[6] = d.z; r[7] = 1e16f;
    }
}

void oracle_hitinfo(const oracle_scene* s, int64_t n, const int32_t* prim, const float* uv, float* out)
{
    for (int64_t i = 0; i < n; ++i) {
        HitInfo h = hit_info(*s, prim[i], uv[2 * i], uv[2 * i + 1]);
        float v[15] = {h.pos.x,   h.pos.y,   h.pos.z,   h.normal.x, h.normal.y, h.normal.z, h.onb.z.x, h.onb.z.y,
                       h.onb.z.z, h.onb.x.x, h.onb.x.y, h.onb.x.z,  h.onb.y.x,  h.onb.y.y,  h.onb.y.z};
        std::memcpy(out + 15 * i, v, sizeof(v));
    }
}

void oracle_light_sample(const oracle_scene* s, int64_t n, const float* u2, int fixed_remap, float* out)
{
    for (int64_t i = 0; i < n; ++i) {
        LSample ls = light_sample(*s, u2[2 * i], u2[2 * i + 1], fixed_remap != 0);
        float* o = out + 10 * i;
        o[0] = ls.pos.x; o[1] = ls.pos.y; o[2] = ls.pos.z;
        o[3] = ls.normal.x; o[4] = ls.normal.y; o[5] = ls.normal.z;
        o[6] = ls.emission.x; o[7] = ls.emission.y; o[8] = ls.emission.z;
        o[9] = ls.pdf;
    }
}

// oracle_render with the per-pixel segment bytes of render_pixel (events:
// uint8[cw * ch * ev_max], zeroed by the caller; may be null).
int oracle_render_events(const oracle_scene* s, int w, int h, int x0, int y0, int cw, int ch,
                         const srt_pt_params* p, int use_bvh, int threads, float* film, double* sum, double* sumsq,
                         int64_t* counters, uint8_t* events, int ev_max)
{
    if (!s || !p || w <= 0 || h <= 0 || x0 < 0 || y0 < 0 || x0 + cw > w || y0 + ch > h) return 1;
    if (s->light_inst.empty() && p->use_nee) return 2;
    if (events && ev_max <= 0) return 1;
    std::vector<int64_t> cnt((size_t)cw * ch * 4, 0);
    parallel_for((int64_t)cw * ch, threads, [&](int64_t k) {
        int ix = x0 + (int)(k % cw), iy = y0 + (int)(k / cw);
        render_pixel(*s, w, h, ix, iy, *p, use_bvh != 0, film + 4 * k, sum + 3 * k, sumsq + 3 * k, &cnt[4 * k],
                     events ? events + (size_t)k * ev_max : nullptr, events ? ev_max : 0);
    });
    for (int j = 0; j < 4; ++j) counters[j] = 0;
    for (size_t k = 0; k < (size_t)cw * ch; ++k)
        for (int j = 0; j < 4; ++j) counters[j] += cnt[4 * k + j];
    return 0;
}

int oracle_render_pixels(const oracle_scene* s, int w, int h, const int32_t* pixels, int64_t n,
                         const srt_pt_params* p, int use_bvh, int threads, float* film, double* sum,
                         double* sumsq, int64_t* counters)
{
    if (!s || !p || w <= 0 || h <= 0 || n < 0 || (n > 0 && !pixels)) return 1;
    if (s->light_inst.empty() && p->use_nee) return 2;
    for (int64_t k = 0; k < n; ++k)
        if (pixels[k] < 0 || (int64_t)pixels[k] >= (int64_t)w * h) return 1;
    std::vector<int64_t> cnt((size_t)n * 4, 0);
    parallel_for(n, threads, [&](int64_t k) {
        int ix = pixels[k] % w, iy = pixels[k] / w;
        render_pixel(*s, w, h, ix, iy, *p, use_bvh != 0, film + 4 * k, sum + 3 * k, sumsq + 3 * k, &cnt[4 * k]);
    });
    for (int j = 0; j < 4; ++j) counters[j] = 0;
    for (size_t k = 0; k < (size_t)n; ++k)
        for (int j = 0; j < 4; ++j) counters[j] += cnt[4 * k + j];
    return 0;
}

int oracle_render(const oracle_scene* s, int w, int h, int x0, int y0, int cw, int ch, const srt_pt_params* p,
                  int use_bvh, int threads, float* film, double* sum, double* sumsq, int64_t* counters)
{
    return oracle_render_events(s, w, h, x0, y0, cw, ch, p, use_bvh, threads, film, sum, sumsq, counters, nullptr,
                                0);
}

// LightTracer raygen (src/shader/integrator/light_tracer.cu:57-175) for
// launch index `idx`; splats go to `film` (double RGB per pixel).
void light_trace_index(const oracle_scene& s, int w, int h, int64_t idx, const srt_pt_params& p, bool use_bvh,
                       double* film, int64_t* cnt)
{
    const bool fixed = (p.flags & SRT_PT_FIXED_CDF_REMAP) != 0;
    const Camera& k = s.cam;
    const float aspect = (float)w / (float)h;
    Rng rng;
    rng.mode = SRT_RNG_CURAND;
    rng.init_curand(p.seed, (int)idx);
    // Camera::get_xy (camera.h:142-148)
    auto get_xy = [&](F3 dir, float& x, float& y) {
        F3 m = dir * -1.0f;
        F3 l(dot(m, k.x), dot(m, k.y), dot(m, k.z));
        float px = l.x / l.z, py = l.y / l.z;
        x = px / k.nw + 0.5f;
        y = py / k.nh + 0.5f;
    };
    auto splat = [&](float x, float y, F3 v) {
        int pix = (int)(x * (float)w) + (int)(y * (float)h) * w;
        film[3 * pix] += v.x;
        film[3 * pix + 1] += v.y;
        film[3 * pix + 2] += v.z;
    };
    for (int i = 0; i < p.samples_per_pixel; ++i) {
        float l1 = rng.next();
        float l2 = rng.next();
        LSample ls = light_sample(s, l1, l2, fixed);
        float s1 = rng.next();
        float s2 = rng.next();
        float sz = 1.0f - 2.0f * s1;  // uniform_sample_sphere (basic.h:83-89)
        float sr = std::sqrt(1.0f - sz * sz);
        float phi = 2.0f * (float)M_PI * s2;
        F3 wi = normalize(ls.normal + F3(sr * std::cos(phi), sr * std::sin(phi), sz));
        F3 ro = ls.pos, rd = wi;
        float cos_theta = dot(wi, ls.normal);
        float pw = cos_theta * (float)M_1_PI;
        F3 beta = ls.emission * cos_theta / ls.pdf;
        bool specular = true;
        for (int depth = 0; depth < p.max_depth; ++depth) {
            cnt[0]++;
            Hit hit = trace(s, ro, rd, 1e-3f, 1e16f, false, use_bvh);
            HitInfo hi;
            if (hit.prim >= 0) hi = hit_info(s, hit.prim, hit.u, hit.v);
            if (specular) {
                F3 to_cam = k.pos - ro;
                float t = length(to_cam);
                to_cam = to_cam / t;
                if ((hit.prim < 0 || t < length(hi.pos - ro)) && dot(to_cam, rd) > 1.0f - 1e-6f) {
                    float x, y;
                    get_xy(rd, x, y);
                    if (x >= 0.0f && x < 1.0f && y >= 0.0f && y < 1.0f) splat(x, y, beta / pw / (float)p.samples_per_pixel);
                }
            }
            if (hit.prim < 0) break;
            const srt_material& mat = s.mats[hi.mat];
            if (mat.intensity > 0.0f) break;
            Bx<float> bx = bx_of(mat.bxdf);
            float cos_i = dot(rd * -1.0f, hi.normal);
            if (cos_i < 0.0f) hi.normal = -hi.normal;
            if (!is_specular(mat.bxdf)) {
                F3 sd = normalize(k.pos - hi.pos);
                float x, y;
                get_xy(sd, x, y);
                if (x >= 0.0f && x < 1.0f && y >= 0.0f && y < 1.0f) {
                    float t = length(k.pos - hi.pos);
                    cnt[1]++;
                    Hit sh = trace(s, hi.pos, sd, 1e-3f, t - 1e-3f, true, use_bvh);
                    if (sh.prim < 0) {
                        F3 fv = mat_eval(bx, hi.onb, rd * -1.0f, sd, hi.color);
                        F3 L = beta * aspect * fv * dot(sd, hi.normal) / t / t / pw;
                        splat(x, y, L / (float)p.samples_per_pixel);
                    }
                }
            }
            float u1 = rng.next();
            float u2 = rng.next();
            BSample<float> ms = mat_sample(bx, hi.onb, rd * -1.0f, u1, u2, hi.color);
            if (ms.pdf <= 1e-5f) break;
            beta = beta * mat_eval(bx, hi.onb, rd * -1.0f, ms.wi, hi.color) * std::fabs(dot(ms.wi, hi.normal)) / pw;
            pw = ms.pdf;
            specular = is_specular(mat.bxdf);
            ro = hi.pos;
            rd = ms.wi;
            if (depth >= p.rr_depth) {
                float q = std::min(std::max(beta.x, std::max(beta.y, beta.z)), 0.95f);
                if (rng.next() > q) break;
                beta = beta / q;
            }
        }
    }
}

// srt_lt_render's restatement: film (w*h RGB, double) is the sum of all
// splats; counters[0] closest rays, [1] camera connections traced.
int oracle_light_trace(const oracle_scene* s, int w, int h, const srt_pt_params* p, int use_bvh, int threads,
                       double* film, int64_t* counters)
{
    if (!s || !p || w <= 0 || h <= 0) return 1;
    if (s->light_inst.empty()) return 2;
    const int64_t n = (int64_t)w * h;
    const int nt = std::max(1, threads);
    std::vector<std::vector<double>> part(nt, std::vector<double>(3 * (size_t)n, 0.0));
    std::vector<int64_t> cnt(2 * (size_t)nt, 0);
    std::vector<std::thread> pool;
    for (int t = 0; t < nt; ++t)
        pool.emplace_back([&, t]() {
            for (int64_t idx = t; idx < n; idx += nt)
                light_trace_index(*s, w, h, idx, *p, use_bvh != 0, part[t].data(), &cnt[2 * t]);
        });
    for (auto& th : pool) th.join();
    for (int64_t i = 0; i < 3 * n; ++i) {
        film[i] = 0.0;
        for (int t = 0; t < nt; ++t) film[i] += part[t][i];
    }
    counters[0] = counters[1] = 0;
    for (int t = 0; t < nt; ++t) {
        counters[0] += cnt[2 * t];
        counters[1] += cnt[2 * t + 1];
    }
    return 0;
}

// ---- NeuralRadiosity (src/shader/npr/nr_lhs.cu, nr_rhs.cu) -------------

// the 12 network inputs of a hit (nr_lhs.cu:69-86)
static void nr_input(float* in, F3 pos, F3 rd, F3 n, F3 c)
{
    F3 d = (rd * -1.0f + F3(1.0f)) * 0.5f;
    F3 m = (n + F3(1.0f)) * 0.5f;
    const float v[12] = {pos.x, pos.y, pos.z, d.x, d.y, d.z, m.x, m.y, m.z, c.x, c.y, c.z};
    for (int k = 0; k < 12; ++k) in[k] = v[k];
}

// One sample of the LHS (type 0) or RHS (type 1) raygen for every pixel.
int oracle_nr_trace(const oracle_scene* sp, int w, int h, int type, int seed, int use_bvh, uint8_t* mask, float* base,
                    float* weight, float* inputs)
{
    const oracle_scene& s = *sp;
    if (w <= 0 || h <= 0) return 1;
    if (type == 1 && s.light_inst.empty()) return 2;
    for (int64_t idx = 0; idx < (int64_t)w * h; ++idx) {
        const int ix = (int)(idx % w), iy = (int)(idx / w);
        F3 b(0.0f), wgt(0.0f);
        uint8_t mk = 1;
        float* in = inputs + 12 * idx;
        for (int k = 0; k < 12; ++k) in[k] = 0.0f;
        Rng rng;
        rng.mode = SRT_RNG_CURAND;
        rng.init_curand(seed, (int)idx);
        float jx = rng.next();
        float jy = rng.next();
        F3 ro, rd;
        camera_ray(s.cam, ((float)ix + jx) / (float)w, ((float)iy + jy) / (float)h, ro, rd);
        Hit hit = trace(s, ro, rd, 1e-3f, 1e16f, false, use_bvh != 0);
        if (hit.prim >= 0) {
            HitInfo hi = hit_info(s, hit.prim, hit.u, hit.v);
            const srt_material& mat = s.mats[hi.mat];
            if (mat.intensity > 0.0f) {
                b = hi.emission;
            } else if (type == 0) {
                mk = 0;
                nr_input(in, hi.pos, rd, hi.normal, hi.color);
            } else {
                Bx<float> bx = bx_of(mat.bxdf);
                const bool transmissive = is_transmissive(mat.bxdf);
                if (!is_specular(mat.bxdf)) {
                    float l1 = rng.next();
                    float l2 = rng.next();
                    LSample ls = light_sample(s, l1, l2, false);
                    F3 sd = normalize(ls.pos - hi.pos);
                    float cos_o = dot(hi.normal, sd);
                    float cos_l = dot(ls.normal, sd * -1.0f);
                    float t = length(ls.pos - hi.pos);
                    if (cos_l > 1e-4f && ls.pdf > 1e-4f && t > 1e-3f && (cos_o > 0.0f || transmissive)) {
                        Hit sh = trace(s, hi.pos, sd, 1e-3f, t - 1e-3f, true, use_bvh != 0);
                        if (sh.prim < 0) {
                            float lpdf = ls.pdf * t * t / cos_l;
                            float mpdf = mat_pdf(bx, hi.onb, sd, rd * -1.0f, hi.color);
                            float mis = lpdf / (lpdf + mpdf);
                            b = mat_eval(bx, hi.onb, sd, rd * -1.0f, hi.color) * std::fabs(cos_o) * ls.emission * mis /
                                lpdf;
                        }
                    }
                }
                float u1 = rng.next();
                float u2 = rng.next();
                BSample<float> ms = mat_sample(bx, hi.onb, rd * -1.0f, u1, u2, hi.color);
                float cos_t = dot(ms.wi, hi.normal);
                if (!(ms.pdf <= 1e-4f) && !(cos_t < 0.0f && !transmissive)) {
                    F3 wv = ms.f / ms.pdf * (ms.delta ? 1.0f : std::fabs(cos_t));
                    Hit h2 = trace(s, hi.pos, ms.wi, 1e-3f, 1e16f, false, use_bvh != 0);
                    if (h2.prim >= 0) {
                        HitInfo h2i = hit_info(s, h2.prim, h2.u, h2.v);
                        const srt_material& m2 = s.mats[h2i.mat];
                        if (m2.intensity > 0.0f) {
                            float cos_i = dot(h2i.normal, ms.wi * -1.0f);
                            if (cos_i > 1e-4f) {
                                float t2 = dot(h2i.pos - hi.pos, h2i.pos - hi.pos);
                                float lpdf = light_pdf_of(s, h2i.light_id) * t2 / cos_i;
                                float mis = ms.pdf / (ms.pdf + lpdf);
                                b = b + wv * h2i.emission * mis;
                            }
                        } else {
                            mk = 0;
                            wgt = wv;
                            nr_input(in, h2i.pos, ms.wi, h2i.normal, h2i.color);
                        }
                    }
                }
            }
        }
        mask[idx] = mk;
        base[3 * idx] = b.x;
        base[3 * idx + 1] = b.y;
        base[3 * idx + 2] = b.z;
        if (weight) {
            weight[3 * idx] = wgt.x;
            weight[3 * idx + 1] = wgt.y;
            weight[3 * idx + 2] = wgt.z;
        }
    }
    return 0;
}

// float -> bfloat16 -> float, round to nearest even (NaN kept quiet)
static float bf16_round(float x)
{
    uint32_t u;
    std::memcpy(&u, &x, 4);
    if ((u & 0x7fffffffu) > 0x7f800000u) {
        u |= 0x00400000u;
    } else {
        u += 0x7fffu + ((u >> 16) & 1u);
    }
    u &= 0xffff0000u;
    float r;
    std::memcpy(&r, &u, 4);
    return r;
}

// The network of the NeuralRadiosity pass, restated from its description
// (hash grid after Mueller et al. 2022 with this library's layout; real
// spherical harmonics; BF16 activations and weights, exact sums).
void oracle_nr_infer(const float* params, int64_t n, const float* inputs, float* out, int threads)
{
    const int L = 8, F = 8, log2T = 19, W = 256, ENC = 96;
    std::vector<int64_t> off(L + 1, 0), res(L), size(L);
    for (int l = 0; l < L; ++l) {
        res[l] = (int64_t)16 << l;
        const int64_t r3 = res[l] * res[l] * res[l];
        size[l] = r3 <= (1ll << log2T) ? r3 : (1ll << log2T);
        off[l + 1] = off[l] + size[l];
    }
    const float* wts = params + off[L] * F;
    const int in_dims[5] = {ENC, W, W, W, W}, out_dims[5] = {W, W, W, W, 16};
    std::vector<int64_t> woff(6, 0);
    for (int l = 0; l < 5; ++l) woff[l + 1] = woff[l] + (int64_t)in_dims[l] * out_dims[l];
    std::vector<float> wb((size_t)woff[5]);
    for (int64_t i = 0; i < woff[5]; ++i) wb[i] = bf16_round(wts[i]);
    parallel_for(n, threads, [&](int64_t q) {
        const float* in = inputs + 12 * q;
        std::vector<float> x(ENC, 1.0f), y(W);
        for (int l = 0; l < L; ++l) {
            const float scale = (float)res[l] - 1.0f;
            const bool dense = size[l] == res[l] * res[l] * res[l];
            const float* g = params + off[l] * F;
            int pi[3];
            float w1[3];
            for (int k = 0; k < 3; ++k) {
                const float sv = in[k] * scale + 0.5f;
                const float fl = std::floor(sv);
                pi[k] = (int)fl;
                const float fr = sv - fl;
                w1[k] = fr * fr * (3.0f - 2.0f * fr);
            }
            float acc[8] = {};
            for (int c = 0; c < 8; ++c) {
                const int dx = c & 1, dy = (c >> 1) & 1, dz = (c >> 2) & 1;
                const float wc = (dx ? w1[0] : 1.0f - w1[0]) * (dy ? w1[1] : 1.0f - w1[1]) * (dz ? w1[2] : 1.0f - w1[2]);
                const uint32_t ux = (uint32_t)(pi[0] + dx), uy = (uint32_t)(pi[1] + dy), uz = (uint32_t)(pi[2] + dz);
                int64_t e;
                if (dense) {
                    const int64_t r = res[l];
                    e = (((int64_t)(int32_t)ux % r + r) % r) + (((int64_t)(int32_t)uy % r + r) % r) * r +
                        (((int64_t)(int32_t)uz % r + r) % r) * r * r;
                } else {
                    e = (int64_t)((ux * 1u ^ uy * 2654435761u ^ uz * 805459861u) & ((1u << log2T) - 1u));
                }
                for (int k = 0; k < F; ++k) acc[k] += wc * g[e * F + k];
            }
            for (int k = 0; k < F; ++k) x[l * F + k] = bf16_round(acc[k]);
        }
        auto sh3 = [](float a, float b2, float c, float* o) {
            o[0] = 0.28209479177387814f;
            o[1] = -0.48860251190291987f * b2;
            o[2] = 0.48860251190291987f * c;
            o[3] = -0.48860251190291987f * a;
            o[4] = 1.0925484305920792f * a * b2;
            o[5] = -1.0925484305920792f * b2 * c;
            o[6] = 0.94617469575755997f * c * c - 0.31539156525251999f;
            o[7] = -1.0925484305920792f * a * c;
            o[8] = 0.54627421529603959f * (a * a - b2 * b2);
        };
        float sd[9], sn[9];
        sh3(in[3] * 2.0f - 1.0f, in[4] * 2.0f - 1.0f, in[5] * 2.0f - 1.0f, sd);
        sh3(in[6] * 2.0f - 1.0f, in[7] * 2.0f - 1.0f, in[8] * 2.0f - 1.0f, sn);
        for (int k = 0; k < 9; ++k) x[64 + k] = bf16_round(sd[k]);
        for (int k = 0; k < 9; ++k) x[73 + k] = bf16_round(sn[k]);
        for (int k = 0; k < 3; ++k) x[82 + k] = bf16_round(in[9 + k]);
        std::vector<float> cur = x;
        for (int l = 0; l < 5; ++l) {
            std::vector<float> nxt((size_t)out_dims[l]);
            for (int o = 0; o < out_dims[l]; ++o) {
                double sacc = 0.0;
                const float* wr = &wb[woff[l] + (int64_t)o * in_dims[l]];
                for (int i = 0; i < in_dims[l]; ++i) sacc += (double)wr[i] * (double)cur[i];
                float v = (float)sacc;
                if (l < 4) v = bf16_round(std::max(v, 0.0f));
                nxt[o] = v;
            }
            cur.swap(nxt);
        }
        for (int k = 0; k < 3; ++k) out[3 * q + k] = cur[k];
    });
}

// Accumulate::render (src/passes/postprocess/accumulate.cu:10-29)
void oracle_accumulate(float* film, float* acc, int64_t n, int frame_count)
{
    float w = 1.0f / (float)(frame_count + 1);
    for (int64_t i = 0; i < 4 * n; ++i) {
        acc[i] = acc[i] * (1.0f - w) + film[i] * w;
        film[i] = acc[i];
    }
}

// ToneMapping::render (src/passes/postprocess/tonemapping.cu:5-70)
void oracle_tonemap(float* film, int64_t n, int type, float exposure, int use_gamma)
{
    float ex = std::pow(2.0f, exposure);
    for (int64_t i = 0; i < n; ++i) {
        float* px = film + 4 * i;
        F3 c = F3(px[0], px[1], px[2]) * ex;
        if (type == SRT_TONE_CLAMP) {
            c = F3(clampv(c.x, 0.0f, 1.0f), clampv(c.y, 0.0f, 1.0f), clampv(c.z, 0.0f, 1.0f));
        } else if (type == SRT_TONE_REINHARD) {
            float l = lum(c);
            c = c / (1.0f + l);
        } else if (type == SRT_TONE_UNCHARTED2) {
            const float A = 0.15f, B = 0.50f, C = 0.10f, D = 0.20f, E = 0.02f, F = 0.30f, W = 11.2f;
            auto curve = [&](F3 x) {
                return (x * (A * x + F3(C * B)) + F3(D * E)) / (x * (A * x + F3(B)) + F3(D * F)) - F3(E / F);
            };
            float white = ((W * (A * W + C * B) + D * E) / (W * (A * W + B) + D * F)) - E / F;
            c = curve(c) / white;
        } else if (type == SRT_TONE_ACES) {
            c = c * 0.6f;
            const float a = 2.51f, b = 0.03f, cc = 2.43f, d = 0.59f, e = 0.14f;
            c = (c * (a * c + F3(b))) / (c * (cc * c + F3(d)) + F3(e));
            c = F3(clampv(c.x, 0.0f, 1.0f), clampv(c.y, 0.0f, 1.0f), clampv(c.z, 0.0f, 1.0f));
        }
        if (use_gamma) {
            float g = 1.0f / 2.2f;
            c = F3(std::pow(c.x, g), std::pow(c.y, g), std::pow(c.z, g));
        }
        px[0] = c.x;
        px[1] = c.y;
        px[2] = c.z;
        px[3] = 1.0f;
    }
}

// Metrics::cal_pixel / cal_image (src/utils/metrics.h:16-70): errors are
// sorted ascending and the mean of the first floor(n * (1 - discard/100))
// is reported (measure.cu:46-49).  The sum is taken in double here.
double oracle_metric(const float* x, const float* ref, int64_t n, int type, float discard, float* errors)
{
    const float eps = 1e-6f;
    std::vector<float> e(n);
    for (int64_t i = 0; i < n; ++i) {
        F3 a(x[4 * i], x[4 * i + 1], x[4 * i + 2]), r(ref[4 * i], ref[4 * i + 1], ref[4 * i + 2]);
        float v = 0.0f;
        if (type == SRT_METRIC_MSE) {
            v = dot(a - r, a - r) / 3.0f;
        } else if (type == SRT_METRIC_MAPE) {
            F3 t = F3(std::fabs(a.x - r.x), std::fabs(a.y - r.y), std::fabs(a.z - r.z)) / (r + F3(eps));
            v = dot(t, F3(1.0f)) / 3.0f;
        } else if (type == SRT_METRIC_SMAPE) {
            F3 t = 2.0f * F3(std::fabs(a.x - r.x), std::fabs(a.y - r.y), std::fabs(a.z - r.z)) / (a + r + F3(eps));
            v = dot(t, F3(1.0f)) / 3.0f;
        } else {
            F3 t = (a - r) / (r + F3(eps));
            v = dot(t, t) / 3.0f;
        }
        e[i] = v;
        if (errors) errors[i] = v;
    }
    std::sort(e.begin(), e.end());
    int64_t keep = (int64_t)((float)n * (1.0f - discard / 100.0f));
    if (keep <= 0) return NAN;  // the reference divides 0 by 0 here
    double acc = 0.0;
    for (int64_t i = 0; i < keep; ++i) acc += e[i];
    return acc / (double)keep;
}

}  // extern "C"
