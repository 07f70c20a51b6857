// trace.cuh — closest-hit and any-hit traversal of the 8-wide quantised BVH
// (replaces optixTrace with OPTIX_RAY_FLAG_DISABLE_ANYHIT, path_tracer.cu:75-78
// and :124-127).
//
// Traversal keeps one "node group" (child_base, internal-slot mask, hit
// bits in octant order) in registers and pushes at most one group per
// visited node onto a short per-thread stack held in shared memory, so the
// stack depth is bounded by the tree depth (Ylitie, Karras, Laine, HPG 2017).
// Triangles hit by a node's leaf children are tested right after the node.
// The triangle test is the watertight test of Woop, Benthin and Wald
// (JCGT 2013); u, v are the barycentrics of vertex 1 and 2, as
// optixGetTriangleBarycentrics returns them.
#pragma once

#include "device_types.h"
#include "vmath.h"

namespace srt {

#ifndef SRT_STACK_ENTRIES
#define SRT_STACK_ENTRIES 24
#endif
constexpr int kStackEntries = SRT_STACK_ENTRIES;  // node groups; at most one per tree level

#ifndef SRT_SLAB_MARGIN
#define SRT_SLAB_MARGIN 1.0f  // quantisation steps added to each slab side
#endif

// shadow rays visit children far-to-near: near the origin the first nodes
// hold the origin's own surface, which a ray leaving it does not hit
// (k_shadow 57.9 -> 56.2 ms per benchmark frame against near-to-far)
#ifndef SRT_SHADOW_FAR_FIRST
#define SRT_SHADOW_FAR_FIRST 1
#endif

// resident 128-thread traversal blocks per SM the compiler budgets registers
// for: 7 (72 registers, no spills)
#ifndef SRT_TRACE_MIN_BLOCKS
#define SRT_TRACE_MIN_BLOCKS 7
#endif

struct Hit {
    float t, u, v;
    int32_t tri;  // BVH-order triangle, -1 on miss
};

struct RayPre {
    float3 o;
    float3 idir;
    float sx, sy, sz;
    // packed: kx (bits 0-1), ky (2-3), kz (4-5) of the watertight test's axis
    // permutation, any-hit ray (7: see trav_advance_impl), octant (8-10), child
    // visiting order (11-13: the octant for near-to-far, its complement for
    // far-to-near); one register instead of six
    uint32_t axes;
    __device__ __forceinline__ int kx() const { return (int)(axes & 3u); }
    __device__ __forceinline__ int ky() const { return (int)((axes >> 2) & 3u); }
    __device__ __forceinline__ int kz() const { return (int)((axes >> 4) & 3u); }
    __device__ __forceinline__ uint32_t oct() const { return (axes >> 8) & 7u; }
    __device__ __forceinline__ uint32_t ord() const { return axes >> 11; }
};

__device__ __forceinline__ float comp(float3 v, int k) { return k == 0 ? v.x : (k == 1 ? v.y : v.z); }

// Two-wide FP32 FMA (fma.rn.f32x2, sm_100 and later): one instruction gives
// two round-to-nearest FMAs, each bit-identical to fmaf of the same operands
// (subnormals kept).
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c)
{
    float2 d;
    asm("{\n .reg .b64 a, b, c, d;\n mov.b64 a, {%2, %3};\n mov.b64 b, {%4, %5};\n mov.b64 c, {%6, %7};\n"
        " fma.rn.f32x2 d, a, b, c;\n mov.b64 {%0, %1}, d;\n}"
        : "=f"(d.x), "=f"(d.y)
        : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y), "f"(c.x), "f"(c.y));
    return d;
}
// two-wide round-to-nearest product (mul.rn.f32x2), each lane equal to
// __fmul_rn; only where the product feeds no add (a product feeding a
// two-wide subtract came back contracted)
__device__ __forceinline__ float2 mul2(float2 a, float2 b)
{
    float2 d;
    asm("{\n .reg .b64 a, b, d;\n mov.b64 a, {%2, %3};\n mov.b64 b, {%4, %5};\n mul.rn.f32x2 d, a, b;\n"
        " mov.b64 {%0, %1}, d;\n}"
        : "=f"(d.x), "=f"(d.y)
        : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));
    return d;
}
// two-wide round-to-nearest difference (sub.rn.f32x2); only where no
// product feeds it
__device__ __forceinline__ float2 sub2(float2 a, float2 b)
{
    float2 d;
    asm("{\n .reg .b64 a, b, d;\n mov.b64 a, {%2, %3};\n mov.b64 b, {%4, %5};\n sub.rn.f32x2 d, a, b;\n"
        " mov.b64 {%0, %1}, d;\n}"
        : "=f"(d.x), "=f"(d.y)
        : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));
    return d;
}
__device__ __forceinline__ RayPre make_ray(float3 o, float3 d)
{
    RayPre r;
    r.o = o;
    float ax = fabsf(d.x), ay = fabsf(d.y), az = fabsf(d.z);
    int kz = 0;
    if (ay > ax) kz = 1;
    if (az > fmaxf(ax, ay)) kz = 2;
    int kx = (kz == 2) ? 0 : kz + 1;
    int ky = (kx == 2) ? 0 : kx + 1;
    float dz = comp(d, kz);
    if (dz < 0.0f) {
        int t = kx;
        kx = ky;
        ky = t;
    }
    r.sx = comp(d, kx) / dz;
    r.sy = comp(d, ky) / dz;
    r.sz = 1.0f / dz;
    const float tiny = 1e-20f;
    float3 dd = make_float3(fabsf(d.x) < tiny ? copysignf(tiny, d.x) : d.x,
                            fabsf(d.y) < tiny ? copysignf(tiny, d.y) : d.y,
                            fabsf(d.z) < tiny ? copysignf(tiny, d.z) : d.z);
    r.idir = make_float3(1.0f / dd.x, 1.0f / dd.y, 1.0f / dd.z);
    // octant = signs of idir (a -0 component counts as negative), so that the
    // near slab plane of every child box is its low plane exactly when the bit is clear
    const uint32_t oct = (r.idir.x < 0.0f ? 1u : 0u) | (r.idir.y < 0.0f ? 2u : 0u) | (r.idir.z < 0.0f ? 4u : 0u);
    r.axes = (uint32_t)kx | ((uint32_t)ky << 2) | ((uint32_t)kz << 4) | (oct << 8) | (oct << 11);
    return r;
}

// Watertight ray/triangle test; on a hit in (tmin, tmax) returns t and the
// barycentrics of v1, v2.
__device__ __forceinline__ bool hit_triangle(const RayPre& r, float3 v0, float3 v1, float3 v2, float tmin,
                                             float tmax, float& t, float& b1, float& b2)
{
    float3 A = v0 - r.o, B = v1 - r.o, C = v2 - r.o;
    const int kx = r.kx(), ky = r.ky(), kz = r.kz();
    float az = comp(A, kz), bz = comp(B, kz), cz = comp(C, kz);
    float Ax = comp(A, kx) - r.sx * az, Ay = comp(A, ky) - r.sy * az;
    float Bx = comp(B, kx) - r.sx * bz, By = comp(B, ky) - r.sy * bz;
    float Cx = comp(C, kx) - r.sx * cz, Cy = comp(C, ky) - r.sy * cz;
    float U = Cx * By - Cy * Bx;
    float V = Ax * Cy - Ay * Cx;
    float W = Bx * Ay - By * Ax;
    if ((U < 0.0f || V < 0.0f || W < 0.0f) && (U > 0.0f || V > 0.0f || W > 0.0f)) return false;
    float det = U + V + W;
    if (det == 0.0f) return false;
    float T = U * (r.sz * az) + V * (r.sz * bz) + W * (r.sz * cz);
    float inv = 1.0f / det;
    float tt = T * inv;
    if (!(tt > tmin && tt < tmax)) return false;
    t = tt;
    b1 = V * inv;
    b2 = W * inv;
    return true;
}

// 2^23 + q as a float, q the low (hi = 0) or high (hi = 1) 16 bits of w: one
// byte permute places q under the exponent of 2^23
__device__ __forceinline__ float q23(uint32_t w, int hi)
{
    return __uint_as_float(__byte_perm(w, 0x4B000000u, hi ? 0x7432u : 0x7410u));
}
__device__ __forceinline__ uint32_t word4(uint4 v, int j)
{
    return j == 0 ? v.x : (j == 1 ? v.y : (j == 2 ? v.z : v.w));
}

// A node is fetched with four 256-bit loads (sm_100 and later): the header
// lines, then the six plane lines, near and far picked in registers by the
// ray's octant (733.9 -> 746.4 Msamples/s against eight 128-bit loads with
// the near / far lines chosen by address; k_closest 89.1 -> 87.8 ms and
// k_shadow 55.9 -> 54.1 ms per benchmark frame).
__device__ __forceinline__ void ld_nc_v8(const uint4* p, uint4& a, uint4& b)
{
    asm("ld.global.nc.v8.u32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
        : "=r"(a.x), "=r"(a.y), "=r"(a.z), "=r"(a.w), "=r"(b.x), "=r"(b.y), "=r"(b.z), "=r"(b.w)
        : "l"(p));
}
// 256-bit load of two consecutive float4 (32-byte aligned address)
__device__ __forceinline__ void ld_nc_v8f(const float4* p, float4& a, float4& b)
{
    asm("ld.global.nc.v8.f32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
        : "=f"(a.x), "=f"(a.y), "=f"(a.z), "=f"(a.w), "=f"(b.x), "=f"(b.y), "=f"(b.z), "=f"(b.w)
        : "l"(p));
}
// Triangle ti's three vertices (48 bytes at 48 * ti): three 128-bit loads
// (one 256-bit load of its 32-byte-aligned half plus one 128-bit load
// measured slower: 740.6 -> 720.1 Msamples/s, k_closest 88.0 -> 91.3 ms)
__device__ __forceinline__ void load_tri(const float4* tris, uint32_t ti, float4& a, float4& b, float4& c)
{
    const float4* tp = tris + 3 * (size_t)ti;
    a = __ldg(tp);
    b = __ldg(tp + 1);
    c = __ldg(tp + 2);
}

__device__ __forceinline__ uint4 sel4(bool c, uint4 x, uint4 y)
{
    return make_uint4(c ? x.x : y.x, c ? x.y : y.y, c ? x.z : y.z, c ? x.w : y.w);
}

// three-input minimum / maximum (one instruction on sm_100 and later; NaN
// inputs are ignored as by fminf / fmaxf)
__device__ __forceinline__ float fmax3(float a, float b, float c)
{
    float r;
    asm("max.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
    return r;
}
__device__ __forceinline__ float fmin3(float a, float b, float c)
{
    float r;
    asm("min.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
    return r;
}

// Stack of node groups in shared memory: entry e of thread `lane_id` is at
// stack[e * stride + lane_id] (stride = threads per block: conflict-free).
struct Stack {
    uint2* base;
    int stride;
    int sp;
    __device__ __forceinline__ void push(uint2 g, int& overflow)
    {
        if (sp < kStackEntries) {
            base[sp * stride] = g;
            ++sp;
        } else {
            overflow = 1;
        }
    }
    __device__ __forceinline__ uint2 pop()
    {
        --sp;
        return base[sp * stride];
    }
};

// Tests the eight children of node `ni`; returns the internal-child group
// and the leaf-triangle mask (bit b -> triangle tri_base + b).
__device__ __forceinline__ void visit_node(const WideNode* __restrict__ nodes, uint32_t ni, const RayPre& r,
                                           float tmin, float tmax, uint2& group, uint32_t& tmask,
                                           uint32_t& tri_base)
{
    const uint4* np = reinterpret_cast<const uint4*>(nodes + ni);
    uint4 w0, w1;
    ld_nc_v8(np, w0, w1);
    // low planes at lines 2..4, high planes at 5..7.  Along an axis where the
    // ray's idir is negative the high plane is the near one: loading the
    // planes in near/far order replaces the per-child min/max of the two slab
    // distances (fmaf is monotonic in the quantised coordinate, so the
    // selected value equals that min/max exactly).
    const int ox = (int)(r.oct() & 1u), oy = (int)((r.oct() >> 1) & 1u), oz = (int)(r.oct() >> 2);
    int ex = (int)(int8_t)(w0.w & 0xffu);
    int ey = (int)(int8_t)((w0.w >> 8) & 0xffu);
    int ez = (int)(int8_t)((w0.w >> 16) & 0xffu);
    uint32_t imask = w0.w >> 24;
    float sx = __int_as_float((ex + 127) << 23), sy = __int_as_float((ey + 127) << 23),
          sz = __int_as_float((ez + 127) << 23);
    // x and y in two-wide operations (each lane equal to the scalar one; the
    // difference feeds a product, which cannot contract)
    const float2 idxy = make_float2(r.idir.x, r.idir.y);
    const float2 Axy = mul2(make_float2(sx, sy), idxy);
    const float2 Bxy = mul2(sub2(make_float2(__uint_as_float(w0.x), __uint_as_float(w0.y)), make_float2(r.o.x, r.o.y)),
                            idxy);
    const float Ax = Axy.x, Ay = Axy.y, Az = sz * r.idir.z;
    const float Bz = (__uint_as_float(w0.z) - r.o.z) * r.idir.z;
    // Plane q of an axis is at t = q A + B = (2^23 + q) A + C with C = B - 2^23 A,
    // so each plane costs one permute and one FMA (the fused product is exact).
    // Rounding C costs at most |A| / 2 (one quantisation step is |A| in t), so
    // near planes move SRT_SLAB_MARGIN * |A| nearer and far planes as much
    // farther: the test stays conservative (no exactly-hit slab missed on 4M
    // random borderline cases from a margin of 0.625 up).
    const float K = 8388608.0f;
    const float2 Cxy = fma2(make_float2(-K, -K), Axy, Bxy);
    const float Cx = Cxy.x, Cy = Cxy.y, Cz = fmaf(-K, Az, Bz);
    const float mx = SRT_SLAB_MARGIN * fabsf(Ax), my = SRT_SLAB_MARGIN * fabsf(Ay), mz = SRT_SLAB_MARGIN * fabsf(Az);
    const float cnx = Cx - mx, cfx = Cx + mx;
    const float cny = Cy - my, cfy = Cy + my;
    const float cnz = Cz - mz, cfz = Cz + mz;
    // Each slot's meta byte holds the bits its child sets in the hit mask
    // (bits 0..23 leaf triangles, 24..31 internal children in octant order),
    // with internal children's slot index XORed with the octant here, four
    // bytes at a time: bits 3 and 4 are both set only in internal bytes.
    const uint32_t oct = r.ord();
    const uint32_t mlo = w1.z ^ ((((w1.z & (w1.z << 1)) & 0x10101010u) >> 4) * oct);
    const uint32_t mhi = w1.w ^ ((((w1.w & (w1.w << 1)) & 0x10101010u) >> 4) * oct);
    uint32_t hitmask = 0;
    // a child's x and y near planes come from one two-wide FMA, and its x and
    // y far planes from another (the same values as four fmaf: 744.6 -> 748.8
    // Msamples/s); the z planes of two siblings, which share a plane word,
    // likewise (880.3 -> 887.1).  Pairing x and y across siblings too needs
    // every scale and offset twice in registers and spills.
    const float2 axy = Axy, cnxy = make_float2(cnx, cny), cfxy = make_float2(cfx, cfy);
    const float2 az2 = make_float2(Az, Az), cnz2 = make_float2(cnz, cnz), cfz2 = make_float2(cfz, cfz);
    const float2 widen2 = make_float2(1.00000024f, 1.00000024f);
    uint4 l2, l3, l4, l5, l6, l7;  // lo x, y, z then hi x, y, z
    ld_nc_v8(np + 2, l2, l3);
    ld_nc_v8(np + 4, l4, l5);
    ld_nc_v8(np + 6, l6, l7);
    const uint4 nqx = sel4(ox, l5, l2), fqx = sel4(ox, l2, l5);
    const uint4 nqy = sel4(oy, l6, l3), fqy = sel4(oy, l3, l6);
    const uint4 nqz = sel4(oz, l7, l4), fqz = sel4(oz, l4, l7);
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        // children 2j (low halves of the plane words) and 2j + 1 (high halves)
        const uint32_t wnx = word4(nqx, j), wfx = word4(fqx, j), wny = word4(nqy, j), wfy = word4(fqy, j);
        const uint32_t wnz = word4(nqz, j), wfz = word4(fqz, j);
        const float2 nz = fma2(make_float2(q23(wnz, 0), q23(wnz, 1)), az2, cnz2);
        const float2 fz = fma2(make_float2(q23(wfz, 0), q23(wfz, 1)), az2, cfz2);
        const float2 n0 = fma2(make_float2(q23(wnx, 0), q23(wny, 0)), axy, cnxy);
        const float2 f0 = fma2(make_float2(q23(wfx, 0), q23(wfy, 0)), axy, cfxy);
        const float2 n1 = fma2(make_float2(q23(wnx, 1), q23(wny, 1)), axy, cnxy);
        const float2 f1 = fma2(make_float2(q23(wfx, 1), q23(wfy, 1)), axy, cfxy);
        const float tn0 = fmax3(n0.x, n0.y, fmaxf(nz.x, tmin)), tn1 = fmax3(n1.x, n1.y, fmaxf(nz.y, tmin));
        // the far distances widened by one two-wide multiply (a lone product: nothing to contract)
        const float2 tf = mul2(make_float2(fmin3(f0.x, f0.y, fminf(fz.x, tmax)), fmin3(f1.x, f1.y, fminf(fz.y, tmax))),
                               widen2);
        // meta bytes 2j and 2j + 1 (one byte permute each, zeros above)
        const uint32_t mw = j < 2 ? mlo : mhi;
        const uint32_t m0 = __byte_perm(mw, 0u, 0x4440u | (2u * (j & 1))), m1 = __byte_perm(mw, 0u, 0x4441u | (2u * (j & 1)));
        // (meta >> 5) << (meta & 31); an empty slot's byte is 0
        if (tn0 <= tf.x) hitmask |= __funnelshift_l(0u, m0 >> 5, m0);
        if (tn1 <= tf.y) hitmask |= __funnelshift_l(0u, m1 >> 5, m1);
    }
    group = make_uint2(w1.x, imask | ((hitmask >> 24) << 8));
    tmask = hitmask & 0x00ffffffu;
    tri_base = w1.y;
}

__device__ __forceinline__ uint32_t group_next_node(uint2& g, uint32_t oct)
{
    uint32_t hits = g.y >> 8;
    uint32_t k = __ffs(hits) - 1;
    hits &= hits - 1;
    uint32_t slot = k ^ oct;
    uint32_t imask = g.y & 0xffu;
    uint32_t rank = __popc(imask & ((1u << slot) - 1u));
    g.y = imask | (hits << 8);
    return g.x + rank;
}

// Per-ray work counters (profiling builds of the kernels only).
struct TraceCount {
    uint32_t nodes = 0, tris = 0;
};

// Closest hit in (tmin, tmax).  `stack` is this thread's shared stack.
template <bool kCount = false>
__device__ __forceinline__ Hit trace_closest(const SceneView& S, float3 o, float3 d, float tmin, float tmax,
                                             Stack& st, int& overflow, TraceCount* cnt = nullptr)
{
    Hit h;
    h.t = tmax;
    h.u = h.v = 0.0f;
    h.tri = -1;
    RayPre r = make_ray(o, d);
    st.sp = 0;
    uint2 group = make_uint2(0u, 1u | ((1u << r.ord()) << 8));  // root = child rank 0 of slot 0
    for (;;) {
        if ((group.y >> 8) == 0u) {
            if (st.sp == 0) break;
            group = st.pop();
            continue;
        }
        uint32_t ni = group_next_node(group, r.ord());
        if ((group.y >> 8) != 0u) st.push(group, overflow);
        uint32_t tmask, tri_base;
        visit_node(S.nodes, ni, r, tmin, h.t, group, tmask, tri_base);
        if (kCount) {
            cnt->nodes += 1;
            cnt->tris += __popc(tmask);
        }
        while (tmask) {
            uint32_t b = __ffs(tmask) - 1;
            tmask &= tmask - 1;
            uint32_t ti = tri_base + b;
            float4 a, bb, c;
            load_tri(S.tris, ti, a, bb, c);
            float t, u, v;
            if (hit_triangle(r, f3(a), f3(bb), f3(c), tmin, h.t, t, u, v)) {
                h.t = t;
                h.u = u;
                h.v = v;
                h.tri = (int32_t)ti;
            }
        }
    }
    return h;
}

// ---------------------------------------------------------------------------
// Persistent traversal with lane refill.  A warp keeps 32 rays in flight;
// each lane advances its own ray by a bounded number of node visits per
// round, and as soon as at least kRefill lanes have finished, the warp
// fetches that many new rays with one atomic (Aila & Laine, "Understanding
// the efficiency of ray traversal on GPUs", HPG 2009), so lanes do not idle
// until the slowest ray of a fixed batch ends.
// ---------------------------------------------------------------------------
#ifndef SRT_TRACE_REFILL
#define SRT_TRACE_REFILL 8
#endif
#ifndef SRT_TRACE_STEPS
#define SRT_TRACE_STEPS 4
#endif
#ifndef SRT_SHADOW_STEPS
#define SRT_SHADOW_STEPS 6
#endif
constexpr int kRefill = SRT_TRACE_REFILL;     // idle lanes that trigger a fetch
constexpr int kStepBudget = SRT_TRACE_STEPS;  // node visits per lane between refill checks
// any-hit rays are longer (about 10 node visits against 6 on the benchmark scene)
constexpr int kShadowStepBudget = SRT_SHADOW_STEPS;

struct TravState {
    RayPre r;
    float tmin, tmax;  // tmax shrinks with closest hits
    uint2 group;
    uint32_t tmask, tri_base;
    int32_t tri;  // closest (or any) hit so far; its barycentrics: hit_barycentrics
    const WideNode* nodes;
    const float4* tris;
};

// far_first: children are visited far-to-near (for any-hit rays, whose first
// nodes near the origin hold the origin's own surface)
__device__ __forceinline__ void trav_init(TravState& s, const WideNode* nodes, const float4* tris, float3 o, float3 d,
                                          float tmin, float tmax, Stack& st, bool far_first = false)
{
    s.r = make_ray(o, d);
    if (far_first) s.r.axes ^= 7u << 11;
    s.tmin = tmin;
    s.tmax = tmax;
    s.group = make_uint2(0u, 1u | ((1u << s.r.ord()) << 8));
    s.tmask = 0;
    s.tri_base = 0;
    s.tri = -1;
    s.nodes = nodes;
    s.tris = tris;
    st.sp = 0;
}

// Barycentrics of a finished ray's hit triangle, recomputed once at the end
// instead of kept in registers through the traversal: the same test on the
// same inputs gives the same u, v (with tmax open it accepts the hit).
__device__ __forceinline__ float2 tri_barycentrics(const RayPre& r, const float4* tris, int32_t tri, float tmin)
{
    float u = 0.0f, v = 0.0f;
    if (tri >= 0) {
        float4 a, bb, c;
        load_tri(tris, (uint32_t)tri, a, bb, c);
        float t;
        if (!hit_triangle(r, f3(a), f3(bb), f3(c), tmin, __int_as_float(0x7f800000), t, u, v)) u = v = 0.0f;
    }
    return make_float2(u, v);
}
__device__ __forceinline__ float2 hit_barycentrics(const TravState& s)
{
    return tri_barycentrics(s.r, s.tris, s.tri, s.tmin);
}

// Advances one ray; returns true when its traversal is complete (for any-hit
// rays: on the first hit, with s.tri set).  `any` is a constant where the
// kind of ray is fixed (trav_advance) and read from the ray where a kernel
// traces both kinds (bit 7 of its axes word, set by mark_any_hit).
template <bool kCount>
__device__ __forceinline__ bool trav_advance_impl(TravState& s, Stack& st, int& overflow, TraceCount& cnt, bool any)
{
    for (int it = 0; it < (any ? kShadowStepBudget : kStepBudget); ++it) {
        while (s.tmask) {
            uint32_t b = __ffs(s.tmask) - 1;
            s.tmask &= s.tmask - 1;
            uint32_t ti = s.tri_base + b;
            float4 a, bb, c;
            load_tri(s.tris, ti, a, bb, c);
            float t, u, v;
            if (hit_triangle(s.r, f3(a), f3(bb), f3(c), s.tmin, s.tmax, t, u, v)) {
                s.tri = (int32_t)ti;
                if (any) return true;
                s.tmax = t;
            }
        }
        if ((s.group.y >> 8) == 0u) {
            if (st.sp == 0) return true;
            s.group = st.pop();
        }
        uint32_t ni = group_next_node(s.group, s.r.ord());
        if ((s.group.y >> 8) != 0u) st.push(s.group, overflow);
        visit_node(s.nodes, ni, s.r, s.tmin, s.tmax, s.group, s.tmask, s.tri_base);
        if (kCount) {
            cnt.nodes += 1;
            cnt.tris += __popc(s.tmask);
        }
    }
    return false;
}
template <bool kAny, bool kCount>
__device__ __forceinline__ bool trav_advance(TravState& s, Stack& st, int& overflow, TraceCount& cnt)
{
    return trav_advance_impl<kCount>(s, st, overflow, cnt, kAny);
}
// a ray of a mixed kernel: any-hit (shadow) or closest-hit, by bit 7 of its axes
__device__ __forceinline__ void mark_any_hit(TravState& s) { s.r.axes |= 1u << 7; }
__device__ __forceinline__ bool is_any_hit(const TravState& s) { return (s.r.axes >> 7) & 1u; }
template <bool kCount>
__device__ __forceinline__ bool trav_advance_mixed(TravState& s, Stack& st, int& overflow, TraceCount& cnt,
                                                   TraceCount& scnt)
{
    const bool any = is_any_hit(s);
    return trav_advance_impl<kCount>(s, st, overflow, any ? scnt : cnt, any);
}

// A lane's ray index in the persistent loop: 64-bit, or 32-bit where the
// caller's n is below 2^32 - 1 (a register fewer beside the traversal state).
template <bool kNarrow>
struct RayIndex {
    using T = int64_t;
    static constexpr T kNone = -1;
};
template <>
struct RayIndex<true> {
    using T = uint32_t;
    static constexpr T kNone = 0xffffffffu;
};

// Drives a warp over rays [0, n) taken from *fetch.  load(i, state, stack)
// starts ray i (calls trav_init); store(i, state, fin) is called by all 32
// lanes after every round (so it may use warp-wide votes and appends), with
// fin set in the lanes whose ray i just finished.  kNarrow: n < 2^32 - 1.
template <bool kNarrow = false, class Advance, class Load, class Store>
__device__ __forceinline__ void trace_persistent_with(int64_t n, unsigned long long* fetch, Stack& st, Advance advance,
                                                      Load load, Store store)
{
    using Index = typename RayIndex<kNarrow>::T;
    constexpr Index kNone = RayIndex<kNarrow>::kNone;
    const uint32_t full = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    // Warps past the first n / 32 leave before touching the fetch counter:
    // the ones below take every ray, and a short queue (the end of a frame)
    // does not cost one contended atomic per resident warp of the grid.
    if ((int64_t)((blockIdx.x * blockDim.x + threadIdx.x) >> 5) * 32 >= n) return;
    Index ray = kNone;
    TravState s;
    bool drained = false;
    for (;;) {
        uint32_t idle = __ballot_sync(full, ray == kNone);
        if (!drained && (int)__popc(idle) >= kRefill) {
            unsigned long long base = 0;
            if (lane == 0) base = atomicAdd(fetch, (unsigned long long)__popc(idle));
            base = __shfl_sync(full, base, 0);
            if (base + __popc(idle) >= (unsigned long long)n) drained = true;
            if (ray == kNone) {
                int64_t idx = (int64_t)base + __popc(idle & ((1u << lane) - 1u));
                if (idx < n) {
                    ray = (Index)idx;
                    load(idx, s, st);
                }
            }
            idle = __ballot_sync(full, ray == kNone);
        }
        if (idle == full && drained) break;
        const bool fin = ray != kNone && advance(s, st);
        store((int64_t)ray, s, fin);
        if (fin) ray = kNone;
    }
}
template <bool kAny, bool kCount, class Load, class Store>
__device__ __forceinline__ void trace_persistent(int64_t n, unsigned long long* fetch, Stack& st, int& overflow,
                                                 TraceCount& cnt, Load load, Store store)
{
    trace_persistent_with(
        n, fetch, st, [&](TravState& s, Stack& stk) { return trav_advance<kAny, kCount>(s, stk, overflow, cnt); },
        load, store);
}

// Any hit in (tmin, tmax): true when occluded.
template <bool kCount = false>
__device__ __forceinline__ bool trace_any(const SceneView& S, float3 o, float3 d, float tmin, float tmax,
                                          Stack& st, int& overflow, TraceCount* cnt = nullptr)
{
    RayPre r = make_ray(o, d);
    st.sp = 0;
    uint2 group = make_uint2(0u, 1u | ((1u << r.ord()) << 8));
    for (;;) {
        if ((group.y >> 8) == 0u) {
            if (st.sp == 0) break;
            group = st.pop();
            continue;
        }
        uint32_t ni = group_next_node(group, r.ord());
        if ((group.y >> 8) != 0u) st.push(group, overflow);
        uint32_t tmask, tri_base;
        visit_node(S.nodes, ni, r, tmin, tmax, group, tmask, tri_base);
        if (kCount) {
            cnt->nodes += 1;
            cnt->tris += __popc(tmask);
        }
        while (tmask) {
            uint32_t b = __ffs(tmask) - 1;
            tmask &= tmask - 1;
            float4 a, bb, c;
            load_tri(S.tris, tri_base + b, a, bb, c);
            float t, u, v;
            if (hit_triangle(r, f3(a), f3(bb), f3(c), tmin, tmax, t, u, v)) return true;
        }
    }
    return false;
}

}  // namespace srt
