// wavefront.cu — kernels and host driver of the streaming wavefront tracer.
//
//   k_start    raygen for every pixel of a newly admitted job (SoA queue)
//   k_trace    one persistent traversal over the previous iteration's shadow
//              rays (any hit; unoccluded contributions added to the pixel)
//              and the current queue's closest-hit rays (-> hit records)
//   k_regen    the previous iteration's ended samples: NaN/Inf filter, film
//              accumulation
//   k_order    shading order: the queue's hits first, then its misses
//   k_shade    miss / emitter-hit MIS / NEE + MIS / BSDF sample / Russian
//              roulette; survivors, and the next sample's camera ray of a
//              path that ended, compacted into the next queue with one
//              atomic per warp; NEE rays into the shadow queue
//   k_advance  one thread: swaps the queue counters, keeps statistics
//   k_finish   the end of a frame (few paths left): each thread carries a
//              path and its pixel's later samples to the end
//
// The per-path arithmetic follows the megakernel raygen program
// src/shader/integrator/path_tracer.cu:50-169 statement by statement.
#include <curand_kernel.h>

#include <algorithm>
#include <chrono>
#include <cstddef>
#include <cstdlib>
#include <cstring>
#include <string>

#include "bxdf.h"
#include "scene.h"
#include "shading.cuh"
#include "trace.cuh"
#include "wavefront.cuh"

namespace srt {

namespace {

constexpr int kThreads = 256;
constexpr int kTraceThreads = 128;
constexpr uint32_t kFull = 0xffffffffu;

// ---------------------------------------------------------------------------
// warp-aggregated queue append: one atomicAdd per warp, lanes get
// consecutive slots in lane order.  All 32 lanes must call it.
// ---------------------------------------------------------------------------
__device__ __forceinline__ int32_t warp_append(int32_t* counter, bool pred)
{
    uint32_t m = __ballot_sync(kFull, pred);
    if (m == 0u) return -1;
    int lane = threadIdx.x & 31;
    int leader = __ffs(m) - 1;
    int32_t base = 0;
    if (lane == leader) base = atomicAdd(counter, __popc(m));
    base = __shfl_sync(kFull, base, leader);
    return pred ? base + __popc(m & ((1u << lane) - 1u)) : -1;
}

static_assert(offsetof(Counters, n_next) % 8 == 0 && offsetof(Counters, n_cam) == offsetof(Counters, n_next) + 4,
              "n_next and n_cam share one 64-bit word");
static_assert(offsetof(Counters, n_shadow) % 8 == 0 && offsetof(Counters, n_done) == offsetof(Counters, n_shadow) + 4,
              "n_shadow and n_done share one 64-bit word");
static_assert(offsetof(Counters, n_hit) % 8 == 0 && offsetof(Counters, n_miss) == offsetof(Counters, n_hit) + 4,
              "n_hit and n_miss share one 64-bit word");

// Two appends with one atomic on a 64-bit word holding both counters (low
// word: a's, high word: b's); a lane may take part in either or both.
__device__ __forceinline__ void warp_append_pair(int32_t* counters, bool a, bool b, int32_t& sa, int32_t& sb)
{
    const uint32_t ma = __ballot_sync(kFull, a), mb = __ballot_sync(kFull, b);
    sa = sb = -1;
    if ((ma | mb) == 0u) return;
    const int lane = threadIdx.x & 31;
    const int leader = __ffs(ma | mb) - 1;
    unsigned long long base = 0;
    if (lane == leader)
        base = atomicAdd(reinterpret_cast<unsigned long long*>(counters),
                         (unsigned long long)__popc(ma) | ((unsigned long long)__popc(mb) << 32));
    base = __shfl_sync(kFull, base, leader);
    const uint32_t below = (1u << lane) - 1u;
    if (a) sa = (int32_t)(uint32_t)base + __popc(ma & below);
    if (b) sb = (int32_t)(uint32_t)(base >> 32) + __popc(mb & below);
}

// Append where lanes may target different counters (one per job): lanes
// with the same counter share one atomic.  All 32 lanes must call it.
__device__ __forceinline__ int32_t warp_append_multi(int32_t* counter, bool pred)
{
    uint32_t active = __ballot_sync(kFull, pred);
    if (!pred) return -1;
    uint32_t peers = __match_any_sync(active, (unsigned long long)counter);
    int lane = threadIdx.x & 31;
    int leader = __ffs(peers) - 1;
    int32_t base = 0;
    if (lane == leader) base = atomicAdd(counter, __popc(peers));
    base = __shfl_sync(peers, base, leader);
    return base + __popc(peers & ((1u << lane) - 1u));
}

// Adds one per lane to *counter (null: nothing); lanes with the same counter
// share one atomic.  All 32 lanes must call it.
__device__ __forceinline__ void warp_count(int32_t* counter)
{
    uint32_t active = __ballot_sync(kFull, counter != nullptr);
    if (!counter) return;
    uint32_t peers = __match_any_sync(active, (unsigned long long)counter);
    if ((int)(threadIdx.x & 31) == __ffs(peers) - 1) atomicAdd(counter, __popc(peers));
}

__device__ __forceinline__ int region_cell(const CacheRec& c, float3 p)
{
    int r = c.region_res;
    int x = min(max((int)((p.x - c.box.lo.x) * c.box.inv_extent.x * r), 0), r - 1);
    int y = min(max((int)((p.y - c.box.lo.y) * c.box.inv_extent.y * r), 0), r - 1);
    int z = min(max((int)((p.z - c.box.lo.z) * c.box.inv_extent.z * r), 0), r - 1);
    return (z * r + y) * r + x;
}

// Slot of entry i of a path queue whose first nf entries fill it from the
// front and the rest from the back (Counters::nf_cur).
__device__ __forceinline__ int64_t qslot(int64_t i, int32_t nf, int64_t capacity)
{
    return i < nf ? i : capacity - 1 - (i - nf);
}

__device__ __forceinline__ uint32_t pack_flags(int depth, bool specular, int job)
{
    return (uint32_t)depth | (specular ? 0x100u : 0u) | ((uint32_t)job << 16);
}

// A sample ends (path_tracer.cu:164-165): its radiance l goes to the film
// unless it is NaN or infinite, and the pixel's finished-sample count (l.w)
// steps.  Sets the progress counters to bump: the progressive frame's and,
// at the pixel's last sample, the finished pixels'.
__device__ __forceinline__ void end_sample(const JobRec& J, int pix, float4 l, int32_t*& frame_ctr,
                                           int32_t*& pixel_ctr)
{
    if (isfinite(l.x) && isfinite(l.y) && isfinite(l.z)) {
        const float4 f = J.film[pix];
        const float s = (float)J.spp;
        J.film[pix] = make_float4(f.x + l.x / s, f.y + l.y / s, f.z + l.z / s, 1.0f);
    }
    const int k = __float_as_int(l.w) + 1;
    J.lpath[pix] = make_float4(0.0f, 0.0f, 0.0f, __int_as_float(k));
    if (J.frame_done) frame_ctr = J.frame_done + (k - 1);
    if (k >= J.spp) pixel_ctr = J.pixels_done;
}

// ---------------------------------------------------------------------------
// kernels
// ---------------------------------------------------------------------------

// Seeds job `job`: RandomGenerator(seed + idx, 0), film = (0, 0, 0, 1),
// sample-0 camera ray (two jitter draws) appended to queue q at *n.
__global__ void __launch_bounds__(kThreads) k_start(const JobRec* __restrict__ jobs, int job, PathQueue q,
                                                    int32_t* n, int32_t* front, int64_t capacity, int32_t* overflow)
{
    const JobRec& J = jobs[job];
    const int npix = J.npix;
    const int stride = gridDim.x * blockDim.x;
    for (int base = (blockIdx.x * blockDim.x + threadIdx.x) & ~31; base < npix; base += stride) {
        int pix = base + (threadIdx.x & 31);
        bool valid = pix < npix;
        float3 o = f3(0.0f), d = f3(0.0f);
        uint4 ra = make_uint4(0, 0, 0, 0);
        uint2 rb = make_uint2(0, 0);
        if (valid) {
            Rng rng;
            curand_init(pixel_seed(J.seed, pix), 0ull, 0ull, &rng.s);
            int ix = pix % J.width, iy = pix / J.width;
            float xx = ((float)ix + rng.next()) / (float)J.width;
            float yy = ((float)iy + rng.next()) / (float)J.height;
            camera_ray(J.cam, xx, yy, o, d);
            rng.store(ra, rb);
            J.film[pix] = make_float4(0.0f, 0.0f, 0.0f, 1.0f);
            J.lpath[pix] = make_float4(0.0f, 0.0f, 0.0f, __int_as_float(0));  // no sample finished
            if (J.cache.w && (pix % J.cache.train_stride) == J.cache.train_phase)
                J.cache.t_len[pix / J.cache.train_stride] = 0;
        }
        // at the front of the current queue (its back may hold other jobs' camera rays)
        int32_t slot = warp_append(front, valid);
        warp_append(n, valid);
        if (valid) {
            if (slot < capacity) {
                q.o[slot] = make_float4(o.x, o.y, o.z, __int_as_float(pix));
                q.d[slot] = make_float4(d.x, d.y, d.z, 1.0f);
                q.beta[slot] = make_float4(1.0f, 1.0f, 1.0f, __uint_as_float(pack_flags(0, true, job)));
                q.ra[slot] = ra;
                q.rb[slot] = rb;
            } else {
                atomicAdd(overflow, 1);
            }
        }
    }
}

// The iteration's traversal: the shadow rays the previous iteration's
// k_shade cast (any hit, far-to-near) and this iteration's closest-hit rays,
// one persistent launch over both (entries [0, n_sp) of the shadow queue,
// then [0, n_cur) of the path queue).  Between the two kinds a frame pays
// one kernel drain per iteration instead of two.  An unoccluded shadow ray
// adds its contribution to its pixel's radiance, before k_regen adds an
// ended sample to the film and before k_shade adds the pixel's next emitted
// radiance, the order of the reference's per-pixel loop (path_tracer.cu:
// 113-142 then 88-106 of the next segment).  shadows_only: the flush after
// the last iteration.
template <bool kCount>
__global__ void __launch_bounds__(kTraceThreads, SRT_TRACE_MIN_BLOCKS) k_trace(const JobRec* __restrict__ jobs, PathQueue q,
                                                                              ShadowQueue sq, float4* __restrict__ hits,
                                                                              Counters* ctr, int64_t capacity,
                                                                              int shadows_only)
{
    // a counter past the capacity (overflow, reported by the host) never indexes past a queue
    const int64_t ns = min((int64_t)ctr->n_sp, capacity);
    const int64_t nc = shadows_only ? 0 : min((int64_t)ctr->n_cur, capacity);
    const int32_t nf = ctr->nf_cur;
    int overflow = 0;
    TraceCount cnt, scnt;
    __shared__ uint2 stack_mem[kStackEntries * kTraceThreads];
    Stack st{stack_mem + threadIdx.x, kTraceThreads, 0};
    // ns + nc <= 2 * capacity < 2^32 - 1 (kMaxCapacity): 32-bit ray indices
    trace_persistent_with<true>(
        ns + nc, &ctr->fetch_closest, st,
        [&](TravState& s, Stack& stk) { return trav_advance_mixed<kCount>(s, stk, overflow, cnt, scnt); },
        [&](int64_t i, TravState& s, Stack& stk) {
            if (i < ns) {
                const float4 o = sq.o[i], d = sq.d[i];
                const SceneView& S = jobs[__float_as_int(sq.c[i].w)].scene;
                trav_init(s, S.nodes, S.tris, f3(o), f3(d), 1e-3f, d.w, stk, SRT_SHADOW_FAR_FIRST != 0);
                mark_any_hit(s);
            } else {
                const int64_t j = qslot(i - ns, nf, capacity);
                const float4 o = q.o[j], d = q.d[j];
                const SceneView& S = jobs[__float_as_uint(q.beta[j].w) >> 16].scene;
                trav_init(s, S.nodes, S.tris, f3(o), f3(d), 1e-3f, 1e16f, stk);
            }
        },
        [&](int64_t i, const TravState& s, bool fin) {
            if (!fin) return;
            if (i < ns) {
                if (s.tri < 0) {
                    // unoccluded; one path per pixel in flight: plain read-modify-write
                    const float4 o = sq.o[i], c = sq.c[i];
                    float4* lp = jobs[__float_as_int(c.w)].lpath + __float_as_int(o.w);
                    const float4 l = *lp;
                    *lp = make_float4(l.x + c.x, l.y + c.y, l.z + c.z, l.w);
                }
            } else {
                const float2 uv = hit_barycentrics(s);
                hits[i - ns] = make_float4(s.tmax, uv.x, uv.y, __int_as_float(s.tri));
            }
        });
    if (overflow) atomicAdd(&ctr->overflow_stack, 1);
    if (kCount && (cnt.nodes | cnt.tris | scnt.nodes | scnt.tris)) {
        atomicAdd(reinterpret_cast<unsigned long long*>(&ctr->c_nodes), (unsigned long long)cnt.nodes);
        atomicAdd(reinterpret_cast<unsigned long long*>(&ctr->c_tris), (unsigned long long)cnt.tris);
        atomicAdd(reinterpret_cast<unsigned long long*>(&ctr->s_nodes), (unsigned long long)scnt.nodes);
        atomicAdd(reinterpret_cast<unsigned long long*>(&ctr->s_tris), (unsigned long long)scnt.tris);
    }
}

// Shading order for k_shade: queue entries whose ray hit the scene first (in
// queue order), then the misses; one pair of atomics per 256 entries.
constexpr int kOrderThreads = 256;
__global__ void __launch_bounds__(kOrderThreads) k_order(const float4* __restrict__ hits,
                                                         int32_t* __restrict__ order, Counters* ctr,
                                                         int64_t capacity)
{
    __shared__ int32_t warp_hits[kOrderThreads / 32];
    __shared__ int32_t base_hit, base_miss;
    const int n = (int)min((int64_t)ctr->n_cur, capacity);
    const int t = threadIdx.x, lane = t & 31, w = t >> 5;
    for (int tile = blockIdx.x * kOrderThreads; tile < n; tile += gridDim.x * kOrderThreads) {
        const int j = tile + t;
        const bool valid = j < n;
        const bool hit = valid && __float_as_int(__ldg(&hits[j].w)) >= 0;
        const uint32_t hb = __ballot_sync(kFull, hit);
        const uint32_t vb = __ballot_sync(kFull, valid);
        if (lane == 0) warp_hits[w] = __popc(hb);
        __syncthreads();
        int before = 0, total = 0;
        for (int k = 0; k < kOrderThreads / 32; ++k) {
            const int c = warp_hits[k];
            total += c;
            if (k < w) before += c;
        }
        if (t == 0) {
            const int tile_valid = min(kOrderThreads, n - tile);
            // both counts with one atomic on their shared 64-bit word (n_hit the low word)
            const unsigned long long b = atomicAdd(reinterpret_cast<unsigned long long*>(&ctr->n_hit),
                                                   (unsigned long long)(uint32_t)total |
                                                       ((unsigned long long)(uint32_t)(tile_valid - total) << 32));
            base_hit = (int)(uint32_t)b;
            base_miss = (int)(uint32_t)(b >> 32);
        }
        __syncthreads();
        const uint32_t below = (1u << lane) - 1u;
        if (hit) order[base_hit + before + __popc(hb & below)] = j;
        if (valid && !hit) {
            // misses of this tile before this lane: earlier warps' valid entries minus their hits
            const int miss_rank = (min(w * 32, n - tile) - before) + __popc(vb & ~hb & below);
            order[n - 1 - (base_miss + miss_rank)] = j;
        }
        __syncthreads();  // warp_hits and the bases are rewritten by the next tile
    }
}

// shading block size and the resident blocks per SM the compiler budgets
// registers for: 256 x 2 (128 registers, 8 bytes spilled); with the shading
// order it measured 1 % faster than 128 x 6 (80 registers, spills) and 128 x 4
#ifndef SRT_SHADE_THREADS
#define SRT_SHADE_THREADS 256
#endif
#ifndef SRT_SHADE_MIN_BLOCKS
#define SRT_SHADE_MIN_BLOCKS 2
#endif
constexpr int kShadeThreads = SRT_SHADE_THREADS;

// Shades one path vertex (path_tracer.cu:79-166 for one segment): the
// path's state (origin and pixel, direction and scatter pdf, throughput and
// flags, rng words ra / rb) and its closest hit h (t, u, v, triangle bits)
// in; the vertex's emitted or environment radiance, the next segment, the
// shadow ray and whether the path ended out.  k_shade runs it for every
// queue entry; k_finish for the paths it carries to their last sample.
template <bool kCache>
__device__ __forceinline__ void shade_vertex(const JobRec* __restrict__ jobs, float4 o4, float4 d4, float4 b4, float4 h,
                                             bool& push_next, bool& push_shadow, bool& terminate, bool& push_query,
                                             float4 (&qrec)[4], float3& ro, float3& rd, float3& beta, float3& L_add,
                                             float3& sh_o, float3& sh_d, float3& sh_c, float& sh_t, float& pdf_next,
                                             uint32_t& flags, int& pix, int& job, uint4& ra, uint2& rb)
{
    flags = __float_as_uint(b4.w);
    job = (int)(flags >> 16);
    int depth = (int)(flags & 0xffu);
    bool specular = (flags & 0x100u) != 0u;
    pix = __float_as_int(o4.w);
    ro = f3(o4);
    rd = f3(d4);
    beta = f3(b4);
    const float scatter_pdf = d4.w;
    const JobRec& J = jobs[job];
    const SceneView& S = J.scene;
    const int tri = __float_as_int(h.w);
    terminate = true;
    if (tri < 0) {
        // miss: environment light (path_tracer.cu:81-85)
        L_add = beta * env_radiance(S, rd);
    } else {
        float4 a, b, c;
        load_tri(S.tris, (uint32_t)tri, a, b, c);
        float3 v0 = f3(a), v1 = f3(b), v2 = f3(c);
        InstanceRec ir = S.insts[__float_as_int(a.w)];
        float3 base_color;
        float4 em;
        int mflags;
        Bxdf bx = unpack_bxdf(S.mats, ir.material, base_color, em, mflags);
        // get_hitinfo (hit_info.h:27-64)
        float u = h.y, v = h.z;
        float3 pos = v0 * (1.0f - u - v) + v1 * u + v2 * v;
        float3 ng = normalize(cross(v1 - v0, v2 - v0));
        float3 sn = ng;
        if (ir.attr & kAttrNormals) {
            const float4* np = S.normals + 3 * (size_t)tri;
            sn = normalize(f3(__ldg(np)) * (1.0f - u - v) + f3(__ldg(np + 1)) * u + f3(__ldg(np + 2)) * v);
        }
        if (mflags & kMatTextured)
            apply_material_textures(S, ir.attr, ir.material, __float_as_int(a.w), tri, u, v, base_color, em, sn);
        if (dot(ng, sn) < 0.0f) ng = -ng;
        if (mflags & kMatEmissive) {
            // emitter hit with MIS (path_tracer.cu:88-106)
            float cos_i = dot(ng, -rd);
            if (cos_i > 1e-4f) {
                float mis = 1.0f;
                if (J.use_nee && !specular) {
                    mis = 0.0f;
                    if (J.use_mis) {
                        float t2 = dot(pos - ro, pos - ro);
                        float lpdf = S.lights[ir.light_id].pdf * t2 / cos_i;
                        mis = scatter_pdf / (lpdf + scatter_pdf);
                    }
                }
                L_add = beta * f3(em) * mis;
            }
        } else {
            if (dot(ng, -rd) < 0.0f) ng = -ng;
            const float3 wo = -rd;
            // radiance cache: non-training pixels end at the second vertex
            const CacheRec& Cc = J.cache;
            const bool cache_job = kCache && Cc.w != nullptr;
            const bool train_pix = cache_job && (pix % Cc.train_stride) == Cc.train_phase;
            if (cache_job && !train_pix && depth == 1) {
                push_query = !Cc.region_off || !Cc.region_off[region_cell(Cc, pos)];
                if (!push_query) atomicAdd(Cc.q_count + 1, 1);
            }
            if (push_query) {
                qrec[0] = make_float4(pos.x, pos.y, pos.z, bx.type == BXDF_DISNEY ? bx.roughness : 1.0f);
                qrec[1] = make_float4(ng.x, ng.y, ng.z, 0.0f);
                qrec[2] = make_float4(wo.x, wo.y, wo.z, 0.0f);
                qrec[3] = make_float4(base_color.x, base_color.y, base_color.z, 0.0f);
            } else {
            if (train_pix && depth >= 1 && depth <= kTrainVertices &&
                __float_as_int(J.lpath[pix].w) == 0) {
                // training vertex: features, arriving throughput, radiance gathered so far
                int slot = (pix / Cc.train_stride) * kTrainVertices + depth - 1;
                float4* tr = Cc.t_rec + 4 * (size_t)slot;
                tr[0] = make_float4(pos.x, pos.y, pos.z, bx.type == BXDF_DISNEY ? bx.roughness : 1.0f);
                tr[1] = make_float4(ng.x, ng.y, ng.z, 0.0f);
                tr[2] = make_float4(wo.x, wo.y, wo.z, 0.0f);
                tr[3] = make_float4(base_color.x, base_color.y, base_color.z, 0.0f);
                float4 lnow = J.lpath[pix];
                Cc.t_aux[2 * (size_t)slot] = make_float4(beta.x, beta.y, beta.z, 0.0f);
                Cc.t_aux[2 * (size_t)slot + 1] = make_float4(lnow.x, lnow.y, lnow.z, 0.0f);
                Cc.t_len[pix / Cc.train_stride] = depth;
            }
            Rng rng;
            rng.load(ra, rb);
            float3 tan = (fabsf(sn.x) > fabsf(sn.y)) ? make_float3(0.f, 1.f, 0.f) : make_float3(1.f, 0.f, 0.f);
            if (ir.attr & kAttrTangents) {
                // the mesh's interpolated tangent (hit_info.h:48-50)
                const float4* gp = S.tangents + 3 * (size_t)tri;
                tan = f3(__ldg(gp)) * (1.0f - u - v) + f3(__ldg(gp + 1)) * u + f3(__ldg(gp + 2)) * v;
            }
            Frame fr = Frame::from_normal_tangent(sn, tan);
            const bool transmissive = (mflags & kMatTransmissive) != 0;
            // NEE with MIS (path_tracer.cu:113-142)
            if (J.use_nee && !(mflags & kMatSpecular) &&
                !(depth > 0 && (J.flags & SRT_PT_NEE_FIRST_VERTEX_ONLY))) {
                float lu = rng.next();
                float lv = rng.next();
                LightSample ls = sample_light(S, lu, lv, (J.flags & SRT_PT_FIXED_CDF_REMAP) != 0);
                float3 sd = normalize(ls.pos - pos);
                float cos_o = dot(ng, sd);
                float cos_l = dot(ls.normal, -sd);
                float t = length(ls.pos - pos);
                if (cos_l > 1e-4f && ls.pdf > 1e-4f && t > 1e-3f && (cos_o > 0.0f || transmissive)) {
                    float lpdf = ls.pdf * t * t / cos_l;
                    float mis = 1.0f;
                    if (J.use_mis) {
                        float mpdf = material_pdf(bx, fr, sd, wo, base_color);
                        mis = lpdf / (lpdf + mpdf);
                    }
                    float3 fv = material_eval(bx, fr, sd, wo, base_color);
                    sh_c = beta * fv * fabsf(cos_o) * ls.emission * mis / lpdf;
                    sh_o = pos;
                    sh_d = sd;
                    sh_t = t - 1e-3f;
                    push_shadow = true;
                }
            }
            // BSDF sample (path_tracer.cu:145-153)
            float bu = rng.next();
            float bv = rng.next();
            BxdfSample ms = material_sample(bx, fr, wo, make_float2(bu, bv), base_color);
            if (ms.pdf > 1e-4f && !(dot(ms.wi, ng) < 0.0f && !transmissive)) {
                beta *= ms.f / ms.pdf;
                if (!ms.delta) beta *= fabsf(dot(ms.wi, ng));
                bool alive = true;
                // Russian roulette (path_tracer.cu:156-161)
                if (depth >= J.rr_depth) {
                    float p = fmaxf(fmaxf(beta.x, fmaxf(beta.y, beta.z)), 0.05f);
                    if (rng.next() > p)
                        alive = false;
                    else
                        beta /= p;
                }
                if (alive && depth + 1 < J.max_depth) {
                    terminate = false;
                    push_next = true;
                    ro = pos;
                    rd = ms.wi;
                    pdf_next = ms.pdf;
                    flags = pack_flags(depth + 1, (mflags & kMatSpecular) != 0, job);
                }
            }
            rng.store(ra, rb);
            }
        }
    }
}

// kCache: the iteration carries radiance-cache jobs (queries and training
// records); the plain variant leaves that code out
template <bool kCache>
__global__ void __launch_bounds__(kShadeThreads, SRT_SHADE_MIN_BLOCKS) k_shade(const JobRec* __restrict__ jobs, PathQueue q,
                                                    const float4* __restrict__ hits,
                                                    const int32_t* __restrict__ order, PathQueue qn, ShadowQueue sq,
                                                    DoneQueue done, Counters* ctr, int64_t capacity)
{
    const int n = (int)min((int64_t)ctr->n_cur, capacity);
    const int32_t nf = ctr->nf_cur;
    const int stride = gridDim.x * blockDim.x;
    for (int base = (blockIdx.x * blockDim.x + threadIdx.x) & ~31; base < n; base += stride) {
        // queue entries in k_order's shading order: hits first, then misses
        const int j = base + (threadIdx.x & 31);
        const bool valid = j < n;
        const int i = valid ? __ldg(order + j) : 0;
        const int64_t si = qslot(i, nf, capacity);
        bool push_next = false, push_shadow = false, terminate = false, push_query = false, push_cam = false;
        float4 qrec[4];
        float3 ro = f3(0.0f), rd = f3(0.0f), beta = f3(0.0f), L_add = f3(0.0f);
        float3 sh_o = f3(0.0f), sh_d = f3(0.0f), sh_c = f3(0.0f);
        float sh_t = 0.0f, pdf_next = 0.0f;
        uint32_t flags = 0;
        int pix = 0, job = 0;
        uint4 ra = make_uint4(0, 0, 0, 0);
        uint2 rb = make_uint2(0, 0);
        if (valid) {
            float4 o4 = q.o[si], d4 = q.d[si], b4 = q.beta[si];
            float4 h = hits[i];
            ra = q.ra[si];
            rb = q.rb[si];
            shade_vertex<kCache>(jobs, o4, d4, b4, h, push_next, push_shadow, terminate, push_query, qrec, ro, rd,
                                 beta, L_add, sh_o, sh_d, sh_c, sh_t, pdf_next, flags, pix, job, ra, rb);
        }
        // network query of a cached path (its radiance is added by k_cache)
        int32_t qslot = kCache ? warp_append_multi(jobs[job].cache.q_count, valid && push_query) : -1;
        if (kCache && push_query) {
            const CacheRec& Cc = jobs[job].cache;
            float4* qr = Cc.q_rec + 4 * (size_t)qslot;
            qr[0] = qrec[0];
            qr[1] = qrec[1];
            qr[2] = qrec[2];
            qr[3] = qrec[3];
            Cc.q_beta[qslot] = make_float4(beta.x, beta.y, beta.z, __int_as_float(pix));
        }
        // emitter / miss radiance of this vertex
        if (valid && (L_add.x != 0.0f || L_add.y != 0.0f || L_add.z != 0.0f || !finite3(L_add))) {
            float4* lp = jobs[job].lpath + pix;
            float4 l = *lp;
            *lp = make_float4(l.x + L_add.x, l.y + L_add.y, l.z + L_add.z, l.w);
        }
        // a path that ended starts its pixel's next sample (path_tracer.cu:64-68):
        // the camera ray continues the pixel's curand stream where shading left it
        const bool fin = valid && terminate;
        if (fin) {
            const JobRec& J = jobs[job];
            if (__float_as_int(J.lpath[pix].w) + 1 < J.spp) {
                Rng rng;
                rng.load(ra, rb);
                const int ix = pix % J.width, iy = pix / J.width;
                const float xx = ((float)ix + rng.next()) / (float)J.width;
                const float yy = ((float)iy + rng.next()) / (float)J.height;
                camera_ray(J.cam, xx, yy, ro, rd);
                rng.store(ra, rb);
                beta = f3(1.0f);
                pdf_next = 1.0f;
                flags = pack_flags(0, true, job);
                push_cam = true;
            }
        }
        // the next queue: continuing paths from the front, camera rays from the
        // back (a lane does at most one of the two; one warp-wide append counts
        // both, as the next one counts the shadow rays and the ended samples)
        int32_t slot, cs;
        warp_append_pair(&ctr->n_next, push_next, push_cam, slot, cs);
        if (push_cam) slot = cs < capacity ? (int32_t)(capacity - 1 - cs) : (int32_t)capacity;
        push_next = push_next || push_cam;
        if (push_next) {
            if (slot < capacity) {
                qn.o[slot] = make_float4(ro.x, ro.y, ro.z, __int_as_float(pix));
                qn.d[slot] = make_float4(rd.x, rd.y, rd.z, pdf_next);
                qn.beta[slot] = make_float4(beta.x, beta.y, beta.z, __uint_as_float(flags));
                qn.ra[slot] = ra;
                qn.rb[slot] = rb;
            } else {
                atomicAdd(&ctr->overflow_queue, 1);
            }
        }
        int32_t dslot;
        warp_append_pair(&ctr->n_shadow, push_shadow, fin, slot, dslot);
        if (push_shadow) {
            if (slot < capacity) {
                sq.o[slot] = make_float4(sh_o.x, sh_o.y, sh_o.z, __int_as_float(pix));
                sq.d[slot] = make_float4(sh_d.x, sh_d.y, sh_d.z, sh_t);
                sq.c[slot] = make_float4(sh_c.x, sh_c.y, sh_c.z, __int_as_float(job));
            } else {
                atomicAdd(&ctr->overflow_queue, 1);
            }
        }
        if (fin) {
            if (dslot < capacity) {
                done.rec[dslot] = make_uint2((uint32_t)job, (uint32_t)pix);
            } else {
                atomicAdd(&ctr->overflow_queue, 1);
            }
        }
    }
}

// Ends the samples that ended in the previous iteration (path_tracer.cu:
// 164-165), after k_trace has traced their last shadow rays: the film takes
// each sample's radiance once every contribution to it is in (its last
// shadow ray, a radiance-cache query); the pixel's next sample was started
// by k_shade.
__global__ void __launch_bounds__(kThreads) k_regen(const JobRec* __restrict__ jobs, DoneQueue done, Counters* ctr,
                                                    int64_t capacity)
{
    const int n = (int)min((int64_t)ctr->n_dp, capacity);
    const int stride = gridDim.x * blockDim.x;
    for (int base = (blockIdx.x * blockDim.x + threadIdx.x) & ~31; base < n; base += stride) {
        const int i = base + (threadIdx.x & 31);
        int32_t* frame_ctr = nullptr;  // progressive-frame counter of the finished sample
        int32_t* pixel_ctr = nullptr;  // finished-pixel counter, when the pixel's last sample ended
        if (i < n) {
            const uint2 e = done.rec[i];
            const int job = (int)e.x, pix = (int)e.y;
            const JobRec& J = jobs[job];
            float4 l = J.lpath[pix];
            const int spp_done = __float_as_int(l.w);
            const CacheRec& Cc = J.cache;
            if (Cc.w && (pix % Cc.train_stride) == Cc.train_phase && spp_done == 0) {
                // targets of the recorded vertices: radiance gathered after the
                // vertex divided by the throughput that arrived there
                const int ts = pix / Cc.train_stride;
                const int nv = Cc.t_len[ts];
                const bool ok = isfinite(l.x) && isfinite(l.y) && isfinite(l.z);
                for (int k = 0; k < nv; ++k) {
                    float4* ax = Cc.t_aux + 2 * ((size_t)ts * kTrainVertices + k);
                    float4 b = ax[0], before = ax[1];
                    bool valid = ok && b.x > 1e-6f && b.y > 1e-6f && b.z > 1e-6f;
                    float4 tgt = make_float4(0.f, 0.f, 0.f, 0.f);
                    if (valid)
                        tgt = make_float4(fmaxf(l.x - before.x, 0.0f) / b.x, fmaxf(l.y - before.y, 0.0f) / b.y,
                                          fmaxf(l.z - before.z, 0.0f) / b.z, 1.0f);
                    ax[1] = tgt;
                }
            }
            end_sample(J, pix, l, frame_ctr, pixel_ctr);
        }
        // progress counters: one atomic per distinct counter in the warp
        warp_count(frame_ctr);
        warp_count(pixel_ctr);
    }
}

// The end of a frame.  A wavefront iteration lasts as long as its slowest
// ray, however few paths are left, and each pixel's samples follow one
// another (one curand stream per pixel), so the last fifth of a frame's
// iterations carries about 2 % of its rays.  Once k_advance finds at most
// tail_below paths in flight, pairs of lanes here take one queue entry each
// and carry that path, and its pixel's later samples, to the pixel's last
// sample.  The even lane owns the path: closest hit (as k_trace),
// shade_vertex (as k_shade), the film and the next sample (as k_regen and
// k_shade).  The odd lane traces the shadow ray the owner's last shading
// cast, in the same traversal phase as the owner's next closest-hit ray, so
// a segment costs the longer of the two traversals, not their sum.  Per
// pixel the radiance additions keep the iterations' order -- the previous
// vertex's NEE contribution, then the film if that vertex ended its sample,
// then the next vertex's emitted radiance -- on the same values, so every
// pixel ends with the value the iterations give.  Plain jobs only (no
// radiance-cache work).
constexpr int kFinishThreads = kTraceThreads;

template <bool kCount>
__global__ void __launch_bounds__(kFinishThreads) k_finish(const JobRec* __restrict__ jobs, PathQueue q, Counters* ctr,
                                                           int64_t capacity)
{
    if (!ctr->tail_go) return;
    const int64_t n = min((int64_t)ctr->n_cur, capacity);
    __shared__ uint2 stack_mem[kStackEntries * kFinishThreads];
    Stack st{stack_mem + threadIdx.x, kFinishThreads, 0};
    const int lane = threadIdx.x & 31;
    const bool owner = (lane & 1) == 0;
    int overflow = 0;
    TraceCount cnt, scnt;  // closest-hit and shadow traversal work (profiling variant)
    int closest = 0, shadow = 0, ended = 0, taken = 0;
    // owner: the path in flight (its next closest-hit ray) and what its last
    // shading left pending for the next round: a shadow ray's contribution
    // and the end of its sample, both for the pixel pend_pix of job pend_job
    bool has_path = false, drained = false;
    float4 o4 = make_float4(0.f, 0.f, 0.f, 0.f), d4 = o4, b4 = o4;
    uint4 ra = make_uint4(0, 0, 0, 0);
    uint2 rb = make_uint2(0, 0);
    bool pend_shadow = false, pend_end = false;
    float3 pend_c = f3(0.0f), sh_o = f3(0.0f), sh_d = f3(0.0f);
    float sh_t = 0.0f;
    int pend_pix = 0, pend_job = 0;
    for (;;) {
        if (owner && !has_path && !drained) {
            const unsigned long long i = atomicAdd(&ctr->fetch_tail, 1ull);
            if (i < (unsigned long long)n) {
                const int64_t si = qslot((int64_t)i, ctr->nf_cur, capacity);
                o4 = q.o[si];
                d4 = q.d[si];
                b4 = q.beta[si];
                ra = q.ra[si];
                rb = q.rb[si];
                has_path = true;
                ++taken;
            } else {
                drained = true;
            }
        }
        if (!__any_sync(kFull, owner && (has_path || pend_shadow || pend_end))) break;
        // the owner's shadow ray to its partner lane
        const bool sh_active = __shfl_sync(kFull, pend_shadow, lane & ~1);
        const float sox = __shfl_sync(kFull, sh_o.x, lane & ~1), soy = __shfl_sync(kFull, sh_o.y, lane & ~1),
                    soz = __shfl_sync(kFull, sh_o.z, lane & ~1);
        const float sdx = __shfl_sync(kFull, sh_d.x, lane & ~1), sdy = __shfl_sync(kFull, sh_d.y, lane & ~1),
                    sdz = __shfl_sync(kFull, sh_d.z, lane & ~1);
        const float stm = __shfl_sync(kFull, sh_t, lane & ~1);
        const int sjob = __shfl_sync(kFull, pend_job, lane & ~1);
        // traversal phase: owner's closest-hit ray, partner's shadow ray
        TravState s;
        bool active = false;
        if (owner && has_path) {
            const SceneView& S = jobs[__float_as_uint(b4.w) >> 16].scene;
            trav_init(s, S.nodes, S.tris, f3(o4), f3(d4), 1e-3f, 1e16f, st);
            active = true;
            ++closest;
        } else if (!owner && sh_active) {
            const SceneView& S = jobs[sjob].scene;
            trav_init(s, S.nodes, S.tris, make_float3(sox, soy, soz), make_float3(sdx, sdy, sdz), 1e-3f, stm, st,
                      SRT_SHADOW_FAR_FIRST != 0);
            mark_any_hit(s);
            active = true;
            ++shadow;
        }
        bool done = !active;
        while (__any_sync(kFull, !done)) {
            if (!done) done = trav_advance_mixed<kCount>(s, st, overflow, cnt, scnt);
        }
        const bool unoccluded = __shfl_sync(kFull, active && s.tri < 0, lane | 1);
        if (owner) {
            // the previous vertex's NEE contribution, then the end of its sample (k_trace)
            if (pend_shadow || pend_end) {
                const JobRec& P = jobs[pend_job];
                float4* lp = P.lpath + pend_pix;
                float4 l = *lp;
                if (pend_shadow && unoccluded) {
                    l = make_float4(l.x + pend_c.x, l.y + pend_c.y, l.z + pend_c.z, l.w);
                    *lp = l;
                }
                if (pend_end) {
                    int32_t* frame_ctr = nullptr;
                    int32_t* pixel_ctr = nullptr;
                    end_sample(P, pend_pix, l, frame_ctr, pixel_ctr);
                    if (frame_ctr) atomicAdd(frame_ctr, 1);
                    if (pixel_ctr) atomicAdd(pixel_ctr, 1);
                    ++ended;
                }
                pend_shadow = pend_end = false;
            }
            if (has_path) {
                const float2 uv = hit_barycentrics(s);
                const float4 h = make_float4(s.tmax, uv.x, uv.y, __int_as_float(s.tri));
                // shading (k_shade)
                bool push_next = false, push_shadow = false, terminate = false, push_query = false;
                float4 qrec[4];
                float3 ro = f3(0.0f), rd = f3(0.0f), beta = f3(0.0f), L_add = f3(0.0f), sh_c = f3(0.0f);
                float pdf_next = 0.0f;
                uint32_t flags = 0;
                int pix = 0, job = 0;
                shade_vertex<false>(jobs, o4, d4, b4, h, push_next, push_shadow, terminate, push_query, qrec, ro, rd,
                                    beta, L_add, sh_o, sh_d, sh_c, sh_t, pdf_next, flags, pix, job, ra, rb);
                const JobRec& J = jobs[job];
                float4* lp = J.lpath + pix;
                if (L_add.x != 0.0f || L_add.y != 0.0f || L_add.z != 0.0f || !finite3(L_add)) {
                    const float4 l = *lp;
                    *lp = make_float4(l.x + L_add.x, l.y + L_add.y, l.z + L_add.z, l.w);
                }
                pend_pix = pix;
                pend_job = job;
                pend_shadow = push_shadow;
                pend_c = sh_c;
                if (push_next) {
                    o4 = make_float4(ro.x, ro.y, ro.z, __int_as_float(pix));
                    d4 = make_float4(rd.x, rd.y, rd.z, pdf_next);
                    b4 = make_float4(beta.x, beta.y, beta.z, __uint_as_float(flags));
                } else {
                    // the sample ends once its last shadow ray is in; the pixel's
                    // next sample starts now, from where shading left the stream
                    pend_end = true;
                    if (__float_as_int(lp->w) + 1 < J.spp) {
                        Rng rng;
                        rng.load(ra, rb);
                        const int ix = pix % J.width, iy = pix / J.width;
                        const float xx = ((float)ix + rng.next()) / (float)J.width;
                        const float yy = ((float)iy + rng.next()) / (float)J.height;
                        float3 o, d;
                        camera_ray(J.cam, xx, yy, o, d);
                        rng.store(ra, rb);
                        o4 = make_float4(o.x, o.y, o.z, __int_as_float(pix));
                        d4 = make_float4(d.x, d.y, d.z, 1.0f);
                        b4 = make_float4(1.0f, 1.0f, 1.0f, __uint_as_float(pack_flags(0, true, job)));
                    } else {
                        has_path = false;
                    }
                }
            }
        }
    }
    // one atomic per warp and counter
    closest = __reduce_add_sync(kFull, closest);
    shadow = __reduce_add_sync(kFull, shadow);
    ended = __reduce_add_sync(kFull, ended);
    taken = __reduce_add_sync(kFull, taken);
    if ((threadIdx.x & 31) == 0) {
        atomicAdd(reinterpret_cast<unsigned long long*>(&ctr->closest_total), (unsigned long long)closest);
        atomicAdd(reinterpret_cast<unsigned long long*>(&ctr->shadow_total), (unsigned long long)shadow);
        atomicAdd(reinterpret_cast<unsigned long long*>(&ctr->started), (unsigned long long)ended);
        atomicAdd(reinterpret_cast<unsigned long long*>(&ctr->tail_paths), (unsigned long long)taken);
    }
    if (overflow) atomicAdd(&ctr->overflow_stack, 1);
    if (kCount && (cnt.nodes | cnt.tris | scnt.nodes | scnt.tris)) {
        atomicAdd(reinterpret_cast<unsigned long long*>(&ctr->c_nodes), (unsigned long long)cnt.nodes);
        atomicAdd(reinterpret_cast<unsigned long long*>(&ctr->c_tris), (unsigned long long)cnt.tris);
        atomicAdd(reinterpret_cast<unsigned long long*>(&ctr->s_nodes), (unsigned long long)scnt.nodes);
        atomicAdd(reinterpret_cast<unsigned long long*>(&ctr->s_tris), (unsigned long long)scnt.tris);
    }
}

// After the flush (k_trace over the pending shadow rays, k_regen over the
// pending ended samples): nothing pending.
__global__ void k_end_flush(Counters* c)
{
    c->n_sp = 0;
    c->n_dp = 0;
    c->fetch_closest = 0;
}

// After k_finish: nothing is left in flight.
__global__ void k_end_tail(Counters* c)
{
    if (!c->tail_go) return;
    c->n_cur = 0;
    c->nf_cur = 0;
    c->fetch_tail = 0;
    c->tail_go = 0;
}

// Ends an iteration: swaps the queues' counts and, in the device-side loop,
// decides whether the loop runs again (paths in flight, no overflow, and the
// launch's iteration bound not reached: the loop always terminates).
template <bool kCond>
__global__ void k_advance(Counters* c, IterCount* history, const JobRec* __restrict__ jobs, int max_jobs,
                          cudaGraphConditionalHandle cond)
{
    if (c->iterations < kIterHistory) {
        IterCount h;
        h.closest = c->n_cur;
        h.hits = c->n_hit;
        h.misses = c->n_miss;
        h.shadow = c->n_shadow;
        h.done = c->n_done;
        h.pad[0] = h.pad[1] = h.pad[2] = 0;
        history[c->iterations] = h;
    }
    for (int j = 0; j < max_jobs; ++j)
        if (jobs[j].cache.q_count) {
            jobs[j].cache.q_count[4] += jobs[j].cache.q_count[0];  // queries of the frame
            jobs[j].cache.q_count[0] = 0;
        }
    c->closest_total += c->n_cur;
    c->shadow_total += c->n_shadow;
    c->iterations += 1;
    c->started += c->n_done;
    c->n_sp = c->n_shadow;  // traced by the next k_trace
    c->n_dp = c->n_done;    // added to the film by the next k_regen
    c->n_cur = c->n_next + c->n_cam;
    c->nf_cur = c->n_next;
    c->n_next = 0;
    c->n_cam = 0;
    c->n_shadow = 0;
    c->n_done = 0;
    c->fetch_closest = 0;
    c->fetch_shadow = 0;
    c->n_hit = 0;
    c->n_miss = 0;
    c->run_iters += 1;
    const bool clean = c->overflow_queue == 0 && c->overflow_stack == 0;
    const bool tail = c->tail_below > 0 && c->n_cur > 0 && c->n_cur <= c->tail_below && clean;
    c->tail_go = tail ? 1 : 0;
    if (kCond) {
        const bool again = c->n_cur > 0 && c->run_iters < c->run_limit && clean && !tail;
        cudaGraphSetConditional(cond, again ? 1u : 0u);
    }
}

// Starts a launch of the device-side loop: at most `limit` iterations,
// handing the frame to k_finish at `tail_below` paths in flight (0: never).
__global__ void k_begin_run(Counters* c, long long limit, int32_t tail_below)
{
    c->run_iters = 0;
    c->run_limit = limit;
    c->tail_below = tail_below;
    c->tail_go = 0;
}

__global__ void k_rng_tape(int32_t seed, int64_t npix, int32_t ndraws, float* out)
{
    int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= npix) return;
    Rng rng;
    curand_init(pixel_seed(seed, (int32_t)p), 0ull, 0ull, &rng.s);
    for (int k = 0; k < ndraws; ++k) out[p * ndraws + k] = rng.next();
}

size_t align_up(size_t x) { return (x + 255) & ~(size_t)255; }

}  // namespace

// ---------------------------------------------------------------------------
// Engine (host)
// ---------------------------------------------------------------------------

Engine::~Engine()
{
    if (graph_) cudaGraphExecDestroy(graph_);
    if (graph_prof_) cudaGraphExecDestroy(graph_prof_);
    for (auto& a : ev_)
        for (auto& b : a)
            for (auto& e : b)
                if (e) cudaEventDestroy(e);
    for (auto& e : ev_tail_)
        if (e) cudaEventDestroy(e);
    if (graph_stream_) cudaStreamDestroy(graph_stream_);
    if (side_stream_) cudaStreamDestroy(side_stream_);
    if (fork_ev_) cudaEventDestroy(fork_ev_);
    if (join_ev_) cudaEventDestroy(join_ev_);
    if (host_counters_) cudaFreeHost(host_counters_);
}

// Largest queue capacity: entry indices fit in int32, and k_trace's rays
// (shadow plus path entries) in its 32-bit ray indices.
constexpr int64_t kMaxCapacity = 0x7ffffff0;
static_assert(2 * kMaxCapacity < (int64_t)RayIndex<true>::kNone, "k_trace ray indices must fit in 32 bits");

srt_status Engine::init(int64_t capacity, int max_jobs)
{
    if (capacity <= 0 || capacity > kMaxCapacity || max_jobs <= 0 || max_jobs > 65535)
        return set_error(SRT_ERR_ARG, "engine capacity out of range");
    capacity_ = capacity;
    max_jobs_ = max_jobs;
    const size_t C = (size_t)capacity;
    // one carve both sizes the buffer (base null) and places the arrays in it
    auto carve = [&](char* base) {
        size_t off = 0;
        auto take = [&](size_t bytes) {
            char* r = reinterpret_cast<char*>(reinterpret_cast<uintptr_t>(base) + off);
            off += align_up(bytes);
            return r;
        };
        for (int k = 0; k < 2; ++k) {
            q_[k].o = (float4*)take(C * 16);
            q_[k].d = (float4*)take(C * 16);
            q_[k].beta = (float4*)take(C * 16);
            q_[k].ra = (uint4*)take(C * 16);
            q_[k].rb = (uint2*)take(C * 8);
        }
        sq_.o = (float4*)take(C * 16);
        sq_.d = (float4*)take(C * 16);
        sq_.c = (float4*)take(C * 16);
        hits_ = (float4*)take(C * 16);
        order_ = (int32_t*)take(C * 4);
        done_.rec = (uint2*)take(C * 8);
        counters_ = (Counters*)take(sizeof(Counters));
        history_ = (IterCount*)take(sizeof(IterCount) * kIterHistory);
        jobs_ = (JobRec*)take(sizeof(JobRec) * max_jobs);
        pixels_done_ = (int32_t*)take(4 * (size_t)max_jobs);
        return off;
    };
    const size_t total = carve(nullptr);
    SRT_TRY(buf_.alloc(total, "wavefront queues"));
    bytes_ = total;
    carve(buf_.as<char>());
    SRT_CUDA_TRY(cudaMemset(counters_, 0, sizeof(Counters)));
    SRT_CUDA_TRY(cudaMemset(jobs_, 0, sizeof(JobRec) * (size_t)max_jobs));  // unused slots read as plain, empty jobs
    SRT_CUDA_TRY(cudaMemset(pixels_done_, 0, 4 * (size_t)max_jobs));
    SRT_CUDA_TRY(cudaMallocHost(reinterpret_cast<void**>(&host_counters_), sizeof(Counters)));
    SRT_CUDA_TRY(cudaStreamCreateWithFlags(&graph_stream_, cudaStreamNonBlocking));
    SRT_CUDA_TRY(cudaStreamCreateWithFlags(&side_stream_, cudaStreamNonBlocking));
    SRT_CUDA_TRY(cudaEventCreateWithFlags(&fork_ev_, cudaEventDisableTiming));
    SRT_CUDA_TRY(cudaEventCreateWithFlags(&join_ev_, cudaEventDisableTiming));
    int sms = device_sm_count();
    // persistent traversal (dynamic ray fetch): as many blocks as are resident at once
    auto resident = [&](const void* fn) {
        int nb = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, fn, kTraceThreads, 0) != cudaSuccess || nb < 1)
            nb = SRT_TRACE_MIN_BLOCKS;
        return sms * nb;
    };
    grid_trace_ = resident(reinterpret_cast<const void*>(k_trace<false>));
    grid_finish_ = resident(reinterpret_cast<const void*>(k_finish<false>));
    grid_stride_ = (int)std::max<int64_t>(1, std::min<int64_t>((capacity + kThreads - 1) / kThreads, sms * 8));
    grid_regen_ = std::max(1, grid_stride_ / 2);
    grid_order_ = (int)std::max<int64_t>(1, std::min<int64_t>((capacity + kOrderThreads - 1) / kOrderThreads, sms * 8));
    grid_shade_ = (int)std::max<int64_t>(
        1, std::min<int64_t>((capacity + kShadeThreads - 1) / kShadeThreads, (int64_t)sms * 8 * (256 / kShadeThreads)));
    return SRT_OK;
}

srt_status Engine::set_job(int job, const JobRec& rec, cudaStream_t st)
{
    if (job < 0 || job >= max_jobs_) return set_error(SRT_ERR_ARG, "job slot out of range");
    SRT_CUDA_TRY(cudaMemcpyAsync(jobs_ + job, &rec, sizeof(JobRec), cudaMemcpyHostToDevice, st));
    SRT_CUDA_TRY(cudaMemsetAsync(pixels_done_ + job, 0, 4, st));
    return SRT_OK;
}

srt_status Engine::start_job(int job, const JobRec& rec, cudaStream_t st)
{
    int blocks = (int)std::max<int64_t>(1, std::min<int64_t>((rec.npix + kThreads - 1) / kThreads,
                                                             (int64_t)device_sm_count() * 16));
    k_start<<<blocks, kThreads, 0, st>>>(jobs_, job, q_[0], &counters_->n_cur, &counters_->nf_cur, capacity_,
                                         &counters_->overflow_queue);
    times_.launches += 1;
    SRT_CUDA_TRY(cudaGetLastError());
    return SRT_OK;
}

void Engine::launch_iteration(int parity, cudaStream_t st, bool prof, const cudaGraphConditionalHandle* cond)
{
    const PathQueue& cur = q_[parity];
    const PathQueue& nxt = q_[parity ^ 1];
    // inside stream capture a plain event record only orders streams; the
    // External flag makes it a real timestamp node of the graph
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    if (prof) cudaStreamIsCapturing(st, &cs);
    auto mark_on = [&](cudaStream_t s, int k, int e) {
        if (!prof) return;
        if (cs == cudaStreamCaptureStatusActive)
            cudaEventRecordWithFlags(ev_[parity][k][e], s, cudaEventRecordExternal);
        else
            cudaEventRecord(ev_[parity][k][e], s);  // direct launches (SRT_NO_GRAPH=1)
    };
    auto mark = [&](int k, int e) { mark_on(st, k, e); };
    mark(0, 0);
    if (prof && count_)
        k_trace<true><<<grid_trace_, kTraceThreads, 0, st>>>(jobs_, cur, sq_, hits_, counters_, capacity_, 0);
    else
        k_trace<false><<<grid_trace_, kTraceThreads, 0, st>>>(jobs_, cur, sq_, hits_, counters_, capacity_, 0);
    mark(0, 1);
    // k_regen (the previous iteration's ended samples) and k_order (this
    // iteration's hits) touch disjoint data: k_regen runs on a forked stream
    // beside k_order, and k_shade, which reads the sample counts k_regen
    // writes, waits for both; k_regen takes half the grid of a lone launch
    // (grid_regen_), which balances the two branches
    cudaEventRecord(fork_ev_, st);
    cudaStreamWaitEvent(side_stream_, fork_ev_, 0);
    mark_on(side_stream_, 3, 0);
    k_regen<<<grid_regen_, kThreads, 0, side_stream_>>>(jobs_, done_, counters_, capacity_);
    mark_on(side_stream_, 3, 1);
    cudaEventRecord(join_ev_, side_stream_);
    mark(2, 0);
    k_order<<<grid_order_, kOrderThreads, 0, st>>>(hits_, order_, counters_, capacity_);
    mark(2, 1);
    cudaStreamWaitEvent(st, join_ev_, 0);
    mark(1, 0);
    if (cache_)
        k_shade<true><<<grid_shade_, kShadeThreads, 0, st>>>(jobs_, cur, hits_, order_, nxt, sq_, done_, counters_,
                                                             capacity_);
    else
        k_shade<false><<<grid_shade_, kShadeThreads, 0, st>>>(jobs_, cur, hits_, order_, nxt, sq_, done_, counters_,
                                                              capacity_);
    if (cache_) launch_cache_queries(jobs_, max_jobs_, st);
    mark(1, 1);
    mark(4, 0);
    if (cond)
        k_advance<true><<<1, 1, 0, st>>>(counters_, history_, jobs_, max_jobs_, *cond);
    else
        k_advance<false><<<1, 1, 0, st>>>(counters_, history_, jobs_, max_jobs_, 0);
    mark(4, 1);
}

void Engine::launch_post(cudaStream_t st, bool prof)
{
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    if (prof) cudaStreamIsCapturing(st, &cs);
    auto mark = [&](int e) {
        if (!prof) return;
        if (cs == cudaStreamCaptureStatusActive)
            cudaEventRecordWithFlags(ev_tail_[e], st, cudaEventRecordExternal);
        else
            cudaEventRecord(ev_tail_[e], st);
    };
    mark(0);
    // the last iteration's shadow rays and ended samples
    if (prof && count_)
        k_trace<true><<<grid_trace_, kTraceThreads, 0, st>>>(jobs_, q_[0], sq_, hits_, counters_, capacity_, 1);
    else
        k_trace<false><<<grid_trace_, kTraceThreads, 0, st>>>(jobs_, q_[0], sq_, hits_, counters_, capacity_, 1);
    k_regen<<<grid_stride_, kThreads, 0, st>>>(jobs_, done_, counters_, capacity_);
    k_end_flush<<<1, 1, 0, st>>>(counters_);
    if (tail_on()) {
        if (prof && count_)
            k_finish<true><<<grid_finish_, kFinishThreads, 0, st>>>(jobs_, q_[0], counters_, capacity_);
        else
            k_finish<false><<<grid_finish_, kFinishThreads, 0, st>>>(jobs_, q_[0], counters_, capacity_);
        k_end_tail<<<1, 1, 0, st>>>(counters_);
    }
    mark(1);
}

void Engine::drop_graphs()
{
    if (graph_) cudaGraphExecDestroy(graph_);
    if (graph_prof_) cudaGraphExecDestroy(graph_prof_);
    graph_ = graph_prof_ = nullptr;
}

srt_status Engine::capture(bool prof)
{
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaSuccess;
    if (prof) {
        // profiling: one iteration pair with timestamps, relaunched by the host
        SRT_CUDA_TRY(cudaStreamBeginCapture(graph_stream_, cudaStreamCaptureModeThreadLocal));
        launch_iteration(0, graph_stream_, true, nullptr);
        launch_iteration(1, graph_stream_, true, nullptr);
        e = cudaStreamEndCapture(graph_stream_, &g);
        if (e != cudaSuccess) return cuda_error(e, "capture wavefront iteration");
    } else {
        // a conditional while node whose body is one iteration pair: a single
        // graph launch iterates on the device until k_advance ends the loop
        SRT_CUDA_TRY(cudaGraphCreate(&g, 0));
        cudaGraphConditionalHandle cond = 0;
        e = cudaGraphConditionalHandleCreate(&cond, g, 1, cudaGraphCondAssignDefault);
        cudaGraphNodeParams np{};
        np.type = cudaGraphNodeTypeConditional;
        np.conditional.handle = cond;
        np.conditional.type = cudaGraphCondTypeWhile;
        np.conditional.size = 1;
        cudaGraphNode_t node = nullptr;
        if (e == cudaSuccess) e = cudaGraphAddNode(&node, g, nullptr, nullptr, 0, &np);
        cudaGraph_t body = e == cudaSuccess ? np.conditional.phGraph_out[0] : nullptr;
        if (e == cudaSuccess)
            e = cudaStreamBeginCaptureToGraph(graph_stream_, body, nullptr, nullptr, 0,
                                              cudaStreamCaptureModeThreadLocal);
        if (e == cudaSuccess) {
            launch_iteration(0, graph_stream_, false, &cond);
            launch_iteration(1, graph_stream_, false, &cond);
            e = cudaStreamEndCapture(graph_stream_, &body);
        }
        // after the loop: the last iteration's shadow rays and ended samples,
        // then the end of the frame when the loop stopped for it
        if (e == cudaSuccess) {
            e = cudaStreamBeginCaptureToGraph(graph_stream_, g, &node, nullptr, 1, cudaStreamCaptureModeThreadLocal);
            if (e == cudaSuccess) {
                launch_post(graph_stream_, false);
                cudaGraph_t same = g;
                e = cudaStreamEndCapture(graph_stream_, &same);
            }
        }
        if (e != cudaSuccess) {
            cudaGraphDestroy(g);
            return cuda_error(e, "build the wavefront loop graph");
        }
    }
    cudaGraphExec_t& out = prof ? graph_prof_ : graph_;
    e = cudaGraphInstantiate(&out, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) {
        out = nullptr;
        return cuda_error(e, "instantiate wavefront graph");
    }
    return SRT_OK;
}

srt_status Engine::reset_counters(cudaStream_t st)
{
    SRT_CUDA_TRY(cudaMemsetAsync(counters_, 0, sizeof(Counters), st));
    return SRT_OK;
}

srt_status Engine::read_counters(Counters& c, cudaStream_t st)
{
    SRT_CUDA_TRY(cudaMemcpyAsync(host_counters_, counters_, sizeof(Counters), cudaMemcpyDeviceToHost, st));
    SRT_CUDA_TRY(cudaStreamSynchronize(st));
    c = *host_counters_;
    return SRT_OK;
}

srt_status Engine::read_history(IterCount* host, int n)
{
    if (n <= 0) return SRT_OK;
    n = std::min(n, kIterHistory);
    SRT_CUDA_TRY(cudaMemcpy(host, history_, sizeof(IterCount) * (size_t)n, cudaMemcpyDeviceToHost));
    return SRT_OK;
}

srt_status Engine::run(cudaStream_t st, long long max_iters, bool until_idle, long long budget_iters)
{
    const bool prof = profile_;
    // direct launches: the handle's launch mode, or SRT_NO_GRAPH=1 for every
    // engine of the process (diagnostics)
    static const bool env_no_graph = [] {
        const char* v = std::getenv("SRT_NO_GRAPH");
        return v && v[0] == '1';
    }();
    const bool no_graph = env_no_graph || direct_;
    if (prof && !ev_[0][0][0]) {
        for (auto& a : ev_)
            for (auto& b : a)
                for (auto& e : b) SRT_CUDA_TRY(cudaEventCreate(&e));
        for (auto& e : ev_tail_) SRT_CUDA_TRY(cudaEventCreate(&e));
    }
    if (!no_graph && prof && !graph_prof_) SRT_TRY(capture(true));
    if (!no_graph && !prof && !graph_) SRT_TRY(capture(false));
    cudaGraphExec_t graph = prof ? graph_prof_ : graph_;
    cudaEvent_t ev = nullptr;
    SRT_CUDA_TRY(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
    const char* what = "record caller-stream event";
    // order the internal stream after the caller's stream
    cudaError_t e = cudaEventRecord(ev, st);
    if (e == cudaSuccess) {
        what = "wait on caller-stream event";
        e = cudaStreamWaitEvent(graph_stream_, ev, 0);
    }
    long long iters = 0;
    srt_status status = SRT_OK;
    if (!prof && !no_graph && e == cudaSuccess) {
        // one graph launch: the device iterates until no path is in flight, a
        // queue or stack overflows, or the launch's iteration bound is reached
        const long long limit = budget_iters > 0 ? budget_iters : (max_iters > 0 ? max_iters + 1 : (1LL << 20));
        what = "start device loop";
        k_begin_run<<<1, 1, 0, graph_stream_>>>(counters_, limit, tail_on() ? tail_below_ : 0);
        e = cudaGetLastError();
        if (e == cudaSuccess) {
            what = "cudaGraphLaunch";
            e = cudaGraphLaunch(graph, graph_stream_);
        }
        if (e == cudaSuccess) {
            what = "copy counters";
            e = cudaMemcpyAsync(host_counters_, counters_, sizeof(Counters), cudaMemcpyDeviceToHost, graph_stream_);
        }
        if (e == cudaSuccess) {
            what = "synchronize iteration graph";
            e = cudaStreamSynchronize(graph_stream_);
        }
        if (e == cudaSuccess) {
            const Counters& c = *host_counters_;
            iters = c.run_iters;
            times_.launches += 1 + iters * (cache_ ? 6 : 5) + 3 + (tail_on() ? 2 : 0);
            if (c.overflow_queue)
                status = set_error(SRT_ERR_ARG, "wavefront queue capacity exceeded");
            else if (c.overflow_stack)
                status = set_error(SRT_ERR_STACK, "traversal stack overflow");
            else if (c.n_cur > 0 && budget_iters <= 0 && iters >= limit)
                status = set_error(SRT_ERR_TIMEOUT, "wavefront did not drain within the iteration bound");
        }
    }
    int per_check = 2;
    if ((prof || no_graph) && e == cudaSuccess) {
        what = "start host loop";
        k_begin_run<<<1, 1, 0, graph_stream_>>>(counters_, 1LL << 40, tail_on() ? tail_below_ : 0);
        e = cudaGetLastError();
        times_.launches += 1;
    }
    auto read_counters_now = [&]() {
        what = "copy counters";
        e = cudaMemcpyAsync(host_counters_, counters_, sizeof(Counters), cudaMemcpyDeviceToHost, graph_stream_);
        if (e == cudaSuccess) {
            what = "synchronize iteration graph";
            e = cudaStreamSynchronize(graph_stream_);
        }
    };
    while ((prof || no_graph) && e == cudaSuccess) {
        if (prof) per_check = 1;  // events are re-recorded by every launch: read them each time
        what = "cudaGraphLaunch";
        for (int k = 0; k < per_check && e == cudaSuccess; ++k) {
            if (no_graph) {
                what = "direct iteration launch";
                launch_iteration(0, graph_stream_, prof, nullptr);
                launch_iteration(1, graph_stream_, prof, nullptr);
                e = cudaGetLastError();
            } else {
                e = cudaGraphLaunch(graph, graph_stream_);
            }
            iters += 2;
            times_.launches += 2 * (cache_ ? 6 : 5);
        }
        if (e != cudaSuccess) break;
        read_counters_now();
        if (e != cudaSuccess) break;
        if (prof) {
            what = "cudaEventElapsedTime";
            for (int par = 0; par < 2 && e == cudaSuccess; ++par)
                for (int k = 0; k < 5 && e == cudaSuccess; ++k) {
                    float ms = 0.0f;
                    e = cudaEventElapsedTime(&ms, ev_[par][k][0], ev_[par][k][1]);
                    times_.ms[k] += ms;
                }
            if (e != cudaSuccess) break;
        }
        const Counters& c = *host_counters_;
        if (c.overflow_queue) {
            status = set_error(SRT_ERR_ARG, "wavefront queue capacity exceeded");
            break;
        }
        if (c.overflow_stack) {
            status = set_error(SRT_ERR_STACK, "traversal stack overflow");
            break;
        }
        // stop: nothing in flight (only a new job can add work), the end of
        // the frame for k_finish, the step's budget, or the bound
        const bool over = max_iters > 0 && iters > max_iters;
        if (c.n_cur == 0 || c.tail_go || (budget_iters > 0 && iters >= budget_iters) || over) {
            what = "flush and end of frame";
            launch_post(graph_stream_, prof);
            e = cudaGetLastError();
            times_.launches += 3 + (tail_on() ? 2 : 0);
            if (e == cudaSuccess) read_counters_now();
            if (e == cudaSuccess && prof) {
                what = "cudaEventElapsedTime";
                float ms = 0.0f;
                e = cudaEventElapsedTime(&ms, ev_tail_[0], ev_tail_[1]);
                times_.tail_ms += ms;
            }
            if (e == cudaSuccess && over && budget_iters <= 0 && host_counters_->n_cur > 0)
                status = set_error(SRT_ERR_TIMEOUT, "wavefront did not drain within the iteration bound");
            break;
        }
        per_check = std::min(per_check * 2, 16);
    }
    if (e == cudaSuccess) {
        what = "record graph-stream event";
        e = cudaEventRecord(ev, graph_stream_);
    }
    if (e == cudaSuccess) {
        what = "caller stream waits on graph stream";
        e = cudaStreamWaitEvent(st, ev, 0);
    }
    cudaEventDestroy(ev);
    if (e != cudaSuccess) {
        std::string msg = std::string("wavefront run (") + what + ", iteration " + std::to_string(iters) + ")";
        return cuda_error(e, msg.c_str());
    }
    return status;
}

}  // namespace srt

// ---------------------------------------------------------------------------
// srt_pt: the PathTracer pass (src/passes/integrator/path_tracer.{h,cu})
// ---------------------------------------------------------------------------
using namespace srt;

extern "C" srt_status srt_pt_create(srt_scene* scene, int32_t width, int32_t height, srt_pt** out)
{
    clear_error();
    if (!out) return set_error(SRT_ERR_ARG, "out is NULL");
    *out = nullptr;
    if (!scene) return set_error(SRT_ERR_ARG, "scene is NULL");
    if (width <= 0 || height <= 0 || (int64_t)width * height > (int64_t)1 << 27)
        return set_error(SRT_ERR_ARG, "film size out of range");
    srt_pt* p = new (std::nothrow) srt_pt();
    if (!p) return set_error(SRT_ERR_OOM, "host allocation failed");
    p->scene = scene;
    p->width = width;
    p->height = height;
    const size_t npix = (size_t)width * height;
    srt_status st = p->engine.init((int64_t)npix, 1);
    // the end of the frame from at most min(SRT_PT_TAIL_DEFAULT, pixels / 8) paths in flight
    p->engine.set_tail((int32_t)std::min<int64_t>(SRT_PT_TAIL_DEFAULT, (int64_t)npix / 8));
    if (st == SRT_OK) st = p->job_buf.alloc(npix * 16 + 1024, "per-pixel path state");
    if (st != SRT_OK) {
        delete p;
        return st;
    }
    char* b = p->job_buf.as<char>();
    p->lpath = (float4*)b;
    *out = p;
    return SRT_OK;
}

extern "C" srt_status srt_pt_render(srt_pt* p, float* film, const srt_pt_params* prm, void* stream)
{
    clear_error();
    if (!p || !film || !prm) return set_error(SRT_ERR_ARG, "NULL argument");
    if (reinterpret_cast<uintptr_t>(film) % 16 != 0) return set_error(SRT_ERR_ARG, "film must be 16-byte aligned");
    if (prm->samples_per_pixel < 0 || prm->max_depth < 0 || prm->max_depth > 255)
        return set_error(SRT_ERR_ARG, "samples_per_pixel / max_depth out of range");
    if (prm->rng_mode != SRT_RNG_CURAND)
        return set_error(SRT_ERR_UNSUPPORTED, "only SRT_RNG_CURAND is available for srt_pt_render");
    auto t0 = std::chrono::steady_clock::now();
    cudaStream_t st = as_stream(stream);
    const int npix = p->width * p->height;
    srt_scene* sc = p->scene;
    if (prm->samples_per_pixel == 0 || prm->max_depth == 0) {
        // no path segment is traced: every pixel is (0, 0, 0, 1)
        std::vector<float4> black((size_t)npix, make_float4(0.0f, 0.0f, 0.0f, 1.0f));
        SRT_CUDA_TRY(cudaMemcpyAsync(film, black.data(), (size_t)npix * 16, cudaMemcpyHostToDevice, st));
        SRT_CUDA_TRY(cudaStreamSynchronize(st));
        p->stats = srt_pt_stats{};
        p->stats.samples = (int64_t)npix * prm->samples_per_pixel;
        return SRT_OK;
    }
    if (prm->use_nee && sc->view.num_lights == 0) {
        // the reference would index an empty light CDF; NEE without lights adds nothing
    }
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
    p->engine.times() = KernelTimes();
    SRT_TRY(p->engine.reset_counters(st));
    SRT_TRY(p->engine.set_job(0, J, st));
    SRT_TRY(p->engine.start_job(0, J, st));
    long long bound = (long long)prm->samples_per_pixel * (prm->max_depth + 1) + 16;
    SRT_TRY(p->engine.run(st, 2 * bound, true, 0));
    Counters c;
    SRT_TRY(p->engine.read_counters(c, st));
    auto t1 = std::chrono::steady_clock::now();
    p->stats.samples = c.started;
    p->stats.closest_rays = c.closest_total;
    p->stats.shadow_rays = c.shadow_total;
    p->stats.iterations = c.iterations;
    p->stats.stack_overflows = c.overflow_stack;
    p->stats.render_ms = (float)std::chrono::duration<double, std::milli>(t1 - t0).count();
    const KernelTimes& kt = p->engine.times();
    p->stats.kernel_launches = kt.launches;
    for (int k = 0; k < 5; ++k) p->stats.kernel_ms[k] = (float)kt.ms[k];
    p->stats.closest_nodes = c.c_nodes;
    p->stats.closest_tris = c.c_tris;
    p->stats.shadow_nodes = c.s_nodes;
    p->stats.shadow_tris = c.s_tris;
    p->stats.tail_paths = c.tail_paths;
    p->stats.tail_ms = (float)kt.tail_ms;
    return SRT_OK;
}

extern "C" srt_status srt_pt_set_profiling(srt_pt* p, int32_t enable)
{
    clear_error();
    if (!p) return set_error(SRT_ERR_ARG, "NULL argument");
    if (enable < 0 || enable > 2) return set_error(SRT_ERR_ARG, "profiling mode must be 0, 1 or 2");
    p->engine.set_profiling(enable);
    return SRT_OK;
}

extern "C" srt_status srt_pt_get_stats(const srt_pt* p, srt_pt_stats* s)
{
    clear_error();
    if (!p || !s) return set_error(SRT_ERR_ARG, "NULL argument");
    *s = p->stats;
    return SRT_OK;
}

extern "C" srt_status srt_pt_set_launch_mode(srt_pt* p, int32_t mode)
{
    clear_error();
    if (!p) return set_error(SRT_ERR_ARG, "NULL argument");
    if (mode != SRT_LAUNCH_GRAPH && mode != SRT_LAUNCH_DIRECT)
        return set_error(SRT_ERR_ARG, "launch mode must be SRT_LAUNCH_GRAPH or SRT_LAUNCH_DIRECT");
    p->engine.set_direct(mode == SRT_LAUNCH_DIRECT);
    return SRT_OK;
}

extern "C" srt_status srt_pt_set_tail(srt_pt* p, int64_t max_paths)
{
    clear_error();
    if (!p) return set_error(SRT_ERR_ARG, "NULL argument");
    if (max_paths < 0 || max_paths > (int64_t)0x7fffffff) return set_error(SRT_ERR_ARG, "max_paths out of range");
    p->engine.set_tail((int32_t)max_paths);
    return SRT_OK;
}

extern "C" srt_status srt_pt_get_iteration_counts(const srt_pt* p, int32_t* counts, int32_t max_iterations,
                                                  int32_t* n_iterations)
{
    clear_error();
    if (!p || !n_iterations || max_iterations < 0 || (max_iterations > 0 && !counts))
        return set_error(SRT_ERR_ARG, "bad arguments");
    const int recorded = (int)std::min<int64_t>(p->stats.iterations, kIterHistory);
    *n_iterations = recorded;
    const int n = std::min(recorded, (int)max_iterations);
    if (n <= 0) return SRT_OK;
    std::vector<IterCount> h((size_t)n);
    SRT_TRY(const_cast<srt_pt*>(p)->engine.read_history(h.data(), n));
    for (int i = 0; i < n; ++i) {
        counts[5 * i + 0] = h[i].closest;
        counts[5 * i + 1] = h[i].hits;
        counts[5 * i + 2] = h[i].misses;
        counts[5 * i + 3] = h[i].shadow;
        counts[5 * i + 4] = h[i].done;
    }
    return SRT_OK;
}

extern "C" srt_status srt_pt_get_pixel_samples(const srt_pt* p, int32_t* samples)
{
    clear_error();
    if (!p || !samples) return set_error(SRT_ERR_ARG, "NULL argument");
    const size_t npix = (size_t)p->width * p->height;
    // the w word of each pixel's 16-byte radiance record counts its finished samples
    SRT_CUDA_TRY(cudaMemcpy2D(samples, 4, reinterpret_cast<const char*>(p->lpath) + 12, 16, 4, npix,
                              cudaMemcpyDeviceToHost));
    return SRT_OK;
}

extern "C" void srt_pt_destroy(srt_pt* p) { delete p; }

extern "C" srt_status srt_rng_tape(int32_t seed, int64_t npix, int32_t ndraws, float* out, void* stream)
{
    clear_error();
    if (npix < 0 || ndraws < 0 || (npix > 0 && ndraws > 0 && !out)) return set_error(SRT_ERR_ARG, "bad arguments");
    if (npix == 0 || ndraws == 0) return SRT_OK;
    int blocks = (int)((npix + 255) / 256);
    k_rng_tape<<<blocks, 256, 0, as_stream(stream)>>>(seed, npix, ndraws, out);
    SRT_CUDA_TRY(cudaGetLastError());
    return SRT_OK;
}
