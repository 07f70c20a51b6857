/*
 * ORACLE — CPU restatement of the reference path-tracing hot path.
 *
 * Test infrastructure only: used by tests/, __graft_entry__.smoke() and
 * bench.py's cpu_baseline / reference arm, as the results the CUDA path is
 * compared against or as the timed CPU baseline, never as the product path.
 * The product library never links it.
 *
 * Parity pins: the BxDF, light, camera and hit-attribute pieces are checked
 * against golden vectors generated from the reference's own headers
 * compiled on the host (oracle/ref, tests/golden/make_golden.py); the RNG is
 * the toolkit's curand XORWOW compiled for the host (oracle/curand_host.cpp).
 * Traversal has no reference implementation here (OptiX is closed and not
 * installed): the brute-force intersector is its pin.
 */
#ifndef SRT_ORACLE_H
#define SRT_ORACLE_H

#include <stdint.h>
#include "../include/srt.h"

#ifdef __cplusplus
extern "C" {
#endif

/* PCG32 stream (O'Neill, pcg-random.org minimal C generator), seeded as
 * pcg32_srandom(initstate = i, initseq = 0); uniform = (next >> 8) * 2^-24. */
void oracle_pcg_uniforms(uint64_t initstate, uint64_t initseq, int n, float* out);

/* Disney batch inputs for points [first, first+n): SoA like srt_bxdf_batch
 * (normal, wo, color, params(12), rnd(2)).  rnd4 gets all 4 uniforms. */
void oracle_bxdf_generate(int64_t first, int64_t n, float* normal, float* wo, float* color,
                          float* params, float* rnd4);

/* GMaterial::sample / eval / sample_pdf over a batch (world space, Onb(n)).
 * precision: 32 = FP32 restatement, 64 = FP64 evaluation of the same formulas.
 * sample writes wi, f, pdf, delta; eval_pdf reads wi and writes f, pdf. */
void oracle_bxdf_sample(int precision, int type, int64_t n, const float* normal, const float* wo,
                        const float* color, const float* params, const float* rnd,
                        double* wi, double* f, double* pdf, int32_t* delta);
void oracle_bxdf_sample_mt(int precision, int type, int64_t n, const float* normal, const float* wo,
                           const float* color, const float* params, const float* rnd, double* wi, double* f,
                           double* pdf, int32_t* delta, int threads);
void oracle_bxdf_eval_pdf(int precision, int type, int64_t n, const float* normal, const float* wo,
                          const float* color, const float* params, const double* wi,
                          double* f, double* pdf);

/* Scene (object-space meshes + instances, as the reference holds them). */
typedef struct oracle_scene oracle_scene;
oracle_scene* oracle_scene_create(const srt_scene_desc* desc);
void oracle_scene_destroy(oracle_scene* s);
int64_t oracle_scene_num_triangles(const oracle_scene* s);
float oracle_scene_light_weight_sum(const oracle_scene* s);
/* Builds the oracle's own binary SAH BVH (needed for large scenes). */
void oracle_scene_build_bvh(oracle_scene* s);

/* Closest hit: rays n x 8 (ox,oy,oz,tmin,dx,dy,dz,tmax) -> hits n x 4
 * (t, u, v, prim bits; prim -1 on miss) and edge[n] = smallest barycentric
 * of the hit (distance-to-edge proxy).  use_bvh = 0 brute force. */
void oracle_trace_closest(const oracle_scene* s, const float* rays, int64_t n, float* hits,
                          float* edge, int use_bvh, int threads);
void oracle_trace_shadow(const oracle_scene* s, const float* rays, int64_t n, int32_t* visible,
                         int use_bvh, int threads);

/* Camera::get_ray for a perspective / orthographic camera at film coords. */
void oracle_camera_rays(const srt_camera_desc* cam, int64_t n, const float* xy, float* rays);

/* get_hitinfo for global primitive ids: pos, normal, onb z, x, y (n x 15). */
void oracle_hitinfo(const oracle_scene* s, int64_t n, const int32_t* prim, const float* uv, float* out);

/* An exact bilinear / sRGB restatement of a tex2D<float4> lookup of the
 * scene's texture `texture` at n coordinates (uv n x 2 -> out n x 4). */
void oracle_texture_lookup(const oracle_scene* s, int texture, int64_t n, const float* uv, float* out);

/* LightTracer (src/shader/integrator/light_tracer.cu:57-175): film gets
 * the sum of all splats (w*h x 3 doubles); counters[0] closest rays,
 * counters[1] camera connections traced.  Returns 2 without lights. */
int oracle_light_trace(const oracle_scene* s, int w, int h, const srt_pt_params* p, int use_bvh, int threads,
                       double* film, int64_t* counters);

/* NeuralRadiosity: one LHS (0) / RHS (1) sample of every pixel (mask,
 * base, weight, inputs as srt_nr_trace), and the network on n inputs
 * (params as srt_nr_get_params; out n x 3). */
int oracle_nr_trace(const oracle_scene* s, int w, int h, int type, int seed, int use_bvh, uint8_t* mask, float* base,
                    float* weight, float* inputs);
void oracle_nr_infer(const float* params, int64_t n, const float* inputs, float* out, int threads);

/* Light::sample(u) -> pos, normal, emission, pdf (n x 10 floats). */
void oracle_light_sample(const oracle_scene* s, int64_t n, const float* u2, int fixed_remap,
                         float* out);

/* Megakernel path tracer (src/shader/integrator/path_tracer.cu:50-169) on
 * the crop [x0, x0+cw) x [y0, y0+ch) of a w x h film.
 * film: cw*ch*4 floats = (result, 1).  sum / sumsq: cw*ch*3 doubles over the
 * per-sample estimates (non-finite samples count as 0).  counters[4]:
 * samples, closest rays, shadow rays, path vertices.  rng_mode SRT_RNG_*. */
int oracle_render(const oracle_scene* s, int w, int h, int x0, int y0, int cw, int ch,
                  const srt_pt_params* p, int use_bvh, int threads, float* film, double* sum,
                  double* sumsq, int64_t* counters);

/* oracle_render plus one byte per traced path segment of each pixel
 * (events: cw*ch*ev_max, zeroed by the caller): bit 0 traced, bit 1 hit,
 * bit 2 shadow ray traced, bit 3 the sample ended there. */
int oracle_render_events(const oracle_scene* s, int w, int h, int x0, int y0, int cw, int ch,
                         const srt_pt_params* p, int use_bvh, int threads, float* film, double* sum,
                         double* sumsq, int64_t* counters, uint8_t* events, int ev_max);
/* oracle_render over an arbitrary list of pixels (index iy*w + ix) of a
 * w x h film; film / sum / sumsq are per listed pixel. */
int oracle_render_pixels(const oracle_scene* s, int w, int h, const int32_t* pixels, int64_t n,
                         const srt_pt_params* p, int use_bvh, int threads, float* film, double* sum,
                         double* sumsq, int64_t* counters);
/* The procedural scene `name` ("cornell" | "spheres") of the benchmark
 * built from the generator source (scene_inputs.cpp), camera aspect set. */
oracle_scene* oracle_scene_create_procedural(const char* name, uint64_t seed, int32_t n_spheres,
                                             int32_t subdiv, float aspect);

/* Film passes. */
void oracle_accumulate(float* film, float* acc, int64_t n, int frame_count);
void oracle_tonemap(float* film, int64_t n, int type, float exposure, int use_gamma);
/* Per-pixel error (errors[n]) and the trimmed mean the reference reports. */
double oracle_metric(const float* x, const float* ref, int64_t n, int type, float discard,
                     float* errors);

/* Hash RNG of SRT_RNG_HASH: uniform for (seed, pixel, sample, dim). */
float oracle_hash_uniform(uint32_t seed, uint32_t pixel, uint32_t sample, uint32_t dim);

/* curand host build (curand_host.cpp). */
void oracle_curand_tape(int seed, long long npix, int ndraws, float* out);

#ifdef __cplusplus
}
#endif

#endif
