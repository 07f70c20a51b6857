/*
 * srt.h — C ABI of the GB300-native wavefront path tracer.
 *
 * Every entry point takes plain pointers and sizes.  Device pointers are
 * passed as `void*` / `float*` and must point to memory on the current CUDA
 * device; `stream` is a `cudaStream_t` passed as `void*` (NULL = legacy
 * default stream).  No entry point calls exit() or traps: failures come back
 * as an `srt_status` and the last message is readable via srt_last_error().
 *
 * Each declaration names the reference interface it replaces (paths are
 * relative to the woAIxuexiSR/SRT source tree).
 */
#ifndef SRT_H
#define SRT_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Replaces `cout << "ERROR::..."; exit(-1)` (src/passes/renderpass.h:59-62,
 * src/main/main.cu:9-13) and checkCudaErrors / OPTIX_CHECK exits
 * (src/device_include/helper_optix.h:12-20). */
typedef enum srt_status {
    SRT_OK = 0,
    SRT_ERR_ARG = 1,         /* invalid argument / inconsistent sizes          */
    SRT_ERR_OOM = 2,         /* device or host allocation failed               */
    SRT_ERR_CUDA = 3,        /* a CUDA runtime call failed                     */
    SRT_ERR_TIMEOUT = 4,     /* a bounded device/host wait ran out             */
    SRT_ERR_BUDGET = 5,      /* admission refused: HBM budget would be exceeded */
    SRT_ERR_STACK = 6,       /* traversal stack overflowed (result incomplete) */
    SRT_ERR_NOT_FOUND = 7,   /* unknown render-pass / scene name               */
    SRT_ERR_PARSE = 8,       /* malformed JSON configuration                   */
    SRT_ERR_UNSUPPORTED = 9  /* feature the library does not support           */
} srt_status;

/* Message of the last failing call on this thread ("" if none). */
const char* srt_last_error(void);
/* Library version string. */
const char* srt_version(void);

/* ------------------------------------------------------------------ */
/* Scene description (host arrays)                                     */
/* ------------------------------------------------------------------ */

/* BxDF::Type, src/device_include/scene/bxdf.h:62 */
typedef enum srt_bxdf_type {
    SRT_BXDF_DIFFUSE = 0,
    SRT_BXDF_DIFFUSE_TRANSMISSION = 1,
    SRT_BXDF_DIELECTRIC = 2,
    SRT_BXDF_DISNEY = 3
} srt_bxdf_type;

/* BxDF parameters, same names, order and defaults as
 * src/device_include/scene/bxdf.h:64-76 (52 bytes). */
typedef struct srt_bxdf {
    int32_t type;
    float ior, metallic, subsurface, roughness, specular, specularTint,
          anisotropic, sheen, sheenTint, clearcoat, clearcoatGloss, specTrans;
} srt_bxdf;

/* Material, src/scene/material.h:8-19 (texture ids unsupported). */
typedef struct srt_material {
    srt_bxdf bxdf;
    float base_color[3];
    float emission_color[3];
    float intensity;          /* > 0 makes every instance of it an area light */
} srt_material;

/* TriangleMesh, src/scene/mesh.h:63-93.  Vertices/normals/tangents are
 * float3 packed (3 floats each), texture coordinates float2 packed;
 * indices are uint3 packed.  Without texcoords a hit's texture coordinate
 * is its barycentric (u, v); without tangents the shading frame's tangent
 * is the reference's axis choice (hit_info.h:48-52). */
typedef struct srt_mesh {
    const float* vertices;     /* 3 * num_vertices                    */
    const uint32_t* indices;   /* 3 * num_faces                       */
    const float* normals;      /* 3 * num_vertices, or NULL           */
    int32_t num_vertices;
    int32_t num_faces;
    int32_t material_id;       /* index into srt_scene_desc.materials */
    int32_t pad;
    const float* texcoords;    /* 2 * num_vertices, or NULL           */
    const float* tangents;     /* 3 * num_vertices, or NULL           */
} srt_mesh;

/* Texture image (Texture / Image, src/scene/texture.h), uploaded as
 * Scene::build_gscene_textures does (src/scene/scene.cu:92-139): a CUDA
 * array read with bilinear filtering, wrap addressing and normalised
 * coordinates; RGBA8 texels decode as sRGB (the reference sets sRGB = 1
 * for 8-bit images) to normalised floats, RGBA32F texels are linear.
 * Row 0 of `pixels` is texture coordinate v = 0. */
enum { SRT_TEXTURE_RGBA8 = 0, SRT_TEXTURE_RGBA32F = 1 };
typedef struct srt_texture {
    int32_t width, height;
    int32_t format;            /* SRT_TEXTURE_*                       */
    int32_t pad;
    const void* pixels;        /* 4 * width * height uint8 or float   */
} srt_texture;

/* Scene::add_instance(transform, mesh), src/scene/scene.cu:194-202.
 * transform: row-major 3x4 (the top 3 rows of the reference's 4x4). */
typedef struct srt_instance {
    int32_t mesh_id;
    float transform[12];
} srt_instance;

/* Camera::Type, src/device_include/scene/camera.h:96 */
typedef enum srt_camera_type {
    SRT_CAMERA_PERSPECTIVE = 0,
    SRT_CAMERA_ORTHOGRAPHIC = 1,
    SRT_CAMERA_THINLENS = 2,
    SRT_CAMERA_ENVIRONMENT = 3
} srt_camera_type;

/* Flag OR'd into srt_camera_desc.type: the camera's x axis is
 * -normalize(cross(up, z)) instead of +normalize(cross(up, z)), the
 * left-handed frame the reference builds from a pbrt camera transform by
 * negating the first column of Inverse(Transpose(M))
 * (src/importer/pbrtparse.cu:346-357).  y stays cross(z, +x). */
#define SRT_CAMERA_MIRROR_X 0x100

/* The "camera" JSON block of Renderer::load_scene, src/renderer/renderer.cu:125-140:
 * LookAt(position, target, up), radius = |position - target|, vertical fov
 * in degrees, aspect = width / height. */
typedef struct srt_camera_desc {
    int32_t type;
    float position[3];
    float target[3];
    float up[3];
    float fov;
    float aspect;
    float aperture;           /* thin lens only (camera.h:101) */
    float focal;              /* thin lens only                */
} srt_camera_desc;

/* Scene::build_gscene inputs, src/scene/scene.cu:214-418; env_color is the
 * constant EnvironmentLight (src/device_include/scene/light.h:204-234). */
typedef struct srt_scene_desc {
    const srt_mesh* meshes;
    int32_t num_meshes;
    const srt_instance* instances;
    int32_t num_instances;
    const srt_material* materials;
    int32_t num_materials;
    srt_camera_desc camera;
    float env_color[3];
    /* textures (zero / NULL: none) */
    const srt_texture* textures;
    int32_t num_textures;
    /* "uvmap" environment (EnvironmentLight::emission, light.h:27-41):
     * texture index + 1, or 0 for the constant env_color */
    int32_t env_map;
    /* per material: color_tex, normal_tex texture indices or -1
     * (GMaterial, gmaterial.h:13-56); NULL: no material is textured */
    const int32_t* material_textures;
} srt_scene_desc;

typedef struct srt_scene srt_scene;

typedef struct srt_scene_info {
    int64_t num_triangles;
    int64_t num_nodes;           /* 128-byte 8-wide BVH nodes              */
    int64_t num_lights;          /* area-light instances                   */
    int64_t device_bytes;        /* resident HBM held by the scene         */
    int32_t bvh_depth;           /* deepest node level                     */
    float build_ms;              /* host BVH build + upload time           */
    float light_weight_sum;      /* Σ intensity·area, scene.cu:388-391     */
} srt_scene_info;

/* Scene::build_gscene + OptixRayTracer GAS/IAS build
 * (src/scene/scene.cu:214-418, src/optix/optix_ray_tracer.cu:213-359):
 * flattens instances, builds the binned-SAH 8-wide BVH, the light CDFs,
 * and uploads everything to the current device. */
srt_status srt_scene_create(const srt_scene_desc* desc, srt_scene** out);
/* Camera change without rebuilding geometry (camera.h:165-170). */
srt_status srt_scene_set_camera(srt_scene* scene, const srt_camera_desc* camera);
srt_status srt_scene_get_info(const srt_scene* scene, srt_scene_info* info);
/* Maps a global primitive id (instance order, then face order) to
 * (instance, face): the OptiX pair (instance, optixGetPrimitiveIndex()). */
srt_status srt_scene_prim_to_instance(const srt_scene* scene, int64_t prim,
                                      int32_t* instance, int32_t* face);
void srt_scene_destroy(srt_scene* scene);

/* ------------------------------------------------------------------ */
/* Ray queries (replace optixTrace of path_tracer.cu:75-78, :124-127)  */
/* ------------------------------------------------------------------ */

/* rays:  n x 8 floats  (ox, oy, oz, tmin, dx, dy, dz, tmax), device.
 * hits:  n x 4 floats  (t, u, v, prim as int32 bits; prim = -1 on miss), device.
 * u, v are the barycentrics of vertex 1 and 2 (optixGetTriangleBarycentrics). */
srt_status srt_trace_closest(const srt_scene* scene, const float* rays, int64_t n,
                             float* hits, void* stream);
/* visible: n int32 (1 = unoccluded in (tmin, tmax), 0 = occluded), device. */
srt_status srt_trace_shadow(const srt_scene* scene, const float* rays, int64_t n,
                            int32_t* visible, void* stream);
/* tex2D<float4> of the scene's texture `texture` (srt_scene_desc.textures
 * order) at n normalised coordinates: uv n x 2 floats, out n x 4 floats,
 * both device memory.  The lookups the shading kernel makes. */
srt_status srt_scene_texture_lookup(const srt_scene* scene, int32_t texture, const float* uv, int64_t n,
                                    float* out, void* stream);

/* ------------------------------------------------------------------ */
/* Path tracing pass (src/passes/integrator/path_tracer.{h,cu})         */
/* ------------------------------------------------------------------ */

/* Random-number modes. */
enum {
    /* per-pixel curand XORWOW stream curand_init(seed + idx, 0, 0),
     * u = 1 - curand_uniform (src/device_include/math/random.h:9-31);
     * one path per pixel in flight, consumption order of path_tracer.cu:50-169 */
    SRT_RNG_CURAND = 0,
    /* counter-based hash of (seed, pixel, sample, dimension): stateless, lets
     * several samples of one pixel be in flight at once */
    SRT_RNG_HASH = 1
};

/* Flags for srt_pt_params.flags. */
enum {
    /* Light / triangle CDF remap done correctly ((u - cdf[i-1]) / pdf_i).
     * Default (0) reproduces the reference's `int lower = cdf[idx-1]`
     * truncation (light.h:65, gmesh.h:49). */
    SRT_PT_FIXED_CDF_REMAP = 1,
    /* Next-event estimation at the first surface vertex only (no shadow rays
     * from later vertices; a later vertex's emission keeps the MIS weight of
     * the previous vertex's light sample).  With max_depth 2 this is the path
     * prefix that a cache ending paths at the second vertex keeps: the
     * benchmark measures its variance to bound what such a cache can gain.
     * No counterpart in the reference. */
    SRT_PT_NEE_FIRST_VERTEX_ONLY = 2
};

/* PathTracer JSON params + frame seed (path_tracer.h:15-19, 30-39;
 * integrator_params.h:9-24). */
typedef struct srt_pt_params {
    int32_t samples_per_pixel;   /* default 1  */
    int32_t max_depth;           /* default 16 */
    int32_t rr_depth;            /* default 4  */
    int32_t use_nee;             /* default 1  */
    int32_t use_mis;             /* default 1  */
    int32_t seed;                /* PathTracerParams::seed (path_tracer.cu:15) */
    int32_t rng_mode;            /* SRT_RNG_*  */
    int32_t flags;               /* SRT_PT_*   */
} srt_pt_params;

/* Counters of the last render (exact integers). */
typedef struct srt_pt_stats {
    int64_t samples;             /* samples finished = w*h*spp                   */
    int64_t closest_rays;        /* rays through the closest-hit kernel          */
    int64_t shadow_rays;         /* rays through the shadow kernel               */
    int64_t iterations;          /* wavefront iterations (closest+shade+shadow)  */
    int64_t stack_overflows;     /* traversal stack overflows (must be 0)        */
    float render_ms;             /* wall time of srt_pt_render (host clock)      */
    int64_t kernel_launches;     /* kernels this library launched for the frame  */
    /* Filled only while profiling is on (srt_pt_set_profiling): summed device
     * time of each kernel of the iteration from CUDA events recorded between
     * them -- [0] the traversal (the previous iteration's shadow rays and this
     * iteration's closest-hit rays), [1] shading, [2] the shading order,
     * [3] film accumulation, [4] the iteration's end -- and the traversal
     * work: 128-byte nodes visited and triangles tested, for closest-hit and
     * for shadow rays. */
    float kernel_ms[5];
    int64_t closest_nodes, closest_tris, shadow_nodes, shadow_tris;
    /* End of the frame (srt_pt_set_tail): paths the finishing kernel took
     * from the queue, each carried to its pixel's last sample, and the device
     * time after the iterations (profiling only: the last iteration's shadow
     * rays and ended samples, then the finishing kernel).  Rays it traced are
     * in closest_rays / shadow_rays; `iterations` counts the wavefront
     * iterations before it. */
    int64_t tail_paths;
    float tail_ms;
} srt_pt_stats;

typedef struct srt_pt srt_pt;

/* PathTracer::init (path_tracer.cu:5-11): allocates the path queues for a
 * width x height film against `scene`. */
srt_status srt_pt_create(srt_scene* scene, int32_t width, int32_t height, srt_pt** out);
/* PathTracer::render (path_tracer.cu:13-33): writes film[i] = (L/spp, 1)
 * for every pixel i = iy*width + ix.  `film` is a device float4[w*h].
 * Stream-ordered; returns after the frame has been enqueued and its
 * completion polled (the reference synchronises at the same point). */
srt_status srt_pt_render(srt_pt* pt, float* film, const srt_pt_params* params, void* stream);
/* LightTracer pass (src/passes/integrator/light_tracer.cu:13-33,
 * src/shader/integrator/light_tracer.cu:57-175): clears `film`
 * (float4[w*h], device) to (0, 0, 0, 1), then traces samples_per_pixel
 * light paths per launch index w*h from that index's curand stream
 * (seed + idx), connecting every non-specular vertex to the pinhole camera
 * and adding the contribution to the pixel it lands on.  Uses
 * samples_per_pixel, max_depth, rr_depth, seed and flags of `params`
 * (curand streams only).  Perspective cameras only (Camera::get_xy).
 * stats may be NULL. */
srt_status srt_lt_render(const srt_scene* scene, int32_t width, int32_t height, float* film,
                         const srt_pt_params* params, srt_pt_stats* stats, void* stream);

/* ------------------------------------------------------------------ */
/* NeuralRadiosity pass (src/passes/npr/neural_radiosity.{h,cu},       */
/* src/shader/npr/nr_lhs.cu, nr_rhs.cu)                                */
/* ------------------------------------------------------------------ */

enum { SRT_NR_LHS = 0, SRT_NR_RHS = 1 };
/* The pass's network in the reference's configuration: hash grid on the
 * position (8 levels x 8 features, 2^19 entries, base resolution 16,
 * scale 2, smoothstep), degree-3 spherical harmonics of direction and
 * normal, the colour, padded with ones to 96; 96 -> 256 x 4 (ReLU) -> 16
 * (3 used), no biases, BF16 with FP32 accumulation.  Parameters are one
 * float vector: grid features level by level (entry-major, 8 per entry),
 * then the layers' W[out][in].  Initialised from `seed` as tiny-cuda-nn
 * initialises (grid U(-1e-4, 1e-4), layers U(+-sqrt(6/(in+out)))). */
typedef struct srt_nr srt_nr;
int64_t srt_nr_num_params(void);
srt_status srt_nr_create(uint64_t seed, srt_nr** out);
srt_status srt_nr_get_params(const srt_nr* nr, float* host_params);
srt_status srt_nr_set_params(srt_nr* nr, const float* host_params);
/* save_model / load_model in this library's own file format (a tiny-cuda-nn
 * serialisation is not read). */
srt_status srt_nr_save(const srt_nr* nr, const char* path);
srt_status srt_nr_load(srt_nr* nr, const char* path);
/* inputs: n x 12 floats (device), out: n x 16 floats (device, 16-byte
 * aligned; 3 used).  The encoding kernel writes 128-row tiles; the five
 * layers run in one fused tensor-core kernel. */
srt_status srt_nr_infer(srt_nr* nr, const float* inputs, int64_t n, float* out, void* stream);
/* Profiling of srt_nr_infer (PROFILE() scopes of src/utils/profiler.h:219
 * applied to its two kernels): enable = 1 records CUDA events around the
 * encoding and the fused network kernel of every call and waits for them;
 * the last call's durations are read with srt_nr_get_stats. */
typedef struct srt_nr_stats {
    int64_t rows;            /* rows of the last profiled call            */
    float encode_ms;         /* hash-grid + SH encoding kernel            */
    float network_ms;        /* fused five-layer tensor-core kernel       */
} srt_nr_stats;
srt_status srt_nr_set_profiling(srt_nr* nr, int32_t enable);
/* Self-test of the bounded waits the tensor-core kernels use (no counterpart
 * in the reference, which has no such kernels): one CTA waits on an mbarrier
 * that nothing completes, gives up after limit_ns nanoseconds (1e3 .. 1e9)
 * and reports it through the flag those kernels set.  Returns
 * SRT_ERR_TIMEOUT, the expected outcome, with the device still usable. */
srt_status srt_selftest_wait_timeout(int64_t limit_ns);
srt_status srt_nr_get_stats(const srt_nr* nr, srt_nr_stats* stats);
void srt_nr_destroy(srt_nr* nr);
/* The LHS / RHS raygen of one sample with frame seed `seed` (curand stream
 * seed + pixel): mask (w*h bytes: 1 = the pixel needs no network), base
 * (w*h x 3), weight (w*h x 3, RHS only; may be NULL for LHS) and the
 * network inputs (w*h x 12; zero where mask = 1), all device memory. */
srt_status srt_nr_trace(const srt_scene* scene, int32_t width, int32_t height, int32_t type, int32_t seed,
                        uint8_t* mask, float* base, float* weight, float* inputs, void* stream);
/* NeuralRadiosity::render: `spp` samples with seeds[i], each traced,
 * inferred and combined (LHS: mask ? base : net; RHS: base + weight * net
 * where mask = 0), averaged into film (float4[w*h], device). */
srt_status srt_nr_render(const srt_scene* scene, srt_nr* nr, int32_t width, int32_t height, int32_t type,
                         int32_t spp, const int32_t* seeds, float* film, void* stream);
srt_status srt_pt_get_stats(const srt_pt* pt, srt_pt_stats* stats);
/* Profiling switch (PROFILE() scopes of src/utils/profiler.h:219 applied per
 * kernel).  enable = 1: the iteration graph carries event records between
 * the kernels, the host reads them after every graph launch, and the
 * traversal kernels are the variants that count their node visits and
 * triangle tests.  enable = 2: event records only, around kernels identical
 * to the unprofiled ones (their durations are the production kernels').
 * 0 turns profiling off.  Results land in srt_pt_stats. */
srt_status srt_pt_set_profiling(srt_pt* pt, int32_t enable);

/* How srt_pt_render issues a frame's wavefront iterations.  The reference
 * issues one optixLaunch per frame (path_tracer.cu:13-33); here a frame is
 * many short kernels per iteration.  SRT_LAUNCH_GRAPH (default): one launch
 * of a captured CUDA graph whose conditional while-node iterates on the
 * device.  SRT_LAUNCH_DIRECT: the same kernels launched one by one from the
 * host, checked every few iterations (same results, more host work; lets
 * kernel-level tools that do not look inside graphs see every kernel). */
enum { SRT_LAUNCH_GRAPH = 0, SRT_LAUNCH_DIRECT = 1 };
srt_status srt_pt_set_launch_mode(srt_pt* pt, int32_t mode);

/* End of a frame.  Each pixel's samples run one after another on its own
 * curand stream (path_tracer.cu:56-68), so near the end of a frame few
 * paths are left while a wavefront iteration still lasts as long as its
 * slowest ray.  Once at most `max_paths` paths are in flight, one kernel
 * takes them over and carries each, with its pixel's remaining samples, to
 * the end, through the same device code (the image is the same bit for
 * bit; iteration counts past that point are not recorded).  0 disables it;
 * the default is min(SRT_PT_TAIL_DEFAULT, width * height / 8) paths.
 * Renders with a radiance cache always run their iterations to the end. */
enum { SRT_PT_TAIL_DEFAULT = 65536 };
srt_status srt_pt_set_tail(srt_pt* pt, int64_t max_paths);

/* Queue counts of the last render's wavefront iterations (no counterpart in
 * the reference's megakernel; these are the integer counts its per-pixel
 * loop, path_tracer.cu:56-166, implies).  Iteration k holds, per pixel, the
 * k-th path segment of its sample sequence, so the counts are a function of
 * the per-pixel streams alone.  counts: host int32[5 * max_iterations]:
 * closest-hit rays, of which hits, misses; shadow rays; samples ended.
 * *n_iterations = the iterations recorded (the first 4096 of a render). */
srt_status srt_pt_get_iteration_counts(const srt_pt* pt, int32_t* counts, int32_t max_iterations,
                                       int32_t* n_iterations);
/* Finished samples per pixel of the last render (host int32[w*h]); equal
 * to samples_per_pixel everywhere after a complete frame (the reference's
 * `for (i < samples_per_pixel)` loop, path_tracer.cu:64). */
srt_status srt_pt_get_pixel_samples(const srt_pt* pt, int32_t* samples);
void srt_pt_destroy(srt_pt* pt);

/* curand tape: out[p * ndraws + k] = k-th draw of the pixel-p stream of
 * SRT_RNG_CURAND for frame seed `seed` (device float[npix*ndraws]). */
srt_status srt_rng_tape(int32_t seed, int64_t npix, int32_t ndraws, float* out, void* stream);

/* ------------------------------------------------------------------ */
/* BxDF batch (src/device_include/scene/gmaterial.h:59-103 over bxdf.h) */
/* ------------------------------------------------------------------ */

/* One shading point: world-space normal n (Onb(n), onb.h:11-16), outgoing
 * wo, surface color, material parameters, two uniforms for sample().
 * SoA device arrays, n points each:
 *   normal[3n] wo[3n] color[3n] params[12n] (ior, metallic, subsurface, roughness,
 *   specular, specularTint, anisotropic, sheen, sheenTint, clearcoat,
 *   clearcoatGloss, specTrans per point) rnd[2n]
 * Outputs (device): wi[3n], f[3n], pdf[n], delta[n] (int32). */
typedef struct srt_bxdf_batch {
    int64_t n;
    int32_t type;               /* srt_bxdf_type, same for all points */
    const float* normal;
    const float* wo;
    const float* color;
    const float* params;
    const float* rnd;
    float* wi;
    float* f;
    float* pdf;
    int32_t* delta;
} srt_bxdf_batch;

/* GMaterial::sample (gmaterial.h:74-89) for every point. */
srt_status srt_bxdf_sample(const srt_bxdf_batch* batch, void* stream);
/* GMaterial::eval / sample_pdf (gmaterial.h:59-72, 91-103) at the given
 * wi (read from batch->wi): writes f and pdf. */
srt_status srt_bxdf_eval(const srt_bxdf_batch* batch, void* stream);
/* Fills the Disney batch inputs in device memory from PCG32(seed=i, seq=0)
 * streams, point i in [first, first + n) (draw order: normal 2, wo 2,
 * color 3, 9 params, roughness 1, rnd 2 of 4). */
srt_status srt_bxdf_generate(int64_t first, const srt_bxdf_batch* batch, void* stream);

/* ------------------------------------------------------------------ */
/* Film passes (src/passes/postprocess/*.cu, src/utils/metrics.h)       */
/* ------------------------------------------------------------------ */

/* Accumulate::render (accumulate.cu:10-29): acc = acc*(1-w) + film*w,
 * w = 1/(frame_count+1); film = acc.  float4[n] device arrays. */
srt_status srt_film_accumulate(float* film, float* acc, int64_t n, int32_t frame_count, void* stream);

/* ToneMapping::Type, tonemapping.h:10 */
enum { SRT_TONE_NONE = 0, SRT_TONE_CLAMP = 1, SRT_TONE_REINHARD = 2,
       SRT_TONE_UNCHARTED2 = 3, SRT_TONE_ACES = 4 };
/* ToneMapping::render (tonemapping.cu:5-70), in place. */
srt_status srt_film_tonemap(float* film, int64_t n, int32_t type, float exposure,
                            int32_t use_gamma, void* stream);

/* Metrics::Type, metrics.h:11 */
enum { SRT_METRIC_MSE = 0, SRT_METRIC_MAPE = 1, SRT_METRIC_SMAPE = 2, SRT_METRIC_RELMSE = 3 };
/* Metrics::cal_image / Measure::render (metrics.h:53-70, measure.cu:35-49):
 * per-pixel error, drop the largest `discard` percent, mean of the rest.
 * `scratch` is a device buffer of at least srt_film_metric_scratch_bytes(n)
 * bytes owned by the caller; *out (host) receives the trimmed mean. */
size_t srt_film_metric_scratch_bytes(int64_t n);
/* Measure's "option" (measure.h:16, measure.cu:29-39): REFERENCE overwrites
 * the film with (ref.rgb, 1), ERROR with the per-pixel error of `type` as
 * (e, e, e, 1); NONE leaves it.  Both buffers float4[n] on the device. */
enum { SRT_MEASURE_NONE = 0, SRT_MEASURE_REFERENCE = 1, SRT_MEASURE_ERROR = 2 };
srt_status srt_film_measure_view(float* film, const float* ref, int64_t n, int32_t type, int32_t option,
                                 void* stream);
srt_status srt_film_metric(const float* x, const float* ref, int64_t n, int32_t type,
                           float discard, void* scratch, float* out, void* stream);

/* ------------------------------------------------------------------ */
/* Radiance-cache network (the learned part)                           */
/* ------------------------------------------------------------------ */

/* Replaces the tiny-cuda-nn network of the NeuralRadiosity pass
 * (src/passes/npr/neural_radiosity.cu:6-52: encoding + CutlassMLP, Adam,
 * relative L2 loss): 96 -> 5 x 64 (ReLU) -> 16 (exp on 3), BF16 weights,
 * FP32 accumulation on tensor cores.  One query record is 16 floats:
 * position, roughness, shading normal, -, direction toward the previous
 * vertex, -, albedo, -.  Outputs are float4 (RGB radiance, 0). */
typedef struct srt_mlp srt_mlp;
#define SRT_MLP_PARAMS 23552
srt_status srt_mlp_create(uint64_t seed, srt_mlp** out);
/* Scene box that normalises positions before the frequency encoding. */
srt_status srt_mlp_set_box(srt_mlp* mlp, const float* lo, const float* hi);
/* FP32 master weights, W_l[out][in] row-major for l = 0..5 (host arrays). */
srt_status srt_mlp_get_params(const srt_mlp* mlp, float* params);
srt_status srt_mlp_set_params(srt_mlp* mlp, const float* params);
/* records: device float[n*16]; out: device float[n*4]. */
srt_status srt_mlp_infer(const srt_mlp* mlp, const float* records, int64_t n, float* out, void* stream);
/* One Adam step (beta 0.9 / 0.99) on the relative L2 loss against
 * targets (device float[n*4], RGB used); *loss (host, may be NULL). */
srt_status srt_mlp_train_step(srt_mlp* mlp, const float* records, const float* targets, int64_t n,
                              float lr, float* loss, void* stream);
/* Loss gradient w.r.t. the weights without updating them (host float[SRT_MLP_PARAMS]). */
srt_status srt_mlp_gradient(srt_mlp* mlp, const float* records, const float* targets, int64_t n,
                            float* grad, float* loss, void* stream);
void srt_mlp_destroy(srt_mlp* mlp);

/* Radiance-cache rendering of one frame with the PathTracer pass (the
 * NeuralRadiosity pass's query-at-the-second-vertex estimator,
 * src/shader/npr/nr_rhs.cu:50-157, with the network trained online on the
 * tracer's own full paths instead of offline). */
typedef struct srt_cache_params {
    int32_t train_paths;      /* full-length training paths per frame (65536)          */
    int32_t train_steps;      /* Adam steps per frame over the gathered vertices (4)  */
    float learning_rate;      /* 1e-2                                                  */
    float region_threshold;   /* relative bias that disables a cell (plain fallback)   */
    int32_t region_res;       /* grid cells per axis over the network's scene box (16) */
    int32_t train;            /* 0: frozen network (inference only)                    */
} srt_cache_params;

typedef struct srt_cache_stats {
    int64_t queries;          /* paths ended by a network query                        */
    int64_t fallback_queries; /* second vertices in disabled cells (traced plainly)     */
    int64_t train_vertices;   /* training vertices gathered this frame                 */
    float loss;               /* mean relative L2 loss of this frame's Adam steps      */
    int32_t disabled_cells;   /* cells traced plainly next frame (unmeasured, or bias
                                 shown above the threshold)                            */
    float trace_ms;           /* host time of the frame's wavefront run                */
    float train_ms;           /* host time of gathering, cell statistics and Adam steps */
} srt_cache_stats;

srt_status srt_pt_render_cached(srt_pt* pt, float* film, const srt_pt_params* params, srt_mlp* mlp,
                                const srt_cache_params* cache, srt_cache_stats* stats, void* stream);

/* ------------------------------------------------------------------ */
/* Render serving: continuous batching over one wavefront engine        */
/* ------------------------------------------------------------------ */

/* The reference renders one scene per process, one pass after another
 * (InteractiveRenderer::run, src/renderer/renderer.cu:199-228); the server
 * keeps scenes, path queues and per-job state resident and packs the rays
 * of every admitted job into shared wavefront queues. */
typedef struct srt_server srt_server;

typedef struct srt_server_config {
    int64_t hbm_budget_bytes;     /* admission budget: engine + job state + films + scenes in use */
    int64_t max_paths;            /* paths in flight across jobs (one per pixel of each running job) */
    int32_t max_jobs;             /* concurrent job slots (<= 65535)                       */
    int32_t iterations_per_step;  /* wavefront iterations run by one srt_server_step (even) */
} srt_server_config;

typedef struct srt_job_desc {
    srt_scene* scene;             /* resident scene, owned by the caller                   */
    int32_t width, height;
    srt_pt_params params;         /* same meaning as for srt_pt_render                      */
    float* film;                  /* caller's device float4[w*h], or NULL: server-owned     */
    struct srt_mlp* cache;        /* radiance cache of this scene, or NULL                  */
    int32_t cache_train;          /* 1: train `cache` online on this job's own paths (one
                                     pixel in 1 + npix / 16384 traces full paths for its
                                     first sample; the network takes Adam steps when the
                                     job's first progressive frame completes); 0: frozen */
    int32_t pad;
} srt_job_desc;

enum { SRT_JOB_QUEUED = 0, SRT_JOB_RUNNING = 1, SRT_JOB_DONE = 2, SRT_JOB_FAILED = 3 };

typedef struct srt_job_info {
    int32_t state;                /* SRT_JOB_*                                              */
    int32_t frames_done;          /* progressive frames completed (every pixel has k samples) */
    double submit_s, admit_s, first_frame_s, done_s;  /* server clock, seconds              */
    int64_t device_bytes;         /* admitted HBM footprint of the job                      */
} srt_job_info;

srt_status srt_server_create(const srt_server_config* config, srt_server** out);
/* Queues a job (admitted by srt_server_step when a slot, paths and the HBM
 * budget allow).  A job that could never fit returns SRT_ERR_BUDGET. */
srt_status srt_server_submit(srt_server* s, const srt_job_desc* job, int64_t* job_id);
/* Admits queued jobs, runs iterations_per_step wavefront iterations over
 * all running jobs, retires finished jobs and records frame times. */
srt_status srt_server_step(srt_server* s, int32_t* running, int32_t* queued);
/* Steps until no job is queued or running, or `timeout_s` passes
 * (SRT_ERR_TIMEOUT). */
srt_status srt_server_drain(srt_server* s, double timeout_s);
srt_status srt_server_job_info(const srt_server* s, int64_t job_id, srt_job_info* info);
/* Completion time (server clock) of each progressive frame; n = frames_done. */
srt_status srt_server_frame_times(const srt_server* s, int64_t job_id, double* times, int32_t max, int32_t* n);
/* Device film of a job (the caller's, or the server-owned one). */
srt_status srt_server_film(const srt_server* s, int64_t job_id, float** film);
/* Frees a finished job's server-owned film and forgets the job. */
srt_status srt_server_release(srt_server* s, int64_t job_id);
/* Server clock now, seconds. */
double srt_server_now(const srt_server* s);
void srt_server_destroy(srt_server* s);

/* srt_film_metric without a scratch argument, for callers that cannot
 * allocate device memory when they measure a film: a serving loop that has
 * reserved its whole HBM budget up front, or code that must not let
 * cudaMalloc / cudaFree synchronise the device while other work is in
 * flight.  No counterpart in the reference (its Measure pass allocates a
 * GPUMemory error buffer per call).  The scratch is a fixed array in device
 * memory of up to 2,097,152 pixels (about 8 MB, held by every GPU that loads
 * the library until the process exits); larger n returns SRT_ERR_ARG.  It
 * allocates nothing.  The first call on a device looks the array's device
 * address up (set-up), so make that first call before any stream capture;
 * a context made anew on the device (after cudaDeviceReset) is looked up
 * again by the next call, which is then a first call too.  All calls on a
 * device share the array: calls that overlap on the GPU (different streams
 * or host threads) race and must be serialised by the caller. */
srt_status srt_film_metric_noalloc(const float* x, const float* ref, int64_t n, int32_t type,
                                   float discard, float* out, void* stream);

/* ------------------------------------------------------------------ */
/* Procedural scenes (inputs of the Cornell and 5.2M-triangle workloads) */
/* ------------------------------------------------------------------ */

typedef struct srt_procedural srt_procedural;
/* name: "cornell" | "spheres".  spheres: n_spheres icospheres of
 * `subdiv` subdivisions (81,920 faces at 6).  Host-side arrays only. */
srt_status srt_procedural_create(const char* name, uint64_t seed, int32_t n_spheres,
                                 int32_t subdiv, srt_procedural** out);
/* Borrowed view of the generated scene (valid until destroy). */
srt_status srt_procedural_desc(const srt_procedural* p, srt_scene_desc* desc);
void srt_procedural_destroy(srt_procedural* p);

/* Scene file into host arrays (Renderer::load_scene's model loading,
 * src/renderer/renderer.cu:102-123): ".pbrt" (the PBRTParser subset,
 * src/importer/pbrtparse.cu: shapes trianglemesh / plymesh, materials
 * diffuse / coateddiffuse / conductor / dielectric / diffusetransmission,
 * diffuse area lights, Film resolution and Camera fov and transform),
 * ".obj" with its ".mtl" (AssimpImporter, src/importer/assimp.cu:17-79) or
 * a lone ".ply" mesh.  Textures are not built: a pbrt Texture statement or
 * texture parameter returns SRT_ERR_UNSUPPORTED.  Malformed files return
 * SRT_ERR_PARSE; unreadable ones SRT_ERR_ARG.  The result is read with
 * srt_procedural_desc and released with srt_procedural_destroy. */
srt_status srt_import_scene(const char* path, srt_procedural** out);
/* Film size a pbrt file asks for (0 x 0 when it gives none). */
srt_status srt_procedural_resolution(const srt_procedural* p, int32_t* width, int32_t* height);

/* ------------------------------------------------------------------ */
/* Render-pass plugin API (src/passes/renderpass.h:10-80)               */
/* ------------------------------------------------------------------ */

/* JSON config with "render", "passes", "scene" (example/example.json).
 * Passes registered: PathTracer, Wavefront, LightTracer, NeuralRadiosity, Accumulate, ToneMapping, Measure.
 * scene.model: "procedural:cornell" | "procedural:spheres[:n[:subdiv[:seed]]]"
 * | a scene file (.pbrt, .obj, .ply). */
typedef struct srt_renderer srt_renderer;
/* create_renderer + load_scene + load_passes (src/main/main.cu:19-41,
 * src/renderer/renderer.cu:3-17, 42-174). */
srt_status srt_renderer_create(const char* json_config, srt_renderer** out);
/* ImageRenderer::run without the file save (renderer.cu:176-191): runs
 * every pass once on the film; `frames` repeats it. */
srt_status srt_renderer_run(srt_renderer* r, int32_t frames);
srt_status srt_renderer_size(const srt_renderer* r, int32_t* width, int32_t* height);
/* Copies the film (float4[w*h]) to host memory. */
srt_status srt_renderer_read_film(const srt_renderer* r, float* host_rgba);
/* Writes the film as a little-endian PFM (RGB float) to `path`. */
srt_status srt_renderer_save_pfm(const srt_renderer* r, const char* path);
/* create_renderer with main.cu's -r / -p / -s overrides (src/main/main.cu:57-62):
 * each non-NULL JSON text replaces that section of `json_config`. */
srt_status srt_renderer_create_ex(const char* json_config, const char* render, const char* passes, const char* scene,
                                  srt_renderer** out);
/* create_renderer(config_path, ...) of src/main/main.cu:19-41 with the same
 * overrides: reads the config file, and a scene.model that names a file
 * (.pbrt, .obj, .ply; see srt_import_scene) resolves against the config
 * file's directory, as Renderer::load_scene does (renderer.cu:44-46).
 * srt_renderer_create / _ex resolve such paths against the working
 * directory.  A pbrt film size stands in for an unset render.resolution;
 * obj / ply scenes need a "camera" block ("No camera specified"). */
srt_status srt_renderer_create_file(const char* config_path, const char* render, const char* passes,
                                    const char* scene, srt_renderer** out);
/* render.output of the config ("" when absent): the image file name, which
 * ImageRenderer::run resolves against the config file's directory. */
const char* srt_renderer_output(const srt_renderer* r);
/* ImageRenderer::run's save step (renderer.cu:183-187): the film through
 * srt_image_write with the reference's flip. */
srt_status srt_renderer_save(const srt_renderer* r, const char* path);
/* Image::save_to_file (src/scene/texture.cu:219-230, save_ldr / save_hdr
 * :132-168), host memory in, no GPU needed: rgba is float4[w*h] in film
 * order (row 0 = bottom of the picture).  By extension: .png (8-bit RGBA,
 * clamp(x,0,1)*255 truncated), .bmp (24-bit), .hdr (Radiance RGBE), .pfm
 * (float RGB), .exr (OpenEXR: channels B, G, R, A as half, no
 * compression, as the reference's save_exr writes them through tinyexr,
 * :69-130), .jpg (baseline JPEG at quality 100, as save_ldr asks
 * stbi_write_jpg for).  flip != 0 mirrors x and y first, as the reference
 * does before saving; PFM keeps its bottom-to-top rows.  Other extensions
 * return SRT_ERR_UNSUPPORTED. */
srt_status srt_image_write(const char* path, int32_t width, int32_t height, const float* rgba, int32_t flip);
/* Image::load_from_file for float images (texture.cu:170-217), by content:
 * OpenEXR (single-part scanline; half / float / uint; no compression, RLE,
 * ZIPS or ZIP; R, G, B and optional A, or one grey channel), Radiance HDR
 * (converted as stbi_loadf does) and PFM.  rgba == NULL asks for the size
 * only; otherwise rgba receives float4[w*h].  flip != 0 undoes
 * srt_image_write's flip (for EXR / HDR: the reference's
 * load_from_file(path, true, true), which the Measure pass uses), so a
 * film written with flip and read with flip comes back in film order.
 * 8-bit formats return SRT_ERR_UNSUPPORTED; malformed files SRT_ERR_PARSE.
 * flip is one of SRT_FLIP_*: XY = load_from_file(path, true, true), Y =
 * load_from_file(path, false, true) (pbrt image textures). */
enum { SRT_FLIP_NONE = 0, SRT_FLIP_XY = 1, SRT_FLIP_Y = 2 };
srt_status srt_image_read(const char* path, int32_t* width, int32_t* height, float* rgba, int32_t flip);
/* load_from_file's 8-bit branch (stbi_load(path, .., 4)): PNG (all colour
 * types and bit depths, palette and tRNS transparency, Adam7; 16-bit
 * samples cut to their high byte), uncompressed 24 / 32-bit BMP and
 * baseline JPEG (grey or YCbCr, any sampling, restart markers; decoded
 * with an exact IDCT, so samples may differ from stbi_load's integer IDCT
 * by a few levels) into RGBA8 (rgba: 4*w*h bytes, NULL for the size).
 * Progressive JPEG and other formats return SRT_ERR_UNSUPPORTED.  flip as
 * srt_image_read. */
srt_status srt_image_read_rgba8(const char* path, int32_t* width, int32_t* height, uint8_t* rgba, int32_t flip);
void srt_renderer_destroy(srt_renderer* r);
/* Names of the registered passes, ';'-separated (print_registered_pass). */
const char* srt_registered_passes(void);

#ifdef __cplusplus
}
#endif

#endif /* SRT_H */
