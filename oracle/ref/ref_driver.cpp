// Reference build driver (test infrastructure only).
//
// Compiles the reference's own device headers for the host
// (src/device_include/scene/{bxdf,gmaterial,gmesh,light,camera}.h,
// params/hit_info.h, math/*.h) and exposes their functions over batches so
// tests/golden/make_golden.py can write golden vectors that pin the CPU
// oracle.  Nothing here is shipped; the library lands in oracle/_ref/ and
// is git-ignored.  The render loop below is a restatement of
// src/shader/integrator/path_tracer.cu:50-169 whose BxDF, light, camera,
// hit-attribute and RNG calls all go to the reference's classes; the
// intersection is a brute-force watertight test (OptiX is not available).
#include "my_math.h"
#include "scene/bxdf.h"
#include "scene/camera.h"
#include "scene/gmaterial.h"
#include "scene/gmesh.h"
#include "scene/light.h"
#include "params/hit_info.h"

#include <algorithm>
#include <cstdint>
#include <cstring>
#include <vector>

#include "../../include/srt.h"

namespace {

BxDF make_bxdf(int type, const float* p)
{
    BxDF b;
    b.type = (BxDF::Type)type;
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

BxDF bxdf_of(const srt_bxdf& m)
{
    float p[12] = {m.ior, m.metallic, m.subsurface, m.roughness, m.specular, m.specularTint,
                   m.anisotropic, m.sheen, m.sheenTint, m.clearcoat, m.clearcoatGloss, m.specTrans};
    return make_bxdf(m.type, p);
}

struct RefScene {
    std::vector<GMaterial> mats;
    std::vector<std::vector<float3>> verts, norms;
    std::vector<std::vector<uint3>> idx;
    std::vector<std::vector<float>> cdf;
    std::vector<GTriangleMesh> meshes;
    std::vector<Transform> xf;
    std::vector<GInstance> inst;
    std::vector<int> inst_light;
    std::vector<GInstance> area_lights;
    std::vector<float> weight_cdf;
    EnvironmentLight env;
    Light light;
    Camera camera;
    // flattened world triangles for the brute-force intersector
    std::vector<float3> w0, w1, w2;
    std::vector<int> tri_inst, tri_face;
};

Transform xf_of(const float* m)
{
    Transform t;
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 4; ++c) t[r][c] = m[4 * r + c];
    t[3][0] = t[3][1] = t[3][2] = 0.0f;
    t[3][3] = 1.0f;
    return t;
}

Camera make_camera(const srt_camera_desc& c)
{
    Camera cam((Camera::Type)c.type, c.aspect, c.fov);
    float3 pos = make_float3(c.position[0], c.position[1], c.position[2]);
    float3 tgt = make_float3(c.target[0], c.target[1], c.target[2]);
    float3 up = make_float3(c.up[0], c.up[1], c.up[2]);
    cam.set_controller(Transform::LookAt(pos, tgt, up), length(pos - tgt));
    cam.aperture = c.aperture;
    cam.focal = c.focal;
    cam.reset();
    return cam;
}

// watertight ray/triangle test (Woop, Benthin, Wald 2013)
bool tri_hit(float3 o, float3 d, float3 v0, float3 v1, float3 v2, float tmin, float tmax, float& t, float& b1,
             float& b2)
{
    float dd[3] = {d.x, d.y, d.z};
    float ad[3] = {fabsf(d.x), fabsf(d.y), fabsf(d.z)};
    int kz = 0;
    if (ad[1] > ad[kz]) kz = 1;
    if (ad[2] > ad[kz]) kz = 2;
    int kx = (kz + 1) % 3, ky = (kx + 1) % 3;
    if (dd[kz] < 0.0f) std::swap(kx, ky);
    float Sx = dd[kx] / dd[kz], Sy = dd[ky] / dd[kz], Sz = 1.0f / dd[kz];
    float3 A = v0 - o, B = v1 - o, C = v2 - o;
    float a[3] = {A.x, A.y, A.z}, b[3] = {B.x, B.y, B.z}, c[3] = {C.x, C.y, C.z};
    float Ax = a[kx] - Sx * a[kz], Ay = a[ky] - Sy * a[kz];
    float Bx = b[kx] - Sx * b[kz], By = b[ky] - Sy * b[kz];
    float Cx = c[kx] - Sx * c[kz], Cy = c[ky] - Sy * c[kz];
    float U = Cx * By - Cy * Bx, V = Ax * Cy - Ay * Cx, W = Bx * Ay - By * Ax;
    if ((U < 0.0f || V < 0.0f || W < 0.0f) && (U > 0.0f || V > 0.0f || W > 0.0f)) return false;
    float det = U + V + W;
    if (det == 0.0f) return false;
    float Tt = U * (Sz * a[kz]) + V * (Sz * b[kz]) + W * (Sz * c[kz]);
    float inv = 1.0f / det;
    float tt = Tt * inv;
    if (!(tt > tmin && tt < tmax)) return false;
    t = tt;
    b1 = V * inv;
    b2 = W * inv;
    return true;
}

int closest(const RefScene& s, float3 o, float3 d, float tmin, float tmax, float& u, float& v, bool any)
{
    int best = -1;
    float t, b1, b2;
    for (size_t i = 0; i < s.w0.size(); ++i) {
        if (tri_hit(o, d, s.w0[i], s.w1[i], s.w2[i], tmin, tmax, t, b1, b2)) {
            tmax = t;
            u = b1;
            v = b2;
            best = (int)i;
            if (any) return best;
        }
    }
    return best;
}

}  // namespace

extern "C" {

void ref_bxdf_sample(int type, int64_t n, const float* normal, const float* wo, const float* color,
                     const float* params, const float* rnd, float* wi, float* f, float* pdf, int32_t* delta)
{
    for (int64_t k = 0; k < n; ++k) {
        GMaterial m;
        m.bxdf = make_bxdf(type, params + 12 * k);
        Onb onb(make_float3(normal[3 * k], normal[3 * k + 1], normal[3 * k + 2]));
        BxDFSample s = m.sample(make_float3(wo[3 * k], wo[3 * k + 1], wo[3 * k + 2]),
                                make_float2(rnd[2 * k], rnd[2 * k + 1]), onb,
                                make_float3(color[3 * k], color[3 * k + 1], color[3 * k + 2]));
        if (s.pdf == 0.0f && !s.delta) {  // BxDFSample(): f and wi left unset by the reference
            s.f = make_float3(0.0f);
            s.wi = make_float3(0.0f);
        }
        wi[3 * k] = s.wi.x; wi[3 * k + 1] = s.wi.y; wi[3 * k + 2] = s.wi.z;
        f[3 * k] = s.f.x; f[3 * k + 1] = s.f.y; f[3 * k + 2] = s.f.z;
        pdf[k] = s.pdf;
        delta[k] = s.delta ? 1 : 0;
    }
}

void ref_bxdf_eval_pdf(int type, int64_t n, const float* normal, const float* wo, const float* color,
                       const float* params, const float* wi, float* f, float* pdf)
{
    for (int64_t k = 0; k < n; ++k) {
        GMaterial m;
        m.bxdf = make_bxdf(type, params + 12 * k);
        Onb onb(make_float3(normal[3 * k], normal[3 * k + 1], normal[3 * k + 2]));
        float3 w = make_float3(wi[3 * k], wi[3 * k + 1], wi[3 * k + 2]);
        float3 o = make_float3(wo[3 * k], wo[3 * k + 1], wo[3 * k + 2]);
        float3 c = make_float3(color[3 * k], color[3 * k + 1], color[3 * k + 2]);
        float3 fv = m.eval(w, o, onb, c);
        f[3 * k] = fv.x; f[3 * k + 1] = fv.y; f[3 * k + 2] = fv.z;
        pdf[k] = m.sample_pdf(w, o, onb, c);
    }
}

void ref_camera_rays(const srt_camera_desc* cd, int64_t n, const float* xy, float* rays)
{
    Camera cam = make_camera(*cd);
    RandomGenerator rng;
    for (int64_t i = 0; i < n; ++i) {
        Ray r = cam.get_ray(xy[2 * i], xy[2 * i + 1], rng);
        float* o = rays + 8 * i;
        o[0] = r.pos.x; o[1] = r.pos.y; o[2] = r.pos.z; o[3] = 0.0f;
        o[4] = r.dir.x; o[5] = r.dir.y; o[6] = r.dir.z; o[7] = 1e16f;
    }
}

// Camera of a pbrt file, built as PBRTParser::parse_options does
// (src/importer/pbrtparse.cu:331-387): the 16 numbers of its Transform
// statement row by row into SquareMatrix<4>, Inverse(Transpose(.)), first
// column negated, CameraController(transform, radius 1).
void ref_pbrt_camera_rays(const float* m16, float fov, float aspect, int64_t n, const float* xy, float* rays)
{
    SquareMatrix<4> mat(m16);
    mat = Inverse(Transpose(mat));
    Transform camera_to_world(SquareMatrix<4>(
        -mat[0][0], mat[0][1], mat[0][2], mat[0][3],
        -mat[1][0], mat[1][1], mat[1][2], mat[1][3],
        -mat[2][0], mat[2][1], mat[2][2], mat[2][3],
        -mat[3][0], mat[3][1], mat[3][2], mat[3][3]));
    Camera cam(Camera::Type::Perspective, aspect, fov);
    cam.set_controller(camera_to_world, 1.0f);
    RandomGenerator rng;
    for (int64_t i = 0; i < n; ++i) {
        Ray r = cam.get_ray(xy[2 * i], xy[2 * i + 1], rng);
        float* o = rays + 8 * i;
        o[0] = r.pos.x; o[1] = r.pos.y; o[2] = r.pos.z; o[3] = 0.0f;
        o[4] = r.dir.x; o[5] = r.dir.y; o[6] = r.dir.z; o[7] = 1e16f;
    }
}

// Scene set-up following Scene::build_gscene_{materials,meshes,instances}
// (src/scene/scene.cu:271-418) and TriangleMesh::compute_area
// (src/scene/mesh.cpp:3-18), in host memory.
void* ref_scene_create(const srt_scene_desc* d)
{
    RefScene* s = new RefScene();
    s->mats.resize(d->num_materials);
    for (int i = 0; i < d->num_materials; ++i) {
        const srt_material& m = d->materials[i];
        s->mats[i].bxdf = bxdf_of(m.bxdf);
        s->mats[i].base_color = make_float3(m.base_color[0], m.base_color[1], m.base_color[2]);
        s->mats[i].emission_color = make_float3(m.emission_color[0], m.emission_color[1], m.emission_color[2]);
        s->mats[i].intensity = m.intensity;
    }
    int nm = d->num_meshes;
    s->verts.resize(nm);
    s->norms.resize(nm);
    s->idx.resize(nm);
    s->cdf.resize(nm);
    s->meshes.resize(nm);
    for (int i = 0; i < nm; ++i) {
        const srt_mesh& m = d->meshes[i];
        for (int k = 0; k < m.num_vertices; ++k) {
            s->verts[i].push_back(make_float3(m.vertices[3 * k], m.vertices[3 * k + 1], m.vertices[3 * k + 2]));
            if (m.normals)
                s->norms[i].push_back(make_float3(m.normals[3 * k], m.normals[3 * k + 1], m.normals[3 * k + 2]));
        }
        for (int f = 0; f < m.num_faces; ++f)
            s->idx[i].push_back(make_uint3(m.indices[3 * f], m.indices[3 * f + 1], m.indices[3 * f + 2]));
        float area = 0.0f;
        s->cdf[i].resize(m.num_faces);
        for (int f = 0; f < m.num_faces; ++f) {
            uint3 t = s->idx[i][f];
            float3 v0 = s->verts[i][t.x], v1 = s->verts[i][t.y], v2 = s->verts[i][t.z];
            area += 0.5f * length(cross(v1 - v0, v2 - v0));
            s->cdf[i][f] = area;
        }
        for (int f = 0; f < m.num_faces; ++f) s->cdf[i][f] /= area;
        GTriangleMesh& g = s->meshes[i];
        g.vert_num = m.num_vertices;
        g.face_num = m.num_faces;
        g.vertices = s->verts[i].data();
        g.indices = s->idx[i].data();
        g.normals = s->norms[i].empty() ? nullptr : s->norms[i].data();
        g.area = area;
        g.area_cdf = s->cdf[i].data();
        g.material = &s->mats[m.material_id];
    }
    int ni = d->num_instances;
    s->xf.resize(ni);
    s->inst.resize(ni);
    s->inst_light.assign(ni, -1);
    for (int i = 0; i < ni; ++i) {
        s->xf[i] = xf_of(d->instances[i].transform);
        s->inst[i].mesh = &s->meshes[d->instances[i].mesh_id];
        s->inst[i].transform = &s->xf[i];
    }
    float wsum = 0.0f;
    for (int i = 0; i < ni; ++i) {
        const GTriangleMesh& g = *s->inst[i].mesh;
        if (g.material->intensity <= 0.0f) continue;
        s->inst_light[i] = (int)s->area_lights.size();
        s->area_lights.push_back(s->inst[i]);
        wsum += g.material->intensity * g.area;
        s->weight_cdf.push_back(wsum);
    }
    for (float& c : s->weight_cdf) c /= wsum;
    s->env.type = EnvironmentLight::Type::Constant;
    s->env.emission_color = make_float3(d->env_color[0], d->env_color[1], d->env_color[2]);
    s->light.num = (int)s->area_lights.size();
    s->light.lights = s->area_lights.data();
    s->light.weight_sum = wsum;
    s->light.weight_cdf = s->weight_cdf.data();
    s->light.env_light = &s->env;
    s->camera = make_camera(d->camera);
    for (int i = 0; i < ni; ++i) {
        const GTriangleMesh& g = *s->inst[i].mesh;
        for (int f = 0; f < g.face_num; ++f) {
            uint3 t = g.indices[f];
            s->w0.push_back(s->xf[i].apply_point(g.vertices[t.x]));
            s->w1.push_back(s->xf[i].apply_point(g.vertices[t.y]));
            s->w2.push_back(s->xf[i].apply_point(g.vertices[t.z]));
            s->tri_inst.push_back(i);
            s->tri_face.push_back(f);
        }
    }
    return s;
}

void ref_scene_destroy(void* p) { delete (RefScene*)p; }

// Light::sample (light.h:61-70): pos, normal, emission, pdf per sample
void ref_light_sample(void* p, int64_t n, const float* u2, float* out)
{
    RefScene* s = (RefScene*)p;
    for (int64_t i = 0; i < n; ++i) {
        LightSample ls = s->light.sample(make_float2(u2[2 * i], u2[2 * i + 1]));
        float* o = out + 10 * i;
        o[0] = ls.pos.x; o[1] = ls.pos.y; o[2] = ls.pos.z;
        o[3] = ls.normal.x; o[4] = ls.normal.y; o[5] = ls.normal.z;
        o[6] = ls.emission.x; o[7] = ls.emission.y; o[8] = ls.emission.z;
        o[9] = ls.pdf;
    }
}

// get_hitinfo (hit_info.h:27-64) for global primitive ids:
// out 15 floats = pos, normal, onb.z, onb.x, onb.y
void ref_hitinfo(void* p, int64_t n, const int32_t* prim, const float* uv, float* out)
{
    RefScene* s = (RefScene*)p;
    for (int64_t i = 0; i < n; ++i) {
        HitInfo h;
        int inst = s->tri_inst[prim[i]], face = s->tri_face[prim[i]];
        get_hitinfo(h, &s->inst[inst], face, make_float2(uv[2 * i], uv[2 * i + 1]), make_float3(0.0f),
                    s->inst_light[inst]);
        float v[15] = {h.pos.x, h.pos.y, h.pos.z, h.normal.x, h.normal.y, h.normal.z, h.onb.z.x, h.onb.z.y,
                       h.onb.z.z, h.onb.x.x, h.onb.x.y, h.onb.x.z, h.onb.y.x, h.onb.y.y, h.onb.y.z};
        std::memcpy(out + 15 * i, v, sizeof(v));
    }
}

// Path tracer loop over the reference's pieces; film: cw*ch*4 floats.
void ref_render(void* p, int w, int h, int x0, int y0, int cw, int ch, int spp, int max_depth, int rr_depth,
                int use_nee, int use_mis, int seed, float* film)
{
    RefScene* s = (RefScene*)p;
    const Light* light = &s->light;
    for (int ky = 0; ky < ch; ++ky)
        for (int kx = 0; kx < cw; ++kx) {
            int ix = x0 + kx, iy = y0 + ky;
            int idx = iy * w + ix;
            RandomGenerator rng(seed + idx, 0);
            float3 result = make_float3(0.0f);
            for (int i = 0; i < spp; ++i) {
                float xx = (ix + rng.random_float()) / w;
                float yy = (iy + rng.random_float()) / h;
                Ray ray = s->camera.get_ray(xx, yy, rng);
                bool specular = true;
                float scatter_pdf = 1.0f;
                float3 L = make_float3(0.0f), beta = make_float3(1.0f);
                for (int depth = 0; depth < max_depth; depth++) {
                    float u = 0, v = 0;
                    int prim = closest(*s, ray.pos, ray.dir, 1e-3f, 1e16f, u, v, false);
                    if (prim < 0) {
                        L += beta * light->environment_emission(ray.dir);
                        break;
                    }
                    HitInfo info;
                    int inst = s->tri_inst[prim];
                    get_hitinfo(info, &s->inst[inst], s->tri_face[prim], make_float2(u, v), ray.dir,
                                s->inst_light[inst]);
                    if (info.mat->is_emissive()) {
                        float cos_i = dot(info.normal, -ray.dir);
                        if (cos_i <= 1e-4f) break;
                        float mis_weight = 1.0f;
                        if (use_nee && !specular) {
                            mis_weight = 0.0f;
                            if (use_mis) {
                                float t2 = dot(info.pos - ray.pos, info.pos - ray.pos);
                                float light_pdf = light->sample_pdf(info.light_id) * t2 / cos_i;
                                mis_weight = scatter_pdf / (light_pdf + scatter_pdf);
                            }
                        }
                        L += beta * info.mat->emission(info.texcoord) * mis_weight;
                        break;
                    }
                    float cos_i = dot(info.normal, -ray.dir);
                    if (cos_i < 0.0f) info.normal = -info.normal;
                    if (use_nee && !info.mat->is_specular()) {
                        float r0 = rng.random_float();
                        float r1 = rng.random_float();
                        LightSample ls = light->sample(make_float2(r0, r1));
                        Ray sr(info.pos, normalize(ls.pos - info.pos));
                        float cos_o = dot(info.normal, sr.dir);
                        float cos_light = dot(ls.normal, -sr.dir);
                        float t = length(ls.pos - info.pos);
                        if ((cos_light > 1e-4f) && (ls.pdf > 1e-4f) && (t > 1e-3f) &&
                            (cos_o > 0.0f || info.mat->is_transmissive())) {
                            float su, sv;
                            bool visible = closest(*s, sr.pos, sr.dir, 1e-3f, t - 1e-3f, su, sv, true) < 0;
                            if (visible) {
                                float mis_weight = 1.0f;
                                float light_pdf = ls.pdf * t * t / cos_light;
                                if (use_mis) {
                                    float mat_pdf = info.mat->sample_pdf(sr.dir, -ray.dir, info.onb, info.color);
                                    mis_weight = light_pdf / (light_pdf + mat_pdf);
                                }
                                L += beta * info.mat->eval(sr.dir, -ray.dir, info.onb, info.color) * fabsf(cos_o) *
                                     ls.emission * mis_weight / light_pdf;
                            }
                        }
                    }
                    float r0 = rng.random_float();
                    float r1 = rng.random_float();
                    BxDFSample ms = info.mat->sample(-ray.dir, make_float2(r0, r1), info.onb, info.color);
                    if (ms.pdf <= 1e-4f) break;
                    if (dot(ms.wi, info.normal) < 0.0f && !info.mat->is_transmissive()) break;
                    beta *= ms.f / ms.pdf;
                    if (!ms.delta) beta *= fabsf(dot(ms.wi, info.normal));
                    specular = info.mat->is_specular();
                    ray = Ray(info.pos, ms.wi);
                    scatter_pdf = ms.pdf;
                    if (depth >= rr_depth) {
                        float q = max(max(beta.x, max(beta.y, beta.z)), 0.05f);
                        if (rng.random_float() > q) break;
                        beta /= q;
                    }
                }
                if (check_valid(L.x) && check_valid(L.y) && check_valid(L.z)) result += L / spp;
            }
            float* o = film + 4 * ((size_t)ky * cw + kx);
            o[0] = result.x; o[1] = result.y; o[2] = result.z; o[3] = 1.0f;
        }
}

}  // extern "C"
