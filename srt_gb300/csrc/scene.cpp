// scene.cpp — srt_scene_create: validation, flattening, light tables, BVH
// build and upload.  Compiled with -ffp-contract=off: the world-space
// vertices, areas and CDFs are the same floats the reference computes on
// its host (mesh.cpp:3-18, scene.cu:370-417, transform.h:225-240).
#include "scene.h"

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <thread>

#include "bvh_build.h"
#include "bxdf.h"

using namespace srt;

namespace {

struct Xf {
    float m[12];
    float3 point(float3 p) const
    {
        return make_float3(m[0] * p.x + m[1] * p.y + m[2] * p.z + m[3], m[4] * p.x + m[5] * p.y + m[6] * p.z + m[7],
                           m[8] * p.x + m[9] * p.y + m[10] * p.z + m[11]);
    }
    float3 vec(float3 v) const
    {
        return make_float3(m[0] * v.x + m[1] * v.y + m[2] * v.z, m[4] * v.x + m[5] * v.y + m[6] * v.z,
                           m[8] * v.x + m[9] * v.y + m[10] * v.z);
    }
};

float3 ld3(const float* p) { return make_float3(p[0], p[1], p[2]); }

srt_status validate(const srt_scene_desc* d)
{
    if (!d) return set_error(SRT_ERR_ARG, "scene desc is NULL");
    if (d->num_meshes < 0 || d->num_instances < 0 || d->num_materials < 0)
        return set_error(SRT_ERR_ARG, "negative counts in scene desc");
    if ((d->num_meshes && !d->meshes) || (d->num_instances && !d->instances) || (d->num_materials && !d->materials))
        return set_error(SRT_ERR_ARG, "NULL array with non-zero count in scene desc");
    for (int i = 0; i < d->num_materials; ++i) {
        int t = d->materials[i].bxdf.type;
        if (t < SRT_BXDF_DIFFUSE || t > SRT_BXDF_DISNEY)
            return set_error(SRT_ERR_ARG, "material " + std::to_string(i) + ": unknown bxdf type");
    }
    for (int i = 0; i < d->num_meshes; ++i) {
        const srt_mesh& m = d->meshes[i];
        if (m.num_vertices < 0 || m.num_faces < 0)
            return set_error(SRT_ERR_ARG, "mesh " + std::to_string(i) + ": negative counts");
        if ((m.num_vertices && !m.vertices) || (m.num_faces && !m.indices))
            return set_error(SRT_ERR_ARG, "mesh " + std::to_string(i) + ": NULL arrays");
        if (m.material_id < 0 || m.material_id >= d->num_materials)
            return set_error(SRT_ERR_ARG, "mesh " + std::to_string(i) + ": material id out of range");
        for (int64_t k = 0; k < 3 * (int64_t)m.num_faces; ++k)
            if (m.indices[k] >= (uint32_t)m.num_vertices)
                return set_error(SRT_ERR_ARG, "mesh " + std::to_string(i) + ": vertex index out of range");
    }
    for (int i = 0; i < d->num_instances; ++i)
        if (d->instances[i].mesh_id < 0 || d->instances[i].mesh_id >= d->num_meshes)
            return set_error(SRT_ERR_ARG, "instance " + std::to_string(i) + ": mesh id out of range");
    const int cam_type = d->camera.type & ~SRT_CAMERA_MIRROR_X;
    if (cam_type != SRT_CAMERA_PERSPECTIVE && cam_type != SRT_CAMERA_ORTHOGRAPHIC)
        return set_error(SRT_ERR_UNSUPPORTED, "only perspective and orthographic cameras are supported");
    if (d->num_textures < 0 || (d->num_textures && !d->textures))
        return set_error(SRT_ERR_ARG, "bad texture array in scene desc");
    for (int i = 0; i < d->num_textures; ++i) {
        const srt_texture& t = d->textures[i];
        if (t.width <= 0 || t.height <= 0 || t.width > 65536 || t.height > 65536 || !t.pixels ||
            (t.format != SRT_TEXTURE_RGBA8 && t.format != SRT_TEXTURE_RGBA32F))
            return set_error(SRT_ERR_ARG, "texture " + std::to_string(i) + ": bad size, format or pixels");
    }
    if (d->env_map < 0 || d->env_map > d->num_textures) return set_error(SRT_ERR_ARG, "env_map out of range");
    if (d->material_textures)
        for (int i = 0; i < 2 * d->num_materials; ++i)
            if (d->material_textures[i] < -1 || d->material_textures[i] >= d->num_textures)
                return set_error(SRT_ERR_ARG, "material " + std::to_string(i / 2) + ": texture index out of range");
    return SRT_OK;
}

// a CUDA array + texture object read as the reference reads its textures
// (Scene::build_gscene_textures, scene.cu:92-139)
srt_status make_texture(const srt_texture& t, cudaArray_t& arr, cudaTextureObject_t& obj)
{
    const bool u8 = t.format == SRT_TEXTURE_RGBA8;
    cudaChannelFormatDesc cd = u8 ? cudaCreateChannelDesc<uchar4>() : cudaCreateChannelDesc<float4>();
    const size_t pitch = (size_t)t.width * (u8 ? 4 : 16);
    if (cudaMallocArray(&arr, &cd, t.width, t.height) != cudaSuccess) {
        arr = nullptr;
        cudaGetLastError();
        return set_error(SRT_ERR_OOM, "texture array allocation failed");
    }
    SRT_CUDA_TRY(cudaMemcpy2DToArray(arr, 0, 0, t.pixels, pitch, pitch, t.height, cudaMemcpyHostToDevice));
    cudaResourceDesc rd{};
    rd.resType = cudaResourceTypeArray;
    rd.res.array.array = arr;
    cudaTextureDesc td{};
    td.addressMode[0] = cudaAddressModeWrap;
    td.addressMode[1] = cudaAddressModeWrap;
    td.filterMode = cudaFilterModeLinear;
    td.readMode = u8 ? cudaReadModeNormalizedFloat : cudaReadModeElementType;
    td.normalizedCoords = 1;
    td.maxAnisotropy = 1;
    td.maxMipmapLevelClamp = 99;
    td.minMipmapLevelClamp = 0;
    td.mipmapFilterMode = cudaFilterModePoint;
    td.borderColor[0] = 1.0f;
    td.sRGB = u8 ? 1 : 0;
    SRT_CUDA_TRY(cudaCreateTextureObject(&obj, &rd, &td, nullptr));
    return SRT_OK;
}

MaterialRec pack_material(const srt_material& m, bool textured)
{
    Bxdf b{m.bxdf.type, m.bxdf.ior, m.bxdf.metallic, m.bxdf.subsurface, m.bxdf.roughness, m.bxdf.specular,
           m.bxdf.specularTint, m.bxdf.anisotropic, m.bxdf.sheen, m.bxdf.sheenTint, m.bxdf.clearcoat,
           m.bxdf.clearcoatGloss, m.bxdf.specTrans};
    int flags = m.bxdf.type & 0xff;
    if (bxdf_is_specular(b)) flags |= 1 << 8;
    if (bxdf_is_transmissive(b)) flags |= 1 << 9;
    if (m.intensity > 0.0f) flags |= 1 << 10;
    if (textured) flags |= 1 << 11;
    MaterialRec r;
    float f;
    std::memcpy(&f, &flags, 4);
    r.m[0] = make_float4(m.base_color[0], m.base_color[1], m.base_color[2], f);
    r.m[1] = make_float4(m.bxdf.ior, m.bxdf.metallic, m.bxdf.subsurface, m.bxdf.roughness);
    r.m[2] = make_float4(m.bxdf.specular, m.bxdf.specularTint, m.bxdf.anisotropic, m.bxdf.sheen);
    r.m[3] = make_float4(m.bxdf.sheenTint, m.bxdf.clearcoat, m.bxdf.clearcoatGloss, m.bxdf.specTrans);
    // GMaterial::emission = emission_color * intensity (gmaterial.h:35-41)
    r.m[4] = make_float4(m.emission_color[0] * m.intensity, m.emission_color[1] * m.intensity,
                         m.emission_color[2] * m.intensity, m.intensity);
    return r;
}

}  // namespace

namespace srt {

CameraRec make_camera(const srt_camera_desc& c)
{
    float3 pos = ld3(c.position), tgt = ld3(c.target), up = ld3(c.up);
    float3 z = normalize(tgt - pos);
    float3 x = normalize(cross(up, z));
    float3 y = cross(z, x);
    CameraRec k{};
    k.pos = pos;
    k.x = normalize(x);
    if (c.type & SRT_CAMERA_MIRROR_X) k.x = -1.0f * k.x;
    k.y = normalize(y);
    k.z = normalize(z);
    k.radius = length(pos - tgt);
    float rad = (c.fov * 0.5f) * (float)M_PI / 180.0f;
    k.nh = 2.0f * std::tan(rad);
    k.nw = k.nh * c.aspect;
    k.aperture = c.aperture;
    k.focal = c.focal;
    k.type = c.type & ~SRT_CAMERA_MIRROR_X;
    return k;
}

}  // namespace srt

extern "C" srt_status srt_scene_create(const srt_scene_desc* d, srt_scene** out)
{
    clear_error();
    if (!out) return set_error(SRT_ERR_ARG, "out is NULL");
    *out = nullptr;
    SRT_TRY(validate(d));
    auto t0 = std::chrono::steady_clock::now();
    srt_scene* s = new (std::nothrow) srt_scene();
    if (!s) return set_error(SRT_ERR_OOM, "host allocation failed");
    cudaGetDevice(&s->device);

    // per-mesh object-space area CDFs (TriangleMesh::compute_area, mesh.cpp:3-18)
    std::vector<float> mesh_area(d->num_meshes, 0.0f);
    std::vector<std::vector<float>> mesh_cdf(d->num_meshes);
    bool any_normals = false, any_tc = false, any_tg = false;
    for (int i = 0; i < d->num_meshes; ++i) {
        const srt_mesh& m = d->meshes[i];
        if (m.normals) any_normals = true;
        if (m.texcoords) any_tc = true;
        if (m.tangents) any_tg = true;
        std::vector<float>& cdf = mesh_cdf[i];
        cdf.resize(m.num_faces);
        float area = 0.0f;
        for (int f = 0; f < m.num_faces; ++f) {
            float3 v0 = ld3(m.vertices + 3 * m.indices[3 * f]);
            float3 v1 = ld3(m.vertices + 3 * m.indices[3 * f + 1]);
            float3 v2 = ld3(m.vertices + 3 * m.indices[3 * f + 2]);
            float A = 0.5f * length(cross(v1 - v0, v2 - v0));
            area += A;
            cdf[f] = area;
        }
        for (int f = 0; f < m.num_faces; ++f) cdf[f] /= area;
        mesh_area[i] = area;
    }

    // flatten instances into world-space triangles (global prim = instance order, face order)
    int64_t ntri = 0;
    s->inst_prim_base.resize(d->num_instances);
    s->inst_faces.resize(d->num_instances);
    for (int i = 0; i < d->num_instances; ++i) {
        s->inst_prim_base[i] = ntri;
        s->inst_faces[i] = d->meshes[d->instances[i].mesh_id].num_faces;
        ntri += s->inst_faces[i];
    }
    if (ntri > (int64_t)0x7fffffff / 3) {
        delete s;
        return set_error(SRT_ERR_ARG, "too many triangles");
    }
    std::vector<float> tri9((size_t)ntri * 9);
    std::vector<float> nrm9(any_normals ? (size_t)ntri * 9 : 0, 0.0f);
    std::vector<float> tc6(any_tc ? (size_t)ntri * 6 : 0, 0.0f), tg9(any_tg ? (size_t)ntri * 9 : 0, 0.0f);
    std::vector<int32_t> prim_inst((size_t)ntri);
    for (int i = 0; i < d->num_instances; ++i) {
        Xf xf;
        std::memcpy(xf.m, d->instances[i].transform, sizeof(xf.m));
        const srt_mesh& m = d->meshes[d->instances[i].mesh_id];
        for (int f = 0; f < m.num_faces; ++f) {
            int64_t g = s->inst_prim_base[i] + f;
            prim_inst[g] = i;
            for (int c = 0; c < 3; ++c) {
                uint32_t vi = m.indices[3 * f + c];
                float3 w = xf.point(ld3(m.vertices + 3 * vi));
                tri9[9 * g + 3 * c] = w.x;
                tri9[9 * g + 3 * c + 1] = w.y;
                tri9[9 * g + 3 * c + 2] = w.z;
                if (m.normals) {
                    float3 n = xf.vec(ld3(m.normals + 3 * vi));
                    nrm9[9 * g + 3 * c] = n.x;
                    nrm9[9 * g + 3 * c + 1] = n.y;
                    nrm9[9 * g + 3 * c + 2] = n.z;
                }
                if (m.texcoords) {
                    tc6[6 * g + 2 * c] = m.texcoords[2 * vi];
                    tc6[6 * g + 2 * c + 1] = m.texcoords[2 * vi + 1];
                }
                if (m.tangents) {
                    float3 t = xf.vec(ld3(m.tangents + 3 * vi));
                    tg9[9 * g + 3 * c] = t.x;
                    tg9[9 * g + 3 * c + 1] = t.y;
                    tg9[9 * g + 3 * c + 2] = t.z;
                }
            }
        }
    }

    // light table (Scene::build_gscene_instances, scene.cu:370-417)
    std::vector<InstanceRec> insts(d->num_instances);
    std::vector<LightRec> lights;
    std::vector<float> light_cdf, face_cdf;
    std::vector<int32_t> light_faces;  // global prim per light face
    std::vector<int> light_inst;       // instance of each light
    float wsum = 0.0f;
    for (int i = 0; i < d->num_instances; ++i) {
        const srt_mesh& m = d->meshes[d->instances[i].mesh_id];
        const srt_material& mat = d->materials[m.material_id];
        insts[i].material = m.material_id;
        insts[i].attr = (m.normals ? kAttrNormals : 0) | (m.texcoords ? kAttrTexcoords : 0) |
                        (m.tangents ? kAttrTangents : 0);
        insts[i].light_id = -1;
        insts[i].pad = 0;
        // an emitter without faces cannot be sampled and is never hit
        if (mat.intensity <= 0.0f || m.num_faces == 0) continue;
        insts[i].light_id = (int32_t)lights.size();
        LightRec L;
        L.face_begin = (int32_t)face_cdf.size();
        L.num_faces = m.num_faces;
        L.pdf = 0.0f;
        L.textured = (d->material_textures && d->material_textures[2 * m.material_id] >= 0) ? 1 : 0;
        lights.push_back(L);
        light_inst.push_back(i);
        const std::vector<float>& cdf = mesh_cdf[d->instances[i].mesh_id];
        for (int f = 0; f < m.num_faces; ++f) {
            face_cdf.push_back(cdf[f]);
            light_faces.push_back((int32_t)(s->inst_prim_base[i] + f));
        }
        wsum += mat.intensity * mesh_area[d->instances[i].mesh_id];
        light_cdf.push_back(wsum);
    }
    for (float& c : light_cdf) c /= wsum;
    for (size_t k = 0; k < lights.size(); ++k) {
        LightRec& L = lights[k];
        const srt_mesh& m = d->meshes[d->instances[light_inst[k]].mesh_id];
        L.pdf = d->materials[m.material_id].intensity / wsum;  // Light::sample_pdf (light.h:73-76)
    }

    // BVH
    WideBvh bvh;
    int threads = (int)std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
    build_wide_bvh(ntri, tri9.data(), threads, bvh);
    std::vector<float4> tris((size_t)ntri * 3);
    std::vector<float4> norms(any_normals ? (size_t)ntri * 3 : 0);
    std::vector<float2> tcs(any_tc ? (size_t)ntri * 3 : 0);
    std::vector<float4> tgs(any_tg ? (size_t)ntri * 3 : 0);
    std::vector<int32_t> tri_prim((size_t)ntri);
    std::vector<int32_t> inv((size_t)ntri);
    for (int64_t k = 0; k < ntri; ++k) {
        int32_t g = bvh.tri_order[k];
        tri_prim[k] = g;
        inv[g] = (int32_t)k;
        float inst_bits;
        int32_t inst = prim_inst[g];
        std::memcpy(&inst_bits, &inst, 4);
        const float* t = &tri9[9 * (size_t)g];
        tris[3 * k] = make_float4(t[0], t[1], t[2], inst_bits);
        tris[3 * k + 1] = make_float4(t[3], t[4], t[5], 0.0f);
        tris[3 * k + 2] = make_float4(t[6], t[7], t[8], 0.0f);
        if (any_normals) {
            const float* n = &nrm9[9 * (size_t)g];
            norms[3 * k] = make_float4(n[0], n[1], n[2], 0.0f);
            norms[3 * k + 1] = make_float4(n[3], n[4], n[5], 0.0f);
            norms[3 * k + 2] = make_float4(n[6], n[7], n[8], 0.0f);
        }
        if (any_tc)
            for (int c = 0; c < 3; ++c) tcs[3 * k + c] = make_float2(tc6[6 * (size_t)g + 2 * c], tc6[6 * (size_t)g + 2 * c + 1]);
        if (any_tg)
            for (int c = 0; c < 3; ++c)
                tgs[3 * k + c] = make_float4(tg9[9 * (size_t)g + 3 * c], tg9[9 * (size_t)g + 3 * c + 1],
                                             tg9[9 * (size_t)g + 3 * c + 2], 0.0f);
    }
    for (int32_t& g : light_faces) g = inv[g];
    std::vector<MaterialRec> mats(d->num_materials);
    auto mat_tex_of = [&](int mat, int k) { return d->material_textures ? d->material_textures[2 * mat + k] : -1; };
    bool any_mat_tex = false, any_normal_tex = false;
    for (int i = 0; i < d->num_materials; ++i) {
        const bool tx = mat_tex_of(i, 0) >= 0 || mat_tex_of(i, 1) >= 0;
        any_mat_tex |= tx;
        any_normal_tex |= mat_tex_of(i, 1) >= 0;
        mats[i] = pack_material(d->materials[i], tx);
    }

    srt_status st = SRT_OK;
    auto up = [&](DeviceBuffer& b, const void* p, size_t bytes, const char* what) {
        if (st == SRT_OK) st = b.upload(p, bytes, what);
    };
    up(s->nodes, bvh.nodes.data(), bvh.nodes.size() * sizeof(WideNode), "bvh nodes");
    up(s->tris, tris.data(), tris.size() * sizeof(float4), "triangles");
    up(s->tri_prim, tri_prim.data(), tri_prim.size() * 4, "triangle ids");
    if (any_normals) up(s->normals, norms.data(), norms.size() * sizeof(float4), "normals");
    up(s->insts, insts.data(), insts.size() * sizeof(InstanceRec), "instances");
    up(s->mats, mats.data(), mats.size() * sizeof(MaterialRec), "materials");
    up(s->lights, lights.data(), lights.size() * sizeof(LightRec), "lights");
    up(s->light_cdf, light_cdf.data(), light_cdf.size() * 4, "light cdf");
    up(s->face_cdf, face_cdf.data(), face_cdf.size() * 4, "face cdf");
    up(s->light_tri, light_faces.data(), light_faces.size() * 4, "light faces");
    if (any_tc) up(s->texcoords, tcs.data(), tcs.size() * sizeof(float2), "texture coordinates");
    if (any_tg) up(s->tangents, tgs.data(), tgs.size() * sizeof(float4), "tangents");
    // textures, and per material the (colour, normal) texture objects
    int64_t tex_bytes = 0;
    for (int i = 0; i < d->num_textures && st == SRT_OK; ++i) {
        cudaArray_t arr = nullptr;
        cudaTextureObject_t obj = 0;
        st = make_texture(d->textures[i], arr, obj);
        if (arr) s->tex_arrays.push_back(arr);
        if (obj) s->tex_objects.push_back(obj);
        tex_bytes += (int64_t)d->textures[i].width * d->textures[i].height *
                     (d->textures[i].format == SRT_TEXTURE_RGBA8 ? 4 : 16);
    }
    if (st == SRT_OK && any_mat_tex) {
        std::vector<unsigned long long> mt(2 * (size_t)d->num_materials, 0ull);
        for (int i = 0; i < 2 * d->num_materials; ++i)
            if (d->material_textures[i] >= 0) mt[i] = s->tex_objects[d->material_textures[i]];
        up(s->mat_tex, mt.data(), mt.size() * 8, "material textures");
    }
    if (st == SRT_OK && any_normal_tex) {
        // instance rows, to turn normal-map normals (object space) into world space
        std::vector<float4> xr(3 * (size_t)d->num_instances);
        for (int i = 0; i < d->num_instances; ++i) {
            const float* t = d->instances[i].transform;
            for (int r = 0; r < 3; ++r) xr[3 * i + r] = make_float4(t[4 * r], t[4 * r + 1], t[4 * r + 2], t[4 * r + 3]);
        }
        up(s->inst_xf, xr.data(), xr.size() * sizeof(float4), "instance transforms");
    }
    if (st != SRT_OK) {
        delete s;
        return st;
    }
    SceneView& v = s->view;
    v.nodes = s->nodes.as<WideNode>();
    v.tris = s->tris.as<float4>();
    v.tri_prim = s->tri_prim.as<int32_t>();
    v.normals = any_normals ? s->normals.as<float4>() : nullptr;
    v.insts = s->insts.as<InstanceRec>();
    v.mats = s->mats.as<MaterialRec>();
    v.lights = s->lights.as<LightRec>();
    v.light_cdf = s->light_cdf.as<float>();
    v.face_cdf = s->face_cdf.as<float>();
    v.light_tri = s->light_tri.as<int32_t>();
    v.num_lights = (int32_t)lights.size();
    v.num_tris = (int32_t)ntri;
    v.env = make_float3(d->env_color[0], d->env_color[1], d->env_color[2]);
    v.weight_sum = wsum;
    v.texcoords = any_tc ? s->texcoords.as<float2>() : nullptr;
    v.tangents = any_tg ? s->tangents.as<float4>() : nullptr;
    v.mat_tex = any_mat_tex ? s->mat_tex.as<unsigned long long>() : nullptr;
    v.inst_xf = any_normal_tex ? s->inst_xf.as<float4>() : nullptr;
    v.env_tex = d->env_map > 0 ? s->tex_objects[d->env_map - 1] : 0ull;
    s->camera_desc = d->camera;
    s->camera = make_camera(d->camera);

    auto t1 = std::chrono::steady_clock::now();
    srt_scene_info& I = s->info;
    I.num_triangles = ntri;
    I.num_nodes = (int64_t)bvh.nodes.size();
    I.num_lights = (int64_t)lights.size();
    I.device_bytes = (int64_t)(s->nodes.bytes() + s->tris.bytes() + s->tri_prim.bytes() + s->normals.bytes() +
                               s->insts.bytes() + s->mats.bytes() + s->lights.bytes() + s->light_cdf.bytes() +
                               s->face_cdf.bytes() + s->light_tri.bytes() + s->texcoords.bytes() +
                               s->tangents.bytes() + s->mat_tex.bytes() + s->inst_xf.bytes() + tex_bytes);
    I.bvh_depth = bvh.depth;
    I.build_ms = (float)std::chrono::duration<double, std::milli>(t1 - t0).count();
    I.light_weight_sum = wsum;
    *out = s;
    return SRT_OK;
}

extern "C" srt_status srt_scene_set_camera(srt_scene* s, const srt_camera_desc* c)
{
    clear_error();
    if (!s || !c) return set_error(SRT_ERR_ARG, "NULL argument");
    const int cam_type = c->type & ~SRT_CAMERA_MIRROR_X;
    if (cam_type != SRT_CAMERA_PERSPECTIVE && cam_type != SRT_CAMERA_ORTHOGRAPHIC)
        return set_error(SRT_ERR_UNSUPPORTED, "only perspective and orthographic cameras are supported");
    s->camera_desc = *c;
    s->camera = make_camera(*c);
    return SRT_OK;
}

extern "C" srt_status srt_scene_get_info(const srt_scene* s, srt_scene_info* info)
{
    clear_error();
    if (!s || !info) return set_error(SRT_ERR_ARG, "NULL argument");
    *info = s->info;
    return SRT_OK;
}

extern "C" srt_status srt_scene_prim_to_instance(const srt_scene* s, int64_t prim, int32_t* instance, int32_t* face)
{
    clear_error();
    if (!s || !instance || !face) return set_error(SRT_ERR_ARG, "NULL argument");
    if (prim < 0 || prim >= s->info.num_triangles) return set_error(SRT_ERR_ARG, "primitive id out of range");
    auto it = std::upper_bound(s->inst_prim_base.begin(), s->inst_prim_base.end(), prim);
    int i = (int)(it - s->inst_prim_base.begin()) - 1;
    while (i > 0 && s->inst_faces[i] == 0) --i;
    *instance = i;
    *face = (int32_t)(prim - s->inst_prim_base[i]);
    return SRT_OK;
}

srt_scene::~srt_scene()
{
    for (cudaTextureObject_t o : tex_objects) cudaDestroyTextureObject(o);
    for (cudaArray_t a : tex_arrays) cudaFreeArray(a);
}

extern "C" void srt_scene_destroy(srt_scene* s) { delete s; }
