// host_scene.h — a scene held in host memory (generated or imported from a
// file) that fills an srt_scene_desc for srt_scene_create.
#pragma once

#include <cstring>
#include <string>
#include <vector>

#include "common.h"

namespace srt {

// One triangle mesh in object space: float3 vertices, optional per-vertex
// normals, uint3 faces (TriangleMesh, src/scene/mesh.h:63-93).
struct HostMesh {
    std::vector<float> v;
    std::vector<float> n;   // empty, or one normal per vertex
    std::vector<float> tc;  // empty, or one (u, v) per vertex
    std::vector<float> tg;  // empty, or one tangent per vertex
    std::vector<uint32_t> idx;
    int material = 0;
    void quad(const float* a, const float* b, const float* c, const float* d)
    {
        uint32_t base = (uint32_t)(v.size() / 3);
        for (const float* p : {a, b, c, d}) v.insert(v.end(), p, p + 3);
        uint32_t t[6] = {base, base + 1, base + 2, base, base + 2, base + 3};
        idx.insert(idx.end(), t, t + 6);
    }
};

struct HostInstance {
    int mesh;
    float xf[12];  // row-major 3x4 object-to-world
};

// A texture image in host memory (Texture / Image, src/scene/texture.h).
struct HostTexture {
    std::string name;
    int width = 0, height = 0;
    int format = SRT_TEXTURE_RGBA8;
    std::vector<uint8_t> u8;   // RGBA8 texels
    std::vector<float> f32;    // RGBA32F texels
};

// Image::load_from_file(path, flip_x = false, flip_y) into a texture:
// float images (exr, hdr, pfm) stay float, 8-bit images (png, bmp) RGBA8.
inline srt_status load_texture_image(const std::string& path, bool flip_y, HostTexture& t)
{
    const int flip = flip_y ? SRT_FLIP_Y : SRT_FLIP_NONE;
    int32_t w = 0, h = 0;
    srt_status st = srt_image_read(path.c_str(), &w, &h, nullptr, flip);
    if (st == SRT_OK) {
        t.format = SRT_TEXTURE_RGBA32F;
        t.f32.resize((size_t)w * h * 4);
        st = srt_image_read(path.c_str(), &w, &h, t.f32.data(), flip);
    } else if (st == SRT_ERR_UNSUPPORTED) {
        st = srt_image_read_rgba8(path.c_str(), &w, &h, nullptr, flip);
        if (st != SRT_OK) return st;
        t.format = SRT_TEXTURE_RGBA8;
        t.u8.resize((size_t)w * h * 4);
        st = srt_image_read_rgba8(path.c_str(), &w, &h, t.u8.data(), flip);
    }
    t.width = w;
    t.height = h;
    return st;
}

}  // namespace srt

struct srt_procedural {
    std::vector<srt::HostMesh> meshes;
    std::vector<srt::HostInstance> instances;  // empty: one identity instance per mesh
    std::vector<srt_material> mats;
    std::vector<srt::HostTexture> textures;
    std::vector<int32_t> mat_tex;  // 2 per material (colour, normal), -1 none; empty: no textured material
    int32_t env_map = 0;           // texture index + 1 of a "uvmap" environment, 0 none
    int width = 0, height = 0;  // film size given by an imported file, 0 when none
    bool has_camera = false;    // generated scenes and pbrt files carry a camera; obj / ply do not
    std::vector<srt_mesh> mesh_desc;
    std::vector<srt_instance> inst;
    std::vector<srt_texture> tex_desc;
    srt_scene_desc desc{};

    // texture / material-texture pointers of desc (after textures change)
    void sync_textures()
    {
        tex_desc.clear();
        for (const srt::HostTexture& t : textures) {
            srt_texture d{};
            d.width = t.width;
            d.height = t.height;
            d.format = t.format;
            d.pixels = t.format == SRT_TEXTURE_RGBA8 ? (const void*)t.u8.data() : (const void*)t.f32.data();
            tex_desc.push_back(d);
        }
        desc.textures = tex_desc.empty() ? nullptr : tex_desc.data();
        desc.num_textures = (int32_t)tex_desc.size();
        desc.env_map = env_map;
        if (!mat_tex.empty()) mat_tex.resize(2 * mats.size(), -1);
        desc.material_textures = mat_tex.empty() ? nullptr : mat_tex.data();
    }

    void finish(const srt_camera_desc& cam, const float env[3])
    {
        mesh_desc.clear();
        inst.clear();
        for (size_t i = 0; i < meshes.size(); ++i) {
            srt_mesh d{};
            d.vertices = meshes[i].v.data();
            d.indices = meshes[i].idx.data();
            d.normals = meshes[i].n.empty() ? nullptr : meshes[i].n.data();
            d.texcoords = meshes[i].tc.empty() ? nullptr : meshes[i].tc.data();
            d.tangents = meshes[i].tg.empty() ? nullptr : meshes[i].tg.data();
            d.num_vertices = (int32_t)(meshes[i].v.size() / 3);
            d.num_faces = (int32_t)(meshes[i].idx.size() / 3);
            d.material_id = meshes[i].material;
            mesh_desc.push_back(d);
        }
        if (instances.empty()) {
            for (size_t i = 0; i < meshes.size(); ++i) {
                srt_instance in{};
                in.mesh_id = (int32_t)i;
                const float id[12] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0};
                std::memcpy(in.transform, id, sizeof(id));
                inst.push_back(in);
            }
        } else {
            for (const srt::HostInstance& h : instances) {
                srt_instance in{};
                in.mesh_id = h.mesh;
                std::memcpy(in.transform, h.xf, sizeof(h.xf));
                inst.push_back(in);
            }
        }
        desc.meshes = mesh_desc.data();
        desc.num_meshes = (int32_t)mesh_desc.size();
        desc.instances = inst.data();
        desc.num_instances = (int32_t)inst.size();
        desc.materials = mats.data();
        desc.num_materials = (int32_t)mats.size();
        desc.camera = cam;
        for (int k = 0; k < 3; ++k) desc.env_color[k] = env[k];
        sync_textures();
    }
};
