// host_scene.h — a scene held in host memory (generated or imported from a
// file) that fills an srt_scene_desc for srt_scene_create.
#pragma once

#include <cstring>
#include <vector>

#include "common.h"

namespace srt {

// One triangle mesh in object space: float3 vertices, optional per-vertex
// normals, uint3 faces (TriangleMesh, src/scene/mesh.h:63-93).
struct HostMesh {
    std::vector<float> v;
    std::vector<float> n;  // empty, or one normal per vertex
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

}  // namespace srt

struct srt_procedural {
    std::vector<srt::HostMesh> meshes;
    std::vector<srt::HostInstance> instances;  // empty: one identity instance per mesh
    std::vector<srt_material> mats;
    int width = 0, height = 0;  // film size given by an imported file, 0 when none
    bool has_camera = false;    // generated scenes and pbrt files carry a camera; obj / ply do not
    std::vector<srt_mesh> mesh_desc;
    std::vector<srt_instance> inst;
    srt_scene_desc desc{};

    void finish(const srt_camera_desc& cam, const float env[3])
    {
        mesh_desc.clear();
        inst.clear();
        for (size_t i = 0; i < meshes.size(); ++i) {
            srt_mesh d{};
            d.vertices = meshes[i].v.data();
            d.indices = meshes[i].idx.data();
            d.normals = meshes[i].n.empty() ? nullptr : meshes[i].n.data();
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
    }
};
