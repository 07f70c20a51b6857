// scene.h — resident scene: flattened world-space triangles, 8-wide BVH,
// materials and light tables in HBM (replaces GScene + the OptiX GAS/IAS,
// src/scene/scene.h:29-63, src/optix/optix_ray_tracer.cu:213-359).
#pragma once

#include <vector>

#include "common.h"
#include "device_types.h"

struct srt_scene {
    srt::DeviceBuffer nodes, tris, tri_prim, normals, insts, mats, lights, light_cdf, face_cdf, light_tri;
    srt::DeviceBuffer texcoords, tangents, mat_tex, inst_xf;
    std::vector<cudaArray_t> tex_arrays;              // Scene::build_gscene_textures (scene.cu:92-139)
    std::vector<cudaTextureObject_t> tex_objects;
    ~srt_scene();
    srt::SceneView view{};
    srt::CameraRec camera{};
    srt_camera_desc camera_desc{};
    srt_scene_info info{};
    std::vector<int64_t> inst_prim_base;  // global prim id of each instance's face 0
    std::vector<int32_t> inst_faces;
    int device = 0;
};

namespace srt {

// Camera::reset + CameraController(LookAt(position, target, up), radius)
// on the host (camera.h:41-53, 165-170; transform.h:136-145).
CameraRec make_camera(const srt_camera_desc& c);

}  // namespace srt
