// device_types.h — layouts shared by the host builders and the kernels.
//
// HBM layout of one scene (all arrays 128-byte aligned, read-only after
// upload):
//   nodes     WideNode[num_nodes]     128 B each: one L2 line per node
//   tris      float4[3 * num_tris]    v0, v1, v2 in world space, BVH leaf
//                                     order; v0.w = instance id (int bits)
//   tri_prim  int32[num_tris]         BVH order -> global primitive id
//   normals   float4[3 * num_tris]    per-corner shading normals (only when
//                                     some mesh has vertex normals)
//   texcoords float2[3 * num_tris]    per-corner texture coordinates (only
//                                     when some mesh has them)
//   tangents  float4[3 * num_tris]    per-corner world tangents (likewise)
//   mat_tex   u64[2 * num_mats]       colour / normal texture objects (only
//                                     when some material is textured)
//   inst_xf   float4[3 * num_insts]   instance rows (only with normal maps)
//   insts     InstanceRec[num_insts]  material / light id per instance
//   mats      MaterialRec[num_mats]   80 B, read with five 16-byte loads
//   lights    LightRec[num_lights]    area-light table
//   light_cdf float[num_lights]       Σ intensity·area CDF (scene.cu:378-393)
//   face_cdf  float[Σ light faces]    per-light object-space area CDFs
//   light_tri int32[Σ light faces]    BVH-order triangle of each light face
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace srt {

// 8-wide BVH node with 16-bit quantised child boxes, exactly 128 bytes.
//   child box lo = origin + q_lo * 2^exp (per axis), hi likewise; the
//   quantisation is conservative (floor for lo, ceil for hi).
//   meta[i]: the bits slot i sets in the node's hit mask when its box is
//   hit, as (meta >> 5) << (meta & 31): 0 = empty slot; a leaf of n (1..3)
//   triangles starting at tri_base + off (off + n <= 24) is
//   ((1 << n) - 1) << 5 | off (triangle bits 0..23); an internal child is
//   kMetaInternal | i (bits 3 and 4 set, which no leaf offset has), and the
//   traversal moves its bit to 24 + (i ^ octant).  Its node is child_base +
//   the number of internal slots below i.
// Children sit in slots ordered for octant traversal: a ray whose
// direction-sign octant is `oct` visits slots in order k ^ oct, k = 0..7,
// which approximates front-to-back (Ylitie, Karras, Laine, HPG 2017).
constexpr uint8_t kMetaInternal = 0x38;
struct alignas(128) WideNode {
    float origin[3];
    int8_t exp[3];
    uint8_t imask;        // bit i set: slot i is an internal child
    uint32_t child_base;  // first internal child node
    uint32_t tri_base;    // first triangle of the leaf children
    uint8_t meta[8];
    uint16_t qlo[3][8];   // [axis][slot]
    uint16_t qhi[3][8];
};
static_assert(sizeof(WideNode) == 128, "WideNode must be one 128-byte line");

// InstanceRec::attr bits: which per-corner arrays the instance's mesh has
constexpr int32_t kAttrNormals = 1, kAttrTexcoords = 2, kAttrTangents = 4;

struct InstanceRec {
    int32_t material;
    int32_t light_id;     // -1 if not an area light
    int32_t attr;         // kAttr* bits
    int32_t pad;
};

// Material packed for 16-byte vector loads (GMaterial, gmaterial.h:6-15):
//   m[0] = base_color.rgb, bxdf type (int bits)
//   m[1] = ior, metallic, subsurface, roughness
//   m[2] = specular, specularTint, anisotropic, sheen
//   m[3] = sheenTint, clearcoat, clearcoatGloss, specTrans
//   m[4] = emission_color * intensity (rgb), intensity
struct alignas(16) MaterialRec {
    float4 m[5];
};

struct LightRec {
    int32_t face_begin;   // into face_cdf / light_tri
    int32_t num_faces;
    float pdf;            // intensity / weight_sum (light.h:73-76)
    int32_t textured;     // the light's material has a colour texture (its emission)
};

// Camera after Camera::reset / CameraController(LookAt) on the host
// (camera.h:14-53, 165-170).
struct CameraRec {
    float3 pos, x, y, z;
    float nw, nh, radius, aperture, focal;
    int32_t type;
};

// Device view of a resident scene.
struct SceneView {
    const WideNode* nodes;
    const float4* tris;
    const int32_t* tri_prim;
    const float4* normals;      // may be null
    const InstanceRec* insts;
    const MaterialRec* mats;
    const LightRec* lights;
    const float* light_cdf;
    const float* face_cdf;
    const int32_t* light_tri;
    int32_t num_lights;
    int32_t num_tris;
    float3 env;
    float weight_sum;
    const float2* texcoords;               // may be null
    const float4* tangents;                // may be null
    const unsigned long long* mat_tex;     // may be null: (color, normal) per material, 0 = none
    const float4* inst_xf;                 // may be null
    unsigned long long env_tex;            // 0: constant env
};

}  // namespace srt
