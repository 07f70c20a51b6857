// bvh_build.h — host builder of the 8-wide quantised BVH (replaces the
// optixAccelBuild GAS/IAS build of src/optix/optix_ray_tracer.cu:213-359).
#pragma once

#include <stdint.h>
#include <vector>

#include "device_types.h"

namespace srt {

struct WideBvh {
    std::vector<WideNode> nodes;
    std::vector<int32_t> tri_order;  // BVH leaf order -> input triangle index
    int depth = 0;                   // number of node levels
    int binary_depth = 0;
};

// Triangles given as 9 floats each (v0, v1, v2).  Binned SAH (32 bins,
// leaves of at most 3 triangles), collapsed to 8-wide nodes by the
// SAH-optimal dynamic programme of Ylitie, Karras and Laine (HPG 2017),
// slots assigned by the octant ordering, boxes quantised to 16 bits per
// axis.  `threads` host threads build independent subtrees.
void build_wide_bvh(int64_t num_tris, const float* tri9, int threads, WideBvh& out);

}  // namespace srt
