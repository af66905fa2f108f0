// rgr_internal.h — host-side structures of librgr (scene, BVH, envmap tables)
// and the device data layout shared by the CUDA kernels.
#pragma once
#include <stdint.h>
#include <string>
#include <vector>
#include <memory>
#include "../../include/rgr.h"

namespace rgr {

void set_error(const std::string& msg);

// ---------------------------------------------------------------- materials
// Per-primitive material record, as MaterialStorage builds it
// (scene_manager.hpp:106-172): a type and an index into the array of that type.
struct MaterialRef {
    int32_t type, index;
};
struct LambertianD {  // kernels/types.cl:78-82
    float le[4];
    float r[4];
};
struct WardD {  // kernels/types.cl:92-97
    float alpha, falloff, pad0, pad1;
    float reflectance[4];
    float edgetint[4];
};
struct VolumeD {  // kernels/types.cl:99-102: R.xyz, C
    float r[3];
    float c;
};

// ---------------------------------------------------------------- BVH
// Device layout of one inner node: 64 bytes, fetched as two 32-byte loads.
//   q0 = (L.lo.x, L.lo.y, L.lo.z, L.hi.x)
//   q1 = (L.hi.y, L.hi.z, R.lo.x, R.lo.y)
//   q2 = (R.lo.z, R.hi.x, R.hi.y, R.hi.z)
//   q3 = (link L, link R, 0, 0) as uint bits
// A link is an inner-node index, or, with bit 31 set, a leaf:
//   bits 0..27 first primitive record, bits 28..30 count-1.
struct alignas(16) NodeD {
    float q[12];
    uint32_t link[2];
    uint32_t pad[2];
};
static_assert(sizeof(NodeD) == 64, "NodeD must be 64 bytes");
constexpr uint32_t kLeafFlag = 0x80000000u;
// inner nodes placed first, in breadth-first order, for shared-memory staging
constexpr size_t kStagedNodes = 1024;
constexpr uint32_t kLeafFirstMask = 0x0fffffffu;
inline uint32_t make_leaf_link(uint32_t first, uint32_t count) {
    return kLeafFlag | ((count - 1u) << 28) | first;
}
// Primitive record, 48 bytes, in leaf order (= the reference primitive_ids order).
//   triangle: (v0.xyz, id) (v1-v0, 0) (v2-v0, 0)
//   sphere:   (center.xyz, id) (radius, 0, 0, flag 1) (0)
struct alignas(16) PrimD {
    float a[4];
    float b[4];
    float c[4];
};
static_assert(sizeof(PrimD) == 48, "PrimD must be 48 bytes");

struct Bvh {
    bool built = false;
    std::vector<rgr_stackless_node> ref_nodes;  // reference layout
    std::vector<uint32_t> ref_prim_ids;
    std::vector<NodeD> nodes;                   // device layout (inner nodes only)
    std::vector<PrimD> prims;
    uint32_t root_link = 0;                     // 0 = inner node 0; leaf link if the root is a leaf
    uint64_t num_leaves = 0;
    int32_t depth = 0;
    double sah_cost = 0.0;
    float bounds[6] = {0, 0, 0, 0, 0, 0};
};

// A linear BVH built on the GPU (bvh_gpu.cu): internal node i has children
// left[i], right[i] (>= 0 internal node, < 0 leaf ~k = sorted primitive k),
// covers sorted primitives [first[i], first[i] + count[i]) and has the box
// box[6i .. 6i+5] (lo xyz, hi xyz); order[k] = primitive id; the root is 0.
struct LbvhTree {
    std::vector<uint32_t> order;
    std::vector<int32_t> left, right, first, count;
    std::vector<float> box;
};
// boxes: 6 floats per primitive (lo xyz, hi xyz); n >= 2
int lbvh_build_gpu(int device, const float* boxes, uint32_t n, const float centroid_lo[3],
                   const float centroid_hi[3], LbvhTree& out);

// ---------------------------------------------------------------- envmap
struct EnvTables {
    bool present = false;
    int32_t w = 0, h = 0;
    std::vector<float> rgba;      // w*h*4 after clamp/scale
    std::vector<float> pdf;       // 7*w*h
    std::vector<float> height;    // 7*w*h
    std::vector<int32_t> alias;   // 7*w*h
    std::vector<float> frag;      // 4*w*h
};
int build_envmap_tables(EnvTables& env);
// the same tables, selection weights and FP64 normalisation on `device`
int build_envmap_tables_gpu(EnvTables& env, int device);
void alias_from_probabilities(int w, int h, const double* prob, const std::vector<double>& sr, float* pdf,
                              float* height, int32_t* alias);
// 7 x w x h normalised selection probabilities (FP64) of the envmap tables, on the GPU
int envmap_probabilities_gpu(int device, const float* rgba, int w, int h, double* prob_out);

}  // namespace rgr

struct rgr_scene {
    std::vector<float> points;          // xyz per vertex
    std::vector<uint32_t> indices;      // 3 per triangle
    std::vector<float> spheres;         // xyzr
    std::vector<rgr::MaterialRef> tri_materials;
    std::vector<rgr::MaterialRef> sphere_materials;
    std::vector<rgr::LambertianD> lambertians;
    std::vector<rgr::WardD> wards;
    std::vector<rgr::VolumeD> volumes;
    int32_t num_speculars = 0, num_dielectrics = 0;
    rgr::EnvTables env;
    rgr::Bvh bvh;
};

namespace rgr {
int build_bvh(rgr_scene* s, const rgr_bvh_params& p);
}
