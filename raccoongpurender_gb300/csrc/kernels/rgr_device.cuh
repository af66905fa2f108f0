// rgr_device.cuh — device-side vector helpers, RNG and the device scene view.
//
// Every translation unit that includes this header is compiled with
// --fmad=false, -prec-div=true, -prec-sqrt=true and without -ftz, so each
// expression below rounds exactly as written: OpenCL dot() is
// (a.x*b.x + a.y*b.y) + a.z*b.z, normalize(v) = v / sqrt(dot(v, v)), and
// transcendental calls go to the deterministic rgr_fmath.h.
#pragma once
#include <stdint.h>
#include <cuda_runtime.h>
#include "../rgr_fmath.h"

#define RGR_DEV __device__ __forceinline__

namespace rgr {
namespace dev {

struct f3 {
    float x, y, z;
};
RGR_DEV f3 mk(float x, float y, float z) { return f3{x, y, z}; }
RGR_DEV f3 operator+(f3 a, f3 b) { return mk(a.x + b.x, a.y + b.y, a.z + b.z); }
RGR_DEV f3 operator-(f3 a, f3 b) { return mk(a.x - b.x, a.y - b.y, a.z - b.z); }
RGR_DEV f3 operator*(f3 a, f3 b) { return mk(a.x * b.x, a.y * b.y, a.z * b.z); }
RGR_DEV f3 operator*(f3 a, float s) { return mk(a.x * s, a.y * s, a.z * s); }
RGR_DEV f3 operator*(float s, f3 a) { return mk(s * a.x, s * a.y, s * a.z); }
RGR_DEV f3 operator/(f3 a, float s) { return mk(a.x / s, a.y / s, a.z / s); }
RGR_DEV f3 operator-(f3 a) { return mk(-a.x, -a.y, -a.z); }
RGR_DEV float dot(f3 a, f3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
RGR_DEV f3 cross(f3 a, f3 b) { return mk(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x); }
RGR_DEV f3 normalize(f3 v) {
    float l = sqrtf(dot(v, v));
    return mk(v.x / l, v.y / l, v.z / l);
}
RGR_DEV f3 xyz(float4 v) { return mk(v.x, v.y, v.z); }
RGR_DEV bool is_finite_nonzero(float x) {
    const uint32_t e = __float_as_uint(x) & 0x7fffffffu;
    return e != 0u && e < 0x7f800000u;
}
RGR_DEV float4 f4(f3 v, float w) { return make_float4(v.x, v.y, v.z, w); }

// ------------------------------------------------------------ RNG
// xoshiro128** and the float/integer draws of kernels/peseudo_random.cl:5-40
struct Rng {
    uint32_t s0, s1, s2, s3;
    RGR_DEV uint32_t next() {
        const uint32_t result = __funnelshift_l(s0 * 5u, s0 * 5u, 7) * 9u;
        const uint32_t t = s1 << 9;
        s2 ^= s0;
        s3 ^= s1;
        s1 ^= s2;
        s0 ^= s3;
        s2 ^= t;
        s3 = __funnelshift_l(s3, s3, 11);
        return result;
    }
    RGR_DEV float uniform() { return __uint_as_float((next() >> 9) | 0x3f800000u) - 1.0f; }
    RGR_DEV uint64_t uniform_integer() {
        uint64_t a = next() >> 1;
        uint64_t b = next() >> 1;
        return (a << 31) | b;
    }
};
// p: a uint4 array or a slot field of uint4
template <class P>
RGR_DEV Rng rng_load(const P& p, uint32_t i) {
    uint4 v = p[i];
    return Rng{v.x, v.y, v.z, v.w};
}
template <class P>
RGR_DEV void rng_store(const P& p, uint32_t i, const Rng& r) { p[i] = make_uint4(r.s0, r.s1, r.s2, r.s3); }

// ------------------------------------------------------------ scene view
struct SceneView {
    const float4* nodes;      // 4 float4 per inner node (NodeD)
    const float4* prims;      // 3 float4 per primitive record (PrimD)
    uint32_t root_link;
    uint32_t num_prims;       // 0 = empty scene
    const float4* points;     // original vertices (Ng of the hit)
    const uint32_t* indices;  // 3 per triangle
    const float4* tri_normals;  // per triangle: the normal as hit_normal computes it from the points,
                                // and in w its material type (or null)
    const float4* spheres;    // center, radius
    int32_t sphere_begin;
    // materials
    const int2* materials;    // (type, index) per primitive
    const float4* lambertians;  // 2 per material: Le, R
    const float4* wards;        // 3 per material: (alpha, falloff, 0, 0), reflectance, edgetint
    const float4* volumes;      // 1 per material: (R.xyz, C)
    // envmap
    const float4* env_rgba;     // w*h texels
    const float* env_pdf;       // 7*w*h
    const int2* env_alias;      // 7*w*h (height bits, alias)
    const float4* env_frag;     // w*h
    int32_t env_w, env_h;
    int32_t has_env;
    int32_t small_coords;       // every scene coordinate within +-1e30 (no NaN in slab products)
    uint32_t num_nodes;         // inner nodes
};

constexpr uint32_t kLeafFlag = 0x80000000u;

}  // namespace dev
}  // namespace rgr
