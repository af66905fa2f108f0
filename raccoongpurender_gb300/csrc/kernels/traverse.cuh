// traverse.cuh — closest-hit BVH traversal on CUDA cores (GB300 has no RT cores).
//
// Visits exactly the nodes and leaves that the reference stackless traversal
// intersect_bvh (kernels/extension_ray_cast_stackless.cl:81-200) visits, in
// the same order, with the same slab arithmetic (:35-50) and the same
// triangle / sphere tests (intersect_triangle.cl:7-44, :52-76), so the
// closest primitive id and t are bit-identical:
//   * at an inner node both child boxes are slab-tested against the current
//     tmin; with both hit the nearer (by entry distance, ties by exit
//     distance, exact == test as in the reference) is entered first;
//   * the reference's 64-bit bit stack + parent/sibling links return to the
//     far child of the deepest pending "both hit" node, without re-testing
//     its box; a short stack of those far links does the same thing.
// Layout: 64-byte inner nodes holding both child boxes (one 64-byte line,
// four 16-byte read-only loads), leaves encoded in the parent's link, and
// primitives pre-gathered in leaf order as 48-byte records (v0, v1-v0, v2-v0:
// the edge subtraction is done once on the host and is bit-identical).
#pragma once
#include "rgr_device.cuh"

namespace rgr {
namespace dev {

constexpr int kStackSize = 64;  // the builder limits tree depth to 63
constexpr uint32_t kDone = 0xffffffffu;

struct Hit {
    float t;
    int32_t prim;
};

// slabs_with_hit (extension_ray_cast_stackless.cl:35-50).  fminf/fmaxf have
// the reference's NaN behaviour; their results only feed comparisons, so the
// sign of a zero result cannot change a decision.
RGR_DEV bool slab(float lox, float loy, float loz, float hix, float hiy, float hiz, f3 ro, f3 inv, float farclip,
                  float& h0, float& h1) {
    float t0x = (lox - ro.x) * inv.x, t0y = (loy - ro.y) * inv.y, t0z = (loz - ro.z) * inv.z;
    float t1x = (hix - ro.x) * inv.x, t1y = (hiy - ro.y) * inv.y, t1z = (hiz - ro.z) * inv.z;
    t0x = isnan(t0x) ? -t1x : t0x;
    t0y = isnan(t0y) ? -t1y : t0y;
    t0z = isnan(t0z) ? -t1z : t0z;
    t1x = isnan(t1x) ? -t0x : t1x;
    t1y = isnan(t1y) ? -t0y : t1y;
    t1z = isnan(t1z) ? -t0z : t1z;
    float rmin = fmaxf(fmaxf(fminf(t0x, t1x), fminf(t0y, t1y)), fminf(t0z, t1z));
    float rmax = fminf(fminf(fmaxf(t0x, t1x), fmaxf(t0y, t1y)), fmaxf(t0z, t1z));
    h0 = fmaxf(0.0f, rmin);
    h1 = fminf(rmax, farclip);
    return rmin <= rmax && 0.0f <= rmax && rmin <= farclip;
}

// intersect_ray_triangle (intersect_triangle.cl:7-44) with precomputed edges
RGR_DEV bool tri_test(f3 ro, f3 rd, f3 v0, f3 e1, f3 e2, float& tmin) {
    f3 pvec = cross(rd, e2);
    float det = dot(e1, pvec);
    if (fabsf(det) < 1.0e-8f) return false;
    float invDet = 1.0f / det;
    f3 tvec = ro - v0;
    float u = dot(tvec, pvec) * invDet;
    if (u < 0.0f || u > 1.0f) return false;
    f3 qvec = cross(tvec, e1);
    float v = dot(rd, qvec) * invDet;
    if (v < 0.0f || u + v > 1.0f) return false;
    float t = dot(e2, qvec) * invDet;
    if (t < 0.0f) return false;
    if (tmin < t) return false;
    tmin = t;
    return true;
}

// intersect_sphere (extension_ray_cast_stackless.cl:52-76)
RGR_DEV bool sphere_test(f3 ro, f3 rd, f3 o, float r, float& tmin) {
    float r_sq = r * r;
    f3 S = ro - o;
    f3 crs = cross(S, rd);
    float d_sq = dot(crs, crs);
    float B = dot(S, rd);
    float D = r_sq - d_sq;
    if (D < 0.0f) return false;
    float D_sqrt = sqrtf(D);
    float t0 = -B - D_sqrt;
    float t1 = -B + D_sqrt;
    if (0.0f < t0 && t0 < tmin) {
        tmin = t0;
        return true;
    }
    if (0.0f < t1 && t1 < tmin) {
        tmin = t1;
        return true;
    }
    return false;
}

struct TraceCounters {
    uint32_t nodes = 0, prims = 0;
};
constexpr uint32_t kErrStackOverflow = 1u;

// Closest hit.  tmin in: the ray's far clip (ExtensionResult.tmin); out: the
// hit distance (unchanged on a miss).  Returns the primitive id or -1.
template <bool kCount>
RGR_DEV int32_t trace_closest(const SceneView& sc, f3 ro, f3 rd, float& tmin, TraceCounters* cnt, uint32_t& err) {
    if (sc.num_prims == 0) return -1;
    const f3 inv = mk(1.0f / rd.x, 1.0f / rd.y, 1.0f / rd.z);
    uint32_t stack[kStackSize];
    int sp = 0;
    int32_t prim = -1;
    uint32_t link = sc.root_link;
    const float4* __restrict__ nodes = sc.nodes;
    const float4* __restrict__ prims = sc.prims;
    for (;;) {
        // inner nodes
        while (!(link & kLeafFlag)) {
            const float4* np = nodes + 4 * (size_t)link;
            const float4 q0 = __ldg(np + 0);
            const float4 q1 = __ldg(np + 1);
            const float4 q2 = __ldg(np + 2);
            const float4 q3 = __ldg(np + 3);
            if (kCount) cnt->nodes++;
            float L0, L1, R0, R1;
            bool L = slab(q0.x, q0.y, q0.z, q0.w, q1.x, q1.y, ro, inv, tmin, L0, L1);
            bool R = slab(q1.z, q1.w, q2.x, q2.y, q2.z, q2.w, ro, inv, tmin, R0, R1);
            const uint32_t cl = __float_as_uint(q3.x), cr = __float_as_uint(q3.y);
            if (L && R) {
                bool left_first = (L0 == R0) ? (L1 < R1) : (L0 < R0);
                uint32_t near_l = left_first ? cl : cr;
                uint32_t far_l = left_first ? cr : cl;
                if (sp < kStackSize) {
                    stack[sp++] = far_l;
                } else {
                    err |= kErrStackOverflow;  // unreachable: tree depth <= 63
                }
                link = near_l;
            } else if (L) {
                link = cl;
            } else if (R) {
                link = cr;
            } else {
                link = (sp == 0) ? kDone : stack[--sp];
            }
        }
        if (link == kDone) break;
        // leaf: primitives in the reference primitive_ids order
        {
            const uint32_t first = link & 0x0fffffffu;
            const uint32_t count = ((link >> 28) & 7u) + 1u;
            for (uint32_t k = 0; k < count; ++k) {
                const float4* pp = prims + 3 * (size_t)(first + k);
                const float4 a = __ldg(pp + 0);
                const float4 b = __ldg(pp + 1);
                if (kCount) cnt->prims++;
                if (__float_as_uint(b.w) == 0u) {
                    const float4 c = __ldg(pp + 2);
                    if (tri_test(ro, rd, xyz(a), xyz(b), xyz(c), tmin)) prim = (int32_t)__float_as_uint(a.w);
                } else {
                    if (sphere_test(ro, rd, xyz(a), b.x, tmin)) prim = (int32_t)__float_as_uint(a.w);
                }
            }
        }
        if (sp == 0) break;
        link = stack[--sp];
    }
    return prim;
}

// geometric normal of a hit (extension_ray_cast_stackless.cl:224-239), from
// the original vertices so the subtractions match the reference exactly
RGR_DEV f3 hit_normal(const SceneView& sc, int32_t prim, f3 ro, f3 rd, float t) {
    if (prim < sc.sphere_begin) {
        const uint32_t i0 = __ldg(sc.indices + 3 * (size_t)prim), i1 = __ldg(sc.indices + 3 * (size_t)prim + 1),
                       i2 = __ldg(sc.indices + 3 * (size_t)prim + 2);
        f3 v0 = xyz(__ldg(sc.points + i0)), v1 = xyz(__ldg(sc.points + i1)), v2 = xyz(__ldg(sc.points + i2));
        return normalize(cross(v2 - v1, v1 - v0));
    }
    float4 s = __ldg(sc.spheres + (prim - sc.sphere_begin));
    return normalize((ro + rd * t) - xyz(s));
}

}  // namespace dev
}  // namespace rgr
