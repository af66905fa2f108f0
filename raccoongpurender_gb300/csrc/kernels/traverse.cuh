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
// two 32-byte read-only loads), leaves encoded in the parent's link, and
// primitives pre-gathered in leaf order as 48-byte records (v0, v1-v0, v2-v0:
// the edge subtraction is done once on the host and is bit-identical).
//
// The state of one ray lives in TraceState so that a warp can run rounds
// (inner nodes down to one leaf, then that leaf) and refill finished lanes
// with new rays between rounds; the visit order of each ray is unchanged.
// trace_warp_round lets the lanes that found their leaf wait while enough
// others still search, instead of waiting for the last one (exact: each lane
// still intersects its leaves in its own order).
// BVH loads carry an L2 evict-last policy so that streaming ray data does not
// push the tree out of L2.
#pragma once
#include "rgr_device.cuh"

namespace rgr {
namespace dev {

constexpr int kStackSize = 64;  // the builder limits tree depth to 63
#ifndef RGR_SMEM_STACK
#define RGR_SMEM_STACK 12
#endif
// The persistent kernels keep the first kSmemStack pending far links of each
// thread in shared memory (entry i of thread t at i * kStackThreads + t: no
// bank conflicts), the deeper ones in local memory.  A local-memory stack of
// a full SM's threads does not fit in L1 and would be written back to L2.
constexpr int kSmemStack = RGR_SMEM_STACK;
constexpr int kStackThreads = 256;  // block size of the kernels that use it
constexpr uint32_t kDone = 0xffffffffu;
constexpr uint32_t kErrStackOverflow = 1u;

// ------------------------------------------------------------ cache policy
RGR_DEV uint64_t l2_evict_last_policy() {
    uint64_t p;
    asm("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(p));
    return p;
}
// read-only 16-byte load with an L2 cache-eviction policy
RGR_DEV float4 ld_keep(const float4* ptr, uint64_t pol) {
    float4 v;
    asm("ld.global.nc.L2::cache_hint.v4.f32 {%0, %1, %2, %3}, [%4], %5;"
        : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w)
        : "l"(ptr), "l"(pol));
    return v;
}

// 32-byte read-only load (sm_100 and later) into two float4, same policy; the
// address must be 32-byte aligned.  A warp's divergent lanes cost the L1 one
// request per lane per load instruction, so a 64-byte node in two of these
// costs half of what four 16-byte loads do.
RGR_DEV void ld_keep8(const float4* ptr, uint64_t pol, float4& a, float4& b) {
    asm("ld.global.nc.L2::cache_hint.v8.f32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8], %9;"
        : "=f"(a.x), "=f"(a.y), "=f"(a.z), "=f"(a.w), "=f"(b.x), "=f"(b.y), "=f"(b.z), "=f"(b.w)
        : "l"(ptr), "l"(pol));
}

// slabs_with_hit (extension_ray_cast_stackless.cl:35-50).  fminf/fmaxf have
// the reference's NaN behaviour; their results only feed comparisons, so the
// sign of a zero result cannot change a decision.  kNanCheck = false is the
// same function for rays whose products (lo - ro) * inv cannot be NaN (see
// ray_is_nan_free); the reference's select(t, -t', isnan(t)) is then the
// identity.
template <bool kNanCheck>
RGR_DEV bool slab(float lox, float loy, float loz, float hix, float hiy, float hiz, f3 ro, f3 inv, float farclip,
                  float& h0, float& h1) {
    float t0x = (lox - ro.x) * inv.x, t0y = (loy - ro.y) * inv.y, t0z = (loz - ro.z) * inv.z;
    float t1x = (hix - ro.x) * inv.x, t1y = (hiy - ro.y) * inv.y, t1z = (hiz - ro.z) * inv.z;
    if (kNanCheck) {
        t0x = isnan(t0x) ? -t1x : t0x;
        t0y = isnan(t0y) ? -t1y : t0y;
        t0z = isnan(t0z) ? -t1z : t0z;
        t1x = isnan(t1x) ? -t0x : t1x;
        t1y = isnan(t1y) ? -t0y : t1y;
        t1z = isnan(t1z) ? -t0z : t1z;
    }
    float rmin = fmaxf(fmaxf(fminf(t0x, t1x), fminf(t0y, t1y)), fminf(t0z, t1z));
    float rmax = fminf(fminf(fmaxf(t0x, t1x), fmaxf(t0y, t1y)), fmaxf(t0z, t1z));
    h0 = fmaxf(0.0f, rmin);
    h1 = fminf(rmax, farclip);
    return rmin <= rmax && 0.0f <= rmax && rmin <= farclip;
}

// (lo - ro) * inv is never NaN when ro is finite and small, every inv
// component is finite and non-zero, and the scene box is small (checked on
// the host): the difference is finite and the product of two finite non-zero
// numbers is a number or an infinity.
RGR_DEV bool ray_is_nan_free(f3 ro, f3 inv, bool scene_small) {
    const float kBig = 1.0e30f;
    return scene_small && fabsf(ro.x) <= kBig && fabsf(ro.y) <= kBig && fabsf(ro.z) <= kBig &&
           is_finite_nonzero(inv.x) && is_finite_nonzero(inv.y) && is_finite_nonzero(inv.z);
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

struct TraceState {
    f3 ro, rd, inv;
    float tmin;       // ExtensionResult.tmin: far clip in, hit distance out
    int32_t prim;     // -1 until a primitive is hit
    uint32_t link;    // next node link; kDone when the ray is finished
    int sp;           // pending far links; the newest is in `top`, older ones in stack[0..sp-2]
    uint32_t top;
    bool nan_free;
    uint32_t* sstk;   // this thread's shared-memory entries (stride kStackThreads), with kSm > 0
    uint32_t stack[kStackSize];
};

template <int kSm>
RGR_DEV void stack_put(TraceState& s, int i, uint32_t v) {
    if (kSm > 0 && i < kSm)
        s.sstk[i * kStackThreads] = v;
    else
        s.stack[i] = v;
}
template <int kSm>
RGR_DEV uint32_t stack_get(const TraceState& s, int i) {
    return (kSm > 0 && i < kSm) ? s.sstk[i * kStackThreads] : s.stack[i];
}

RGR_DEV void trace_begin(const SceneView& sc, TraceState& s, f3 ro, f3 rd, float tmax) {
    s.ro = ro;
    s.rd = rd;
    s.inv = mk(1.0f / rd.x, 1.0f / rd.y, 1.0f / rd.z);
    s.tmin = tmax;
    s.prim = -1;
    s.link = sc.num_prims == 0 ? kDone : sc.root_link;
    s.sp = 0;
    s.nan_free = ray_is_nan_free(ro, s.inv, sc.small_coords != 0);
}

// the newest pending far link, or kDone; the next one is fetched from the
// stack now but needed only at the following pop
template <int kSm>
RGR_DEV uint32_t pop(TraceState& s) {
    if (s.sp == 0) return kDone;
    const uint32_t link = s.top;
    --s.sp;
    if (s.sp > 0) s.top = stack_get<kSm>(s, s.sp - 1);
    return link;
}

// Shared-memory copy of the first inner nodes (the builder puts the top levels
// there, breadth-first); links below `n` are read from it.
struct StagedNodes {
    const float4* smem;
    uint32_t n;
};

// One inner node: both child boxes slab-tested against the current tmin
// (extension_ray_cast_stackless.cl:81-200); returns the next link (the
// nearer hit child, the only hit child, or the newest pending far link).
template <bool kNanCheck, bool kCount, bool kStaged, int kSm>
RGR_DEV uint32_t node_step(const SceneView& sc, TraceState& s, uint32_t link, TraceCounters* cnt, uint32_t& err,
                           uint64_t pol, StagedNodes st) {
    float4 q0, q1, q2, q3;
    if (kStaged && link < st.n) {
        const float4* np = st.smem + 4 * link;
        q0 = np[0];
        q1 = np[1];
        q2 = np[2];
        q3 = np[3];
    } else {
        const float4* np = sc.nodes + 4 * (size_t)link;  // 64-byte aligned
        ld_keep8(np, pol, q0, q1);
        ld_keep8(np + 2, pol, q2, q3);
    }
    if (kCount) cnt->nodes++;
    float L0, L1, R0, R1;
    const bool L = slab<kNanCheck>(q0.x, q0.y, q0.z, q0.w, q1.x, q1.y, s.ro, s.inv, s.tmin, L0, L1);
    const bool R = slab<kNanCheck>(q1.z, q1.w, q2.x, q2.y, q2.z, q2.w, s.ro, s.inv, s.tmin, R0, R1);
    const uint32_t cl = __float_as_uint(q3.x), cr = __float_as_uint(q3.y);
    if (L && R) {
        const bool left_first = (L0 == R0) ? (L1 < R1) : (L0 < R0);
        if (s.sp < kStackSize) {  // push the far child
            if (s.sp > 0) stack_put<kSm>(s, s.sp - 1, s.top);
            s.top = left_first ? cr : cl;
            s.sp++;
        } else {
            err |= kErrStackOverflow;  // unreachable: tree depth <= 63
        }
        return left_first ? cl : cr;
    }
    if (L) return cl;
    if (R) return cr;
    return pop<kSm>(s);
}

// The primitives of the leaf `link` in the reference primitive_ids order;
// returns the newest pending far link.
template <bool kCount, int kSm>
RGR_DEV uint32_t leaf_step(const SceneView& sc, TraceState& s, uint32_t link, TraceCounters* cnt, uint64_t pol) {
    const float4* __restrict__ prims = sc.prims;
    const uint32_t first = link & 0x0fffffffu;
    const uint32_t count = ((link >> 28) & 7u) + 1u;
    for (uint32_t k = 0; k < count; ++k) {
        // a 48-byte record starts on a 32-byte boundary when its index is even:
        // (a, b) in one 32-byte load and c in a 16-byte one; when it is odd, a in
        // a 16-byte load and (b, c) in a 32-byte one
        const uint32_t rec = first + k;
        const float4* pp = prims + 3 * (size_t)rec;
        const bool even = (rec & 1u) == 0u;
        float4 w0, w1;
        ld_keep8(even ? pp : pp + 1, pol, w0, w1);
        const float4 w2 = ld_keep(even ? pp + 2 : pp, pol);
        const float4 a = even ? w0 : w2, b = even ? w1 : w0, c = even ? w2 : w1;
        if (kCount) cnt->prims++;
        if (__float_as_uint(b.w) == 0u) {
            if (tri_test(s.ro, s.rd, xyz(a), xyz(b), xyz(c), s.tmin)) s.prim = (int32_t)__float_as_uint(a.w);
        } else {
            if (sphere_test(s.ro, s.rd, xyz(a), b.x, s.tmin)) s.prim = (int32_t)__float_as_uint(a.w);
        }
    }
    return pop<kSm>(s);
}

// One round: inner nodes down to the next leaf, then that leaf.  On return
// s.link is the next link to visit, or kDone.
template <bool kNanCheck, bool kCount, bool kStaged, int kSm>
RGR_DEV void trace_round_t(const SceneView& sc, TraceState& s, TraceCounters* cnt, uint32_t& err, uint64_t pol,
                           StagedNodes st) {
    uint32_t link = s.link;
    while (!(link & kLeafFlag)) link = node_step<kNanCheck, kCount, kStaged, kSm>(sc, s, link, cnt, err, pol, st);
    if (link != kDone) link = leaf_step<kCount, kSm>(sc, s, link, cnt, pol);
    s.link = link;
}

// kSm: stack entries in shared memory (s.sstk set), 0 for a local-memory stack
template <bool kCount, bool kStaged = false, int kSm = 0>
RGR_DEV void trace_round(const SceneView& sc, TraceState& s, TraceCounters* cnt, uint32_t& err, uint64_t pol,
                         StagedNodes st = StagedNodes{nullptr, 0u}) {
    if (s.nan_free) {
        trace_round_t<false, kCount, kStaged, kSm>(sc, s, cnt, err, pol, st);
    } else {
        trace_round_t<true, kCount, kStaged, kSm>(sc, s, cnt, err, pol, st);
    }
}

// A round of the whole warp; all 32 lanes call it, `active` on the lanes
// whose ray is not finished (s.link != kDone).  The active lanes take node
// steps while at least `min_search` of them are still searching for their
// next leaf (lanes that reached a leaf, or the end, wait; with min_search =
// 1 all of them wait for the last), then the lanes at a leaf intersect it.
// The warp votes once per two node steps (measured: 3702 against 3591
// Mrays/s with a vote per step on the 1.31M-triangle closest-hit workload).
// A lane still searching keeps its place and goes on in the next round, so
// each ray visits the same nodes and leaves in the same order as in
// trace_round.  `sc` must be a valid scene on every lane.
template <bool kCount, bool kStaged, int kSm>
RGR_DEV void trace_warp_round(const SceneView& sc, TraceState& s, bool active, int min_search, TraceCounters* cnt,
                              uint32_t& err, uint64_t pol, StagedNodes st = StagedNodes{nullptr, 0u}) {
    const unsigned full = 0xffffffffu;
    const unsigned act = __ballot_sync(full, active);
    const bool all_nan_free = __all_sync(full, !active || s.nan_free);
    uint32_t link = active ? s.link : kDone;
    for (;;) {
        const bool searching = !(link & kLeafFlag);  // kDone carries the leaf flag
        const unsigned sm = __ballot_sync(full, searching);
        if (sm == 0u || (sm != act && (int)__popc(sm) < min_search)) break;
        if (searching) {
            if (all_nan_free) {
                link = node_step<false, kCount, kStaged, kSm>(sc, s, link, cnt, err, pol, st);
                if (!(link & kLeafFlag)) link = node_step<false, kCount, kStaged, kSm>(sc, s, link, cnt, err, pol, st);
            } else {
                link = s.nan_free ? node_step<false, kCount, kStaged, kSm>(sc, s, link, cnt, err, pol, st)
                                  : node_step<true, kCount, kStaged, kSm>(sc, s, link, cnt, err, pol, st);
            }
        }
    }
    if (link != kDone && (link & kLeafFlag)) link = leaf_step<kCount, kSm>(sc, s, link, cnt, pol);
    if (active) s.link = link;
}

// Closest hit of one ray.  tmin in: the ray's far clip (ExtensionResult.tmin);
// out: the hit distance (unchanged on a miss).  Returns the primitive id or -1.
template <bool kCount>
RGR_DEV int32_t trace_closest(const SceneView& sc, f3 ro, f3 rd, float& tmin, TraceCounters* cnt, uint32_t& err) {
    TraceState s;
    trace_begin(sc, s, ro, rd, tmin);
    const uint64_t pol = l2_evict_last_policy();
    while (s.link != kDone) trace_round<kCount>(sc, s, cnt, err, pol);
    tmin = s.tmin;
    return s.prim;
}

// geometric normal of a hit (extension_ray_cast_stackless.cl:224-239), from
// the original vertices so the subtractions match the reference exactly
RGR_DEV f3 triangle_normal(const SceneView& sc, int32_t prim) {
    const uint32_t i0 = __ldg(sc.indices + 3 * (size_t)prim), i1 = __ldg(sc.indices + 3 * (size_t)prim + 1),
                   i2 = __ldg(sc.indices + 3 * (size_t)prim + 2);
    f3 v0 = xyz(__ldg(sc.points + i0)), v1 = xyz(__ldg(sc.points + i1)), v2 = xyz(__ldg(sc.points + i2));
    return normalize(cross(v2 - v1, v1 - v0));
}
// a triangle's normal comes from the per-triangle table the upload fills with
// triangle_normal (one gather instead of the indices, then the points)
RGR_DEV f3 hit_normal(const SceneView& sc, int32_t prim, f3 ro, f3 rd, float t) {
    if (prim < sc.sphere_begin) return sc.tri_normals ? xyz(__ldg(sc.tri_normals + prim)) : triangle_normal(sc, prim);
    float4 s = __ldg(sc.spheres + (prim - sc.sphere_begin));
    return normalize((ro + rd * t) - xyz(s));
}

}  // namespace dev
}  // namespace rgr
