// rgr_oracle.cpp — CPU oracle for the RaccoonGPURender wavefront hot path.
//
// TEST INFRASTRUCTURE ONLY.  This file restates, function by function, the
// reference OpenCL kernels (kernels/*.cl) and the host table builders
// (common/share/envmap.hpp, common/share/alias_method.hpp) as sequential C++,
// so the CUDA product can be checked against it.  It is imported only by
// tests/, __graft_entry__.smoke() and bench.py's cpu_baseline leg.
//
// Arithmetic conventions (stated once, applied everywhere):
//  * compiled with -ffp-contract=off: no fused multiply-add anywhere;
//  * OpenCL dot(a,b) = (a.x*b.x + a.y*b.y) + a.z*b.z, cross() by its
//    definition, normalize(v) = v / sqrt(dot(v,v)) per component;
//  * sin/cos/log/exp/atan/atan2/pow are the deterministic implementations of
//    rgr_fmath.h (the same ones the CUDA kernels use);
//  * "/" and sqrt are IEEE correctly rounded; denormals are kept (no FTZ);
//  * M_PI without a cast promotes to double exactly as C/OpenCL C does.
// Queue order: the reference fills queues with atomics (order unspecified);
// the oracle uses slot order, which is one valid execution.  Only the
// new-path queue order is observable (it assigns pixels, new_path.cl:41-43),
// and the CUDA path produces the same slot order for it.
#include "rgr_oracle.h"
#include "../raccoongpurender_gb300/csrc/rgr_fmath.h"

#include <cmath>
#include <cfloat>
#include <cstring>
#include <vector>
#include <thread>
#include <algorithm>
#include <atomic>
#include <memory>

using namespace rgr::fm;

namespace {

// ------------------------------------------------------------ float3 helpers
struct f3 {
    float x, y, z;
};
inline f3 mk(float x, float y, float z) { return f3{x, y, z}; }
inline f3 ld3(const float* p) { return f3{p[0], p[1], p[2]}; }
inline void st3(float* p, f3 v) { p[0] = v.x; p[1] = v.y; p[2] = v.z; }
inline f3 operator+(f3 a, f3 b) { return mk(a.x + b.x, a.y + b.y, a.z + b.z); }
inline f3 operator-(f3 a, f3 b) { return mk(a.x - b.x, a.y - b.y, a.z - b.z); }
inline f3 operator*(f3 a, f3 b) { return mk(a.x * b.x, a.y * b.y, a.z * b.z); }
inline f3 operator/(f3 a, f3 b) { return mk(a.x / b.x, a.y / b.y, a.z / b.z); }
inline f3 operator*(f3 a, float s) { return mk(a.x * s, a.y * s, a.z * s); }
inline f3 operator*(float s, f3 a) { return mk(s * a.x, s * a.y, s * a.z); }
inline f3 operator/(f3 a, float s) { return mk(a.x / s, a.y / s, a.z / s); }
inline f3 operator-(f3 a) { return mk(-a.x, -a.y, -a.z); }
inline float dot(f3 a, f3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline f3 cross(f3 a, f3 b) {
    return mk(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
inline f3 normalize(f3 v) {
    float l = sqrt_(dot(v, v));
    return mk(v.x / l, v.y / l, v.z / l);
}
inline float sqr(float x) { return x * x; }
inline f3 mix3(f3 a, f3 b, float t) {
    return mk(mix_(a.x, b.x, t), mix_(a.y, b.y, t), mix_(a.z, b.z, t));
}
// OpenCL float M_PI cast, e.g. (float)(M_PI)
const float kPiF = (float)M_PI;

// ------------------------------------------------------------ RNG
// kernels/peseudo_random.cl:5-64 (CPU twin common/share/peseudo_random.hpp:160-272)
inline uint32_t rotl(uint32_t x, int k) { return (x << k) | (x >> (32 - k)); }
struct Rng {
    uint32_t s[4];
    uint32_t next() {  // xoshiro128_star_star_next, peseudo_random.cl:10-24
        const uint32_t result = rotl(s[0] * 5u, 7) * 9u;
        const uint32_t t = s[1] << 9;
        s[2] ^= s[0];
        s[3] ^= s[1];
        s[1] ^= s[2];
        s[0] ^= s[3];
        s[2] ^= t;
        s[3] = rotl(s[3], 11);
        return result;
    }
    float uniform() {  // random_uniform, peseudo_random.cl:26-29
        uint32_t bits = (next() >> 9) | 0x3f800000u;
        return as_float(bits) - 1.0f;
    }
    uint64_t uniform_integer() {  // random_uniform_integer, peseudo_random.cl:35-40
        uint64_t a = next() >> 1;
        uint64_t b = next() >> 1;
        return (a << 31) | b;
    }
};
inline uint64_t splitmix64(uint64_t* x) {  // peseudo_random.cl:42-47
    uint64_t z = (*x += 0x9e3779b97f4a7c15ull);
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    return z ^ (z >> 31);
}
inline void random_initialize_one(uint32_t* s, uint64_t x) {  // peseudo_random.cl:48-64
    uint64_t r0 = splitmix64(&x);
    uint64_t r1 = splitmix64(&x);
    s[0] = (uint32_t)(r0 & 0xffffffffu);
    s[1] = (uint32_t)(r0 >> 32);
    s[2] = (uint32_t)(r1 & 0xffffffffu);
    s[3] = (uint32_t)(r1 >> 32);
    if (s[0] == 0 && s[1] == 0 && s[2] == 0 && s[3] == 0) s[0] = 1;
}

// ------------------------------------------------------------ traversal
// slabs_with_hit, extension_ray_cast_stackless.cl:35-50 (slab.cl:10-21)
inline bool slabs_with_hit(f3 p0, f3 p1, f3 ro, f3 inv, float farclip, float* h0, float* h1) {
    f3 t0 = (p0 - ro) * inv;
    f3 t1 = (p1 - ro) * inv;
    // select(t0, -t1, isnan(t0)); select(t1, -t0, isnan(t1))
    t0.x = is_nan(t0.x) ? -t1.x : t0.x;
    t0.y = is_nan(t0.y) ? -t1.y : t0.y;
    t0.z = is_nan(t0.z) ? -t1.z : t0.z;
    t1.x = is_nan(t1.x) ? -t0.x : t1.x;
    t1.y = is_nan(t1.y) ? -t0.y : t1.y;
    t1.z = is_nan(t1.z) ? -t0.z : t1.z;
    f3 tmin = mk(fmin_(t0.x, t1.x), fmin_(t0.y, t1.y), fmin_(t0.z, t1.z));
    f3 tmax = mk(fmax_(t0.x, t1.x), fmax_(t0.y, t1.y), fmax_(t0.z, t1.z));
    float region_min = fmax_(fmax_(tmin.x, tmin.y), tmin.z);  // compMax
    float region_max = fmin_(fmin_(tmax.x, tmax.y), tmax.z);  // compMin
    *h0 = fmax_(0.0f, region_min);
    *h1 = fmin_(region_max, farclip);
    return region_min <= region_max && 0.0f <= region_max && region_min <= farclip;
}
// intersect_ray_triangle, intersect_triangle.cl:7-44
inline bool intersect_ray_triangle(f3 ro, f3 rd, f3 v0, f3 v1, f3 v2, float* tmin) {
    const float kEpsilon = 1.0e-8f;
    f3 v0v1 = v1 - v0;
    f3 v0v2 = v2 - v0;
    f3 pvec = cross(rd, v0v2);
    float det = dot(v0v1, pvec);
    if (fabs_(det) < kEpsilon) return false;
    float invDet = 1.0f / det;
    f3 tvec = ro - v0;
    float u = dot(tvec, pvec) * invDet;
    if (u < 0.0f || u > 1.0f) return false;
    f3 qvec = cross(tvec, v0v1);
    float v = dot(rd, qvec) * invDet;
    if (v < 0.0f || u + v > 1.0f) return false;
    float t = dot(v0v2, qvec) * invDet;
    if (t < 0.0f) return false;
    if (*tmin < t) return false;
    *tmin = t;
    return true;
}
// intersect_sphere, extension_ray_cast_stackless.cl:52-76
inline bool intersect_sphere(f3 ro, f3 rd, f3 o, float r, float* tmin) {
    float r_sq = r * r;
    f3 S = ro - o;
    f3 crs = cross(S, rd);
    float d_sq = dot(crs, crs);
    float B = dot(S, rd);
    float D = r_sq - d_sq;
    if (D < 0.0f) return false;
    float D_sqrt = sqrt_(D);
    float t0 = -B - D_sqrt;
    float t1 = -B + D_sqrt;
    if (0.0f < t0 && t0 < *tmin) {
        *tmin = t0;
        return true;
    }
    if (0.0f < t1 && t1 < *tmin) {
        *tmin = t1;
        return true;
    }
    return false;
}
inline f3 pt(const orc_scene* s, uint32_t i) { return ld3(s->points + 4 * (size_t)i); }

// intersect_bvh, extension_ray_cast_stackless.cl:81-200 (64-bit bitstack,
// parent/sibling links, near child first with the exact == tie rule).
inline bool intersect_bvh(const orc_scene* s, f3 ro, f3 rd, float tmin, float* t_out,
                          int32_t* prim_out, uint32_t* visits, uint32_t* tests) {
    bool intersected = false;
    f3 inv = mk(1.0f / rd.x, 1.0f / rd.y, 1.0f / rd.z);
    int32_t primitive_index = -1;
    uint64_t bitstack = 0;
    uint32_t node = 0;
    uint32_t nv = 0, nt = 0;
    for (;;) {
        const orc_node& N = s->nodes[node];
        bool branch = N.primitive_indices_end == 0;
        if (branch) {
            nv++;
            float L0, L1, R0, R1;
            bool L = slabs_with_hit(ld3(N.L_lower), ld3(N.L_upper), ro, inv, tmin, &L0, &L1);
            bool R = slabs_with_hit(ld3(N.R_lower), ld3(N.R_upper), ro, inv, tmin, &R0, &R1);
            if (L || R) {
                bitstack = bitstack << 1;
                if (L && R) {
                    uint32_t near_node;
                    if (L0 == R0) {
                        near_node = L1 < R1 ? N.link_L : N.link_R;
                    } else {
                        near_node = L0 < R0 ? N.link_L : N.link_R;
                    }
                    node = near_node;
                    bitstack = bitstack | 1;
                } else if (L) {
                    node = N.link_L;
                } else {
                    node = N.link_R;
                }
                continue;
            }
        } else {
            int beg = (int)N.primitive_indices_beg;
            int end = (int)N.primitive_indices_end;
            for (int i = beg; i < end; ++i) {
                uint32_t p = s->prim_ids[i];
                nt++;
                if (p < (uint32_t)s->sphere_begin) {
                    size_t b = (size_t)p * 3;
                    if (intersect_ray_triangle(ro, rd, pt(s, s->indices[b]), pt(s, s->indices[b + 1]),
                                               pt(s, s->indices[b + 2]), &tmin)) {
                        primitive_index = (int32_t)p;
                        intersected = true;
                    }
                } else {
                    const float* sp = s->spheres + 4 * (size_t)(p - (uint32_t)s->sphere_begin);
                    if (intersect_sphere(ro, rd, ld3(sp), sp[3], &tmin)) {
                        primitive_index = (int32_t)p;
                        intersected = true;
                    }
                }
            }
        }
        // backtrack
        while ((bitstack & 1) == 0) {
            if (bitstack == 0) {
                *t_out = tmin;
                *prim_out = primitive_index;
                if (visits) *visits = nv;
                if (tests) *tests = nt;
                return intersected;
            }
            node = s->nodes[node].link_parent;
            bitstack = bitstack >> 1;
        }
        node = s->nodes[node].link_sibling;
        bitstack = bitstack ^ 1;
    }
}
// geometric normal of the hit, extension_ray_cast_stackless.cl:224-239
inline f3 hit_normal(const orc_scene* s, int32_t prim, f3 ro, f3 rd, float t) {
    if (prim < s->sphere_begin) {
        size_t b = (size_t)prim * 3;
        f3 v0 = pt(s, s->indices[b]), v1 = pt(s, s->indices[b + 1]), v2 = pt(s, s->indices[b + 2]);
        return normalize(cross(v2 - v1, v1 - v0));  // clockwise
    }
    const float* sp = s->spheres + 4 * (size_t)(prim - s->sphere_begin);
    return normalize((ro + rd * t) - ld3(sp));
}

// ------------------------------------------------------------ envmap
// cartesian_to_polar, envmap_sampling.cl:25-34
inline void cartesian_to_polar(f3 rd, float* theta, float* phi) {
    float z = rd.y, x = rd.z, y = rd.x;
    *theta = atan2_(sqrt_(x * x + y * y), z);
    *phi = atan2_(y, x);
    if (!is_finite(*phi)) *phi = 0.0f;
}
inline int fract_int(int x, int m) {  // envmap_sampling.cl:75-78
    int r = x % m;
    return r < 0 ? r + m : r;
}
inline int to_int(float x) {  // (int) conversion with NaN -> 0 and saturation
    if (is_nan(x)) return 0;
    if (x >= 2147483648.0f) return 2147483647;
    if (x <= -2147483648.0f) return (-2147483647 - 1);
    return (int)x;
}
// envmap_index, envmap_sampling.cl:80-95
inline int envmap_index(f3 wi, int width, int height) {
    float theta, phi;
    cartesian_to_polar(wi, &theta, &phi);
    const float pi = kPiF;
    float u = 1.0f - phi / (2.0f * pi);
    float v = theta / pi;
    int ix = to_int(floor_(u * (float)width));
    int iy = to_int(floor_(v * (float)height));
    ix = fract_int(ix, width);
    iy = std::min(std::max(iy, 0), height - 1);
    return iy * width + ix;
}
// read_imagef with CLK_NORMALIZED_COORDS_TRUE | CLK_ADDRESS_REPEAT and
// CLK_FILTER_NEAREST / CLK_FILTER_LINEAR, following the OpenCL 1.2
// specification's addressing formulas with FP32 weights.
inline f3 texel(const orc_scene* s, int i, int j) {
    const float* p = s->env_rgba + 4 * ((size_t)j * s->env_w + i);
    return mk(p[0], p[1], p[2]);
}
inline f3 read_image_repeat(const orc_scene* s, float su, float sv, bool linear) {
    int w = s->env_w, h = s->env_h;
    float u = (su - floor_(su)) * (float)w;
    float v = (sv - floor_(sv)) * (float)h;
    if (!linear) {
        int i = to_int(floor_(u));
        int j = to_int(floor_(v));
        if (i > w - 1) i = i - w;
        if (j > h - 1) j = j - h;
        i = std::min(std::max(i, 0), w - 1);
        j = std::min(std::max(j, 0), h - 1);
        return texel(s, i, j);
    }
    float uu = u - 0.5f, vv = v - 0.5f;
    int i0 = to_int(floor_(uu)), j0 = to_int(floor_(vv));
    int i1 = i0 + 1, j1 = j0 + 1;
    if (i0 < 0) i0 = w + i0;
    if (i1 > w - 1) i1 = i1 - w;
    if (j0 < 0) j0 = h + j0;
    if (j1 > h - 1) j1 = j1 - h;
    i0 = std::min(std::max(i0, 0), w - 1);
    i1 = std::min(std::max(i1, 0), w - 1);
    j0 = std::min(std::max(j0, 0), h - 1);
    j1 = std::min(std::max(j1, 0), h - 1);
    float a = uu - floor_(uu);
    float b = vv - floor_(vv);
    float w00 = (1.0f - a) * (1.0f - b), w10 = a * (1.0f - b);
    float w01 = (1.0f - a) * b, w11 = a * b;
    f3 t00 = texel(s, i0, j0), t10 = texel(s, i1, j0), t01 = texel(s, i0, j1), t11 = texel(s, i1, j1);
    return ((t00 * w00 + t10 * w10) + t01 * w01) + t11 * w11;
}
// The bilinear lookup above with the two filter weights rounded to multiples of
// 2^-frac_bits, as GPU texture units hold them (8 fractional bits on NVIDIA
// hardware): the filtering an OpenCL image sampler gives, for bounding the
// difference to the FP32-weight filter that both this file and the CUDA path use.
inline f3 read_image_repeat_quantized(const orc_scene* s, float su, float sv, int frac_bits) {
    int w = s->env_w, h = s->env_h;
    float u = (su - floor_(su)) * (float)w;
    float v = (sv - floor_(sv)) * (float)h;
    float uu = u - 0.5f, vv = v - 0.5f;
    int i0 = to_int(floor_(uu)), j0 = to_int(floor_(vv));
    int i1 = i0 + 1, j1 = j0 + 1;
    if (i0 < 0) i0 = w + i0;
    if (i1 > w - 1) i1 = i1 - w;
    if (j0 < 0) j0 = h + j0;
    if (j1 > h - 1) j1 = j1 - h;
    i0 = std::min(std::max(i0, 0), w - 1);
    i1 = std::min(std::max(i1, 0), w - 1);
    j0 = std::min(std::max(j0, 0), h - 1);
    j1 = std::min(std::max(j1, 0), h - 1);
    const float scale = (float)(1 << frac_bits);
    float a = std::nearbyint((uu - floor_(uu)) * scale) / scale;
    float b = std::nearbyint((vv - floor_(vv)) * scale) / scale;
    float w00 = (1.0f - a) * (1.0f - b), w10 = a * (1.0f - b);
    float w01 = (1.0f - a) * b, w11 = a * b;
    f3 t00 = texel(s, i0, j0), t10 = texel(s, i1, j0), t01 = texel(s, i0, j1), t11 = texel(s, i1, j1);
    return ((t00 * w00 + t10 * w10) + t01 * w01) + t11 * w11;
}
// get_envmap_value, envmap_sampling.cl:36-52
inline f3 get_envmap_value(const orc_scene* s, f3 rd, bool use_filter) {
    float theta, phi;
    cartesian_to_polar(rd, &theta, &phi);
    const float pi = kPiF;
    float u = 1.0f - phi / (2.0f * pi);
    float v = theta / pi;
    return read_image_repeat(s, u, v, use_filter);
}
struct AliasBucket {
    float height;
    int32_t alias;
};
// alias_method, envmap_sampling.cl:54-66
inline uint32_t alias_method(Rng* st, const float* heights, const int32_t* aliases, uint32_t count) {
    uint32_t idx = (uint32_t)(st->uniform_integer() % (uint64_t)count);
    int alias = aliases[idx];
    if (alias < 0) return idx;
    float height = heights[idx];
    float u = st->uniform();
    if (u < height) return idx;
    return (uint32_t)alias;
}
// sample_from_fragment + project_cylinder_to_sphere, envmap_sampling.cl:68-73, 158-167
inline f3 sample_from_fragment(const float* frag, Rng* st) {
    float y = mix_(frag[0], frag[1], st->uniform());
    float phi = mix_(frag[2], frag[3], st->uniform());
    f3 p = mk(sin_(phi), y, cos_(phi));
    float r_xz = sqrt_(fmax_(1.0f - p.y * p.y, 0.0f));
    p.x *= r_xz;
    p.z *= r_xz;
    return p;
}
inline size_t tbl(const orc_scene* s, int t) { return (size_t)t * (size_t)s->env_w * (size_t)s->env_h; }
// six-axis table bases, envmap_sampling.cl:134-139 (table 1+k holds CubeSection k)
inline void six_axis_bases(const orc_scene* s, f3 n, size_t* xb, size_t* yb, size_t* zb) {
    *xb = tbl(s, 0.0f < n.x ? 1 : 2);
    *yb = tbl(s, 0.0f < n.y ? 3 : 4);
    *zb = tbl(s, 0.0f < n.z ? 5 : 6);
}
// envmap_pdf_sixAxis, envmap_sampling.cl:100-124
inline float envmap_pdf_six_axis(const orc_scene* s, f3 wi, f3 n) {
    size_t xb, yb, zb;
    six_axis_bases(s, n, &xb, &yb, &zb);
    f3 ap = n * n;
    int index = envmap_index(wi, s->env_w, s->env_h);
    float pdf = 0.0f;
    pdf = pdf + ap.x * s->env_pdf[xb + index];
    pdf = pdf + ap.y * s->env_pdf[yb + index];
    pdf = pdf + ap.z * s->env_pdf[zb + index];
    return pdf;
}

// ------------------------------------------------------------ BSDF helpers
// cosine_weighted_hemisphere_z_up, lambertian.cl:9-20
inline f3 cosine_weighted_hemisphere_z_up(float a, float b) {
    float r = sqrt_(a);
    float theta = (float)((double)b * M_PI * 2.0);
    float x = r * cos_(theta);
    float y = r * sin_(theta);
    float z = sqrt_(fmax_(1.0f - a, 0.0f));
    return mk(x, y, z);
}
// get_orthonormal_basis, lambertian.cl:26-32 / ward.cl:9-15
inline void get_orthonormal_basis(f3 z, f3* xa, f3* ya) {
    const float sign = copysign_(1.0f, z.z);
    const float a = -1.0f / (sign + z.z);
    const float b = z.x * z.y * a;
    *xa = mk(1.0f + sign * z.x * z.x * a, sign * b, -sign * z.x);
    *ya = mk(b, sign + z.y * z.y * a, -z.y);
}
inline f3 reflect(f3 d, f3 n) { return d - (2.0f * dot(d, n)) * n; }  // ward.cl:35-37
// sample_ward, ward.cl:40-53
inline f3 sample_ward(f3 wo, f3 zaxis, float alpha, float u0, float u1) {
    const float pi = kPiF;
    float phiH = u0 * 2.0f * pi;
    float thetaH = atan_(alpha * sqrt_(-log_(u1)));
    float sinT = sin_(thetaH);  // polar_to_cartesian_z_up, ward.cl:27-33
    f3 hl = mk(sinT * cos_(phiH), sinT * sin_(phiH), cos_(thetaH));
    f3 xa, ya;
    get_orthonormal_basis(zaxis, &xa, &ya);
    f3 h = xa * hl.x + ya * hl.y + zaxis * hl.z;
    return reflect(-wo, h);
}
// pdf_ward, ward.cl:55-74
inline float pdf_ward(f3 wo, f3 wi, f3 zaxis, float alpha) {
    if (dot(wo, zaxis) * dot(wi, zaxis) < 0.0f) return 0.0f;
    const float alpha2 = sqr(alpha);
    const float pi = kPiF;
    f3 h = normalize(wi + wo);
    float c = dot(h, zaxis);
    float cosThetaH2 = sqr(c);
    float tanTheta2 = (1.0f - cosThetaH2) / cosThetaH2;
    float k0 = 1.0f / (4.0f * pi * alpha2 * dot(h, wi) * (c * c * c));
    float k1 = exp_(-tanTheta2 / alpha2);
    return k0 * k1;
}
// fresnel_dielectrics, delta_materials.cl:25-32
inline float fresnel_dielectrics(float c, float eta_t, float eta_i) {
    float g = sqrt_(eta_t * eta_t / sqr(eta_i) - 1.0f + sqr(c));
    float a = 0.5f * sqr(g - c) / sqr(g + c);
    float b = 1.0f + sqr(c * (g + c) - 1.0f) / sqr(c * (g - c) + 1.0f);
    return a * b;
}
// refract, delta_materials.cl:11-20
inline bool refract(f3* out, f3 d, f3 n, float eta_i, float eta_t) {
    float eta = eta_i / eta_t;
    float NoD = dot(n, d);
    float k = 1.0f - eta * eta * (1.0f - NoD * NoD);
    if (k <= 0.0f) return false;
    *out = eta * d - (eta * NoD + sqrt_(k)) * n;
    return true;
}
// uniform_on_unit_sphere, homogeneous_volume.cl:7-14
inline f3 uniform_on_unit_sphere(float u0, float u1) {
    float phi = (float)((double)u0 * M_PI * 2.0);
    float z = mix_(-1.0f, 1.0f, u1);
    float r_xy = sqrt_(fmax_(1.0f - z * z, 0.0f));
    return mk(r_xy * cos_(phi), r_xy * sin_(phi), z);
}
const float kPdfUniformSphere = (float)(1.0 / (M_PI * 4.0));  // homogeneous_volume.cl:15-17
const float kFourPiF = (float)(4.0 * M_PI);                   // homogeneous_volume.cl:120

inline uint32_t volume_hash(const orc_volume& v) {  // types.cl:104-106
    return as_uint(v.C) ^ as_uint(v.R[0]) ^ as_uint(v.R[1]) ^ as_uint(v.R[2]);
}

// ------------------------------------------------------------ wavefront
enum { kStrategyBxdf = 0, kStrategyEnv = 1, kStrategyNone = 2 };
enum {
    kMatNone = 0, kMatLambertian = 1, kMatSpecular = 2, kMatDielectric = 3, kMatWard = 4,
    kMatVolume = 5, kMatVolumeInside = 6
};
struct Slot {
    f3 T{0, 0, 0}, L{0, 0, 0}, ro{0, 0, 0}, rd{0, 0, 0};
    uint32_t logic_i = 0, pixel_index = 0;
    Rng rng;
    int32_t hit_surface = -1, hit_volume = -1;  // hit_volume initialised to -1 (reference leaves it unset)
    float tmin = FLT_MAX;
    f3 Ng{0, 0, 0};
    int32_t vol_count = 0;
    int32_t vols[7] = {0, 0, 0, 0, 0, 0, 0};
    int32_t queue = 0;  // next-step queue id; 0 = new path; -1 idle
    int32_t req = 0;    // request (batched renders)
};
struct Incident {
    f3 wi{0, 0, 0};
    float sel[2] = {0, 0};
    float pdf[2] = {0, 0};
    uint32_t strategy = 0;
};
inline float incident_pdf(const Incident& is) {  // types.cl:65-71
    float pdf = 0.0f;
    pdf = pdf + is.sel[0] * is.pdf[0];
    pdf = pdf + is.sel[1] * is.pdf[1];
    return pdf;
}

struct Ctx {
    const orc_scene* s;
    const orc_camera* cam;
    const orc_config* cfg;
    bool has_env;
};

// new_path, new_path.cl:17-83 (pixel already assigned)
void new_path(const Ctx& c, Slot& p, uint64_t global_pixel_index) {
    const orc_camera* cam = c.cam;
    p.T = mk(1, 1, 1);
    p.L = mk(0, 0, 0);
    p.logic_i = 0;
    uint32_t npix = cam->image_w * cam->image_h;
    uint32_t pixel_index = (uint32_t)(global_pixel_index % (uint64_t)npix);
    p.pixel_index = pixel_index;
    uint32_t x = pixel_index % cam->image_w;
    uint32_t y = pixel_index / cam->image_w;
    float ux, uy;
    if (c.cfg->new_path_y_first) {
        uy = p.rng.uniform();
        ux = p.rng.uniform();
    } else {
        ux = p.rng.uniform();
        uy = p.rng.uniform();
    }
    f3 sop = ld3(cam->imageplane_o) + ld3(cam->imageplane_r) * ((float)x + ux) +
             ld3(cam->imageplane_b) * ((float)y + uy);
    float u0 = p.rng.uniform();
    float u1 = p.rng.uniform();
    float dof = c.cfg->dof;
    float r = sqrt_(u0);
    float theta = (float)((double)u1 * M_PI * 2.0);
    float lensx = dof * r * cos_(theta);
    float lensy = dof * r * sin_(theta);
    f3 lens = ld3(cam->eye) + ld3(cam->up) * lensx + ld3(cam->right) * lensy;
    p.ro = lens;
    p.rd = normalize(sop - lens);
    p.vol_count = 0;
    p.hit_surface = -1;
    p.tmin = FLT_MAX;
    p.Ng = mk(0, 0, 0);
}

// strategy_selection, mixture_density.cl:7-133 (one slot). Returns the env
// queue: -1 none, 0 sample uniform, 1 eval uniform, 2 sample 6-axis, 3 eval 6-axis.
int strategy_selection(const Ctx& c, Slot& p, Incident& is) {
    bool surface_hit = 0 <= p.hit_surface;
    bool volume_hit = 0 <= p.hit_volume;
    bool any_hit = surface_hit || volume_hit;
    is = Incident();
    float env_p = c.has_env ? c.cfg->env_select_prob : 0.0f;
    if (any_hit) {
        if (surface_hit) {
            int mt = c.s->materials[p.hit_surface].type;
            if (mt == kMatLambertian || mt == kMatWard) {
                const float bxdf_p = 1.0f - env_p;
                is.sel[kStrategyBxdf] = bxdf_p;
                is.sel[kStrategyEnv] = 1.0f - bxdf_p;
            } else {
                is.sel[kStrategyBxdf] = 1.0f;
                is.sel[kStrategyEnv] = 0.0f;
            }
        } else {
            const float bxdf_p = 1.0f - env_p;
            is.sel[kStrategyBxdf] = bxdf_p;
            is.sel[kStrategyEnv] = 1.0f - bxdf_p;
        }
        float u = p.rng.uniform();
        is.strategy = (u <= is.sel[kStrategyBxdf]) ? kStrategyBxdf : kStrategyEnv;
    } else {
        is.strategy = kStrategyNone;
    }
    if (any_hit && is.sel[kStrategyEnv] != 0.0f) {
        int sample_q = volume_hit ? 0 : 2;
        int eval_q = volume_hit ? 1 : 3;
        return is.strategy == kStrategyEnv ? sample_q : eval_q;
    }
    return -1;
}

void step_slot(const Ctx& c, Slot& p, double* accum, bool is_new, uint64_t gpix) {
    const orc_scene* s = c.s;
    Incident is;
    if (is_new) new_path(c, p, gpix);
    // shading result (Le, T) of this step; new_path.cl:77-78 resets it
    f3 shadeLe = mk(0, 0, 0), shadeT = mk(1, 1, 1);
    int mq = is_new ? 0 : p.queue;

    int envq = strategy_selection(c, p, is);
    // sample env, envmap_sampling.cl:169-248
    if (envq == 2) {
        f3 n = p.Ng;
        f3 wo = -p.rd;
        if (dot(n, wo) < 0.0f) n = -n;
        size_t xb, yb, zb;
        six_axis_bases(s, n, &xb, &yb, &zb);
        uint32_t count = (uint32_t)(s->env_w * s->env_h);
        float u = p.rng.uniform();
        f3 ap = n * n;
        size_t sel;
        if (u < ap.x) sel = xb;
        else if (u < ap.x + ap.y) sel = yb;
        else sel = zb;
        uint32_t idx = alias_method(&p.rng, s->env_height + sel, s->env_alias + sel, count);
        float pdf = 0.0f;
        pdf = pdf + ap.x * s->env_pdf[xb + idx];
        pdf = pdf + ap.y * s->env_pdf[yb + idx];
        pdf = pdf + ap.z * s->env_pdf[zb + idx];
        is.wi = sample_from_fragment(s->env_frag + 4 * (size_t)idx, &p.rng);
        is.pdf[kStrategyEnv] = pdf;
    } else if (envq == 0) {
        uint32_t count = (uint32_t)(s->env_w * s->env_h);
        uint32_t idx = alias_method(&p.rng, s->env_height, s->env_alias, count);
        float pdf = s->env_pdf[idx];
        is.wi = sample_from_fragment(s->env_frag + 4 * (size_t)idx, &p.rng);
        is.pdf[kStrategyEnv] = pdf;
    }
    // sample or eval BSDF
    if (mq == kMatLambertian) {  // lambertian.cl:34-71
        f3 Ng = p.Ng;  // the raw Ng (lambertian.cl:49-68), or flipped toward the viewer
        if (c.cfg->two_sided_lambertian && dot(Ng, -p.rd) < 0.0f) Ng = -Ng;
        float cosTheta;
        if (is.strategy == kStrategyBxdf) {
            float u0 = p.rng.uniform();
            float u1 = p.rng.uniform();
            f3 wl = cosine_weighted_hemisphere_z_up(u0, u1);
            f3 xa, ya;
            get_orthonormal_basis(Ng, &xa, &ya);
            is.wi = xa * wl.x + ya * wl.y + Ng * wl.z;
            cosTheta = wl.z;
        } else {
            cosTheta = dot(Ng, is.wi);
        }
        is.pdf[kStrategyBxdf] = fmax_(cosTheta, 0.0f) / kPiF;
    } else if (mq == kMatWard) {  // ward.cl:76-117
        const orc_ward& w = s->wards[s->materials[p.hit_surface].index];
        f3 wo = -p.rd;
        f3 Ng = p.Ng;
        if (dot(Ng, wo) < 0.0f) Ng = -Ng;
        f3 wi;
        if (is.strategy == kStrategyBxdf) {
            float u0 = p.rng.uniform();
            float u1 = p.rng.uniform();
            wi = sample_ward(wo, Ng, w.alpha, u0, u1);
        } else {
            wi = is.wi;
        }
        is.wi = wi;
        is.pdf[kStrategyBxdf] = pdf_ward(wo, wi, Ng, w.alpha);
    } else if (mq == kMatVolumeInside) {  // homogeneous_volume.cl:66-88
        if (is.strategy == kStrategyBxdf) {
            float u0 = p.rng.uniform();
            float u1 = p.rng.uniform();
            is.wi = uniform_on_unit_sphere(u0, u1);
        }
        is.pdf[kStrategyBxdf] = kPdfUniformSphere;
    }
    // evaluate env pdf, envmap_sampling.cl:250-281
    if (envq == 3) {
        f3 n = p.Ng;  // the raw Ng (envmap_sampling.cl:263), or flipped like the sampler
        if (c.cfg->fix_backside_env_pdf && dot(n, -p.rd) < 0.0f) n = -n;
        is.pdf[kStrategyEnv] = envmap_pdf_six_axis(s, is.wi, n);
    } else if (envq == 1) {
        is.pdf[kStrategyEnv] = s->env_pdf[envmap_index(is.wi, s->env_w, s->env_h)];
    }
    // material stages
    if (mq == kMatLambertian) {  // lambertian_stage, lambertian.cl:73-123
        const orc_lambertian& m = s->lambertians[s->materials[p.hit_surface].index];
        f3 Ng = p.Ng;
        f3 wo = -p.rd;
        if (dot(Ng, wo) < 0.0f) Ng = -Ng;
        f3 wi = is.wi;
        float pdf = incident_pdf(is);
        float cosTheta = dot(wi, Ng);
        f3 T = mk(0, 0, 0);
        if (0.0f < cosTheta) T = ld3(m.R) / kPiF * cosTheta / pdf;
        shadeLe = ld3(m.Le);
        shadeT = T;
        p.ro = p.ro + p.rd * p.tmin + wi * 1.0e-5f + Ng * 1.0e-5f;
        p.rd = wi;
    } else if (mq == kMatWard) {  // ward_stage, ward.cl:119-186
        const orc_ward& w = s->wards[s->materials[p.hit_surface].index];
        f3 Ng = p.Ng;
        f3 wo = -p.rd;
        if (dot(Ng, wo) < 0.0f) Ng = -Ng;
        f3 wi = is.wi;
        float pdf = incident_pdf(is);
        float cosTheta = dot(wi, Ng);
        f3 T = mk(0, 0, 0);
        if (0.0f < cosTheta) {
            f3 lv = wi + wo;
            f3 h = normalize(lv);
            const float pi = kPiF;
            float alpha2 = sqr(w.alpha);
            float cosThetaH = dot(h, Ng);
            float cosThetaH2 = sqr(cosThetaH);
            float tanTheta2 = (1.0f - cosThetaH2) / cosThetaH2;
            float mu = dot(h, wi);
            f3 rho = mix3(ld3(w.reflectance), ld3(w.edgetint), pow_(1.0f - mu, 1.0f / w.falloff));
            f3 k0 = rho / (pi * alpha2);
            float k1 = exp_(-tanTheta2 / alpha2);
            float dn = dot(lv, Ng);
            float k2 = dot(lv, lv) / sqr(sqr(dn));
            T = k0 * k1 * k2 * cosTheta / pdf;
        }
        shadeLe = mk(0, 0, 0);
        shadeT = T;
        p.ro = p.ro + p.rd * p.tmin + wi * 1.0e-5f + Ng * 1.0e-5f;
        p.rd = wi;
    } else if (mq == kMatVolume) {  // homogeneous_volume_stage, homogeneous_volume.cl:19-64
        f3 wo = -p.rd;
        bool backside = dot(p.Ng, wo) < 0.0f;
        shadeLe = mk(0, 0, 0);
        shadeT = mk(1, 1, 1);
        int vm = p.hit_surface;
        if (backside) {  // inVolumeList_Remove, types.cl:115-132
            uint32_t hsh = volume_hash(s->volumes[s->materials[vm].index]);
            bool move = false;
            for (int i = 0; i < p.vol_count; ++i) {
                if (move) {
                    p.vols[i - 1] = p.vols[i];
                } else if (volume_hash(s->volumes[s->materials[p.vols[i]].index]) == hsh) {
                    move = true;
                }
            }
            if (move) p.vol_count--;
        } else {  // inVolumeList_Add, types.cl:108-114
            if (p.vol_count < 7) {
                p.vols[p.vol_count] = vm;
                p.vol_count++;
            }
        }
        p.ro = p.ro + p.rd * (p.tmin + 1.0e-5f);
    } else if (mq == kMatVolumeInside) {  // homogeneous_volume_inside_stage, homogeneous_volume.cl:90-129
        const orc_volume& v = s->volumes[s->materials[p.hit_volume].index];
        f3 wi = is.wi;
        float pdf = incident_pdf(is);
        shadeLe = mk(0, 0, 0);
        shadeT = ld3(v.R) / kFourPiF / pdf;
        p.ro = p.ro + p.rd * p.tmin;
        p.rd = wi;
    } else if (mq == kMatSpecular) {  // delta_materials.cl:34-64
        f3 Ng = p.Ng;
        f3 wo = -p.rd;
        if (dot(Ng, wo) < 0.0f) Ng = -Ng;
        f3 wi = reflect(p.rd, Ng);
        shadeLe = mk(0, 0, 0);
        shadeT = mk(1, 1, 1);
        p.ro = p.ro + p.rd * p.tmin + wi * 1.0e-5f;
        p.rd = wi;
    } else if (mq == kMatDielectric) {  // delta_materials.cl:66-121
        f3 Ng = p.Ng;
        f3 wo = -p.rd;
        bool backside = dot(Ng, wo) < 0.0f;
        float eta_i = 1.0f, eta_t = 1.5f;
        if (backside) {
            float e = eta_i;
            eta_i = eta_t;
            eta_t = e;
        }
        if (backside) Ng = -Ng;
        float f = fresnel_dielectrics(fabs_(dot(Ng, wo)), eta_t, eta_i);
        float u = p.rng.uniform();
        float rc = 1.0f;
        f3 wi;
        if (u < f) {
            wi = reflect(p.rd, Ng);
        } else {
            if (!refract(&wi, p.rd, Ng, eta_i, eta_t)) {
                wi = reflect(p.rd, Ng);
            } else {
                rc = sqr(eta_t / eta_i);
            }
        }
        shadeLe = mk(0, 0, 0);
        shadeT = mk(rc, rc, rc);
        p.ro = p.ro + p.rd * p.tmin + wi * 1.0e-5f;
        p.rd = wi;
    }

    // homogeneous_volume_through, homogeneous_volume_through.cl:7-44
    {
        p.hit_surface = -1;
        int hv = -1;
        if (0 < p.vol_count) {
            uint64_t u = p.rng.uniform_integer();
            hv = p.vols[u % (uint64_t)p.vol_count];
        }
        p.hit_volume = hv;
        float tmin = FLT_MAX;
        if (0 <= hv) {
            const orc_volume& v = s->volumes[s->materials[hv].index];
            float u = p.rng.uniform();
            tmin = -1.0f / v.C * log_(u);
        }
        p.tmin = tmin;
    }
    // extension_ray_cast, extension_ray_cast_stackless.cl:202-246
    {
        float t;
        int32_t prim;
        if (intersect_bvh(s, p.ro, p.rd, p.tmin, &t, &prim, nullptr, nullptr)) {
            p.Ng = hit_normal(s, prim, p.ro, p.rd, t);
            p.hit_surface = prim;
            p.tmin = t;
            p.hit_volume = -1;
        }
    }
    // logic, logic.cl:27-190
    {
        uint32_t logic_i = p.logic_i++;
        f3 L = p.L, T = p.T;
        L = L + T * shadeLe;
        T = T * shadeT;
        bool evalEnv, newPath;
        if (p.hit_surface < 0 && p.hit_volume < 0) {
            newPath = true;
            evalEnv = true;
        } else {
            newPath = false;
            evalEnv = false;
        }
        float luminanceT = 0.2126f * T.x + 0.7152f * T.y + 0.0722f * T.z;
        float cp = 1.0f;
        if ((int64_t)c.cfg->rr_depth < (int64_t)logic_i) cp = fmin_(luminanceT, 1.0f);
        float u = p.rng.uniform();
        if (u < cp) {
            T = T / cp;
        } else {
            newPath = true;
        }
        if (luminanceT < 1.0e-5f) newPath = true;
        if (evalEnv && c.has_env) {
            f3 e = get_envmap_value(s, p.rd, logic_i == 0);
            L = L + T * e;
        }
        // max-depth extension: terminate after segment max_depth, adding the
        // emission the next material stage would have added.
        if (c.cfg->max_depth > 0 && !newPath && (int64_t)logic_i >= (int64_t)c.cfg->max_depth) {
            if (0 <= p.hit_surface) {
                const orc_material& m = s->materials[p.hit_surface];
                f3 Le = mk(0, 0, 0);
                if (m.type == kMatLambertian) Le = ld3(s->lambertians[m.index].Le);
                L = L + T * Le;
            }
            newPath = true;
        }
        if (newPath) {
            float clampv = c.cfg->radiance_clamp;
            if (is_finite(L.x) && is_finite(L.y) && is_finite(L.z) && L.x < clampv && L.y < clampv &&
                L.z < clampv) {
                double* a = accum + 4 * (size_t)p.pixel_index;
                a[0] += (double)L.x;
                a[1] += (double)L.y;
                a[2] += (double)L.z;
                a[3] += 1.0;
            }
        }
        p.L = L;
        p.T = T;
        if (newPath) {
            p.queue = 0;
        } else if (0 <= p.hit_surface) {
            p.queue = s->materials[p.hit_surface].type;
        } else {
            p.queue = kMatVolumeInside;
        }
    }
}

void dump_slot(const Slot& p, orc_slot* o) {
    st3(o->T, p.T);
    st3(o->L, p.L);
    st3(o->ro, p.ro);
    st3(o->rd, p.rd);
    o->logic_i = p.logic_i;
    o->pixel_index = p.pixel_index;
    memcpy(o->rng, p.rng.s, 16);
    o->hit_surface = p.hit_surface;
    o->hit_volume = p.hit_volume;
    o->tmin = p.tmin;
    st3(o->Ng, p.Ng);
    o->queue = p.queue;
    o->vol_count = p.vol_count;
    memcpy(o->vols, p.vols, sizeof(o->vols));
}

// half conversion with round-to-nearest-even (vstore_half / vload_half)
uint16_t f2h(float f) {
    uint32_t x = as_uint(f);
    uint32_t sign = (x >> 16) & 0x8000u;
    uint32_t ax = x & 0x7fffffffu;
    if (ax > 0x7f800000u) return (uint16_t)(sign | 0x7e00u);
    if (ax >= 0x477ff000u) return (uint16_t)(sign | 0x7c00u);  // rounds to inf
    if (ax < 0x38800000u) {                                    // half sub-normal or zero
        if (ax < 0x33000000u) return (uint16_t)sign;           // < 2^-25 rounds to 0
        uint32_t e = ax >> 23;
        uint32_t m = (ax & 0x7fffffu) | 0x800000u;
        uint32_t shift = 126 - e;  // 14 + (113 - e) - 1
        uint32_t q = m >> shift;
        uint32_t rem = m & ((1u << shift) - 1);
        uint32_t half = 1u << (shift - 1);
        if (rem > half || (rem == half && (q & 1))) q++;
        return (uint16_t)(sign | q);
    }
    uint32_t e = (ax >> 23) - 112;
    uint32_t m = ax & 0x7fffffu;
    uint32_t q = (e << 10) | (m >> 13);
    uint32_t rem = m & 0x1fffu;
    if (rem > 0x1000u || (rem == 0x1000u && (q & 1))) q++;
    return (uint16_t)(sign | q);
}
float h2f(uint16_t h) {
    uint32_t sign = (uint32_t)(h & 0x8000u) << 16;
    uint32_t e = (h >> 10) & 0x1fu;
    uint32_t m = h & 0x3ffu;
    if (e == 0) {
        float v = (float)m * 5.9604644775390625e-08f;  // m * 2^-24, exact
        return sign ? -v : v;
    }
    if (e == 31) return as_float(sign | 0x7f800000u | (m << 13));
    return as_float(sign | ((e + 112) << 23) | (m << 13));
}

}  // namespace

// ============================================================== C API
extern "C" {

void orc_random_initialize(uint32_t* states, uint64_t n, uint64_t seed_offset) {
    for (uint64_t i = 0; i < n; ++i) random_initialize_one(states + 4 * i, seed_offset + i);
}
void orc_random_uniform(uint32_t* state4, float* out, int32_t n) {
    Rng r;
    memcpy(r.s, state4, 16);
    for (int i = 0; i < n; ++i) out[i] = r.uniform();
    memcpy(state4, r.s, 16);
}
void orc_random_uniform_integer(uint32_t* state4, uint64_t* out, int32_t n) {
    Rng r;
    memcpy(r.s, state4, 16);
    for (int i = 0; i < n; ++i) out[i] = r.uniform_integer();
    memcpy(state4, r.s, 16);
}

void orc_trace(const orc_scene* s, const float* rays, uint64_t n, int32_t* prim, float* t,
               float* ng, uint32_t* node_visits, uint32_t* prim_tests, int32_t nthreads) {
    auto trace_range = [&](uint64_t beg, uint64_t end) {
        for (uint64_t i = beg; i < end; ++i) {
            const float* r = rays + 8 * i;
            f3 ro = ld3(r), rd = ld3(r + 4);
            float tt;
            int32_t pp;
            uint32_t nv = 0, nt = 0;
            bool hit = intersect_bvh(s, ro, rd, r[3], &tt, &pp, &nv, &nt);
            prim[i] = hit ? pp : -1;
            t[i] = hit ? tt : r[3];
            if (ng) {
                f3 n = hit ? hit_normal(s, pp, ro, rd, tt) : mk(0, 0, 0);
                st3(ng + 3 * i, n);
            }
            if (node_visits) node_visits[i] = nv;
            if (prim_tests) prim_tests[i] = nt;
        }
    };
    if (nthreads <= 1 || n < 4096) {
        trace_range(0, n);
        return;
    }
    // threads take chunks of 4096 rays from a shared counter: coherent and
    // incoherent rays cost very different amounts, so static halves would idle
    std::atomic<uint64_t> next{0};
    auto worker = [&]() {
        for (;;) {
            uint64_t b = next.fetch_add(4096);
            if (b >= n) return;
            trace_range(b, std::min<uint64_t>(n, b + 4096));
        }
    };
    std::vector<std::thread> th;
    for (int k = 0; k < nthreads; ++k) th.emplace_back(worker);
    for (auto& x : th) x.join();
}

// ImageEnvmap constructor (envmap.hpp:160-242) for one direction weight, and
// AliasMethod::prepare (alias_method.hpp:47-114) with its Kahan sums.
static void build_one_table(const float* rgba, int w, int h, int weight_kind, const double* frag_d,
                            const double* sr, float* pdf_out, float* height_out, int32_t* alias_out) {
    const double two_pi = 6.28318530717958647692;
    int N = w * h;
    std::vector<double> weights(N);
    for (int y = 0; y < h; ++y) {
        const double* af = frag_d + 4 * (size_t)y * w;
        double theta = (std::acos(af[0]) + std::acos(af[1])) * 0.5;
        for (int x = 0; x < w; ++x) {
            int index = y * w + x;
            const double* f = frag_d + 4 * (size_t)index;
            double phi = (f[2] + f[3]) * 0.5;
            // polar_to_cartesian (envmap.hpp:79-86) returns (y, z, x)
            double st = std::sin(theta);
            double dx = st * std::sin(phi), dy = std::cos(theta), dz = st * std::cos(phi);
            const float* rad = rgba + 4 * (size_t)index;
            float Y = 0.2126f * rad[0] + 0.7152f * rad[1] + 0.0722f * rad[2];
            double dw = 1.0;  // UniformDirectionWeight / SixAxisDirectionWeight (envmap.hpp:144-149, 291-312)
            switch (weight_kind) {
                case 1: dw = std::max(dx, 0.0); break;
                case 2: dw = std::max(-dx, 0.0); break;
                case 3: dw = std::max(dy, 0.0); break;
                case 4: dw = std::max(-dy, 0.0); break;
                case 5: dw = std::max(dz, 0.0); break;
                case 6: dw = std::max(-dz, 0.0); break;
                default: break;
            }
            weights[index] = (double)Y * sr[y] * dw;
        }
    }
    // AliasMethod::prepare
    double ksum = 0.0, kc = 0.0;  // Kahan
    for (double v : weights) {
        double yv = v - kc;
        double t = ksum + yv;
        kc = (t - ksum) - yv;
        ksum = t;
    }
    double one_over = 1.0 / (ksum - kc);
    std::vector<double> probs(N), hs(N), hc(N, 0.0);
    std::vector<int32_t> alias(N, -1);
    for (int i = 0; i < N; ++i) {
        probs[i] = weights[i] * one_over;
        hs[i] = probs[i] * N;
    }
    auto hget = [&](int i) { return hs[i] - hc[i]; };
    std::vector<int> lower, upper;
    lower.reserve(N);
    upper.reserve(N);
    for (int i = 0; i < N; ++i) {
        if (hget(i) < 1.0) lower.push_back(i);
        else upper.push_back(i);
    }
    while (!lower.empty() && !upper.empty()) {
        int li = lower.back();
        lower.pop_back();
        int ui = upper.back();
        upper.pop_back();
        double mov = 1.0 - hget(li);
        double x = -mov;  // Kahan sub
        double yv = x - hc[ui];
        double t = hs[ui] + yv;
        hc[ui] = (t - hs[ui]) - yv;
        hs[ui] = t;
        alias[li] = ui;
        if (hget(ui) < 1.0) lower.push_back(ui);
        else upper.push_back(ui);
    }
    for (int y = 0; y < h; ++y) {
        for (int x = 0; x < w; ++x) {
            int i = y * w + x;
            pdf_out[i] = (float)(probs[i] * (1.0 / sr[y]));
            height_out[i] = (float)hget(i);
            alias_out[i] = alias[i];
        }
    }
}

int32_t orc_envmap_build(const float* rgba, int32_t w, int32_t h, float* pdf, float* height,
                         int32_t* alias, float* frag) {
    if (w <= 0 || h <= 0) return -1;
    const double two_pi = 6.28318530717958647692;
    const double pi = 3.14159265358979323846;
    double phi_step = two_pi / w, theta_step = pi / h;
    int N = w * h;
    std::vector<double> frag_d(4 * (size_t)N);
    std::vector<double> sr(h);
    for (int y = 0; y < h; ++y) {
        double beg_theta = theta_step * y, end_theta = theta_step * (y + 1);
        double beg_y = std::cos(end_theta), end_y = std::cos(beg_theta);
        for (int x = 0; x < w; ++x) {
            double upper = two_pi - x * phi_step;
            double lower = two_pi - (x + 1) * phi_step;
            double* f = &frag_d[4 * ((size_t)y * w + x)];
            f[0] = beg_y;
            f[1] = end_y;
            f[2] = lower;
            f[3] = upper;
        }
        sr[y] = ((std::cos(beg_theta) - std::cos(end_theta)) * two_pi) / w;
    }
    for (int i = 0; i < 4 * N; ++i) frag[i] = (float)frag_d[i];
    std::vector<std::thread> th;
    for (int k = 0; k < 7; ++k) {
        th.emplace_back(build_one_table, rgba, w, h, k, frag_d.data(), sr.data(), pdf + (size_t)k * N,
                        height + (size_t)k * N, alias + (size_t)k * N);
    }
    for (auto& x : th) x.join();
    return 0;
}

// One pool of npaths slots serving nreq requests in order: request r owns the
// global sample indices [begin[r], end[r]); a new path takes the request
// whose range holds its index (the single-request render is nreq = 1).
static uint64_t render_impl(const Ctx* ctxs, const uint64_t* begin, const uint64_t* end, int nreq,
                            uint32_t seed_offset, uint64_t limit, uint32_t npaths, int32_t steps,
                            double* const* accums, orc_slot* slots_out, int32_t nthreads) {
    std::vector<Slot> slots(npaths);
    for (uint32_t i = 0; i < npaths; ++i) {
        random_initialize_one(slots[i].rng.s, (uint64_t)seed_offset + i);
        slots[i].queue = 0;  // initialize_all_as_new_path (new_path.cl:9-15)
    }
    uint64_t next_pixel = 0;
    std::vector<uint64_t> gpix(npaths);
    std::vector<uint8_t> is_new(npaths);
    if (nthreads < 1) nthreads = 1;
    // per-thread private accumulators keep the sums deterministic
    std::vector<std::vector<std::vector<double>>> acc(nthreads);
    for (int k = 0; k < nthreads; ++k) {
        acc[k].resize(nreq);
        for (int r = 0; r < nreq; ++r)
            acc[k][r].assign(4 * (size_t)ctxs[r].cam->image_w * ctxs[r].cam->image_h, 0.0);
    }
    for (int st = 0; st < steps; ++st) {
        // new-path queue in slot order (new_path.cl:41-43, finalize_new_path :85-88)
        uint64_t rank = 0;
        for (uint32_t i = 0; i < npaths; ++i) {
            is_new[i] = 0;
            if (slots[i].queue != 0) continue;
            uint64_t g = next_pixel + rank;
            rank++;
            if (limit != 0 && g >= limit) {
                slots[i].queue = -1;  // idle: the sample budget is exhausted
                continue;
            }
            int r = 0;
            while (r + 1 < nreq && g >= end[r]) ++r;
            slots[i].req = r;
            is_new[i] = 1;
            gpix[i] = g - begin[r];
        }
        next_pixel += rank;
        auto work = [&](int k, uint32_t b, uint32_t e) {
            for (uint32_t i = b; i < e; ++i) {
                if (slots[i].queue < 0) continue;
                const int r = slots[i].req;
                step_slot(ctxs[r], slots[i], acc[k][r].data(), is_new[i] != 0, gpix[i]);
            }
        };
        if (nthreads == 1) {
            work(0, 0, npaths);
        } else {
            std::vector<std::thread> th;
            uint32_t chunk = (npaths + nthreads - 1) / nthreads;
            for (int k = 0; k < nthreads; ++k) {
                uint32_t b = k * chunk, e = std::min<uint32_t>(npaths, b + chunk);
                if (b < e) th.emplace_back(work, k, b, e);
            }
            for (auto& x : th) x.join();
        }
    }
    for (int r = 0; r < nreq; ++r) {
        size_t n4 = 4 * (size_t)ctxs[r].cam->image_w * ctxs[r].cam->image_h;
        memset(accums[r], 0, sizeof(double) * n4);
        for (int k = 0; k < nthreads; ++k)
            for (size_t i = 0; i < n4; ++i) accums[r][i] += acc[k][r][i];
    }
    if (slots_out)
        for (uint32_t i = 0; i < npaths; ++i) dump_slot(slots[i], slots_out + i);
    return next_pixel;
}

uint64_t orc_render(const orc_scene* s, const orc_camera* cam, const orc_config* cfg, uint32_t npaths,
                    int32_t steps, double* accum, orc_slot* slots_out, int32_t nthreads) {
    Ctx c{s, cam, cfg, s->env_rgba != nullptr && s->env_w > 0};
    uint64_t begin = 0, end = cfg->sample_limit ? cfg->sample_limit : ~0ull;
    double* accs[1] = {accum};
    return render_impl(&c, &begin, &end, 1, cfg->seed_offset, cfg->sample_limit, npaths, steps, accs, slots_out,
                       nthreads);
}

uint64_t orc_render_batch(const orc_scene* const* scenes, const orc_camera* cams, const orc_config* cfgs,
                          const uint64_t* begin, const uint64_t* end, int32_t nreq, uint32_t npaths, int32_t steps,
                          double* const* accums, orc_slot* slots_out, int32_t nthreads) {
    std::vector<Ctx> ctxs(nreq);
    for (int r = 0; r < nreq; ++r)
        ctxs[r] = Ctx{scenes[r], cams + r, cfgs + r, scenes[r]->env_rgba != nullptr && scenes[r]->env_w > 0};
    return render_impl(ctxs.data(), begin, end, nreq, cfgs[0].seed_offset, end[nreq - 1], npaths, steps, accums,
                       slots_out, nthreads);
}

// accumlation_to_intermediate (accumlation.cl:6-25) on FP64 sums: mean in
// double, rounded to float, then to half; count truncated to 16 bits.
void orc_intermediate(const double* accum, uint64_t npix, uint16_t* out) {
    for (uint64_t i = 0; i < npix; ++i) {
        const double* a = accum + 4 * i;
        double cnt = a[3];
        for (int k = 0; k < 3; ++k) {
            float m = cnt > 0.0 ? (float)(a[k] / cnt) : 0.0f;
            out[4 * i + k] = f2h(m);
        }
        out[4 * i + 3] = (uint16_t)((uint64_t)cnt & 0xffffu);
    }
}
// tonemap, accumlation.cl:68-79
void orc_tonemap(const uint16_t* in, uint64_t npix, uint8_t* rgba8) {
    for (uint64_t i = 0; i < npix; ++i) {
        for (int k = 0; k < 3; ++k) {
            float c = h2f(in[4 * i + k]);
            int v = to_int(pow_(c * 1.0f, 1.0f / 2.2f) * 256.0f);
            v = std::min(std::max(v, 0), 255);
            rgba8[4 * i + k] = (uint8_t)v;
        }
        rgba8[4 * i + 3] = 255;
    }
}
uint16_t orc_float_to_half(float f) { return f2h(f); }
float orc_half_to_float(uint16_t h) { return h2f(h); }

void orc_cosine_hemisphere(float a, float b, float* out3) { st3(out3, cosine_weighted_hemisphere_z_up(a, b)); }
void orc_uniform_sphere(float u0, float u1, float* out3) { st3(out3, uniform_on_unit_sphere(u0, u1)); }
void orc_sample_from_fragment(const float* frag4, uint32_t* state4, float* out3) {
    Rng r;
    memcpy(r.s, state4, 16);
    st3(out3, sample_from_fragment(frag4, &r));
    memcpy(state4, r.s, 16);
}
void orc_orthonormal_basis(const float* z3, float* x3, float* y3) {
    f3 x, y;
    get_orthonormal_basis(ld3(z3), &x, &y);
    st3(x3, x);
    st3(y3, y);
}
void orc_sample_ward(const float* wo3, const float* z3, float alpha, float u0, float u1, float* wi3) {
    st3(wi3, sample_ward(ld3(wo3), ld3(z3), alpha, u0, u1));
}
float orc_pdf_ward(const float* wo3, const float* wi3, const float* z3, float alpha) {
    return pdf_ward(ld3(wo3), ld3(wi3), ld3(z3), alpha);
}
void orc_envmap_value(const orc_scene* s, const float* rd3, int32_t filter, float* out3) {
    st3(out3, get_envmap_value(s, ld3(rd3), filter != 0));
}
int32_t orc_envmap_index(const float* wi3, int32_t w, int32_t h) { return envmap_index(ld3(wi3), w, h); }
void orc_envmap_filter_compare(const orc_scene* s, const float* rd3, uint64_t n, int32_t frac_bits, float* exact3,
                               float* quant3) {
    const float pi = kPiF;
    for (uint64_t i = 0; i < n; ++i) {
        float theta, phi;
        cartesian_to_polar(ld3(rd3 + 3 * i), &theta, &phi);
        st3(exact3 + 3 * i, get_envmap_value(s, ld3(rd3 + 3 * i), true));
        st3(quant3 + 3 * i, read_image_repeat_quantized(s, 1.0f - phi / (2.0f * pi), theta / pi, frac_bits));
    }
}

float orc_fm(int32_t fn, float x, float y) {
    switch (fn) {
        case 0: return sin_(x);
        case 1: return cos_(x);
        case 2: return log_(x);
        case 3: return exp_(x);
        case 4: return atan_(x);
        case 5: return atan2_(x, y);
        case 6: return pow_(x, y);
        default: return 0.0f;
    }
}

}  // extern "C"

// ------------------------------------------------------------ tree build
// The reference builds a binary tree with Embree (rtcBuildBVH, RTC_BUILD_QUALITY_HIGH,
// maxBranchingFactor 2, leaves of 1..5 primitives, Embree's default SAH costs;
// common/stackless_bvh.hpp:108-130) and flattens it with create_stackless_bvh
// (stackless_bvh.hpp:283-341).  Embree is not vendored, so a plain binned SAH stands in
// for it here (node visit and primitive test priced 1 : 1, as Embree's defaults), and
// the flattening follows the reference: node indices in preorder (left subtree first,
// allocate_stacklessBVH), each child's sibling link pointing at the other child, the
// root's parent and sibling links 0, and each leaf's primitive ids appended to one list
// in that same preorder (build_stacklessBVH).  Leaves are the nodes with
// primitive_indices_end > 0, as the traversal tells them apart.
// This builder exists so that the reference arm of the benchmark can run without the
// product library; closest hits do not depend on the tree except for exact ties.
namespace {

struct BuildPrim {
    float lo[3], hi[3], c[3];
    uint32_t id;
};

struct BuildNode {
    float lo[3], hi[3];
    std::unique_ptr<BuildNode> L, R;
    uint32_t beg = 0, end = 0;  // leaf: range into the primitive array
    bool leaf = false;
};

inline float half_area(const float* lo, const float* hi) {
    float dx = hi[0] - lo[0], dy = hi[1] - lo[1], dz = hi[2] - lo[2];
    return dx * dy + dy * dz + dz * dx;
}

struct Builder {
    std::vector<BuildPrim>& prims;
    int max_leaf;
    int bins;
    int spawn_depth;

    std::unique_ptr<BuildNode> build(uint32_t b, uint32_t e, int depth) {
        auto node = std::make_unique<BuildNode>();
        float clo[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, chi[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
        for (int a = 0; a < 3; ++a) {
            node->lo[a] = FLT_MAX;
            node->hi[a] = -FLT_MAX;
        }
        for (uint32_t i = b; i < e; ++i) {
            const BuildPrim& p = prims[i];
            for (int a = 0; a < 3; ++a) {
                node->lo[a] = std::min(node->lo[a], p.lo[a]);
                node->hi[a] = std::max(node->hi[a], p.hi[a]);
                clo[a] = std::min(clo[a], p.c[a]);
                chi[a] = std::max(chi[a], p.c[a]);
            }
        }
        uint32_t n = e - b;
        if (n == 1) {
            node->leaf = true;
            node->beg = b;
            node->end = e;
            return node;
        }
        // binned SAH over the centroid bounds: cost = 1 + (A_L N_L + A_R N_R) / A
        int best_axis = -1, best_bin = -1;
        float best_cost = FLT_MAX;
        const float parent_area = half_area(node->lo, node->hi);
        std::vector<float> blo(3 * bins), bhi(3 * bins), rarea(bins);
        std::vector<uint32_t> bcount(bins), rcount(bins);
        for (int a = 0; a < 3; ++a) {
            float extent = chi[a] - clo[a];
            if (!(extent > 0.0f)) continue;
            float scale = (float)bins / extent;
            std::fill(bcount.begin(), bcount.end(), 0u);
            for (int k = 0; k < bins; ++k)
                for (int c = 0; c < 3; ++c) {
                    blo[3 * k + c] = FLT_MAX;
                    bhi[3 * k + c] = -FLT_MAX;
                }
            for (uint32_t i = b; i < e; ++i) {
                const BuildPrim& p = prims[i];
                int k = std::min(bins - 1, (int)((p.c[a] - clo[a]) * scale));
                bcount[k]++;
                for (int c = 0; c < 3; ++c) {
                    blo[3 * k + c] = std::min(blo[3 * k + c], p.lo[c]);
                    bhi[3 * k + c] = std::max(bhi[3 * k + c], p.hi[c]);
                }
            }
            // right sweep: area and count of bins k..bins-1
            float rlo[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, rhi[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
            uint32_t rc = 0;
            for (int k = bins - 1; k >= 1; --k) {
                rc += bcount[k];
                for (int c = 0; c < 3; ++c) {
                    rlo[c] = std::min(rlo[c], blo[3 * k + c]);
                    rhi[c] = std::max(rhi[c], bhi[3 * k + c]);
                }
                rcount[k] = rc;
                rarea[k] = rc ? half_area(rlo, rhi) : 0.0f;
            }
            float llo[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, lhi[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
            uint32_t lc = 0;
            for (int k = 1; k < bins; ++k) {  // split between bin k-1 and bin k
                lc += bcount[k - 1];
                for (int c = 0; c < 3; ++c) {
                    llo[c] = std::min(llo[c], blo[3 * (k - 1) + c]);
                    lhi[c] = std::max(lhi[c], bhi[3 * (k - 1) + c]);
                }
                if (lc == 0 || rcount[k] == 0) continue;
                float cost = 1.0f + (half_area(llo, lhi) * (float)lc + rarea[k] * (float)rcount[k]) / parent_area;
                if (cost < best_cost) {
                    best_cost = cost;
                    best_axis = a;
                    best_bin = k;
                }
            }
        }
        if (n <= (uint32_t)max_leaf && (best_axis < 0 || (float)n <= best_cost)) {
            node->leaf = true;
            node->beg = b;
            node->end = e;
            return node;
        }
        uint32_t mid;
        if (best_axis >= 0 && depth < 56) {
            float extent = chi[best_axis] - clo[best_axis];
            float scale = (float)bins / extent;
            auto it = std::partition(prims.begin() + b, prims.begin() + e, [&](const BuildPrim& p) {
                return std::min(bins - 1, (int)((p.c[best_axis] - clo[best_axis]) * scale)) < best_bin;
            });
            mid = (uint32_t)(it - prims.begin());
        } else {
            // all centroids equal (or the tree is too deep for the traversal's 64-bit bit
            // stack): split the range at its middle, ordered along the widest axis
            int a = 0;
            for (int c = 1; c < 3; ++c)
                if (chi[c] - clo[c] > chi[a] - clo[a]) a = c;
            mid = b + n / 2;
            std::nth_element(prims.begin() + b, prims.begin() + mid, prims.begin() + e,
                             [&](const BuildPrim& x, const BuildPrim& y) {
                                 return x.c[a] < y.c[a] || (x.c[a] == y.c[a] && x.id < y.id);
                             });
        }
        if (mid == b || mid == e) mid = b + n / 2;
        if (depth < spawn_depth && n > 65536) {
            std::unique_ptr<BuildNode> right;
            std::thread th([&]() { right = build(mid, e, depth + 1); });
            node->L = build(b, mid, depth + 1);
            th.join();
            node->R = std::move(right);
        } else {
            node->L = build(b, mid, depth + 1);
            node->R = build(mid, e, depth + 1);
        }
        return node;
    }
};

uint64_t count_nodes(const BuildNode* n) { return n->leaf ? 1 : 1 + count_nodes(n->L.get()) + count_nodes(n->R.get()); }

// allocate_stacklessBVH + build_stacklessBVH (stackless_bvh.hpp:283-326)
uint32_t flatten(const BuildNode* n, const std::vector<BuildPrim>& prims, orc_node* nodes, uint32_t* prim_ids,
                 uint32_t* next_node, uint32_t* next_prim, uint32_t parent, bool has_parent) {
    uint32_t me = (*next_node)++;
    orc_node& o = nodes[me];
    memset(&o, 0, sizeof(o));
    if (has_parent) o.link_parent = parent;
    if (!n->leaf) {
        uint32_t L = flatten(n->L.get(), prims, nodes, prim_ids, next_node, next_prim, me, true);
        uint32_t R = flatten(n->R.get(), prims, nodes, prim_ids, next_node, next_prim, me, true);
        orc_node& p = nodes[me];
        p.link_L = L;
        p.link_R = R;
        for (int a = 0; a < 3; ++a) {
            p.L_lower[a] = n->L->lo[a];
            p.L_upper[a] = n->L->hi[a];
            p.R_lower[a] = n->R->lo[a];
            p.R_upper[a] = n->R->hi[a];
        }
        nodes[L].link_sibling = R;
        nodes[R].link_sibling = L;
    } else {
        o.primitive_indices_beg = *next_prim;
        for (uint32_t i = n->beg; i < n->end; ++i) prim_ids[(*next_prim)++] = prims[i].id;
        o.primitive_indices_end = *next_prim;
    }
    return me;
}

}  // namespace

extern "C" int64_t orc_build_bvh(const float* points4, const uint32_t* indices, uint32_t ntris, const float* spheres4,
                                 uint32_t nspheres, int32_t max_leaf, int32_t bins, int32_t nthreads, orc_node* nodes,
                                 uint64_t node_cap, uint32_t* prim_ids, uint64_t prim_cap) {
    uint64_t nprim = (uint64_t)ntris + nspheres;
    if (nprim == 0 || max_leaf < 1 || max_leaf > 5 || bins < 2 || prim_cap < nprim) return -1;
    std::vector<BuildPrim> prims(nprim);
    for (uint64_t i = 0; i < ntris; ++i) {
        BuildPrim& p = prims[i];
        p.id = (uint32_t)i;
        for (int a = 0; a < 3; ++a) {
            float v0 = points4[4 * (size_t)indices[3 * i] + a], v1 = points4[4 * (size_t)indices[3 * i + 1] + a],
                  v2 = points4[4 * (size_t)indices[3 * i + 2] + a];
            p.lo[a] = std::min(v0, std::min(v1, v2));
            p.hi[a] = std::max(v0, std::max(v1, v2));
        }
    }
    for (uint64_t k = 0; k < nspheres; ++k) {
        BuildPrim& p = prims[ntris + k];
        p.id = (uint32_t)(ntris + k);
        for (int a = 0; a < 3; ++a) {
            p.lo[a] = spheres4[4 * k + a] - spheres4[4 * k + 3];
            p.hi[a] = spheres4[4 * k + a] + spheres4[4 * k + 3];
        }
    }
    for (auto& p : prims)
        for (int a = 0; a < 3; ++a) p.c[a] = (p.lo[a] + p.hi[a]) * 0.5f;
    int spawn = 0;
    while ((1 << spawn) < std::max(1, nthreads)) ++spawn;
    Builder bld{prims, max_leaf, bins, spawn};
    std::unique_ptr<BuildNode> root = bld.build(0, (uint32_t)nprim, 0);
    uint64_t nn = count_nodes(root.get());
    if (nodes == nullptr || node_cap < nn) return (int64_t)nn;  // size query
    uint32_t next_node = 0, next_prim = 0;
    flatten(root.get(), prims, nodes, prim_ids, &next_node, &next_prim, 0, false);
    return (int64_t)nn;
}
