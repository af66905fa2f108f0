// clshim_body.h — OpenCL C built-ins for compiling the reference kernels
// (kernels/*.cl) unchanged, as C++, on the host.  Test infrastructure only.
//
// Included INSIDE a per-translation-unit namespace, immediately before a
// reference .cl file, so each .cl file gets its own copy of these types and
// functions (the reference reuses helper names such as sqr() and
// get_orthonormal_basis() across files).
//
// Limitation: an OpenCL vector literal with several components, e.g.
// (float3)(a, b, c), parses in C++ as a cast of the comma expression and
// yields (c, c, c).  Literals with a single component, (float3)(1.0f), and
// those whose components are all equal, are correct.  Only reference
// functions free of multi-component literals are called through this shim;
// the list is in oracle/ref/ref_kernels.cpp.
//
// The float built-ins (sin, cos, log, exp, atan, atan2, pow, min, max) are
// the deterministic definitions of rgr_fmath.h, the ones the oracle and the
// CUDA kernels use, so outputs are comparable bit for bit.

typedef unsigned int uint;
typedef unsigned long ulong;
typedef unsigned short ushort;
typedef unsigned char uchar;
typedef unsigned short half;

struct int3 {
    int x, y, z, w_;
};
struct float2 {
    float x, y;
    float2() : x(0), y(0) {}
    float2(float s) : x(s), y(s) {}
};
struct alignas(16) float3 {
    float x, y, z, w_;  // 16 bytes, as OpenCL float3
    float3() : x(0), y(0), z(0), w_(0) {}
    float3(float s) : x(s), y(s), z(s), w_(0) {}
    float3(float a, float b, float c) : x(a), y(b), z(c), w_(0) {}
};
struct alignas(16) float4 {
    union {
        struct {
            float x, y, z, w;
        };
        float3 xyz;
    };
    float4() : x(0), y(0), z(0), w(0) {}
};
struct uint2 {
    uint x, y;
};
struct alignas(16) uint4 {
    uint x, y, z, w;
    uint4() : x(0), y(0), z(0), w(0) {}
    uint4(uint s) : x(s), y(s), z(s), w(s) {}
};
struct uchar4 {
    uchar x, y, z, w;
};
struct int4b {
    int x, y, z, w;
};
inline int4b operator==(uint4 a, uint4 b) {
    return int4b{a.x == b.x ? -1 : 0, a.y == b.y ? -1 : 0, a.z == b.z ? -1 : 0, a.w == b.w ? -1 : 0};
}
inline int all(int4b c) { return (c.x < 0) && (c.y < 0) && (c.z < 0) && (c.w < 0); }
inline int all(int3 c) { return (c.x < 0) && (c.y < 0) && (c.z < 0); }

inline float3 operator+(float3 a, float3 b) { return float3(a.x + b.x, a.y + b.y, a.z + b.z); }
inline float3 operator-(float3 a, float3 b) { return float3(a.x - b.x, a.y - b.y, a.z - b.z); }
inline float3 operator*(float3 a, float3 b) { return float3(a.x * b.x, a.y * b.y, a.z * b.z); }
inline float3 operator/(float3 a, float3 b) { return float3(a.x / b.x, a.y / b.y, a.z / b.z); }
inline float3 operator*(float3 a, float s) { return float3(a.x * s, a.y * s, a.z * s); }
inline float3 operator*(float s, float3 a) { return float3(s * a.x, s * a.y, s * a.z); }
inline float3 operator/(float3 a, float s) { return float3(a.x / s, a.y / s, a.z / s); }
inline float3 operator-(float3 a) { return float3(-a.x, -a.y, -a.z); }
inline float3& operator+=(float3& a, float3 b) { a = a + b; return a; }
inline float3& operator*=(float3& a, float3 b) { a = a * b; return a; }
inline float3& operator/=(float3& a, float s) { a = a / s; return a; }
inline int3 operator<(float3 a, float3 b) {
    return int3{a.x < b.x ? -1 : 0, a.y < b.y ? -1 : 0, a.z < b.z ? -1 : 0, 0};
}

inline float dot(float3 a, float3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline float3 cross(float3 a, float3 b) {
    return float3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
inline float sqrt(float x) { return ::rgr::fm::sqrt_(x); }
inline float3 normalize(float3 v) {
    float l = sqrt(dot(v, v));
    return float3(v.x / l, v.y / l, v.z / l);
}
inline float fabs(float x) { return ::rgr::fm::fabs_(x); }
inline float copysign(float x, float y) { return ::rgr::fm::copysign_(x, y); }
inline float floor(float x) { return ::rgr::fm::floor_(x); }
inline float sin(float x) { return ::rgr::fm::sin_(x); }
inline float cos(float x) { return ::rgr::fm::cos_(x); }
inline float log(float x) { return ::rgr::fm::log_(x); }
inline float exp(float x) { return ::rgr::fm::exp_(x); }
inline float atan(float x) { return ::rgr::fm::atan_(x); }
inline float atan2(float y, float x) { return ::rgr::fm::atan2_(y, x); }
inline float pow(float x, float y) { return ::rgr::fm::pow_(x, y); }
inline float min(float a, float b) { return ::rgr::fm::fmin_(a, b); }
inline float max(float a, float b) { return ::rgr::fm::fmax_(a, b); }
inline float3 min(float3 a, float3 b) { return float3(min(a.x, b.x), min(a.y, b.y), min(a.z, b.z)); }
inline float3 max(float3 a, float3 b) { return float3(max(a.x, b.x), max(a.y, b.y), max(a.z, b.z)); }
inline int min(int a, int b) { return b < a ? b : a; }
inline int max(int a, int b) { return a < b ? b : a; }
inline int clamp(int x, int lo, int hi) { return min(max(x, lo), hi); }
inline float mix(float a, float b, float t) { return a + (b - a) * t; }
inline float3 mix(float3 a, float3 b, float t) { return float3(mix(a.x, b.x, t), mix(a.y, b.y, t), mix(a.z, b.z, t)); }
inline int isnan(float x) { return ::rgr::fm::is_nan(x) ? 1 : 0; }
inline int3 isnan(float3 v) {
    return int3{::rgr::fm::is_nan(v.x) ? -1 : 0, ::rgr::fm::is_nan(v.y) ? -1 : 0,
                ::rgr::fm::is_nan(v.z) ? -1 : 0, 0};
}
inline int isfinite(float x) { return ::rgr::fm::is_finite(x) ? 1 : 0; }
inline int3 isfinite(float3 v) {
    return int3{::rgr::fm::is_finite(v.x) ? -1 : 0, ::rgr::fm::is_finite(v.y) ? -1 : 0,
                ::rgr::fm::is_finite(v.z) ? -1 : 0, 0};
}
inline float3 select(float3 a, float3 b, int3 c) {
    return float3(c.x < 0 ? b.x : a.x, c.y < 0 ? b.y : a.y, c.z < 0 ? b.z : a.z);
}
inline float as_float(uint u) { return ::rgr::fm::as_float(u); }
inline uint as_uint(float f) { return ::rgr::fm::as_uint(f); }

// work-item functions: one work-item per work-group, driven by the harness
inline size_t get_global_id(int) { return ::rgr_cl_gid; }
inline size_t get_local_id(int) { return 0; }
inline size_t get_global_size(int) { return ::rgr_cl_gsize; }
inline size_t get_local_size(int) { return 1; }
enum { CLK_LOCAL_MEM_FENCE = 1, CLK_GLOBAL_MEM_FENCE = 2 };
inline void barrier(int) {}
inline uint atomic_inc(volatile uint* p) { uint o = *p; *p = o + 1; return o; }
inline uint atomic_add(volatile uint* p, uint v) { uint o = *p; *p = o + v; return o; }
inline uint atom_add(volatile uint* p, uint v) { return atomic_add(p, v); }
inline uint atomic_cmpxchg(volatile uint* p, uint cmp, uint val) {
    uint o = *p;
    if (o == cmp) *p = val;
    return o;
}
inline int atomic_cmpxchg(volatile int* p, int cmp, int val) {
    int o = *p;
    if (o == cmp) *p = val;
    return o;
}
inline int atomic_xchg(volatile int* p, int val) { int o = *p; *p = val; return o; }

// half conversions (round to nearest even), defined by the oracle
inline void vstore_half(float v, size_t off, half* p) { p[off] = orc_float_to_half(v); }
inline float vload_half(size_t off, const half* p) { return orc_half_to_float(p[off]); }

// images: the harness supplies a constant-radiance image (coordinates ignored)
struct cl_image {
    float value[4];
};
typedef const cl_image* image2d_t;
typedef int sampler_t;
enum {
    CLK_NORMALIZED_COORDS_TRUE = 1, CLK_ADDRESS_REPEAT = 2, CLK_FILTER_NEAREST = 4, CLK_FILTER_LINEAR = 8
};
inline float4 read_imagef(image2d_t img, sampler_t, float2) {
    float4 r;
    r.x = img->value[0];
    r.y = img->value[1];
    r.z = img->value[2];
    r.w = img->value[3];
    return r;
}
