/* rgr_oracle.h — C interface of the CPU oracle (test infrastructure only).
 *
 * The oracle is a single-threaded-per-path C++ restatement of the reference
 * OpenCL wavefront path tracer (kernels/*.cl and the host table builders in
 * common/share/envmap.hpp, common/share/alias_method.hpp).  It is used only
 * by tests/, by __graft_entry__.smoke() and by bench.py's CPU baseline, as the
 * checker.  The product never links, loads or calls it.
 *
 * Layouts here are the reference layouts (float3 occupies 16 bytes, as
 * OpenCL float3 does), so that nodes exported by the product in the
 * reference StacklessBVHNode format (common/stackless_bvh.hpp:264-275) can
 * be traversed exactly as kernels/extension_ray_cast_stackless.cl does.
 */
#ifndef RGR_ORACLE_H
#define RGR_ORACLE_H
#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* reference StacklessBVHNode (stackless_bvh.hpp:264-275), 96 bytes */
typedef struct orc_node {
    float L_lower[4];
    float L_upper[4];
    float R_lower[4];
    float R_upper[4];
    uint32_t link_parent, link_L, link_R, link_sibling;
    uint32_t primitive_indices_beg, primitive_indices_end;
    uint32_t pad[2];
} orc_node;

typedef struct orc_material { int32_t type, index; } orc_material;       /* types.cl:73-76 */
typedef struct orc_lambertian { float Le[4]; float R[4]; int32_t back_emission; int32_t pad[3]; } orc_lambertian; /* types.cl:78-82 */
typedef struct orc_ward { float alpha; float pad0[3]; float reflectance[4]; float edgetint[4]; float falloff; float pad1[3]; } orc_ward; /* types.cl:92-97 */
typedef struct orc_volume { float C; float pad0[3]; float R[4]; } orc_volume; /* types.cl:99-102 */

typedef struct orc_scene {
    const float* points;        /* float4 per vertex */
    const uint32_t* indices;    /* 3 per triangle */
    uint32_t ntris;
    const float* spheres;       /* float4 (center, radius) */
    uint32_t nspheres;
    int32_t sphere_begin;
    const orc_node* nodes;
    uint32_t nnodes;
    const uint32_t* prim_ids;
    uint32_t nprim_ids;
    const orc_material* materials;  /* one per primitive */
    const orc_lambertian* lambertians;
    const orc_ward* wards;
    const orc_volume* volumes;
    /* environment map (NULL image = none) */
    const float* env_rgba;      /* w*h*4 float, after clamp/scale */
    int32_t env_w, env_h;
    const float* env_pdf;       /* 7*w*h: [0] uniform, [1..6] six axis (+x,-x,+y,-y,+z,-z) */
    const float* env_height;    /* 7*w*h */
    const int32_t* env_alias;   /* 7*w*h */
    const float* env_frag;      /* 4*w*h: beg_y, end_y, beg_phi, end_phi */
} orc_scene;

/* StandardCamera (kernels/camera.cl:4-22) with float3 as 4 floats */
typedef struct orc_camera {
    float eye[4], forward[4], up[4], right[4];
    float imageplane_o[4], imageplane_r[4], imageplane_b[4];
    uint32_t image_w, image_h;
} orc_camera;

typedef struct orc_config {
    float dof;                 /* new_path.cl:61 (reference 0.0045) */
    int32_t rr_depth;          /* logic.cl:76 (reference 25) */
    float radiance_clamp;      /* logic.cl:125 (reference 1000) */
    float env_select_prob;     /* mixture_density.cl:38 (reference 0.5) */
    int32_t max_depth;         /* 0 = unlimited (reference) */
    uint32_t seed_offset;      /* peseudo_random.cl random_initialize */
    uint64_t sample_limit;     /* 0 = progressive forever (reference); else W*H*spp */
    /* new_path.cl:50-51 draws the x and y pixel jitter inside one expression
       whose operand order C and OpenCL C leave unspecified.  LLVM-based OpenCL
       compilers (and the CUDA path) evaluate left to right: x first (0).  GCC,
       which compiles the reference kernels here, evaluates y first (1). */
    int32_t new_path_y_first;
    /* 1: evaluate the 6-axis envmap pdf of a BSDF-sampled direction with the
       normal flipped toward the viewer, as the sampler does (the reference
       uses the raw normal, envmap_sampling.cl:263 vs :195-198) */
    int32_t fix_backside_env_pdf;
    /* 1: sample the Lambertian BSDF around the normal flipped toward the viewer
       (the reference samples around the raw normal, lambertian.cl:49-68) */
    int32_t two_sided_lambertian;
} orc_config;

/* per-slot state in a canonical layout used to compare with the GPU */
typedef struct orc_slot {
    float T[3], L[3], ro[3], rd[3];
    uint32_t logic_i, pixel_index;
    uint32_t rng[4];
    int32_t hit_surface, hit_volume;
    float tmin;
    float Ng[3];
    int32_t queue;             /* next-step queue: 0 new path, 1..6 material type, -1 idle */
    int32_t vol_count;
    int32_t vols[7];
} orc_slot;

/* RNG (kernels/peseudo_random.cl) */
void orc_random_initialize(uint32_t* states, uint64_t n, uint64_t seed_offset);
void orc_random_uniform(uint32_t* state4, float* out, int32_t n);
void orc_random_uniform_integer(uint32_t* state4, uint64_t* out, int32_t n);

/* closest hit (extension_ray_cast_stackless.cl:81-246); rays as float[8]
   (ro.xyz, tmax, rd.xyz, pad).  prim = -1 on miss.  Counters optional. */
void orc_trace(const orc_scene* s, const float* rays, uint64_t n, int32_t* prim,
               float* t, float* ng, uint32_t* node_visits, uint32_t* prim_tests,
               int32_t nthreads);

/* tree build: binned SAH (1:1 costs, standing in for the reference's Embree build,
   stackless_bvh.hpp:108-130) flattened as create_stackless_bvh does
   (stackless_bvh.hpp:283-341).  points4 is float4 per vertex, spheres4 (center, radius).
   Returns the node count, or -1 on bad arguments; with nodes == NULL or node_cap too
   small it only returns the count (prim_ids still needs ntris + nspheres entries). */
int64_t orc_build_bvh(const float* points4, const uint32_t* indices, uint32_t ntris, const float* spheres4,
                      uint32_t nspheres, int32_t max_leaf, int32_t bins, int32_t nthreads, orc_node* nodes,
                      uint64_t node_cap, uint32_t* prim_ids, uint64_t prim_cap);

/* envmap tables (envmap.hpp:160-242, alias_method.hpp:47-114) */
int32_t orc_envmap_build(const float* rgba, int32_t w, int32_t h, float* pdf,
                         float* height, int32_t* alias, float* frag);

/* wavefront render: runs `steps` reference step()s on a pool of `npaths` slots
   and leaves FP64 per-pixel sums (r,g,b,count) in accum[4*W*H].  If slots is
   non-NULL the per-slot state after the last step is written there.  Returns
   next_pixel_index. */
uint64_t orc_render(const orc_scene* s, const orc_camera* cam, const orc_config* cfg,
                    uint32_t npaths, int32_t steps, double* accum, orc_slot* slots,
                    int32_t nthreads);

/* batched requests sharing one pool: request r owns global samples
   [begin[r], end[r]) in order; accums[r] gets its FP64 sums */
uint64_t orc_render_batch(const orc_scene* const* scenes, const orc_camera* cams, const orc_config* cfgs,
                          const uint64_t* begin, const uint64_t* end, int32_t nreq, uint32_t npaths, int32_t steps,
                          double* const* accums, orc_slot* slots, int32_t nthreads);

/* readback helpers (accumlation.cl) */
void orc_intermediate(const double* accum, uint64_t npix, uint16_t* rgb16c);
void orc_tonemap(const uint16_t* rgb16c, uint64_t npix, uint8_t* rgba8);
uint16_t orc_float_to_half(float f);
float orc_half_to_float(uint16_t h);

/* shading-stage unit entry points for golden vectors */
void orc_cosine_hemisphere(float a, float b, float* out3);
void orc_uniform_sphere(float u0, float u1, float* out3);
void orc_sample_from_fragment(const float* frag4, uint32_t* state4, float* out3);
void orc_orthonormal_basis(const float* z3, float* x3, float* y3);
void orc_sample_ward(const float* wo3, const float* z3, float alpha, float u0, float u1, float* wi3);
float orc_pdf_ward(const float* wo3, const float* wi3, const float* z3, float alpha);
void orc_envmap_value(const orc_scene* s, const float* rd3, int32_t filter, float* out3);
int32_t orc_envmap_index(const float* wi3, int32_t w, int32_t h);
/* for n directions (3 floats each): get_envmap_value's filtered lookup (exact3) and the
   same lookup with its filter weights rounded to multiples of 2^-frac_bits, as texture
   units filter (quant3): bounds the software filter's difference to hardware filtering */
void orc_envmap_filter_compare(const orc_scene* s, const float* rd3, uint64_t n, int32_t frac_bits, float* exact3,
                               float* quant3);

/* deterministic math wrappers (rgr_fmath.h), for accuracy tests */
float orc_fm(int32_t fn, float x, float y);

#ifdef __cplusplus
}
#endif
#endif
