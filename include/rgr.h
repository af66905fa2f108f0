/* rgr.h — C ABI of the GB300 wavefront path tracer (librgr.so).
 *
 * This is the drop-in boundary for the RaccoonGPURender hot path.  Each entry
 * point replaces one call of the reference host API; the reference interface
 * it stands in for is cited beside it (paths are relative to the reference
 * project).  All functions return RGR_OK (0) or a negative status; none throw.
 * Plain pointers and sizes only.  Host pointers unless a name says "device".
 *
 * Threading: a scene is not thread safe while it is being built; a context
 * may be driven by one host thread at a time (the reference drives each
 * WavefrontLane from one std::thread, common/wavefront_path_tracing.hpp:1299-1303).
 */
#ifndef RGR_H
#define RGR_H
#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ---------------------------------------------------- */
#define RGR_OK 0
#define RGR_E_INVALID (-1)   /* bad argument (the reference printf-skips non-triangle meshes, scene_manager.hpp:343-347) */
#define RGR_E_CUDA (-2)      /* CUDA runtime error; rgr_last_error() has the text */
#define RGR_E_OOM (-3)       /* device or host allocation failed */
#define RGR_E_STATE (-4)     /* call out of order (e.g. render before upload) */
#define RGR_E_OVERFLOW (-5)  /* a device-side capacity check fired (stack, queue) */
#define RGR_E_NODEVICE (-6)  /* no CUDA device / CUDA path unavailable */

/* ---- materials (common/material_type.hpp:14-63, kernels/types.cl:73-102) */
#define RGR_MAT_LAMBERTIAN 1
#define RGR_MAT_SPECULAR 2
#define RGR_MAT_DIELECTRIC 3
#define RGR_MAT_WARD 4
#define RGR_MAT_HOMOGENEOUS_VOLUME 5

typedef struct rgr_material {
    int32_t type;          /* RGR_MAT_* */
    int32_t back_emission; /* Lambertian::BackEmission (stored, unused by the kernels, as in the reference) */
    float le[3];           /* Lambertian::Le */
    float r[3];            /* Lambertian::R, Ward::reflectance, HomogeneousVolume::R */
    float edgetint[3];     /* Ward::edgetint */
    float alpha;           /* Ward::alpha */
    float falloff;         /* Ward::falloff */
    float c;               /* HomogeneousVolume::C */
} rgr_material;

/* ---- scene (replaces rt::SceneManager, common/scene_manager.hpp:330-672) */
typedef struct rgr_scene rgr_scene;

typedef struct rgr_bvh_params {
    int32_t max_leaf_size;   /* primitives per leaf, 1..8 (reference Embree build: maxLeafSize 5) */
    int32_t sah_bins;        /* binned SAH bins per axis */
    float traversal_cost;    /* SAH cost of one node visit */
    float intersect_cost;    /* SAH cost of one primitive test (0.5; the reference's Embree build uses
                                its default of 1: measured below) */
    int32_t max_depth;       /* <= 63: the reference traversal's 64-bit bit stack */
    int32_t num_threads;     /* host threads for the build (0 = all) */
    int32_t builder;         /* RGR_BVH_SAH (default): binned SAH on the host threads;
                                RGR_BVH_LBVH_GPU: linear BVH (Morton order, radix tree) on `device`,
                                subtrees of at most max_leaf_size primitives collapsed into leaves */
    int32_t device;          /* the GPU of RGR_BVH_LBVH_GPU */
} rgr_bvh_params;
#define RGR_BVH_SAH 0
#define RGR_BVH_LBVH_GPU 1

typedef struct rgr_scene_info {
    uint64_t num_triangles, num_spheres, num_vertices;
    uint64_t num_nodes_stackless;  /* nodes in the reference StacklessBVHNode layout */
    uint64_t num_inner_nodes;      /* 64-byte inner nodes in the device layout */
    uint64_t num_leaves;
    int32_t depth;                 /* tree depth (root = 0) */
    int32_t sphere_begin;          /* first sphere primitive id */
    float bounds[6];               /* scene AABB: lower xyz, upper xyz */
    double sah_cost;
} rgr_scene_info;

/* reference StacklessBVHNode (common/stackless_bvh.hpp:264-275), 96 bytes */
typedef struct rgr_stackless_node {
    float L_lower[4], L_upper[4], R_lower[4], R_upper[4];
    uint32_t link_parent, link_L, link_R, link_sibling;
    uint32_t primitive_indices_beg, primitive_indices_end;
    uint32_t pad[2];
} rgr_stackless_node;

void rgr_bvh_params_default(rgr_bvh_params* p);
int rgr_scene_create(rgr_scene** out);
void rgr_scene_destroy(rgr_scene* s);
/* SceneManager::addPolymesh (scene_manager.hpp:339-370) + add_materials (:197-277):
   P is xyz per vertex (already transformed), idx 3 per triangle, one material per triangle. */
int rgr_scene_add_mesh(rgr_scene* s, const float* P, uint64_t nverts, const uint32_t* idx, uint64_t ntris,
                       const rgr_material* per_tri);
/* SceneManager::addPointPrimitive (scene_manager.hpp:372-431): xyzr per sphere */
int rgr_scene_add_spheres(rgr_scene* s, const float* xyzr, uint64_t n, const rgr_material* per_sphere);
/* SceneManager::addPoint "ImageEnvmap" branch (scene_manager.hpp:432-497): RGBA float image,
   clamp_rgb(0, clamp_max) then scale; builds the uniform and six axis alias tables
   (common/share/envmap.hpp:160-242, alias_method.hpp:47-114).  Without an envmap the
   renderer selects BSDF sampling only (the reference requires one). */
int rgr_scene_set_envmap(rgr_scene* s, const float* rgba, int32_t w, int32_t h, float clamp_max, float scale);
/* Rebuild the scene's envmap tables with the selection weights and their FP64
   normalisation computed on `device` (fixed-order reduction); the alias
   pairing stays the reference's sequential one, on the host.  The tables
   rgr_scene_set_envmap builds on the host follow the reference bit for bit;
   these agree with them to FP64 rounding (a pdf may differ in its last bit,
   and an alias pairing where a height lands on 1.0 exactly). */
int rgr_scene_envmap_tables_gpu(rgr_scene* s, int32_t device);
/* SceneManager::buildBVH (scene_manager.hpp:517-577): binned-SAH build, deterministic. */
int rgr_scene_build_bvh(rgr_scene* s, const rgr_bvh_params* p);
int rgr_scene_get_info(const rgr_scene* s, rgr_scene_info* info);
/* create_stackless_bvh (stackless_bvh.hpp:283-341): the same tree in the reference layout */
int rgr_bvh_export_stackless(const rgr_scene* s, rgr_stackless_node* nodes, uint64_t node_cap, uint32_t* prim_ids,
                             uint64_t prim_cap);
/* createEnvmapBuffer (scene_manager.hpp:604-650): tables as uploaded.  pdf/height/alias hold
   7*w*h entries (uniform, then +x,-x,+y,-y,+z,-z); frag holds 4*w*h (beg_y,end_y,beg_phi,end_phi). */
int rgr_scene_export_envmap(const rgr_scene* s, float* pdf, float* height, int32_t* alias, float* frag);
/* The scene as built (SceneManager's _points, _indices, _spheres and MaterialStorage): 3 floats
   per vertex, 3 indices per triangle, xyzr per sphere, one material per primitive (triangles,
   then spheres; back_emission reads 0: the material tables do not keep it).  Sizes from
   rgr_scene_get_info; a null pointer skips that array. */
int rgr_scene_export_geometry(const rgr_scene* s, float* points, uint32_t* indices, float* spheres,
                              rgr_material* materials);
/* The envmap image after clamp and scale (SceneManager::_envmapImage), RGBA float rows */
int rgr_scene_export_envmap_image(const rgr_scene* s, int32_t* w, int32_t* h, float* rgba);

/* ---- device context (replaces rt::WavefrontLane, wavefront_path_tracing.hpp:339-1153) */
typedef struct rgr_context rgr_context;

/* StandardCamera (kernels/camera.cl:4-22, host standardCamera wavefront_path_tracing.hpp:103-118) */
typedef struct rgr_camera {
    float eye[3], forward[3], up[3], right[3];
    float imageplane_o[3], imageplane_r[3], imageplane_b[3];
    uint32_t image_w, image_h;
} rgr_camera;

/* Constants the reference hard-codes, as fields whose defaults equal the reference. */
typedef struct rgr_render_config {
    float dof;              /* thin-lens radius, new_path.cl:61 (0.0045) */
    int32_t rr_depth;       /* Russian roulette after this many segments, logic.cl:76 (25) */
    float radiance_clamp;   /* discard finished samples >= this, logic.cl:125 (1000) */
    float env_select_prob;  /* one-sample MIS env probability, mixture_density.cl:38 (0.5) */
    int32_t max_depth;      /* bounces; 0 = unlimited (reference) */
    uint32_t seed_offset;   /* random_initialize seed offset (lane_index * pool, :544-548) */
    uint64_t spp;           /* 0 = progressive round robin forever (reference); else stop
                               generating paths after W*H*spp samples */
    uint32_t flags;         /* RGR_RENDER_* below; 0 = the reference's behaviour */
    uint32_t reserved;
} rgr_render_config;

/* Evaluate the 6-axis envmap pdf of a BSDF-sampled direction with the normal
   flipped toward the viewer, as the envmap sampler does.  The reference uses
   the raw normal there (envmap_sampling.cl:263-265 vs :195-198), so back-face
   hits are weighted with a pdf that is not the one they were sampled from.
   Guided renders always apply it; plain renders do when this flag is set. */
#define RGR_RENDER_FIX_BACKSIDE_ENV_PDF 1u
/* Sample the Lambertian BSDF around the normal flipped toward the viewer.  The
   reference samples around the raw normal (lambertian.cl:49-68) but evaluates
   with the flipped one (:98-102), so at a back-face hit no BSDF sample carries
   light.  Guided renders always apply it; plain renders do when this flag is set. */
#define RGR_RENDER_TWO_SIDED_LAMBERTIAN 2u

typedef struct rgr_stats {
    uint64_t steps;             /* bounces of the whole pool run since render_begin */
    uint64_t paths_started;     /* next_pixel_index */
    uint64_t samples_accumulated;
    uint64_t rays_traced;       /* extension rays cast */
    double avg_spp;             /* stat kernel (stat.cl), wavefront_path_tracing.hpp:919-934 */
    uint32_t active_paths;
    uint32_t error_flags;       /* device-side checks (RGR_E_OVERFLOW causes) */
} rgr_stats;

#define RGR_FMT_RGBA8 0        /* tonemap (accumlation.cl:68-79) */
#define RGR_FMT_RGB16 1        /* RGB16IntermediateValueType: half mean + ushort count (accumlation.cl:6-25) */
#define RGR_FMT_FP64_SUMS 2    /* double r,g,b sums and count per pixel */

void rgr_render_config_default(rgr_render_config* c);
int rgr_camera_look_at(rgr_camera* c, const float eye[3], const float target[3], const float up[3], float vfov_deg,
                       uint32_t image_w, uint32_t image_h);

/* ---- scene front-end: Alembic files (replaces houdini_alembic::AlembicStorage,
   libs/houdini_alembic/houdini_alembic.hpp:417-432, and the scene loading of
   WavefrontPathTracing's constructor, wavefront_path_tracing.hpp:1170-1216).
   Reads Ogawa-container Alembic archives as a Houdini export writes them
   (transform hierarchy, polygon meshes, point objects, cameras, geometry
   parameters as attribute columns) without the Alembic SDK. */
typedef struct rgr_alembic rgr_alembic;
typedef struct rgr_alembic_info {
    uint32_t frame_count;     /* AlembicStorage::frameCount (the "1.samples" property, else 1) */
    uint32_t meshes;          /* visible triangle meshes added */
    uint32_t meshes_skipped;  /* visible meshes with non-triangle faces (skipped, scene_manager.hpp:343-347) */
    uint32_t triangles;
    uint32_t spheres;         /* from visible point objects with pscale (addPointPrimitive) */
    int32_t has_envmap;       /* an "ImageEnvmap" point set the envmap */
    int32_t has_camera;       /* the first visible camera, as standardCamera builds it */
    rgr_camera camera;
    float lens_radius, focus_distance, fov_horizontal_degree, fov_vertical_degree;
} rgr_alembic_info;
/* AlembicStorage::open: RGR_E_INVALID (rgr_last_error() says why) if the file is not an
   Ogawa Alembic archive */
int rgr_alembic_open(rgr_alembic** out, const char* path);
void rgr_alembic_close(rgr_alembic* a);
uint32_t rgr_alembic_frame_count(const rgr_alembic* a);
/* AlembicStorage::read(frame) as JSON text: every object the Houdini reader returns (type,
   parent transform name, visibility, transforms, topology, P, attribute columns by scope,
   camera parameters).  *needed = bytes including the terminating zero; cap 0 only asks. */
int rgr_alembic_describe(rgr_alembic* a, uint32_t frame, char* buf, uint64_t cap, uint64_t* needed);
/* The reference's scene load for `frame`: visible triangle meshes through their combined
   transform with per-triangle materials from the "material" column and its property
   columns (SceneManager::addPolymesh / add_materials, scene_manager.hpp:197-370), then
   visible point objects (spheres, or the "ImageEnvmap" point's Radiance .hdr image relative
   to the archive's directory: addPoint, :372-497), and the first visible camera.  Unknown
   material names and malformed files return RGR_E_INVALID. */
int rgr_alembic_load(rgr_alembic* a, uint32_t frame, rgr_scene* scene, rgr_alembic_info* info);

/* OpenCLContext::lane_initialize + WavefrontLane ctor (raccoon_ocl.hpp:752-771, :341-349).
   path_count = resident paths (reference kWavefrontPathCountGPU = 2^22). */
int rgr_context_create(rgr_context** out, int32_t device, uint32_t path_count);
void rgr_context_destroy(rgr_context* c);
/* WavefrontLane::setup (wavefront_path_tracing.hpp:451-522): upload scene, materials, envmap */
int rgr_device_upload(rgr_context* c, const rgr_scene* s);
/* WavefrontLane::initialize / re_start (:532-570, :1013-1018) */
int rgr_render_begin(rgr_context* c, const rgr_camera* cam, const rgr_render_config* cfg);
/* WavefrontLane::step() x steps (:591-939); launch_fixed(steps) (:1443-1458).  Asynchronous. */
int rgr_render_step(rgr_context* c, int32_t steps);
/* step until every generated sample has finished (needs cfg.spp > 0) or max_steps ran */
int rgr_render_until_done(rgr_context* c, int32_t max_steps, int32_t* steps_done);
/* update_intermediate + finalize_color (:942-1007), stat_avg_sample (:1148-1151); synchronous */
int rgr_render_readback(rgr_context* c, int32_t fmt, void* dst, uint64_t dst_bytes);
int rgr_render_stats(rgr_context* c, rgr_stats* st);
/* Checkpoint / resume of a render begun with rgr_render_begin (not a guided one): the
   resident path pool, its queues and counters, the RNG states and the FP64 accumulator, as
   an opaque host blob.  rgr_render_restore loads it into a context on which rgr_render_begin
   was called with the same scene, camera, config and path_count; continuing from there
   renders the same samples as the original context would have (FP64 sums equal up to the
   order of their atomic additions; counts exactly).  Synchronous. */
int rgr_render_checkpoint_size(rgr_context* c, uint64_t* bytes);
int rgr_render_checkpoint(rgr_context* c, void* dst, uint64_t dst_bytes);
int rgr_render_restore(rgr_context* c, const void* src, uint64_t src_bytes);
/* merge_from (:963-991): add src's accumulation into dst (replicas on several GPUs) */
int rgr_accum_merge(rgr_context* dst, rgr_context* src);
int rgr_synchronize(rgr_context* c);
/* capture the bounce loop in a CUDA graph (1) or launch stage by stage (0; default 1) */
int rgr_set_graph_mode(rgr_context* c, int32_t enabled);

/* merge_intermediate (accumlation.cl:27-49): a <- count-weighted merge of two
   RGB16 intermediates (device arrays of RGR_FMT_RGB16 pixels), FP32 math,
   half results, 16-bit counts; the reference's multi-device image merge. */
int rgr_intermediate_merge_device(void* a, const void* b, uint64_t npix, void* stream);

/* ---- batched requests --------------------------------------------------
   Many renders of uneven resolution, spp and scene share one resident path
   pool and one bounce loop (no reference counterpart: the reference renders
   one scene per lane).  Each request owns a range of the global sample index
   in run order; free slots go to the requests in that order. */
typedef struct rgr_batch rgr_batch;
#define RGR_ORDER_FIFO 0            /* submission order */
#define RGR_ORDER_SHORTEST_FIRST 1  /* fewest samples first */
typedef struct rgr_request_stats {
    double complete_ms;   /* device time from the start of the run to the request's last path; -1 if unfinished */
    uint64_t samples;     /* W*H*spp */
    uint64_t pixels;
    uint32_t order;       /* position in the run order */
} rgr_request_stats;
int rgr_batch_create(rgr_batch** out, int32_t device, uint32_t path_count);
void rgr_batch_destroy(rgr_batch* b);
/* the scene is uploaded once per distinct scene; cfg->spp must be > 0 */
int rgr_batch_add(rgr_batch* b, const rgr_scene* scene, const rgr_camera* cam, const rgr_render_config* cfg,
                  int32_t* request_id);
/* render every request to completion, replaying a CUDA graph of steps_per_launch bounces */
int rgr_batch_run(rgr_batch* b, int32_t order_policy, int32_t steps_per_launch, int32_t max_steps,
                  int32_t* steps_done);
int rgr_batch_readback(rgr_batch* b, int32_t request_id, int32_t fmt, void* dst, uint64_t dst_bytes);
int rgr_batch_request_stats(rgr_batch* b, int32_t request_id, rgr_request_stats* st);
/* the batch's context (its stream, stats, slot state, launch tuning) */
rgr_context* rgr_batch_context(rgr_batch* b);

/* ---- closest hit as a service (extension_ray_cast_stackless.cl:202-246) */
typedef struct rgr_ray_soa {
    const float *ox, *oy, *oz, *dx, *dy, *dz, *tmax;
} rgr_ray_soa;
/* host arrays in, host arrays out.  RGR_TRACE_HOST_AUTO (default): on a system whose GPU
   shares the host's page tables (a coherent link such as NVLink-C2C), one traversal launch
   reads the rays from and writes the hits to the host arrays directly (page-locked or
   pageable); otherwise, and with RGR_TRACE_HOST_COPY, the rays go through device buffers
   in chunks of 2^20 on four streams, copies overlapping traversal. */
int rgr_trace_closest(rgr_context* c, const rgr_ray_soa* rays, uint64_t n, int32_t* prim, float* t);
#define RGR_TRACE_HOST_AUTO 0
#define RGR_TRACE_HOST_COPY 1
int rgr_set_trace_host_mode(rgr_context* c, int32_t mode);
/* device arrays in and out, enqueued on `stream` (cudaStream_t, NULL = context stream).
   The calls of one context share its work counter (and, with ray reordering, its sort
   buffers): calls on different streams must not overlap.  A call that needs a larger
   sort buffer than the context holds allocates it (cudaMalloc), so the first call of a
   size with reordering on cannot be made under stream capture. */
int rgr_trace_closest_device(rgr_context* c, const rgr_ray_soa* rays, uint64_t n, int32_t* prim, float* t,
                             float* ng_xyz, void* stream);

/* Instrumented closest hit (same results) that also returns, per ray, the
   inner nodes visited and primitives tested: the algorithmic traffic of the
   traversal (bytes = 64 per node + 48 per primitive record). */
int rgr_trace_closest_counts_device(rgr_context* c, const rgr_ray_soa* rays, uint64_t n, int32_t* prim, float* t,
                                    uint32_t* node_visits, uint32_t* prim_tests, void* stream);

/* Render without allocating device memory.  No counterpart in the reference:
   it exists for callers that cannot call cudaMalloc at render time (a host
   application whose device memory is owned by its own allocator and fixed at
   start-up, or a real-time loop that cannot afford cudaMalloc's implicit
   device synchronisation).  Same kernels and results as rgr_render_begin() +
   rgr_render_step(steps), but the path pool, queues and counters live in one
   fixed array inside librgr (about 5 MB of device memory per GPU that loads
   the library, held until exit); path_count above 32768 is rejected with
   RGR_E_INVALID.  The caller passes a context with an uploaded scene (input)
   and accum_out, a device buffer of 4 doubles (r, g, b, count) per pixel
   (output, cleared by the call).  Runs on `stream` (NULL: the default stream)
   and is synchronous: it waits for that work to finish before it returns, and
   leaves the caller's current device unchanged.  All calls on a device share
   the array: calls that overlap on the GPU race and give wrong results.  The
   first call on a device looks up the array's address, so make that first call
   before any stream capture starts on that device. */
int rgr_render_noalloc(rgr_context* c, const rgr_camera* cam, const rgr_render_config* cfg, uint32_t path_count,
                       int32_t steps, double* accum_out, void* stream);

/* Launch shape of the bounce loop: resident 256-thread shade blocks per SM
   (1..64) and bounces per replayed CUDA graph (1..256).  Chosen by the
   autotuner (raccoongpurender_gb300/autotune.py). */
int rgr_set_render_tuning(rgr_context* c, int32_t shade_blocks_per_sm, int32_t graph_steps);

/* Launch shape of the closest-hit kernel: refill a warp with new rays when at
   least `refill` of its 32 lanes are idle (1..32); `blocks_per_sm` resident
   256-thread blocks per SM (0 = as many as fit).  Chosen by the autotuner. */
int rgr_set_trace_tuning(rgr_context* c, int32_t refill, int32_t blocks_per_sm);

/* How a bounce casts its extension rays: persistent = 1 runs a persistent
   closest-hit kernel over the slots just shaded whose warps take new slots
   when at least `refill` (1..32, default 12) lanes are idle, then the logic
   kernel; persistent = 0 traces and runs the logic in one kernel, one thread
   per slot; persistent = -1 (default) picks 1 for scenes of at least 4096
   inner BVH nodes.  Results are identical.  Takes effect at the next
   rgr_render_begin. */
int rgr_set_render_trace(rgr_context* c, int32_t persistent, int32_t refill);

/* Leaf batching of the persistent traversal kernels: within a round a warp's
   lanes take node steps while at least `search` (1..32) of them still search
   for their next leaf; the lanes that reached one wait there, then all of
   them intersect their leaves together (1 = every lane waits for the last
   one).  `closest` sets the closest-hit kernel (rgr_trace_closest*),
   `render` the extension rays of a render's bounces (takes effect at the
   next rgr_render_begin); 0 leaves that one unchanged.  Results are
   identical for every value.  Default 8 and 8; chosen by the autotuner. */
int rgr_set_trace_search(rgr_context* c, int32_t closest, int32_t render);

/* Shared-memory staging of the closest-hit kernel: each CTA copies the first
   staged_nodes (0..1024) inner nodes — the top levels of the tree, which the
   builder stores first in breadth-first order — into shared memory and reads
   them from there (64 bytes each; more staging means fewer resident CTAs).
   0 = off.  Chosen by the autotuner. */
int rgr_set_trace_staging(rgr_context* c, uint32_t staged_nodes);

/* Ray reordering of rgr_trace_closest_device (no counterpart in the
   reference): reorder = 1 sorts the rays by a 16-bit key of their origin and
   direction before the traversal (a counting sort on the device, 36 bytes of
   scratch per ray; calls of 2^32 rays or more are traced unsorted), so that a
   warp's rays walk similar paths through the tree; it pays for incoherent rays
   and costs more than it saves on coherent ones (camera rays).  0 = off
   (default).  Results are identical either way; the order only changes the
   schedule.  Chosen by the autotuner. */
int rgr_set_trace_reorder(rgr_context* c, int32_t reorder);

/* ---- learned path guiding (no counterpart in the reference) --------------
   A small MLP maps a shading vertex (frequency-encoded position, normal and
   outgoing direction: 36 inputs) through 4 hidden layers of 64 (ReLU) to an
   8-lobe von Mises-Fisher mixture over the incident direction (40 outputs).
   It runs in BF16 on the tensor cores with FP32 accumulation.  Attached to a
   context, it becomes a third strategy of the one-sample MIS at Lambertian,
   Ward and (optionally) in-volume vertices, next to BSDF and envmap
   sampling: p = s_bsdf p_bsdf + s_guide p_guide + s_env p_env, so the
   estimator stays unbiased for any network state.  While rendering, each
   path records its first guided vertices; when it ends, the radiance that
   arrived along each sampled direction becomes a training sample, and after
   every bounce one Adam step on up to batch_samples samples (loss: the KL
   divergence to f cos L_i, estimated as -w log q) runs in the same CUDA graph. */
typedef struct rgr_guide rgr_guide;
typedef struct rgr_guide_config {
    float learning_rate;     /* Adam (1e-3) */
    float beta1, beta2;      /* Adam (0.9, 0.999) */
    float epsilon;           /* Adam (1e-8) */
    uint32_t batch_samples;  /* training samples per iteration (2^18); while rendering, an iteration
                                waits (over several bounces if need be) for 1/16 of it */
    float guide_fraction;    /* share of the non-envmap selection probability given to the guide when
                                learn_fraction is 0 (0.5) */
    int32_t train;           /* train online while rendering (1), or keep the weights fixed (0) */
    int32_t guide_volumes;   /* guide in-volume scattering too (0: the isotropic phase function and
                                envmap sampling stay; guiding it doubles the largest per-vertex weight) */
    uint32_t train_interval; /* bounces per training iteration (1): samples of all of them feed it */
    uint32_t max_iterations; /* stop training (and recording samples) after this many iterations (0: never) */
    int32_t inference_kernel; /* RGR_GUIDE_TCGEN05 (default): tcgen05.mma with TMEM accumulators and
                                 activations, MMA-issuing warps apart from the row threads, five
                                 128-row tiles in flight per SM (2x faster than mma.sync);
                                 RGR_GUIDE_MMA_SYNC: warp-level mma.sync with the whole network in
                                 register fragments. */
    uint32_t max_depth;      /* guide only the first max_depth vertices of a path (0: every vertex); the
                                others use BSDF and envmap sampling alone and cost no inference */
    uint64_t seed;           /* weight initialisation (1) */
    int32_t training_kernel; /* RGR_GUIDE_TCGEN05 (default): forward, backward and the weight gradients
                                as tcgen05.mma from shared memory into TMEM accumulators, two 128-sample
                                tiles in flight per SM, per-SM gradient slots summed in a fixed order;
                                RGR_GUIDE_MMA_SYNC: warp-level mma.sync with a shared-memory gradient
                                accumulator per CTA */
    int32_t learn_fraction;  /* 1 (default): the guide's share of the non-envmap selection probability is a
                                network output per vertex, in [0.05, 0.95], trained on the KL divergence of
                                the guide-BSDF mixture (Mueller et al. 2019); 0: guide_fraction everywhere */
} rgr_guide_config;
typedef struct rgr_guide_stats {
    uint64_t iterations;     /* Adam steps taken */
    float last_loss;         /* loss of the last iteration (sum over its samples of -w log q, w normalised) */
    float accept;            /* probability with which a finished record is offered as a sample */
} rgr_guide_stats;
#define RGR_GUIDE_TCGEN05 0
#define RGR_GUIDE_MMA_SYNC 1
#define RGR_GUIDE_LAYERS 5
#define RGR_GUIDE_WIDTH 64   /* every layer is stored as a zero-padded 64 x 64 W[in][out] */

void rgr_guide_config_default(rgr_guide_config* c);
/* the network on `device`, weights initialised from cfg->seed (He uniform) */
int rgr_guide_create(rgr_guide** out, int32_t device, const rgr_guide_config* cfg);
void rgr_guide_destroy(rgr_guide* g);
int rgr_guide_set_config(rgr_guide* g, const rgr_guide_config* cfg);
/* position normalisation of the input encoding; by default the bounds of the
   scene uploaded to the context it is first rendered with */
int rgr_guide_set_bounds(rgr_guide* g, const float lo[3], const float hi[3]);
/* FP32 weights W[l][in][out] (5*64*64 floats) and biases b[l][out] (5*64);
   set also resets the Adam state */
int rgr_guide_get_weights(rgr_guide* g, float* w, float* b);
int rgr_guide_set_weights(rgr_guide* g, const float* w, const float* b);
/* Use the guide in the context's next rgr_render_begin (NULL: plain rendering).
   The guide must live on the context's device and outlive its renders. */
int rgr_context_set_guide(rgr_context* c, rgr_guide* g);
/* Raw network outputs, 48 floats per row (the mixture's 40, field-major; the selection
   logit; 7 zeros), of rows of 16 floats whose first 9 are (position, normal, outgoing
   direction); device pointers, on `stream`. */
int rgr_guide_infer_device(rgr_guide* g, const float* rows, uint32_t n, float* out, void* stream);
/* One training step on n samples of 16 floats (position, normal, outgoing,
   incident direction, weight, BSDF pdf of the incident direction (0: none, no
   selection-probability term), 2 unused), each weight multiplied by
   weight_scale.  grads (device, may be NULL) receives the gradient of the
   loss, weights then biases (5*64*64 + 5*64 floats); *loss (host, may be NULL)
   the loss.  apply_adam = 0 leaves the network unchanged. Synchronous. */
int rgr_guide_train_device(rgr_guide* g, const float* samples, uint32_t n, float weight_scale, int32_t apply_adam,
                           float* grads, float* loss, void* stream);
/* The same training step with Adam, enqueued on `stream` without waiting for it (the
   loss is in rgr_guide_loss_history once the stream has run it): for timing
   iterations back to back.  samples must stay valid until the stream has run it. */
int rgr_guide_train_device_async(rgr_guide* g, const float* samples, uint32_t n, float weight_scale, void* stream);
int rgr_guide_stats_get(rgr_guide* g, rgr_guide_stats* st);
/* RGR_OK, or RGR_E_CUDA when a tensor-core wait of the guide's kernels timed out since the
   last check (each wait gives up after about a second; the kernel then stops, frees its
   tensor memory and records the error, and the guide stays usable) */
int rgr_guide_check(rgr_guide* g);
/* Failure-detection tests: with on != 0 the MMA-issuing warps of the tcgen05 inference kernel
   issue nothing, so its row threads' waits run out and the next rgr_guide_check reports it.
   No GPU fault is involved. */
int rgr_guide_set_stall(rgr_guide* g, int32_t on);
/* losses of the last min(max, iterations) iterations, oldest first; *count receives how many */
int rgr_guide_loss_history(rgr_guide* g, float* out, uint32_t max, uint32_t* count);
/* the training samples of the last iteration of a guided render (16 floats each, as
   rgr_guide_train_device takes them), at most max; *count receives how many */
int rgr_guide_last_batch(rgr_guide* g, float* out, uint32_t max, uint32_t* count);

/* ---- diagnostics --------------------------------------------------------- */
/* Read bandwidth of `device` over a buffer of `bytes` (no reference counterpart: the
   denominator of the closest-hit roofline).  Streams the buffer with 16-byte loads that
   bypass L1 after a warm-up pass, so a buffer smaller than L2 measures L2 read bandwidth
   and a larger one HBM; each of the `reps` timed launches reads the buffer as many times
   as make 1 GiB; *gbs = bytes read / time.  Allocates its own buffer.  Lines another
   kernel marked evict-last stay in L2 and shrink what the buffer can use. */
int rgr_probe_read_bandwidth(int32_t device, uint64_t bytes, int32_t reps, double* gbs);
const char* rgr_status_string(int status);
const char* rgr_last_error(void);
/* per-slot path state after the last step, 34 uint32 words per slot in this order:
   T[3] L[3] ro[3] rd[3] logic_i pixel_index rng[4] hit_surface hit_volume tmin Ng[3]
   queue vol_count vols[7]  (queue: 0 new path, 1..6 material type, -1 idle) */
int rgr_debug_read_slots(rgr_context* c, uint32_t* out, uint64_t nslots);

#ifdef __cplusplus
}
#endif
#endif
