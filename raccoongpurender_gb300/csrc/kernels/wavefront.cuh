// wavefront.cuh — device data of the wavefront renderer and the launchers
// that the host orchestration (context.cu) calls.
#pragma once
#include "rgr_device.cuh"

namespace rgr {
namespace dev {

constexpr uint32_t kTile = 4096;         // slots per compaction tile
constexpr uint8_t kQueueIdle = 0xff;     // slot finished its sample budget
constexpr int kNumQueues = 7;            // 0 new path, 1..6 material types (logic.cl:317-331)
// material types = queue numbers (kernels/types.cl:5-11)
enum { kMatLambertian = 1, kMatSpecular = 2, kMatDielectric = 3, kMatWard = 4, kMatVolume = 5, kMatVolumeInside = 6 };

// Path state, structure of arrays, one entry per resident path slot.
// Reference fields (kernels/types.cl:18-63) are packed into 16-byte vectors:
//   ro   = (WavefrontPath.ro, ExtensionResult.tmin)
//   rd   = (WavefrontPath.rd, ExtensionResult.hit_volume_material as int bits)
//   T    = (WavefrontPath.T, WavefrontPath.pixel_index bits)
//   L    = (WavefrontPath.L, WavefrontPath.logic_i bits)
//   ng   = (ExtensionResult.Ng, ExtensionResult.hit_surface_material bits)
//   vols = InVolumeList as two int4: volumes[0..3], (volumes[4..6], count)
// ShadingResult and IncidentSample never leave registers: the stage that
// produces them also consumes them.
// Path state of a slot: kSlotVecs 16-byte vectors, the slots' records one
// after another (128 bytes per slot).  The fields a stage uses together share
// a 32-byte sector: (ro, rd) for the closest hit, (T, L) and (ng, rng) for
// the logic, the volume list (va, vb) when the path is in a volume.  A queue
// holds a sparse subset of the slots, so a stage reading a queue item's state
// pulls only sectors it uses (with one array per field each 16-byte vector
// cost a 32-byte sector of its own).
constexpr int kSlotVecs = 8;
constexpr size_t kSlotBytes = 16 * kSlotVecs;
template <class V, int kField>
struct SlotField {
    V* base;  // the first slot's record
    __host__ __device__ __forceinline__ V& operator[](size_t i) const { return base[i * kSlotVecs + kField]; }
};
struct PathsView {
    SlotField<float4, 0> ro;   // origin, tmin (t of the hit)
    SlotField<float4, 1> rd;   // direction, volume hit
    SlotField<float4, 2> T;    // throughput, pixel
    SlotField<float4, 3> L;    // radiance, logic step
    SlotField<float4, 4> ng;   // geometric normal, primitive
    SlotField<uint4, 5> rng;   // xoshiro128** state
    SlotField<int4, 6> va;     // volume list, entries 0..3
    SlotField<int4, 7> vb;     // entries 4..6, count
    uint8_t* qid;    // queue of the next step, kQueueIdle when done
    uint16_t* req;   // request of the path in the slot
    uint32_t n;
    // all fields over one buffer of n * kSlotBytes bytes
    __host__ void set_slots(void* p) {
        ro.base = rd.base = T.base = L.base = ng.base = static_cast<float4*>(p);
        rng.base = static_cast<uint4*>(p);
        va.base = vb.base = static_cast<int4*>(p);
    }
};

// The two vectors of a slot's 32-byte sector kSector (fields 2 kSector and
// 2 kSector + 1) in one 32-byte access (sm_100 and later): a warp over
// consecutive slots then makes one request per sector instead of two, and a
// store writes the whole sector.
template <int kSector>
__device__ __forceinline__ void ld_sector(const PathsView& P, uint32_t slot, float4& a, float4& b) {
    const float4* p = P.ro.base + (size_t)slot * kSlotVecs + 2 * kSector;
    asm("ld.global.v8.f32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
        : "=f"(a.x), "=f"(a.y), "=f"(a.z), "=f"(a.w), "=f"(b.x), "=f"(b.y), "=f"(b.z), "=f"(b.w)
        : "l"(p)
        : "memory");
}
// two float4 at a 32-byte aligned address in one 32-byte access
__device__ __forceinline__ void ld_v8(const float4* p, float4& a, float4& b) {
    asm("ld.global.v8.f32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
        : "=f"(a.x), "=f"(a.y), "=f"(a.z), "=f"(a.w), "=f"(b.x), "=f"(b.y), "=f"(b.z), "=f"(b.w)
        : "l"(p)
        : "memory");
}
__device__ __forceinline__ void st_v8(float4* p, const float4& a, const float4& b) {
    asm volatile("st.global.v8.f32 [%0], {%1, %2, %3, %4, %5, %6, %7, %8};" ::"l"(p), "f"(a.x), "f"(a.y), "f"(a.z),
                 "f"(a.w), "f"(b.x), "f"(b.y), "f"(b.z), "f"(b.w)
                 : "memory");
}
template <int kSector>
__device__ __forceinline__ void st_sector(const PathsView& P, uint32_t slot, const float4& a, const float4& b) {
    float4* p = P.ro.base + (size_t)slot * kSlotVecs + 2 * kSector;
    asm volatile("st.global.v8.f32 [%0], {%1, %2, %3, %4, %5, %6, %7, %8};" ::"l"(p), "f"(a.x), "f"(a.y), "f"(a.z),
                 "f"(a.w), "f"(b.x), "f"(b.y), "f"(b.z), "f"(b.w)
                 : "memory");
}
// L.w of a slot record: the path's segment count (logic_i, low 24 bits) and the
// number of volumes it is inside (high 8 bits; their ids are the record's last
// sector), so that a stage that reads (T, L) knows without reading the list
// whether it needs it
constexpr uint32_t kDepthMask = 0x00ffffffu;
__device__ __forceinline__ uint32_t depth_of(uint32_t w) { return w & kDepthMask; }
__device__ __forceinline__ int vcount_of(uint32_t w) { return (int)(w >> 24); }
__device__ __forceinline__ uint32_t depth_word(uint32_t depth, int vcount) {
    return (depth & kDepthMask) | ((uint32_t)vcount << 24);
}
__device__ __forceinline__ float4 rng_bits(const Rng& r) {
    return make_float4(__uint_as_float(r.s0), __uint_as_float(r.s1), __uint_as_float(r.s2), __uint_as_float(r.s3));
}
__device__ __forceinline__ Rng rng_of_bits(const float4& v) {
    return Rng{__float_as_uint(v.x), __float_as_uint(v.y), __float_as_uint(v.z), __float_as_uint(v.w)};
}

struct QueueView {
    uint32_t* items[kNumQueues];
    uint32_t* counts;               // [kNumQueues]
    uint32_t* tile_new;             // new paths per tile, for the ordered compaction
    uint32_t ntiles;
    unsigned long long* next_pixel; // new_path.cl next_pixel_index
    unsigned long long* step_base;  // next_pixel_index at the start of this step
};

// Queue q's item array, chosen by selects: indexing the kernel-parameter
// array with a run-time q would copy it to local memory in every thread.
__device__ __forceinline__ uint32_t* queue_items(const QueueView& Q, int q) {
    uint32_t* p = Q.items[0];
#pragma unroll
    for (int j = 1; j < kNumQueues; ++j) p = (q == j) ? Q.items[j] : p;
    return p;
}

// a[k] of a small register array, by selects (no local-memory copy)
template <int N, class T>
__device__ __forceinline__ T pick(const T (&a)[N], int k) {
    T v = a[0];
#pragma unroll
    for (int j = 1; j < N; ++j) v = (k == j) ? a[j] : v;
    return v;
}

struct CameraD {
    float eye[3], up[3], right[3];
    float o[3], r[3], b[3];
    uint32_t w, h;
};

// One render request: its scene, camera, the reference constants of
// rgr_render_config, its accumulation buffer and its range of the global
// sample index.  A single render is a table of one request; a batch of
// requests shares one path pool, each slot carrying its request id.
struct RequestD {
    SceneView sc;
    CameraD cam;
    float dof;
    int32_t rr_depth;
    float radiance_clamp;
    float env_p;
    int32_t max_depth;
    uint32_t flags;                    // kFlagFixBacksideEnvPdf | kFlagTwoSidedLambertian
    double* accum;                     // 4 doubles per pixel: r, g, b, count
    unsigned long long sample_begin;   // global sample indices [begin, end) are this request's
    unsigned long long sample_end;     // ~0: progressive, no end
    unsigned long long* done;          // paths of this request that finished (kept or discarded)
    unsigned long long* done_ns;       // %globaltimer after the bounce in which the last one finished
};

// RequestD.flags: evaluate the 6-axis envmap pdf of a BSDF-sampled direction
// with the normal flipped toward the viewer, as the envmap sampler does
// (the reference evaluates it with the raw normal, envmap_sampling.cl:263-265
// vs :195-198, which biases back-face hits).  Always on in guided renders.
constexpr uint32_t kFlagFixBacksideEnvPdf = 1u;
// RequestD.flags: sample the Lambertian BSDF around the normal flipped toward
// the viewer (the reference samples around the raw normal, lambertian.cl:49-68,
// but evaluates with the flipped one, :98-102, so a back-face hit can never
// reflect a BSDF sample).  Always on in guided renders.
constexpr uint32_t kFlagTwoSidedLambertian = 2u;

// ------------------------------------------------------------ path guiding
// training-sample stream of a guided render, all counters on the device so
// that the whole bounce (inference, shading, recording, training, Adam) is
// one CUDA graph
struct GuideTrainD {
    float* samples;                 // 16 floats each: x, n, wo, wi, weight, 3 spare
    uint32_t cap;                   // samples per training iteration
    uint32_t* count;                // appended this iteration (may exceed cap; extra dropped)
    float* wsum;                    // sum of appended weights
    unsigned long long* candidates; // finished records offered this iteration
    float* accept;                  // acceptance probability of a finished record
    uint32_t* iter;                 // completed training iterations (Adam step)
    uint32_t max_iter;              // no recording or training once *iter reaches it (0: no limit)
    uint32_t* last;                 // samples the last iteration trained on
    uint32_t min_count;             // an iteration trains once this many samples are in; until then
                                    // they carry over to the next bounce (0: always train)
    float* loss_hist;               // loss of every iteration, ring of kLossHist
};
constexpr uint32_t kLossHist = 4096;
constexpr int kGuideRecords = 3;   // training records kept per path (its first guided vertices)
// A training record: three whole 32-byte sectors (a partial store to a line that
// is not in L2 costs a read of the sector from DRAM): (L, T.x) (T.yz, cos/pdf,
// BSDF pdf) | (x, n.x) (n.yz, wo.xy) | (wo.z, wi) (unused).  The first sector is
// what the logic kernel reads of every record of an ending path.
constexpr int kGuideRecordVecs = 6;
constexpr int kGuideMixVecs = 5;    // 16-byte words per inferred mixture: 8 x FP16 (mean xyz, kappa) + 8 FP16 weights

// training still wanted (iteration budget not used up)
__device__ __forceinline__ bool guide_training_open(const GuideTrainD& t) {
    return t.max_iter == 0u || *t.iter < t.max_iter;
}

// per-render guiding state the wavefront kernels read
struct GuideRenderD {
    uint4* lobes;         // kGuideMixVecs per guided queue item of this bounce
    float4* records;      // per slot kGuideRecords x kGuideRecordVecs float4
    uint8_t* nrec;        // records written on the slot's current path
    GuideTrainD train;
    float guide_frac;     // share of the non-envmap selection probability given to the guide (learn_frac = 0)
    int32_t learn_frac;   // 1: that share is the network's selection output, per vertex
    int32_t volumes;      // guide in-volume vertices too
    int32_t record;       // record training samples
    uint32_t max_depth;   // guide vertices 1..max_depth of a path only (0: all); then, per bounce:
    uint32_t* sel;        //   the selected guided items' slots (the inference rows),
    uint32_t* remap;      //   per guided item number its row, ~0u when not selected,
    uint32_t* nsel;       //   and the number selected
};

// The guided items of this bounce as the shading kernel numbers them:
// queue 1 (Lambertian), queue 4 (Ward), then queue 6 (in-volume) when
// volumes are guided.
__device__ __forceinline__ uint32_t guided_items(const QueueView& Q, const GuideRenderD& gd) {
    return Q.counts[kMatLambertian] + Q.counts[kMatWard] + (gd.volumes ? Q.counts[kMatVolumeInside] : 0u);
}
__device__ __forceinline__ uint32_t guided_item_slot(const QueueView& Q, uint32_t gi) {
    const uint32_t c1 = Q.counts[kMatLambertian], c4 = Q.counts[kMatWard];
    if (gi < c1) return Q.items[kMatLambertian][gi];
    if (gi < c1 + c4) return Q.items[kMatWard][gi - c1];
    return Q.items[kMatVolumeInside][gi - c1 - c4];
}
// the inference rows: every guided item, or the selected ones
__device__ __forceinline__ uint32_t guide_rows(const QueueView& Q, const GuideRenderD& gd) {
    return gd.max_depth ? *gd.nsel : guided_items(Q, gd);
}
__device__ __forceinline__ uint32_t guide_row_slot(const QueueView& Q, const GuideRenderD& gd, uint32_t r) {
    return gd.max_depth ? gd.sel[r] : guided_item_slot(Q, r);
}

struct RenderParams {
    const RequestD* reqs;             // device table, nreq entries, sample ranges ascending
    int32_t nreq;
    unsigned long long sample_limit;  // end of the last range; 0 = progressive
    uint32_t* err;
    unsigned long long* rays;         // extension rays cast
    GuideRenderD gd;                  // guided renders only (gd.lobes == nullptr otherwise)
};

// launchers (wavefront.cu)
void launch_init(const PathsView& p, const QueueView& q, uint32_t seed_offset, cudaStream_t st);
void launch_compact_new(const PathsView& p, const QueueView& q, cudaStream_t st);
void launch_shade(const PathsView& p, const QueueView& q, const RenderParams& rp, int grid, cudaStream_t st);
// the guided items at vertices 1..gd.max_depth of their paths (gd.sel / remap / nsel; *nsel zeroed first)
void launch_guide_select(const PathsView& p, const QueueView& q, const GuideRenderD& gd, int grid, cudaStream_t st);
// How a bounce casts its extension rays: persistent = a separate persistent
// closest-hit kernel over the slots just shaded (warps refilled when `refill`
// lanes are idle, node steps while `search` lanes still search for a leaf,
// `grid` CTAs, `counter` a device word it may use; launch_trace_paths, between
// the shading kernel and the queue resets), then the logic kernel; otherwise
// one kernel traces and runs the logic per slot (launch_trace_paths does
// nothing).
struct TraceShape {
    bool persistent;
    int refill;
    int search;
    int grid;
    unsigned long long* counter;
};
// returns the status of its counter reset (launch errors: cudaGetLastError)
cudaError_t launch_trace_paths(const PathsView& p, const QueueView& q, const RenderParams& rp, const TraceShape& ts,
                               cudaStream_t st);
void launch_trace_logic(const PathsView& p, const QueueView& q, const RenderParams& rp, const TraceShape& ts,
                        cudaStream_t st);
int trace_paths_max_blocks_per_sm();
// per-request completion stamps of a batch (after the logic kernel of a bounce)
void launch_stamp_done(const RenderParams& rp, cudaStream_t st);
void launch_readback(int fmt, const double* accum, uint32_t npix, void* dev_out, cudaStream_t st);
void launch_sum_counts(const double* accum, uint32_t npix, unsigned long long* out, cudaStream_t st);
void launch_debug_slots(const PathsView& p, uint32_t* out, cudaStream_t st);
void launch_accum_add(double* dst, const double* src, uint32_t npix, cudaStream_t st);
void launch_merge_intermediate(void* a, const void* b, uint32_t n, cudaStream_t st);
// trace.cu
// stage: inner nodes (the breadth-first top of the tree) each CTA copies to
// shared memory, 0..kMaxStagedNodes
constexpr uint32_t kMaxStagedNodes = 1024;
void launch_trace_rays(const SceneView& sc, const float* ox, const float* oy, const float* oz, const float* dx,
                       const float* dy, const float* dz, const float* tmax, uint64_t n, int32_t* prim, float* t,
                       float* ng, uint32_t* err, unsigned long long* counter, int refill, int search, int grid,
                       uint32_t stage, cudaStream_t st);
void launch_trace_rays_counts(const SceneView& sc, const float* ox, const float* oy, const float* oz, const float* dx,
                              const float* dy, const float* dz, const float* tmax, uint64_t n, int32_t* prim,
                              float* t, uint32_t* nodes, uint32_t* prims, uint32_t* err, unsigned long long* counter,
                              int grid, cudaStream_t st);
// resident 256-thread blocks per SM of the closest-hit kernel with `stage` staged nodes
int trace_rays_max_blocks_per_sm(uint32_t stage = 0);
// the per-triangle normal table (ntri float4) of a scene whose tri_normals is null
void launch_tri_normals(const SceneView& sc, uint32_t ntri, float4* out, cudaStream_t st);
// Ray reordering: a 16-bit key per ray from its origin and the point `reach`
// along it, each quantised to 3 bits per axis: (x - lo) * scale in [0, 8)
constexpr int kRayKeyBits = 16;
constexpr uint32_t kRayBins = 1u << kRayKeyBits;
struct RayKeyBox {
    float lo[3], scale[3];          // the origin's box
    float lo_far[3], scale_far[3];  // the far point's box
    float reach;
};
// counting sort of n < 2^32 rays into `packed` (32 bytes per ray); bins: 2 x kRayBins
// words (counts, bucket starts); rank: n words; grid: the most blocks of the key passes
void launch_ray_reorder(const float* ox, const float* oy, const float* oz, const float* dx, const float* dy,
                        const float* dz, const float* tmax, uint64_t n, const RayKeyBox& kb, uint32_t* bins,
                        uint32_t* rank, float4* packed, int grid, cudaStream_t st);
// closest hit of reordered records; hits written at each record's ray index
void launch_trace_packed(const SceneView& sc, const float4* packed, uint64_t n, int32_t* prim, float* t, float* ng,
                         uint32_t* err, unsigned long long* counter, int refill, int search, int grid,
                         cudaStream_t st);

}  // namespace dev
}  // namespace rgr
