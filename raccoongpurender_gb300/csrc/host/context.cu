// context.cu — the device half of the C ABI: upload, render loop, readback,
// ray-cast service.  Replaces rt::WavefrontLane
// (common/wavefront_path_tracing.hpp:339-1153) on one GPU.  The per-bounce
// launch sequence is captured once into a CUDA graph and replayed, instead of
// the reference's ~24 enqueued NDRange launches per bounce.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "../kernels/wavefront.cuh"
#include "../rgr_internal.h"
#include "devbuf.h"
#include "guide_host.h"
#include "nvtx.h"

using namespace rgr;
using namespace rgr::dev;

namespace {

// A scene's device buffers and the SceneView the kernels read
// (SceneManager::createBuffer / createMaterialBuffer / createEnvmapBuffer,
// scene_manager.hpp:579-650).
struct DeviceScene {
    DevBuf nodes, prims, points, indices, spheres, materials, lambertians, wards, volumes, tri_normals;
    DevBuf env_rgba, env_pdf, env_alias, env_frag;
    SceneView sv{};
    bool valid = false;

    int upload(const rgr_scene* s, cudaStream_t st) {
        if (!s->bvh.built) {
            set_error("upload: build the BVH first");
            return RGR_E_STATE;
        }
        const Bvh& b = s->bvh;
        int r;
#define UP(buf, ptr, bytes) \
    if ((r = buf.upload((ptr), (bytes), st)) != RGR_OK) return r;
        UP(nodes, b.nodes.data(), b.nodes.size() * sizeof(NodeD));
        UP(prims, b.prims.data(), b.prims.size() * sizeof(PrimD));
        const size_t nv = s->points.size() / 3, ntri = s->indices.size() / 3;
        std::vector<float> p4(4 * nv);
        for (size_t i = 0; i < nv; ++i) {
            p4[4 * i] = s->points[3 * i];
            p4[4 * i + 1] = s->points[3 * i + 1];
            p4[4 * i + 2] = s->points[3 * i + 2];
            p4[4 * i + 3] = 0.0f;
        }
        UP(points, p4.data(), p4.size() * 4);
        UP(indices, s->indices.data(), s->indices.size() * 4);
        UP(spheres, s->spheres.data(), s->spheres.size() * 4);
        std::vector<MaterialRef> mats(s->tri_materials);
        mats.insert(mats.end(), s->sphere_materials.begin(), s->sphere_materials.end());
        UP(materials, mats.data(), mats.size() * sizeof(MaterialRef));
        UP(lambertians, s->lambertians.data(), s->lambertians.size() * sizeof(LambertianD));
        UP(wards, s->wards.data(), s->wards.size() * sizeof(WardD));
        UP(volumes, s->volumes.data(), s->volumes.size() * sizeof(VolumeD));
        const EnvTables& e = s->env;
        std::vector<int32_t> alias2;
        if (e.present) {
            size_t n7 = e.alias.size();
            alias2.resize(2 * n7);
            for (size_t i = 0; i < n7; ++i) {
                memcpy(&alias2[2 * i], &e.height[i], 4);
                alias2[2 * i + 1] = e.alias[i];
            }
            UP(env_rgba, e.rgba.data(), e.rgba.size() * 4);
            UP(env_pdf, e.pdf.data(), e.pdf.size() * 4);
            UP(env_alias, alias2.data(), alias2.size() * 4);
            UP(env_frag, e.frag.data(), e.frag.size() * 4);
        } else {
            UP(env_rgba, nullptr, 0);
            UP(env_pdf, nullptr, 0);
            UP(env_alias, nullptr, 0);
            UP(env_frag, nullptr, 0);
        }
#undef UP
        RGR_CUDA(cudaStreamSynchronize(st));  // host staging vectors go out of scope
        SceneView& v = sv;
        v.nodes = nodes.as<float4>();
        v.prims = prims.as<float4>();
        v.root_link = b.root_link;
        v.num_prims = (uint32_t)b.prims.size();
        v.points = points.as<float4>();
        v.indices = indices.as<uint32_t>();
        v.spheres = spheres.as<float4>();
        v.sphere_begin = (int32_t)ntri;
        v.materials = materials.as<int2>();
        v.lambertians = lambertians.as<float4>();
        v.wards = wards.as<float4>();
        v.volumes = volumes.as<float4>();
        v.env_rgba = env_rgba.as<float4>();
        v.env_pdf = env_pdf.as<float>();
        v.env_alias = env_alias.as<int2>();
        v.env_frag = env_frag.as<float4>();
        v.env_w = e.present ? e.w : 0;
        v.env_h = e.present ? e.h : 0;
        v.has_env = e.present ? 1 : 0;
        bool small = true;
        for (int k = 0; k < 6; ++k) small = small && std::fabs(b.bounds[k]) <= 1.0e30f;
        v.small_coords = small ? 1 : 0;
        v.num_nodes = (uint32_t)b.nodes.size();
        // the hit normals, computed once here by the kernels' own function
        v.tri_normals = nullptr;
        if ((r = tri_normals.alloc(16 * std::max<size_t>(ntri, 1))) != RGR_OK) return r;
        launch_tri_normals(v, (uint32_t)ntri, tri_normals.as<float4>(), st);
        RGR_CUDA(cudaGetLastError());
        RGR_CUDA(cudaStreamSynchronize(st));  // calls on other streams read the table
        v.tri_normals = ntri ? tri_normals.as<float4>() : nullptr;
        valid = true;
        return RGR_OK;
    }
};

CameraD camera_d(const rgr_camera& cam) {
    CameraD cd;
    for (int i = 0; i < 3; ++i) {
        cd.eye[i] = cam.eye[i];
        cd.up[i] = cam.up[i];
        cd.right[i] = cam.right[i];
        cd.o[i] = cam.imageplane_o[i];
        cd.r[i] = cam.imageplane_r[i];
        cd.b[i] = cam.imageplane_b[i];
    }
    cd.w = cam.image_w;
    cd.h = cam.image_h;
    return cd;
}

RequestD request_d(const SceneView& sv, const rgr_camera& cam, const rgr_render_config& k, double* accum,
                   unsigned long long begin, unsigned long long end, unsigned long long* done) {
    RequestD q;
    memset(&q, 0, sizeof(q));
    q.sc = sv;
    q.cam = camera_d(cam);
    q.dof = k.dof;
    q.rr_depth = k.rr_depth;
    q.radiance_clamp = k.radiance_clamp;
    q.env_p = k.env_select_prob;
    q.max_depth = k.max_depth;
    q.flags = k.flags;
    q.accum = accum;
    q.sample_begin = begin;
    q.sample_end = end;
    q.done = done;
    q.done_ns = done ? done + 1 : nullptr;
    return q;
}

}  // namespace

// scenes with fewer inner BVH nodes run the fused trace + logic kernel by default
constexpr uint32_t kPersistentTraceMinNodes = 4096;
// rgr_trace_closest: 2^20-ray chunks in flight on their own streams, so that
// the copies of some overlap the traversal of another (measured end to end
// on the closest-hit workload: 2 slots 2500 Mrays/s, 3: 2647, 4: 2705-2728,
// 6: 2682, 8: 2627; 8 slots of 2^19 rays: 2749)
constexpr int kZeroCopyRefill = 32;  // refill threshold of the zero-copy closest-hit launch
constexpr int kTraceSlots = 4;

struct rgr_context {
    int device = 0;
    cudaStream_t stream = nullptr;
    int num_sms = 152;
    uint32_t npaths = 0, ntiles = 0;
    DeviceScene scene;
    // paths
    DevBuf slots, qid, req, queues[kNumQueues], counts, tile_new, scalars, accum, err;
    DevBuf reqtab, done;  // request table and its per-request (done, done_ns) counters
    PathsView pv{};
    QueueView qv{};
    RenderParams rp{};
    bool begun = false;
    // set by rgr_render_begin (one request accumulating into `accum`), cleared by
    // every other start: only such a render can be checkpointed
    bool single_render = false;
    uint64_t render_sig = 0;  // render_signature() of that render
    uint64_t steps = 0;
    uint32_t npix = 0;
    int shade_grid = 0;
    int shade_blocks_per_sm = 8;
    // CUDA graph of `graph_steps` bounces
    bool graph_mode = true;
    int graph_steps = 1;
    int graph_steps_default = 1;
    cudaGraphExec_t graph_exec = nullptr;
    std::string graph_exec_key;  // graph_key() when graph_exec was captured
    // ray-cast service buffers
    DevBuf trays[7], tprim, tt, tread, tcounter;
    // rgr_trace_closest pipeline: kTraceSlots stream slots, each with its chunk's buffers
    struct TraceSlot {
        DevBuf rays[7], prim, t, counter, err;
    } tslot[kTraceSlots];
    cudaStream_t tstream[kTraceSlots] = {};  // [0] unused: slot 0 runs on `stream`
    int trace_host_mode = RGR_TRACE_HOST_AUTO;  // rgr_trace_closest: zero copy where it can, or staged copies
    int trace_grid = 0;      // persistent traversal grid (SMs x resident blocks)
    int trace_refill = 24;   // refill a warp when this many lanes are idle (measured best of 1..32)
    int trace_blocks = 0;    // resident blocks per SM asked for (0: as many as fit)
    // node steps while this many lanes of a warp search for a leaf: 8 measured best of
    // 1..24 with refill 24 (3702 Mrays/s, 3319 with every lane waiting for the last)
    int trace_search = 8;
    // extension rays of a bounce: persistent refilling kernel, then logic (or fused)
    // refill 12: the mixed 1080p render at 2^24 paths runs 1047.7 / 1066.6 / 1067.6 / 1066.5 /
    // 1059.5 Mpaths/s with a warp refilled at 24 / 8 / 12 / 16 / 20 idle lanes
    // search 8: 1114.8 Mpaths/s against 1032.8 with every lane waiting for the last
    TraceShape render_trace{true, 12, 8, 0, nullptr};
    int render_trace_mode = -1;  // 1 persistent, 0 fused, -1 by scene size at render begin
    uint32_t trace_stage = 0;  // top BVH nodes staged in shared memory per CTA
    int trace_reorder = 0;     // rgr_trace_closest_device sorts the rays first
    int packed_grid = 0;       // its traversal grid (no staged nodes)
    DevBuf tbins, trank, tpacked;  // its bucket counts, the rays' ranks, the reordered 32-byte records
    // learned path guiding: the attached network and this render's per-slot buffers
    rgr_guide* guide = nullptr;
    bool guided = false;      // the current render uses `guide`
    DevBuf globes, grecords, gnrec, gsel, gremap, gnsel;
    float scene_bounds[6] = {0, 0, 0, 0, 0, 0};

    ~rgr_context() {
        if (graph_exec) cudaGraphExecDestroy(graph_exec);
        for (cudaStream_t s : tstream)
            if (s) cudaStreamDestroy(s);
        if (stream) cudaStreamDestroy(stream);
    }
    // the resident path pool: state, queues, counters (WavefrontLane::setup, :451-522)
    int alloc_pool() {
        const size_t n = (size_t)ntiles * kTile;  // padded to whole tiles
        int r;
#define AL(buf, bytes) \
    if ((r = buf.alloc(bytes)) != RGR_OK) return r;
        AL(slots, kSlotBytes * n);
        AL(qid, n);
        AL(req, 2 * n);
        for (int q = 0; q < kNumQueues; ++q) AL(queues[q], 4 * n);
        AL(counts, 4 * 8);
        AL(tile_new, 4 * (size_t)ntiles);
        AL(scalars, 8 * 8);
        AL(err, 16);
#undef AL
        PathsView& p = pv;
        p.set_slots(slots.p);
        p.qid = qid.as<uint8_t>();
        p.req = req.as<uint16_t>();
        p.n = npaths;
        QueueView& q = qv;
        for (int i = 0; i < kNumQueues; ++i) q.items[i] = queues[i].as<uint32_t>();
        q.counts = counts.as<uint32_t>();
        q.tile_new = tile_new.as<uint32_t>();
        q.ntiles = ntiles;
        unsigned long long* sc = scalars.as<unsigned long long>();
        q.next_pixel = sc + 0;
        q.step_base = sc + 1;
        rp.err = err.as<uint32_t>();
        rp.rays = sc + 2;
        render_trace.counter = sc + 3;
        return RGR_OK;
    }
    // reset the pool and counters for a new render with `nreq` requests in reqtab
    int start(const RequestD* host_reqs, int nreq, unsigned long long limit, uint32_t seed_offset) {
        cudaStream_t st = stream;
        int r;
        if (render_trace_mode < 0) {
            // the separate persistent trace kernel pays for its launch when traversal
            // dominates (measured: +11 % on 1.3M triangles, -30 % on 36)
            uint32_t nodes = 0;
            for (int k = 0; k < nreq; ++k) nodes = std::max(nodes, host_reqs[k].sc.num_nodes);
            render_trace.persistent = nodes >= kPersistentTraceMinNodes;
        } else {
            render_trace.persistent = render_trace_mode != 0;
        }
        if ((r = reqtab.alloc(sizeof(RequestD) * nreq)) != RGR_OK) return r;
        RGR_CUDA(cudaMemcpyAsync(reqtab.p, host_reqs, sizeof(RequestD) * nreq, cudaMemcpyHostToDevice, st));
        rp.reqs = reqtab.as<RequestD>();
        rp.nreq = nreq;
        rp.sample_limit = limit;
        RGR_CUDA(cudaMemsetAsync(counts.p, 0, 32, st));
        RGR_CUDA(cudaMemsetAsync(scalars.p, 0, 64, st));
        RGR_CUDA(cudaMemsetAsync(err.p, 0, 16, st));
        launch_init(pv, qv, seed_offset, st);
        RGR_CUDA(cudaGetLastError());
        RGR_CUDA(cudaStreamSynchronize(st));  // host_reqs may be a temporary
        shade_grid = num_sms * shade_blocks_per_sm;
        graph_steps = graph_steps_default;
        // a replayed graph holds whole training intervals
        const int ti = train_interval();
        graph_steps = (graph_steps + ti - 1) / ti * ti;
        steps = 0;
        begun = true;
        single_render = false;
        return RGR_OK;
    }
    // train_now: a guided render ends a training interval with this bounce
    int step_launches(cudaStream_t st, bool train_now = true) {
        launch_compact_new(pv, qv, st);
        if (guided && rp.gd.max_depth) launch_guide_select(pv, qv, rp.gd, shade_grid, st);
        if (guided) guide->infer_paths(pv, qv, rp.gd, st);
        launch_shade(pv, qv, rp, shade_grid, st);
        RGR_CUDA(launch_trace_paths(pv, qv, rp, render_trace, st));
        RGR_CUDA(cudaMemsetAsync(qv.counts + 1, 0, sizeof(uint32_t) * (kNumQueues - 1), st));
        RGR_CUDA(cudaMemsetAsync(qv.tile_new, 0, sizeof(uint32_t) * ntiles, st));
        launch_trace_logic(pv, qv, rp, render_trace, st);
        if (!single_render) launch_stamp_done(rp, st);  // batches: per-request completion times
        RGR_CUDA(cudaGetLastError());
        if (guided && train_now) return guide->train_launches(st);
        return RGR_OK;
    }
    // bounces per training iteration of a guided render (1 otherwise)
    int train_interval() const { return guided ? (int)guide->cfg.train_interval : 1; }
    // per-slot guiding buffers and the kernels' view of them, or plain rendering
    int setup_guiding() {
        rp.gd = GuideRenderD{};
        guided = false;
        if (!guide) return RGR_OK;
        if (guide->device != device) {
            set_error("the guide lives on another device than the context");
            return RGR_E_INVALID;
        }
        const size_t n = (size_t)ntiles * kTile;
        int r;
        if ((r = globes.alloc(16 * kGuideMixVecs * n)) != RGR_OK) return r;
        if ((r = grecords.alloc(16 * kGuideRecordVecs * kGuideRecords * n)) != RGR_OK) return r;
        if ((r = gnrec.alloc(n)) != RGR_OK) return r;
        if (guide->cfg.max_depth) {
            if ((r = gsel.alloc(4 * n)) != RGR_OK) return r;
            if ((r = gremap.alloc(4 * n)) != RGR_OK) return r;
            if ((r = gnsel.alloc(16)) != RGR_OK) return r;
        }
        RGR_CUDA(cudaMemsetAsync(gnrec.p, 0, n, stream));
        if (!guide->bounds_set) {
            // the scene's bounds, widened by 1 % so that hit points stay inside
            float lo[3], hi[3];
            for (int k = 0; k < 3; ++k) {
                const float e = std::max(scene_bounds[3 + k] - scene_bounds[k], 1.0e-3f);
                lo[k] = scene_bounds[k] - 0.01f * e;
                hi[k] = scene_bounds[3 + k] + 0.01f * e;
            }
            if ((r = guide->set_bounds(lo, hi)) != RGR_OK) return r;
        }
        GuideRenderD& gd = rp.gd;
        gd.lobes = globes.as<uint4>();
        gd.records = grecords.as<float4>();
        gd.nrec = gnrec.as<uint8_t>();
        gd.train = guide->train;
        gd.guide_frac = guide->cfg.guide_fraction;
        gd.learn_frac = guide->cfg.learn_fraction != 0 ? 1 : 0;
        gd.volumes = guide->cfg.guide_volumes ? 1 : 0;
        gd.record = guide->cfg.train ? 1 : 0;
        gd.max_depth = guide->cfg.max_depth;
        if (gd.max_depth) {
            gd.sel = gsel.as<uint32_t>();
            gd.remap = gremap.as<uint32_t>();
            gd.nsel = gnsel.as<uint32_t>();
        }
        guided = true;
        return RGR_OK;
    }
    // run `n` bounces: replays of a graph of graph_steps bounces, then single ones
    int run_steps(int n) {
        cudaStream_t st = stream;
        while (n > 0) {
            if (graph_mode) {
                const int k = n >= graph_steps ? graph_steps : 1;
                if (k == graph_steps || graph_steps == 1) {
                    const std::string key = graph_key();
                    if (graph_exec && key != graph_exec_key) drop_graph();
                    if (!graph_exec) {
                        graph_exec_key = key;
                        cudaGraph_t g = nullptr;
                        RGR_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
                        int r = RGR_OK;
                        for (int i = 0; i < graph_steps && r == RGR_OK; ++i)
                            r = step_launches(st, (i + 1) % train_interval() == 0);
                        cudaError_t e = cudaStreamEndCapture(st, &g);
                        if (r != RGR_OK) return r;
                        RGR_CUDA(e);
                        e = cudaGraphInstantiate(&graph_exec, g, 0);
                        cudaGraphDestroy(g);
                        RGR_CUDA(e);
                    }
                    RGR_CUDA(cudaGraphLaunch(graph_exec, st));
                    n -= graph_steps;
                    steps += graph_steps;
                    continue;
                }
            }
            int r = step_launches(st, (steps + 1) % (uint64_t)train_interval() == 0);
            if (r != RGR_OK) return r;
            n -= 1;
            steps += 1;
        }
        return RGR_OK;
    }
    void drop_graph() {
        if (graph_exec) cudaGraphExecDestroy(graph_exec);
        graph_exec = nullptr;
    }
    // Everything a captured bounce graph bakes in: the kernels' parameter
    // structs and launch shapes.  A new render whose key is unchanged (same
    // pool, request table, sample limit and guide) replays the graph it has;
    // the request table's contents (scene, camera, accumulation buffer) are
    // read from device memory and may change freely.
    std::string graph_key() const {
        std::string k;
        auto add = [&k](const void* p, size_t n) { k.append(static_cast<const char*>(p), n); };
        add(&pv, sizeof(pv));
        add(&qv, sizeof(qv));
        add(&rp, sizeof(rp));
        add(&shade_grid, sizeof(shade_grid));
        add(&render_trace, sizeof(render_trace));
        add(&graph_steps, sizeof(graph_steps));
        add(&guided, sizeof(guided));
        add(&single_render, sizeof(single_render));  // batches add the completion stamps
        if (guided) {
            add(&guide->view, sizeof(guide->view));
            add(&guide->cfg, sizeof(guide->cfg));
            add(&num_sms, sizeof(num_sms));
        }
        return k;
    }
};

// read-only view of a context's uploaded scene, for rgr_render_noalloc (noalloc.cu)
const rgr::dev::SceneView* rgr_context_scene_view(const rgr_context* c, int* device) {
    if (!c || !c->scene.valid) return nullptr;
    if (device) *device = c->device;
    return &c->scene.sv;
}

namespace {
// FNV-1a over the pointer-free description of a render begun with rgr_render_begin:
// the scene's sizes and bounds, the camera, every config field and the pool size.
// A checkpoint carries it, and a restore into a render of another scene, camera,
// spp, seed or flags is refused.
uint64_t render_signature(const SceneView& sv, const rgr_camera& cam, const rgr_render_config& k, uint32_t npaths) {
    uint64_t h = 1469598103934665603ull;
    auto mix = [&h](const void* p, size_t n) {
        const unsigned char* b = static_cast<const unsigned char*>(p);
        for (size_t i = 0; i < n; ++i) h = (h ^ b[i]) * 1099511628211ull;
    };
    const uint32_t scene[8] = {sv.root_link, sv.num_prims, (uint32_t)sv.sphere_begin, sv.num_nodes,
                               (uint32_t)sv.env_w, (uint32_t)sv.env_h, (uint32_t)sv.has_env, npaths};
    mix(scene, sizeof(scene));
    mix(&cam, sizeof(cam));
    mix(&k.dof, 4);
    mix(&k.rr_depth, 4);
    mix(&k.radiance_clamp, 4);
    mix(&k.env_select_prob, 4);
    mix(&k.max_depth, 4);
    mix(&k.seed_offset, 4);
    mix(&k.spp, 8);
    mix(&k.flags, 4);
    return h;
}
}  // namespace

extern "C" {

int rgr_context_create(rgr_context** out, int32_t device, uint32_t path_count) {
    if (!out || path_count == 0 || path_count > (1u << 28)) return RGR_E_INVALID;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        set_error("no CUDA device");
        return RGR_E_NODEVICE;
    }
    if (device < 0 || device >= ndev) return RGR_E_INVALID;
    rgr_context* c = new (std::nothrow) rgr_context();
    if (!c) return RGR_E_OOM;
    c->device = device;
    if (!cuda_ok(cudaSetDevice(device), "cudaSetDevice") ||
        !cuda_ok(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking), "cudaStreamCreate")) {
        delete c;
        return RGR_E_CUDA;
    }
    cudaDeviceGetAttribute(&c->num_sms, cudaDevAttrMultiProcessorCount, device);
    c->trace_grid = c->num_sms * std::max(1, trace_rays_max_blocks_per_sm());
    c->packed_grid = c->trace_grid;
    c->render_trace.grid = c->num_sms * std::max(1, trace_paths_max_blocks_per_sm());
    c->npaths = path_count;
    c->ntiles = (path_count + kTile - 1) / kTile;
    *out = c;
    return RGR_OK;
}

void rgr_context_destroy(rgr_context* c) {
    if (!c) return;
    cudaSetDevice(c->device);
    if (c->stream) cudaStreamSynchronize(c->stream);
    delete c;
}

int rgr_set_graph_mode(rgr_context* c, int32_t enabled) {
    if (!c) return RGR_E_INVALID;
    c->graph_mode = enabled != 0;
    c->drop_graph();
    return RGR_OK;
}

int rgr_device_upload(rgr_context* c, const rgr_scene* s) {
    RGR_NVTX_RANGE("rgr_device_upload");
    if (!c || !s) return RGR_E_INVALID;
    RGR_CUDA(cudaSetDevice(c->device));
    int r = c->scene.upload(s, c->stream);
    if (r != RGR_OK) return r;
    for (int k = 0; k < 6; ++k) c->scene_bounds[k] = s->bvh.bounds[k];
    c->begun = false;
    c->drop_graph();
    return RGR_OK;
}

int rgr_render_begin(rgr_context* c, const rgr_camera* cam, const rgr_render_config* cfg) {
    RGR_NVTX_RANGE("rgr_render_begin");
    if (!c || !cam) return RGR_E_INVALID;
    if (!c->scene.valid) {
        set_error("rgr_render_begin: upload a scene first");
        return RGR_E_STATE;
    }
    if (cam->image_w == 0 || cam->image_h == 0 || (uint64_t)cam->image_w * cam->image_h > (1ull << 31))
        return RGR_E_INVALID;
    rgr_render_config d;
    rgr_render_config_default(&d);
    const rgr_render_config& k = cfg ? *cfg : d;
    RGR_CUDA(cudaSetDevice(c->device));
    int r = c->alloc_pool();
    if (r != RGR_OK) return r;
    c->npix = cam->image_w * cam->image_h;
    if ((r = c->accum.alloc(32 * (size_t)c->npix)) != RGR_OK) return r;
    if ((r = c->done.alloc(16)) != RGR_OK) return r;
    RGR_CUDA(cudaMemsetAsync(c->accum.p, 0, 32 * (size_t)c->npix, c->stream));
    RGR_CUDA(cudaMemsetAsync(c->done.p, 0, 16, c->stream));
    const unsigned long long limit = k.spp ? (unsigned long long)k.spp * c->npix : 0ull;
    // no completion counter: nothing reads a single render's completion time, and
    // the counter cost every warp of the logic kernel an atomic on one address
    RequestD q = request_d(c->scene.sv, *cam, k, c->accum.as<double>(), 0ull, limit ? limit : ~0ull, nullptr);
    if ((r = c->setup_guiding()) != RGR_OK) return r;
    if (c->guided) q.flags |= kFlagFixBacksideEnvPdf | kFlagTwoSidedLambertian;
    if ((r = c->start(&q, 1, limit, k.seed_offset)) != RGR_OK) return r;
    c->single_render = true;
    c->render_sig = render_signature(c->scene.sv, *cam, k, c->npaths);
    return RGR_OK;
}

int rgr_context_set_guide(rgr_context* c, rgr_guide* g) {
    if (!c) return RGR_E_INVALID;
    if (g && g->device != c->device) {
        set_error("rgr_context_set_guide: the guide lives on another device than the context");
        return RGR_E_INVALID;
    }
    c->guide = g;
    c->begun = false;  // takes effect at the next rgr_render_begin
    c->guided = false;
    c->rp.gd = GuideRenderD{};
    c->drop_graph();
    return RGR_OK;
}

int rgr_render_step(rgr_context* c, int32_t steps) {
    RGR_NVTX_RANGE("rgr_render_step");
    if (!c || steps < 0) return RGR_E_INVALID;
    if (!c->begun) return RGR_E_STATE;
    RGR_CUDA(cudaSetDevice(c->device));
    return c->run_steps(steps);
}

int rgr_synchronize(rgr_context* c) {
    if (!c) return RGR_E_INVALID;
    RGR_CUDA(cudaSetDevice(c->device));
    RGR_CUDA(cudaStreamSynchronize(c->stream));
    uint32_t err = 0;
    if (c->begun) {
        RGR_CUDA(cudaMemcpy(&err, c->err.p, 4, cudaMemcpyDeviceToHost));
        if (err) {
            set_error("device capacity check fired (flags " + std::to_string(err) + ")");
            return RGR_E_OVERFLOW;
        }
    }
    return RGR_OK;
}

int rgr_render_until_done(rgr_context* c, int32_t max_steps, int32_t* steps_done) {
    RGR_NVTX_RANGE("rgr_render_until_done");
    if (!c || max_steps < 0) return RGR_E_INVALID;
    if (!c->begun || c->rp.sample_limit == 0) return RGR_E_STATE;
    int32_t done = 0;
    while (done < max_steps) {
        int batch = std::min<int32_t>(8, max_steps - done);
        int r = rgr_render_step(c, batch);
        if (r != RGR_OK) return r;
        done += batch;
        uint32_t counts[8];
        unsigned long long np = 0;
        RGR_CUDA(cudaMemcpyAsync(counts, c->counts.p, 32, cudaMemcpyDeviceToHost, c->stream));
        RGR_CUDA(cudaMemcpyAsync(&np, c->scalars.p, 8, cudaMemcpyDeviceToHost, c->stream));
        RGR_CUDA(cudaStreamSynchronize(c->stream));
        uint64_t live = 0;
        for (int k = 1; k < kNumQueues; ++k) live += counts[k];
        if (np >= c->rp.sample_limit && live == 0) break;
    }
    if (steps_done) *steps_done = done;
    return rgr_synchronize(c);
}

namespace {
// the device state of a begun render, in checkpoint order
struct StatePart {
    DevBuf* buf;
    size_t bytes;
};
std::vector<StatePart> render_state(rgr_context* c) {
    const size_t n = (size_t)c->ntiles * kTile;
    std::vector<StatePart> v = {{&c->slots, kSlotBytes * n}, {&c->qid, n},     {&c->req, 2 * n},
                                {&c->counts, 32},             {&c->tile_new, 4 * (size_t)c->ntiles},
                                {&c->scalars, 64},            {&c->err, 16},   {&c->accum, 32 * (size_t)c->npix},
                                {&c->done, 16}};
    for (int q = 0; q < kNumQueues; ++q) v.push_back({&c->queues[q], 4 * n});
    return v;
}
struct CheckpointHeader {
    char magic[8];  // "RGRCKPT2"
    uint64_t npaths, ntiles, npix, steps, bytes;
    uint64_t signature;  // render_signature() of the render: scene, camera, config
};
int checkpointable(rgr_context* c) {
    if (!c) return RGR_E_INVALID;
    if (!c->begun || !c->single_render || c->guided || c->rp.nreq != 1 || c->npix == 0) {
        set_error("checkpoint: a render begun with rgr_render_begin, not a guided one or a batch, is needed");
        return RGR_E_STATE;
    }
    return RGR_OK;
}
uint64_t checkpoint_bytes(rgr_context* c) {
    uint64_t b = sizeof(CheckpointHeader);
    for (const StatePart& s : render_state(c)) b += s.bytes;
    return b;
}
}  // namespace

int rgr_render_checkpoint_size(rgr_context* c, uint64_t* bytes) {
    int r = checkpointable(c);
    if (r != RGR_OK) return r;
    if (!bytes) return RGR_E_INVALID;
    *bytes = checkpoint_bytes(c);
    return RGR_OK;
}

int rgr_render_checkpoint(rgr_context* c, void* dst, uint64_t dst_bytes) {
    RGR_NVTX_RANGE("rgr_render_checkpoint");
    int r = checkpointable(c);
    if (r != RGR_OK) return r;
    const uint64_t total = checkpoint_bytes(c);
    if (!dst || dst_bytes < total) return RGR_E_INVALID;
    RGR_CUDA(cudaSetDevice(c->device));
    RGR_CUDA(cudaStreamSynchronize(c->stream));
    CheckpointHeader h{{'R', 'G', 'R', 'C', 'K', 'P', 'T', '2'}, c->npaths, c->ntiles, c->npix, c->steps, total,
                       c->render_sig};
    unsigned char* p = static_cast<unsigned char*>(dst);
    memcpy(p, &h, sizeof(h));
    p += sizeof(h);
    for (const StatePart& s : render_state(c)) {
        RGR_CUDA(cudaMemcpy(p, s.buf->p, s.bytes, cudaMemcpyDeviceToHost));
        p += s.bytes;
    }
    return RGR_OK;
}

int rgr_render_restore(rgr_context* c, const void* src, uint64_t src_bytes) {
    RGR_NVTX_RANGE("rgr_render_restore");
    int r = checkpointable(c);
    if (r != RGR_OK) return r;
    CheckpointHeader h;
    if (!src || src_bytes < sizeof(h)) return RGR_E_INVALID;
    memcpy(&h, src, sizeof(h));
    if (memcmp(h.magic, "RGRCKPT2", 8) != 0 || h.npaths != c->npaths || h.ntiles != c->ntiles ||
        h.npix != c->npix || h.bytes != checkpoint_bytes(c) || src_bytes < h.bytes) {
        set_error("rgr_render_restore: not a checkpoint of a render of this shape");
        return RGR_E_INVALID;
    }
    if (h.signature != c->render_sig) {
        set_error("rgr_render_restore: the checkpoint is of a render with another scene, camera or config");
        return RGR_E_INVALID;
    }
    RGR_CUDA(cudaSetDevice(c->device));
    RGR_CUDA(cudaStreamSynchronize(c->stream));
    const unsigned char* p = static_cast<const unsigned char*>(src) + sizeof(h);
    for (const StatePart& s : render_state(c)) {
        RGR_CUDA(cudaMemcpy(s.buf->p, p, s.bytes, cudaMemcpyHostToDevice));
        p += s.bytes;
    }
    c->steps = h.steps;
    return RGR_OK;
}

int rgr_render_readback(rgr_context* c, int32_t fmt, void* dst, uint64_t dst_bytes) {
    RGR_NVTX_RANGE("rgr_render_readback");
    if (!c || !dst) return RGR_E_INVALID;
    if (!c->begun) return RGR_E_STATE;
    RGR_CUDA(cudaSetDevice(c->device));
    cudaStream_t st = c->stream;
    const size_t npix = c->npix;
    if (fmt == RGR_FMT_FP64_SUMS) {
        if (dst_bytes < 32 * npix) return RGR_E_INVALID;
        RGR_CUDA(cudaMemcpyAsync(dst, c->accum.p, 32 * npix, cudaMemcpyDeviceToHost, st));
    } else if (fmt == RGR_FMT_RGBA8 || fmt == RGR_FMT_RGB16) {
        size_t bytes = (fmt == RGR_FMT_RGBA8 ? 4 : 8) * npix;
        if (dst_bytes < bytes) return RGR_E_INVALID;
        int r = c->tread.alloc(bytes);
        if (r != RGR_OK) return r;
        launch_readback(fmt, c->accum.as<double>(), (uint32_t)npix, c->tread.p, st);
        RGR_CUDA(cudaGetLastError());
        RGR_CUDA(cudaMemcpyAsync(dst, c->tread.p, bytes, cudaMemcpyDeviceToHost, st));
    } else {
        return RGR_E_INVALID;
    }
    return rgr_synchronize(c);
}

int rgr_render_stats(rgr_context* c, rgr_stats* s) {
    if (!c || !s) return RGR_E_INVALID;
    memset(s, 0, sizeof(*s));
    if (!c->begun) return RGR_E_STATE;
    RGR_CUDA(cudaSetDevice(c->device));
    cudaStream_t st = c->stream;
    int r = c->tread.alloc(std::max<size_t>(c->tread.bytes, 64));
    if (r != RGR_OK) return r;
    RGR_CUDA(cudaMemsetAsync(c->tread.p, 0, 8, st));
    launch_sum_counts(c->accum.as<double>(), c->npix, c->tread.as<unsigned long long>(), st);
    RGR_CUDA(cudaGetLastError());
    unsigned long long vals[3] = {0, 0, 0}, total = 0;
    uint32_t counts[8], err = 0;
    RGR_CUDA(cudaMemcpyAsync(vals, c->scalars.p, 24, cudaMemcpyDeviceToHost, st));
    RGR_CUDA(cudaMemcpyAsync(&total, c->tread.p, 8, cudaMemcpyDeviceToHost, st));
    RGR_CUDA(cudaMemcpyAsync(counts, c->counts.p, 32, cudaMemcpyDeviceToHost, st));
    RGR_CUDA(cudaMemcpyAsync(&err, c->err.p, 4, cudaMemcpyDeviceToHost, st));
    RGR_CUDA(cudaStreamSynchronize(st));
    s->steps = c->steps;
    s->paths_started = vals[0];
    s->rays_traced = vals[2];
    s->samples_accumulated = total;
    s->avg_spp = (double)total / (double)c->npix;
    uint64_t live = 0;
    for (int k = 0; k < kNumQueues; ++k) live += counts[k];
    s->active_paths = (uint32_t)std::min<uint64_t>(live, c->npaths);
    s->error_flags = err;
    return RGR_OK;
}

int rgr_accum_merge(rgr_context* dst, rgr_context* src) {
    if (!dst || !src || !dst->begun || !src->begun || dst->npix != src->npix) return RGR_E_INVALID;
    RGR_CUDA(cudaSetDevice(src->device));
    RGR_CUDA(cudaStreamSynchronize(src->stream));
    RGR_CUDA(cudaSetDevice(dst->device));
    int r = dst->tread.alloc(32 * (size_t)dst->npix);
    if (r != RGR_OK) return r;
    RGR_CUDA(cudaMemcpyPeerAsync(dst->tread.p, dst->device, src->accum.p, src->device, 32 * (size_t)src->npix,
                                 dst->stream));
    launch_accum_add(dst->accum.as<double>(), dst->tread.as<double>(), dst->npix, dst->stream);
    RGR_CUDA(cudaGetLastError());
    return rgr_synchronize(dst);
}

int rgr_trace_closest_device(rgr_context* c, const rgr_ray_soa* rays, uint64_t n, int32_t* prim, float* t,
                             float* ng_xyz, void* stream) {
    RGR_NVTX_RANGE("rgr_trace_closest_device");
    if (!c || !rays || !prim || !t) return RGR_E_INVALID;
    if (!c->scene.valid) return RGR_E_STATE;
    if (n == 0) return RGR_OK;
    if (!rays->ox || !rays->oy || !rays->oz || !rays->dx || !rays->dy || !rays->dz || !rays->tmax)
        return RGR_E_INVALID;
    RGR_CUDA(cudaSetDevice(c->device));
    cudaStream_t st = stream ? (cudaStream_t)stream : c->stream;
    int r = c->err.alloc(16);
    if (r != RGR_OK) return r;
    if ((r = c->tcounter.alloc(8)) != RGR_OK) return r;
    if (c->trace_reorder && n < (1ull << 32)) {
        if ((r = c->tbins.alloc(2 * sizeof(uint32_t) * kRayBins)) != RGR_OK) return r;
        if ((r = c->tpacked.alloc(32 * (size_t)n)) != RGR_OK) return r;
        if ((r = c->trank.alloc(4 * (size_t)n)) != RGR_OK) return r;
        // the key's boxes: the scene's, and for the point half its diagonal along
        // the ray the same box widened by that reach
        RayKeyBox kb;
        const float* b = c->scene_bounds;
        float d2 = 0.0f;
        for (int k = 0; k < 3; ++k) d2 += (b[3 + k] - b[k]) * (b[3 + k] - b[k]);
        kb.reach = 0.5f * std::sqrt(d2);
        for (int k = 0; k < 3; ++k) {
            const float e = b[3 + k] - b[k];
            kb.lo[k] = b[k];
            kb.scale[k] = e > 0.0f ? 8.0f / e : 0.0f;
            kb.lo_far[k] = b[k] - kb.reach;
            kb.scale_far[k] = e + 2.0f * kb.reach > 0.0f ? 8.0f / (e + 2.0f * kb.reach) : 0.0f;
        }
        launch_ray_reorder(rays->ox, rays->oy, rays->oz, rays->dx, rays->dy, rays->dz, rays->tmax, n, kb,
                           c->tbins.as<uint32_t>(), c->trank.as<uint32_t>(), c->tpacked.as<float4>(),
                           c->num_sms * 64, st);
        launch_trace_packed(c->scene.sv, c->tpacked.as<float4>(), n, prim, t, ng_xyz, c->err.as<uint32_t>(),
                            c->tcounter.as<unsigned long long>(), c->trace_refill, c->trace_search, c->packed_grid,
                            st);
        RGR_CUDA(cudaGetLastError());
        return RGR_OK;
    }
    launch_trace_rays(c->scene.sv, rays->ox, rays->oy, rays->oz, rays->dx, rays->dy, rays->dz, rays->tmax, n, prim, t, ng_xyz,
                      c->err.as<uint32_t>(), c->tcounter.as<unsigned long long>(), c->trace_refill, c->trace_search,
                      c->trace_grid, c->trace_stage, st);
    RGR_CUDA(cudaGetLastError());
    return RGR_OK;
}

int rgr_intermediate_merge_device(void* a, const void* b, uint64_t npix, void* stream) {
    if (!a || !b || npix > 0xffffffffull) return RGR_E_INVALID;
    if (npix == 0) return RGR_OK;
    launch_merge_intermediate(a, b, (uint32_t)npix, (cudaStream_t)stream);
    RGR_CUDA(cudaGetLastError());
    return RGR_OK;
}

int rgr_set_render_tuning(rgr_context* c, int32_t shade_blocks_per_sm, int32_t graph_steps) {
    if (!c || shade_blocks_per_sm < 1 || shade_blocks_per_sm > 64 || graph_steps < 1 || graph_steps > 256)
        return RGR_E_INVALID;
    c->shade_blocks_per_sm = shade_blocks_per_sm;
    c->shade_grid = c->num_sms * shade_blocks_per_sm;
    c->graph_steps_default = graph_steps;
    c->graph_steps = graph_steps;
    c->drop_graph();
    return RGR_OK;
}

int rgr_set_trace_tuning(rgr_context* c, int32_t refill, int32_t blocks_per_sm) {
    if (!c || refill < 1 || refill > 32 || blocks_per_sm < 0) return RGR_E_INVALID;
    RGR_CUDA(cudaSetDevice(c->device));
    int maxb = std::max(1, trace_rays_max_blocks_per_sm(c->trace_stage));
    if (blocks_per_sm > maxb) return RGR_E_INVALID;
    c->trace_refill = refill;
    c->trace_blocks = blocks_per_sm;
    c->trace_grid = c->num_sms * (blocks_per_sm ? blocks_per_sm : maxb);
    const int maxb0 = std::max(1, trace_rays_max_blocks_per_sm(0));
    c->packed_grid = c->num_sms * (blocks_per_sm ? std::min(blocks_per_sm, maxb0) : maxb0);
    return RGR_OK;
}

int rgr_set_render_trace(rgr_context* c, int32_t persistent, int32_t refill) {
    if (!c || refill < 1 || refill > 32 || persistent < -1 || persistent > 1) return RGR_E_INVALID;
    c->render_trace_mode = persistent;
    c->render_trace.refill = refill;
    c->begun = false;  // takes effect at the next render begin
    c->drop_graph();
    return RGR_OK;
}

int rgr_set_trace_search(rgr_context* c, int32_t closest, int32_t render) {
    if (!c || closest < 0 || closest > 32 || render < 0 || render > 32) return RGR_E_INVALID;
    if (closest > 0) c->trace_search = closest;
    if (render > 0 && render != c->render_trace.search) {
        c->render_trace.search = render;
        c->begun = false;  // takes effect at the next render begin
        c->drop_graph();
    }
    return RGR_OK;
}

int rgr_set_trace_host_mode(rgr_context* c, int32_t mode) {
    if (!c || (mode != RGR_TRACE_HOST_AUTO && mode != RGR_TRACE_HOST_COPY)) return RGR_E_INVALID;
    c->trace_host_mode = mode;
    return RGR_OK;
}

int rgr_set_trace_reorder(rgr_context* c, int32_t reorder) {
    if (!c || reorder < 0 || reorder > 1) return RGR_E_INVALID;
    c->trace_reorder = reorder;
    return RGR_OK;
}

int rgr_set_trace_staging(rgr_context* c, uint32_t staged_nodes) {
    if (!c || staged_nodes > kMaxStagedNodes) return RGR_E_INVALID;
    RGR_CUDA(cudaSetDevice(c->device));
    int maxb = std::max(1, trace_rays_max_blocks_per_sm(staged_nodes));
    c->trace_stage = staged_nodes;
    c->trace_grid = c->num_sms * (c->trace_blocks ? std::min(c->trace_blocks, maxb) : maxb);
    return RGR_OK;
}

int rgr_trace_closest_counts_device(rgr_context* c, const rgr_ray_soa* rays, uint64_t n, int32_t* prim, float* t,
                                    uint32_t* node_visits, uint32_t* prim_tests, void* stream) {
    if (!c || !rays || !prim || !t || !node_visits || !prim_tests) return RGR_E_INVALID;
    if (!c->scene.valid) return RGR_E_STATE;
    if (n == 0) return RGR_OK;
    RGR_CUDA(cudaSetDevice(c->device));
    cudaStream_t st = stream ? (cudaStream_t)stream : c->stream;
    int r = c->err.alloc(16);
    if (r != RGR_OK) return r;
    if ((r = c->tcounter.alloc(8)) != RGR_OK) return r;
    launch_trace_rays_counts(c->scene.sv, rays->ox, rays->oy, rays->oz, rays->dx, rays->dy, rays->dz, rays->tmax, n, prim, t,
                             node_visits, prim_tests, c->err.as<uint32_t>(), c->tcounter.as<unsigned long long>(),
                             c->trace_grid, st);
    RGR_CUDA(cudaGetLastError());
    return RGR_OK;
}

// Host arrays in and out: the rays go in chunks of up to 2^20, round robin
// over kTraceSlots streams, so that the copies of some chunks overlap the
// traversal of another (with page-locked host memory; pageable memory still
// works, its copies just do not overlap).
namespace {
// The address under which the GPU reads or writes host array p, or null:
// page-locked (or registered) host memory has a device address; on a system
// whose GPU walks the host's page tables (NVLink-C2C with address
// translation) any host address is one.
void* device_view(const void* p, bool pageable_ok) {
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    if (a.type == cudaMemoryTypeHost || a.type == cudaMemoryTypeManaged || a.type == cudaMemoryTypeDevice)
        return a.devicePointer;
    return pageable_ok ? const_cast<void*>(p) : nullptr;
}
}  // namespace

int rgr_trace_closest(rgr_context* c, const rgr_ray_soa* rays, uint64_t n, int32_t* prim, float* t) {
    RGR_NVTX_RANGE("rgr_trace_closest");
    if (!c || !rays || !prim || !t) return RGR_E_INVALID;
    if (!c->scene.valid) return RGR_E_STATE;
    if (n == 0) return RGR_OK;
    const float* src[7] = {rays->ox, rays->oy, rays->oz, rays->dx, rays->dy, rays->dz, rays->tmax};
    for (int k = 0; k < 7; ++k)
        if (!src[k]) return RGR_E_INVALID;
    RGR_CUDA(cudaSetDevice(c->device));
    int r;
    int pageable = 0;  // the GPU shares the host's page tables: a coherent CPU-GPU link (NVLink-C2C)
    cudaDeviceGetAttribute(&pageable, cudaDevAttrPageableMemoryAccessUsesHostPageTables, c->device);
    if (c->trace_host_mode == RGR_TRACE_HOST_AUTO && pageable) {
        // zero copy: the traversal kernel reads the rays from, and writes the hits to, host
        // memory across the link, one launch over all rays.  Over PCIe the staged copies
        // below are faster, so zero copy is only taken on a coherent link.
        const float* dsrc[7];
        bool direct = true;
        for (int k = 0; k < 7 && direct; ++k) direct = (dsrc[k] = (const float*)device_view(src[k], pageable)) != nullptr;
        int32_t* dprim = direct ? (int32_t*)device_view(prim, pageable) : nullptr;
        float* dt = direct ? (float*)device_view(t, pageable) : nullptr;
        if (direct && dprim && dt) {
            rgr_context::TraceSlot& ts = c->tslot[0];
            if ((r = ts.counter.alloc(8)) != RGR_OK || (r = ts.err.alloc(16)) != RGR_OK) return r;
            cudaStream_t st = c->stream;
            RGR_CUDA(cudaMemsetAsync(ts.err.p, 0, 4, st));
            // a warp refills only when all its lanes are idle: each refill's reads across
            // the link then serve 32 rays (measured: 3030 Mrays/s end to end, against
            // 2905 with the threshold tuned for rays in device memory)
            launch_trace_rays(c->scene.sv, dsrc[0], dsrc[1], dsrc[2], dsrc[3], dsrc[4], dsrc[5], dsrc[6], n, dprim, dt,
                              nullptr, ts.err.as<uint32_t>(), ts.counter.as<unsigned long long>(), kZeroCopyRefill,
                              c->trace_search, c->trace_grid, c->trace_stage, st);
            RGR_CUDA(cudaGetLastError());
            uint32_t err = 0;
            RGR_CUDA(cudaMemcpyAsync(&err, ts.err.p, 4, cudaMemcpyDeviceToHost, st));
            RGR_CUDA(cudaStreamSynchronize(st));
            if (err) {
                set_error("traversal stack overflow");
                return RGR_E_OVERFLOW;
            }
            return RGR_OK;
        }
    }
    cudaStream_t streams[kTraceSlots];
    for (int s = 0; s < kTraceSlots; ++s) {
        if (s > 0 && !c->tstream[s]) RGR_CUDA(cudaStreamCreateWithFlags(&c->tstream[s], cudaStreamNonBlocking));
        streams[s] = s == 0 ? c->stream : c->tstream[s];
    }
    const uint64_t kChunk = 1ull << 20;
    const uint64_t chunk = std::min(n, kChunk);
    for (int s = 0; s < kTraceSlots; ++s) {
        rgr_context::TraceSlot& ts = c->tslot[s];
        for (int k = 0; k < 7; ++k)
            if ((r = ts.rays[k].alloc(4 * chunk)) != RGR_OK) return r;
        if ((r = ts.prim.alloc(4 * chunk)) != RGR_OK || (r = ts.t.alloc(4 * chunk)) != RGR_OK ||
            (r = ts.counter.alloc(8)) != RGR_OK || (r = ts.err.alloc(16)) != RGR_OK)
            return r;
        RGR_CUDA(cudaMemsetAsync(ts.err.p, 0, 4, streams[s]));
    }
    for (uint64_t off = 0, i = 0; off < n; off += chunk, ++i) {
        const int s = (int)(i % kTraceSlots);
        cudaStream_t st = streams[s];
        rgr_context::TraceSlot& ts = c->tslot[s];
        const uint64_t m = std::min(chunk, n - off);
        for (int k = 0; k < 7; ++k)
            RGR_CUDA(cudaMemcpyAsync(ts.rays[k].p, src[k] + off, 4 * m, cudaMemcpyHostToDevice, st));
        launch_trace_rays(c->scene.sv, ts.rays[0].as<float>(), ts.rays[1].as<float>(), ts.rays[2].as<float>(),
                          ts.rays[3].as<float>(), ts.rays[4].as<float>(), ts.rays[5].as<float>(),
                          ts.rays[6].as<float>(), m, ts.prim.as<int32_t>(), ts.t.as<float>(), nullptr,
                          ts.err.as<uint32_t>(), ts.counter.as<unsigned long long>(), c->trace_refill,
                          c->trace_search, c->trace_grid, c->trace_stage, st);
        RGR_CUDA(cudaGetLastError());
        RGR_CUDA(cudaMemcpyAsync(prim + off, ts.prim.p, 4 * m, cudaMemcpyDeviceToHost, st));
        RGR_CUDA(cudaMemcpyAsync(t + off, ts.t.p, 4 * m, cudaMemcpyDeviceToHost, st));
    }
    uint32_t err[kTraceSlots] = {};
    uint32_t any = 0;
    for (int s = 0; s < kTraceSlots; ++s) {
        RGR_CUDA(cudaMemcpyAsync(&err[s], c->tslot[s].err.p, 4, cudaMemcpyDeviceToHost, streams[s]));
        RGR_CUDA(cudaStreamSynchronize(streams[s]));
        any |= err[s];
    }
    if (any) {
        set_error("traversal stack overflow");
        return RGR_E_OVERFLOW;
    }
    return RGR_OK;
}

int rgr_debug_read_slots(rgr_context* c, uint32_t* out, uint64_t nslots) {
    if (!c || !out) return RGR_E_INVALID;
    if (!c->begun) return RGR_E_STATE;
    if (nslots < c->npaths) return RGR_E_INVALID;
    RGR_CUDA(cudaSetDevice(c->device));
    cudaStream_t st = c->stream;
    size_t bytes = 34 * 4 * (size_t)c->npaths;
    int r = c->tread.alloc(bytes);
    if (r != RGR_OK) return r;
    launch_debug_slots(c->pv, c->tread.as<uint32_t>(), st);
    RGR_CUDA(cudaGetLastError());
    RGR_CUDA(cudaMemcpyAsync(out, c->tread.p, bytes, cudaMemcpyDeviceToHost, st));
    return rgr_synchronize(c);
}

}  // extern "C"

// ======================================================================
// Batched requests: many renders of uneven size share one path pool.  Each
// request owns a range of the global sample index (in run order), so the
// new-path compaction hands free slots to the requests in that order and a
// slot renders its request's scene with its camera and constants.  The
// bounce loop is replayed from a CUDA graph; every request's last finished
// path stamps %globaltimer, giving per-request completion latency.
struct rgr_batch {
    rgr_context* ctx = nullptr;
    struct Req {
        const rgr_scene* scene;
        int scene_index;
        rgr_camera cam;
        rgr_render_config cfg;
        uint64_t npix, samples;
        DevBuf accum;
        double complete_ms = -1.0;
        uint32_t order = 0;
        uint64_t accumulated = 0;
    };
    std::vector<std::unique_ptr<DeviceScene>> scenes;
    std::vector<const rgr_scene*> scene_keys;
    std::vector<std::unique_ptr<Req>> reqs;
    DevBuf stamp;  // start time of the run (%globaltimer)
    ~rgr_batch() { delete ctx; }
};

namespace {
__global__ void k_stamp(unsigned long long* out) {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    *out = t;
}
}  // namespace

extern "C" {

int rgr_batch_create(rgr_batch** out, int32_t device, uint32_t path_count) {
    if (!out) return RGR_E_INVALID;
    rgr_batch* b = new (std::nothrow) rgr_batch();
    if (!b) return RGR_E_OOM;
    int r = rgr_context_create(&b->ctx, device, path_count);
    if (r != RGR_OK) {
        delete b;
        return r;
    }
    *out = b;
    return RGR_OK;
}

void rgr_batch_destroy(rgr_batch* b) {
    if (!b) return;
    if (b->ctx) {
        cudaSetDevice(b->ctx->device);
        cudaStreamSynchronize(b->ctx->stream);
    }
    delete b;
}

int rgr_batch_add(rgr_batch* b, const rgr_scene* s, const rgr_camera* cam, const rgr_render_config* cfg,
                  int32_t* id) {
    if (!b || !s || !cam || !cfg || cfg->spp == 0) {
        set_error("rgr_batch_add: every request needs a scene, a camera and spp > 0");
        return RGR_E_INVALID;
    }
    if (b->reqs.size() >= 65535) return RGR_E_INVALID;
    if (cam->image_w == 0 || cam->image_h == 0 || (uint64_t)cam->image_w * cam->image_h > (1ull << 31))
        return RGR_E_INVALID;
    rgr_context* c = b->ctx;
    RGR_CUDA(cudaSetDevice(c->device));
    int si = -1;
    for (size_t i = 0; i < b->scene_keys.size(); ++i)
        if (b->scene_keys[i] == s) si = (int)i;
    if (si < 0) {
        std::unique_ptr<DeviceScene> ds(new DeviceScene());
        int r = ds->upload(s, c->stream);
        if (r != RGR_OK) return r;
        si = (int)b->scenes.size();
        b->scenes.push_back(std::move(ds));
        b->scene_keys.push_back(s);
    }
    std::unique_ptr<rgr_batch::Req> q(new rgr_batch::Req());
    q->scene = s;
    q->scene_index = si;
    q->cam = *cam;
    q->cfg = *cfg;
    q->npix = (uint64_t)cam->image_w * cam->image_h;
    q->samples = q->npix * cfg->spp;
    int r = q->accum.alloc(32 * q->npix);
    if (r != RGR_OK) return r;
    if (id) *id = (int32_t)b->reqs.size();
    b->reqs.push_back(std::move(q));
    return RGR_OK;
}

int rgr_batch_run(rgr_batch* b, int32_t order_policy, int32_t steps_per_launch, int32_t max_steps,
                  int32_t* steps_done) {
    RGR_NVTX_RANGE("rgr_batch_run");
    if (!b || b->reqs.empty() || steps_per_launch < 1 || max_steps < 1) return RGR_E_INVALID;
    rgr_context* c = b->ctx;
    RGR_CUDA(cudaSetDevice(c->device));
    cudaStream_t st = c->stream;
    const int n = (int)b->reqs.size();
    // run order: submission order, or fewest samples first (shortest job first)
    std::vector<int> order(n);
    for (int i = 0; i < n; ++i) order[i] = i;
    if (order_policy == RGR_ORDER_SHORTEST_FIRST)
        std::stable_sort(order.begin(), order.end(),
                         [&](int x, int y) { return b->reqs[x]->samples < b->reqs[y]->samples; });
    int r = c->alloc_pool();
    if (r != RGR_OK) return r;
    if ((r = c->done.alloc(16 * (size_t)n)) != RGR_OK) return r;
    if ((r = b->stamp.alloc(8)) != RGR_OK) return r;
    RGR_CUDA(cudaMemsetAsync(c->done.p, 0, 16 * (size_t)n, st));
    std::vector<RequestD> table(n);
    unsigned long long begin = 0;
    for (int k = 0; k < n; ++k) {
        rgr_batch::Req& q = *b->reqs[order[k]];
        q.order = (uint32_t)k;
        RGR_CUDA(cudaMemsetAsync(q.accum.p, 0, 32 * q.npix, st));
        table[k] = request_d(b->scenes[q.scene_index]->sv, q.cam, q.cfg, q.accum.as<double>(), begin,
                             begin + q.samples, c->done.as<unsigned long long>() + 2 * k);
        begin += q.samples;
    }
    c->npix = 0;
    r = c->start(table.data(), n, begin, b->reqs[order[0]]->cfg.seed_offset);
    if (r != RGR_OK) return r;
    c->graph_steps = steps_per_launch;
    k_stamp<<<1, 1, 0, st>>>(b->stamp.as<unsigned long long>());
    std::vector<unsigned long long> done(2 * n);
    int32_t ran = 0;
    bool all = false;
    while (ran < max_steps && !all) {
        r = c->run_steps(steps_per_launch);
        if (r != RGR_OK) return r;
        ran += steps_per_launch;
        RGR_CUDA(cudaMemcpyAsync(done.data(), c->done.p, 16 * (size_t)n, cudaMemcpyDeviceToHost, st));
        RGR_CUDA(cudaStreamSynchronize(st));
        all = true;
        for (int k = 0; k < n; ++k) all = all && done[2 * k] == table[k].sample_end - table[k].sample_begin;
    }
    c->graph_steps = c->graph_steps_default;
    c->drop_graph();
    unsigned long long t0 = 0;
    RGR_CUDA(cudaMemcpy(&t0, b->stamp.p, 8, cudaMemcpyDeviceToHost));
    for (int k = 0; k < n; ++k) {
        rgr_batch::Req& q = *b->reqs[order[k]];
        const bool fin = done[2 * k] == table[k].sample_end - table[k].sample_begin;
        q.complete_ms = fin ? (double)(done[2 * k + 1] - t0) * 1e-6 : -1.0;
    }
    if (steps_done) *steps_done = ran;
    uint32_t err = 0;
    RGR_CUDA(cudaMemcpy(&err, c->err.p, 4, cudaMemcpyDeviceToHost));
    if (err) {
        set_error("device capacity check fired (flags " + std::to_string(err) + ")");
        return RGR_E_OVERFLOW;
    }
    return all ? RGR_OK : RGR_E_STATE;
}

int rgr_batch_readback(rgr_batch* b, int32_t id, int32_t fmt, void* dst, uint64_t dst_bytes) {
    if (!b || !dst || id < 0 || id >= (int32_t)b->reqs.size()) return RGR_E_INVALID;
    rgr_context* c = b->ctx;
    rgr_batch::Req& q = *b->reqs[id];
    RGR_CUDA(cudaSetDevice(c->device));
    cudaStream_t st = c->stream;
    if (fmt == RGR_FMT_FP64_SUMS) {
        if (dst_bytes < 32 * q.npix) return RGR_E_INVALID;
        RGR_CUDA(cudaMemcpyAsync(dst, q.accum.p, 32 * q.npix, cudaMemcpyDeviceToHost, st));
    } else if (fmt == RGR_FMT_RGBA8 || fmt == RGR_FMT_RGB16) {
        size_t bytes = (fmt == RGR_FMT_RGBA8 ? 4 : 8) * q.npix;
        if (dst_bytes < bytes) return RGR_E_INVALID;
        int r = c->tread.alloc(bytes);
        if (r != RGR_OK) return r;
        launch_readback(fmt, q.accum.as<double>(), (uint32_t)q.npix, c->tread.p, st);
        RGR_CUDA(cudaGetLastError());
        RGR_CUDA(cudaMemcpyAsync(dst, c->tread.p, bytes, cudaMemcpyDeviceToHost, st));
    } else {
        return RGR_E_INVALID;
    }
    RGR_CUDA(cudaStreamSynchronize(st));
    return RGR_OK;
}

int rgr_batch_request_stats(rgr_batch* b, int32_t id, rgr_request_stats* out) {
    if (!b || !out || id < 0 || id >= (int32_t)b->reqs.size()) return RGR_E_INVALID;
    const rgr_batch::Req& q = *b->reqs[id];
    out->complete_ms = q.complete_ms;
    out->samples = q.samples;
    out->order = q.order;
    out->pixels = q.npix;
    return RGR_OK;
}

rgr_context* rgr_batch_context(rgr_batch* b) { return b ? b->ctx : nullptr; }

}  // extern "C"
