// noalloc.cu — a render entry point that allocates no device memory.
//
// rgr_render_begin() allocates the resident path pool with cudaMalloc.  Some
// callers cannot do that at render time: a host application whose device
// memory belongs to its own pool allocator and is fixed at start-up, or a
// real-time loop in which cudaMalloc's implicit device synchronisation would
// stall the frame.  rgr_render_noalloc() serves them.  It renders with the
// same kernels as rgr_render_step(), but its path state, queues and counters
// live in the file-scope array below, which the CUDA runtime places in device
// memory when the library is loaded.  The caller passes the inputs (a context
// with an uploaded scene, camera, config) and the output (a device buffer of
// 4 doubles per pixel).
//
// Limits and sharing:
//  * at most kNoAllocMaxPaths resident paths (larger path_count is rejected);
//  * every GPU that loads the library holds kScratchBytes (about 5 MB) of
//    device memory until the process exits;
//  * every call on a device reuses the same array, and the array keeps what
//    the previous call left in it; each call re-initialises what must start
//    from zero.  Calls whose work overlaps on the GPU (two streams, or two
//    host threads) race on the array and give wrong results;
//  * the first call on a device looks up the array's device address
//    (cudaGetSymbolAddress), so that first call should come before any stream
//    capture begins on that device;
//  * the call is synchronous: it waits for its work on `stream` before it
//    returns, and it leaves the caller's current device as it found it.
#include <cuda_runtime.h>

#include <cstring>
#include <mutex>
#include <string>

#include "../kernels/wavefront.cuh"
#include "../rgr_internal.h"

using namespace rgr;
using namespace rgr::dev;

// the context's uploaded scene (context.cu)
const rgr::dev::SceneView* rgr_context_scene_view(const rgr_context* c, int* device);

namespace {

constexpr uint32_t kNoAllocMaxPaths = 1u << 15;
constexpr uint32_t kNoAllocTiles = kNoAllocMaxPaths / kTile;
static_assert(kNoAllocMaxPaths % kTile == 0, "whole tiles");

// byte offsets inside the scratch array (every region 256-byte aligned)
constexpr size_t align256(size_t x) { return (x + 255) & ~size_t(255); }
constexpr size_t kN = kNoAllocMaxPaths;
constexpr size_t kOffSlots = 0;
constexpr size_t kOffQid = kOffSlots + align256(kSlotBytes * kN);
constexpr size_t kOffReq = kOffQid + align256(kN);
constexpr size_t kOffQueues = kOffReq + align256(2 * kN);
constexpr size_t kOffCounts = kOffQueues + align256(4 * kN) * kNumQueues;
constexpr size_t kOffTiles = kOffCounts + 256;
constexpr size_t kOffScalars = kOffTiles + align256(4 * kNoAllocTiles);
constexpr size_t kOffErr = kOffScalars + 256;
constexpr size_t kOffRequest = kOffErr + 256;
constexpr size_t kScratchBytes = kOffRequest + align256(sizeof(RequestD));

static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

std::mutex g_mu;
void* g_scratch_addr[128] = {};

// Once per device, with that device current: the device address of the array.
int scratch_address(int device, unsigned char** out) {
    if (device < 0 || device >= 128) return RGR_E_INVALID;
    std::lock_guard<std::mutex> lock(g_mu);
    if (!g_scratch_addr[device]) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || p == nullptr) {
            set_error(std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
            return RGR_E_CUDA;
        }
        g_scratch_addr[device] = p;
    }
    *out = static_cast<unsigned char*>(g_scratch_addr[device]);
    return RGR_OK;
}

bool ok(cudaError_t e, const char* what) {
    if (e == cudaSuccess) return true;
    set_error(std::string(what) + ": " + cudaGetErrorString(e));
    return false;
}

// puts the caller's current device back on every return
struct DeviceRestore {
    int prev = -1;
    DeviceRestore() {
        if (cudaGetDevice(&prev) != cudaSuccess) prev = -1;
    }
    ~DeviceRestore() {
        if (prev >= 0) cudaSetDevice(prev);
    }
};

}  // namespace

extern "C" int rgr_render_noalloc(rgr_context* c, const rgr_camera* cam, const rgr_render_config* cfg,
                                  uint32_t path_count, int32_t steps, double* accum_out, void* stream) {
    if (!c || !cam || !accum_out || steps < 0) return RGR_E_INVALID;
    if (path_count == 0 || path_count > kNoAllocMaxPaths) {
        set_error("rgr_render_noalloc: path_count must be 1.." + std::to_string(kNoAllocMaxPaths) +
                  " (the fixed scratch holds at most that many paths)");
        return RGR_E_INVALID;
    }
    if (cam->image_w == 0 || cam->image_h == 0 || (uint64_t)cam->image_w * cam->image_h > (1ull << 31))
        return RGR_E_INVALID;
    int device = 0;
    const SceneView* sv = rgr_context_scene_view(c, &device);
    if (!sv) {
        set_error("rgr_render_noalloc: upload a scene to the context first");
        return RGR_E_STATE;
    }
    DeviceRestore restore_device;
    if (!ok(cudaSetDevice(device), "cudaSetDevice")) return RGR_E_CUDA;
    int sms = 0;
    if (!ok(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device), "cudaDeviceGetAttribute"))
        return RGR_E_CUDA;
    unsigned char* base = nullptr;
    int r = scratch_address(device, &base);
    if (r != RGR_OK) return r;
    cudaStream_t st = (cudaStream_t)stream;

    rgr_render_config d;
    rgr_render_config_default(&d);
    const rgr_render_config& k = cfg ? *cfg : d;
    const uint32_t npix = cam->image_w * cam->image_h;
    const uint32_t ntiles = (path_count + kTile - 1) / kTile;

    PathsView p;
    p.set_slots(base + kOffSlots);
    p.qid = base + kOffQid;
    p.req = reinterpret_cast<uint16_t*>(base + kOffReq);
    p.n = path_count;
    QueueView q;
    for (int i = 0; i < kNumQueues; ++i) q.items[i] = reinterpret_cast<uint32_t*>(base + kOffQueues + align256(4 * kN) * i);
    q.counts = reinterpret_cast<uint32_t*>(base + kOffCounts);
    q.tile_new = reinterpret_cast<uint32_t*>(base + kOffTiles);
    q.ntiles = ntiles;
    unsigned long long* scal = reinterpret_cast<unsigned long long*>(base + kOffScalars);
    q.next_pixel = scal + 0;
    q.step_base = scal + 1;
    // the one-request table (kernels read scene, camera and constants from it)
    RequestD rq;
    memset(&rq, 0, sizeof(rq));
    rq.sc = *sv;
    CameraD& cd = rq.cam;
    for (int i = 0; i < 3; ++i) {
        cd.eye[i] = cam->eye[i];
        cd.up[i] = cam->up[i];
        cd.right[i] = cam->right[i];
        cd.o[i] = cam->imageplane_o[i];
        cd.r[i] = cam->imageplane_r[i];
        cd.b[i] = cam->imageplane_b[i];
    }
    cd.w = cam->image_w;
    cd.h = cam->image_h;
    rq.dof = k.dof;
    rq.rr_depth = k.rr_depth;
    rq.radiance_clamp = k.radiance_clamp;
    rq.env_p = k.env_select_prob;
    rq.max_depth = k.max_depth;
    rq.flags = k.flags;
    rq.accum = accum_out;
    const unsigned long long limit = k.spp ? (unsigned long long)k.spp * npix : 0ull;
    rq.sample_begin = 0;
    rq.sample_end = limit ? limit : ~0ull;
    rq.done = nullptr;
    rq.done_ns = nullptr;
    RenderParams rp{};  // value-initialised: no guiding (rp.gd.lobes == nullptr)
    rp.reqs = reinterpret_cast<const RequestD*>(base + kOffRequest);
    rp.nreq = 1;
    rp.sample_limit = limit;
    rp.err = reinterpret_cast<uint32_t*>(base + kOffErr);
    rp.rays = scal + 2;

    // the array keeps the previous call's contents: reset counters and output
    if (!ok(cudaMemsetAsync(base + kOffCounts, 0, 256, st), "cudaMemsetAsync") ||
        !ok(cudaMemsetAsync(base + kOffScalars, 0, 256, st), "cudaMemsetAsync") ||
        !ok(cudaMemsetAsync(base + kOffErr, 0, 256, st), "cudaMemsetAsync") ||
        !ok(cudaMemsetAsync(accum_out, 0, sizeof(double) * 4 * (size_t)npix, st), "cudaMemsetAsync") ||
        !ok(cudaMemcpyAsync(base + kOffRequest, &rq, sizeof(rq), cudaMemcpyHostToDevice, st), "cudaMemcpyAsync"))
        return RGR_E_CUDA;
    launch_init(p, q, k.seed_offset, st);
    if (!ok(cudaGetLastError(), "kernel launch")) return RGR_E_CUDA;
    const TraceShape ts{true, 24, 8,
                        sms * (trace_paths_max_blocks_per_sm() > 0 ? trace_paths_max_blocks_per_sm() : 1), scal + 3};
    for (int32_t i = 0; i < steps; ++i) {
        launch_compact_new(p, q, st);
        launch_shade(p, q, rp, sms * 8, st);
        if (!ok(launch_trace_paths(p, q, rp, ts, st), "cudaMemsetAsync") ||
            !ok(cudaMemsetAsync(q.counts + 1, 0, sizeof(uint32_t) * (kNumQueues - 1), st), "cudaMemsetAsync") ||
            !ok(cudaMemsetAsync(q.tile_new, 0, sizeof(uint32_t) * ntiles, st), "cudaMemsetAsync"))
            return RGR_E_CUDA;
        launch_trace_logic(p, q, rp, ts, st);
        // a failed launch stops the call at the bounce it happened in
        if (!ok(cudaGetLastError(), "kernel launch")) return RGR_E_CUDA;
    }
    uint32_t err = 0;
    if (!ok(cudaMemcpyAsync(&err, rp.err, 4, cudaMemcpyDeviceToHost, st), "cudaMemcpyAsync") ||
        !ok(cudaStreamSynchronize(st), "cudaStreamSynchronize"))
        return RGR_E_CUDA;
    if (err) {
        set_error("device capacity check fired (flags " + std::to_string(err) + ")");
        return RGR_E_OVERFLOW;
    }
    return RGR_OK;
}
