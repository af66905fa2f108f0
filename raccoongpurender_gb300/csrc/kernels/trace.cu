// trace.cu — closest hit for a batch of rays (extension_ray_cast as a
// service), the kernel of the ray-cast microbenchmark.
//
// Rays arrive as structure-of-arrays FP32 (ox, oy, oz, dx, dy, dz, tmax:
// 28 bytes per ray); results are the primitive id (-1 on a miss), t (tmax on
// a miss) and optionally the geometric normal.
//
// Persistent warps: each warp keeps 32 rays in flight and, between traversal
// rounds, hands finished lanes new rays from a global counter (one atomic per
// refill per warp).  Within a round the lanes take node steps while at least
// `search` of them still search for their next leaf; the others wait at
// theirs.  Rays are read and results written with streaming (evict-first)
// cache hints; the tree is read with an L2 evict-last policy.
// Each ray's traversal is unchanged, so results do not depend on the
// schedule.
#include "wavefront.cuh"
#include "traverse.cuh"

#ifndef RGR_TRACE_MIN_BLOCKS
#define RGR_TRACE_MIN_BLOCKS 5  // resident 256-thread blocks per SM the register budget must allow
#endif

namespace rgr {
namespace dev {
namespace {

struct RayBatch {
    const float *ox, *oy, *oz, *dx, *dy, *dz, *tmax;
    uint64_t n;
    int32_t* prim;
    float* t;
    float* ng;                   // optional, 3 floats per ray
    uint32_t* nodes;             // optional counters (instrumented kernel)
    uint32_t* prims;
    uint32_t* err;
    unsigned long long* next;    // work counter, zero at launch
    int refill;                  // refill when at least this many lanes are idle
    int search;                  // node steps while at least this many lanes search
    uint32_t stage;              // inner nodes copied to shared memory (kStaged)
};

template <bool kCount, bool kStaged>
__global__ void __launch_bounds__(256, RGR_TRACE_MIN_BLOCKS) k_trace_rays(SceneView sc, RayBatch b) {
    const unsigned full = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const unsigned lt = (1u << lane) - 1u;
    const uint64_t pol = l2_evict_last_policy();
    extern __shared__ float4 s_nodes[];
    StagedNodes stn{s_nodes, 0u};
    if (kStaged) {
        stn.n = min(b.stage, sc.num_nodes);
        for (uint32_t i = threadIdx.x; i < 4u * stn.n; i += blockDim.x) s_nodes[i] = __ldg(sc.nodes + i);
        __syncthreads();
    }
    __shared__ uint32_t s_stack[kSmemStack > 0 ? kSmemStack * kStackThreads : 1];
    TraceState s;
    s.sstk = s_stack + threadIdx.x;
    TraceCounters cnt;
    uint64_t ray = ~0ull;  // ~0: idle
    bool exhausted = false;
    uint32_t err = 0;
    for (;;) {
        const unsigned idle = __ballot_sync(full, ray == ~0ull);
        if (!exhausted && (int)__popc(idle) >= b.refill) {
            const uint32_t need = __popc(idle);
            unsigned long long base = 0;
            if (lane == 0) base = atomicAdd(b.next, (unsigned long long)need);
            base = __shfl_sync(full, base, 0);
            if (base + need >= b.n) exhausted = true;
            if (ray == ~0ull) {
                const uint64_t r = base + __popc(idle & lt);
                if (r < b.n) {
                    ray = r;
                    trace_begin(sc, s, mk(__ldcs(b.ox + r), __ldcs(b.oy + r), __ldcs(b.oz + r)),
                                mk(__ldcs(b.dx + r), __ldcs(b.dy + r), __ldcs(b.dz + r)), __ldcs(b.tmax + r));
                    if (kCount) cnt = TraceCounters();
                }
            }
        }
        if (__ballot_sync(full, ray != ~0ull) == 0u) {
            if (exhausted) break;
            continue;
        }
        trace_warp_round<kCount, kStaged, kSmemStack>(sc, s, ray != ~0ull && s.link != kDone, b.search, &cnt, err, pol,
                                                      stn);
        if (ray != ~0ull && s.link == kDone) {
            __stcs(b.prim + ray, s.prim);
            __stcs(b.t + ray, s.tmin);
            if (b.ng) {
                f3 n = s.prim >= 0 ? hit_normal(sc, s.prim, s.ro, s.rd, s.tmin) : mk(0.0f, 0.0f, 0.0f);
                b.ng[3 * ray + 0] = n.x;
                b.ng[3 * ray + 1] = n.y;
                b.ng[3 * ray + 2] = n.z;
            }
            if (kCount) {
                b.nodes[ray] = cnt.nodes;
                b.prims[ray] = cnt.prims;
            }
            ray = ~0ull;
        }
    }
    if (err) atomicOr(b.err, err);
}

}  // namespace

void launch_trace_rays(const SceneView& sc, const float* ox, const float* oy, const float* oz, const float* dx,
                       const float* dy, const float* dz, const float* tmax, uint64_t n, int32_t* prim, float* t,
                       float* ng, uint32_t* err, unsigned long long* counter, int refill, int search, int grid,
                       uint32_t stage, cudaStream_t st) {
    if (n == 0) return;
    RayBatch b{ox, oy, oz, dx, dy, dz, tmax, n, prim, t, ng, nullptr, nullptr, err, counter, refill, search, stage};
    cudaMemsetAsync(counter, 0, sizeof(unsigned long long), st);
    if (stage > 0)
        k_trace_rays<false, true><<<grid, kStackThreads, 64 * (size_t)stage, st>>>(sc, b);
    else
        k_trace_rays<false, false><<<grid, kStackThreads, 0, st>>>(sc, b);
}

void launch_trace_rays_counts(const SceneView& sc, const float* ox, const float* oy, const float* oz, const float* dx,
                              const float* dy, const float* dz, const float* tmax, uint64_t n, int32_t* prim,
                              float* t, uint32_t* nodes, uint32_t* prims, uint32_t* err, unsigned long long* counter,
                              int grid, cudaStream_t st) {
    if (n == 0) return;
    RayBatch b{ox, oy, oz, dx, dy, dz, tmax, n, prim, t, nullptr, nodes, prims, err, counter, 16, 1, 0u};
    cudaMemsetAsync(counter, 0, sizeof(unsigned long long), st);
    k_trace_rays<true, false><<<grid, kStackThreads, 0, st>>>(sc, b);
}

int trace_rays_max_blocks_per_sm(uint32_t stage) {
    int nb = 0;
    if (stage > 0) {
        cudaFuncSetAttribute(k_trace_rays<false, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)(64 * kMaxStagedNodes));
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_trace_rays<false, true>, 256, 64 * (size_t)stage);
    } else {
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_trace_rays<false, false>, 256, 0);
    }
    return nb;
}

}  // namespace dev
}  // namespace rgr
