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
//
// Ray reordering (optional, for incoherent rays): a counting sort by a 16-bit
// key puts rays that start close together and head the same way next to each
// other, so that the 32 lanes of a warp walk similar paths through the tree.
// The key is a 6-D Morton code of the ray's origin and of the point half the
// scene's diagonal along it, three bits per coordinate over the scene's box
// (the far point's box widened by that reach), top 16 of the 18 bits.  Three
// passes: the key histogram (rays read once), its exclusive scan (one block),
// and the scatter of each ray as a 32-byte record (origin, tmax, direction,
// its index) to its bucket; the traversal then takes the records in bucket
// order and writes each hit at the ray's own index.  Within a bucket the
// order is that of the atomic cursor, which changes nothing but the schedule.
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
    const float4* packed;        // reordered records (kPacked): 2 float4 per ray
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

// 32-byte read of a reordered ray record, not kept in L1 and first out of L2
RGR_DEV void ld_record(const float4* ptr, float4& a, float4& b) {
    asm("ld.global.nc.L1::no_allocate.L2::evict_first.v8.f32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
        : "=f"(a.x), "=f"(a.y), "=f"(a.z), "=f"(a.w), "=f"(b.x), "=f"(b.y), "=f"(b.z), "=f"(b.w)
        : "l"(ptr));
}

template <bool kCount, bool kStaged, bool kPacked = false>
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
                    if (kPacked) {
                        float4 o4, d4;
                        ld_record(b.packed + 2 * r, o4, d4);
                        const uint32_t idx = __float_as_uint(d4.w);
                        if (idx < b.n) {  // every record holds one of the n rays
                            ray = idx;
                            trace_begin(sc, s, xyz(o4), xyz(d4), o4.w);
                        }
                    } else {
                        ray = r;
                        trace_begin(sc, s, mk(__ldcs(b.ox + r), __ldcs(b.oy + r), __ldcs(b.oz + r)),
                                    mk(__ldcs(b.dx + r), __ldcs(b.dy + r), __ldcs(b.dz + r)), __ldcs(b.tmax + r));
                    }
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

// ---------------------------------------------------------------- reordering
struct RaySoA {
    const float *ox, *oy, *oz, *dx, *dy, *dz, *tmax;
};

// one coordinate in 3 bits: floor((x - lo) * scale) clamped to [0, 7]; NaN
// goes to 0 (fmaxf returns the other operand), infinities to an end.  Explicit
// roundings: the histogram and the scatter must compute the same key.
RGR_DEV uint32_t key3(float x, float lo, float scale) {
    return (uint32_t)fminf(fmaxf(floorf(__fmul_rn(__fsub_rn(x, lo), scale)), 0.0f), 7.0f);
}

RGR_DEV uint32_t ray_key(const RayKeyBox& kb, f3 o, f3 d) {
    const uint32_t c[6] = {key3(o.x, kb.lo[0], kb.scale[0]),
                           key3(o.y, kb.lo[1], kb.scale[1]),
                           key3(o.z, kb.lo[2], kb.scale[2]),
                           key3(__fmaf_rn(d.x, kb.reach, o.x), kb.lo_far[0], kb.scale_far[0]),
                           key3(__fmaf_rn(d.y, kb.reach, o.y), kb.lo_far[1], kb.scale_far[1]),
                           key3(__fmaf_rn(d.z, kb.reach, o.z), kb.lo_far[2], kb.scale_far[2])};
    uint32_t k = 0;
#pragma unroll
    for (int bit = 2; bit >= 0; --bit)
#pragma unroll
        for (int j = 0; j < 6; ++j) k = (k << 1) | ((c[j] >> bit) & 1u);
    return k >> (18 - kRayKeyBits);
}

// The histogram and the scatter: a warp takes kKeyRays x 32 consecutive rays
// at a time, lane l the rays l, l + 32, ... (coalesced loads, kKeyRays of
// each array in flight per thread; full tiles without predicates).  Lanes
// past n form a suffix of the warp and take no part.  Equal keys are
// gathered per run of consecutive lanes: the run's first lane takes the
// run's atomic (camera rays share keys in long runs; for incoherent rays
// each lane is its own run).
constexpr int kKeyRays = 4;

// this lane's run of equal keys among the valid lanes (a prefix of `nvalid`):
// its first lane and its length
RGR_DEV void key_run(uint32_t key, int lane, int nvalid, int& head, int& len) {
    const unsigned full = 0xffffffffu;
    const uint32_t prev = __shfl_up_sync(full, key, 1);
    const unsigned heads = __ballot_sync(full, lane < nvalid && (lane == 0 || prev != key));
    head = 31 - __clz(heads & ((2u << lane) - 1u));
    const unsigned after = heads & ~((2u << head) - 1u);
    len = (after ? __ffs(after) - 1 : nvalid) - head;
}

template <bool kStream>
RGR_DEV float ld_ray(const float* p) {
    return kStream ? __ldcs(p) : __ldg(p);
}

// the kKeyRays rays of this lane, arrays a[0..kArrays-1]; lanes past n get zeros
template <int kArrays, bool kStream>
RGR_DEV void load_rays(const float* const* a, uint64_t i0, uint64_t n, int lane, float (&v)[kArrays][kKeyRays]) {
    if (i0 + 32 * kKeyRays <= n) {
#pragma unroll
        for (int j = 0; j < kKeyRays; ++j)
#pragma unroll
            for (int c = 0; c < kArrays; ++c) v[c][j] = ld_ray<kStream>(a[c] + i0 + lane + 32 * j);
    } else {
#pragma unroll
        for (int j = 0; j < kKeyRays; ++j) {
            const uint64_t i = i0 + lane + 32 * j;
#pragma unroll
            for (int c = 0; c < kArrays; ++c) v[c][j] = i < n ? ld_ray<kStream>(a[c] + i) : 0.0f;
        }
    }
}

// The counts of the keys, and each ray's rank among the rays of its key: the
// run's atomic returns the rays of that key counted before it
__global__ void __launch_bounds__(256) k_ray_bins(RaySoA r, uint64_t n, RayKeyBox kb, uint32_t* __restrict__ bins,
                                                 uint32_t* __restrict__ rank) {
    const unsigned full = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const float* const a[6] = {r.ox, r.oy, r.oz, r.dx, r.dy, r.dz};
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x * kKeyRays;
    for (uint64_t i0 = ((uint64_t)blockIdx.x * blockDim.x + (threadIdx.x & ~31u)) * kKeyRays; i0 < n; i0 += stride) {
        float v[6][kKeyRays];
        load_rays<6, false>(a, i0, n, lane, v);
        uint32_t base[kKeyRays];
        int off[kKeyRays], head[kKeyRays];
#pragma unroll
        for (int j = 0; j < kKeyRays; ++j) {
            const uint64_t left = n - (i0 + 32 * j);
            const int nvalid = i0 + 32 * j >= n ? 0 : (left >= 32 ? 32 : (int)left);
            base[j] = 0u;
            head[j] = 0;
            off[j] = -1;
            if (nvalid == 0) continue;
            const uint32_t key = ray_key(kb, mk(v[0][j], v[1][j], v[2][j]), mk(v[3][j], v[4][j], v[5][j]));
            int len;
            key_run(key, lane, nvalid, head[j], len);
            if (lane == head[j] && lane < nvalid) base[j] = atomicAdd(bins + key, (uint32_t)len);
            if (lane < nvalid) off[j] = lane - head[j];
        }
        // the ranks, once the atomics of all kKeyRays rows are in flight
#pragma unroll
        for (int j = 0; j < kKeyRays; ++j) {
            const uint32_t b = __shfl_sync(full, base[j], head[j]);
            if (off[j] >= 0) rank[i0 + lane + 32 * j] = b + (uint32_t)off[j];
        }
    }
}

// Exclusive scan of the kRayBins counts into the cursors: 32 blocks of 1024
// threads, block b the bins [2048 b, 2048 b + 2048), two per thread.  Each
// block first sums all the bins before its own (at most 62 K reads from L2,
// the blocks in parallel), so no block waits for another.
constexpr int kScanBlocks = 32;
RGR_DEV uint32_t block_sum_1024(uint32_t v, uint32_t* s_warp) {
    v = __reduce_add_sync(0xffffffffu, v);
    if ((threadIdx.x & 31) == 0) s_warp[threadIdx.x >> 5] = v;
    __syncthreads();
    uint32_t t = 0;
#pragma unroll
    for (int w = 0; w < 32; ++w) t += s_warp[w];
    __syncthreads();  // s_warp reused
    return t;
}

__global__ void __launch_bounds__(1024) k_ray_bins_scan(const uint32_t* __restrict__ bins,
                                                        uint32_t* __restrict__ cursor) {
    static_assert(kRayBins == kScanBlocks * 2048, "32 blocks of 2048 bins");
    const unsigned full = 0xffffffffu;
    __shared__ uint32_t s_warp[32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint4* p4 = reinterpret_cast<const uint4*>(bins);
    uint32_t pre = 0;
    for (uint32_t q = threadIdx.x; q < 512u * blockIdx.x; q += 1024u) {
        const uint4 v = p4[q];
        pre += v.x + v.y + v.z + v.w;
    }
    pre = block_sum_1024(pre, s_warp);
    const uint2 v = reinterpret_cast<const uint2*>(bins)[1024 * blockIdx.x + threadIdx.x];
    const uint32_t t = v.x + v.y;
    uint32_t x = t;  // inclusive scan over the warp
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(full, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) s_warp[warp] = x;
    __syncthreads();
    uint32_t wpre = 0;
    for (int w = 0; w < warp; ++w) wpre += s_warp[w];
    const uint32_t e = pre + wpre + x - t;
    reinterpret_cast<uint2*>(cursor)[1024 * blockIdx.x + threadIdx.x] = make_uint2(e, e + v.x);
}

// each ray's 32-byte record to its place: the start of its key's bucket (the
// scanned counts) plus its rank there
__global__ void __launch_bounds__(256) k_ray_scatter(RaySoA r, uint64_t n, RayKeyBox kb,
                                                    const uint32_t* __restrict__ start,
                                                    const uint32_t* __restrict__ rank, float4* __restrict__ packed) {
    const int lane = threadIdx.x & 31;
    const float* const a[7] = {r.ox, r.oy, r.oz, r.dx, r.dy, r.dz, r.tmax};
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x * kKeyRays;
    for (uint64_t i0 = ((uint64_t)blockIdx.x * blockDim.x + (threadIdx.x & ~31u)) * kKeyRays; i0 < n; i0 += stride) {
        float v[7][kKeyRays];
        load_rays<7, true>(a, i0, n, lane, v);
#pragma unroll
        for (int j = 0; j < kKeyRays; ++j) {
            const uint64_t i = i0 + lane + 32 * j;
            if (i >= n) continue;
            const uint32_t key = ray_key(kb, mk(v[0][j], v[1][j], v[2][j]), mk(v[3][j], v[4][j], v[5][j]));
            const uint32_t pos = __ldg(start + key) + __ldcs(rank + i);
            // pos < n always (both passes compute the same key)
            if (pos >= n) continue;
            float4* q = packed + 2 * (size_t)pos;
            asm volatile("st.global.v8.f32 [%0], {%1, %2, %3, %4, %5, %6, %7, %8};" ::"l"(q), "f"(v[0][j]),
                         "f"(v[1][j]), "f"(v[2][j]), "f"(v[6][j]), "f"(v[3][j]), "f"(v[4][j]), "f"(v[5][j]),
                         "f"(__uint_as_float((uint32_t)i))
                         : "memory");
        }
    }
}

}  // namespace

void launch_trace_rays(const SceneView& sc, const float* ox, const float* oy, const float* oz, const float* dx,
                       const float* dy, const float* dz, const float* tmax, uint64_t n, int32_t* prim, float* t,
                       float* ng, uint32_t* err, unsigned long long* counter, int refill, int search, int grid,
                       uint32_t stage, cudaStream_t st) {
    if (n == 0) return;
    RayBatch b{ox, oy, oz, dx, dy, dz, tmax, nullptr, n, prim, t, ng, nullptr, nullptr, err, counter, refill, search,
               stage};
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
    RayBatch b{ox, oy, oz, dx, dy, dz, tmax, nullptr, n, prim, t, nullptr, nodes, prims, err, counter, 16, 1, 0u};
    cudaMemsetAsync(counter, 0, sizeof(unsigned long long), st);
    k_trace_rays<true, false><<<grid, kStackThreads, 0, st>>>(sc, b);
}

// the per-triangle table of a scene (its tri_normals still null): the normal,
// and in w the triangle's material type (the queue of its next stage)
__global__ void k_tri_normals(SceneView sc, uint32_t ntri, float4* __restrict__ out) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= ntri) return;
    const f3 n = triangle_normal(sc, (int32_t)i);
    out[i] = make_float4(n.x, n.y, n.z, __int_as_float(__ldg(sc.materials + i).x));
}

void launch_tri_normals(const SceneView& sc, uint32_t ntri, float4* out, cudaStream_t st) {
    if (ntri == 0) return;
    k_tri_normals<<<(ntri + 255) / 256, 256, 0, st>>>(sc, ntri, out);
}

void launch_ray_reorder(const float* ox, const float* oy, const float* oz, const float* dx, const float* dy,
                        const float* dz, const float* tmax, uint64_t n, const RayKeyBox& kb, uint32_t* bins,
                        uint32_t* rank, float4* packed, int grid, cudaStream_t st) {
    if (n == 0) return;
    RaySoA r{ox, oy, oz, dx, dy, dz, tmax};
    // one pass of 256 x kKeyRays rays per block where the grid allows (the
    // block scheduler then overlaps one block's loads with another's work)
    const uint64_t tiles = (n + 256 * kKeyRays - 1) / (256 * kKeyRays);
    const int g = (int)std::min<uint64_t>(tiles, (uint64_t)grid);
    uint32_t* start = bins + kRayBins;
    cudaMemsetAsync(bins, 0, sizeof(uint32_t) * kRayBins, st);
    k_ray_bins<<<g, 256, 0, st>>>(r, n, kb, bins, rank);
    k_ray_bins_scan<<<kScanBlocks, 1024, 0, st>>>(bins, start);
    k_ray_scatter<<<g, 256, 0, st>>>(r, n, kb, start, rank, packed);
}

void launch_trace_packed(const SceneView& sc, const float4* packed, uint64_t n, int32_t* prim, float* t, float* ng,
                         uint32_t* err, unsigned long long* counter, int refill, int search, int grid,
                         cudaStream_t st) {
    if (n == 0) return;
    RayBatch b{nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, packed, n, prim, t, ng, nullptr,
               nullptr, err, counter, refill, search, 0u};
    cudaMemsetAsync(counter, 0, sizeof(unsigned long long), st);
    k_trace_rays<false, false, true><<<grid, kStackThreads, 0, st>>>(sc, b);
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
