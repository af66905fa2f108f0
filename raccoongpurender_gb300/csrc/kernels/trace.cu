// trace.cu — closest hit for a batch of rays (extension_ray_cast as a
// service), the kernel of the ray-cast microbenchmark.
//
// Rays arrive as structure-of-arrays FP32 (ox, oy, oz, dx, dy, dz, tmax:
// 28 bytes per ray, coalesced 128-byte warp loads per component); results
// are the primitive id (-1 on a miss) and t (tmax on a miss), and optionally
// the geometric normal.
#include "wavefront.cuh"
#include "traverse.cuh"

namespace rgr {
namespace dev {
namespace {

__global__ void __launch_bounds__(128) k_trace_rays(SceneView sc, const float* __restrict__ ox,
                                                    const float* __restrict__ oy, const float* __restrict__ oz,
                                                    const float* __restrict__ dx, const float* __restrict__ dy,
                                                    const float* __restrict__ dz, const float* __restrict__ tmax,
                                                    uint64_t n, int32_t* __restrict__ prim, float* __restrict__ tout,
                                                    float* __restrict__ ng, uint32_t* err_out) {
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    f3 ro = mk(__ldg(ox + i), __ldg(oy + i), __ldg(oz + i));
    f3 rd = mk(__ldg(dx + i), __ldg(dy + i), __ldg(dz + i));
    float t = __ldg(tmax + i);
    uint32_t err = 0;
    int32_t p = trace_closest<false>(sc, ro, rd, t, nullptr, err);
    prim[i] = p;
    tout[i] = t;
    if (ng) {
        f3 n = p >= 0 ? hit_normal(sc, p, ro, rd, t) : mk(0.0f, 0.0f, 0.0f);
        ng[3 * i + 0] = n.x;
        ng[3 * i + 1] = n.y;
        ng[3 * i + 2] = n.z;
    }
    if (err) atomicOr(err_out, err);
}

__global__ void __launch_bounds__(128) k_trace_rays_counts(SceneView sc, const float* __restrict__ ox,
                                                           const float* __restrict__ oy, const float* __restrict__ oz,
                                                           const float* __restrict__ dx, const float* __restrict__ dy,
                                                           const float* __restrict__ dz,
                                                           const float* __restrict__ tmax, uint64_t n,
                                                           int32_t* __restrict__ prim, float* __restrict__ tout,
                                                           uint32_t* nodes, uint32_t* prims, uint32_t* err_out) {
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    f3 ro = mk(ox[i], oy[i], oz[i]);
    f3 rd = mk(dx[i], dy[i], dz[i]);
    float t = tmax[i];
    uint32_t err = 0;
    TraceCounters c;
    int32_t p = trace_closest<true>(sc, ro, rd, t, &c, err);
    prim[i] = p;
    tout[i] = t;
    nodes[i] = c.nodes;
    prims[i] = c.prims;
    if (err) atomicOr(err_out, err);
}

}  // namespace

void launch_trace_rays_counts(const SceneView& sc, const float* ox, const float* oy, const float* oz, const float* dx,
                              const float* dy, const float* dz, const float* tmax, uint64_t n, int32_t* prim,
                              float* t, uint32_t* nodes, uint32_t* prims, uint32_t* err, cudaStream_t st) {
    if (n == 0) return;
    k_trace_rays_counts<<<(unsigned)((n + 127) / 128), 128, 0, st>>>(sc, ox, oy, oz, dx, dy, dz, tmax, n, prim, t,
                                                                     nodes, prims, err);
}

void launch_trace_rays(const SceneView& sc, const float* ox, const float* oy, const float* oz, const float* dx,
                       const float* dy, const float* dz, const float* tmax, uint64_t n, int32_t* prim, float* t,
                       float* ng, uint32_t* err, int block, cudaStream_t st) {
    (void)block;
    if (n == 0) return;
    k_trace_rays<<<(unsigned)((n + 127) / 128), 128, 0, st>>>(sc, ox, oy, oz, dx, dy, dz, tmax, n, prim, t, ng, err);
}

}  // namespace dev
}  // namespace rgr
