// kernels/extension_ray_cast_stackless.cl (with slab.cl, types.cl,
// intersect_triangle.cl) compiled unchanged through the OpenCL shim.
#include "clshim_pre.h"
namespace rk_trace {
#include "clshim_body.h"
#include "extension_ray_cast_stackless.cl"
}
extern "C" void ref_extension_ray_cast(void* paths, void* results, const void* nodes, const uint32_t* prim_ids,
                                       const uint32_t* indices, const float* points, int32_t sphere_begin,
                                       const float* spheres, uint64_t n) {
    using namespace rk_trace;
    rgr_cl_gsize = n;
    for (uint64_t i = 0; i < n; ++i) {
        rgr_cl_gid = i;
        extension_ray_cast((WavefrontPath*)paths, (ExtensionResult*)results, (StacklessBVHNode*)nodes,
                           (uint*)prim_ids, (uint*)indices, (float4*)points, sphere_begin, (float4*)spheres);
    }
}
// rays as float[8] (ro.xyz, tmax, rd.xyz, pad); prim -1 and t = tmax on miss
extern "C" void ref_trace(const void* nodes, const uint32_t* prim_ids, const uint32_t* indices, const float* points,
                          int32_t sphere_begin, const float* spheres, const float* rays, uint64_t n, int32_t* prim,
                          float* t, float* ng) {
    using namespace rk_trace;
    rgr_cl_gsize = n;
    for (uint64_t i = 0; i < n; ++i) {
        WavefrontPath p;
        memset(&p, 0, sizeof(p));
        ExtensionResult r;
        memset(&r, 0, sizeof(r));
        const float* ray = rays + 8 * i;
        p.ro = float3(ray[0], ray[1], ray[2]);
        p.rd = float3(ray[4], ray[5], ray[6]);
        r.tmin = ray[3];
        r.hit_surface_material = -1;
        rgr_cl_gid = 0;
        extension_ray_cast(&p, &r, (StacklessBVHNode*)nodes, (uint*)prim_ids, (uint*)indices, (float4*)points,
                           sphere_begin, (float4*)spheres);
        prim[i] = r.hit_surface_material;
        t[i] = r.tmin;
        if (ng) {
            ng[3 * i] = r.Ng.x;
            ng[3 * i + 1] = r.Ng.y;
            ng[3 * i + 2] = r.Ng.z;
        }
    }
}
