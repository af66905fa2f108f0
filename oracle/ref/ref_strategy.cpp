// kernels/mixture_density.cl compiled unchanged through the OpenCL shim
// (work-group size 1, so the two-stage local/global enqueue appends in gid order).
#include "clshim_pre.h"
namespace rk_ms {
#include "clshim_body.h"
#include "mixture_density.cl"
}
extern "C" void ref_strategy_selection(uint32_t* rng, const void* ext, const void* materials, uint32_t* q0i,
                                       uint32_t* q0c, uint32_t* q1i, uint32_t* q1c, uint32_t* q2i, uint32_t* q2c,
                                       uint32_t* q3i, uint32_t* q3c, void* incident, uint64_t n) {
    using namespace rk_ms;
    rgr_cl_gsize = n;
    for (uint64_t i = 0; i < n; ++i) {
        rgr_cl_gid = i;
        strategy_selection((uint4*)rng, (const ExtensionResult*)ext, (const Material*)materials, q0i, q0c, q1i, q1c,
                           q2i, q2c, q3i, q3c, (IncidentSample*)incident);
    }
}
