// kernels/lambertian.cl compiled unchanged through the OpenCL shim.
// Called: lambertian_stage, and sample_or_eval_lambertian_stage only for
// items whose strategy is not BSDF sampling (its sampling branch uses
// multi-component vector literals).
#include "clshim_pre.h"
namespace rk_lam {
#include "clshim_body.h"
#include "lambertian.cl"
}
extern "C" void ref_sample_or_eval_lambertian_stage(const void* ext, uint32_t* rng, const uint32_t* qi,
                                                    const uint32_t* qc, void* incident, uint64_t n) {
    using namespace rk_lam;
    rgr_cl_gsize = n;
    for (uint64_t i = 0; i < n; ++i) {
        rgr_cl_gid = i;
        sample_or_eval_lambertian_stage((const ExtensionResult*)ext, (uint4*)rng, qi, qc, (IncidentSample*)incident);
    }
}
extern "C" void ref_lambertian_stage(void* paths, const void* ext, void* shading, const uint32_t* qi,
                                     const uint32_t* qc, const void* materials, const void* lambertians,
                                     void* incident, uint64_t n) {
    using namespace rk_lam;
    rgr_cl_gsize = n;
    for (uint64_t i = 0; i < n; ++i) {
        rgr_cl_gid = i;
        lambertian_stage((WavefrontPath*)paths, (const ExtensionResult*)ext, (ShadingResult*)shading, qi, qc,
                         (const Material*)materials, (const Lambertian*)lambertians, (IncidentSample*)incident);
    }
}
