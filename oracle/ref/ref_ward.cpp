// kernels/ward.cl compiled unchanged through the OpenCL shim.
// Called: ward_stage, pdf_ward, and sample_or_eval_ward_stage only for items
// whose strategy is not BSDF sampling (sample_ward builds its half vector
// with multi-component vector literals).
#include "clshim_pre.h"
namespace rk_ward {
#include "clshim_body.h"
#include "ward.cl"
}
extern "C" float ref_pdf_ward(const float* wo, const float* wi, const float* z, float alpha) {
    using namespace rk_ward;
    return pdf_ward(float3(wo[0], wo[1], wo[2]), float3(wi[0], wi[1], wi[2]), float3(z[0], z[1], z[2]), alpha);
}
extern "C" void ref_sample_or_eval_ward_stage(void* paths, const void* ext, const void* materials, const void* wards,
                                              uint32_t* rng, const uint32_t* qi, const uint32_t* qc, void* incident,
                                              uint64_t n) {
    using namespace rk_ward;
    rgr_cl_gsize = n;
    for (uint64_t i = 0; i < n; ++i) {
        rgr_cl_gid = i;
        sample_or_eval_ward_stage((WavefrontPath*)paths, (const ExtensionResult*)ext, (const Material*)materials,
                                  (const Ward*)wards, (uint4*)rng, qi, qc, (IncidentSample*)incident);
    }
}
extern "C" void ref_ward_stage(void* paths, const void* ext, void* shading, const uint32_t* qi, const uint32_t* qc,
                               const void* materials, const void* wards, void* incident, uint64_t n) {
    using namespace rk_ward;
    rgr_cl_gsize = n;
    for (uint64_t i = 0; i < n; ++i) {
        rgr_cl_gid = i;
        ward_stage((WavefrontPath*)paths, (const ExtensionResult*)ext, (ShadingResult*)shading, qi, qc,
                   (const Material*)materials, (const Ward*)wards, (IncidentSample*)incident);
    }
}
