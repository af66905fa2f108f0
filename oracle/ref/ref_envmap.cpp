// kernels/envmap_sampling.cl compiled unchanged through the OpenCL shim.
// Called: alias_method, sample_envmap_6axis, envmap_index, envmap_pdf,
// envmap_pdf_sixAxis, evaluate_envmap_pdf_stage, evaluate_envmap_6axis_pdf_stage.
// Not called: sample_from_fragment (multi-component vector literal) and the
// two sampling stages that use it.
#include "clshim_pre.h"
namespace rk_env {
#include "clshim_body.h"
#include "envmap_sampling.cl"
}
extern "C" uint32_t ref_alias_method(uint32_t* state4, const void* buckets, uint32_t count) {
    return rk_env::alias_method((rk_env::uint4*)state4, (const rk_env::AliasBucket*)buckets, count);
}
extern "C" void ref_sample_envmap_6axis(float* pdf, uint32_t* idx, uint32_t* state4, const float* n3,
                                        const float* pdfsN, const void* bucketsN, uint32_t count) {
    using namespace rk_env;
    sample_envmap_6axis(pdf, idx, (uint4*)state4, float3(n3[0], n3[1], n3[2]), pdfsN, (const AliasBucket*)bucketsN,
                        count);
}
extern "C" int32_t ref_envmap_index(const float* wi3, int32_t w, int32_t h) {
    return rk_env::envmap_index(rk_env::float3(wi3[0], wi3[1], wi3[2]), w, h);
}
extern "C" float ref_envmap_pdf_six_axis(const float* wi3, const float* n3, const float* pdfsN, int32_t w, int32_t h) {
    using namespace rk_env;
    return envmap_pdf_sixAxis(float3(wi3[0], wi3[1], wi3[2]), float3(n3[0], n3[1], n3[2]), pdfsN, w, h);
}
extern "C" void ref_evaluate_envmap_6axis_pdf_stage(const void* ext, const uint32_t* qi, const uint32_t* qc,
                                                    void* incident, const float* pdfsN, uint32_t w, uint32_t h,
                                                    uint64_t n) {
    using namespace rk_env;
    rgr_cl_gsize = n;
    for (uint64_t i = 0; i < n; ++i) {
        rgr_cl_gid = i;
        evaluate_envmap_6axis_pdf_stage((const ExtensionResult*)ext, qi, qc, (IncidentSample*)incident, pdfsN, w, h);
    }
}
extern "C" void ref_evaluate_envmap_pdf_stage(const uint32_t* qi, const uint32_t* qc, void* incident,
                                              const float* pdfs, uint32_t w, uint32_t h, uint64_t n) {
    using namespace rk_env;
    rgr_cl_gsize = n;
    for (uint64_t i = 0; i < n; ++i) {
        rgr_cl_gid = i;
        evaluate_envmap_pdf_stage(qi, qc, (IncidentSample*)incident, pdfs, w, h);
    }
}
