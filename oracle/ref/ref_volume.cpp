// kernels/homogeneous_volume.cl compiled unchanged through the OpenCL shim.
// Called: homogeneous_volume_stage, homogeneous_volume_inside_stage, and
// sample_or_eval_homogeneous_volume_inside_stage only for items whose
// strategy is not BSDF sampling (uniform_on_unit_sphere returns a
// multi-component vector literal).
#include "clshim_pre.h"
namespace rk_vol {
#include "clshim_body.h"
#include "homogeneous_volume.cl"
}
extern "C" void ref_homogeneous_volume_stage(void* paths, void* vlists, const void* ext, void* shading,
                                             uint32_t* qi, uint32_t* qc, const void* materials, const void* volumes,
                                             uint64_t n) {
    using namespace rk_vol;
    rgr_cl_gsize = n;
    for (uint64_t i = 0; i < n; ++i) {
        rgr_cl_gid = i;
        homogeneous_volume_stage((WavefrontPath*)paths, (InVolumeList*)vlists, (const ExtensionResult*)ext,
                                 (ShadingResult*)shading, qi, qc, (const Material*)materials,
                                 (const HomogeneousVolume*)volumes);
    }
}
extern "C" void ref_sample_or_eval_homogeneous_volume_inside_stage(uint32_t* rng, const uint32_t* qi,
                                                                   const uint32_t* qc, void* incident, uint64_t n) {
    using namespace rk_vol;
    rgr_cl_gsize = n;
    for (uint64_t i = 0; i < n; ++i) {
        rgr_cl_gid = i;
        sample_or_eval_homogeneous_volume_inside_stage((uint4*)rng, qi, qc, (IncidentSample*)incident);
    }
}
extern "C" void ref_homogeneous_volume_inside_stage(void* paths, const void* ext, void* shading, uint32_t* rng,
                                                    uint32_t* qi, uint32_t* qc, const void* materials,
                                                    const void* volumes, void* incident, uint64_t n) {
    using namespace rk_vol;
    rgr_cl_gsize = n;
    for (uint64_t i = 0; i < n; ++i) {
        rgr_cl_gid = i;
        homogeneous_volume_inside_stage((WavefrontPath*)paths, (const ExtensionResult*)ext, (ShadingResult*)shading,
                                        (uint4*)rng, qi, qc, (const Material*)materials,
                                        (const HomogeneousVolume*)volumes, (IncidentSample*)incident);
    }
}
