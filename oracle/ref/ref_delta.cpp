// kernels/delta_materials.cl compiled unchanged through the OpenCL shim
// (its vector literals all have equal components).
#include "clshim_pre.h"
namespace rk_delta {
#include "clshim_body.h"
#include "delta_materials.cl"
}
static char g_empty_storage[1 << 16];
extern "C" void ref_delta_materials(void* paths, uint32_t* rng, const void* ext, void* shading, uint32_t* sqi,
                                    uint32_t* sqc, uint32_t* dqi, uint32_t* dqc, const void* materials, uint64_t n) {
    using namespace rk_delta;
    rgr_cl_gsize = n;
    for (uint64_t i = 0; i < n; ++i) {
        rgr_cl_gid = i;
        delta_materials((WavefrontPath*)paths, (uint4*)rng, (const ExtensionResult*)ext, (ShadingResult*)shading, sqi,
                        sqc, dqi, dqc, (const Material*)materials, (const Specular*)g_empty_storage,
                        (const Dierectric*)g_empty_storage);
    }
}
