// kernels/homogeneous_volume_through.cl compiled unchanged through the OpenCL shim.
#include "clshim_pre.h"
namespace rk_thr {
#include "clshim_body.h"
#include "homogeneous_volume_through.cl"
}
extern "C" void ref_homogeneous_volume_through(void* paths, void* vlists, void* ext, uint32_t* rng,
                                               const void* materials, const void* volumes, uint64_t n) {
    using namespace rk_thr;
    rgr_cl_gsize = n;
    for (uint64_t i = 0; i < n; ++i) {
        rgr_cl_gid = i;
        homogeneous_volume_through((WavefrontPath*)paths, (InVolumeList*)vlists, (ExtensionResult*)ext, (uint4*)rng,
                                   (const Material*)materials, (const HomogeneousVolume*)volumes);
    }
}
