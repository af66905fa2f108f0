// kernels/logic.cl compiled unchanged through the OpenCL shim.  Its envmap
// lookup passes (float2)(u, v) to read_imagef, which the shim cannot
// evaluate, so the harness supplies an image of constant radiance (the shim's
// read_imagef ignores coordinates); callers compare with a constant envmap.
#include "clshim_pre.h"
namespace rk_logic {
#include "clshim_body.h"
#include "logic.cl"
}
extern "C" void ref_logic(void* paths, uint32_t* rng, void* ext, void* shading, const float* env_rgba_const,
                          void* accum, const void* materials, uint32_t** qitems, uint32_t** qcounts, uint64_t n) {
    using namespace rk_logic;
    cl_image img;
    memcpy(img.value, env_rgba_const, 16);
    rgr_cl_gsize = n;
    for (uint64_t i = 0; i < n; ++i) {
        rgr_cl_gid = i;
        logic((WavefrontPath*)paths, (uint4*)rng, (ExtensionResult*)ext, (ShadingResult*)shading, &img,
              (RGB32AccumulationValueType*)accum, (const Material*)materials, qitems[0], qcounts[0], qitems[1],
              qcounts[1], qitems[2], qcounts[2], qitems[3], qcounts[3], qitems[4], qcounts[4], qitems[5], qcounts[5],
              qitems[6], qcounts[6]);
    }
}
