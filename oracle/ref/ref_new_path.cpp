// kernels/new_path.cl compiled unchanged through the OpenCL shim.  Its vector
// literals all have equal components, so the shim evaluates them correctly.
#include "clshim_pre.h"
namespace rk_np {
#include "clshim_body.h"
#include "new_path.cl"
}
extern "C" void ref_initialize_all_as_new_path(uint32_t* qitem, uint32_t* qcount, uint64_t n) {
    rgr_cl_gsize = n;
    for (uint64_t i = 0; i < n; ++i) {
        rgr_cl_gid = i;
        rk_np::initialize_all_as_new_path(qitem, qcount);
    }
}
extern "C" void ref_new_path(const uint32_t* qitem, const uint32_t* qcount, void* paths, void* vlists, void* shading,
                             void* ext, uint32_t* rng, const uint64_t* next_pixel, const orc_camera* cam, uint64_t n) {
    using namespace rk_np;
    StandardCamera c;
    memset(&c, 0, sizeof(c));
    c.eye = float3(cam->eye[0], cam->eye[1], cam->eye[2]);
    c.forward = float3(cam->forward[0], cam->forward[1], cam->forward[2]);
    c.up = float3(cam->up[0], cam->up[1], cam->up[2]);
    c.right = float3(cam->right[0], cam->right[1], cam->right[2]);
    c.imageplane_o = float3(cam->imageplane_o[0], cam->imageplane_o[1], cam->imageplane_o[2]);
    c.imageplane_r = float3(cam->imageplane_r[0], cam->imageplane_r[1], cam->imageplane_r[2]);
    c.imageplane_b = float3(cam->imageplane_b[0], cam->imageplane_b[1], cam->imageplane_b[2]);
    c.image_size.x = cam->image_w;
    c.image_size.y = cam->image_h;
    rgr_cl_gsize = n;
    for (uint64_t i = 0; i < n; ++i) {
        rgr_cl_gid = i;
        new_path(qitem, qcount, (WavefrontPath*)paths, (InVolumeList*)vlists, (ShadingResult*)shading,
                 (ExtensionResult*)ext, (uint4*)rng, (const ulong*)next_pixel, c);
    }
}
extern "C" void ref_finalize_new_path(uint64_t* next_pixel, uint32_t* qcount) {
    rgr_cl_gid = 0;
    rgr_cl_gsize = 1;
    rk_np::finalize_new_path((ulong*)next_pixel, qcount);
}
