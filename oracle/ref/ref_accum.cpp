// kernels/accumlation.cl and kernels/stat.cl compiled unchanged through the OpenCL shim.
#include "clshim_pre.h"
namespace rk_acc {
#include "clshim_body.h"
#include "accumlation.cl"
}
extern "C" void ref_accumlation_to_intermediate(const void* src, void* dst, uint64_t n) {
    using namespace rk_acc;
    int holding = 1;
    rgr_cl_gsize = n;
    for (uint64_t i = 0; i < n; ++i) {
        rgr_cl_gid = i;
        accumlation_to_intermediate((RGB32AccumulationValueType*)src, (RGB16IntermediateValueType*)dst, &holding);
    }
}
extern "C" void ref_merge_intermediate(void* a, void* b, uint64_t n) {
    using namespace rk_acc;
    rgr_cl_gsize = n;
    for (uint64_t i = 0; i < n; ++i) {
        rgr_cl_gid = i;
        merge_intermediate((RGB16IntermediateValueType*)a, (RGB16IntermediateValueType*)b);
    }
}
extern "C" void ref_tonemap(void* rgb16, void* rgba8, uint64_t n) {
    using namespace rk_acc;
    rgr_cl_gsize = n;
    for (uint64_t i = 0; i < n; ++i) {
        rgr_cl_gid = i;
        tonemap((RGB16IntermediateValueType*)rgb16, (uchar4*)rgba8);
    }
}
