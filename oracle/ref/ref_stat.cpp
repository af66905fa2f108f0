// kernels/stat.cl compiled unchanged through the OpenCL shim.
#include "clshim_pre.h"
namespace rk_stat {
#include "clshim_body.h"
#include "stat.cl"
}
extern "C" void ref_stat(const void* accum, uint32_t* all_sample_count, uint64_t n) {
    using namespace rk_stat;
    rgr_cl_gsize = n;
    for (uint64_t i = 0; i < n; ++i) {
        rgr_cl_gid = i;
        stat((RGB32AccumulationValueType*)accum, all_sample_count);
    }
}
