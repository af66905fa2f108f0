// kernels/peseudo_random.cl compiled unchanged through the OpenCL shim.
#include "clshim_pre.h"
namespace rk_rng {
#include "clshim_body.h"
#include "peseudo_random.cl"
}
extern "C" void ref_random_initialize(uint32_t* states, uint64_t n, uint32_t seed_offset) {
    rgr_cl_gsize = n;
    for (uint64_t i = 0; i < n; ++i) {
        rgr_cl_gid = i;
        rk_rng::random_initialize((rk_rng::uint4*)states, seed_offset);
    }
}
extern "C" void ref_random_uniform(uint32_t* state4, float* out, int32_t n) {
    for (int i = 0; i < n; ++i) out[i] = rk_rng::random_uniform((rk_rng::uint4*)state4);
}
extern "C" void ref_random_uniform_integer(uint32_t* state4, uint64_t* out, int32_t n) {
    for (int i = 0; i < n; ++i) out[i] = rk_rng::random_uniform_integer((rk_rng::uint4*)state4);
}
