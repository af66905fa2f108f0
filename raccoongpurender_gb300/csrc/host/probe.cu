// probe.cu — read-bandwidth probe: the denominator of the closest-hit roofline.
//
// The closest-hit working set of the 1.31M-triangle scene (64-byte inner nodes
// plus 48-byte primitive records, about 92 MB) fits in the 129 MB L2, so the
// roof that bounds the traversal is the L2 read bandwidth, not HBM.  This
// probe measures it: a grid of 256-thread blocks (a multiple of the SM count)
// streams a buffer of the chosen size with 16-byte loads that bypass L1
// (ld.global.cg), four loads in flight per thread, the buffer read several
// times per launch (at least 1 GiB); the first launch brings the buffer into
// L2, the timed launches read it from there.  A buffer larger
// than L2 measures HBM instead.  Diagnostic entry point: it allocates its own
// buffer and changes no device setting.
#include <cuda_runtime.h>

#include <algorithm>
#include <string>

#include "../rgr_internal.h"

namespace {

__device__ __forceinline__ uint4 ld_cg(const uint4* p) {
    uint4 v;
    asm volatile("ld.global.cg.v4.u32 {%0, %1, %2, %3}, [%4];"
                 : "=r"(v.x), "=r"(v.y), "=r"(v.z), "=r"(v.w)
                 : "l"(p));
    return v;
}

// `passes` reads of the whole buffer per launch, so that launch overhead does not
// count against a buffer that L2 serves in a few microseconds
__global__ void __launch_bounds__(256) k_read_probe(const uint4* __restrict__ buf, uint64_t n16, uint32_t passes,
                                                    uint32_t* sink) {
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    uint32_t acc = 0;
    for (uint32_t p = 0; p < passes; ++p) {
        uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
        for (; i + 3 * stride < n16; i += 4 * stride) {
            uint4 a = ld_cg(buf + i), b = ld_cg(buf + i + stride), c = ld_cg(buf + i + 2 * stride),
                  d = ld_cg(buf + i + 3 * stride);
            acc ^= a.x ^ a.y ^ a.z ^ a.w ^ b.x ^ b.y ^ b.z ^ b.w ^ c.x ^ c.y ^ c.z ^ c.w ^ d.x ^ d.y ^ d.z ^ d.w;
        }
        for (; i < n16; i += stride) {
            uint4 a = ld_cg(buf + i);
            acc ^= a.x ^ a.y ^ a.z ^ a.w;
        }
    }
    if (acc == 0x9e3779b9u) *sink = acc;  // keeps the loads; the buffer is zero, so never taken
}

}  // namespace

extern "C" int rgr_probe_read_bandwidth(int32_t device, uint64_t bytes, int32_t reps, double* gbs) {
    if (gbs == nullptr || reps < 1 || bytes < (1u << 20) || bytes > (64ull << 30)) {
        rgr::set_error("rgr_probe_read_bandwidth: bytes in [1 MiB, 64 GiB], reps >= 1");
        return RGR_E_INVALID;
    }
    int prev = 0;
    cudaGetDevice(&prev);
    cudaError_t e = cudaSetDevice(device);
    if (e != cudaSuccess) {
        rgr::set_error(std::string("rgr_probe_read_bandwidth: ") + cudaGetErrorString(e));
        return RGR_E_NODEVICE;
    }
    int sms = 0;
    e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    void* buf = nullptr;
    uint32_t* sink = nullptr;
    cudaStream_t st = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    const uint64_t n16 = bytes / 16;
    if (e == cudaSuccess) e = cudaMalloc(&buf, n16 * 16);
    if (e == cudaSuccess) e = cudaMalloc(&sink, 4);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreate(&e0);
    if (e == cudaSuccess) e = cudaEventCreate(&e1);
    if (e == cudaSuccess) e = cudaMemsetAsync(buf, 0, n16 * 16, st);
    float ms = 0.0f;
    // at least 1 GiB read per launch
    const uint32_t passes = (uint32_t)std::max<uint64_t>(1, (1ull << 30) / (n16 * 16));
    if (e == cudaSuccess) {
        const int grid = sms * 8;  // 8 resident 256-thread blocks per SM
        for (int w = 0; w < 3; ++w) k_read_probe<<<grid, 256, 0, st>>>((const uint4*)buf, n16, 1u, sink);
        cudaEventRecord(e0, st);
        for (int r = 0; r < reps; ++r) k_read_probe<<<grid, 256, 0, st>>>((const uint4*)buf, n16, passes, sink);
        cudaEventRecord(e1, st);
        e = cudaEventSynchronize(e1);
        if (e == cudaSuccess) e = cudaGetLastError();
        if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
    }
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    if (st) cudaStreamDestroy(st);
    if (sink) cudaFree(sink);
    if (buf) cudaFree(buf);
    cudaSetDevice(prev);
    if (e != cudaSuccess) {
        rgr::set_error(std::string("rgr_probe_read_bandwidth: ") + cudaGetErrorString(e));
        return e == cudaErrorMemoryAllocation ? RGR_E_OOM : RGR_E_CUDA;
    }
    *gbs = (double)(n16 * 16) * passes * reps / (ms * 1e-3) / 1e9;
    return RGR_OK;
}
