// envmap_gpu.cu — the selection probabilities of the seven envmap tables on
// the GPU in FP64: per texel the luminance (FP32, 0.2126/0.7152/0.0722) times
// the texel's solid angle times the table's direction weight (1, or the
// clamped cosine to one cube axis; envmap.hpp:160-242, :291-312), summed per
// table by a fixed-order two-pass reduction (so the result does not depend on
// scheduling) and normalised.  The host pairs the alias tables from them
// (the reference's stack pairing is sequential).
#include <cuda_runtime.h>

#include <string>

#include "../rgr_internal.h"

namespace rgr {
namespace {

constexpr int kTables = 7;
constexpr int kReduceThreads = 256;
constexpr double kTwoPiD = 6.28318530717958647692;
constexpr double kPiD = 3.14159265358979323846;

// weights[k * n + i] of texel i for the 7 tables; geometry as the host builder:
// theta from the row's fragment (acos of its cosine bounds), phi from its
// column, direction (sin t sin p, cos t, sin t cos p) (envmap.hpp:79-86)
__global__ void k_env_weights(const float4* __restrict__ rgba, int w, int h, double* __restrict__ weights) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int n = w * h;
    if (i >= n) return;
    const int y = i / w, x = i % w;
    const double phi_step = kTwoPiD / w, theta_step = kPiD / h;
    const double t0 = theta_step * y, t1 = theta_step * (y + 1);
    const double beg_y = cos(t1), end_y = cos(t0);
    const double theta = (acos(beg_y) + acos(end_y)) * 0.5;
    const double st = sin(theta), ct = cos(theta);
    const double f2 = kTwoPiD - (x + 1) * phi_step, f3 = kTwoPiD - x * phi_step;
    const double phi = (f2 + f3) * 0.5;
    const double d[3] = {st * sin(phi), ct, st * cos(phi)};
    const double sr = ((cos(t0) - cos(t1)) * kTwoPiD) / w;
    const float4 px = rgba[i];
    const float lum = 0.2126f * px.x + 0.7152f * px.y + 0.0722f * px.z;
    const double base = (double)lum * sr;
    weights[i] = base * 1.0;
    for (int k = 1; k < kTables; ++k) {
        const int axis = (k - 1) / 2;
        const double v = ((k - 1) % 2 == 0) ? d[axis] : -d[axis];
        weights[(size_t)k * n + i] = base * fmax(v, 0.0);
    }
}

// fixed-order block sums: partial[k * nb + b] = sum of weights[k][b*chunk ...]
__global__ void k_env_partial(const double* __restrict__ weights, int n, int chunk, double* __restrict__ partial) {
    __shared__ double s[kReduceThreads];
    const int k = blockIdx.y, b = blockIdx.x, nb = gridDim.x;
    const int beg = b * chunk, end = min(n, beg + chunk);
    double acc = 0.0;
    for (int i = beg + threadIdx.x; i < end; i += kReduceThreads) acc += weights[(size_t)k * n + i];
    s[threadIdx.x] = acc;
    __syncthreads();
    for (int o = kReduceThreads / 2; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o) s[threadIdx.x] += s[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) partial[(size_t)k * nb + b] = s[0];
}

// total[k] = sum of the partials in block order; inv[k] = 1 / total[k]
__global__ void k_env_total(const double* __restrict__ partial, int nb, double* __restrict__ inv) {
    if (threadIdx.x != 0) return;
    const int k = blockIdx.x;
    double t = 0.0;
    for (int b = 0; b < nb; ++b) t += partial[(size_t)k * nb + b];
    inv[k] = 1.0 / t;
}

__global__ void k_env_normalize(double* __restrict__ weights, int n, const double* __restrict__ inv) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (size_t)kTables * n) return;
    weights[i] = weights[i] * inv[i / n];
}

bool ok(cudaError_t e, const char* what) {
    if (e == cudaSuccess) return true;
    set_error(std::string("envmap tables on the GPU: ") + what + ": " + cudaGetErrorString(e));
    return false;
}

}  // namespace

int envmap_probabilities_gpu(int device, const float* rgba, int w, int h, double* prob_out) {
    if (w <= 0 || h <= 0) return RGR_E_INVALID;
    const int n = w * h;
    const int chunk = 4096, nb = (n + chunk - 1) / chunk;
    if (!ok(cudaSetDevice(device), "cudaSetDevice")) return RGR_E_CUDA;
    float4* d_rgba = nullptr;
    double *d_w = nullptr, *d_part = nullptr, *d_inv = nullptr;
    int r = RGR_OK;
    cudaStream_t st = nullptr;
    if (!ok(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking), "cudaStreamCreate")) return RGR_E_CUDA;
    if (!ok(cudaMalloc(&d_rgba, sizeof(float4) * (size_t)n), "cudaMalloc") ||
        !ok(cudaMalloc(&d_w, sizeof(double) * kTables * (size_t)n), "cudaMalloc") ||
        !ok(cudaMalloc(&d_part, sizeof(double) * kTables * (size_t)nb), "cudaMalloc") ||
        !ok(cudaMalloc(&d_inv, sizeof(double) * kTables), "cudaMalloc")) {
        r = RGR_E_OOM;
    } else if (!ok(cudaMemcpyAsync(d_rgba, rgba, sizeof(float4) * (size_t)n, cudaMemcpyHostToDevice, st),
                   "cudaMemcpyAsync")) {
        r = RGR_E_CUDA;
    } else {
        k_env_weights<<<(n + 255) / 256, 256, 0, st>>>(d_rgba, w, h, d_w);
        k_env_partial<<<dim3(nb, kTables), kReduceThreads, 0, st>>>(d_w, n, chunk, d_part);
        k_env_total<<<kTables, 32, 0, st>>>(d_part, nb, d_inv);
        const size_t all = (size_t)kTables * n;
        k_env_normalize<<<(unsigned)((all + 255) / 256), 256, 0, st>>>(d_w, n, d_inv);
        if (!ok(cudaGetLastError(), "launch") ||
            !ok(cudaMemcpyAsync(prob_out, d_w, sizeof(double) * all, cudaMemcpyDeviceToHost, st),
                "cudaMemcpyAsync") ||
            !ok(cudaStreamSynchronize(st), "cudaStreamSynchronize"))
            r = RGR_E_CUDA;
    }
    cudaFree(d_rgba);
    cudaFree(d_w);
    cudaFree(d_part);
    cudaFree(d_inv);
    cudaStreamDestroy(st);
    return r;
}

}  // namespace rgr
