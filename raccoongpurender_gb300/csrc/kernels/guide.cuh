// guide.cuh — learned path guiding: the network's device view, the
// von Mises-Fisher mixture it parameterises, and the per-render buffers that
// connect it to the wavefront (inference per bounce, training samples
// recorded by the tracer).
//
// The network maps a shading vertex (position, normal facing the outgoing
// direction, outgoing direction) to 8 vMF lobes over the incident direction.
// At Lambertian, Ward and in-volume vertices the guided renderer adds it as a
// third strategy of the one-sample MIS that already combines BSDF and
// envmap sampling:  p(wi) = s_bsdf p_bsdf + s_guide p_guide + s_env p_env,
// so every sample stays unbiased whatever the network has learned.
#pragma once
#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include "wavefront.cuh"

namespace rgr {
namespace dev {

constexpr int kGuideLobes = 8;
constexpr int kGuideLayers = 5;
constexpr int kGuideWidth = 64;
constexpr int kGuideWeights = kGuideLayers * kGuideWidth * kGuideWidth;  // W[l][in][out], zero padded
constexpr int kGuideBiases = kGuideLayers * kGuideWidth;
constexpr int kGuideParams = kGuideWeights + kGuideBiases;
constexpr int kGuideInputs = 36;   // 9 coordinates x 2 octaves x (sin, cos)
constexpr int kGuideOutputs = 40;  // field-major: output 8 f + i is field f (mean xyz, concentration, weight) of lobe i
constexpr int kGuideSelOutput = 40;  // the logit z of the guide's share of the non-envmap sampling probability
constexpr int kGuideNetOutputs = 41; // the mixture's outputs and the selection logit
constexpr int kGuideRowOutputs = 48; // raw outputs per row written by the inference entry point (41 and 7 zeros)
// the guide's share a = kGuideAlphaMin + (kGuideAlphaMax - kGuideAlphaMin) sigmoid(z): the
// BSDF always keeps at least 5 % of the non-envmap probability, and the guide as much
constexpr float kGuideAlphaMin = 0.05f, kGuideAlphaMax = 0.95f;
constexpr float kGuideKappaMax = 5000.0f;
constexpr float kGuideLogitBound = 5.0f;    // lobe weight logits lie in (-5, 5)
constexpr float kGuideNormPenalty = 0.01f;  // pull of each direction output's length toward 1
// one CTA's slot in the tcgen05 training kernel's partials buffer: its weight
// gradient, bias gradient and loss (kGuideParams + 1 floats), padded to 128 bytes
constexpr uint32_t kGuidePartStride = kGuideParams + 32;

// position normalisation of the input encoding (scene bounds)
struct GuideParams {
    float lo[3];
    float inv_ext[3];
};

// the network and its optimiser state (device pointers)
struct GuideView {
    float* w;              // FP32 master weights, kGuideWeights
    float* b;              // FP32 biases, kGuideBiases
    __nv_bfloat16* wbf;    // BF16 copy of w that the tensor cores read
    unsigned char* wt_sw;  // the BF16 weights as the tcgen05 kernel stages them: per layer W^T
                           // (64 output rows x 64 inputs, K-major, 128-byte swizzle), 8 KB each
    float* gW;             // gradient accumulators (zeroed by Adam)
    float* gb;
    float* m;              // Adam moments, kGuideParams each (weights then biases)
    float* v;
    float* loss;           // sum of sample losses of the last batch
    GuideParams params;
    uint32_t stall_mma;    // failure-detection tests: the tcgen05 inference kernel's MMA warps
                           // issue nothing, so its row threads' bounded waits run out
};

// wt_sw: the five W^T tiles (8 KB each), then per layer a 16-wide K chunk
// (64 output rows x 16 bf16, 2 KB) whose columns 0 and 1 hold each bias as the
// sum of two bf16 values; the tcgen05 kernel multiplies it by a chunk of ones
// to start the accumulator at the bias (layers 1..4; layer 0's chunk stays
// zero, wt_bias_offset).
constexpr uint32_t kGuideWtMainBytes = kGuideLayers * 64 * 128;
constexpr uint32_t kGuideWtBytes = kGuideWtMainBytes + kGuideLayers * 64 * 32;

// byte offset of 16-byte chunk c of row r in a K-major 128-byte-swizzled tile
// (the chunk sits at position c ^ (r % 8) of its 128-byte line; 8-line groups
// are 1024 bytes apart)
__host__ __device__ __forceinline__ uint32_t sw128_offset(uint32_t r, uint32_t c) {
    return (r >> 3) * 1024u + (r & 7u) * 128u + ((c ^ (r & 7u)) << 4);
}
// where weight W[l][in][out] lives in wt_sw
__host__ __device__ __forceinline__ uint32_t wt_sw_offset(uint32_t l, uint32_t in, uint32_t out) {
    return l * 8192u + sw128_offset(out, in >> 3) + (in & 7u) * 2u;
}
// byte offset of element (r, k) of a K-major 16-wide chunk without swizzle:
// 8-row x 16-byte core matrices, the two K halves 128 bytes apart, 8-row
// groups 256 bytes apart
__host__ __device__ __forceinline__ uint32_t k16_offset(uint32_t r, uint32_t k) {
    return (r >> 3) * 256u + (k >> 3) * 128u + (r & 7u) * 16u + (k & 7u) * 2u;
}
// where part h (0: bf16 of the bias, 1: bf16 of the remainder) of the bias of
// output `out` of layer l lives in wt_sw.  Layer 0's rides on the padding
// inputs 36 and 37 of its W^T tile instead (the kernel sets those inputs to
// 1.0), which saves that layer the bias chunk's MMA.
__host__ __device__ __forceinline__ uint32_t wt_bias_offset(uint32_t l, uint32_t out, uint32_t h) {
    return l == 0u ? wt_sw_offset(0u, (uint32_t)kGuideInputs + h, out)
                   : kGuideWtMainBytes + l * 2048u + k16_offset(out, h);
}
// W^T entries of wt_sw that hold layer 0's bias, not a (zero) padding weight
__host__ __device__ __forceinline__ bool wt_is_bias_slot(uint32_t l, uint32_t in) {
    return l == 0u && (in == (uint32_t)kGuideInputs || in == (uint32_t)kGuideInputs + 1u);
}

// ------------------------------------------------------------ vMF mixture
// vMF density on the sphere, kappa / (2 pi (1 - e^{-2 kappa})) e^{kappa (c - 1)}
__device__ __forceinline__ float vmf_pdf(float kappa, float c) {
    return kappa / (6.283185307179586f * -expm1f(-2.0f * kappa)) * expf(kappa * (c - 1.0f));
}
__device__ __forceinline__ float softplus(float x) { return x > 20.0f ? x : log1pf(expf(x)); }
__device__ __forceinline__ float sigmoid(float x) { return 1.0f / (1.0f + expf(-x)); }

// One lobe of the mixture from its five raw outputs (the training kernels):
//   mean = o / |o|, kappa = min(softplus(o_3) + 0.01, kGuideKappaMax),
//   logit = kGuideLogitBound tanh(o_4 / kGuideLogitBound)
// (bounded so that no lobe's weight can saturate to zero and stop learning).
struct LobeOut {
    float mx, my, mz, kappa, norm, th, logit;
};
__device__ __forceinline__ LobeOut lobe_of(float o0, float o1, float o2, float o3, float o4) {
    LobeOut L;
    L.norm = fmaxf(sqrtf(o0 * o0 + o1 * o1 + o2 * o2), 1.0e-12f);
    L.mx = o0 / L.norm;
    L.my = o1 / L.norm;
    L.mz = o2 / L.norm;
    L.kappa = fminf(softplus(o3) + 0.01f, kGuideKappaMax);
    L.th = tanhf(o4 * (1.0f / kGuideLogitBound));
    L.logit = kGuideLogitBound * L.th;
    return L;
}
// The gradient, with respect to the raw outputs of one lobe (g[0..4] = mean xyz,
// concentration, weight logit), of -wt log q(d) + wt kGuideNormPenalty (|o| - 1)^2,
// given the lobe L, its mixture weight pi and its responsibility r = pi f / q
// for the sample direction d; raw_k is the lobe's raw concentration output.  The
// second term holds the length of each direction output near 1 (the direction
// o / |o| does not depend on it, and the first term's gradient shrinks as 1 / |o|).
__device__ __forceinline__ void lobe_grad(const LobeOut& L, float pi, float r, float raw_k, float dx, float dy,
                                          float dz, float wt, float* g) {
    // weight logit: d(-log q)/d l = -(r - pi), through l = B tanh(o / B)
    g[4] = -wt * (r - pi) * (1.0f - L.th * L.th);
    // concentration: d log f / d kappa = 1/kappa - 2 e^{-2k} / (1 - e^{-2k}) + (mu.d - 1)
    const float k = L.kappa;
    const float md = L.mx * dx + L.my * dy + L.mz * dz;
    const float dlogf = 1.0f / k - 2.0f * expf(-2.0f * k) / -expm1f(-2.0f * k) + (md - 1.0f);
    const float dk = (softplus(raw_k) + 0.01f < kGuideKappaMax) ? sigmoid(raw_k) : 0.0f;
    g[3] = -wt * r * dlogf * dk;
    // mean: d log f / d mu = kappa d, through mu = o / |o|: (I - mu mu^T) / |o|;
    // plus the length penalty 2 wt c (|o| - 1) mu
    const float gx = -wt * r * k * dx, gy = -wt * r * k * dy, gz = -wt * r * k * dz;
    const float gm = gx * L.mx + gy * L.my + gz * L.mz;
    const float pen = 2.0f * wt * kGuideNormPenalty * (L.norm - 1.0f);
    g[0] = (gx - gm * L.mx) / L.norm + pen * L.mx;
    g[1] = (gy - gm * L.my) / L.norm + pen * L.my;
    g[2] = (gz - gm * L.mz) / L.norm + pen * L.mz;
}

// The inferred mixture of one guided vertex as the shading kernel reads it,
// kGuideMixVecs 16-byte words in global memory (FP16): lobe i's mean xyz and
// kappa in halves 4i..4i+3, the eight weights in halves 32..39, scaled so that
// they sum to the guide's share a of the non-envmap sampling probability at
// the vertex.  Sampling and the pdf decode it the same way (means and weights
// normalised after the FP16 rounding, a = the sum of the stored weights), so
// the density evaluated and the share used are exactly the ones sampled with.
__device__ __forceinline__ uint32_t half2_bits(float lo, float hi) {
    const __half2 h = __floats2half2_rn(lo, hi);
    return *reinterpret_cast<const uint32_t*>(&h);
}
__device__ __forceinline__ float2 half2_float2(uint32_t v) {
    return __half22float2(*reinterpret_cast<const __half2*>(&v));
}
// lobe i of the record: unit mean (xyz) and kappa (w)
__device__ __forceinline__ float4 mixture_lobe(const uint4* p, int i) {
    const uint2 q = __ldg(reinterpret_cast<const uint2*>(p) + i);
    const float2 xy = half2_float2(q.x), zk = half2_float2(q.y);
    const float inv = rsqrtf(fmaxf(xy.x * xy.x + xy.y * xy.y + zk.x * zk.x, 1.0e-30f));
    return make_float4(xy.x * inv, xy.y * inv, zk.x * inv, zk.y);
}
// The vMF density as the shading kernel evaluates it: the SFU's exponential and
// reciprocal.  Sampling (mixture_sample) and evaluation (mixture_pdf) decode the
// record with the same functions, so the pdf a sample is weighted with is the
// density it was drawn from up to the SFU's relative error (about 2^-21); the
// compiler's IEEE division and square root, which the path arithmetic needs for
// parity with the reference, are not used here.
__device__ __forceinline__ float vmf_pdf_fast(float kappa, float c) {
    return __fdividef(kappa, 6.283185307179586f * (1.0f - __expf(-2.0f * kappa))) * __expf(kappa * (c - 1.0f));
}
// the guide's share of the non-envmap probability at the vertex: the sum of the stored weights
__device__ __forceinline__ float mixture_alpha(const uint4* p) {
    const uint4 q = __ldg(p + 4);
    const float2 a = half2_float2(q.x), b = half2_float2(q.y), c = half2_float2(q.z), d = half2_float2(q.w);
    return ((a.x + a.y) + (b.x + b.y)) + ((c.x + c.y) + (d.x + d.y));
}
__device__ __forceinline__ float alpha_of(float z) {
    return kGuideAlphaMin + (kGuideAlphaMax - kGuideAlphaMin) / (1.0f + __expf(-z));
}
// The gradient, with respect to the selection logit z, of the selection term
// -wt log(a q + (1 - a) pb), a = alpha_of(z), with the mixture density q held
// fixed; zero for a sample without a BSDF pdf (pb = 0).  Accurate functions:
// the training kernels use it.
__device__ __forceinline__ float selection_grad(float z, float q, float pb, float wt) {
    if (!(pb > 0.0f)) return 0.0f;
    const float sg = 1.0f / (1.0f + expf(-z));
    const float a = kGuideAlphaMin + (kGuideAlphaMax - kGuideAlphaMin) * sg;
    const float mix = fmaxf(a * q + (1.0f - a) * pb, 1.0e-30f);
    return -wt * (q - pb) / mix * (kGuideAlphaMax - kGuideAlphaMin) * sg * (1.0f - sg);
}
// the eight weights of the record, normalised
__device__ __forceinline__ void mixture_weights(const uint4* p, float* w) {
    const uint4 q = __ldg(p + 4);
    const float2 a = half2_float2(q.x), b = half2_float2(q.y), c = half2_float2(q.z), d = half2_float2(q.w);
    w[0] = a.x, w[1] = a.y, w[2] = b.x, w[3] = b.y, w[4] = c.x, w[5] = c.y, w[6] = d.x, w[7] = d.y;
    float sum = 0.0f;
#pragma unroll
    for (int i = 0; i < kGuideLobes; ++i) sum += w[i];
    const float inv = __fdividef(1.0f, fmaxf(sum, 1.0e-30f));
#pragma unroll
    for (int i = 0; i < kGuideLobes; ++i) w[i] *= inv;
}
__device__ __forceinline__ float mixture_pdf(const uint4* p, float dx, float dy, float dz) {
    float w[kGuideLobes];
    mixture_weights(p, w);
    float pdf = 0.0f;
#pragma unroll
    for (int i = 0; i < kGuideLobes; ++i) {
        const float4 L = mixture_lobe(p, i);
        pdf += w[i] * vmf_pdf_fast(L.w, L.x * dx + L.y * dy + L.z * dz);
    }
    return pdf;
}
// Sample the mixture with three uniforms: lobe by weight, then the vMF
// cosine by inversion (W = 1 + log(u + (1 - u) e^{-2 kappa}) / kappa) and a
// uniform azimuth in the lobe's frame (Frisvad / Duff branchless basis).
__device__ __forceinline__ void mixture_sample(const uint4* p, float u0, float u1, float u2, float* d) {
    float w[kGuideLobes];
    mixture_weights(p, w);
    int k = kGuideLobes - 1;
    float acc = 0.0f;
#pragma unroll
    for (int i = 0; i < kGuideLobes - 1; ++i) {
        acc += w[i];
        if (u0 < acc && k == kGuideLobes - 1) k = i;
    }
    const float4 L = mixture_lobe(p, k);
    const float kappa = L.w;
    float wc = 1.0f + __fdividef(__logf(u1 + (1.0f - u1) * __expf(-2.0f * kappa)), kappa);
    wc = fminf(fmaxf(wc, -1.0f), 1.0f);
    const float s = sqrtf(fmaxf(0.0f, 1.0f - wc * wc));
    float sp, cp;
    __sincosf(6.283185307179586f * u2, &sp, &cp);
    const float sign = L.z >= 0.0f ? 1.0f : -1.0f;
    const float a = __fdividef(-1.0f, sign + L.z);  // |sign + z| >= 1
    const float bb = L.x * L.y * a;
    const float tx = 1.0f + sign * L.x * L.x * a, ty = sign * bb, tz = -sign * L.x;
    const float bx = bb, by = sign + L.y * L.y * a, bz = -L.y;
    float x = wc * L.x + s * (cp * tx + sp * bx);
    float y = wc * L.y + s * (cp * ty + sp * by);
    float z = wc * L.z + s * (cp * tz + sp * bz);
    const float n = rsqrtf(x * x + y * y + z * z);
    d[0] = x * n;
    d[1] = y * n;
    d[2] = z * n;
}

// ------------------------------------------------------------ launchers (guide_mlp.cu)
size_t guide_infer_smem();
size_t guide_train_smem();
// opt the kernels into their dynamic shared memory on the current device (cudaError_t)
int guide_kernel_attributes();
// persistent grid of the inference kernels (resident CTAs)
int guide_infer_grid(int num_sms);
// raw network outputs (kGuideRowOutputs floats per row: the 40 mixture outputs, the
// selection logit, zeros) of rows of 16 floats (x, n, wo in the first 9)
void launch_guide_infer(const GuideView& g, const float* rows, uint32_t n, float* out, int grid, cudaStream_t st);
// mixtures of this bounce's guided queue items (Lambertian, Ward, in-volume when enabled)
void launch_guide_infer_paths(const GuideView& g, const PathsView& p, const QueueView& q, const GuideRenderD& gd,
                              int grid, cudaStream_t st);
// one training iteration over min(*count, cap) samples: gradients into gW/gb,
// loss; nothing while fewer than min_count samples are in
void launch_guide_train(const GuideView& g, const float* samples, const uint32_t* count, uint32_t cap,
                        uint32_t min_count, const float* wsum, float weight_scale, int grid, cudaStream_t st);
// Adam on the accumulated gradients when *count > 0 and >= min_count; iteration number from *iter + 1
void launch_guide_adam(const GuideView& g, const uint32_t* count, uint32_t min_count, const uint32_t* iter,
                       float lr, float beta1, float beta2, float eps, cudaStream_t st);
// *count = n, in stream order (the sample count of an iteration enqueued from the host)
void launch_guide_set_count(uint32_t* count, uint32_t n, cudaStream_t st);
// after an iteration: advance *iter, log the loss, retune the acceptance, reset counters
void launch_guide_finish(const GuideView& g, const GuideTrainD& t, cudaStream_t st);

// tcgen05 / TMEM training (guide_train_tc.cu): one iteration over min(*count, cap)
// samples into the CTAs' slots of `part` (grid x kGuidePartStride floats), nothing
// while fewer than min_count samples are in; then launch_guide_grad_reduce sums
// the grid's slots into gW, gb and the loss.  A timed-out wait sets bit 1 of *err.
size_t guide_train_tc_smem();
int guide_train_tc_attributes();  // cudaError_t of opting the kernel into its shared memory
void launch_guide_train_tc(const GuideView& g, const float* samples, const uint32_t* count, uint32_t cap,
                           uint32_t min_count, const float* wsum, float weight_scale, int grid, float* part,
                           uint32_t* err, cudaStream_t st);
void launch_guide_grad_reduce(const GuideView& g, const float* part, uint32_t nparts, const uint32_t* count,
                              uint32_t min_count, cudaStream_t st);

// tcgen05 / TMEM inference (guide_tc.cu): same results as the mma.sync kernels up
// to FP32 accumulation order; a timed-out tensor-core wait sets bit 0 of *err
size_t guide_tc_smem();
int guide_tc_attributes();  // cudaError_t of opting the kernels into their shared memory
int guide_tc_grid(int num_sms);
void launch_guide_infer_tc(const GuideView& g, const float* rows, uint32_t n, float* out, int grid, uint32_t* err,
                           cudaStream_t st);
void launch_guide_infer_paths_tc(const GuideView& g, const PathsView& p, const QueueView& q, const GuideRenderD& gd,
                                 int grid, uint32_t* err, cudaStream_t st);

}  // namespace dev
}  // namespace rgr
