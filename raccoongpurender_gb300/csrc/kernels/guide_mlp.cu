// guide_mlp.cu — the path-guiding network: a fully fused BF16 MLP on the
// tensor cores (FP32 accumulation), its loss gradient, backward pass and Adam.
//
// Network: 36 frequency-encoding inputs (position, normal, outgoing
// direction), four hidden layers of 64 with ReLU, 40 outputs = 8 von
// Mises-Fisher lobes x (mean direction xyz, concentration, weight).  Every
// layer is stored as a 64 x 64 matrix W[l][in][out] (padding rows and columns
// are zero, receive zero gradient and stay zero under Adam), so one code path
// serves all five layers.
//
// Tensor-core tiling (mma.sync m16n8k16 bf16 -> f32): a warp owns 16 rows.
// Forward keeps the activations in registers from layer to layer: the
// accumulator fragment of two adjacent m16n8 tiles is exactly the A-operand
// fragment of the next m16n8k16 product, so nothing moves between layers
// except through bias + ReLU + bf16 conversion.  Weights live in shared
// memory as W[in][out] (row stride 72 bf16, so the 8 rows an ldmatrix phase
// reads fall in distinct banks); the forward B operand is loaded with
// ldmatrix.trans, the backward one with plain 32-bit loads.  Training
// processes 64-row chunks per CTA: the layer inputs of the chunk stay in
// shared memory, dW = A^T dY runs on the tensor cores with the chunk's rows as
// the reduction dimension, and each warp accumulates its 16 input rows of dW
// in shared FP32 across all chunks of the CTA; one atomicAdd per weight per
// CTA flushes it.
#include <cuda_bf16.h>

#include "guide.cuh"

namespace rgr {
namespace dev {
namespace {

constexpr int kH = kGuideWidth;  // padded width of every layer
constexpr int kLayers = kGuideLayers;
constexpr int kStride = 72;      // shared-memory row stride of bf16 tiles (elements)
constexpr int kWarps = 4;        // warps per CTA (training and inference)
constexpr int kRows = 16 * kWarps;

__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi) {
    __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<uint32_t*>(&v);
}
__device__ __forceinline__ float bf16_lo(uint32_t v) { return __uint_as_float(v << 16); }
__device__ __forceinline__ float bf16_hi(uint32_t v) { return __uint_as_float(v & 0xffff0000u); }

__device__ __forceinline__ void mma16816(float* d, const uint32_t* a, uint32_t b0, uint32_t b1) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}
__device__ __forceinline__ void ldsm_x4_trans(uint32_t* r, const void* smem_row) {
    const uint32_t a = (uint32_t)__cvta_generic_to_shared(smem_row);
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.trans.shared.b16 {%0,%1,%2,%3}, [%4];\n"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
                 : "r"(a));
}

// ---------------------------------------------------------------- encoding
// Frequency encoding: for v in (position mapped to [0,1]^3, (n+1)/2,
// (wo+1)/2) and octave k in {0, 1}: sin(2^k pi v_c), cos(2^k pi v_c).  The
// lowest frequency has period 2, so that cos(pi v) is monotonic on [0, 1] and
// opposite directions (v = 0 and v = 1) encode differently.
__device__ __forceinline__ void encode(const float* x9, const GuideParams& gp, float* f36) {
    float v[9];
    for (int c = 0; c < 3; ++c) {
        v[c] = (x9[c] - gp.lo[c]) * gp.inv_ext[c];
        v[3 + c] = 0.5f * (x9[3 + c] + 1.0f);
        v[6 + c] = 0.5f * (x9[6 + c] + 1.0f);
    }
    int o = 0;
    for (int i = 0; i < 9; ++i) {
        for (int k = 0; k < 2; ++k) {
            float s, c;
            sincospif(v[i] * (float)(1 << k), &s, &c);
            f36[o++] = s;
            f36[o++] = c;
        }
    }
}

// ---------------------------------------------------------------- vMF mixture
__device__ __forceinline__ float softplus(float x) { return x > 20.0f ? x : log1pf(expf(x)); }
__device__ __forceinline__ float sigmoid(float x) { return 1.0f / (1.0f + expf(-x)); }

// raw outputs (5 per lobe: mean xyz, concentration, weight logit) -> mixture
//   mean = o / |o|, kappa = min(softplus(o_k) + 0.01, kGuideKappaMax),
//   weight = softmax over the 8 bounded logits kGuideLogitBound tanh(o_w / kGuideLogitBound)
// (bounded so that no lobe's weight can saturate to zero and stop learning)
__device__ __forceinline__ void mixture_from_raw(const float* o, GuideMixture& m, float* norms, float* th) {
    float lg[kGuideLobes];
    float mx = -3.0e38f;
    for (int i = 0; i < kGuideLobes; ++i) {
        th[i] = tanhf(o[5 * i + 4] * (1.0f / kGuideLogitBound));
        lg[i] = kGuideLogitBound * th[i];
        mx = fmaxf(mx, lg[i]);
    }
    float den = 0.0f;
    for (int i = 0; i < kGuideLobes; ++i) {
        const float x = o[5 * i], y = o[5 * i + 1], z = o[5 * i + 2];
        const float n = fmaxf(sqrtf(x * x + y * y + z * z), 1.0e-12f);
        norms[i] = n;
        const float kappa = fminf(softplus(o[5 * i + 3]) + 0.01f, kGuideKappaMax);
        m.lobe[i] = make_float4(x / n, y / n, z / n, kappa);
        m.w[i] = expf(lg[i] - mx);
        den += m.w[i];
    }
    for (int i = 0; i < kGuideLobes; ++i) m.w[i] /= den;
}

// Sample loss  -w log q(d)  and the gradient with respect to the 40 raw
// outputs of  -w log q(d) + w kGuideNormPenalty sum_i (|o_i| - 1)^2,  the
// second term holding the scale of each lobe's direction output near 1 (the
// direction o / |o| does not depend on it, and the gradient of the first term
// shrinks as 1 / |o|).  Returns the first term.
__device__ __forceinline__ float vmf_loss_grad(const float* o, float dx, float dy, float dz, float w, float* g) {
    GuideMixture M;
    float norms[kGuideLobes], th[kGuideLobes];
    mixture_from_raw(o, M, norms, th);
    float f[kGuideLobes], q = 0.0f;
    for (int i = 0; i < kGuideLobes; ++i) {
        const float4 L = M.lobe[i];
        f[i] = vmf_pdf(L.w, L.x * dx + L.y * dy + L.z * dz);
        q += M.w[i] * f[i];
    }
    q = fmaxf(q, 1.0e-30f);
    for (int i = 0; i < kGuideLobes; ++i) {
        const float4 L = M.lobe[i];
        const float r = M.w[i] * f[i] / q;  // responsibility of lobe i
        // weight logit: d(-log q)/d l_i = -(r_i - pi_i), through l = B tanh(o / B)
        g[5 * i + 4] = -w * (r - M.w[i]) * (1.0f - th[i] * th[i]);
        // concentration: d log f / d kappa = 1/kappa - 2 e^{-2k} / (1 - e^{-2k}) + (mu.d - 1)
        const float k = L.w;
        const float e2 = expf(-2.0f * k);
        const float md = L.x * dx + L.y * dy + L.z * dz;
        const float dlogf = 1.0f / k - 2.0f * e2 / -expm1f(-2.0f * k) + (md - 1.0f);
        const float raw_k = o[5 * i + 3];
        const float dk = (softplus(raw_k) + 0.01f < kGuideKappaMax) ? sigmoid(raw_k) : 0.0f;
        g[5 * i + 3] = -w * r * dlogf * dk;
        // mean: d log f / d mu = kappa d, through mu = o / |o|: (I - mu mu^T) / |o|;
        // plus the scale penalty 2 w c (|o| - 1) mu
        const float gx = -w * r * k * dx, gy = -w * r * k * dy, gz = -w * r * k * dz;
        const float gm = gx * L.x + gy * L.y + gz * L.z;
        const float pen = 2.0f * w * kGuideNormPenalty * (norms[i] - 1.0f);
        g[5 * i + 0] = (gx - gm * L.x) / norms[i] + pen * L.x;
        g[5 * i + 1] = (gy - gm * L.y) / norms[i] + pen * L.y;
        g[5 * i + 2] = (gz - gm * L.z) / norms[i] + pen * L.z;
    }
    return -w * logf(q);
}

// ---------------------------------------------------------------- shared tiles
struct SmemFwd {
    __nv_bfloat16 W[kLayers][kH][kStride];  // W[l][in][out]
    float b[kLayers][kH];
    __nv_bfloat16 x[kWarps][16][kStride];   // encoded inputs of each warp's rows
    float out[kWarps][16][kH + 4];          // raw outputs
};

__device__ void load_weights(__nv_bfloat16 (*W)[kH][kStride], float (*b)[kH], const GuideView& g) {
    const uint32_t* src = reinterpret_cast<const uint32_t*>(g.wbf);
    for (int i = threadIdx.x; i < kLayers * kH * kH / 2; i += blockDim.x) {
        const int e = 2 * i;
        const int l = e / (kH * kH), r = (e / kH) % kH, c = e % kH;
        *reinterpret_cast<uint32_t*>(&W[l][r][c]) = src[i];
    }
    for (int i = threadIdx.x; i < kLayers * kH; i += blockDim.x) b[i / kH][i % kH] = g.b[i];
}

// A fragments (16 rows x 64) of a bf16 tile in shared memory (row stride kStride)
__device__ __forceinline__ void load_a(uint32_t a[4][4], const __nv_bfloat16 (*t)[kStride], int lane) {
    const int g = lane >> 2, q = lane & 3;
    for (int kt = 0; kt < 4; ++kt) {
        a[kt][0] = *reinterpret_cast<const uint32_t*>(&t[g][16 * kt + 2 * q]);
        a[kt][1] = *reinterpret_cast<const uint32_t*>(&t[g + 8][16 * kt + 2 * q]);
        a[kt][2] = *reinterpret_cast<const uint32_t*>(&t[g][16 * kt + 8 + 2 * q]);
        a[kt][3] = *reinterpret_cast<const uint32_t*>(&t[g + 8][16 * kt + 8 + 2 * q]);
    }
}

// acc[16 x 64] = a[16 x 64] * W (B operand from W[in][out] via ldmatrix.trans)
__device__ __forceinline__ void layer_fwd(float acc[8][4], const uint32_t a[4][4], const __nv_bfloat16 (*W)[kStride],
                                          int lane) {
    for (int j = 0; j < 8; ++j) acc[j][0] = acc[j][1] = acc[j][2] = acc[j][3] = 0.0f;
    const int m = lane >> 3, r = lane & 7;
    for (int kt = 0; kt < 4; ++kt) {
        for (int jp = 0; jp < 4; ++jp) {
            // 8x8 blocks m = 0..3: (k rows 16kt + 8(m&1) + r, n columns 16jp + 8(m>>1))
            uint32_t bq[4];
            ldsm_x4_trans(bq, &W[16 * kt + 8 * (m & 1) + r][16 * jp + 8 * (m >> 1)]);
            mma16816(acc[2 * jp], a[kt], bq[0], bq[1]);
            mma16816(acc[2 * jp + 1], a[kt], bq[2], bq[3]);
        }
    }
}

// bias (+ ReLU) and repack the accumulator as the next layer's A operand
__device__ __forceinline__ void activate(uint32_t a[4][4], float acc[8][4], const float* bias, bool relu, int lane) {
    const int q = lane & 3;
    for (int j = 0; j < 8; ++j) {
        const float b0 = bias[8 * j + 2 * q], b1 = bias[8 * j + 2 * q + 1];
        acc[j][0] += b0;
        acc[j][1] += b1;
        acc[j][2] += b0;
        acc[j][3] += b1;
        if (relu)
            for (int e = 0; e < 4; ++e) acc[j][e] = fmaxf(acc[j][e], 0.0f);
    }
    for (int kt = 0; kt < 4; ++kt) {
        a[kt][0] = pack_bf16(acc[2 * kt][0], acc[2 * kt][1]);
        a[kt][1] = pack_bf16(acc[2 * kt][2], acc[2 * kt][3]);
        a[kt][2] = pack_bf16(acc[2 * kt + 1][0], acc[2 * kt + 1][1]);
        a[kt][3] = pack_bf16(acc[2 * kt + 1][2], acc[2 * kt + 1][3]);
    }
}

__device__ __forceinline__ void store_acc(float (*out)[kH + 4], const float acc[8][4], int lane) {
    const int g = lane >> 2, q = lane & 3;
    for (int j = 0; j < 8; ++j) {
        out[g][8 * j + 2 * q] = acc[j][0];
        out[g][8 * j + 2 * q + 1] = acc[j][1];
        out[g + 8][8 * j + 2 * q] = acc[j][2];
        out[g + 8][8 * j + 2 * q + 1] = acc[j][3];
    }
}

__device__ __forceinline__ void store_inputs(__nv_bfloat16* row, const float* f) {
    for (int c = 0; c < kH; c += 2)
        *reinterpret_cast<uint32_t*>(row + c) =
            pack_bf16(c < kGuideInputs ? f[c] : 0.0f, c + 1 < kGuideInputs ? f[c + 1] : 0.0f);
}

// forward of one warp's 16 staged rows; raw outputs into S.out[warp]
__device__ __forceinline__ void forward_tile(SmemFwd& S, int warp, int lane) {
    uint32_t a[4][4];
    float acc[8][4];
    load_a(a, S.x[warp], lane);
    for (int l = 0; l < kLayers; ++l) {
        layer_fwd(acc, a, S.W[l], lane);
        activate(a, acc, S.b[l], l + 1 < kLayers, lane);
    }
    store_acc(S.out[warp], acc, lane);
}

// ---------------------------------------------------------------- inference
// rows: 16 floats each (x, n, wo in the first 9); out: 40 raw floats per row
__global__ void __launch_bounds__(128) k_guide_infer(GuideView g, const float* __restrict__ rows, uint32_t n,
                                                     float* __restrict__ out) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    SmemFwd& S = *reinterpret_cast<SmemFwd*>(smem_raw);
    load_weights(S.W, S.b, g);
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (uint32_t base = (blockIdx.x * kWarps + warp) * 16u; base < n; base += gridDim.x * kWarps * 16u) {
        if (lane < 16) {
            const uint32_t r = base + lane;
            float f[kGuideInputs];
            if (r < n) {
                float x9[9];
                for (int c = 0; c < 9; ++c) x9[c] = rows[16 * (size_t)r + c];
                encode(x9, g.params, f);
            } else {
                for (int c = 0; c < kGuideInputs; ++c) f[c] = 0.0f;
            }
            store_inputs(S.x[warp][lane], f);
        }
        __syncwarp();
        forward_tile(S, warp, lane);
        __syncwarp();
        for (int e = lane; e < 16 * kGuideOutputs; e += 32) {
            const uint32_t r = base + e / kGuideOutputs;
            if (r < n)
                out[kGuideOutputs * (size_t)r + e % kGuideOutputs] = S.out[warp][e / kGuideOutputs][e % kGuideOutputs];
        }
        __syncwarp();
    }
}

// The guided items of this bounce, in the order the shading kernel numbers
// them: queue 1 (Lambertian), queue 4 (Ward), then queue 6 (in-volume) when
// volumes are guided.
__device__ __forceinline__ uint32_t guided_count(const QueueView& Q, const GuideRenderD& gd) {
    return Q.counts[kMatLambertian] + Q.counts[kMatWard] + (gd.volumes ? Q.counts[kMatVolumeInside] : 0u);
}
__device__ __forceinline__ uint32_t guided_slot(const QueueView& Q, uint32_t gi) {
    const uint32_t c1 = Q.counts[kMatLambertian], c4 = Q.counts[kMatWard];
    if (gi < c1) return Q.items[kMatLambertian][gi];
    if (gi < c1 + c4) return Q.items[kMatWard][gi - c1];
    return Q.items[kMatVolumeInside][gi - c1 - c4];
}

// Vertex of a slot as the network sees it: hit point, normal facing the
// outgoing direction (zero inside a volume), outgoing direction.
__device__ __forceinline__ void vertex_of(const PathsView& P, uint32_t slot, float* x9) {
    const float4 ro = P.ro[slot], rd = P.rd[slot], ng = P.ng[slot];
    x9[0] = ro.x + rd.x * ro.w;
    x9[1] = ro.y + rd.y * ro.w;
    x9[2] = ro.z + rd.z * ro.w;
    const bool surface = __float_as_int(ng.w) >= 0;
    float nx = ng.x, ny = ng.y, nz = ng.z;
    if (!surface) {
        nx = ny = nz = 0.0f;
    } else if (-(nx * rd.x + ny * rd.y + nz * rd.z) < 0.0f) {
        nx = -nx;
        ny = -ny;
        nz = -nz;
    }
    x9[3] = nx;
    x9[4] = ny;
    x9[5] = nz;
    x9[6] = -rd.x;
    x9[7] = -rd.y;
    x9[8] = -rd.z;
}

__global__ void __launch_bounds__(128) k_guide_infer_paths(GuideView g, PathsView P, QueueView Q, GuideRenderD gd) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    SmemFwd& S = *reinterpret_cast<SmemFwd*>(smem_raw);
    const uint32_t n = guided_count(Q, gd);
    if (blockIdx.x * kRows >= n) return;
    load_weights(S.W, S.b, g);
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (uint32_t base = (blockIdx.x * kWarps + warp) * 16u; base < n; base += gridDim.x * kWarps * 16u) {
        if (lane < 16) {
            const uint32_t r = base + lane;
            float f[kGuideInputs];
            if (r < n) {
                float x9[9];
                vertex_of(P, guided_slot(Q, r), x9);
                encode(x9, g.params, f);
            } else {
                for (int c = 0; c < kGuideInputs; ++c) f[c] = 0.0f;
            }
            store_inputs(S.x[warp][lane], f);
        }
        __syncwarp();
        forward_tile(S, warp, lane);
        __syncwarp();
        if (lane < 16 && base + lane < n) {
            GuideMixture M;
            float norms[kGuideLobes], th[kGuideLobes];
            mixture_from_raw(S.out[warp][lane], M, norms, th);
            float4* dst = gd.lobes + (size_t)kGuideLobeVecs * (base + lane);
            for (int i = 0; i < kGuideLobes; ++i) dst[i] = M.lobe[i];
            dst[8] = make_float4(M.w[0], M.w[1], M.w[2], M.w[3]);
            dst[9] = make_float4(M.w[4], M.w[5], M.w[6], M.w[7]);
        }
        __syncwarp();
    }
}

// ---------------------------------------------------------------- training
struct SmemTrain {
    __nv_bfloat16 W[kLayers][kH][kStride];
    float b[kLayers][kH];
    __nv_bfloat16 act[kLayers][kRows][kStride];  // input of layer l for the chunk's rows
    __nv_bfloat16 dy[kRows][kStride];            // gradient at the output of the current layer
    float out[kWarps][16][kH + 4];
    float gW[kLayers][kH][kH];                   // this CTA's dW; warp w owns input rows 16w..16w+15
    float gb[kLayers][kH];
    float loss[kWarps];
};

// samples: 16 floats each (x, n, wo, wi, weight); loss weight = weight * scale / wsum
__global__ void __launch_bounds__(128) k_guide_train(GuideView g, const float* __restrict__ samples,
                                                     const uint32_t* __restrict__ count, uint32_t cap,
                                                     const float* __restrict__ wsum, float weight_scale) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    SmemTrain& S = *reinterpret_cast<SmemTrain*>(smem_raw);
    const uint32_t n = min(*count, cap);
    if (blockIdx.x * kRows >= n) return;
    float scale = weight_scale;
    if (wsum) {
        const float s = *wsum;
        scale = s > 0.0f ? weight_scale / s : 0.0f;
    }
    load_weights(S.W, S.b, g);
    for (int i = threadIdx.x; i < kLayers * kH * kH; i += blockDim.x) (&S.gW[0][0][0])[i] = 0.0f;
    for (int i = threadIdx.x; i < kLayers * kH; i += blockDim.x) (&S.gb[0][0])[i] = 0.0f;
    if (threadIdx.x < kWarps) S.loss[threadIdx.x] = 0.0f;
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int gq = lane >> 2, q = lane & 3;
    const int r0 = 16 * warp;  // this warp's rows within the chunk
    for (uint32_t chunk = blockIdx.x * (uint32_t)kRows; chunk < n; chunk += gridDim.x * (uint32_t)kRows) {
        // ---- forward, keeping each layer's input
        float dirw[4] = {0.0f, 0.0f, 0.0f, 0.0f};
        if (lane < 16) {
            const uint32_t r = chunk + r0 + lane;
            float f[kGuideInputs];
            if (r < n) {
                const float* s = samples + 16 * (size_t)r;
                float x9[9];
                for (int c = 0; c < 9; ++c) x9[c] = s[c];
                encode(x9, g.params, f);
                dirw[0] = s[9];
                dirw[1] = s[10];
                dirw[2] = s[11];
                dirw[3] = s[12] * scale;
            } else {
                for (int c = 0; c < kGuideInputs; ++c) f[c] = 0.0f;
            }
            store_inputs(S.act[0][r0 + lane], f);
        }
        __syncwarp();
        uint32_t a[4][4];
        float acc[8][4];
        load_a(a, &S.act[0][r0], lane);
        for (int l = 0; l < kLayers; ++l) {
            layer_fwd(acc, a, S.W[l], lane);
            activate(a, acc, S.b[l], l + 1 < kLayers, lane);
            if (l + 1 < kLayers) {
                // keep the next layer's input (the bf16 fragments just packed)
                for (int kt = 0; kt < 4; ++kt) {
                    *reinterpret_cast<uint32_t*>(&S.act[l + 1][r0 + gq][16 * kt + 2 * q]) = a[kt][0];
                    *reinterpret_cast<uint32_t*>(&S.act[l + 1][r0 + gq + 8][16 * kt + 2 * q]) = a[kt][1];
                    *reinterpret_cast<uint32_t*>(&S.act[l + 1][r0 + gq][16 * kt + 8 + 2 * q]) = a[kt][2];
                    *reinterpret_cast<uint32_t*>(&S.act[l + 1][r0 + gq + 8][16 * kt + 8 + 2 * q]) = a[kt][3];
                }
            }
        }
        store_acc(S.out[warp], acc, lane);
        __syncwarp();
        // ---- loss gradient at the output, one lane per row
        float lossv = 0.0f;
        if (lane < 16) {
            float gr[kGuideOutputs];
            if (dirw[3] > 0.0f) {
                lossv = vmf_loss_grad(S.out[warp][lane], dirw[0], dirw[1], dirw[2], dirw[3], gr);
            } else {
                for (int c = 0; c < kGuideOutputs; ++c) gr[c] = 0.0f;
            }
            for (int c = 0; c < kH; c += 2)
                *reinterpret_cast<uint32_t*>(&S.dy[r0 + lane][c]) =
                    pack_bf16(c < kGuideOutputs ? gr[c] : 0.0f, c + 1 < kGuideOutputs ? gr[c + 1] : 0.0f);
        }
        for (int off = 16; off > 0; off >>= 1) lossv += __shfl_xor_sync(0xffffffffu, lossv, off);
        if (lane == 0) S.loss[warp] += lossv;
        __syncthreads();
        // ---- backward, layer by layer over the chunk
        for (int l = kLayers - 1; l >= 0; --l) {
            // dW[l] += act[l]^T dy  (the chunk's rows are the reduction dimension)
            {
                float dw[8][4];
                for (int j = 0; j < 8; ++j) dw[j][0] = dw[j][1] = dw[j][2] = dw[j][3] = 0.0f;
                const int m = lane >> 3, rr = lane & 7;
                for (int ks = 0; ks < kRows / 16; ++ks) {
                    // A = act^T (inputs x rows): 8x8 block m of the A fragment is the
                    // transpose of act rows 16ks + 8(m>>1).., input columns 16w + 8(m&1)..
                    uint32_t af[4];
                    ldsm_x4_trans(af, &S.act[l][16 * ks + 8 * (m >> 1) + rr][16 * warp + 8 * (m & 1)]);
                    for (int jp = 0; jp < 4; ++jp) {
                        uint32_t bq[4];
                        ldsm_x4_trans(bq, &S.dy[16 * ks + 8 * (m & 1) + rr][16 * jp + 8 * (m >> 1)]);
                        mma16816(dw[2 * jp], af, bq[0], bq[1]);
                        mma16816(dw[2 * jp + 1], af, bq[2], bq[3]);
                    }
                }
                for (int j = 0; j < 8; ++j) {
                    S.gW[l][16 * warp + gq][8 * j + 2 * q] += dw[j][0];
                    S.gW[l][16 * warp + gq][8 * j + 2 * q + 1] += dw[j][1];
                    S.gW[l][16 * warp + gq + 8][8 * j + 2 * q] += dw[j][2];
                    S.gW[l][16 * warp + gq + 8][8 * j + 2 * q + 1] += dw[j][3];
                }
            }
            // db[l] += column sums of dy
            if (threadIdx.x < kH) {
                float s = 0.0f;
                for (int r = 0; r < kRows; ++r) s += __bfloat162float(S.dy[r][threadIdx.x]);
                S.gb[l][threadIdx.x] += s;
            }
            if (l == 0) break;
            // dx = dy W^T (B operand (k = out, n = in) read from W[in][out]), masked by ReLU'
            float dx[8][4];
            {
                uint32_t ad[4][4];
                load_a(ad, &S.dy[r0], lane);
                for (int j = 0; j < 8; ++j) dx[j][0] = dx[j][1] = dx[j][2] = dx[j][3] = 0.0f;
                for (int kt = 0; kt < 4; ++kt)
                    for (int j = 0; j < 8; ++j) {
                        const uint32_t b0 = *reinterpret_cast<const uint32_t*>(&S.W[l][8 * j + gq][16 * kt + 2 * q]);
                        const uint32_t b1 =
                            *reinterpret_cast<const uint32_t*>(&S.W[l][8 * j + gq][16 * kt + 8 + 2 * q]);
                        mma16816(dx[j], ad[kt], b0, b1);
                    }
            }
            __syncthreads();  // every warp has read dy of the chunk
            for (int j = 0; j < 8; ++j) {
                const int c = 8 * j + 2 * q;
                const uint32_t m0 = *reinterpret_cast<const uint32_t*>(&S.act[l][r0 + gq][c]);
                const uint32_t m1 = *reinterpret_cast<const uint32_t*>(&S.act[l][r0 + gq + 8][c]);
                const float v0 = bf16_lo(m0) > 0.0f ? dx[j][0] : 0.0f;
                const float v1 = bf16_hi(m0) > 0.0f ? dx[j][1] : 0.0f;
                const float v2 = bf16_lo(m1) > 0.0f ? dx[j][2] : 0.0f;
                const float v3 = bf16_hi(m1) > 0.0f ? dx[j][3] : 0.0f;
                *reinterpret_cast<uint32_t*>(&S.dy[r0 + gq][c]) = pack_bf16(v0, v1);
                *reinterpret_cast<uint32_t*>(&S.dy[r0 + gq + 8][c]) = pack_bf16(v2, v3);
            }
            __syncthreads();
        }
        __syncthreads();
    }
    // flush this CTA's gradient
    for (int i = threadIdx.x; i < kLayers * kH * kH; i += blockDim.x) {
        const float v = (&S.gW[0][0][0])[i];
        if (v != 0.0f) atomicAdd(g.gW + i, v);
    }
    for (int i = threadIdx.x; i < kLayers * kH; i += blockDim.x) {
        const float v = (&S.gb[0][0])[i];
        if (v != 0.0f) atomicAdd(g.gb + i, v);
    }
    if (threadIdx.x == 0) {
        float s = 0.0f;
        for (int w = 0; w < kWarps; ++w) s += S.loss[w];
        atomicAdd(g.loss, s);
    }
}

// ---------------------------------------------------------------- Adam
__global__ void k_guide_adam(GuideView g, const uint32_t* count, const uint32_t* iter, float lr, float beta1,
                             float beta2, float eps) {
    if (*count == 0u) return;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= kGuideParams) return;
    const float t = (float)(*iter + 1u);
    const float bc1 = 1.0f - powf(beta1, t), bc2 = 1.0f - powf(beta2, t);
    const bool is_w = i < kGuideWeights;
    float* p = is_w ? g.w + i : g.b + (i - kGuideWeights);
    float* grad = is_w ? g.gW + i : g.gb + (i - kGuideWeights);
    const float gr = *grad;
    const float mm = beta1 * g.m[i] + (1.0f - beta1) * gr;
    const float vv = beta2 * g.v[i] + (1.0f - beta2) * gr * gr;
    g.m[i] = mm;
    g.v[i] = vv;
    // a parameter whose gradient was always zero (the padding) keeps m = v = 0 and does not move
    const float nv = *p - lr * (mm / bc1) / (sqrtf(vv / bc2) + eps);
    *p = nv;
    *grad = 0.0f;
    if (is_w) g.wbf[i] = __float2bfloat16_rn(nv);
}

__global__ void k_guide_finish(GuideView g, GuideTrainD t) {
    const uint32_t c = *t.count;
    if (c > 0u) {
        const uint32_t it = *t.iter;
        t.loss_hist[it % kLossHist] = *g.loss;
        *t.iter = it + 1u;
    }
    *t.last = min(c, t.cap);
    // aim the next iteration at `cap` accepted records
    const unsigned long long cand = *t.candidates;
    if (cand > 0ull) *t.accept = fminf(1.0f, (float)t.cap / (float)cand);
    *t.count = 0u;
    *t.wsum = 0.0f;
    *t.candidates = 0ull;
    *g.loss = 0.0f;
}

}  // namespace

size_t guide_infer_smem() { return sizeof(SmemFwd); }
size_t guide_train_smem() { return sizeof(SmemTrain); }

int guide_kernel_attributes() {
    const int a = (int)cudaFuncAttributeMaxDynamicSharedMemorySize;
    cudaError_t e = cudaFuncSetAttribute(k_guide_infer, (cudaFuncAttribute)a, (int)sizeof(SmemFwd));
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k_guide_infer_paths, (cudaFuncAttribute)a, (int)sizeof(SmemFwd));
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k_guide_train, (cudaFuncAttribute)a, (int)sizeof(SmemTrain));
    return (int)e;
}

void launch_guide_infer(const GuideView& g, const float* rows, uint32_t n, float* out, int grid, cudaStream_t st) {
    if (n == 0) return;
    k_guide_infer<<<grid, 128, sizeof(SmemFwd), st>>>(g, rows, n, out);
}

void launch_guide_infer_paths(const GuideView& g, const PathsView& p, const QueueView& q, const GuideRenderD& gd,
                              int grid, cudaStream_t st) {
    k_guide_infer_paths<<<grid, 128, sizeof(SmemFwd), st>>>(g, p, q, gd);
}

void launch_guide_train(const GuideView& g, const float* samples, const uint32_t* count, uint32_t cap,
                        const float* wsum, float weight_scale, int grid, cudaStream_t st) {
    k_guide_train<<<grid, 128, sizeof(SmemTrain), st>>>(g, samples, count, cap, wsum, weight_scale);
}

void launch_guide_adam(const GuideView& g, const uint32_t* count, const uint32_t* iter, float lr, float beta1,
                       float beta2, float eps, cudaStream_t st) {
    k_guide_adam<<<(kGuideParams + 255) / 256, 256, 0, st>>>(g, count, iter, lr, beta1, beta2, eps);
}

void launch_guide_finish(const GuideView& g, const GuideTrainD& t, cudaStream_t st) {
    k_guide_finish<<<1, 1, 0, st>>>(g, t);
}

}  // namespace dev
}  // namespace rgr
