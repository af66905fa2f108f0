// guide_mlp.cu — the path-guiding network: a fully fused BF16 MLP on the
// tensor cores (FP32 accumulation), its loss gradient, backward pass and Adam.
//
// Network: 36 frequency-encoding inputs (position, normal, outgoing
// direction), four hidden layers of 64 with ReLU, 40 outputs = 8 von
// Mises-Fisher lobes x (mean direction xyz, concentration, weight logit).
// Every layer is stored as a 64 x 64 matrix W[l][in][out] (padding rows and
// columns are zero, receive zero gradient and stay zero under Adam), so one
// code path serves all five layers.  The outputs are field-major: output
// 8 f + i is field f (0..2 mean, 3 concentration, 4 weight logit) of lobe i.
//
// Tensor-core tiling (mma.sync m16n8k16 bf16 -> f32): a warp owns 16 rows;
// lane (g, q) = (lane / 4, lane % 4) holds rows g and g + 8 of every
// fragment.  Everything stays in registers from the input encoding to the
// mixture:
//  * each lane computes the encoding features its A fragment needs (sin/cos
//    pairs 8 kt + q and 8 kt + 4 + q of its two rows), so no input tile is
//    staged in shared memory;
//  * the accumulator fragment of two adjacent m16n8 tiles is the A fragment
//    of the next m16n8k16 product, so layers chain through bias + ReLU +
//    bf16 conversion only;
//  * with the field-major output order, the last layer's accumulators of a
//    lane hold all five fields of lobes 2q and 2q + 1 for its two rows, and
//    the mixture (softmax, densities, loss gradient) needs only shuffles
//    within the quad.
// Weights live in shared memory as W[in][out] (row stride 72 bf16, so the 8
// rows an ldmatrix phase reads fall in distinct banks); the forward B operand
// is loaded with ldmatrix.trans, the backward one with plain 32-bit loads.
// Training processes 64-row chunks per CTA: each layer's input stays in
// shared memory for the chunk, dW = A^T dY runs on the tensor cores with the
// chunk's rows as the reduction dimension, and each warp accumulates its 16
// input rows of dW in shared FP32 across all chunks of the CTA; one atomicAdd
// per weight per CTA flushes it.
#include <cuda_bf16.h>

#include "guide.cuh"

namespace rgr {
namespace dev {
namespace {

constexpr int kH = kGuideWidth;  // padded width of every layer
constexpr int kLayers = kGuideLayers;
constexpr int kStride = 72;      // shared-memory row stride of bf16 tiles (elements)
constexpr int kTrainWarps = 4;   // warps per training CTA
constexpr int kRows = 16 * kTrainWarps;
constexpr int kInferWarps = 8;   // warps per inference CTA
constexpr int kOutTiles = 5;     // n tiles (of 8) holding the mixture's 40 outputs
constexpr int kNetTiles = 6;     // and the selection logit (output 40, tile 5)

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
// opposite directions (v = 0 and v = 1) encode differently.  Feature pair p
// (columns 2p = sin, 2p + 1 = cos) is coordinate p / 2 at octave p % 2.
__device__ __forceinline__ void coords(const float* x9, const GuideParams& gp, float* v) {
    for (int c = 0; c < 3; ++c) {
        v[c] = (x9[c] - gp.lo[c]) * gp.inv_ext[c];
        v[3 + c] = 0.5f * (x9[3 + c] + 1.0f);
        v[6 + c] = 0.5f * (x9[6 + c] + 1.0f);
    }
}
// Pair p = 8 kt + 4 h + q is coordinate 4 kt + 2 h + q / 2 at octave q % 2:
// the coordinate is chosen between two registers, not indexed at run time.
__device__ __forceinline__ uint32_t feature_pair(const float* v, int i0, int q) {
    const int i = i0 + (q >> 1);
    if (i >= 9) return 0u;  // padding columns 36..63
    const float x = (q >> 1) ? v[i0 + 1 < 9 ? i0 + 1 : 8] : v[i0];
    float s, c;
    sincospif(x * ((q & 1) ? 2.0f : 1.0f), &s, &c);
    return pack_bf16(s, c);
}
// the A fragments of the encoded inputs of this lane's rows g (v0) and g + 8 (v1)
__device__ __forceinline__ void encode_frag(const float* v0, const float* v1, int q, uint32_t a[4][4]) {
#pragma unroll
    for (int kt = 0; kt < 4; ++kt) {
        a[kt][0] = feature_pair(v0, 4 * kt, q);
        a[kt][1] = feature_pair(v1, 4 * kt, q);
        a[kt][2] = feature_pair(v0, 4 * kt + 2, q);
        a[kt][3] = feature_pair(v1, 4 * kt + 2, q);
    }
}

// ---------------------------------------------------------------- layers
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
__device__ __forceinline__ void store_a(__nv_bfloat16 (*t)[kStride], const uint32_t a[4][4], int lane) {
    const int g = lane >> 2, q = lane & 3;
    for (int kt = 0; kt < 4; ++kt) {
        *reinterpret_cast<uint32_t*>(&t[g][16 * kt + 2 * q]) = a[kt][0];
        *reinterpret_cast<uint32_t*>(&t[g + 8][16 * kt + 2 * q]) = a[kt][1];
        *reinterpret_cast<uint32_t*>(&t[g][16 * kt + 8 + 2 * q]) = a[kt][2];
        *reinterpret_cast<uint32_t*>(&t[g + 8][16 * kt + 8 + 2 * q]) = a[kt][3];
    }
}

// acc[16 x 16 NP] = a[16 x 64] * W[:, 0 : 16 NP] (B operand via ldmatrix.trans)
template <int NP>
__device__ __forceinline__ void layer_fwd(float acc[8][4], const uint32_t a[4][4], const __nv_bfloat16 (*W)[kStride],
                                          int lane) {
    for (int j = 0; j < 2 * NP; ++j) acc[j][0] = acc[j][1] = acc[j][2] = acc[j][3] = 0.0f;
    const int m = lane >> 3, r = lane & 7;
    for (int kt = 0; kt < 4; ++kt) {
        for (int jp = 0; jp < NP; ++jp) {
            // 8x8 blocks m = 0..3: (k rows 16kt + 8(m&1) + r, n columns 16jp + 8(m>>1))
            uint32_t bq[4];
            ldsm_x4_trans(bq, &W[16 * kt + 8 * (m & 1) + r][16 * jp + 8 * (m >> 1)]);
            mma16816(acc[2 * jp], a[kt], bq[0], bq[1]);
            mma16816(acc[2 * jp + 1], a[kt], bq[2], bq[3]);
        }
    }
}

// bias + ReLU, repacked as the next layer's A operand
__device__ __forceinline__ void activate(uint32_t a[4][4], float acc[8][4], const float* bias, int lane) {
    const int q = lane & 3;
    for (int j = 0; j < 8; ++j) {
        const float b0 = bias[8 * j + 2 * q], b1 = bias[8 * j + 2 * q + 1];
        acc[j][0] = fmaxf(acc[j][0] + b0, 0.0f);
        acc[j][1] = fmaxf(acc[j][1] + b1, 0.0f);
        acc[j][2] = fmaxf(acc[j][2] + b0, 0.0f);
        acc[j][3] = fmaxf(acc[j][3] + b1, 0.0f);
    }
    for (int kt = 0; kt < 4; ++kt) {
        a[kt][0] = pack_bf16(acc[2 * kt][0], acc[2 * kt][1]);
        a[kt][1] = pack_bf16(acc[2 * kt][2], acc[2 * kt][3]);
        a[kt][2] = pack_bf16(acc[2 * kt + 1][0], acc[2 * kt + 1][1]);
        a[kt][3] = pack_bf16(acc[2 * kt + 1][2], acc[2 * kt + 1][3]);
    }
}

// Raw outputs of the 16 rows whose input fragments are `a`: o[f][h][s] =
// field f of lobe 2q + s of row g + 8h (bias added).  With keep != nullptr the
// inputs of layers 1..4 are also stored there (training).
__device__ __forceinline__ void forward_frag(uint32_t a[4][4], const __nv_bfloat16 (*W)[kH][kStride],
                                             const float (*b)[kH], int lane, float o[kNetTiles][2][2],
                                             __nv_bfloat16 (*keep)[kRows][kStride]) {
    float acc[8][4];
    for (int l = 0; l + 1 < kLayers; ++l) {
        layer_fwd<4>(acc, a, W[l], lane);
        activate(a, acc, b[l], lane);
        if (keep) store_a(keep[l + 1], a, lane);
    }
    layer_fwd<3>(acc, a, W[kLayers - 1], lane);
    const int q = lane & 3;
    for (int f = 0; f < kNetTiles; ++f) {
        const float b0 = b[kLayers - 1][8 * f + 2 * q], b1 = b[kLayers - 1][8 * f + 2 * q + 1];
        o[f][0][0] = acc[f][0] + b0;
        o[f][0][1] = acc[f][1] + b1;
        o[f][1][0] = acc[f][2] + b0;
        o[f][1][1] = acc[f][3] + b1;
    }
}

// ---------------------------------------------------------------- vMF mixture
__device__ __forceinline__ float quad_max(float x) {
    x = fmaxf(x, __shfl_xor_sync(0xffffffffu, x, 1));
    return fmaxf(x, __shfl_xor_sync(0xffffffffu, x, 2));
}
__device__ __forceinline__ float quad_sum(float x) {
    x += __shfl_xor_sync(0xffffffffu, x, 1);
    return x + __shfl_xor_sync(0xffffffffu, x, 2);
}


// The mixture of row h of this lane (its lobes 2q, 2q + 1; weights by softmax
// across the quad).  All 32 lanes must call it.
__device__ __forceinline__ void mixture_quad(const float o[kNetTiles][2][2], int h, LobeOut L[2], float w[2]) {
    for (int s = 0; s < 2; ++s) L[s] = lobe_of(o[0][h][s], o[1][h][s], o[2][h][s], o[3][h][s], o[4][h][s]);
    const float mx = quad_max(fmaxf(L[0].logit, L[1].logit));
    w[0] = expf(L[0].logit - mx);
    w[1] = expf(L[1].logit - mx);
    const float den = quad_sum(w[0] + w[1]);
    w[0] /= den;
    w[1] /= den;
}

// Loss of row h, -wt log q(d) (returned by every lane of the quad), and its
// gradient with respect to this lane's raw outputs g[f][s] (lobes 2q + s) of
// -wt log q(d) + wt kGuideNormPenalty sum_i (|o_i| - 1)^2; the second term
// holds the length of each lobe's direction output near 1 (the direction
// o / |o| does not depend on it, and the gradient of the first term shrinks
// as 1 / |o|).  Tile 5 (lane q = 0, column 0: output 40) gets the gradient of
// the selection term -wt log(a q + (1 - a) pb) with respect to the selection
// logit, q held fixed (pb = the sample's BSDF pdf; none when 0).  All 32 lanes
// must call it.
__device__ __forceinline__ float loss_grad_quad(const float o[kNetTiles][2][2], int h, float dx, float dy, float dz,
                                                float wt, float pb, float g[kNetTiles][2]) {
    LobeOut L[2];
    float pi[2];
    mixture_quad(o, h, L, pi);
    float f[2];
    for (int s = 0; s < 2; ++s) f[s] = vmf_pdf(L[s].kappa, L[s].mx * dx + L[s].my * dy + L[s].mz * dz);
    const float q = fmaxf(quad_sum(pi[0] * f[0] + pi[1] * f[1]), 1.0e-30f);
    for (int s = 0; s < 2; ++s) {
        const float r = pi[s] * f[s] / q;  // responsibility of the lobe
        float gl[5];
        lobe_grad(L[s], pi[s], r, o[3][h][s], dx, dy, dz, wt, gl);
        for (int k = 0; k < 5; ++k) g[k][s] = gl[k];
    }
    const float z = __shfl_sync(0xffffffffu, o[5][h][0], (threadIdx.x & 31u) & ~3u);  // output 40, held by q = 0
    g[5][0] = ((threadIdx.x & 3u) == 0u) ? selection_grad(z, q, pb, wt) : 0.0f;
    g[5][1] = 0.0f;
    return -wt * logf(q);
}

// ---------------------------------------------------------------- inference
struct SmemFwd {
    __nv_bfloat16 W[kLayers][kH][kStride];  // W[l][in][out]
    float b[kLayers][kH];
};

// rows: 16 floats each (x, n, wo in the first 9); out: kGuideRowOutputs raw floats per row
__global__ void __launch_bounds__(32 * kInferWarps, 4) k_guide_infer(GuideView gv, const float* __restrict__ rows,
                                                                      uint32_t n, float* __restrict__ out) {
    __shared__ SmemFwd S;
    load_weights(S.W, S.b, gv);
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, q = lane & 3;
    for (uint32_t base = (blockIdx.x * kInferWarps + warp) * 16u; base < n; base += gridDim.x * kInferWarps * 16u) {
        float v[2][9];
        for (int h = 0; h < 2; ++h) {
            const uint32_t r = base + g + 8 * h;
            float x9[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
            if (r < n)
                for (int c = 0; c < 9; ++c) x9[c] = rows[16 * (size_t)r + c];
            coords(x9, gv.params, v[h]);
        }
        uint32_t a[4][4];
        encode_frag(v[0], v[1], q, a);
        float o[kNetTiles][2][2];
        forward_frag(a, S.W, S.b, lane, o, nullptr);
        for (int h = 0; h < 2; ++h) {
            const uint32_t r = base + g + 8 * h;
            if (r >= n) continue;
            for (int f = 0; f < kNetTiles; ++f)
                *reinterpret_cast<float2*>(out + kGuideRowOutputs * (size_t)r + 8 * f + 2 * q) =
                    make_float2(o[f][h][0], o[f][h][1]);
        }
    }
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

__global__ void __launch_bounds__(32 * kInferWarps, 4) k_guide_infer_paths(GuideView gv, PathsView P, QueueView Q,
                                                                            GuideRenderD gd) {
    __shared__ SmemFwd S;
    const uint32_t n = guide_rows(Q, gd);
    if (blockIdx.x * kInferWarps * 16u >= n) return;
    load_weights(S.W, S.b, gv);
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, q = lane & 3;
    for (uint32_t base = (blockIdx.x * kInferWarps + warp) * 16u; base < n; base += gridDim.x * kInferWarps * 16u) {
        float v[2][9];
        for (int h = 0; h < 2; ++h) {
            const uint32_t r = base + g + 8 * h;
            float x9[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
            if (r < n) vertex_of(P, guide_row_slot(Q, gd, r), x9);
            coords(x9, gv.params, v[h]);
        }
        uint32_t a[4][4];
        encode_frag(v[0], v[1], q, a);
        float o[kNetTiles][2][2];
        forward_frag(a, S.W, S.b, lane, o, nullptr);
        for (int h = 0; h < 2; ++h) {
            LobeOut L[2];
            float w[2];
            mixture_quad(o, h, L, w);
            // the weights carry the guide's share of the vertex (their sum)
            const float z = __shfl_sync(0xffffffffu, o[5][h][0], lane & ~3);
            const float alpha = gd.learn_frac ? alpha_of(z) : gd.guide_frac;
            w[0] *= alpha;
            w[1] *= alpha;
            const uint32_t r = base + g + 8 * h;
            if (r >= n) continue;
            uint4* dst = gd.lobes + (size_t)kGuideMixVecs * r;  // FP16 record (guide.cuh)
            dst[q] = make_uint4(half2_bits(L[0].mx, L[0].my), half2_bits(L[0].mz, L[0].kappa),
                                half2_bits(L[1].mx, L[1].my), half2_bits(L[1].mz, L[1].kappa));
            reinterpret_cast<uint32_t*>(dst + 4)[q] = half2_bits(w[0], w[1]);
        }
    }
}

// ---------------------------------------------------------------- training
struct SmemTrain {
    __nv_bfloat16 W[kLayers][kH][kStride];
    float b[kLayers][kH];
    __nv_bfloat16 act[kLayers][kRows][kStride];  // input of layer l for the chunk's rows
    __nv_bfloat16 dy[kRows][kStride];            // gradient at the output of the current layer
    float gW[kLayers][kH][kH];                   // this CTA's dW; warp w owns input rows 16w..16w+15
    float gb[kTrainWarps][kLayers][kH];          // db per warp (its rows), summed at the flush
    float loss[kTrainWarps];
};

// Column sums over a warp's 16 rows of a gradient in the fragment layout (lane
// (g, q) holds columns 2q, 2q + 1 of an 8-column tile for rows g (p0) and
// g + 8 (p1), as packed bf16): added to gb[col] by lanes 0..3.
__device__ __forceinline__ void add_colsums(float* gb, int col, uint32_t p0, uint32_t p1, int lane) {
    float s0 = bf16_lo(p0) + bf16_lo(p1), s1 = bf16_hi(p0) + bf16_hi(p1);
    for (int o = 4; o < 32; o <<= 1) {
        s0 += __shfl_xor_sync(0xffffffffu, s0, o);
        s1 += __shfl_xor_sync(0xffffffffu, s1, o);
    }
    if (lane < 4) {
        gb[col] += s0;
        gb[col + 1] += s1;
    }
}

// samples: 16 floats each (x, n, wo, wi, weight); loss weight = weight * scale / wsum
__global__ void __launch_bounds__(32 * kTrainWarps) k_guide_train(GuideView gv, const float* __restrict__ samples,
                                                                  const uint32_t* __restrict__ count, uint32_t cap,
                                                                  uint32_t min_count, const float* __restrict__ wsum,
                                                                  float weight_scale) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    SmemTrain& S = *reinterpret_cast<SmemTrain*>(smem_raw);
    const uint32_t n = min(*count, cap);
    if (n < min_count) return;            // too few yet: they carry over to the next bounce
    if (blockIdx.x * kRows >= n) return;  // (no samples are recorded once the iteration budget is used up)
    float scale = weight_scale;
    if (wsum) {
        const float s = *wsum;
        scale = s > 0.0f ? weight_scale / s : 0.0f;
    }
    load_weights(S.W, S.b, gv);
    for (int i = threadIdx.x; i < kLayers * kH * kH; i += blockDim.x) (&S.gW[0][0][0])[i] = 0.0f;
    for (int i = threadIdx.x; i < kTrainWarps * kLayers * kH; i += blockDim.x) (&S.gb[0][0][0])[i] = 0.0f;
    if (threadIdx.x < kTrainWarps) S.loss[threadIdx.x] = 0.0f;
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int gq = lane >> 2, q = lane & 3;
    const int r0 = 16 * warp;  // this warp's rows within the chunk
    for (uint32_t chunk = blockIdx.x * (uint32_t)kRows; chunk < n; chunk += gridDim.x * (uint32_t)kRows) {
        // ---- forward, keeping each layer's input
        float v[2][9], dir[2][3], wt[2], pb[2];
        for (int h = 0; h < 2; ++h) {
            const uint32_t r = chunk + r0 + gq + 8 * h;
            float x9[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
            dir[h][0] = dir[h][1] = dir[h][2] = 0.0f;
            wt[h] = 0.0f;
            pb[h] = 0.0f;
            if (r < n) {
                const float* s = samples + 16 * (size_t)r;
                for (int c = 0; c < 9; ++c) x9[c] = s[c];
                dir[h][0] = s[9];
                dir[h][1] = s[10];
                dir[h][2] = s[11];
                wt[h] = s[12] * scale;
                pb[h] = s[13];
            }
            coords(x9, gv.params, v[h]);
        }
        uint32_t a[4][4];
        encode_frag(v[0], v[1], q, a);
        store_a(&S.act[0][r0], a, lane);
        float o[kNetTiles][2][2];
        forward_frag(a, S.W, S.b, lane, o, reinterpret_cast<__nv_bfloat16(*)[kRows][kStride]>(&S.act[0][r0]));
        // ---- loss gradient at the output, in the fragment layout
        float lossv = 0.0f;
        uint32_t gp[2][kNetTiles];  // the output gradient, packed bf16, per row half
        for (int h = 0; h < 2; ++h) {
            float gr[kNetTiles][2];
            const float lh = loss_grad_quad(o, h, dir[h][0], dir[h][1], dir[h][2], wt[h], pb[h], gr);
            const bool live = wt[h] > 0.0f;
            if (live && q == 0) lossv += lh;
            for (int f = 0; f < kNetTiles; ++f) {
                gp[h][f] = live ? pack_bf16(gr[f][0], gr[f][1]) : 0u;
                *reinterpret_cast<uint32_t*>(&S.dy[r0 + gq + 8 * h][8 * f + 2 * q]) = gp[h][f];
            }
            for (int f = kNetTiles; f < 8; ++f)
                *reinterpret_cast<uint32_t*>(&S.dy[r0 + gq + 8 * h][8 * f + 2 * q]) = 0u;
        }
        for (int f = 0; f < kNetTiles; ++f) add_colsums(S.gb[warp][kLayers - 1], 8 * f + 2 * q, gp[0][f], gp[1][f], lane);
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
            // (db[l], the column sums of this dy, was added when dy was formed)
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
                const uint32_t p0 = pack_bf16(v0, v1), p1 = pack_bf16(v2, v3);
                *reinterpret_cast<uint32_t*>(&S.dy[r0 + gq][c]) = p0;
                *reinterpret_cast<uint32_t*>(&S.dy[r0 + gq + 8][c]) = p1;
                add_colsums(S.gb[warp][l - 1], c, p0, p1, lane);
            }
            __syncthreads();
        }
        __syncthreads();
    }
    // flush this CTA's gradient
    for (int i = threadIdx.x; i < kLayers * kH * kH; i += blockDim.x) {
        const float v = (&S.gW[0][0][0])[i];
        if (v != 0.0f) atomicAdd(gv.gW + i, v);
    }
    for (int i = threadIdx.x; i < kLayers * kH; i += blockDim.x) {
        float v = 0.0f;
        for (int w = 0; w < kTrainWarps; ++w) v += (&S.gb[w][0][0])[i];
        if (v != 0.0f) atomicAdd(gv.gb + i, v);
    }
    if (threadIdx.x == 0) {
        float s = 0.0f;
        for (int w = 0; w < kTrainWarps; ++w) s += S.loss[w];
        atomicAdd(gv.loss, s);
    }
}

// ---------------------------------------------------------------- Adam
__global__ void k_guide_adam(GuideView g, const uint32_t* count, uint32_t min_count, const uint32_t* iter, float lr,
                             float beta1, float beta2, float eps) {
    if (*count == 0u || *count < min_count) return;
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
    if (is_w) {
        const __nv_bfloat16 h = __float2bfloat16_rn(nv);
        g.wbf[i] = h;
        const uint32_t l = (uint32_t)i / 4096u, in = ((uint32_t)i / 64u) % 64u, out = (uint32_t)i % 64u;
        if (!wt_is_bias_slot(l, in)) *reinterpret_cast<__nv_bfloat16*>(g.wt_sw + wt_sw_offset(l, in, out)) = h;
    } else {
        const uint32_t j = (uint32_t)(i - kGuideWeights), l = j / 64u, out = j % 64u;
        const __nv_bfloat16 hi = __float2bfloat16_rn(nv);
        const __nv_bfloat16 lo = __float2bfloat16_rn(nv - __bfloat162float(hi));
        *reinterpret_cast<__nv_bfloat16*>(g.wt_sw + wt_bias_offset(l, out, 0)) = hi;
        *reinterpret_cast<__nv_bfloat16*>(g.wt_sw + wt_bias_offset(l, out, 1)) = lo;
    }
}

__global__ void k_guide_finish(GuideView g, GuideTrainD t) {
    const uint32_t c = *t.count;
    if (c < t.min_count) {
        // no step this bounce: the samples stay for the next one.  Few paths
        // end at the tail of a render, and Adam's normalised step would turn
        // a handful of samples into a full-size, noisy update.
        const unsigned long long cand = *t.candidates;
        if (cand > 0ull) *t.accept = fminf(1.0f, (float)t.cap / (float)cand);
        return;
    }
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

__global__ void k_guide_set_count(uint32_t* count, uint32_t n) { *count = n; }

}  // namespace

size_t guide_infer_smem() { return sizeof(SmemFwd); }

void launch_guide_set_count(uint32_t* count, uint32_t n, cudaStream_t st) { k_guide_set_count<<<1, 1, 0, st>>>(count, n); }
size_t guide_train_smem() { return sizeof(SmemTrain); }

int guide_kernel_attributes() {
    return (int)cudaFuncSetAttribute(k_guide_train, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)sizeof(SmemTrain));
}

int guide_infer_grid(int num_sms) { return num_sms * 4; }

void launch_guide_infer(const GuideView& g, const float* rows, uint32_t n, float* out, int grid, cudaStream_t st) {
    if (n == 0) return;
    k_guide_infer<<<grid, 32 * kInferWarps, 0, st>>>(g, rows, n, out);
}

void launch_guide_infer_paths(const GuideView& g, const PathsView& p, const QueueView& q, const GuideRenderD& gd,
                              int grid, cudaStream_t st) {
    k_guide_infer_paths<<<grid, 32 * kInferWarps, 0, st>>>(g, p, q, gd);
}

void launch_guide_train(const GuideView& g, const float* samples, const uint32_t* count, uint32_t cap,
                        uint32_t min_count, const float* wsum, float weight_scale, int grid, cudaStream_t st) {
    k_guide_train<<<grid, 32 * kTrainWarps, sizeof(SmemTrain), st>>>(g, samples, count, cap, min_count, wsum,
                                                                     weight_scale);
}

void launch_guide_adam(const GuideView& g, const uint32_t* count, uint32_t min_count, const uint32_t* iter,
                       float lr, float beta1, float beta2, float eps, cudaStream_t st) {
    k_guide_adam<<<(kGuideParams + 255) / 256, 256, 0, st>>>(g, count, min_count, iter, lr, beta1, beta2, eps);
}

void launch_guide_finish(const GuideView& g, const GuideTrainD& t, cudaStream_t st) {
    k_guide_finish<<<1, 1, 0, st>>>(g, t);
}

}  // namespace dev
}  // namespace rgr
