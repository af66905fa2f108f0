// guide_train_tc.cu — one training iteration of the path-guiding network on the
// 5th-generation tensor cores: forward, loss gradient, backward and the weight
// gradients as tcgen05.mma with the operands in shared memory and every
// accumulator in tensor memory (TMEM).
//
// A CTA (one per SM) holds kTrGroups groups of 128 row threads and one warp
// that only issues MMAs.  A group works on tiles of 128 samples; thread t owns
// sample t of the tile from its input encoding to its output gradient.  The
// layer inputs live in shared memory as one 128-byte line per sample (64 bf16,
// 128-byte swizzle, 8-line groups 1024 bytes apart), and that single layout
// is read three ways by the tensor core:
//  * as A of the forward product act . W (M = samples, K-major);
//  * as A of the weight gradient act^T . dY (M = layer inputs, K = samples,
//    MN-major), which accumulates in TMEM over every tile the CTA trains on;
//  * the output gradient dY, in the same layout, as A of dX = dY . W^T
//    (K-major) and as B of act^T . dY (MN-major).
// The weights stay in shared memory as W[in][out] lines, B of the forward
// product (MN-major) and of dX (K-major) alike.  The weight-gradient MMAs have
// M = 128: rows 0..63 are the layer's 64 inputs, rows 64..127 read a region of
// bf16 ones, so TMEM lanes 64..127 accumulate the column sums of dY, the bias
// gradient, in the same instructions.
//
// Per tile the group and the MMA warp take ten turns (the group writes an
// operand into shared memory and arrives on a_full; the MMA warp issues the
// turn's MMAs and commits them to d_full; the group waits and reads the
// accumulators with tcgen05.ld):
//   0..4  forward, layer 0..4: D = act_l . W_l    (the group then adds the
//         bias, applies ReLU, rounds to bf16 and writes act_l+1; after layer 4
//         it computes the loss gradient of the 41 outputs and writes dY_4)
//   5..8  backward, layer 4..1: D = dY_l . W_l^T and dW_l += act_l^T . dY_l
//         (the group masks D by ReLU' of act_l, rounds, and writes dY_l-1)
//   9     dW_0 += act_0^T . dY_0
// Buffers per group: B1..B3 hold act_1..act_3; B0 holds act_0, then act_4
// once layer 0 has run, then act_0 again (re-encoded) once dW_4 is done; BY
// holds the output gradient of the current layer.  The two groups alternate on
// the tensor core: while one waits for its MMAs the other runs its epilogue.
//
// After its last tile each CTA writes its weight and bias gradients and loss
// to its own slot of a partials buffer; a second kernel sums the slots in a
// fixed order (no atomics).  Inside a CTA the two groups' tiles add into the
// same accumulators in the order their turns reach the tensor core, so FP32
// rounding differs slightly from run to run.  Every wait is
// bounded: on a timeout the CTA records an error, stops, waits (bounded) for
// the MMAs it issued and frees its TMEM.
//
// Arithmetic follows the mma.sync training kernel (guide_mlp.cu): BF16
// operands with FP32 accumulation, FP32 bias adds, layer inputs and output
// gradients rounded to bf16, ReLU' from the stored bf16 input.
#include <cuda_bf16.h>

#include "guide.cuh"

namespace rgr {
namespace dev {
namespace {

constexpr int kTrGroups = 2;                           // 128-sample tiles in flight per CTA
constexpr int kTrRows = 128;                           // samples per tile, one per row thread
constexpr int kTrMmaWarp = kTrGroups * 4;              // the MMA-issuing warp
constexpr int kTrThreads = kTrGroups * kTrRows + 32;
constexpr uint32_t kTileBytes = kTrRows * 128u;        // a tile's lines: 16 KB
constexpr int kTrBufs = 5;                             // B0..B3 and BY
constexpr int kBufY = 4;
constexpr uint32_t kWLayerBytes = 64u * 128u;          // W[in][out] of a layer, 64 lines
constexpr int kTurns = 10;                             // MMA turns per tile
// TMEM: dW of layer l in columns 64 l .. 64 l + 63 (lanes 0..63 dW[in][out],
// lanes 64..127 the bias gradient); group g's accumulator D at 320 + 64 g
constexpr uint32_t kDwCols = 64u * kGuideLayers;
constexpr int kTrCols = 512;
static_assert(kDwCols + 64u * kTrGroups <= (uint32_t)kTrCols, "TMEM columns");
constexpr uint32_t kWaitNs = 1000000000u;              // a wait gives up after 1 s (%globaltimer)
constexpr uint32_t kWaitPolls = 1u << 30;              // and after this many polls whatever the timer says
constexpr uint32_t kErrTrainTimeout = 2u;

struct __align__(1024) SmemTr {
    unsigned char w[kGuideLayers][kWLayerBytes];        // W[l][in][out], 128-byte swizzle (40 KB)
    unsigned char buf[kTrGroups][kTrBufs][kTileBytes];  // per group B0..B3, BY (160 KB)
    unsigned char ones[kTileBytes];                     // bf16 1.0: rows 64..127 of the dW MMAs' A (16 KB)
    float bias[kGuideLayers][kGuideWidth];
    unsigned long long a_full[kTrGroups];               // the turn's operand is written (128 arrivals)
    unsigned long long d_full[kTrGroups];               // the turn's MMAs are done (one commit)
    unsigned long long fin;                             // every MMA the CTA issued is done
    uint32_t tmem_base;
    uint32_t error;
    uint32_t trained;                                   // the MMA warp issued every turn of at least one tile
    float loss;
};
// the ones sit above every activation buffer: the dW MMAs reach them with a
// positive leading-byte offset of at most 160 KB (14 bits of 16-byte units)
static_assert(sizeof(SmemTr) + 1024 <= 232448, "shared memory");

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// shared-memory descriptor, 128-byte swizzle, version 1 (bits 46-47), swizzle
// mode 2 (bits 61-63), start address >> 4 (bits 0-13), leading byte offset
// >> 4 (bits 16-29), stride byte offset >> 4 (bits 32-45).
//  K-major: lines are M (or N) rows of 64 K elements; SBO 1024 between
//    8-row groups; LBO unused (16).
//  MN-major: lines are K rows of 64 M (or N) elements; SBO 1024 between
//    8-line groups along K; LBO between 64-element groups along M (or N).
__device__ __forceinline__ uint64_t desc_sw128(uint32_t saddr, uint32_t lbo) {
    return (uint64_t)((saddr & 0x3ffffu) >> 4) | ((uint64_t)((lbo >> 4) & 0x3fffu) << 16) |
           ((uint64_t)(1024 >> 4) << 32) | ((uint64_t)1 << 46) | ((uint64_t)2 << 61);
}
// instruction descriptors of kind::f16, D FP32 (bits 4-5 = 1), A and B BF16
// (bits 7-9, 10-12 = 1), N 64 (bits 17-22 = N >> 3), M 128 (bits 24-28 =
// M >> 4); bit 15 / 16 = A / B MN-major
constexpr uint32_t kIdescBase = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(64 >> 3) << 17) |
                                ((uint32_t)(128 >> 4) << 24);
constexpr uint32_t kIdescFwd = kIdescBase | (1u << 16);              // act (K-major) . W (MN-major)
constexpr uint32_t kIdescDx = kIdescBase;                             // dY (K-major) . W^T (K-major)
constexpr uint32_t kIdescDw = kIdescBase | (1u << 15) | (1u << 16);  // act^T (MN-major) . dY (MN-major)

__device__ __forceinline__ void mma_ss(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                       uint32_t accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(tmem_d),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate));
}
__device__ __forceinline__ void mma_commit(uint32_t mbar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(mbar)
                 : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint32_t mbar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}\n"
        : "=r"(ok)
        : "r"(mbar), "r"(parity)
        : "memory");
    return ok != 0u;
}
__device__ __forceinline__ bool mbar_test(uint32_t mbar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}\n"
        : "=r"(ok)
        : "r"(mbar), "r"(parity)
        : "memory");
    return ok != 0u;
}
__device__ __forceinline__ uint32_t global_ns() {
    uint32_t t;
    asm volatile("mov.u32 %0, %%globaltimer_lo;" : "=r"(t));
    return t;
}
// bounded wait for the phase with the given parity: false after kWaitNs (or kWaitPolls polls)
__device__ __forceinline__ bool mbar_wait(uint32_t mbar, uint32_t parity) {
    const uint32_t t0 = global_ns();
    for (uint32_t i = 0; i < kWaitPolls; ++i) {
        if (mbar_try_wait(mbar, parity)) return true;
        if ((i & 63u) == 63u && global_ns() - t0 > kWaitNs) return false;
    }
    return false;
}
__device__ __forceinline__ void mbar_arrive(uint32_t mbar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];\n" ::"r"(mbar) : "memory");
}
__device__ __forceinline__ void fence_before() { asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory"); }
__device__ __forceinline__ void fence_after() { asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory"); }
// generic-proxy shared-memory writes visible to the tensor core
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory"); }

__device__ __forceinline__ void tmem_ld32(uint32_t taddr, uint32_t* r) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
        "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
        "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];\n"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
          "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
          "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr));
}
__device__ __forceinline__ void tmem_ld8(uint32_t taddr, uint32_t* r) {
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];\n"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
                 : "r"(taddr));
}
__device__ __forceinline__ void tmem_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory"); }

__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi) {
    __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<uint32_t*>(&v);
}
__device__ __forceinline__ uint32_t relu_pack2(float lo, float hi) {
    uint32_t d;
    asm("cvt.rn.relu.bf16x2.f32 %0, %1, %2;\n" : "=r"(d) : "f"(hi), "f"(lo));
    return d;
}

// this sample's 128-byte line (64 bf16 packed in 32 words, element 2j in the
// low half of word j) into a tile buffer, 16-byte chunks at their swizzled
// places
__device__ __forceinline__ void store_line(unsigned char* tile, uint32_t r, const uint32_t* w) {
#pragma unroll
    for (uint32_t c = 0; c < 8; ++c)
        *reinterpret_cast<uint4*>(tile + sw128_offset(r, c)) = make_uint4(w[4 * c], w[4 * c + 1], w[4 * c + 2],
                                                                          w[4 * c + 3]);
}

// Frequency encoding of the sample (as guide_mlp.cu and guide_tc.cu):
// coordinate i gives the features 4i .. 4i + 3 = sin(pi v), cos(pi v),
// sin(2 pi v), cos(2 pi v), the first octave by the SFU's sine and cosine
// (absolute error near 2^-21 for these arguments, far below the bf16 rounding
// that follows), the second by the double-angle identities; inputs 36..63 are
// zero.
__device__ __forceinline__ void encode_line(const float* v, uint32_t* w) {
#pragma unroll
    for (int i = 0; i < 9; ++i) {
        float s, c;
        __sincosf(3.14159265358979f * v[i], &s, &c);
        w[2 * i] = pack_bf16(s, c);
        w[2 * i + 1] = pack_bf16(2.0f * s * c, (c - s) * (c + s));
    }
#pragma unroll
    for (int i = 18; i < 32; ++i) w[i] = 0u;
}

// One lobe of the mixture (guide.cuh's lobe_of) and its density, in the SFU's
// exponential, logarithm and reciprocal: the loss gradient is rounded to bf16
// right after, so their relative errors near 2^-21 do not show.  The weight
// logit keeps the accurate tanh, whose error would otherwise reach 2^-11.
struct LobeT {
    float mx, my, mz, kappa, inv_norm, norm, th, logit, sp;
};
__device__ __forceinline__ LobeT lobe_t(float o0, float o1, float o2, float o3, float o4) {
    LobeT L;
    const float ss = fmaxf(o0 * o0 + o1 * o1 + o2 * o2, 1.0e-24f);
    L.inv_norm = rsqrtf(ss);
    L.norm = ss * L.inv_norm;
    L.mx = o0 * L.inv_norm;
    L.my = o1 * L.inv_norm;
    L.mz = o2 * L.inv_norm;
    L.sp = o3 > 20.0f ? o3 : __logf(1.0f + __expf(o3));
    L.kappa = fminf(L.sp + 0.01f, kGuideKappaMax);
    L.th = tanhf(o4 * (1.0f / kGuideLogitBound));
    L.logit = kGuideLogitBound * L.th;
    return L;
}
__device__ __forceinline__ float vmf_t(float kappa, float c) {
    return __fdividef(kappa, 6.283185307179586f * (1.0f - __expf(-2.0f * kappa))) * __expf(kappa * (c - 1.0f));
}

// The loss of one sample, -wt log q(d), and its gradient with respect to the
// 41 raw outputs o (field-major mixture outputs, then the selection logit,
// whose term -wt log(a q + (1 - a) pb) holds q fixed), packed as the 32 words
// of dY's line: the derivatives of guide.cuh's lobe_grad.  The lobes are
// evaluated twice (once for q, once per pair for the gradient) instead of
// being kept, which holds the row thread's registers down.
__device__ __forceinline__ float row_loss_grad(const float* o, float dx, float dy, float dz, float wt, float pb,
                                               uint32_t* w) {
    float lg[kGuideLobes], f[kGuideLobes];
    float mx = -3.0e38f;
#pragma unroll
    for (int i = 0; i < kGuideLobes; ++i) {
        const LobeT L = lobe_t(o[i], o[8 + i], o[16 + i], o[24 + i], o[32 + i]);
        lg[i] = L.logit;
        f[i] = vmf_t(L.kappa, L.mx * dx + L.my * dy + L.mz * dz);
        mx = fmaxf(mx, L.logit);
    }
    float den = 0.0f;
#pragma unroll
    for (int i = 0; i < kGuideLobes; ++i) {
        lg[i] = __expf(lg[i] - mx);
        den += lg[i];
    }
    const float rden = __fdividef(1.0f, den);
    float q = 0.0f;
#pragma unroll
    for (int i = 0; i < kGuideLobes; ++i) {
        lg[i] *= rden;  // the lobe's weight pi
        q += lg[i] * f[i];
    }
    q = fmaxf(q, 1.0e-30f);
    const float rq = __fdividef(1.0f, q);
    const bool live = wt > 0.0f;
    // lobes 2m and 2m + 1 give field k's outputs 8k + 2m, 8k + 2m + 1: word 4k + m
#pragma unroll
    for (int m = 0; m < kGuideLobes / 2; ++m) {
        float gg[2][5];
#pragma unroll
        for (int s2 = 0; s2 < 2; ++s2) {
            const int i = 2 * m + s2;
            const LobeT L = lobe_t(o[i], o[8 + i], o[16 + i], o[24 + i], o[32 + i]);
            const float pi = lg[i], r = pi * f[i] * rq;
            float* g = gg[s2];
            g[4] = -wt * (r - pi) * (1.0f - L.th * L.th);
            const float k = L.kappa, e2 = __expf(-2.0f * k);
            const float md = L.mx * dx + L.my * dy + L.mz * dz;
            const float dlogf = __fdividef(1.0f, k) - __fdividef(2.0f * e2, 1.0f - e2) + (md - 1.0f);
            const float dk = (L.sp + 0.01f < kGuideKappaMax) ? __fdividef(1.0f, 1.0f + __expf(-o[24 + i])) : 0.0f;
            g[3] = -wt * r * dlogf * dk;
            const float gx = -wt * r * k * dx, gy = -wt * r * k * dy, gz = -wt * r * k * dz;
            const float gm = gx * L.mx + gy * L.my + gz * L.mz;
            const float pen = 2.0f * wt * kGuideNormPenalty * (L.norm - 1.0f);
            g[0] = (gx - gm * L.mx) * L.inv_norm + pen * L.mx;
            g[1] = (gy - gm * L.my) * L.inv_norm + pen * L.my;
            g[2] = (gz - gm * L.mz) * L.inv_norm + pen * L.mz;
        }
#pragma unroll
        for (int k = 0; k < 5; ++k) w[4 * k + m] = live ? pack_bf16(gg[0][k], gg[1][k]) : 0u;
    }
    w[kGuideSelOutput / 2] = live ? pack_bf16(selection_grad(o[kGuideSelOutput], q, pb, wt), 0.0f) : 0u;
#pragma unroll
    for (int j = kGuideSelOutput / 2 + 1; j < 32; ++j) w[j] = 0u;
    return live ? -wt * __logf(q) : 0.0f;
}

// the layer whose weight gradient turn `turn` accumulates (turns 5..9), or -1
__device__ __forceinline__ int dw_layer_of(uint32_t turn) { return turn >= 5u ? 9 - (int)turn : -1; }

// The MMAs of one turn of group g (the turns are listed at the top of the file).
// dw_started: bit l is set once a weight-gradient MMA of layer l has been issued
// (the first one of the CTA starts the accumulator, the others add to it).
__device__ __forceinline__ void issue_turn(uint32_t turn, uint32_t d, uint32_t dw, uint32_t w_addr,
                                           const uint32_t* bufs, uint32_t ones, uint32_t dw_started) {
    const uint32_t by = bufs[kBufY];
    auto fwd = [&](uint32_t act, uint32_t l, uint32_t ksteps) {
        for (uint32_t s = 0; s < ksteps; ++s)
            mma_ss(d, desc_sw128(act + 32u * s, 16u), desc_sw128(w_addr + l * kWLayerBytes + 2048u * s, 8192u),
                   kIdescFwd, s > 0u ? 1u : 0u);
    };
    auto dx = [&](uint32_t l) {
        for (uint32_t s = 0; s < 4u; ++s)
            mma_ss(d, desc_sw128(by + 32u * s, 16u), desc_sw128(w_addr + l * kWLayerBytes + 32u * s, 16u), kIdescDx,
                   s > 0u ? 1u : 0u);
    };
    auto dwl = [&](uint32_t act, uint32_t l) {
        const uint32_t acc = (dw_started >> l) & 1u;
        for (uint32_t s = 0; s < (uint32_t)kTrRows / 16u; ++s)
            mma_ss(dw + 64u * l, desc_sw128(act + 2048u * s, ones - act), desc_sw128(by + 2048u * s, 8192u),
                   kIdescDw, (acc || s > 0u) ? 1u : 0u);
    };
    switch (turn) {
        case 0: fwd(bufs[0], 0, 3); break;  // the encoding's 36 inputs fit in K = 48
        case 1: fwd(bufs[1], 1, 4); break;
        case 2: fwd(bufs[2], 2, 4); break;
        case 3: fwd(bufs[3], 3, 4); break;
        case 4: fwd(bufs[0], 4, 4); break;  // B0 holds act_4
        case 5: dx(4); dwl(bufs[0], 4); break;
        case 6: dx(3); dwl(bufs[3], 3); break;
        case 7: dx(2); dwl(bufs[2], 2); break;
        case 8: dx(1); dwl(bufs[1], 1); break;
        default: dwl(bufs[0], 0); break;    // B0 holds act_0 again
    }
}

// samples: 16 floats each (x, n, wo, wi, weight); loss weight = weight * scale,
// scale = weight_scale / *wsum (weight_scale without wsum).  part: this CTA's
// slot (kGuidePartStride floats) of the partials buffer.
// 168 registers a thread: the nine warps are spread over the SM's four 16,384-register
// sub-partitions, three on one of them
__global__ void __launch_bounds__(kTrThreads, 1)
    k_guide_train_tc(GuideView gv, const float* __restrict__ samples, const uint32_t* __restrict__ count, uint32_t cap,
                     uint32_t min_count, const float* __restrict__ wsum, float weight_scale, float* __restrict__ part,
                     uint32_t* err) {
    const uint32_t n = min(*count, cap);
    if (n < min_count) return;  // too few yet: the samples carry over (the reduction skips too)
    float* my_part = part + (size_t)blockIdx.x * kGuidePartStride;
    const uint32_t ntiles = (n + kTrRows - 1u) / kTrRows, stride = gridDim.x * kTrGroups;
    if (blockIdx.x * kTrGroups >= ntiles) {  // no tile here: an empty slot
        for (uint32_t i = threadIdx.x; i < kGuidePartStride; i += blockDim.x) my_part[i] = 0.0f;
        return;
    }
    extern __shared__ unsigned char smem_raw[];
    SmemTr& S = *reinterpret_cast<SmemTr*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    const uint32_t t = threadIdx.x, lt = t & 127u, lane = t & 31u;
    const uint32_t warp = __shfl_sync(0xffffffffu, t >> 5, 0), g = warp >> 2;
    float scale = weight_scale;
    if (wsum) {
        const float s = *wsum;
        scale = s > 0.0f ? weight_scale / s : 0.0f;
    }
    // stage the weights as W[in][out] lines, the biases and the ones
    {
        const uint4* src = reinterpret_cast<const uint4*>(gv.wbf);
        for (uint32_t i = t; i < (uint32_t)kGuideLayers * 64u * 8u; i += blockDim.x) {
            const uint32_t l = i >> 9, in = (i >> 3) & 63u, c = i & 7u;
            *reinterpret_cast<uint4*>(S.w[l] + sw128_offset(in, c)) = src[i];
        }
        for (uint32_t i = t; i < (uint32_t)kGuideBiases; i += blockDim.x) (&S.bias[0][0])[i] = gv.b[i];
        for (uint32_t i = t; i < kTileBytes / 16u; i += blockDim.x)
            reinterpret_cast<uint4*>(S.ones)[i] = make_uint4(0x3f803f80u, 0x3f803f80u, 0x3f803f80u, 0x3f803f80u);
    }
    if (t == 0) {
        S.error = 0u;
        S.trained = 0u;
        S.loss = 0.0f;
        for (int i = 0; i < kTrGroups; ++i) {
            asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(smem_u32(&S.a_full[i])), "r"(kTrRows)
                         : "memory");
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(smem_u32(&S.d_full[i])) : "memory");
        }
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(smem_u32(&S.fin)) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(smem_u32(&S.tmem_base)),
                     "r"(kTrCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
    }
    fence_async_smem();
    fence_before();
    __syncthreads();
    fence_after();
    const uint32_t tmem = S.tmem_base;
    auto tiles_of = [&](uint32_t gg) -> uint32_t {
        const uint32_t base = blockIdx.x * kTrGroups + gg;
        return base < ntiles ? (ntiles - base + stride - 1u) / stride : 0u;
    };

    if (warp == (uint32_t)kTrMmaWarp) {
        // ------------------------------------------------------------ MMA warp
        uint32_t left[kTrGroups], turn[kTrGroups], ph[kTrGroups], bufs[kTrGroups][kTrBufs];
#pragma unroll
        for (int i = 0; i < kTrGroups; ++i) {
            left[i] = kTurns * tiles_of(i);
            turn[i] = 0u;
            ph[i] = 0u;
#pragma unroll
            for (int b = 0; b < kTrBufs; ++b) bufs[i][b] = smem_u32(S.buf[i][b]);
        }
        const uint32_t w_addr = smem_u32(S.w), ones = smem_u32(S.ones);
        uint32_t dw_started = 0u;
        uint32_t last = global_ns(), idle = 0u;
        for (;;) {
            bool any = false, progressed = false;
#pragma unroll
            for (int i = 0; i < kTrGroups; ++i) {
                if (left[i] == 0u) continue;
                any = true;
                const bool ready = __shfl_sync(0xffffffffu, (uint32_t)mbar_test(smem_u32(&S.a_full[i]), ph[i]), 0) != 0u;
                if (!ready) continue;
                ph[i] ^= 1u;
                fence_after();
                // lane 0 issues every MMA of the CTA and the commits that track them:
                // one thread's tcgen05 operations run in issue order, which the two
                // groups' additions into the shared dW accumulators rely on
                if (lane == 0u) {
                    issue_turn(turn[i], tmem + kDwCols + 64u * i, tmem, w_addr, bufs[i], ones, dw_started);
                    mma_commit(smem_u32(&S.d_full[i]));
                }
                __syncwarp();
                const int dl = dw_layer_of(turn[i]);
                if (dl >= 0) dw_started |= 1u << dl;
                turn[i] = turn[i] + 1u == (uint32_t)kTurns ? 0u : turn[i] + 1u;
                --left[i];
                progressed = true;
            }
            if (!any) break;
            idle = progressed ? 0u : idle + 1u;
            if (progressed) last = global_ns();
            else if (idle > 4u) __nanosleep(32);  // leave the issue slots to the row threads
            if (idle >= kWaitPolls || ((idle & 63u) == 63u && global_ns() - last > kWaitNs)) {
                if (lane == 0u) S.error = kErrTrainTimeout;  // a group stopped arriving
                break;
            }
        }
        // every MMA issued above has completed before TMEM is read or freed
        if (lane == 0u) mma_commit(smem_u32(&S.fin));
        __syncwarp();
        const bool fin_ok = mbar_wait(smem_u32(&S.fin), 0u);
        if (lane == 0u) {
            if (!fin_ok) S.error = kErrTrainTimeout;
            if (dw_started == (1u << kGuideLayers) - 1u) S.trained = 1u;
        }
    } else {
        // ------------------------------------------------------------ row threads
        const uint32_t lane_off = (32u * (warp & 3u)) << 16;  // this warp's 32 TMEM lanes
        const uint32_t d = tmem + kDwCols + 64u * g + lane_off;
        unsigned char* B0 = S.buf[g][0];
        unsigned char* BY = S.buf[g][kBufY];
        const uint32_t af = smem_u32(&S.a_full[g]), df = smem_u32(&S.d_full[g]);
        const uint32_t kt = tiles_of(g), base = blockIdx.x * kTrGroups + g;
        uint32_t pd = 0u;
        bool timed_out = false;
        float lsum = 0.0f;
        // hand the turn's operand to the MMA warp, then wait for its MMAs
        auto handoff = [&]() -> bool {
            fence_async_smem();  // the lines just written, to the tensor core
            fence_before();      // the accumulator reads just done, before the next MMAs
            mbar_arrive(af);
            if (!mbar_wait(df, pd)) {
                S.error = kErrTrainTimeout;
                return false;
            }
            pd ^= 1u;
            fence_after();
            return true;
        };
        for (uint32_t k = 0; k < kt && !timed_out; ++k) {
            const uint32_t r = (base + k * stride) * (uint32_t)kTrRows + lt;
            float v[9], dir[3] = {0.0f, 0.0f, 0.0f}, wt = 0.0f, pb = 0.0f;
            {
                float x9[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
                if (r < n) {
                    const float4* s4 = reinterpret_cast<const float4*>(samples + 16 * (size_t)r);
                    const float4 a = __ldg(s4), b = __ldg(s4 + 1), c = __ldg(s4 + 2), e = __ldg(s4 + 3);
                    x9[0] = a.x, x9[1] = a.y, x9[2] = a.z, x9[3] = a.w, x9[4] = b.x, x9[5] = b.y;
                    x9[6] = b.z, x9[7] = b.w, x9[8] = c.x;
                    dir[0] = c.y, dir[1] = c.z, dir[2] = c.w;
                    wt = e.x * scale;
                    pb = e.y;
                }
#pragma unroll
                for (int c = 0; c < 3; ++c) {
                    v[c] = (x9[c] - gv.params.lo[c]) * gv.params.inv_ext[c];
                    v[3 + c] = 0.5f * (x9[3 + c] + 1.0f);
                    v[6 + c] = 0.5f * (x9[6 + c] + 1.0f);
                }
            }
            uint32_t line[32];
            encode_line(v, line);
            store_line(B0, lt, line);
            // forward: turns 0..4
            float o[kGuideNetOutputs];
#pragma unroll 1
            for (uint32_t l = 0; l < (uint32_t)kGuideLayers; ++l) {
                if (!handoff()) {
                    timed_out = true;
                    break;
                }
                if (l + 1u < (uint32_t)kGuideLayers) {
                    unsigned char* next = l + 1u < 4u ? S.buf[g][l + 1u] : B0;  // act_4 into B0
                    // two halves of 32 accumulators: 16 words, 4 chunks of the line each
#pragma unroll
                    for (uint32_t h = 0; h < 2u; ++h) {
                        uint32_t x[32], y[16];
                        tmem_ld32(d + 32u * h, x);
                        tmem_wait_ld();
#pragma unroll
                        for (int c = 0; c < 16; ++c) {
                            const int e = 32 * (int)h + 2 * c;
                            y[c] = relu_pack2(__uint_as_float(x[2 * c]) + S.bias[l][e],
                                              __uint_as_float(x[2 * c + 1]) + S.bias[l][e + 1]);
                        }
#pragma unroll
                        for (uint32_t c = 0; c < 4u; ++c)
                            *reinterpret_cast<uint4*>(next + sw128_offset(lt, 4u * h + c)) =
                                make_uint4(y[4 * c], y[4 * c + 1], y[4 * c + 2], y[4 * c + 3]);
                    }
                } else {
                    uint32_t x[48];
                    tmem_ld32(d, x);
                    tmem_ld8(d + 32u, x + 32);
                    tmem_ld8(d + 40u, x + 40);
                    tmem_wait_ld();
#pragma unroll
                    for (int c = 0; c < kGuideNetOutputs; ++c) o[c] = __uint_as_float(x[c]) + S.bias[l][c];
                }
            }
            if (timed_out) break;
            // loss gradient: dY_4 (turn 5)
            lsum += row_loss_grad(o, dir[0], dir[1], dir[2], wt, pb, line);
            store_line(BY, lt, line);
            // backward: turns 5..8 give dX of layers 4..1; masked by ReLU' of the layer's
            // input (read back from this sample's line: act_l is > 0 where its bf16 is
            // not zero), it is dY of layers 3..0
#pragma unroll 1
            for (int l = 4; l >= 1; --l) {
                if (!handoff()) {
                    timed_out = true;
                    break;
                }
                const unsigned char* act = l == 4 ? B0 : S.buf[g][l];
#pragma unroll
                for (uint32_t h = 0; h < 2u; ++h) {
                    uint32_t x[32], y[16];
                    tmem_ld32(d + 32u * h, x);
                    tmem_wait_ld();
#pragma unroll
                    for (uint32_t c = 0; c < 4u; ++c) {
                        const uint4 a = *reinterpret_cast<const uint4*>(act + sw128_offset(lt, 4u * h + c));
                        const uint32_t aw[4] = {a.x, a.y, a.z, a.w};
#pragma unroll
                        for (int j = 0; j < 4; ++j) {
                            const int k = 4 * (int)c + j;  // word k of the half: inputs 32 h + 2k, + 1
                            y[k] = pack_bf16((aw[j] & 0xffffu) ? __uint_as_float(x[2 * k]) : 0.0f,
                                             (aw[j] >> 16) ? __uint_as_float(x[2 * k + 1]) : 0.0f);
                        }
                    }
#pragma unroll
                    for (uint32_t c = 0; c < 4u; ++c)
                        *reinterpret_cast<uint4*>(BY + sw128_offset(lt, 4u * h + c)) =
                            make_uint4(y[4 * c], y[4 * c + 1], y[4 * c + 2], y[4 * c + 3]);
                }
                if (l == 4) {  // dW_4 has read act_4: act_0 back into B0 for dW_0
                    uint32_t e[32];
                    encode_line(v, e);
                    store_line(B0, lt, e);
                }
            }
            if (timed_out) break;
            // turn 9: dW_0; its end frees B0 and BY for the next tile
            if (!handoff()) timed_out = true;
        }
        // this group's loss
        for (int off = 16; off > 0; off >>= 1) lsum += __shfl_xor_sync(0xffffffffu, lsum, off);
        if ((t & 31u) == 0u) atomicAdd(&S.loss, lsum);
    }
    fence_before();
    __syncthreads();
    fence_after();
    // the CTA's gradients: dW rows from TMEM lanes 0..63 (warps 0 and 1), the bias
    // gradient from lane 64 (warp 2); zeros if a timeout left them incomplete
    const bool ok = S.trained != 0u && S.error == 0u;
    if (warp < 3u) {
        for (uint32_t l = 0; l < (uint32_t)kGuideLayers; ++l) {
            for (uint32_t h = 0; h < 2u; ++h) {
                uint32_t x[32];
                tmem_ld32(tmem + 64u * l + 32u * h + ((32u * warp) << 16), x);
                tmem_wait_ld();
                float* row = warp < 2u ? my_part + (size_t)l * 4096u + (size_t)t * 64u : my_part + kGuideWeights + l * 64u;
                if (warp < 2u || lt == 64u) {
                    float4* dst = reinterpret_cast<float4*>(row + 32u * h);
#pragma unroll
                    for (int c = 0; c < 8; ++c)
                        dst[c] = ok ? make_float4(__uint_as_float(x[4 * c]), __uint_as_float(x[4 * c + 1]),
                                                  __uint_as_float(x[4 * c + 2]), __uint_as_float(x[4 * c + 3]))
                                    : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
                }
            }
        }
    }
    if (t == 0) my_part[kGuideParams] = ok ? S.loss : 0.0f;
    fence_before();
    __syncthreads();
    if (warp == 0) {
        fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(kTrCols) : "memory");
    }
    if (t == 0 && S.error && err) atomicOr(err, S.error);
}

// gW, gb and the loss as the sums of the CTAs' slots, in a fixed order: a
// block covers 32 parameters; its 8 warps each sum every 8th slot (a warp's
// loads are 32 consecutive floats of one slot), then one warp adds the 8
// partial sums in warp order.
constexpr int kReduceParams = 32, kReduceWarps = 8;
__global__ void __launch_bounds__(32 * kReduceWarps) k_guide_grad_reduce(GuideView g, const float* __restrict__ part,
                                                                          uint32_t nparts, const uint32_t* count,
                                                                          uint32_t min_count) {
    if (*count == 0u || *count < min_count) return;
    __shared__ float partial[kReduceWarps][kReduceParams];
    const uint32_t lane = threadIdx.x & 31u, w = threadIdx.x >> 5;
    const uint32_t i = blockIdx.x * kReduceParams + lane;
    float s = 0.0f;
    if (i <= (uint32_t)kGuideParams)
        for (uint32_t c = w; c < nparts; c += kReduceWarps) s += __ldg(part + (size_t)c * kGuidePartStride + i);
    partial[w][lane] = s;
    __syncthreads();
    if (w != 0u || i > (uint32_t)kGuideParams) return;
    float t = 0.0f;
#pragma unroll
    for (int k = 0; k < kReduceWarps; ++k) t += partial[k][lane];
    if (i < (uint32_t)kGuideWeights) g.gW[i] = t;
    else if (i < (uint32_t)kGuideParams) g.gb[i - kGuideWeights] = t;
    else *g.loss = t;
}

}  // namespace

size_t guide_train_tc_smem() { return sizeof(SmemTr) + 1024; }

int guide_train_tc_attributes() {
    return (int)cudaFuncSetAttribute(k_guide_train_tc, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)guide_train_tc_smem());
}

void launch_guide_train_tc(const GuideView& g, const float* samples, const uint32_t* count, uint32_t cap,
                           uint32_t min_count, const float* wsum, float weight_scale, int grid, float* part,
                           uint32_t* err, cudaStream_t st) {
    k_guide_train_tc<<<grid, kTrThreads, guide_train_tc_smem(), st>>>(g, samples, count, cap, min_count, wsum,
                                                                      weight_scale, part, err);
}

void launch_guide_grad_reduce(const GuideView& g, const float* part, uint32_t nparts, const uint32_t* count,
                              uint32_t min_count, cudaStream_t st) {
    k_guide_grad_reduce<<<(kGuideParams + kReduceParams) / kReduceParams, 32 * kReduceWarps, 0, st>>>(
        g, part, nparts, count, min_count);
}

}  // namespace dev
}  // namespace rgr
