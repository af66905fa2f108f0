// guide_tc.cu — inference of the path-guiding network on the 5th-generation
// tensor cores: tcgen05.mma with the accumulators and the activations in
// tensor memory (TMEM) and the weights in shared memory.
//
// A CTA (one per SM) holds kTcGroups groups of 128 row threads and kMmaWarps
// warps that only issue MMAs.  A group works on tiles of 128 rows, kBufs tiles
// in flight (buffers); thread t of the group owns row t of each from the input
// encoding to the result.  Per tile in flight TMEM holds the
// 128 x 64 FP32 accumulator and the layer's input as 64 bf16 a row (lane =
// row).  Per layer and buffer:
//  * the row threads write the layer's input into TMEM (tcgen05.st): the
//    encoding for the first layer, else the ReLU of the previous layer's
//    accumulators, packed to bf16 in the same conversion (cvt.rn.relu.bf16x2);
//    then they arrive on the buffer's a_full mbarrier;
//  * an MMA warp, polling its buffers' a_full barriers, issues the layer
//    (M 128, N 64, K 16, BF16 x BF16 -> FP32, A from TMEM, B = the layer's W^T
//    from shared memory, 128-byte swizzle): for a hidden or the output layer
//    one MMA that starts the accumulator at the bias (a TMEM chunk of ones
//    times a B chunk holding each bias as the sum of two bf16 values), then
//    one per 16 inputs; the first layer's 3 MMAs cover the encoding's 36
//    inputs and two inputs fixed at 1.0 that carry its bias.  It commits them
//    to the buffer's d_full mbarrier;
//  * the row threads wait on d_full (a bounded wait) and read the
//    accumulators back (tcgen05.ld).
// While the tensor core runs one tile's layer, the row threads of the other
// tiles (other groups, or the group's other buffers) run their epilogues.  After the last layer each thread has its row's 40
// outputs in registers and computes the mixture (or keeps the raw outputs)
// without any exchange; the tile's results (80-byte FP16 mixture records, or
// 192 bytes of raw outputs) are staged in shared memory and leave in one bulk
// copy.  Weights and bias chunks are staged once
// per CTA by one bulk copy.  Every wait is bounded: on a timeout the CTA
// records an error, stops issuing and frees its TMEM.
#include <cuda_bf16.h>

#include "guide.cuh"

namespace rgr {
namespace dev {
namespace {

// 128-row groups of row threads per CTA, and tiles in flight per group.  Five
// groups of one tile each (2^18 rows: 19.0 us) beat two of two tiles (21.1 us)
// and one of four or five (27 us): the row threads' encoding, epilogues and
// mixtures, more than the MMAs, need the parallelism.  Five tiles of 96 TMEM
// columns and the ones chunk fill the SM's 512 columns.
#ifndef RGR_GUIDE_TC_GROUPS
#define RGR_GUIDE_TC_GROUPS 5
#endif
constexpr int kTcGroups = RGR_GUIDE_TC_GROUPS;
#ifndef RGR_GUIDE_TC_BUFS
#define RGR_GUIDE_TC_BUFS 1
#endif
constexpr int kBufs = RGR_GUIDE_TC_BUFS;              // tiles in flight per group
constexpr int kGroupThreads = 128;                    // rows per tile, one per thread
// warps that issue the MMAs: warp kMmaWarp + m serves the buffers b = i kBufs + j
// (group i, buffer j) with b % kMmaWarps == m (an issuing thread waits out
// most of each MMA's issue latency, so buffers that share a warp share it)
#ifndef RGR_GUIDE_TC_MMA_WARPS
#define RGR_GUIDE_TC_MMA_WARPS 3
#endif
constexpr int kMmaWarps = RGR_GUIDE_TC_MMA_WARPS;
constexpr int kMmaWarp = kTcGroups * 4;               // the first MMA warp
constexpr int kTcThreads = kTcGroups * kGroupThreads + 32 * kMmaWarps;
constexpr uint32_t kCtaRows = kTcGroups * 128u;       // rows of one tile per group
constexpr int kAccs = kTcGroups * kBufs;              // tiles in flight per CTA
// TMEM per tile in flight: the 128 x 64 FP32 accumulator (columns 0..63) and
// the layer's input, 64 bf16 a row packed in pairs (columns 64..95); then the
// ones chunk of the bias MMAs (row elements 0 and 1 are 1.0; 8 columns read,
// 32 written)
constexpr uint32_t kAccCols = 96;
constexpr uint32_t kOnesCol = kAccs * kAccCols;
constexpr int kTcCols = 512;                          // TMEM columns allocated (a power of two)
static_assert(kOnesCol + 32 <= (uint32_t)kTcCols, "TMEM columns");
constexpr uint32_t kWaitNs = 1000000000u;             // a wait gives up after 1 s (%globaltimer)
constexpr uint32_t kWaitPolls = 1u << 30;             // and after this many polls whatever the timer says
constexpr uint32_t kErrTimeout = 1u;

struct __align__(1024) SmemTc {
    unsigned char wt[kGuideWtBytes];                // the staged weights and bias chunks (50 x 1024 B)
    unsigned char out[kTcGroups][128 * 4 * kGuideRowOutputs];  // a tile's output rows (80 or 192 bytes), one bulk copy
    unsigned long long wbar;                        // the weights' bulk copy
    unsigned long long a_full[kTcGroups][kBufs];    // the A tile of the next layer is written (128 arrivals)
    unsigned long long d_full[kTcGroups][kBufs];    // the layer's MMAs are done (one commit)
    uint32_t tmem_base;
    uint32_t error;
};

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// shared-memory matrix descriptor of a K-major, 128-byte-swizzled operand:
// start address >> 4 (bits 0-13), leading byte offset 1 (unused with this
// swizzle, bits 16-29), stride byte offset 1024 >> 4 between 8-row groups
// (bits 32-45), descriptor version 1 (bits 46-47), swizzle mode 2 = 128 B
// (bits 61-63)
__device__ __forceinline__ uint64_t desc_sw128(uint32_t saddr) {
    return (uint64_t)((saddr & 0x3ffffu) >> 4) | ((uint64_t)1 << 16) | ((uint64_t)(1024 >> 4) << 32) |
           ((uint64_t)1 << 46) | ((uint64_t)2 << 61);
}
// descriptor of a K-major 16-wide chunk without swizzle (k16_offset): leading
// byte offset 128 between the two core matrices along K, stride byte offset
// 256 between 8-row groups, swizzle mode 0
__device__ __forceinline__ uint64_t desc_k16(uint32_t saddr) {
    return (uint64_t)((saddr & 0x3ffffu) >> 4) | ((uint64_t)(128 >> 4) << 16) | ((uint64_t)(256 >> 4) << 32) |
           ((uint64_t)1 << 46);
}

// instruction descriptor of kind::f16: D FP32 (bits 4-5 = 1), A and B BF16
// (bits 7-9 and 10-12 = 1), both K-major (bits 15, 16 = 0), N >> 3 in bits
// 17-22, M >> 4 in bits 24-28
constexpr uint32_t kIdesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(64 >> 3) << 17) |
                            ((uint32_t)(128 >> 4) << 24);

// D (+)= A B with A (128 rows x 16 bf16 in 8 TMEM columns, a row per lane) in
// TMEM and B in shared memory
__device__ __forceinline__ void mma_bf16_ts(uint32_t tmem_d, uint32_t tmem_a, uint64_t bdesc, uint32_t accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], [%1], %2, %3, p;\n\t}\n"
        :
        : "r"(tmem_d), "r"(tmem_a), "l"(bdesc), "r"(kIdesc), "r"(accumulate));
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
// low 32 bits of %globaltimer (ns): differences stay right across its
// 4.3 s wrap, far longer than kWaitNs
__device__ __forceinline__ uint32_t global_ns() {
    uint32_t t;
    asm volatile("mov.u32 %0, %%globaltimer_lo;" : "=r"(t));
    return t;
}
// bounded wait for the phase with the given parity: false after kWaitNs (or
// kWaitPolls polls)
__device__ __forceinline__ bool mbar_wait(uint32_t mbar, uint32_t parity) {
    const uint32_t t0 = global_ns();
    for (uint32_t i = 0; i < kWaitPolls; ++i) {
        if (mbar_try_wait(mbar, parity)) return true;
        if ((i & 63u) == 63u && global_ns() - t0 > kWaitNs) return false;
    }
    return false;
}
// true in one lane of the (converged) warp
__device__ __forceinline__ bool elect_one() {
    uint32_t p;
    asm volatile(
        "{\n\t.reg .pred e;\n\t"
        "elect.sync _|e, 0xffffffff;\n\t"
        "selp.u32 %0, 1, 0, e;\n\t}\n"
        : "=r"(p));
    return p != 0u;
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
__device__ __forceinline__ void mbar_arrive(uint32_t mbar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];\n" ::"r"(mbar) : "memory");
}
__device__ __forceinline__ void fence_before() { asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory"); }
__device__ __forceinline__ void fence_after() { asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory"); }
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory"); }

// barrier of group g's 128 threads (named barrier g + 1) that also returns
// whether any of them passed `mine` = true, the same answer in every thread
__device__ __forceinline__ bool group_sync_any(uint32_t g, bool mine) {
    uint32_t r;
    asm volatile(
        "{\n\t.reg .pred p, q;\n\t"
        "setp.ne.u32 q, %1, 0;\n\t"
        "bar.red.or.pred p, %2, %3, q;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}\n"
        : "=r"(r)
        : "r"((uint32_t)mine), "r"(g + 1u), "r"((uint32_t)kGroupThreads)
        : "memory");
    return r != 0u;
}

// FP32 accumulators of this thread's TMEM lane: 32 columns / 8 columns from taddr
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
__device__ __forceinline__ void tmem_ld1(uint32_t taddr, uint32_t* r) {
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x1.b32 {%0}, [%1];\n" : "=r"(r[0]) : "r"(taddr));
}
__device__ __forceinline__ void tmem_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory"); }
// 32 columns of this thread's TMEM lane from registers
__device__ __forceinline__ void tmem_st32(uint32_t taddr, const uint32_t* r) {
    asm volatile(
        "tcgen05.st.sync.aligned.32x32b.x32.b32 [%0], "
        "{%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,"
        "%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31,%32};\n" ::"r"(taddr),
        "r"(r[0]), "r"(r[1]), "r"(r[2]), "r"(r[3]), "r"(r[4]), "r"(r[5]), "r"(r[6]), "r"(r[7]), "r"(r[8]),
        "r"(r[9]), "r"(r[10]), "r"(r[11]), "r"(r[12]), "r"(r[13]), "r"(r[14]), "r"(r[15]), "r"(r[16]),
        "r"(r[17]), "r"(r[18]), "r"(r[19]), "r"(r[20]), "r"(r[21]), "r"(r[22]), "r"(r[23]), "r"(r[24]),
        "r"(r[25]), "r"(r[26]), "r"(r[27]), "r"(r[28]), "r"(r[29]), "r"(r[30]), "r"(r[31])
        : "memory");
}
__device__ __forceinline__ void tmem_wait_st() { asm volatile("tcgen05.wait::st.sync.aligned;\n" ::: "memory"); }

__device__ __forceinline__ uint32_t pack2(float lo, float hi) {
    __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<uint32_t*>(&v);
}
// bf16 pair (max(lo, 0), max(hi, 0)), lo in the low half
__device__ __forceinline__ uint32_t relu_pack2(uint32_t lo, uint32_t hi) {
    uint32_t d;
    asm("cvt.rn.relu.bf16x2.f32 %0, %1, %2;\n" : "=r"(d) : "f"(__uint_as_float(hi)), "f"(__uint_as_float(lo)));
    return d;
}

// Encoding (as guide_mlp.cu): coordinate i gives the features 4i .. 4i + 3 =
// sin(pi v), cos(pi v), sin(2 pi v), cos(2 pi v), the second octave by the
// double-angle identities, the first by the SFU's sine and cosine (absolute
// error near 2^-21 for these arguments, far below the bf16 rounding that
// follows).  The row's 48 inputs as the first layer's A: 24 TMEM columns of
// bf16 pairs (features 2c, 2c + 1 in column c, the lower one in the low
// half); inputs 36 and 37 are 1.0 and carry the layer's bias, 38..47 zero.
__device__ __forceinline__ void encode_store(uint32_t taddr, const float* x9, const GuideParams& gp) {
    float v[9];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        v[c] = (x9[c] - gp.lo[c]) * gp.inv_ext[c];
        v[3 + c] = 0.5f * (x9[3 + c] + 1.0f);
        v[6 + c] = 0.5f * (x9[6 + c] + 1.0f);
    }
    uint32_t w[32];
#pragma unroll
    for (int i = 0; i < 9; ++i) {
        float s, c;
        __sincosf(3.14159265358979f * v[i], &s, &c);
        w[2 * i] = pack2(s, c);
        w[2 * i + 1] = pack2(2.0f * s * c, (c - s) * (c + s));
    }
    w[18] = 0x3f803f80u;
#pragma unroll
    for (int i = 19; i < 32; ++i) w[i] = 0u;
    tmem_st32(taddr, w);
}

// ReLU of this row's 64 accumulators, as the next layer's A (32 columns at a_taddr)
__device__ __forceinline__ void relu_store(uint32_t d_taddr, uint32_t a_taddr) {
    uint32_t x[64], y[32];
    tmem_ld32(d_taddr, x);
    tmem_ld32(d_taddr + 32u, x + 32);
    tmem_wait_ld();
#pragma unroll
    for (int c = 0; c < 32; ++c) y[c] = relu_pack2(x[2 * c], x[2 * c + 1]);
    tmem_st32(a_taddr, y);
}

__device__ __forceinline__ float tanh_approx(float x) {
    float y;
    asm("tanh.approx.f32 %0, %1;\n" : "=f"(y) : "f"(x));
    return y;
}
__device__ __forceinline__ float softplus_fast(float x) { return x > 20.0f ? x : __logf(1.0f + __expf(x)); }

// The mixture of one row's 40 raw outputs (field-major) as the FP16 record
// the shading kernel reads (guide.cuh), the functions of guide_mlp.cu's
// lobe_of in hardware approximations: the mixture only has to be the one the
// shading kernel samples and evaluates, which decodes it from here.  The
// weights are stored scaled by the guide's share `alpha` of the vertex.
__device__ __forceinline__ void row_mixture(const float* o, float alpha, uint4* dst) {
    float w[kGuideLobes], mx = -3.0e38f;
#pragma unroll
    for (int i = 0; i < kGuideLobes; ++i) {
        w[i] = kGuideLogitBound * tanh_approx(o[32 + i] * (1.0f / kGuideLogitBound));
        mx = fmaxf(mx, w[i]);
    }
    float den = 0.0f;
    uint2 lobe[kGuideLobes];
#pragma unroll
    for (int i = 0; i < kGuideLobes; ++i) {
        const float x = o[i], y = o[8 + i], z = o[16 + i];
        const float inv = rsqrtf(fmaxf(x * x + y * y + z * z, 1.0e-24f));
        lobe[i] = make_uint2(half2_bits(x * inv, y * inv),
                             half2_bits(z * inv, fminf(softplus_fast(o[24 + i]) + 0.01f, kGuideKappaMax)));
        w[i] = __expf(w[i] - mx);
        den += w[i];
    }
    const float r = alpha / den;
#pragma unroll
    for (int i = 0; i < 4; ++i) dst[i] = make_uint4(lobe[2 * i].x, lobe[2 * i].y, lobe[2 * i + 1].x, lobe[2 * i + 1].y);
    dst[4] = make_uint4(half2_bits(w[0] * r, w[1] * r), half2_bits(w[2] * r, w[3] * r), half2_bits(w[4] * r, w[5] * r),
                        half2_bits(w[6] * r, w[7] * r));
}

// The 48 bytes a row's input comes from: the slot's (ro, rd, ng) for a
// path vertex, the first 12 floats of a 16-float row otherwise.
struct RowIn {
    float4 a, b, c;
};
template <bool kPaths>
__device__ __forceinline__ RowIn load_row(const PathsView& P, const float* rows, uint32_t r, uint32_t slot) {
    if (kPaths) return RowIn{P.ro[slot], P.rd[slot], P.ng[slot]};
    const float4* p = reinterpret_cast<const float4*>(rows + 16 * (size_t)r);
    return RowIn{p[0], p[1], p[2]};
}
// the network's input: hit point, normal facing the outgoing direction (zero
// inside a volume), outgoing direction; or the row's first 9 floats
template <bool kPaths>
__device__ __forceinline__ void row_x9(const RowIn& in, float* x9) {
    if (!kPaths) {
        x9[0] = in.a.x, x9[1] = in.a.y, x9[2] = in.a.z, x9[3] = in.a.w;
        x9[4] = in.b.x, x9[5] = in.b.y, x9[6] = in.b.z, x9[7] = in.b.w;
        x9[8] = in.c.x;
        return;
    }
    const float4 ro = in.a, rd = in.b, ng = in.c;
    x9[0] = ro.x + rd.x * ro.w;
    x9[1] = ro.y + rd.y * ro.w;
    x9[2] = ro.z + rd.z * ro.w;
    float nx = ng.x, ny = ng.y, nz = ng.z;
    if (__float_as_int(ng.w) < 0) {
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

// the layer's MMAs into accumulator `tm` from its A columns `ta`, committed to
// `done`: the bias (ones times the layer's bias chunk; layer 0's rides on its
// inputs), then 16 inputs per step
__device__ __forceinline__ void issue_layer(uint32_t l, uint32_t tm, uint32_t ta, uint32_t ones, uint32_t wt_addr,
                                            uint32_t done) {
    if (l > 0u) mma_bf16_ts(tm, ones, desc_k16(wt_addr + wt_bias_offset(l, 0, 0)), 0u);
    const uint32_t b_base = wt_addr + 8192u * l;
    // K = 16 per step: 8 TMEM columns of A, 32 B inside B's swizzled line
    for (uint32_t k = 0; k < (l == 0u ? 3u : 4u); ++k)
        mma_bf16_ts(tm, ta + 8u * k, desc_sw128(b_base + 32u * k), (l > 0u || k > 0u) ? 1u : 0u);
    mma_commit(done);
}

// kPaths: rows are this bounce's guided queue items, output their mixtures;
// otherwise rows of 16 floats in `rows`, output 40 raw floats per row.
//
// Tile k of group g is tile (blockIdx.x + k gridDim.x) kTcGroups + g of the
// rows; the group runs its tiles kBufs at a time, tile k in buffer k % kBufs.
// Per layer and buffer the group's threads write the layer's input and arrive
// on a_full; the MMA warp serving the buffer, polling its a_full barriers,
// issues that buffer's next layer and commits it to d_full; the threads wait
// on d_full and run the epilogue.
template <bool kPaths>
__global__ void __launch_bounds__(kTcThreads, 1)
    k_guide_infer_tc(GuideView gv, const float* __restrict__ rows, uint32_t nrows, float* __restrict__ out,
                     PathsView P, QueueView Q, GuideRenderD gd, uint32_t* err) {
    extern __shared__ unsigned char smem_raw[];
    SmemTc& S = *reinterpret_cast<SmemTc*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    const uint32_t n = kPaths ? guide_rows(Q, gd) : nrows;
    if (blockIdx.x * kCtaRows >= n) return;
    const uint32_t t = threadIdx.x, lt = t & 127u;
    // warp and group indices the compiler knows to be warp-uniform, so that the
    // MMA operands derived from them live in uniform registers
    const uint32_t warp = __shfl_sync(0xffffffffu, t >> 5, 0), g = warp >> 2;
    if (t == 0) {
        S.error = 0u;
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(smem_u32(&S.wbar)) : "memory");
        for (int i = 0; i < kTcGroups; ++i)
            for (int j = 0; j < kBufs; ++j) {
                asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(smem_u32(&S.a_full[i][j])),
                             "r"(kGroupThreads)
                             : "memory");
                asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(smem_u32(&S.d_full[i][j])) : "memory");
            }
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
        // the weights and bias chunks, already in the staged layout (wt_sw), by
        // one bulk copy completing on wbar's first phase
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(smem_u32(&S.wbar)),
                     "r"(kGuideWtBytes)
                     : "memory");
        asm volatile(
            "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];\n" ::"r"(
                smem_u32(S.wt)),
            "l"(gv.wt_sw), "r"(kGuideWtBytes), "r"(smem_u32(&S.wbar))
            : "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(smem_u32(&S.tmem_base)),
                     "r"(kTcCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
    }
    fence_before();
    __syncthreads();
    fence_after();
    const uint32_t tmem = S.tmem_base;
    const uint32_t ones = tmem + kOnesCol, wt_addr = smem_u32(S.wt);
    if (warp < 4) {  // the ones chunk, one row per lane of the first four warps
        uint32_t r32[32] = {0x3f803f80u};
        tmem_st32(ones + ((32u * warp) << 16), r32);
        tmem_wait_st();
    }
    fence_before();
    __syncthreads();
    fence_after();
    const bool failed0 = __syncthreads_or(!mbar_wait(smem_u32(&S.wbar), 0u)) != 0;  // the weights have landed
    if (failed0 && t == 0) S.error = kErrTimeout;
    const uint32_t ntiles = (n + 127u) / 128u, stride = gridDim.x * kTcGroups;
    // tiles of group gg: tile k is base + k stride while below ntiles
    auto tiles_of = [&](uint32_t gg) -> uint32_t {
        const uint32_t base = blockIdx.x * kTcGroups + gg;
        return base < ntiles ? (ntiles - base + stride - 1u) / stride : 0u;
    };

    if (warp >= (uint32_t)kMmaWarp) {
        const uint32_t mw = warp - (uint32_t)kMmaWarp;
        // ---------------------------------------------------- MMA warp
        uint32_t left[kTcGroups][kBufs], lay[kTcGroups][kBufs], ph[kTcGroups][kBufs];
#pragma unroll
        for (int i = 0; i < kTcGroups; ++i) {
            const uint32_t k = (failed0 || gv.stall_mma) ? 0u : tiles_of(i);  // a stalled warp issues nothing
#pragma unroll
            for (int j = 0; j < kBufs; ++j) {
                const bool mine = (uint32_t)((i * kBufs + j) % kMmaWarps) == mw;
                left[i][j] = mine ? kGuideLayers * ((k + (uint32_t)(kBufs - 1 - j)) / kBufs) : 0u;  // layers to issue
                lay[i][j] = 0u;
                ph[i][j] = 0u;
            }
        }
        uint32_t last = global_ns();  // when the warp last issued
        uint32_t idle = 0;
        for (;;) {
            bool any = false, progressed = false;
#pragma unroll
            for (int i = 0; i < kTcGroups; ++i) {
#pragma unroll
                for (int j = 0; j < kBufs; ++j) {
                    if (left[i][j] == 0u) continue;
                    any = true;
                    const bool ready = __shfl_sync(0xffffffffu, (uint32_t)mbar_test(smem_u32(&S.a_full[i][j]), ph[i][j]), 0) != 0u;
                    if (!ready) continue;
                    ph[i][j] ^= 1u;
                    fence_after();
                    if (elect_one()) {
                        const uint32_t acc = tmem + kAccCols * (kBufs * i + j);
                        issue_layer(lay[i][j], acc, acc + 64u, ones, wt_addr, smem_u32(&S.d_full[i][j]));
                    }
                    __syncwarp();
                    lay[i][j] = lay[i][j] + 1u == (uint32_t)kGuideLayers ? 0u : lay[i][j] + 1u;
                    --left[i][j];
                    progressed = true;
                }
            }
            if (!any) break;
            idle = progressed ? 0u : idle + 1u;
            if (progressed) last = global_ns();
            if (idle >= kWaitPolls || ((idle & 63u) == 63u && global_ns() - last > kWaitNs)) {
                if (elect_one()) S.error = kErrTimeout;  // no buffer became ready within the limit
                break;
            }
        }
    } else {
        // ---------------------------------------------------- epilogue groups
        const uint32_t lane_off = (32u * (warp & 3u)) << 16;  // this warp's 32 TMEM lanes
        const uint32_t kt = failed0 ? 0u : tiles_of(g);
        const uint32_t base = blockIdx.x * kTcGroups + g;
        uint32_t pd[kBufs] = {};
        bool timed_out = false;
        // inputs of the next pair, loaded while the current pair runs its layers
        RowIn in[kBufs] = {};
#pragma unroll
        for (int j = 0; j < kBufs; ++j) {
            const uint32_t r = (base + j * stride) * 128u + lt;
            if ((uint32_t)j < kt && r < n) in[j] = load_row<kPaths>(P, rows, r, kPaths ? guide_row_slot(Q, gd, r) : 0u);
        }
        for (uint32_t k = 0; k < kt; k += kBufs) {
            const uint32_t nb = min((uint32_t)kBufs, kt - k);
#pragma unroll
            for (int j = 0; j < kBufs; ++j) {
                if ((uint32_t)j >= nb) break;
                const uint32_t r = (base + (k + j) * stride) * 128u + lt;
                float x9[9];
                row_x9<kPaths>(in[j], x9);
                if (r >= n) x9[0] = x9[1] = x9[2] = x9[3] = x9[4] = x9[5] = x9[6] = x9[7] = x9[8] = 0.0f;
                encode_store(tmem + kAccCols * (kBufs * g + j) + 64u + lane_off, x9, gv.params);
                tmem_wait_st();  // this thread's A row is in TMEM before the MMA warp learns of it
                fence_before();
                mbar_arrive(smem_u32(&S.a_full[g][j]));
            }
            uint32_t next_slot[kBufs];
#pragma unroll
            for (int j = 0; j < kBufs; ++j) {
                const uint32_t r = (base + (k + kBufs + j) * stride) * 128u + lt;
                next_slot[j] = (kPaths && k + kBufs + j < kt && r < n) ? guide_row_slot(Q, gd, r) : 0u;
            }
            for (int l = 0; l < kGuideLayers; ++l) {
#pragma unroll
                for (int j = 0; j < kBufs; ++j) {
                    if ((uint32_t)j >= nb) break;
                    const uint32_t tile = base + (k + j) * stride, r = tile * 128u + lt;
                    if (timed_out || !mbar_wait(smem_u32(&S.d_full[g][j]), pd[j])) {  // after one timeout, no more waits
                        timed_out = true;
                        S.error = kErrTimeout;
                    }
                    pd[j] ^= 1u;
                    fence_after();
                    const uint32_t tm = tmem + kAccCols * (kBufs * g + j) + lane_off;
                    if (l + 1 < kGuideLayers) {
                        relu_store(tm, tm + 64u);
                        tmem_wait_st();
                        fence_before();
                        mbar_arrive(smem_u32(&S.a_full[g][j]));
                        continue;
                    }
                    uint32_t o[kGuideRowOutputs];
                    tmem_ld32(tm, o);
                    tmem_ld8(tm + 32u, o + 32);
                    if (kPaths) {
                        tmem_ld1(tm + 40u, o + 40);  // the selection logit only
                    } else {
                        tmem_ld8(tm + 40u, o + 40);
                    }
                    tmem_wait_ld();
                    fence_before();
                    // the staging rows are free once the previous bulk copy has read them
                    if (lt == 0u) asm volatile("cp.async.bulk.wait_group.read 0;\n" ::: "memory");
                    if (group_sync_any(g, timed_out)) {
                        timed_out = true;
                        break;
                    }
                    // the row's result (the 80-byte FP16 mixture record, or the 192
                    // bytes of raw outputs), then the tile's rows to global memory
                    // in one bulk copy
                    constexpr uint32_t kRowBytes = kPaths ? 16u * kGuideMixVecs : 4u * kGuideRowOutputs;
                    unsigned char* row_out = S.out[g] + kRowBytes * lt;
                    if (r < n) {
                        if (kPaths) {
                            float of[kGuideOutputs];
#pragma unroll
                            for (int q = 0; q < kGuideOutputs; ++q) of[q] = __uint_as_float(o[q]);
                            const float alpha =
                                gd.learn_frac ? alpha_of(__uint_as_float(o[kGuideSelOutput])) : gd.guide_frac;
                            row_mixture(of, alpha, reinterpret_cast<uint4*>(row_out));
                        } else {
#pragma unroll
                            for (int q = 0; q < kGuideRowOutputs / 4; ++q)
                                reinterpret_cast<uint4*>(row_out)[q] = make_uint4(o[4 * q], o[4 * q + 1], o[4 * q + 2],
                                                                                  o[4 * q + 3]);
                        }
                    }
                    fence_async_smem();
                    asm volatile("bar.sync %0, %1;\n" ::"r"(g + 1u), "r"((uint32_t)kGroupThreads) : "memory");
                    if (lt == 0u) {
                        unsigned char* dst =
                            kPaths ? reinterpret_cast<unsigned char*>(gd.lobes) : reinterpret_cast<unsigned char*>(out);
                        asm volatile(
                            "cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;\n"
                            "cp.async.bulk.commit_group;\n" ::"l"(dst + (size_t)kRowBytes * tile * 128u),
                            "r"(smem_u32(S.out[g])), "r"(kRowBytes * min(128u, n - tile * 128u))
                            : "memory");
                    }
                }
                if (timed_out) break;
                if (l == 1) {
#pragma unroll
                    for (int j = 0; j < kBufs; ++j) {
                        const uint32_t r = (base + (k + kBufs + j) * stride) * 128u + lt;
                        if (k + kBufs + j < kt && r < n) in[j] = load_row<kPaths>(P, rows, r, next_slot[j]);
                    }
                }
            }
            if (timed_out) break;
        }
        if (lt == 0u) asm volatile("cp.async.bulk.wait_group 0;\n" ::: "memory");  // this group's stores are done
    }
    fence_before();
    __syncthreads();
    if (warp == 0) {
        fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(kTcCols) : "memory");
    }
    if (t == 0 && S.error && err) atomicOr(err, S.error);
}

}  // namespace

size_t guide_tc_smem() { return sizeof(SmemTc) + 1024; }

int guide_tc_attributes() {
    cudaError_t e = cudaFuncSetAttribute(k_guide_infer_tc<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)guide_tc_smem());
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_guide_infer_tc<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)guide_tc_smem());
    return (int)e;
}

// one CTA per SM: its staging rows take most of the shared memory, its
// accumulators most of the 512 TMEM columns
int guide_tc_grid(int num_sms) { return num_sms; }

void launch_guide_infer_tc(const GuideView& g, const float* rows, uint32_t n, float* out, int grid, uint32_t* err,
                           cudaStream_t st) {
    if (n == 0) return;
    const uint32_t need = (n + kCtaRows - 1u) / kCtaRows;
    if ((uint32_t)grid > need) grid = (int)need;
    k_guide_infer_tc<false><<<grid, kTcThreads, guide_tc_smem(), st>>>(g, rows, n, out, PathsView{}, QueueView{},
                                                                      GuideRenderD{}, err);
}

void launch_guide_infer_paths_tc(const GuideView& g, const PathsView& p, const QueueView& q, const GuideRenderD& gd,
                                 int grid, uint32_t* err, cudaStream_t st) {
    k_guide_infer_tc<true><<<grid, kTcThreads, guide_tc_smem(), st>>>(g, nullptr, 0, nullptr, p, q, gd, err);
}

}  // namespace dev
}  // namespace rgr
