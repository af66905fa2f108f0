// guide_tc.cu — inference of the path-guiding network on the 5th-generation
// tensor cores: tcgen05.mma with operands in shared memory and the
// accumulator in tensor memory (TMEM).
//
// A CTA of 128 threads (4 warps) works on tiles of 128 rows; thread t owns
// row t of the tile from the input encoding to the mixture:
//  * the encoded inputs (36 features, zero padded to 64) and, later, each
//    hidden layer's output are written by their row's thread as bf16 into the
//    A tile (128 x 64, K-major, 128-byte swizzle: the 16-byte chunk c of row r
//    sits at chunk c ^ (r % 8) of its 128-byte line, 8-line groups 1024 B apart);
//  * one thread issues the layer's four tcgen05.mma (M 128, N 64, K 16 each,
//    BF16 x BF16 -> FP32) against the layer's weights, staged once per CTA as
//    W^T (64 x 64, same layout), and commits them to an mbarrier;
//  * every thread waits on the mbarrier (a bounded wait: on timeout the CTA
//    records an error and stops), reads its row's 64 accumulators from TMEM
//    with tcgen05.ld (lane = row), adds the bias and applies ReLU, and writes
//    the next A tile; after the last layer it has all 40 outputs of its row in
//    registers and computes the mixture without any exchange.
// TMEM: 64 columns per CTA (the 128 x 64 FP32 accumulator), allocated by warp 0
// at the start and freed at the end, also after a timeout.
#include <cuda_bf16.h>

#include "guide.cuh"

namespace rgr {
namespace dev {
namespace {

constexpr int kTcThreads = 128;   // rows per tile, one per thread
constexpr int kTcCols = 64;       // TMEM columns (FP32 accumulator width)
constexpr uint32_t kWaitLimit = 1u << 26;  // mbarrier polls before giving up
constexpr uint32_t kErrTimeout = 1u;

struct __align__(1024) SmemTc {
    unsigned char wt[kGuideLayers][64 * 128];  // W^T per layer, 64 rows (outputs) x 128 B (64 bf16 inputs)
    unsigned char a[kTcThreads * 128];         // A tile, 128 rows x 128 B
    float bias[kGuideLayers][64];
    unsigned long long mbar;
    uint32_t tmem_base;
    uint32_t error;
};

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ uint32_t sw128(uint32_t r, uint32_t c) { return sw128_offset(r, c); }

// shared-memory matrix descriptor of a K-major, 128-byte-swizzled operand:
// start address >> 4 (bits 0-13), leading byte offset 1 (unused with this
// swizzle, bits 16-29), stride byte offset 1024 >> 4 between 8-row groups
// (bits 32-45), descriptor version 1 (bits 46-47), swizzle mode 2 = 128 B
// (bits 61-63)
__device__ __forceinline__ uint64_t desc_sw128(uint32_t saddr) {
    return (uint64_t)((saddr & 0x3ffffu) >> 4) | ((uint64_t)1 << 16) | ((uint64_t)(1024 >> 4) << 32) |
           ((uint64_t)1 << 46) | ((uint64_t)2 << 61);
}

// instruction descriptor of kind::f16: D FP32 (bits 4-5 = 1), A and B BF16
// (bits 7-9 and 10-12 = 1), both K-major (bits 15, 16 = 0), N >> 3 in bits
// 17-22, M >> 4 in bits 24-28
constexpr uint32_t kIdesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(64 >> 3) << 17) |
                            ((uint32_t)(128 >> 4) << 24);

__device__ __forceinline__ void mma_bf16(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n"
        :
        : "r"(tmem_d), "l"(adesc), "l"(bdesc), "r"(kIdesc), "r"(accumulate));
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
// bounded wait for the phase with the given parity; false after kWaitLimit polls
__device__ __forceinline__ bool mbar_wait(uint32_t mbar, uint32_t parity) {
    for (uint32_t i = 0; i < kWaitLimit; ++i)
        if (mbar_try_wait(mbar, parity)) return true;
    return false;
}
__device__ __forceinline__ void fence_before() { asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory"); }
__device__ __forceinline__ void fence_after() { asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory"); }
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory"); }

// 64 FP32 accumulators of this thread's TMEM lane (32x32b shape, 64 columns)
__device__ __forceinline__ void tmem_ld64(uint32_t taddr, float* v) {
    uint32_t r[64];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x64.b32 "
        "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
        "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31,"
        "%32,%33,%34,%35,%36,%37,%38,%39,%40,%41,%42,%43,%44,%45,%46,%47,"
        "%48,%49,%50,%51,%52,%53,%54,%55,%56,%57,%58,%59,%60,%61,%62,%63}, [%64];\n"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
          "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
          "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31]),
          "=r"(r[32]), "=r"(r[33]), "=r"(r[34]), "=r"(r[35]), "=r"(r[36]), "=r"(r[37]), "=r"(r[38]), "=r"(r[39]),
          "=r"(r[40]), "=r"(r[41]), "=r"(r[42]), "=r"(r[43]), "=r"(r[44]), "=r"(r[45]), "=r"(r[46]), "=r"(r[47]),
          "=r"(r[48]), "=r"(r[49]), "=r"(r[50]), "=r"(r[51]), "=r"(r[52]), "=r"(r[53]), "=r"(r[54]), "=r"(r[55]),
          "=r"(r[56]), "=r"(r[57]), "=r"(r[58]), "=r"(r[59]), "=r"(r[60]), "=r"(r[61]), "=r"(r[62]), "=r"(r[63])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
#pragma unroll
    for (int i = 0; i < 64; ++i) v[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ uint32_t pack2(float lo, float hi) {
    __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<uint32_t*>(&v);
}

// row r of the A tile from 64 values (bf16, swizzled)
__device__ __forceinline__ void store_row(unsigned char* a, uint32_t r, const float* x) {
#pragma unroll
    for (int c = 0; c < 8; ++c) {
        uint4 q;
        q.x = pack2(x[8 * c + 0], x[8 * c + 1]);
        q.y = pack2(x[8 * c + 2], x[8 * c + 3]);
        q.z = pack2(x[8 * c + 4], x[8 * c + 5]);
        q.w = pack2(x[8 * c + 6], x[8 * c + 7]);
        *reinterpret_cast<uint4*>(a + sw128(r, c)) = q;
    }
}

// encoding (see guide_mlp.cu): pair p = coordinate p / 2 at octave p % 2 -> (sin, cos)
__device__ __forceinline__ void encode_row(const float* x9, const GuideParams& gp, float* f64) {
    float v[9];
    for (int c = 0; c < 3; ++c) {
        v[c] = (x9[c] - gp.lo[c]) * gp.inv_ext[c];
        v[3 + c] = 0.5f * (x9[3 + c] + 1.0f);
        v[6 + c] = 0.5f * (x9[6 + c] + 1.0f);
    }
#pragma unroll
    for (int i = 0; i < 9; ++i) {
#pragma unroll
        for (int k = 0; k < 2; ++k) {
            float s, c;
            sincospif(v[i] * (k ? 2.0f : 1.0f), &s, &c);
            f64[4 * i + 2 * k] = s;
            f64[4 * i + 2 * k + 1] = c;
        }
    }
#pragma unroll
    for (int i = kGuideInputs; i < 64; ++i) f64[i] = 0.0f;
}

__device__ __forceinline__ float softplus_(float x) { return x > 20.0f ? x : log1pf(expf(x)); }

// the mixture of one row's 40 raw outputs (field-major), as guide_mlp.cu
__device__ __forceinline__ void row_mixture(const float* o, float4* dst) {
    float w[kGuideLobes], mx = -3.0e38f;
#pragma unroll
    for (int i = 0; i < kGuideLobes; ++i) {
        w[i] = kGuideLogitBound * tanhf(o[32 + i] * (1.0f / kGuideLogitBound));
        mx = fmaxf(mx, w[i]);
    }
    float den = 0.0f;
#pragma unroll
    for (int i = 0; i < kGuideLobes; ++i) {
        const float x = o[i], y = o[8 + i], z = o[16 + i];
        const float n = fmaxf(sqrtf(x * x + y * y + z * z), 1.0e-12f);
        dst[i] = make_float4(x / n, y / n, z / n, fminf(softplus_(o[24 + i]) + 0.01f, kGuideKappaMax));
        w[i] = expf(w[i] - mx);
        den += w[i];
    }
    dst[8] = make_float4(w[0] / den, w[1] / den, w[2] / den, w[3] / den);
    dst[9] = make_float4(w[4] / den, w[5] / den, w[6] / den, w[7] / den);
}

__device__ __forceinline__ void vertex_of_tc(const PathsView& P, uint32_t slot, float* x9) {
    const float4 ro = P.ro[slot], rd = P.rd[slot], ng = P.ng[slot];
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

// kPaths: rows are this bounce's guided queue items, output their mixtures;
// otherwise rows of 16 floats in `rows`, output 40 raw floats per row.
template <bool kPaths>
__global__ void __launch_bounds__(kTcThreads) k_guide_infer_tc(GuideView gv, const float* __restrict__ rows,
                                                               uint32_t nrows, float* __restrict__ out, PathsView P,
                                                               QueueView Q, GuideRenderD gd, uint32_t* err) {
    extern __shared__ unsigned char smem_raw[];
    SmemTc& S = *reinterpret_cast<SmemTc*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    const uint32_t n = kPaths ? guide_rows(Q, gd) : nrows;
    if (blockIdx.x * kTcThreads >= n) return;
    const uint32_t t = threadIdx.x, warp = t >> 5;
    // the weights, already in the staged layout (wt_sw), by one bulk copy
    // completing on the mbarrier's first phase; biases by the threads
    for (uint32_t i = t; i < kGuideLayers * 64; i += kTcThreads) S.bias[i / 64][i % 64] = gv.b[i];
    const uint32_t mbar = smem_u32(&S.mbar);
    if (t == 0) {
        S.error = 0u;
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(mbar) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(mbar), "r"(kGuideWtBytes)
                     : "memory");
        asm volatile(
            "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];\n" ::"r"(
                smem_u32(S.wt[0])),
            "l"(gv.wt_sw), "r"(kGuideWtBytes), "r"(mbar)
            : "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(smem_u32(&S.tmem_base)),
                     "r"(kTcCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
    }
    fence_async_smem();
    fence_before();
    __syncthreads();
    fence_after();
    const uint32_t tmem = S.tmem_base;
    const uint32_t my_lane_addr = tmem + ((warp * 32u) << 16);  // this warp's 32 TMEM lanes
    const uint32_t a_base = smem_u32(S.a);
    uint32_t phase = 0;
    bool failed = false;
    if (!mbar_wait(mbar, phase & 1u)) S.error = kErrTimeout;  // the weights have landed
    ++phase;
    __syncthreads();
    if (S.error) failed = true;
    for (uint32_t base = blockIdx.x * kTcThreads; base < n && !failed; base += gridDim.x * kTcThreads) {
        const uint32_t r = base + t;
        {
            float x9[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
            if (r < n) {
                if (kPaths) {
                    vertex_of_tc(P, guide_row_slot(Q, gd, r), x9);
                } else {
#pragma unroll
                    for (int c = 0; c < 9; ++c) x9[c] = rows[16 * (size_t)r + c];
                }
            }
            float f[64];
            encode_row(x9, gv.params, f);
            store_row(S.a, t, f);
        }
        float acc[64];
        for (int l = 0; l < kGuideLayers; ++l) {
            fence_async_smem();  // this thread's A row is visible to the tensor core
            fence_before();
            __syncthreads();
            if (t == 0) {
                fence_after();
                const uint32_t b_base = smem_u32(S.wt[l]);
#pragma unroll
                for (int k = 0; k < 4; ++k)  // K 64 = 4 x 16 bf16 = 4 x 32 B inside the swizzled line
                    mma_bf16(tmem, desc_sw128(a_base + 32u * k), desc_sw128(b_base + 32u * k), k > 0 ? 1u : 0u);
                mma_commit(mbar);
            }
            if (!mbar_wait(mbar, phase & 1u)) {
                S.error = kErrTimeout;
                failed = true;
            }
            ++phase;
            __syncthreads();
            if (S.error) {
                failed = true;
                break;
            }
            fence_after();
            tmem_ld64(my_lane_addr, acc);
            if (l + 1 < kGuideLayers) {
#pragma unroll
                for (int j = 0; j < 64; ++j) acc[j] = fmaxf(acc[j] + S.bias[l][j], 0.0f);
                store_row(S.a, t, acc);
            } else {
#pragma unroll
                for (int j = 0; j < kGuideOutputs; ++j) acc[j] += S.bias[l][j];
            }
        }
        if (failed) break;
        if (r < n) {
            if (kPaths) {
                row_mixture(acc, gd.lobes + (size_t)kGuideLobeVecs * r);
            } else {
                float4* o4 = reinterpret_cast<float4*>(out + (size_t)kGuideOutputs * r);
#pragma unroll
                for (int j = 0; j < kGuideOutputs / 4; ++j)
                    o4[j] = make_float4(acc[4 * j], acc[4 * j + 1], acc[4 * j + 2], acc[4 * j + 3]);
            }
        }
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

int guide_tc_grid(int num_sms) {
    int nb = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_guide_infer_tc<true>, kTcThreads, guide_tc_smem());
    return num_sms * (nb > 0 ? nb : 1);
}

void launch_guide_infer_tc(const GuideView& g, const float* rows, uint32_t n, float* out, int grid, uint32_t* err,
                           cudaStream_t st) {
    if (n == 0) return;
    k_guide_infer_tc<false><<<grid, kTcThreads, guide_tc_smem(), st>>>(g, rows, n, out, PathsView{}, QueueView{},
                                                                      GuideRenderD{}, err);
}

void launch_guide_infer_paths_tc(const GuideView& g, const PathsView& p, const QueueView& q, const GuideRenderD& gd,
                                 int grid, uint32_t* err, cudaStream_t st) {
    k_guide_infer_tc<true><<<grid, kTcThreads, guide_tc_smem(), st>>>(g, nullptr, 0, nullptr, p, q, gd, err);
}

}  // namespace dev
}  // namespace rgr
