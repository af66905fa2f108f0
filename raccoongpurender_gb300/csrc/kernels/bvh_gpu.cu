// bvh_gpu.cu — linear BVH construction on the GPU (Karras, "Maximizing
// parallelism in the construction of BVHs, octrees, and k-d trees", HPG
// 2012): 30-bit Morton codes of the primitive centroids in the scene's
// centroid box, a radix sort of (code, primitive) pairs, one thread per
// internal node finding its key range and split from the common prefix of
// neighbouring codes (ties broken by index), and a bottom-up pass that
// unions child boxes (the second child to arrive at a node computes it).
// The host turns the radix tree into the renderer's layout, collapsing
// subtrees of at most max_leaf_size primitives into leaves (their primitives
// are contiguous in the sorted order).
#include <cuda_runtime.h>
#include <cub/device/device_radix_sort.cuh>

#include <string>
#include <vector>

#include "../rgr_internal.h"

namespace rgr {
namespace {

__device__ __forceinline__ uint32_t expand_bits(uint32_t v) {  // 10 bits -> every third bit
    v = (v * 0x00010001u) & 0xFF0000FFu;
    v = (v * 0x00000101u) & 0x0F00F00Fu;
    v = (v * 0x00000011u) & 0xC30C30C3u;
    v = (v * 0x00000005u) & 0x49249249u;
    return v;
}

__global__ void k_morton(const float* __restrict__ boxes, uint32_t n, float3 lo, float3 inv_ext,
                         uint32_t* __restrict__ codes, uint32_t* __restrict__ ids) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float* b = boxes + 6 * (size_t)i;
    const float c[3] = {0.5f * (b[0] + b[3]), 0.5f * (b[1] + b[4]), 0.5f * (b[2] + b[5])};
    const float lo3[3] = {lo.x, lo.y, lo.z}, ie[3] = {inv_ext.x, inv_ext.y, inv_ext.z};
    uint32_t q[3];
    for (int k = 0; k < 3; ++k) {
        float u = (c[k] - lo3[k]) * ie[k];
        u = fminf(fmaxf(u, 0.0f), 1.0f);
        q[k] = min((uint32_t)(u * 1024.0f), 1023u);
    }
    codes[i] = (expand_bits(q[0]) << 2) | (expand_bits(q[1]) << 1) | expand_bits(q[2]);
    ids[i] = i;
}

// length of the common prefix of keys i and j (index bits appended on ties); -1 outside
__device__ __forceinline__ int delta(const uint32_t* codes, int n, int i, int j) {
    if (j < 0 || j >= n) return -1;
    const uint32_t a = codes[i], b = codes[j];
    if (a == b) return 32 + __clz((uint32_t)i ^ (uint32_t)j);
    return __clz(a ^ b);
}

// children of internal node i: >= 0 internal node, < 0 leaf ~k (sorted primitive k)
__global__ void k_radix_tree(const uint32_t* __restrict__ codes, int n, int* __restrict__ left,
                             int* __restrict__ right, int* __restrict__ parent_inner, int* __restrict__ parent_leaf,
                             int* __restrict__ first, int* __restrict__ count) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n - 1) return;
    const int d = (delta(codes, n, i, i + 1) - delta(codes, n, i, i - 1)) >= 0 ? 1 : -1;
    const int dmin = delta(codes, n, i, i - d);
    int lmax = 2;
    while (delta(codes, n, i, i + lmax * d) > dmin) lmax *= 2;
    int l = 0;
    for (int t = lmax / 2; t >= 1; t /= 2)
        if (delta(codes, n, i, i + (l + t) * d) > dmin) l += t;
    const int j = i + l * d;
    const int dnode = delta(codes, n, i, j);
    int s = 0;
    for (int t = (l + 1) / 2;; t = (t + 1) / 2) {
        if (delta(codes, n, i, i + (s + t) * d) > dnode) s += t;
        if (t == 1) break;
    }
    const int gamma = i + s * d + min(d, 0);
    const int lo = min(i, j), hi = max(i, j);
    const int L = (lo == gamma) ? ~gamma : gamma;
    const int R = (hi == gamma + 1) ? ~(gamma + 1) : gamma + 1;
    left[i] = L;
    right[i] = R;
    first[i] = lo;
    count[i] = hi - lo + 1;
    if (L < 0) parent_leaf[~L] = i; else parent_inner[L] = i;
    if (R < 0) parent_leaf[~R] = i; else parent_inner[R] = i;
}

// bottom-up boxes of the internal nodes: each leaf climbs; the second child to
// reach a node computes its box and goes on
__global__ void k_refit(const float* __restrict__ boxes, const uint32_t* __restrict__ ids, int n,
                        const int* __restrict__ left, const int* __restrict__ right,
                        const int* __restrict__ parent_inner, const int* __restrict__ parent_leaf,
                        float* __restrict__ node_box, int* __restrict__ visits) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    int node = parent_leaf[k];
    while (node >= 0) {
        __threadfence();
        if (atomicAdd(visits + node, 1) == 0) return;  // the sibling is not done yet
        __threadfence();
        float lo[3] = {3.0e38f, 3.0e38f, 3.0e38f}, hi[3] = {-3.0e38f, -3.0e38f, -3.0e38f};
        const int kids[2] = {left[node], right[node]};
        for (int c = 0; c < 2; ++c) {
            const float* b = kids[c] < 0 ? boxes + 6 * (size_t)ids[~kids[c]] : node_box + 6 * (size_t)kids[c];
            for (int a = 0; a < 3; ++a) {
                lo[a] = fminf(lo[a], __ldcg(b + a));
                hi[a] = fmaxf(hi[a], __ldcg(b + 3 + a));
            }
        }
        float* o = node_box + 6 * (size_t)node;
        for (int a = 0; a < 3; ++a) {
            __stcg(o + a, lo[a]);
            __stcg(o + 3 + a, hi[a]);
        }
        node = parent_inner[node];
    }
}

struct Dev {
    void* p = nullptr;
    ~Dev() {
        if (p) cudaFree(p);
    }
    template <class T>
    T* as() {
        return reinterpret_cast<T*>(p);
    }
};

bool ok(cudaError_t e, const char* what) {
    if (e == cudaSuccess) return true;
    set_error(std::string("BVH build on the GPU: ") + what + ": " + cudaGetErrorString(e));
    return false;
}

}  // namespace

int lbvh_build_gpu(int device, const float* boxes, uint32_t n, const float centroid_lo[3],
                   const float centroid_hi[3], LbvhTree& out) {
    if (n < 2) return RGR_E_INVALID;
    if (!ok(cudaSetDevice(device), "cudaSetDevice")) return RGR_E_CUDA;
    cudaStream_t st = nullptr;
    if (!ok(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking), "cudaStreamCreate")) return RGR_E_CUDA;
    struct StreamGuard {
        cudaStream_t s;
        ~StreamGuard() { cudaStreamDestroy(s); }
    } guard{st};
    const size_t ni = n - 1;
    Dev d_boxes, d_codes, d_codes2, d_ids, d_ids2, d_left, d_right, d_pi, d_pl, d_first, d_count, d_nbox, d_visits,
        d_tmp;
    auto al = [](Dev& b, size_t bytes) { return ok(cudaMalloc(&b.p, bytes > 0 ? bytes : 4), "cudaMalloc"); };
    if (!al(d_boxes, 24 * (size_t)n) || !al(d_codes, 4 * (size_t)n) || !al(d_codes2, 4 * (size_t)n) ||
        !al(d_ids, 4 * (size_t)n) || !al(d_ids2, 4 * (size_t)n) || !al(d_left, 4 * ni) || !al(d_right, 4 * ni) ||
        !al(d_pi, 4 * ni) || !al(d_pl, 4 * (size_t)n) || !al(d_first, 4 * ni) || !al(d_count, 4 * ni) ||
        !al(d_nbox, 24 * ni) || !al(d_visits, 4 * ni))
        return RGR_E_OOM;
    if (!ok(cudaMemcpyAsync(d_boxes.p, boxes, 24 * (size_t)n, cudaMemcpyHostToDevice, st), "cudaMemcpyAsync"))
        return RGR_E_CUDA;
    float3 lo = make_float3(centroid_lo[0], centroid_lo[1], centroid_lo[2]);
    float3 ie;
    float* iep = &ie.x;
    for (int k = 0; k < 3; ++k) {
        const float e = centroid_hi[k] - centroid_lo[k];
        iep[k] = e > 0.0f ? 1.0f / e : 0.0f;
    }
    const unsigned nb = (n + 255) / 256;
    k_morton<<<nb, 256, 0, st>>>(d_boxes.as<float>(), n, lo, ie, d_codes.as<uint32_t>(), d_ids.as<uint32_t>());
    size_t tmp_bytes = 0;
    cub::DeviceRadixSort::SortPairs(nullptr, tmp_bytes, d_codes.as<uint32_t>(), d_codes2.as<uint32_t>(),
                                    d_ids.as<uint32_t>(), d_ids2.as<uint32_t>(), (int)n, 0, 30, st);
    if (!al(d_tmp, tmp_bytes)) return RGR_E_OOM;
    cub::DeviceRadixSort::SortPairs(d_tmp.p, tmp_bytes, d_codes.as<uint32_t>(), d_codes2.as<uint32_t>(),
                                    d_ids.as<uint32_t>(), d_ids2.as<uint32_t>(), (int)n, 0, 30, st);
    if (!ok(cudaMemsetAsync(d_pi.p, 0xff, 4 * ni, st), "cudaMemsetAsync") ||
        !ok(cudaMemsetAsync(d_visits.p, 0, 4 * ni, st), "cudaMemsetAsync"))
        return RGR_E_CUDA;
    k_radix_tree<<<(unsigned)((ni + 255) / 256), 256, 0, st>>>(d_codes2.as<uint32_t>(), (int)n, d_left.as<int>(),
                                                               d_right.as<int>(), d_pi.as<int>(), d_pl.as<int>(),
                                                               d_first.as<int>(), d_count.as<int>());
    k_refit<<<nb, 256, 0, st>>>(d_boxes.as<float>(), d_ids2.as<uint32_t>(), (int)n, d_left.as<int>(),
                                d_right.as<int>(), d_pi.as<int>(), d_pl.as<int>(), d_nbox.as<float>(),
                                d_visits.as<int>());
    if (!ok(cudaGetLastError(), "launch")) return RGR_E_CUDA;
    out.order.resize(n);
    out.left.resize(ni);
    out.right.resize(ni);
    out.first.resize(ni);
    out.count.resize(ni);
    out.box.resize(6 * ni);
    if (!ok(cudaMemcpyAsync(out.order.data(), d_ids2.p, 4 * (size_t)n, cudaMemcpyDeviceToHost, st), "copy") ||
        !ok(cudaMemcpyAsync(out.left.data(), d_left.p, 4 * ni, cudaMemcpyDeviceToHost, st), "copy") ||
        !ok(cudaMemcpyAsync(out.right.data(), d_right.p, 4 * ni, cudaMemcpyDeviceToHost, st), "copy") ||
        !ok(cudaMemcpyAsync(out.first.data(), d_first.p, 4 * ni, cudaMemcpyDeviceToHost, st), "copy") ||
        !ok(cudaMemcpyAsync(out.count.data(), d_count.p, 4 * ni, cudaMemcpyDeviceToHost, st), "copy") ||
        !ok(cudaMemcpyAsync(out.box.data(), d_nbox.p, 24 * ni, cudaMemcpyDeviceToHost, st), "copy") ||
        !ok(cudaStreamSynchronize(st), "cudaStreamSynchronize"))
        return RGR_E_CUDA;
    return RGR_OK;
}

}  // namespace rgr
