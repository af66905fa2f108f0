// bvh_build.cpp — deterministic binned-SAH BVH builder (host, multi-threaded).
//
// Replaces the reference's Embree build (common/stackless_bvh.hpp:63-130,
// scene_manager.hpp:517-577: binary tree, leaves of up to maxLeafSize
// primitives) and its flattening create_stackless_bvh
// (stackless_bvh.hpp:283-341).  Embree is not available; this builder makes
// its own SAH tree.  The tree is emitted twice from one DFS:
//   * the reference StacklessBVHNode layout (96 B, parent/sibling links,
//     pre-order numbering with the left subtree first), exported for parity;
//   * the device layout: 64-byte inner nodes carrying both child boxes, and
//     48-byte primitive records pre-gathered in leaf order.
// Both carry bit-identical child boxes, so a traversal of either visits the
// same leaves in the same order.  Parallel subtree builds do not change the
// result: every split decision depends only on the node's own primitives.
#include "../rgr_internal.h"

#include <algorithm>
#include <atomic>
#include <cfloat>
#include <cmath>
#include <cstring>
#include <future>
#include <thread>

namespace rgr {
namespace {

struct PrimBox {
    float lo[3], hi[3], c[3];
};

struct BNode {
    float lo[3], hi[3];
    BNode* kid[2] = {nullptr, nullptr};
    uint32_t first = 0, count = 0;  // leaf range in `order`
    ~BNode() {
        delete kid[0];
        delete kid[1];
    }
};

struct Builder {
    const PrimBox* prims;
    uint32_t* order;
    rgr_bvh_params p;
    std::atomic<int> spare_threads{0};

    static float area(const float* lo, const float* hi) {
        float dx = hi[0] - lo[0], dy = hi[1] - lo[1], dz = hi[2] - lo[2];
        if (!(dx >= 0.0f)) return 0.0f;
        return 2.0f * (dx * dy + dy * dz + dz * dx);
    }

    BNode* make_leaf(uint32_t b, uint32_t e, const float* lo, const float* hi) {
        BNode* n = new BNode();
        memcpy(n->lo, lo, 12);
        memcpy(n->hi, hi, 12);
        n->first = b;
        n->count = e - b;
        return n;
    }

    // levels needed below this node if every further split halves the range
    static int levels_needed(uint32_t count, int leaf) {
        int l = 0;
        uint64_t cap = (uint64_t)leaf;
        while (cap < count) {
            cap <<= 1;
            l++;
        }
        return l;
    }

    BNode* build(uint32_t b, uint32_t e, int depth) {
        const uint32_t n = e - b;
        float lo[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, hi[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
        float clo[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, chi[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
        for (uint32_t i = b; i < e; ++i) {
            const PrimBox& pb = prims[order[i]];
            for (int k = 0; k < 3; ++k) {
                lo[k] = std::min(lo[k], pb.lo[k]);
                hi[k] = std::max(hi[k], pb.hi[k]);
                clo[k] = std::min(clo[k], pb.c[k]);
                chi[k] = std::max(chi[k], pb.c[k]);
            }
        }
        const int leaf = p.max_leaf_size;
        if (n <= 1) return make_leaf(b, e, lo, hi);

        // choose the split
        int best_axis = -1;
        int best_bin = -1;
        double best_cost = DBL_MAX;
        const int nb = std::max(2, std::min(p.sah_bins, 256));
        const bool force_median = depth + 1 + levels_needed(n, leaf) >= p.max_depth;
        float parent_area = area(lo, hi);
        if (!force_median && parent_area > 0.0f) {
            for (int axis = 0; axis < 3; ++axis) {
                float ext = chi[axis] - clo[axis];
                if (!(ext > 0.0f)) continue;
                float scale = (float)nb / ext;
                uint32_t cnt[256];
                float blo[256][3], bhi[256][3];
                for (int k = 0; k < nb; ++k) {
                    cnt[k] = 0;
                    for (int d = 0; d < 3; ++d) {
                        blo[k][d] = FLT_MAX;
                        bhi[k][d] = -FLT_MAX;
                    }
                }
                for (uint32_t i = b; i < e; ++i) {
                    const PrimBox& pb = prims[order[i]];
                    int bi = (int)((pb.c[axis] - clo[axis]) * scale);
                    bi = std::min(std::max(bi, 0), nb - 1);
                    cnt[bi]++;
                    for (int d = 0; d < 3; ++d) {
                        blo[bi][d] = std::min(blo[bi][d], pb.lo[d]);
                        bhi[bi][d] = std::max(bhi[bi][d], pb.hi[d]);
                    }
                }
                // sweep: right-side areas, then left-to-right
                double rarea[256];
                uint32_t rcnt[256];
                float rlo[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, rhi[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
                uint32_t rc = 0;
                for (int k = nb - 1; k > 0; --k) {
                    rc += cnt[k];
                    for (int d = 0; d < 3; ++d) {
                        rlo[d] = std::min(rlo[d], blo[k][d]);
                        rhi[d] = std::max(rhi[d], bhi[k][d]);
                    }
                    rcnt[k] = rc;
                    rarea[k] = rc ? area(rlo, rhi) : 0.0;
                }
                float llo[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, lhi[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
                uint32_t lc = 0;
                for (int k = 0; k < nb - 1; ++k) {
                    lc += cnt[k];
                    for (int d = 0; d < 3; ++d) {
                        llo[d] = std::min(llo[d], blo[k][d]);
                        lhi[d] = std::max(lhi[d], bhi[k][d]);
                    }
                    if (lc == 0 || rcnt[k + 1] == 0) continue;
                    double cost = (double)p.traversal_cost +
                                  ((double)area(llo, lhi) * lc + rarea[k + 1] * rcnt[k + 1]) * p.intersect_cost /
                                      parent_area;
                    if (cost < best_cost) {
                        best_cost = cost;
                        best_axis = axis;
                        best_bin = k;
                    }
                }
            }
        }
        double leaf_cost = (double)n * p.intersect_cost;
        if ((int)n <= leaf && (best_axis < 0 || leaf_cost <= best_cost)) return make_leaf(b, e, lo, hi);

        uint32_t mid;
        if (best_axis >= 0) {
            float ext = chi[best_axis] - clo[best_axis];
            float scale = (float)nb / ext;
            const int axis = best_axis, bin = best_bin;
            uint32_t* m = std::partition(order + b, order + e, [&](uint32_t id) {
                int bi = (int)((prims[id].c[axis] - clo[axis]) * scale);
                bi = std::min(std::max(bi, 0), nb - 1);
                return bi <= bin;
            });
            mid = (uint32_t)(m - order);
        } else {
            // object median on the widest centroid axis (degenerate or depth-limited)
            int axis = 0;
            float best_ext = -1.0f;
            for (int k = 0; k < 3; ++k) {
                float ext = chi[k] - clo[k];
                if (ext > best_ext) {
                    best_ext = ext;
                    axis = k;
                }
            }
            mid = b + n / 2;
            if (best_ext > 0.0f) {
                std::nth_element(order + b, order + mid, order + e, [&](uint32_t x, uint32_t y) {
                    if (prims[x].c[axis] != prims[y].c[axis]) return prims[x].c[axis] < prims[y].c[axis];
                    return x < y;
                });
            }
        }
        if (mid == b || mid == e) mid = b + n / 2;

        BNode* node = new BNode();
        memcpy(node->lo, lo, 12);
        memcpy(node->hi, hi, 12);
        if (n > 65536 && spare_threads.fetch_sub(1) > 0) {
            auto fut = std::async(std::launch::async, [this, b, mid, depth]() { return build(b, mid, depth + 1); });
            node->kid[1] = build(mid, e, depth + 1);
            node->kid[0] = fut.get();
            spare_threads.fetch_add(1);
        } else {
            if (n > 65536) spare_threads.fetch_add(1);
            node->kid[0] = build(b, mid, depth + 1);
            node->kid[1] = build(mid, e, depth + 1);
        }
        return node;
    }
};

struct Flattener {
    const uint32_t* order;
    const PrimD* prim_records;  // indexed by primitive id
    Bvh* out;
    int max_depth_seen = 0;
    double sah = 0.0;
    double root_area = 0.0;

    static float area(const float* lo, const float* hi) { return Builder::area(lo, hi); }

    // reference pre-order numbering (allocate_stacklessBVH, stackless_bvh.hpp:283-292)
    uint32_t count_nodes(const BNode* n) {
        if (!n->kid[0]) return 1;
        return 1 + count_nodes(n->kid[0]) + count_nodes(n->kid[1]);
    }
    // build_stacklessBVH (stackless_bvh.hpp:294-327) and the device layout in one DFS.
    // Returns the device link of this node.
    uint32_t emit(const BNode* n, uint32_t parent, uint32_t* next_ref, int depth) {
        max_depth_seen = std::max(max_depth_seen, depth);
        uint32_t me = (*next_ref)++;
        rgr_stackless_node& r = out->ref_nodes[me];
        r.link_parent = parent;
        if (!n->kid[0]) {
            r.primitive_indices_beg = (uint32_t)out->ref_prim_ids.size();
            uint32_t first = (uint32_t)out->prims.size();
            for (uint32_t i = 0; i < n->count; ++i) {
                uint32_t id = order[n->first + i];
                out->ref_prim_ids.push_back(id);
                out->prims.push_back(prim_records[id]);
            }
            r.primitive_indices_end = (uint32_t)out->ref_prim_ids.size();
            out->num_leaves++;
            sah += (double)area(n->lo, n->hi) * n->count;
            return make_leaf_link(first, n->count);
        }
        sah += (double)area(n->lo, n->hi);
        uint32_t dev_index = (uint32_t)out->nodes.size();
        out->nodes.emplace_back();
        const BNode* L = n->kid[0];
        const BNode* R = n->kid[1];
        auto set_box = [](float* lo4, float* hi4, const BNode* c) {
            for (int k = 0; k < 3; ++k) {
                lo4[k] = c->lo[k];
                hi4[k] = c->hi[k];
            }
            lo4[3] = 0.0f;
            hi4[3] = 0.0f;
        };
        set_box(r.L_lower, r.L_upper, L);
        set_box(r.R_lower, r.R_upper, R);
        uint32_t lref = *next_ref;
        uint32_t llink = emit(L, me, next_ref, depth + 1);
        uint32_t rref = *next_ref;
        uint32_t rlink = emit(R, me, next_ref, depth + 1);
        // note: emit() may reallocate out->ref_nodes? no: sized up front
        rgr_stackless_node& r2 = out->ref_nodes[me];
        r2.link_L = lref;
        r2.link_R = rref;
        out->ref_nodes[lref].link_sibling = rref;
        out->ref_nodes[rref].link_sibling = lref;
        NodeD& d = out->nodes[dev_index];
        const float q[12] = {L->lo[0], L->lo[1], L->lo[2], L->hi[0], L->hi[1], L->hi[2],
                             R->lo[0], R->lo[1], R->lo[2], R->hi[0], R->hi[1], R->hi[2]};
        memcpy(d.q, q, sizeof(q));
        d.link[0] = llink;
        d.link[1] = rlink;
        d.pad[0] = d.pad[1] = 0;
        return dev_index;
    }
};

// The builder's tree from a GPU radix tree: child c >= 0 is internal node c,
// c < 0 the single sorted primitive ~c; nodes covering at most `leaf`
// primitives become leaves over their (contiguous) sorted range.
BNode* lbvh_node(const LbvhTree& t, const PrimBox* boxes, int32_t c, int leaf) {
    BNode* n = new BNode();
    if (c < 0) {
        const uint32_t k = (uint32_t)~c;
        const PrimBox& pb = boxes[t.order[k]];
        memcpy(n->lo, pb.lo, 12);
        memcpy(n->hi, pb.hi, 12);
        n->first = k;
        n->count = 1;
        return n;
    }
    memcpy(n->lo, &t.box[6 * (size_t)c], 12);
    memcpy(n->hi, &t.box[6 * (size_t)c + 3], 12);
    if (t.count[c] <= leaf) {
        n->first = (uint32_t)t.first[c];
        n->count = (uint32_t)t.count[c];
        return n;
    }
    n->kid[0] = lbvh_node(t, boxes, t.left[c], leaf);
    n->kid[1] = lbvh_node(t, boxes, t.right[c], leaf);
    return n;
}

}  // namespace

// Device-layout order for shared-memory staging: the first `k` inner nodes a
// breadth-first walk from the root meets (the levels every ray passes
// through) move to the front of the node array in that order, the others keep
// their depth-first order; links are renumbered.  The traversal kernel copies
// a prefix of the array into shared memory and reads those nodes from there.
// Results do not depend on the order: links are explicit.
void stage_top_levels(Bvh& b, size_t k) {
    const size_t n = b.nodes.size();
    if (n == 0 || (b.root_link & kLeafFlag)) return;
    k = std::min(k, n);
    std::vector<uint32_t> bfs;
    bfs.reserve(k);
    std::vector<uint8_t> taken(n, 0);
    bfs.push_back(b.root_link);
    taken[b.root_link] = 1;
    for (size_t head = 0; head < bfs.size() && bfs.size() < k; ++head) {
        const NodeD& d = b.nodes[bfs[head]];
        for (int c = 0; c < 2 && bfs.size() < k; ++c) {
            const uint32_t l = d.link[c];
            if (!(l & kLeafFlag) && !taken[l]) {
                taken[l] = 1;
                bfs.push_back(l);
            }
        }
    }
    std::vector<uint32_t> to_new(n);
    uint32_t next = 0;
    for (uint32_t old : bfs) to_new[old] = next++;
    for (uint32_t i = 0; i < n; ++i)
        if (!taken[i]) to_new[i] = next++;
    std::vector<NodeD> out(n);
    for (uint32_t i = 0; i < n; ++i) {
        NodeD d = b.nodes[i];
        for (int c = 0; c < 2; ++c)
            if (!(d.link[c] & kLeafFlag)) d.link[c] = to_new[d.link[c]];
        out[to_new[i]] = d;
    }
    b.nodes.swap(out);
    b.root_link = to_new[b.root_link];
}

int build_bvh(rgr_scene* s, const rgr_bvh_params& params) {
    rgr_bvh_params p = params;
    if (p.max_leaf_size < 1 || p.max_leaf_size > 8) {
        set_error("max_leaf_size must be in 1..8");
        return RGR_E_INVALID;
    }
    if (p.max_depth < 2 || p.max_depth > 63) p.max_depth = 63;
    if (p.sah_bins < 2) p.sah_bins = 32;
    const uint64_t ntri = s->indices.size() / 3;
    const uint64_t nsph = s->spheres.size() / 4;
    const uint64_t nprim = ntri + nsph;
    if (nprim >= (1ull << 28)) {
        set_error("too many primitives (limit 2^28)");
        return RGR_E_INVALID;
    }
    Bvh& out = s->bvh;
    out = Bvh();
    std::vector<PrimBox> boxes(nprim);
    std::vector<PrimD> records(nprim);
    const float* P = s->points.data();
    for (uint64_t t = 0; t < ntri; ++t) {
        const uint32_t* id = &s->indices[3 * t];
        const float* v[3] = {P + 3 * (size_t)id[0], P + 3 * (size_t)id[1], P + 3 * (size_t)id[2]};
        PrimBox& pb = boxes[t];
        for (int k = 0; k < 3; ++k) {
            pb.lo[k] = std::min(std::min(v[0][k], v[1][k]), v[2][k]);
            pb.hi[k] = std::max(std::max(v[0][k], v[1][k]), v[2][k]);
            pb.c[k] = 0.5f * (pb.lo[k] + pb.hi[k]);
        }
        PrimD& r = records[t];
        uint32_t pid = (uint32_t)t;
        for (int k = 0; k < 3; ++k) {
            r.a[k] = v[0][k];
            r.b[k] = v[1][k] - v[0][k];  // bit-identical to the kernel's v1 - v0
            r.c[k] = v[2][k] - v[0][k];
        }
        memcpy(&r.a[3], &pid, 4);
        r.b[3] = 0.0f;
        r.c[3] = 0.0f;
    }
    for (uint64_t i = 0; i < nsph; ++i) {
        const float* sp = &s->spheres[4 * i];
        PrimBox& pb = boxes[ntri + i];
        for (int k = 0; k < 3; ++k) {
            pb.lo[k] = sp[k] - sp[3];
            pb.hi[k] = sp[k] + sp[3];
            pb.c[k] = sp[k];
        }
        PrimD& r = records[ntri + i];
        uint32_t pid = (uint32_t)(ntri + i), flag = 1;
        r.a[0] = sp[0];
        r.a[1] = sp[1];
        r.a[2] = sp[2];
        memcpy(&r.a[3], &pid, 4);
        r.b[0] = sp[3];
        r.b[1] = 0.0f;
        r.b[2] = 0.0f;
        memcpy(&r.b[3], &flag, 4);
        r.c[0] = r.c[1] = r.c[2] = r.c[3] = 0.0f;
    }
    if (nprim == 0) {
        out.built = true;
        return RGR_OK;
    }
    std::vector<uint32_t> order(nprim);
    for (uint64_t i = 0; i < nprim; ++i) order[i] = (uint32_t)i;
    std::unique_ptr<BNode> root;
    if (p.builder == RGR_BVH_LBVH_GPU && nprim >= 2) {
        // Morton-order radix tree on the GPU; subtrees of <= max_leaf_size primitives become leaves
        std::vector<float> b6(6 * nprim);
        float clo[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, chi[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
        for (uint64_t i = 0; i < nprim; ++i) {
            for (int k = 0; k < 3; ++k) {
                b6[6 * i + k] = boxes[i].lo[k];
                b6[6 * i + 3 + k] = boxes[i].hi[k];
                clo[k] = std::min(clo[k], boxes[i].c[k]);
                chi[k] = std::max(chi[k], boxes[i].c[k]);
            }
        }
        LbvhTree t;
        int r = lbvh_build_gpu(p.device, b6.data(), (uint32_t)nprim, clo, chi, t);
        if (r != RGR_OK) return r;
        order = t.order;
        root.reset(lbvh_node(t, boxes.data(), 0, p.max_leaf_size));
    } else {
        Builder b;
        b.prims = boxes.data();
        b.order = order.data();
        b.p = p;
        int nth = p.num_threads > 0 ? p.num_threads : (int)std::max(1u, std::thread::hardware_concurrency());
        b.spare_threads = nth - 1;
        root.reset(b.build(0, (uint32_t)nprim, 0));
    }

    Flattener f;
    f.order = order.data();
    f.prim_records = records.data();
    f.out = &out;
    uint32_t total = f.count_nodes(root.get());
    out.ref_nodes.assign(total, rgr_stackless_node());
    memset(out.ref_nodes.data(), 0, sizeof(rgr_stackless_node) * total);
    out.ref_prim_ids.reserve(nprim);
    out.prims.reserve(nprim);
    out.nodes.reserve(total / 2 + 1);
    uint32_t next_ref = 0;
    uint32_t root_link = f.emit(root.get(), 0, &next_ref, 0);
    out.root_link = root_link;  // 0 for an inner root, a leaf link otherwise
    stage_top_levels(out, kStagedNodes);
    out.depth = f.max_depth_seen;
    float ra = Builder::area(root->lo, root->hi);
    out.sah_cost = ra > 0.0f ? f.sah / ra : 0.0;
    for (int k = 0; k < 3; ++k) {
        out.bounds[k] = root->lo[k];
        out.bounds[3 + k] = root->hi[k];
    }
    out.built = true;
    if (out.depth > 63) {
        set_error("BVH deeper than 63 levels");
        return RGR_E_INVALID;
    }
    return RGR_OK;
}

}  // namespace rgr
