// integration_example.cpp — the call sequence a C++ host of the reference
// (SceneManager + WavefrontLane, common/scene_manager.hpp and
// common/wavefront_path_tracing.hpp) runs against librgr through include/rgr.h,
// compiled as plain C++ and linked to librgr.so.
//
//   integration_example            full sequence on GPU 0: scene, BVH, upload,
//                                  render to a fixed spp, readback (RGBA8 and
//                                  FP64 sums), stats, closest-hit queries with
//                                  known answers, merge_from of two lanes,
//                                  checkpoint size; prints "integration ok"
//   integration_example --host     the host-side calls only (no GPU needed):
//                                  scene, BVH, stackless export, and a context
//                                  creation that must fail with RGR_E_NODEVICE
//                                  when no GPU is present
// Exit status 0 on success, 1 on the first failed check.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>

#include "rgr.h"

#define CHECK(cond)                                                                    \
    do {                                                                               \
        if (!(cond)) {                                                                 \
            std::fprintf(stderr, "check failed at line %d: %s (%s)\n", __LINE__, #cond, \
                         rgr_last_error() ? rgr_last_error() : "");                    \
            return 1;                                                                  \
        }                                                                              \
    } while (0)

namespace {

rgr_material lambertian(float r, float g, float b, float le_r = 0, float le_g = 0, float le_b = 0) {
    rgr_material m;
    std::memset(&m, 0, sizeof(m));
    m.type = RGR_MAT_LAMBERTIAN;
    m.r[0] = r, m.r[1] = g, m.r[2] = b;
    m.le[0] = le_r, m.le[1] = le_g, m.le[2] = le_b;
    return m;
}

// a floor quad (y = 0, x and z in [-1, 1], facing up) under a light quad
// (y = 1.2, x and z in [-0.8, 0.8], facing down): triangles 0-1 floor, 2-3 light
int build_scene(rgr_scene** out) {
    const float P[] = {-1, 0, -1, 1, 0, -1, 1, 0, 1, -1, 0, 1,
                       -0.8f, 1.2f, -0.8f, 0.8f, 1.2f, -0.8f, 0.8f, 1.2f, 0.8f, -0.8f, 1.2f, 0.8f};
    const uint32_t idx[] = {0, 1, 2, 0, 2, 3, 4, 6, 5, 4, 7, 6};
    const rgr_material mats[] = {lambertian(0.73f, 0.73f, 0.73f), lambertian(0.73f, 0.73f, 0.73f),
                                 lambertian(0, 0, 0, 17, 12, 4), lambertian(0, 0, 0, 17, 12, 4)};
    rgr_scene* s = nullptr;
    CHECK(rgr_scene_create(&s) == RGR_OK);
    CHECK(rgr_scene_add_mesh(s, P, 8, idx, 4, mats) == RGR_OK);
    rgr_bvh_params bp;
    rgr_bvh_params_default(&bp);
    bp.max_leaf_size = 1;
    CHECK(rgr_scene_build_bvh(s, &bp) == RGR_OK);
    rgr_scene_info info;
    CHECK(rgr_scene_get_info(s, &info) == RGR_OK);
    CHECK(info.num_triangles == 4 && info.num_vertices == 8);
    std::vector<rgr_stackless_node> nodes(info.num_nodes_stackless);
    std::vector<uint32_t> ids(4);
    CHECK(rgr_bvh_export_stackless(s, nodes.data(), nodes.size(), ids.data(), ids.size()) == RGR_OK);
    CHECK(info.num_nodes_stackless == 7);  // 4 leaves of one triangle under 3 inner nodes
    *out = s;
    return 0;
}

int render(rgr_context* lane, const rgr_camera& cam, uint32_t seed, std::vector<double>& sums) {
    rgr_render_config cfg;
    rgr_render_config_default(&cfg);
    cfg.spp = 4;
    cfg.max_depth = 5;
    cfg.dof = 0.0f;
    cfg.seed_offset = seed;
    CHECK(rgr_render_begin(lane, &cam, &cfg) == RGR_OK);
    int32_t steps = 0;
    CHECK(rgr_render_until_done(lane, 1000, &steps) == RGR_OK);
    sums.assign(4 * (size_t)cam.image_w * cam.image_h, 0.0);
    CHECK(rgr_render_readback(lane, RGR_FMT_FP64_SUMS, sums.data(), sums.size() * 8) == RGR_OK);
    return 0;
}

}  // namespace

int main(int argc, char** argv) {
    const bool host_only = argc > 1 && std::strcmp(argv[1], "--host") == 0;
    rgr_scene* scene = nullptr;
    if (build_scene(&scene)) return 1;
    rgr_context* lane = nullptr;
    int st = rgr_context_create(&lane, 0, 1 << 14);
    if (host_only) {
        CHECK(st == RGR_E_NODEVICE);
        rgr_scene_destroy(scene);
        std::puts("integration host ok");
        return 0;
    }
    CHECK(st == RGR_OK);
    CHECK(rgr_device_upload(lane, scene) == RGR_OK);
    const uint32_t W = 64, H = 48;
    rgr_camera cam;
    const float eye[3] = {0.0f, 1.0f, 2.6f}, target[3] = {0.0f, 0.0f, 0.0f}, up[3] = {0.0f, 1.0f, 0.0f};
    CHECK(rgr_camera_look_at(&cam, eye, target, up, 45.0f, W, H) == RGR_OK);

    std::vector<double> a, b, merged;
    if (render(lane, cam, 1, a)) return 1;
    std::vector<uint8_t> rgba(4 * (size_t)W * H);
    CHECK(rgr_render_readback(lane, RGR_FMT_RGBA8, rgba.data(), rgba.size()) == RGR_OK);
    size_t lit = 0;
    for (size_t i = 0; i < (size_t)W * H; ++i) lit += (rgba[4 * i] | rgba[4 * i + 1] | rgba[4 * i + 2]) != 0;
    CHECK(lit > (size_t)W * H / 20);  // the floor under the light shows
    rgr_stats stats;
    CHECK(rgr_render_stats(lane, &stats) == RGR_OK);
    CHECK(stats.samples_accumulated == 4ull * W * H && stats.error_flags == 0);
    double count = 0;
    for (size_t i = 0; i < (size_t)W * H; ++i) count += a[4 * i + 3];
    CHECK(count == 4.0 * W * H);
    uint64_t ckpt = 0;
    CHECK(rgr_render_checkpoint_size(lane, &ckpt) == RGR_OK && ckpt > 32ull * W * H);

    // closest hit with known answers: down onto the floor, up into the light, a miss
    const float ox[] = {0.0f, 0.0f, 5.0f}, oy[] = {1.0f, 1.0f, 1.0f}, oz[] = {0.0f, 0.0f, 0.0f};
    const float dx[] = {0.0f, 0.0f, 0.0f}, dy[] = {-1.0f, 1.0f, -1.0f}, dz[] = {0.0f, 0.0f, 0.0f};
    const float tmax[] = {1e30f, 1e30f, 1e30f};
    rgr_ray_soa rays = {ox, oy, oz, dx, dy, dz, tmax};
    int32_t prim[3];
    float t[3];
    CHECK(rgr_trace_closest(lane, &rays, 3, prim, t) == RGR_OK);
    CHECK((prim[0] == 0 || prim[0] == 1) && std::fabs(t[0] - 1.0f) < 1e-6f);
    CHECK((prim[1] == 2 || prim[1] == 3) && std::fabs(t[1] - 0.2f) < 1e-5f);
    CHECK(prim[2] == -1);

    // merge_from: a second lane renders other samples of the same view; its sums add in
    rgr_context* lane2 = nullptr;
    CHECK(rgr_context_create(&lane2, 0, 1 << 14) == RGR_OK);
    CHECK(rgr_device_upload(lane2, scene) == RGR_OK);
    if (render(lane2, cam, 1u << 20, b)) return 1;
    CHECK(rgr_accum_merge(lane, lane2) == RGR_OK);
    merged.assign(a.size(), 0.0);
    CHECK(rgr_render_readback(lane, RGR_FMT_FP64_SUMS, merged.data(), merged.size() * 8) == RGR_OK);
    for (size_t i = 0; i < a.size(); ++i) CHECK(merged[i] == a[i] + b[i]);

    rgr_context_destroy(lane2);
    rgr_context_destroy(lane);
    rgr_scene_destroy(scene);
    std::puts("integration ok");
    return 0;
}
