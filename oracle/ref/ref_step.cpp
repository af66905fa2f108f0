// ref_step.cpp — drives the reference wavefront step() sequence
// (common/wavefront_path_tracing.hpp:532-570 initialize, :591-939 step) over
// the reference kernels compiled from kernels/*.cl through the OpenCL shim.
// Test infrastructure only.
//
// Five stage kernels cannot be called as compiled because helpers they use
// build vectors with multi-component OpenCL literals: the BSDF-sampling
// branches of sample_or_eval_{lambertian,ward,homogeneous_volume_inside}_stage
// and the fragment-to-direction step of sample_envmap_{6axis_,}stage.  For
// those, this runner calls the reference's own pieces where they compile
// (sample_envmap_6axis, alias_method, pdf_ward, the eval branches) and the
// oracle's restatement for the five helpers (cosine_weighted_hemisphere_z_up,
// get_orthonormal_basis, sample_ward, uniform_on_unit_sphere,
// sample_from_fragment).  Everything else is the reference's code.
// Work-group size is 1, so every atomic queue fills in work-item order.
#include <stdint.h>
#include <string.h>
#include <math.h>
#include <vector>
#include "../rgr_oracle.h"

extern "C" {
void ref_random_initialize(uint32_t*, uint64_t, uint32_t);
void ref_random_uniform(uint32_t*, float*, int32_t);
void ref_initialize_all_as_new_path(uint32_t*, uint32_t*, uint64_t);
void ref_new_path(const uint32_t*, const uint32_t*, void*, void*, void*, void*, uint32_t*, const uint64_t*,
                  const orc_camera*, uint64_t);
void ref_finalize_new_path(uint64_t*, uint32_t*);
void ref_strategy_selection(uint32_t*, const void*, const void*, uint32_t*, uint32_t*, uint32_t*, uint32_t*,
                            uint32_t*, uint32_t*, uint32_t*, uint32_t*, void*, uint64_t);
uint32_t ref_alias_method(uint32_t*, const void*, uint32_t);
void ref_sample_envmap_6axis(float*, uint32_t*, uint32_t*, const float*, const float*, const void*, uint32_t);
void ref_evaluate_envmap_6axis_pdf_stage(const void*, const uint32_t*, const uint32_t*, void*, const float*, uint32_t,
                                         uint32_t, uint64_t);
void ref_evaluate_envmap_pdf_stage(const uint32_t*, const uint32_t*, void*, const float*, uint32_t, uint32_t, uint64_t);
void ref_sample_or_eval_lambertian_stage(const void*, uint32_t*, const uint32_t*, const uint32_t*, void*, uint64_t);
void ref_lambertian_stage(void*, const void*, void*, const uint32_t*, const uint32_t*, const void*, const void*, void*,
                          uint64_t);
float ref_pdf_ward(const float*, const float*, const float*, float);
void ref_sample_or_eval_ward_stage(void*, const void*, const void*, const void*, uint32_t*, const uint32_t*,
                                   const uint32_t*, void*, uint64_t);
void ref_ward_stage(void*, const void*, void*, const uint32_t*, const uint32_t*, const void*, const void*, void*,
                    uint64_t);
void ref_delta_materials(void*, uint32_t*, const void*, void*, uint32_t*, uint32_t*, uint32_t*, uint32_t*,
                         const void*, uint64_t);
void ref_homogeneous_volume_stage(void*, void*, const void*, void*, uint32_t*, uint32_t*, const void*, const void*,
                                  uint64_t);
void ref_sample_or_eval_homogeneous_volume_inside_stage(uint32_t*, const uint32_t*, const uint32_t*, void*, uint64_t);
void ref_homogeneous_volume_inside_stage(void*, const void*, void*, uint32_t*, uint32_t*, uint32_t*, const void*,
                                         const void*, void*, uint64_t);
void ref_homogeneous_volume_through(void*, void*, void*, uint32_t*, const void*, const void*, uint64_t);
void ref_extension_ray_cast(void*, void*, const void*, const uint32_t*, const uint32_t*, const float*, int32_t,
                            const float*, uint64_t);
void ref_logic(void*, uint32_t*, void*, void*, const float*, void*, const void*, uint32_t**, uint32_t**, uint64_t);
}

namespace {
struct alignas(16) F3 {
    float x, y, z, w;
};
struct WP {
    F3 T, L, ro, rd;
    uint32_t logic_i, pixel_index;
};
struct VL {
    int32_t volumes[7];
    int32_t count;
};
struct ER {
    int32_t hs, hv;
    float tmin;
    F3 Ng;
};
struct SR {
    F3 Le, T;
};
struct IS {
    F3 wi;
    float sel[2];
    float pdf[2];
    uint32_t strategy;
};
struct AB {
    float height;
    int32_t alias;
};
static_assert(sizeof(WP) == 80, "WavefrontPath");
static_assert(sizeof(ER) == 32, "ExtensionResult");
static_assert(sizeof(IS) == 48, "IncidentSample");
struct Queue {
    std::vector<uint32_t> item;
    uint32_t count = 0;
};
inline float dot3(const F3& a, const F3& b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline float fmaxr(float a, float b) { return (a < b) ? b : a; }
}  // namespace

// Returns next_pixel_index.  accum_rgb32: 4 floats per pixel (r, g, b, count as uint bits).
extern "C" uint64_t ref_render(const orc_scene* s, const orc_camera* cam, uint32_t seed_offset, uint32_t npaths,
                               int32_t steps, const float* env_const_rgba, float* accum_rgb32, orc_slot* slots_out) {
    const uint64_t N = npaths;
    const uint32_t npix = cam->image_w * cam->image_h;
    const uint32_t W = (uint32_t)s->env_w, H = (uint32_t)s->env_h, count = W * H;
    std::vector<WP> paths(N);
    std::vector<VL> vl(N);
    std::vector<ER> ext(N);
    std::vector<SR> shade(N);
    std::vector<IS> inc(N);
    std::vector<uint32_t> rng(4 * N);
    memset(paths.data(), 0, N * sizeof(WP));
    memset(vl.data(), 0, N * sizeof(VL));
    memset(ext.data(), 0, N * sizeof(ER));
    for (uint64_t i = 0; i < N; ++i) {
        ext[i].hs = -1;
        ext[i].hv = -1;  // defined initial value (the reference leaves it unset)
    }
    memset(shade.data(), 0, N * sizeof(SR));
    memset(inc.data(), 0, N * sizeof(IS));
    Queue q[11];  // 0 new, 1 lambert, 2 spec, 3 diel, 4 ward, 5 vol surf, 6 vol inside, 7..10 env
    for (auto& x : q) x.item.assign(N, 0);
    std::vector<AB> buckets(7 * (size_t)count);
    for (size_t i = 0; i < buckets.size(); ++i) {
        buckets[i].height = s->env_height[i];
        buckets[i].alias = s->env_alias[i];
    }
    const float* pdf6 = s->env_pdf + count;
    const AB* b6 = buckets.data() + count;
    uint64_t next_pixel = 0;
    memset(accum_rgb32, 0, sizeof(float) * 4 * (size_t)npix);
    // initialize (wavefront_path_tracing.hpp:532-570)
    ref_random_initialize(rng.data(), N, seed_offset);
    ref_initialize_all_as_new_path(q[0].item.data(), &q[0].count, N);
    for (int k = 1; k < 11; ++k) q[k].count = 0;

    for (int st = 0; st < steps; ++st) {
        ref_new_path(q[0].item.data(), &q[0].count, paths.data(), vl.data(), shade.data(), ext.data(), rng.data(),
                     &next_pixel, cam, N);
        ref_finalize_new_path(&next_pixel, &q[0].count);
        // env queues: 7 sample uniform, 8 eval uniform, 9 sample 6-axis, 10 eval 6-axis
        ref_strategy_selection(rng.data(), ext.data(), s->materials, q[7].item.data(), &q[7].count, q[8].item.data(),
                               &q[8].count, q[9].item.data(), &q[9].count, q[10].item.data(), &q[10].count,
                               inc.data(), N);
        // sample_envmap_6axis_stage (envmap_sampling.cl:169-217)
        for (uint32_t g = 0; g < q[9].count; ++g) {
            uint32_t idx = q[9].item[g];
            F3 n = ext[idx].Ng;
            F3 wo{-paths[idx].rd.x, -paths[idx].rd.y, -paths[idx].rd.z, 0};
            if (dot3(n, wo) < 0.0f) n = F3{-n.x, -n.y, -n.z, 0};
            float nn[3] = {n.x, n.y, n.z}, pdf, wi[3];
            uint32_t frag;
            ref_sample_envmap_6axis(&pdf, &frag, &rng[4 * idx], nn, pdf6, b6, count);
            orc_sample_from_fragment(s->env_frag + 4 * (size_t)frag, &rng[4 * idx], wi);
            inc[idx].wi = F3{wi[0], wi[1], wi[2], 0};
            inc[idx].pdf[1] = pdf;
        }
        // sample_envmap_stage (envmap_sampling.cl:219-248)
        for (uint32_t g = 0; g < q[7].count; ++g) {
            uint32_t idx = q[7].item[g];
            uint32_t frag = ref_alias_method(&rng[4 * idx], buckets.data(), count);
            float pdf = s->env_pdf[frag], wi[3];
            orc_sample_from_fragment(s->env_frag + 4 * (size_t)frag, &rng[4 * idx], wi);
            inc[idx].wi = F3{wi[0], wi[1], wi[2], 0};
            inc[idx].pdf[1] = pdf;
        }
        // sample_or_eval_lambertian_stage (lambertian.cl:34-71)
        for (uint32_t g = 0; g < q[1].count; ++g) {
            uint32_t idx = q[1].item[g];
            if (inc[idx].strategy == 0) {
                float u[2], wl[3], xa[3], ya[3], ng[3] = {ext[idx].Ng.x, ext[idx].Ng.y, ext[idx].Ng.z};
                ref_random_uniform(&rng[4 * idx], u, 2);
                orc_cosine_hemisphere(u[0], u[1], wl);
                orc_orthonormal_basis(ng, xa, ya);
                inc[idx].wi = F3{xa[0] * wl[0] + ya[0] * wl[1] + ng[0] * wl[2],
                                 xa[1] * wl[0] + ya[1] * wl[1] + ng[1] * wl[2],
                                 xa[2] * wl[0] + ya[2] * wl[1] + ng[2] * wl[2], 0};
                inc[idx].pdf[0] = fmaxr(wl[2], 0.0f) / (float)(M_PI);
            } else {
                uint32_t one = 1;
                ref_sample_or_eval_lambertian_stage(ext.data(), rng.data(), &idx, &one, inc.data(), 1);
            }
        }
        // sample_or_eval_ward_stage (ward.cl:76-117)
        for (uint32_t g = 0; g < q[4].count; ++g) {
            uint32_t idx = q[4].item[g];
            if (inc[idx].strategy == 0) {
                const orc_ward& w = s->wards[s->materials[ext[idx].hs].index];
                F3 wo{-paths[idx].rd.x, -paths[idx].rd.y, -paths[idx].rd.z, 0};
                F3 n = ext[idx].Ng;
                if (dot3(n, wo) < 0.0f) n = F3{-n.x, -n.y, -n.z, 0};
                float u[2], wi[3], wo3[3] = {wo.x, wo.y, wo.z}, n3[3] = {n.x, n.y, n.z};
                ref_random_uniform(&rng[4 * idx], u, 2);
                orc_sample_ward(wo3, n3, w.alpha, u[0], u[1], wi);
                inc[idx].wi = F3{wi[0], wi[1], wi[2], 0};
                inc[idx].pdf[0] = ref_pdf_ward(wo3, wi, n3, w.alpha);
            } else {
                uint32_t one = 1;
                ref_sample_or_eval_ward_stage(paths.data(), ext.data(), s->materials, s->wards, rng.data(), &idx, &one,
                                              inc.data(), 1);
            }
        }
        // sample_or_eval_homogeneous_volume_inside_stage (homogeneous_volume.cl:66-88)
        for (uint32_t g = 0; g < q[6].count; ++g) {
            uint32_t idx = q[6].item[g];
            if (inc[idx].strategy == 0) {
                float u[2], wi[3];
                ref_random_uniform(&rng[4 * idx], u, 2);
                orc_uniform_sphere(u[0], u[1], wi);
                inc[idx].wi = F3{wi[0], wi[1], wi[2], 0};
                inc[idx].pdf[0] = 1.0f / (M_PI * 4.0f);
            } else {
                uint32_t one = 1;
                ref_sample_or_eval_homogeneous_volume_inside_stage(rng.data(), &idx, &one, inc.data(), 1);
            }
        }
        ref_evaluate_envmap_6axis_pdf_stage(ext.data(), q[10].item.data(), &q[10].count, inc.data(), pdf6, W, H, N);
        ref_evaluate_envmap_pdf_stage(q[8].item.data(), &q[8].count, inc.data(), s->env_pdf, W, H, N);
        ref_lambertian_stage(paths.data(), ext.data(), shade.data(), q[1].item.data(), &q[1].count, s->materials,
                             s->lambertians, inc.data(), N);
        ref_ward_stage(paths.data(), ext.data(), shade.data(), q[4].item.data(), &q[4].count, s->materials, s->wards,
                       inc.data(), N);
        ref_homogeneous_volume_stage(paths.data(), vl.data(), ext.data(), shade.data(), q[5].item.data(), &q[5].count,
                                     s->materials, s->volumes, N);
        ref_homogeneous_volume_inside_stage(paths.data(), ext.data(), shade.data(), rng.data(), q[6].item.data(),
                                            &q[6].count, s->materials, s->volumes, inc.data(), N);
        ref_delta_materials(paths.data(), rng.data(), ext.data(), shade.data(), q[2].item.data(), &q[2].count,
                            q[3].item.data(), &q[3].count, s->materials, N);
        ref_homogeneous_volume_through(paths.data(), vl.data(), ext.data(), rng.data(), s->materials, s->volumes, N);
        ref_extension_ray_cast(paths.data(), ext.data(), s->nodes, s->prim_ids, s->indices, s->points, s->sphere_begin,
                               s->spheres, N);
        for (int k = 1; k < 11; ++k) q[k].count = 0;  // clearStrategyQueue / clearMaterialQueue
        uint32_t* qi[7];
        uint32_t* qc[7];
        for (int k = 0; k < 7; ++k) {
            qi[k] = q[k].item.data();
            qc[k] = &q[k].count;
        }
        ref_logic(paths.data(), rng.data(), ext.data(), shade.data(), env_const_rgba, accum_rgb32, s->materials, qi, qc,
                  N);
    }
    if (slots_out) {
        std::vector<int32_t> qid(N, -1);
        for (int k = 0; k < 7; ++k)
            for (uint32_t g = 0; g < q[k].count; ++g) qid[q[k].item[g]] = k;
        for (uint64_t i = 0; i < N; ++i) {
            orc_slot& o = slots_out[i];
            const WP& p = paths[i];
            float* dst[4] = {o.T, o.L, o.ro, o.rd};
            const F3* src[4] = {&p.T, &p.L, &p.ro, &p.rd};
            for (int k = 0; k < 4; ++k) {
                dst[k][0] = src[k]->x;
                dst[k][1] = src[k]->y;
                dst[k][2] = src[k]->z;
            }
            o.logic_i = p.logic_i;
            o.pixel_index = p.pixel_index;
            memcpy(o.rng, &rng[4 * i], 16);
            o.hit_surface = ext[i].hs;
            o.hit_volume = ext[i].hv;
            o.tmin = ext[i].tmin;
            o.Ng[0] = ext[i].Ng.x;
            o.Ng[1] = ext[i].Ng.y;
            o.Ng[2] = ext[i].Ng.z;
            o.queue = qid[i];
            o.vol_count = vl[i].count;
            memcpy(o.vols, vl[i].volumes, sizeof(o.vols));
        }
    }
    return next_pixel;
}
