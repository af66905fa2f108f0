// wavefront.cu — the per-bounce kernels of the wavefront path tracer (sm_103a).
//
// One reference step() (common/wavefront_path_tracing.hpp:591-939) is about
// twenty launches of 2^22 work items.  Here it is three kernels and a memset:
//   1. compact_new  — ordered compaction of the slots logic marked "new path"
//      (slot order, so pixels are assigned exactly as a sequential run of
//      new_path.cl:41-43 over that queue would);
//   2. shade        — persistent kernel draining the new-path queue and the six
//      material queues back to back; per item it runs, in the reference stage
//      order, new_path / strategy_selection / envmap sample / BSDF sample or
//      pdf / envmap pdf / material stage / homogeneous_volume_through, keeping
//      IncidentSample and ShadingResult in registers;
//   3. trace_logic  — logic.cl after the bounce's closest hits (cast by the
//      persistent trace kernel, or fused for small scenes): throughput update,
//      envmap on miss, Russian roulette, FP64 per-pixel accumulation, and the
//      appends to the next step's material queues, aggregated per warp
//      (match_any) and per block (shared-memory counts, one global atomic per
//      queue per block).
// Every slot's arithmetic is the reference kernels' arithmetic (see the
// file:line notes); the translation unit is built with --fmad=false.
#include <cuda_fp16.h>

#include "wavefront.cuh"
#include "traverse.cuh"
#include "guide.cuh"

namespace rgr {
namespace dev {
namespace {

using namespace rgr::fm;

constexpr float kPiF = 3.14159274f;                 // (float)(M_PI)
constexpr float kPdfUniformSphere = 0.0795774683f;  // (float)(1.0 / (M_PI * 4.0))
constexpr float kFourPiF = 12.566371f;              // (float)(4.0 * M_PI)
constexpr double kPiD = 3.14159265358979323846;     // M_PI
constexpr float kFltMax = 3.40282347e+38f;

enum { kBxdf = 0, kEnv = 1, kNone = 2, kGuide = 3 };

RGR_DEV f3 mix3(f3 a, f3 b, float t) { return mk(mix_(a.x, b.x, t), mix_(a.y, b.y, t), mix_(a.z, b.z, t)); }
RGR_DEV float sqr(float x) { return x * x; }
RGR_DEV int to_int(float x) {
    if (isnan(x)) return 0;
    if (x >= 2147483648.0f) return 2147483647;
    if (x <= -2147483648.0f) return (-2147483647 - 1);
    return (int)x;
}

// ------------------------------------------------------------ envmap
// cartesian_to_polar (envmap_sampling.cl:25-34)
RGR_DEV void cartesian_to_polar(f3 rd, float& theta, float& phi) {
    float z = rd.y, x = rd.z, y = rd.x;
    theta = atan2_(sqrtf(x * x + y * y), z);
    phi = atan2_(y, x);
    if (!is_finite(phi)) phi = 0.0f;
}
// envmap_index (envmap_sampling.cl:75-95)
RGR_DEV int envmap_index(f3 wi, int width, int height) {
    float theta, phi;
    cartesian_to_polar(wi, theta, phi);
    float u = 1.0f - phi / (2.0f * kPiF);
    float v = theta / kPiF;
    int ix = to_int(floorf(u * (float)width));
    int iy = to_int(floorf(v * (float)height));
    int r = ix % width;
    ix = r < 0 ? r + width : r;
    iy = min(max(iy, 0), height - 1);
    return iy * width + ix;
}
RGR_DEV f3 texel(const SceneView& sc, int i, int j) { return xyz(__ldg(sc.env_rgba + (size_t)j * sc.env_w + i)); }
// get_envmap_value (envmap_sampling.cl:36-52): read_imagef with normalized
// coordinates, CLK_ADDRESS_REPEAT, nearest or bilinear (OpenCL 1.2 sampler
// formulas, FP32 weights)
RGR_DEV f3 envmap_value(const SceneView& sc, f3 rd, bool linear) {
    float theta, phi;
    cartesian_to_polar(rd, theta, phi);
    float su = 1.0f - phi / (2.0f * kPiF);
    float sv = theta / kPiF;
    const int w = sc.env_w, h = sc.env_h;
    float u = (su - floorf(su)) * (float)w;
    float v = (sv - floorf(sv)) * (float)h;
    if (!linear) {
        int i = to_int(floorf(u)), j = to_int(floorf(v));
        if (i > w - 1) i = i - w;
        if (j > h - 1) j = j - h;
        i = min(max(i, 0), w - 1);
        j = min(max(j, 0), h - 1);
        return texel(sc, i, j);
    }
    float uu = u - 0.5f, vv = v - 0.5f;
    int i0 = to_int(floorf(uu)), j0 = to_int(floorf(vv));
    int i1 = i0 + 1, j1 = j0 + 1;
    if (i0 < 0) i0 = w + i0;
    if (i1 > w - 1) i1 = i1 - w;
    if (j0 < 0) j0 = h + j0;
    if (j1 > h - 1) j1 = j1 - h;
    i0 = min(max(i0, 0), w - 1);
    i1 = min(max(i1, 0), w - 1);
    j0 = min(max(j0, 0), h - 1);
    j1 = min(max(j1, 0), h - 1);
    float a = uu - floorf(uu), b = vv - floorf(vv);
    float w00 = (1.0f - a) * (1.0f - b), w10 = a * (1.0f - b);
    float w01 = (1.0f - a) * b, w11 = a * b;
    return ((texel(sc, i0, j0) * w00 + texel(sc, i1, j0) * w10) + texel(sc, i0, j1) * w01) + texel(sc, i1, j1) * w11;
}
// alias_method (envmap_sampling.cl:54-66); table t of 7
RGR_DEV uint32_t alias_method(const SceneView& sc, size_t base, Rng& st, uint32_t count) {
    uint32_t idx = (uint32_t)(st.uniform_integer() % (uint64_t)count);
    int2 b = __ldg(sc.env_alias + base + idx);
    if (b.y < 0) return idx;
    float u = st.uniform();
    if (u < __int_as_float(b.x)) return idx;
    return (uint32_t)b.y;
}
// sample_from_fragment (envmap_sampling.cl:68-73, 158-167)
RGR_DEV f3 sample_from_fragment(const SceneView& sc, uint32_t idx, Rng& st) {
    float4 fr = __ldg(sc.env_frag + idx);
    float y = mix_(fr.x, fr.y, st.uniform());
    float phi = mix_(fr.z, fr.w, st.uniform());
    float sp, cp;
    sincos_(phi, &sp, &cp);
    f3 p = mk(sp, y, cp);
    float r_xz = sqrtf(fmax_(1.0f - p.y * p.y, 0.0f));
    p.x *= r_xz;
    p.z *= r_xz;
    return p;
}
RGR_DEV void six_axis_bases(size_t count, f3 n, size_t& xb, size_t& yb, size_t& zb) {
    xb = count * (0.0f < n.x ? 1 : 2);
    yb = count * (0.0f < n.y ? 3 : 4);
    zb = count * (0.0f < n.z ? 5 : 6);
}

// ------------------------------------------------------------ BSDFs
// cosine_weighted_hemisphere_z_up (lambertian.cl:9-20)
RGR_DEV f3 cosine_hemisphere(float a, float b) {
    float r = sqrtf(a);
    float theta = (float)((double)b * kPiD * 2.0);
    float s, c;
    sincos_(theta, &s, &c);
    return mk(r * c, r * s, sqrtf(fmax_(1.0f - a, 0.0f)));
}
// get_orthonormal_basis (lambertian.cl:26-32)
RGR_DEV void orthonormal_basis(f3 z, f3& xa, f3& ya) {
    const float sign = copysign_(1.0f, z.z);
    const float a = -1.0f / (sign + z.z);
    const float b = z.x * z.y * a;
    xa = mk(1.0f + sign * z.x * z.x * a, sign * b, -sign * z.x);
    ya = mk(b, sign + z.y * z.y * a, -z.y);
}
RGR_DEV f3 reflect(f3 d, f3 n) { return d - (2.0f * dot(d, n)) * n; }
// sample_ward (ward.cl:40-53)
RGR_DEV f3 sample_ward(f3 wo, f3 zaxis, float alpha, float u0, float u1) {
    float phiH = u0 * 2.0f * kPiF;
    float thetaH = atan_(alpha * sqrtf(-log_(u1)));
    float st, ct, sp, cp;
    sincos_(thetaH, &st, &ct);
    sincos_(phiH, &sp, &cp);
    f3 hl = mk(st * cp, st * sp, ct);
    f3 xa, ya;
    orthonormal_basis(zaxis, xa, ya);
    f3 h = xa * hl.x + ya * hl.y + zaxis * hl.z;
    return reflect(-wo, h);
}
// pdf_ward (ward.cl:55-74)
RGR_DEV float pdf_ward(f3 wo, f3 wi, f3 zaxis, float alpha) {
    if (dot(wo, zaxis) * dot(wi, zaxis) < 0.0f) return 0.0f;
    const float alpha2 = sqr(alpha);
    f3 h = normalize(wi + wo);
    float c = dot(h, zaxis);
    float c2 = sqr(c);
    float tan2 = (1.0f - c2) / c2;
    float k0 = 1.0f / (4.0f * kPiF * alpha2 * dot(h, wi) * (c * c * c));
    float k1 = exp_(-tan2 / alpha2);
    return k0 * k1;
}
// fresnel_dielectrics, refract (delta_materials.cl:11-32)
RGR_DEV float fresnel_dielectrics(float c, float eta_t, float eta_i) {
    float g = sqrtf(eta_t * eta_t / sqr(eta_i) - 1.0f + sqr(c));
    float a = 0.5f * sqr(g - c) / sqr(g + c);
    float b = 1.0f + sqr(c * (g + c) - 1.0f) / sqr(c * (g - c) + 1.0f);
    return a * b;
}
RGR_DEV bool refract(f3& out, f3 d, f3 n, float eta_i, float eta_t) {
    float eta = eta_i / eta_t;
    float NoD = dot(n, d);
    float k = 1.0f - eta * eta * (1.0f - NoD * NoD);
    if (k <= 0.0f) return false;
    out = eta * d - (eta * NoD + sqrtf(k)) * n;
    return true;
}
// uniform_on_unit_sphere (homogeneous_volume.cl:7-14)
RGR_DEV f3 uniform_sphere(float u0, float u1) {
    float phi = (float)((double)u0 * kPiD * 2.0);
    float z = mix_(-1.0f, 1.0f, u1);
    float r_xy = sqrtf(fmax_(1.0f - z * z, 0.0f));
    float s, c;
    sincos_(phi, &s, &c);
    return mk(r_xy * c, r_xy * s, z);
}
RGR_DEV uint32_t volume_hash(float4 v) {  // types.cl:104-106 (C, R.x, R.y, R.z)
    return __float_as_uint(v.w) ^ __float_as_uint(v.x) ^ __float_as_uint(v.y) ^ __float_as_uint(v.z);
}

// sel0/pdf0: BSDF (or phase function), sel1/pdf1: envmap, sel2/pdf2: the
// learned guide (guided renders only)
struct Incident {
    f3 wi;
    float sel0, sel1, pdf0, pdf1, sel2, pdf2;
    int strategy;
};
template <bool kGuided>
RGR_DEV float incident_pdf(const Incident& is) {  // types.cl:65-71
    float pdf = 0.0f;
    pdf = pdf + is.sel0 * is.pdf0;
    pdf = pdf + is.sel1 * is.pdf1;
    if (kGuided) pdf = pdf + is.sel2 * is.pdf2;
    return pdf;
}

// One slot's share of a step, from new_path to homogeneous_volume_through.
// k: the queue the slot came from (0 = new path, else its material type).
// Guided renders: gi is the slot's index among this bounce's guided items
// (its mixture in gd.lobes), ~0u when the vertex is not guided.
template <bool kGuided>
RGR_DEV void shade_slot(const RequestD& rq, const PathsView& P, int k, uint32_t slot, unsigned long long gpix,
                        const GuideRenderD& gd, uint32_t gi) {
    const SceneView& sc = rq.sc;
    // Path state moves by 32-byte sector of the slot record and only where this
    // item uses it (a material queue is a sparse subset of the slots, so each
    // sector touched costs a DRAM sector): a new path (k = 0) replaces everything
    // but its RNG state and the volume hit of the ended path, so it skips the
    // (T, L) sector and the volume list; L is stored only when the stage changes
    // it; the first half of the volume list is loaded only when the list is used.
    const bool fresh = k == 0;
    float4 ro4, rd4, ng4, rng4, T4 = make_float4(0.0f, 0.0f, 0.0f, 0.0f), L4 = T4;
    int4 va = make_int4(0, 0, 0, 0), vb = va;
    // the ray's sector and the (ng, rng) sector, each in one access; (T, L) likewise
    ld_sector<0>(P, slot, ro4, rd4);
    ld_sector<2>(P, slot, ng4, rng4);
    int vcount = 0;
    if (!fresh) {
        ld_sector<1>(P, slot, T4, L4);
        vcount = vcount_of(__float_as_uint(L4.w));
        if (k == kMatVolume || vcount > 0) {
            float4 a, b;
            ld_sector<3>(P, slot, a, b);
            va = make_int4(__float_as_int(a.x), __float_as_int(a.y), __float_as_int(a.z), __float_as_int(a.w));
            vb = make_int4(__float_as_int(b.x), __float_as_int(b.y), __float_as_int(b.z), __float_as_int(b.w));
        }
    } else {
        ro4 = ng4 = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    }
    Rng rng = rng_of_bits(rng4);
    f3 ro = xyz(ro4), rd = xyz(rd4), T = xyz(T4), L = mk(0, 0, 0), Ng = xyz(ng4);
    float tmin = ro4.w;
    int32_t hv = __float_as_int(rd4.w);
    int32_t hs = __float_as_int(ng4.w);
    uint32_t pixel = __float_as_uint(T4.w);
    uint32_t logic_i = 0;

    if (k == 0) {  // new_path (new_path.cl:17-83)
        const CameraD& cam = rq.cam;
        T = mk(1, 1, 1);
        L = mk(0, 0, 0);
        logic_i = 0;
        uint32_t npix = cam.w * cam.h;
        pixel = (uint32_t)(gpix % (unsigned long long)npix);
        uint32_t x = pixel % cam.w, y = pixel / cam.w;
        float ux = rng.uniform();
        float uy = rng.uniform();
        f3 sop = mk(cam.o[0], cam.o[1], cam.o[2]) + mk(cam.r[0], cam.r[1], cam.r[2]) * ((float)x + ux) +
                 mk(cam.b[0], cam.b[1], cam.b[2]) * ((float)y + uy);
        float u0 = rng.uniform();
        float u1 = rng.uniform();
        float r = sqrtf(u0);
        float theta = (float)((double)u1 * kPiD * 2.0);
        float s, c;
        sincos_(theta, &s, &c);
        float lensx = rq.dof * r * c;
        float lensy = rq.dof * r * s;
        f3 lens = mk(cam.eye[0], cam.eye[1], cam.eye[2]) + mk(cam.up[0], cam.up[1], cam.up[2]) * lensx +
                  mk(cam.right[0], cam.right[1], cam.right[2]) * lensy;
        ro = lens;
        rd = normalize(sop - lens);
        vcount = 0;
        hs = -1;
        tmin = kFltMax;
        Ng = mk(0, 0, 0);
        if (kGuided) gd.nrec[slot] = 0;
    }
    f3 shLe = mk(0, 0, 0), shT = mk(1, 1, 1);

    // strategy_selection (mixture_density.cl:7-133)
    Incident is;
    is.wi = mk(0, 0, 0);
    is.sel0 = is.sel1 = is.pdf0 = is.pdf1 = is.sel2 = is.pdf2 = 0.0f;
    is.strategy = kNone;
    const bool surface_hit = 0 <= hs, volume_hit = 0 <= hv;
    int envq = -1;
    if (surface_hit || volume_hit) {
        const float env_p = sc.has_env ? rq.env_p : 0.0f;
        if (surface_hit) {
            int mt = __ldg(sc.materials + hs).x;
            if (mt == kMatLambertian || mt == kMatWard) {
                const float bxdf_p = 1.0f - env_p;
                is.sel0 = bxdf_p;
                is.sel1 = 1.0f - bxdf_p;
            } else {
                is.sel0 = 1.0f;
                is.sel1 = 0.0f;
            }
        } else {
            const float bxdf_p = 1.0f - env_p;
            is.sel0 = bxdf_p;
            is.sel1 = 1.0f - bxdf_p;
        }
        if (kGuided && gi != ~0u) {
            // the guide takes its share of the non-envmap probability: the sum of the
            // record's stored weights (the network's selection output, or the fixed
            // fraction), decoded identically wherever the record is read
            is.sel2 = is.sel0 * mixture_alpha(gd.lobes + (size_t)kGuideMixVecs * gi);
            is.sel0 = is.sel0 - is.sel2;
        }
        float u = rng.uniform();
        if (kGuided) {
            is.strategy = (u <= is.sel0) ? kBxdf : ((u <= is.sel0 + is.sel2) ? kGuide : kEnv);
        } else {
            is.strategy = (u <= is.sel0) ? kBxdf : kEnv;
        }
        if (is.sel1 != 0.0f) {
            const int sq = volume_hit ? 0 : 2, eq = volume_hit ? 1 : 3;
            envq = is.strategy == kEnv ? sq : eq;
        }
    }
    const uint4* mix = (kGuided && gi != ~0u) ? gd.lobes + (size_t)kGuideMixVecs * gi : nullptr;
    if (kGuided && gi != ~0u && is.strategy == kGuide) {
        const float u0 = rng.uniform();
        const float u1 = rng.uniform();
        const float u2 = rng.uniform();
        float d[3];
        mixture_sample(mix, u0, u1, u2, d);
        is.wi = mk(d[0], d[1], d[2]);
    }
    const size_t count = (size_t)sc.env_w * sc.env_h;
    // sample_envmap_6axis_stage / sample_envmap_stage (envmap_sampling.cl:169-248)
    if (envq == 2) {
        f3 n = Ng;
        if (dot(n, -rd) < 0.0f) n = -n;
        size_t xb, yb, zb;
        six_axis_bases(count, n, xb, yb, zb);
        float u = rng.uniform();
        f3 ap = n * n;
        size_t sel = (u < ap.x) ? xb : ((u < ap.x + ap.y) ? yb : zb);
        uint32_t idx = alias_method(sc, sel, rng, (uint32_t)count);
        float pdf = 0.0f;
        pdf = pdf + ap.x * __ldg(sc.env_pdf + xb + idx);
        pdf = pdf + ap.y * __ldg(sc.env_pdf + yb + idx);
        pdf = pdf + ap.z * __ldg(sc.env_pdf + zb + idx);
        is.wi = sample_from_fragment(sc, idx, rng);
        is.pdf1 = pdf;
    } else if (envq == 0) {
        uint32_t idx = alias_method(sc, 0, rng, (uint32_t)count);
        float pdf = __ldg(sc.env_pdf + idx);
        is.wi = sample_from_fragment(sc, idx, rng);
        is.pdf1 = pdf;
    }
    // BSDF sample or pdf
    int2 mref = make_int2(0, 0);
    if (k >= 1 && k <= 5) mref = __ldg(sc.materials + hs);
    if (k == kMatLambertian) {  // sample_or_eval_lambertian_stage (lambertian.cl:34-71)
        float cosTheta;
        f3 ns = Ng;  // the raw Ng, as the reference samples, unless two-sided sampling is on
        if ((kGuided || (rq.flags & kFlagTwoSidedLambertian)) && dot(ns, -rd) < 0.0f) ns = -ns;
        if (is.strategy == kBxdf) {
            float u0 = rng.uniform();
            float u1 = rng.uniform();
            f3 wl = cosine_hemisphere(u0, u1);
            f3 xa, ya;
            orthonormal_basis(ns, xa, ya);
            is.wi = xa * wl.x + ya * wl.y + ns * wl.z;
            cosTheta = wl.z;
        } else {
            cosTheta = dot(ns, is.wi);
        }
        is.pdf0 = fmax_(cosTheta, 0.0f) / kPiF;
    } else if (k == kMatWard) {  // sample_or_eval_ward_stage (ward.cl:76-117)
        float4 w0 = __ldg(sc.wards + 3 * (size_t)mref.y);
        f3 wo = -rd;
        f3 n = Ng;
        if (dot(n, wo) < 0.0f) n = -n;
        f3 wi;
        if (is.strategy == kBxdf) {
            float u0 = rng.uniform();
            float u1 = rng.uniform();
            wi = sample_ward(wo, n, w0.x, u0, u1);
        } else {
            wi = is.wi;
        }
        is.wi = wi;
        is.pdf0 = pdf_ward(wo, wi, n, w0.x);
    } else if (k == kMatVolumeInside) {  // homogeneous_volume.cl:66-88
        if (is.strategy == kBxdf) {
            float u0 = rng.uniform();
            float u1 = rng.uniform();
            is.wi = uniform_sphere(u0, u1);
        }
        is.pdf0 = kPdfUniformSphere;
    }
    // evaluate_envmap_6axis_pdf_stage / evaluate_envmap_pdf_stage (envmap_sampling.cl:250-281)
    if (envq == 3) {
        size_t xb, yb, zb;
        f3 n = Ng;  // the raw Ng, as the reference does, unless the backside fix is on
        if ((kGuided || (rq.flags & kFlagFixBacksideEnvPdf)) && dot(n, -rd) < 0.0f) n = -n;
        six_axis_bases(count, n, xb, yb, zb);
        f3 ap = n * n;
        int index = envmap_index(is.wi, sc.env_w, sc.env_h);
        float pdf = 0.0f;
        pdf = pdf + ap.x * __ldg(sc.env_pdf + xb + index);
        pdf = pdf + ap.y * __ldg(sc.env_pdf + yb + index);
        pdf = pdf + ap.z * __ldg(sc.env_pdf + zb + index);
        is.pdf1 = pdf;
    } else if (envq == 1) {
        is.pdf1 = __ldg(sc.env_pdf + envmap_index(is.wi, sc.env_w, sc.env_h));
    }
    if (kGuided && is.sel2 != 0.0f) is.pdf2 = mixture_pdf(mix, is.wi.x, is.wi.y, is.wi.z);
    // the guided vertex as the network saw it (before the stage moves ro)
    f3 gx = mk(0, 0, 0), gn = mk(0, 0, 0);
    if (kGuided && is.sel2 != 0.0f) {
        gx = ro + rd * tmin;
        if (hs >= 0) {
            gn = Ng;
            if (dot(gn, -rd) < 0.0f) gn = -gn;
        }
    }
    const f3 wo_in = -rd;
    // material stages
    if (k == kMatLambertian) {  // lambertian_stage (lambertian.cl:73-123)
        float4 le = __ldg(sc.lambertians + 2 * (size_t)mref.y), R = __ldg(sc.lambertians + 2 * (size_t)mref.y + 1);
        f3 n = Ng;
        if (dot(n, -rd) < 0.0f) n = -n;
        f3 wi = is.wi;
        float pdf = incident_pdf<kGuided>(is);
        float cosTheta = dot(wi, n);
        f3 Ts = mk(0, 0, 0);
        if (0.0f < cosTheta) Ts = xyz(R) / kPiF * cosTheta / pdf;
        shLe = xyz(le);
        shT = Ts;
        ro = ro + rd * tmin + wi * 1.0e-5f + n * 1.0e-5f;
        rd = wi;
    } else if (k == kMatWard) {  // ward_stage (ward.cl:119-186)
        float4 w0 = __ldg(sc.wards + 3 * (size_t)mref.y);
        float4 refl = __ldg(sc.wards + 3 * (size_t)mref.y + 1), edge = __ldg(sc.wards + 3 * (size_t)mref.y + 2);
        f3 n = Ng;
        f3 wo = -rd;
        if (dot(n, wo) < 0.0f) n = -n;
        f3 wi = is.wi;
        float pdf = incident_pdf<kGuided>(is);
        float cosTheta = dot(wi, n);
        f3 Ts = mk(0, 0, 0);
        if (0.0f < cosTheta) {
            f3 lv = wi + wo;
            f3 h = normalize(lv);
            float alpha2 = sqr(w0.x);
            float cth = dot(h, n);
            float cth2 = sqr(cth);
            float tan2 = (1.0f - cth2) / cth2;
            float mu = dot(h, wi);
            f3 rho = mix3(xyz(refl), xyz(edge), pow_(1.0f - mu, 1.0f / w0.y));
            f3 k0 = rho / (kPiF * alpha2);
            float k1 = exp_(-tan2 / alpha2);
            float dn = dot(lv, n);
            float k2 = dot(lv, lv) / sqr(sqr(dn));
            Ts = k0 * k1 * k2 * cosTheta / pdf;
        }
        shT = Ts;
        ro = ro + rd * tmin + wi * 1.0e-5f + n * 1.0e-5f;
        rd = wi;
    } else if (k == kMatVolume) {  // homogeneous_volume_stage (homogeneous_volume.cl:19-64)
        bool backside = dot(Ng, -rd) < 0.0f;
        int vols[8] = {va.x, va.y, va.z, va.w, vb.x, vb.y, vb.z, 0};
        if (backside) {  // inVolumeList_Remove (types.cl:115-132)
            uint32_t hsh = volume_hash(__ldg(sc.volumes + mref.y));
            bool move = false;
#pragma unroll
            for (int i = 0; i < 7; ++i) {  // constant indices keep the list in registers
                if (i < vcount) {
                    if (move) {
                        if (i > 0) vols[i - 1] = vols[i];
                    } else {
                        int2 mi = __ldg(sc.materials + vols[i]);
                        if (volume_hash(__ldg(sc.volumes + mi.y)) == hsh) move = true;
                    }
                }
            }
            if (move) vcount--;
        } else if (vcount < 7) {  // inVolumeList_Add (types.cl:108-114)
#pragma unroll
            for (int i = 0; i < 7; ++i)
                if (i == vcount) vols[i] = hs;
            vcount++;
        }
        va = make_int4(vols[0], vols[1], vols[2], vols[3]);
        vb = make_int4(vols[4], vols[5], vols[6], vcount);
        ro = ro + rd * (tmin + 1.0e-5f);
    } else if (k == kMatVolumeInside) {  // homogeneous_volume_inside_stage (homogeneous_volume.cl:90-129)
        int2 mi = __ldg(sc.materials + hv);
        float4 vol = __ldg(sc.volumes + mi.y);
        float pdf = incident_pdf<kGuided>(is);
        shT = xyz(vol) / kFourPiF / pdf;
        ro = ro + rd * tmin;
        rd = is.wi;
    } else if (k == kMatSpecular) {  // delta_materials.cl:34-64
        f3 n = Ng;
        if (dot(n, -rd) < 0.0f) n = -n;
        f3 wi = reflect(rd, n);
        ro = ro + rd * tmin + wi * 1.0e-5f;
        rd = wi;
    } else if (k == kMatDielectric) {  // delta_materials.cl:66-121
        f3 n = Ng;
        f3 wo = -rd;
        bool backside = dot(n, wo) < 0.0f;
        float eta_i = 1.0f, eta_t = 1.5f;
        if (backside) {
            float e = eta_i;
            eta_i = eta_t;
            eta_t = e;
            n = -n;
        }
        float f = fresnel_dielectrics(fabs_(dot(n, wo)), eta_t, eta_i);
        float u = rng.uniform();
        float rc = 1.0f;
        f3 wi;
        if (u < f) {
            wi = reflect(rd, n);
        } else if (!refract(wi, rd, n, eta_i, eta_t)) {
            wi = reflect(rd, n);
        } else {
            rc = sqr(eta_t / eta_i);
        }
        shT = mk(rc, rc, rc);
        ro = ro + rd * tmin + wi * 1.0e-5f;
        rd = wi;
    }
    // logic.cl:31-33, applied here: the stage that made the shading result consumes it.
    // L + T * shLe leaves L's bits unchanged when shLe is zero and T finite (L is
    // never -0), so L is read and written only otherwise, for new paths and in
    // guided renders (the training records carry it).
    const bool touch_L = fresh || kGuided || shLe.x != 0.0f || shLe.y != 0.0f || shLe.z != 0.0f ||
                         !is_finite(T.x) || !is_finite(T.y) || !is_finite(T.z);
    // the volume stage changes the volume count, which L.w carries
    const bool store_L = touch_L || k == kMatVolume;
    if (store_L && !fresh) {
        L = xyz(L4);
        logic_i = depth_of(__float_as_uint(L4.w));
    }
    L = L + T * shLe;
    T = T * shT;
    if (kGuided && is.sel2 != 0.0f && gd.record && guide_training_open(gd.train)) {
        // training record: the vertex, the sampled direction, the path's (L, T) just
        // after this vertex, so that the logic can recover the radiance L_i that
        // arrived along wi when the path ends, and cos / pdf of the sample
        const uint32_t r = gd.nrec[slot];
        if (r < (uint32_t)kGuideRecords) {
            const float c = (hs >= 0) ? fmax_(dot(is.wi, gn), 0.0f) : 1.0f;
            const float cp = c / incident_pdf<kGuided>(is);
            float4* rec = gd.records + ((size_t)slot * kGuideRecords + r) * kGuideRecordVecs;
            st_v8(rec, make_float4(L.x, L.y, L.z, T.x),
                  make_float4(T.y, T.z, cp, is.pdf0));  // pdf0: the BSDF (phase) pdf of wi
            st_v8(rec + 2, make_float4(gx.x, gx.y, gx.z, gn.x), make_float4(gn.y, gn.z, wo_in.x, wo_in.y));
            st_v8(rec + 4, make_float4(wo_in.z, is.wi.x, is.wi.y, is.wi.z), make_float4(0.0f, 0.0f, 0.0f, 0.0f));
            gd.nrec[slot] = (uint8_t)(r + 1);
        }
    }

    // homogeneous_volume_through (homogeneous_volume_through.cl:7-44)
    hs = -1;
    hv = -1;
    if (0 < vcount) {
        uint64_t u = rng.uniform_integer();
        int sel = (int)(u % (uint64_t)vcount);
        const int vols[7] = {va.x, va.y, va.z, va.w, vb.x, vb.y, vb.z};
        hv = pick(vols, sel < 7 ? sel : 6);
    }
    tmin = kFltMax;
    if (0 <= hv) {
        int2 mi = __ldg(sc.materials + hv);
        float4 vol = __ldg(sc.volumes + mi.y);
        float u = rng.uniform();
        tmin = -1.0f / vol.w * log_(u);
    }
    st_sector<0>(P, slot, f4(ro, tmin), f4(rd, __int_as_float(hv)));
    if (store_L)  // a new path's count is 0; its list keeps the stale ids
        st_sector<1>(P, slot, f4(T, __uint_as_float(pixel)), f4(L, __uint_as_float(depth_word(logic_i, vcount))));
    else  // the sector was read above: this half store finds it in L2
        P.T[slot] = f4(T, __uint_as_float(pixel));
    if (k == kMatVolume) {
        vb.w = vcount;
        st_sector<3>(P, slot,
                     make_float4(__int_as_float(va.x), __int_as_float(va.y), __int_as_float(va.z), __int_as_float(va.w)),
                     make_float4(__int_as_float(vb.x), __int_as_float(vb.y), __int_as_float(vb.z), __int_as_float(vb.w)));
    }
    st_sector<2>(P, slot, f4(Ng, __int_as_float(hs)), rng_bits(rng));
}

// ------------------------------------------------------------ kernels
__global__ void k_init(PathsView P, QueueView Q, uint32_t seed_offset) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < Q.ntiles) {
        uint32_t beg = i * kTile;
        Q.tile_new[i] = min(kTile, P.n - beg);
    }
    if (i >= Q.ntiles * kTile) return;
    if (i >= P.n) {
        P.qid[i] = kQueueIdle;  // padding up to a whole tile
        return;
    }
    // random_initialize (peseudo_random.cl:48-64)
    unsigned long long x = (unsigned long long)seed_offset + i;
    unsigned long long r[2];
    for (int k = 0; k < 2; ++k) {
        unsigned long long z = (x += 0x9e3779b97f4a7c15ull);
        z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
        z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
        r[k] = z ^ (z >> 31);
    }
    uint4 s = make_uint4((uint32_t)r[0], (uint32_t)(r[0] >> 32), (uint32_t)r[1], (uint32_t)(r[1] >> 32));
    if ((s.x | s.y | s.z | s.w) == 0u) s.x = 1u;
    P.rng[i] = s;
    P.ro[i] = make_float4(0, 0, 0, kFltMax);
    P.rd[i] = make_float4(0, 0, 0, __int_as_float(-1));
    P.T[i] = make_float4(0, 0, 0, 0);
    P.L[i] = make_float4(0, 0, 0, 0);
    P.ng[i] = make_float4(0, 0, 0, __int_as_float(-1));
    P.va[i] = make_int4(0, 0, 0, 0);
    P.vb[i] = make_int4(0, 0, 0, 0);
    P.qid[i] = 0;  // initialize_all_as_new_path (new_path.cl:9-15)
    P.req[i] = 0;
}

// Ordered compaction of new-path slots: block t owns slots [t*4096, (t+1)*4096).
__global__ void __launch_bounds__(256) k_compact_new(PathsView P, QueueView Q) {
    __shared__ uint32_t s_warp[8];
    __shared__ uint32_t s_prefix;
    const uint32_t t = blockIdx.x, tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    // prefix of the tile counts before this tile
    uint32_t sum = 0;
    for (uint32_t j = tid; j < t; j += 256) sum += Q.tile_new[j];
    for (int o = 16; o > 0; o >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, o);
    if (lane == 0) s_warp[warp] = sum;
    __syncthreads();
    if (tid == 0) {
        uint32_t p = 0;
        for (int w = 0; w < 8; ++w) p += s_warp[w];
        s_prefix = p;
    }
    __syncthreads();
    const uint32_t prefix = s_prefix;
    // 16 consecutive slots per thread
    const uint32_t base = t * kTile + tid * 16;
    uint4 q = *reinterpret_cast<const uint4*>(P.qid + base);
    uint32_t words[4] = {q.x, q.y, q.z, q.w};
    uint32_t mask = 0;
    for (int k = 0; k < 16; ++k) {
        uint32_t b = (words[k >> 2] >> (8 * (k & 3))) & 0xffu;
        if (b == 0u) mask |= 1u << k;
    }
    uint32_t c = __popc(mask);
    // block exclusive scan of c
    uint32_t inc = c;
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t v = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= (uint32_t)o) inc += v;
    }
    __syncthreads();
    if (lane == 31) s_warp[warp] = inc;
    __syncthreads();
    uint32_t woff = 0, total = 0;
    for (int w = 0; w < 8; ++w) {
        uint32_t v = s_warp[w];
        if (w < (int)warp) woff += v;
        total += v;
    }
    uint32_t pos = prefix + woff + inc - c;
    uint32_t* out = Q.items[0];
    while (mask) {
        int k = __ffs(mask) - 1;
        mask &= mask - 1;
        out[pos++] = base + k;
    }
    if (t == Q.ntiles - 1 && tid == 0) {
        uint32_t all = prefix + total;
        Q.counts[0] = all;
        unsigned long long np = *Q.next_pixel;
        *Q.step_base = np;
        *Q.next_pixel = np + all;  // finalize_new_path (new_path.cl:85-88)
    }
}

template <bool kGuided>
__device__ __forceinline__ void shade_items(const PathsView& P, const QueueView& Q, const RenderParams& rp) {
    uint32_t off[kNumQueues + 1];
    off[0] = 0;
#pragma unroll
    for (int k = 0; k < kNumQueues; ++k) off[k + 1] = off[k] + Q.counts[k];
    const uint32_t total = off[kNumQueues];
    // guided items are numbered Lambertian, Ward, in-volume (as the inference kernel does)
    const uint32_t g4 = off[kMatLambertian + 1] - off[kMatLambertian];
    const uint32_t g6 = g4 + (off[kMatWard + 1] - off[kMatWard]);
    const unsigned long long base_pixel = *Q.step_base;
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < total; i += stride) {
        int k = 0;
#pragma unroll
        for (int j = 1; j < kNumQueues; ++j) k += (i >= off[j]) ? 1 : 0;
        const uint32_t slot = queue_items(Q, k)[i - pick(off, k)];
        unsigned long long gpix = 0;
        int r;
        if (k == 0) {
            gpix = base_pixel + (i - off[0]);
            if (rp.sample_limit != 0ull && gpix >= rp.sample_limit) {
                P.qid[slot] = kQueueIdle;  // sample budget reached: the slot retires
                continue;
            }
            // the request whose sample range holds this global sample index
            r = 0;
            while (r + 1 < rp.nreq && gpix >= rp.reqs[r].sample_end) ++r;
            P.req[slot] = (uint16_t)r;
            gpix -= rp.reqs[r].sample_begin;
        } else {
            r = P.req[slot];
        }
        uint32_t gi = ~0u;
        if (kGuided) {
            if (k == kMatLambertian) gi = i - off[kMatLambertian];
            else if (k == kMatWard) gi = g4 + (i - off[kMatWard]);
            else if (k == kMatVolumeInside && rp.gd.volumes) gi = g6 + (i - off[kMatVolumeInside]);
            if (gi != ~0u && rp.gd.max_depth) gi = rp.gd.remap[gi];  // its inference row, or unguided
        }
        shade_slot<kGuided>(rp.reqs[r], P, k, slot, gpix, rp.gd, gi);
    }
}

// The plain and guided shading kernels: one queue item per thread, all
// queues in one launch, held to 4 resident 256-thread blocks per SM (64
// registers, a few spilled: the mixed 1080p render 1370 against 1347 Mpaths/s
// with the compiler's 78 registers and 3 blocks; the guided render 1.6 %
// faster than at 3 blocks and 80 registers).
#ifndef RGR_SHADE_MIN_BLOCKS
#define RGR_SHADE_MIN_BLOCKS 4
#endif
#ifndef RGR_SHADE_GUIDED_MIN_BLOCKS
#define RGR_SHADE_GUIDED_MIN_BLOCKS 4
#endif
__global__ void __launch_bounds__(256, RGR_SHADE_MIN_BLOCKS) k_shade(PathsView P, QueueView Q, RenderParams rp) {
    shade_items<false>(P, Q, rp);
}
__global__ void __launch_bounds__(256, RGR_SHADE_GUIDED_MIN_BLOCKS) k_shade_guided(PathsView P, QueueView Q,
                                                                                  RenderParams rp) {
    shade_items<true>(P, Q, rp);
}

// Depth-limited guiding: the guided items whose vertex is among the first
// max_depth of its path (logic_i counts the path's segments so far) become
// the inference rows, appended with one atomic per warp; the others keep
// BSDF and envmap sampling.  The row order does not matter: a row's mixture
// depends on that row alone.
__global__ void __launch_bounds__(256) k_guide_select(PathsView P, QueueView Q, GuideRenderD gd) {
    const uint32_t n = guided_items(Q, gd);
    const int lane = threadIdx.x & 31;
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t base = blockIdx.x * blockDim.x + (threadIdx.x & ~31u); base < n; base += stride) {
        const uint32_t gi = base + lane;
        uint32_t slot = 0;
        bool take = false;
        if (gi < n) {
            slot = guided_item_slot(Q, gi);
            take = depth_of(__float_as_uint(P.L[slot].w)) <= gd.max_depth;
        }
        const unsigned m = __ballot_sync(0xffffffffu, take);
        uint32_t first = 0;
        if (lane == 0 && m) first = atomicAdd(gd.nsel, (uint32_t)__popc(m));
        first = __shfl_sync(0xffffffffu, first, 0);
        if (gi < n) {
            const uint32_t row = first + (uint32_t)__popc(m & ((1u << lane) - 1u));
            gd.remap[gi] = take ? row : ~0u;
            if (take) gd.sel[row] = slot;
        }
    }
}

RGR_DEV uint32_t mix32(uint32_t h) {  // murmur3 finaliser
    h ^= h >> 16;
    h *= 0x85ebca6bu;
    h ^= h >> 13;
    h *= 0xc2b2ae35u;
    h ^= h >> 16;
    return h;
}

// A guided path ended with radiance L: its training records become samples.
// Record r holds the vertex, the sampled wi, the (L, T) of the path just after
// the vertex (its emission added, its throughput factor applied) and cos / pdf
// of wi, so the radiance that arrived along wi is L_i = (L_end - L_r) / T_r
// per channel, and the sample's weight in the KL loss is lum(L_i) cos / pdf:
// the guide learns the cosine-weighted incident radiance, which the MIS
// combines with the BSDF (the network does not see the material).
// Records are offered with the acceptance probability the last iteration set
// (a hash of slot, record and iteration, not the path's RNG, so rendering is
// unchanged) until `cap` samples are in.  guide_offer decides a lane's records;
// the logic kernel gathers the counts per block (one atomic for the block's
// samples, one for its offered count) and guide_write stores them.
struct GuideOffer {
    uint32_t take = 0;     // bit r: record r is accepted
    uint32_t offered = 0;  // records with a positive, finite weight
    float w[kGuideRecords] = {};
};
RGR_DEV void guide_offer(const GuideRenderD& gd, uint32_t slot, f3 L, bool ending, GuideOffer& o) {
    const GuideTrainD& tr = gd.train;
    const uint32_t nr = ending ? min((uint32_t)gd.nrec[slot], (uint32_t)kGuideRecords) : 0u;
    if (!nr) return;
    const float accept = *tr.accept;
    const uint32_t it = *tr.iter;
    for (uint32_t r = 0; r < (uint32_t)kGuideRecords; ++r) {
        if (r >= nr) continue;
        const float4* rec = gd.records + ((size_t)slot * kGuideRecords + r) * kGuideRecordVecs;
        float4 d, e;
        ld_v8(rec, d, e);
        const float lx = d.w > 0.0f ? (L.x - d.x) / d.w : 0.0f;
        const float ly = e.x > 0.0f ? (L.y - d.y) / e.x : 0.0f;
        const float lz = e.y > 0.0f ? (L.z - d.z) / e.y : 0.0f;
        const float wr = (0.2126f * lx + 0.7152f * ly + 0.0722f * lz) * e.z;
        if (!(wr > 0.0f) || !is_finite(wr)) continue;
        ++o.offered;
        const uint32_t h = mix32(slot * 0x9e3779b1u ^ (r + 1u) * 0x85ebca77u ^ (it + 1u) * 0xc2b2ae3du);
        if ((float)(h >> 8) * (1.0f / 16777216.0f) >= accept) continue;
        o.w[r] = wr;
        o.take |= 1u << r;
    }
}
// The accepted records of a lane as samples idx, idx + 1, ... (those below
// the cap); returns the sum of their weights.
RGR_DEV float guide_write(const GuideRenderD& gd, uint32_t slot, const GuideOffer& o, uint32_t idx) {
    const GuideTrainD& tr = gd.train;
    float wsum = 0.0f;
    for (uint32_t r = 0; r < (uint32_t)kGuideRecords; ++r) {
        if (!((o.take >> r) & 1u)) continue;
        if (idx < tr.cap) {
            const float4* rec = gd.records + ((size_t)slot * kGuideRecords + r) * kGuideRecordVecs;
            float4* dst = reinterpret_cast<float4*>(tr.samples + 16 * (size_t)idx);  // 64 bytes
            float4 x, n, wi, d;
            ld_v8(rec + 2, x, n);
            ld_v8(rec + 4, wi, d);
            st_v8(dst, x, n);                                                // x, n.x | n.yz, wo.xy
            st_v8(dst + 2, wi, make_float4(o.w[r], rec[1].w, 0.0f, 0.0f));  // wo.z, wi | weight, BSDF pdf of wi
            wsum += o.w[r];
        }
        ++idx;
    }
    return wsum;
}

// extension_ray_cast (extension_ray_cast_stackless.cl:202-246) of the slots
// this bounce shaded — the items of the seven queues, concatenated as the
// shading kernel reads them, less the new-path slots it retired — by
// persistent warps that hand finished lanes the next items (one atomic per
// refill per warp), as the closest-hit service kernel does with rays.  Runs
// between the shading kernel and the queue resets.  A hit writes the ray's
// sector once: t into P.ro.w and the primitive, as -2 - prim, into the volume-hit
// field P.rd.w (its readers take a negative id as none); the logic kernel computes
// Ng into P.ng.  A miss leaves P.ng.w at the -1 the shading stage wrote.  Each slot may belong
// to another request (scene).
#ifndef RGR_TRACE_PATHS_MIN_BLOCKS  // 4 / 5 / 6 (64 / 48 / 40 registers, 6 spilling): 1428 / 1473 / 1442 Mpaths/s
#define RGR_TRACE_PATHS_MIN_BLOCKS 5
#endif
__global__ void __launch_bounds__(256, RGR_TRACE_PATHS_MIN_BLOCKS) k_trace_paths(PathsView P, QueueView Q, RenderParams rp,
                                                         unsigned long long* next, int refill, int search) {
    const unsigned full = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const unsigned lt = (1u << lane) - 1u;
    const uint64_t pol = l2_evict_last_policy();
    uint32_t off[kNumQueues + 1];
    off[0] = 0;
#pragma unroll
    for (int k = 0; k < kNumQueues; ++k) off[k + 1] = off[k] + Q.counts[k];
    const uint32_t total = off[kNumQueues];
    __shared__ uint32_t s_stack[kSmemStack > 0 ? kSmemStack * kStackThreads : 1];
    TraceState s;
    s.sstk = s_stack + threadIdx.x;
    const SceneView* scp = &rp.reqs[0].sc;  // a valid scene on idle lanes too
    uint32_t slot = ~0u;  // ~0: idle
    bool exhausted = false;
    uint32_t err = 0;
    for (;;) {
        const unsigned idle = __ballot_sync(full, slot == ~0u);
        if (!exhausted && (int)__popc(idle) >= refill) {
            const uint32_t need = __popc(idle);
            unsigned long long base = 0;
            if (lane == 0) base = atomicAdd(next, (unsigned long long)need);
            base = __shfl_sync(full, base, 0);
            if (base + need >= total) exhausted = true;
            if (slot == ~0u) {
                const unsigned long long i = base + __popc(idle & lt);
                if (i < total) {
                    int k = 0;
#pragma unroll
                    for (int j = 1; j < kNumQueues; ++j) k += ((uint32_t)i >= off[j]) ? 1 : 0;
                    const uint32_t r = queue_items(Q, k)[(uint32_t)i - pick(off, k)];
                    // only a new-path item can have retired (sample budget reached in
                    // the shading kernel): material-queue items skip the check
                    if (k != 0 || P.qid[r] != kQueueIdle) {
                        slot = r;
                        scp = &rp.reqs[P.req[r]].sc;
                        float4 ro4, rd4;
                        ld_sector<0>(P, r, ro4, rd4);
                        trace_begin(*scp, s, xyz(ro4), xyz(rd4), ro4.w);
                    }
                }
            }
        }
        if (__ballot_sync(full, slot != ~0u) == 0u) {
            if (exhausted) break;
            continue;
        }
        trace_warp_round<false, false, kSmemStack>(*scp, s, slot != ~0u && s.link != kDone, search, nullptr, err,
                                                   pol);
        if (slot != ~0u && s.link == kDone) {
            if (s.prim >= 0) {
                // the ray's whole sector in one store (a partial store to a line that is
                // not in L2 costs a read of the sector from DRAM); the hit primitive
                // rides where the volume-hit id goes (none after a surface hit: every
                // reader takes a negative id as none), and the logic kernel, which
                // writes the (ng, rng) sector anyway, computes the normal
                st_sector<0>(P, slot, f4(s.ro, s.tmin), f4(s.rd, __int_as_float(-2 - s.prim)));
            }
            slot = ~0u;
        }
    }
    if (err) atomicOr(rp.err, err);
}

// The logic of one live slot (logic.cl:27-190) after its extension ray;
// returns the queue of its next step (0: a new path, counted per tile here;
// a material queue: appended by the caller).  kPreTraced: k_trace_paths has
// cast the extension rays of this bounce; otherwise the thread traces first.
template <bool kGuided, bool kPreTraced>
RGR_DEV int logic_slot(const PathsView& P, const QueueView& Q, const RenderParams& rp, uint32_t slot,
                       unsigned active, GuideOffer& go) {
    const int req = P.req[slot];
    const RequestD& rq = rp.reqs[req];
    const SceneView& sc = rq.sc;
    float4 ro4, rd4, ng4, rng4, T4, L4;
    ld_sector<0>(P, slot, ro4, rd4);
    if (kPreTraced) {  // the trace kernel wrote the hit; else loaded after the traversal
        ld_sector<1>(P, slot, T4, L4);
        ld_sector<2>(P, slot, ng4, rng4);
    }
    f3 rd = xyz(rd4);
    int32_t hv = __float_as_int(rd4.w);
    uint32_t err = 0;
    int32_t hs;
    int mtype = -1;  // the hit triangle's material type, where the triangle table gave it
    if (kPreTraced) {
        hs = __float_as_int(ng4.w);
        if (hv <= -2) {  // k_trace_paths found primitive -2 - hv
            hs = -2 - hv;
            hv = -1;
            if (sc.tri_normals && hs < sc.sphere_begin) {
                const float4 tn = __ldg(sc.tri_normals + hs);
                ng4 = f4(xyz(tn), __int_as_float(hs));
                mtype = __float_as_int(tn.w);
            } else {
                ng4 = f4(hit_normal(sc, hs, xyz(ro4), rd, ro4.w), __int_as_float(hs));
            }
        }
    } else {
        // extension_ray_cast (extension_ray_cast_stackless.cl:202-246)
        f3 ro = xyz(ro4);
        float tmin = ro4.w;
        hs = trace_closest<false>(sc, ro, rd, tmin, nullptr, err);
        ld_sector<1>(P, slot, T4, L4);
        ld_sector<2>(P, slot, ng4, rng4);
        if (hs >= 0) {
            ng4 = f4(hit_normal(sc, hs, ro, rd, tmin), __int_as_float(hs));
            hv = -1;
            st_sector<0>(P, slot, f4(ro, tmin), f4(rd, __int_as_float(-1)));
        }
    }
    // logic (logic.cl:27-190)
    f3 T = xyz(T4), L = xyz(L4);
    const uint32_t lw = __float_as_uint(L4.w);  // segment count and volume count
    uint32_t logic_i = depth_of(lw);
    Rng rng = rng_of_bits(rng4);
    bool evalEnv = false, newPath = false;
    if (hs < 0 && hv < 0) {
        newPath = true;
        evalEnv = true;
    }
    float lum = 0.2126f * T.x + 0.7152f * T.y + 0.0722f * T.z;
    float cp = 1.0f;
    if ((long long)rq.rr_depth < (long long)logic_i) cp = fmin_(lum, 1.0f);
    float u = rng.uniform();
    if (u < cp) {
        T = T / cp;
    } else {
        newPath = true;
    }
    if (lum < 1.0e-5f) newPath = true;
    if (evalEnv && sc.has_env) L = L + T * envmap_value(sc, rd, logic_i == 0);
    // depth limit: end after segment max_depth, adding the emission that the
    // next material stage would add (lambertian.cl:395)
    if (rq.max_depth > 0 && !newPath && (long long)logic_i >= (long long)rq.max_depth) {
        if (0 <= hs) {
            int2 m = __ldg(sc.materials + hs);
            f3 Le = mk(0, 0, 0);
            if (m.x == kMatLambertian) Le = xyz(__ldg(sc.lambertians + 2 * (size_t)m.y));
            L = L + T * Le;
        }
        newPath = true;
    }
    if (newPath) {
        const float cl = rq.radiance_clamp;
        if (is_finite(L.x) && is_finite(L.y) && is_finite(L.z) && L.x < cl && L.y < cl && L.z < cl) {
            double* a = rq.accum + 4 * (size_t)__float_as_uint(T4.w);
            atomicAdd(a + 0, (double)L.x);
            atomicAdd(a + 1, (double)L.y);
            atomicAdd(a + 2, (double)L.z);
            atomicAdd(a + 3, 1.0);
        }
    }
    // No samples once the sample budget is handed out: the paths still in
    // flight are the long ones, and a few iterations on that subset alone
    // undo much of what the guide learned (the same for every thread).
    if (kGuided && rp.gd.record && guide_training_open(rp.gd.train) &&
        !(rp.sample_limit != 0ull && *Q.next_pixel >= rp.sample_limit)) {
        const float cl = rq.radiance_clamp;
        const bool kept = is_finite(L.x) && is_finite(L.y) && is_finite(L.z) && L.x < cl && L.y < cl && L.z < cl;
        guide_offer(rp.gd, slot, L, newPath && kept, go);
    }
    st_sector<1>(P, slot, f4(T, T4.w), f4(L, __uint_as_float(depth_word(logic_i + 1, vcount_of(lw)))));
    st_sector<2>(P, slot, ng4, rng_bits(rng));
    int q;
    if (newPath) {
        q = 0;
    } else if (0 <= hs) {
        q = mtype >= 0 ? mtype : __ldg(sc.materials + hs).x;
    } else {
        q = kMatVolumeInside;
    }
    P.qid[slot] = (uint8_t)q;
    {
        // new paths: count per tile for the ordered compaction
        const unsigned newmask = __ballot_sync(active, q == 0);
        if (q == 0) {
            unsigned tp = __match_any_sync(newmask, (int)(slot / kTile));
            int leader = __ffs(tp) - 1;
            if ((int)(threadIdx.x & 31) == leader) atomicAdd(Q.tile_new + slot / kTile, (uint32_t)__popc(tp));
        }
    }
    {
        int lane = threadIdx.x & 31;
        if (err) atomicOr(rp.err, err);
        // finished paths per request (k_stamp_done stamps the completion times)
        const unsigned donemask = __ballot_sync(active, newPath);
        if (newPath && rq.done != nullptr) {
            unsigned peers = __match_any_sync(donemask, req);
            if (lane == __ffs(peers) - 1) {
                atomicAdd(rq.done, (unsigned long long)__popc(peers));
            }
        }
    }
    return q;
}

// The logic kernel, one thread per slot.  Material-queue appends are gathered
// per block (shared-memory counts, then one global atomic per queue), and so
// is the ray count: with one atomic per warp all warps of the launch queued on
// the same few counters.
constexpr int kLogicThreads = 256;
template <bool kGuided, bool kPreTraced>
// latency-bound: 6 resident blocks per SM for the logic alone (40 registers; the
// render 0.6 % faster than at 5), 5 while it records guide samples, 4 with the
// traversal fused in
#ifndef RGR_LOGIC_MIN_BLOCKS  // the plain pre-traced logic: 5 / 6 / 7 give 1464 / 1472 / 1436 Mpaths/s
#define RGR_LOGIC_MIN_BLOCKS 6
#endif
__global__ void __launch_bounds__(kLogicThreads, kPreTraced ? (kGuided ? 5 : RGR_LOGIC_MIN_BLOCKS) : 4) k_trace_logic(PathsView P, QueueView Q, RenderParams rp) {
    const unsigned full = 0xffffffffu;
    __shared__ uint32_t s_q[kNumQueues];  // items per queue, then the block's base in it
    __shared__ uint32_t s_samples, s_offered;  // guided recording: accepted samples (then their base), offered
    if (threadIdx.x < kNumQueues) s_q[threadIdx.x] = 0;
    if (kGuided && threadIdx.x == 32) s_samples = s_offered = 0u;
    const int lane = threadIdx.x & 31;
    const unsigned lt = (1u << lane) - 1u;
    const uint32_t slot = blockIdx.x * blockDim.x + threadIdx.x;
    const bool live = slot < P.n && P.qid[slot] != kQueueIdle;
    const unsigned active = __ballot_sync(full, live);
    int q = 0;
    GuideOffer go;
    if (live) q = logic_slot<kGuided, kPreTraced>(P, Q, rp, slot, active, go);
    const bool mat = live && q != 0;
    const unsigned matmask = __ballot_sync(full, mat);
    __syncthreads();  // s_q, s_samples, s_offered cleared
    uint32_t off = 0;
    if (mat) {
        const unsigned peers = __match_any_sync(matmask, q);
        const int leader = __ffs(peers) - 1;
        uint32_t base = 0;
        if (lane == leader) base = atomicAdd(&s_q[q], (uint32_t)__popc(peers));
        off = __shfl_sync(peers, base, leader) + __popc(peers & lt);
    }
    uint32_t sidx = 0;  // this lane's first sample within the block's
    if (kGuided) {
        // exclusive prefix of the accepted counts (0..3: two ballots)
        const uint32_t mine = __popc(go.take);
        const unsigned b0 = __ballot_sync(full, mine & 1u), b1 = __ballot_sync(full, (mine >> 1) & 1u);
        const uint32_t wtot = __popc(b0) + 2u * __popc(b1);
        const uint32_t offered = __reduce_add_sync(full, go.offered);
        uint32_t wbase = 0;
        if (lane == 0 && wtot) wbase = atomicAdd(&s_samples, wtot);
        if (lane == 0 && offered) atomicAdd(&s_offered, offered);
        sidx = __shfl_sync(full, wbase, 0) + __popc(b0 & lt) + 2u * __popc(b1 & lt);
    }
    const int nlive = __syncthreads_count(live);
    if (threadIdx.x < kNumQueues) {
        const uint32_t n = s_q[threadIdx.x];
        if (n) s_q[threadIdx.x] = atomicAdd(Q.counts + threadIdx.x, n);
    }
    if (kGuided && threadIdx.x == 32) {
        if (s_samples) s_samples = atomicAdd(rp.gd.train.count, s_samples);
        if (s_offered) atomicAdd(rp.gd.train.candidates, (unsigned long long)s_offered);
    }
    if (threadIdx.x == 0 && nlive) atomicAdd(rp.rays, (unsigned long long)nlive);
    __syncthreads();
    if (mat) queue_items(Q, q)[s_q[q] + off] = slot;
    if (kGuided && __any_sync(full, go.take != 0u)) {
        float ws = go.take ? guide_write(rp.gd, slot, go, s_samples + sidx) : 0.0f;
        for (int o = 16; o > 0; o >>= 1) ws += __shfl_xor_sync(full, ws, o);
        if (lane == 0 && ws > 0.0f) atomicAdd(rp.gd.train.wsum, ws);
    }
}

// The completion time of each request whose paths have all finished, stamped
// once by the bounce in which its last path ended (after that bounce's logic
// kernel, when its accumulation is complete).  The logic kernel only counts
// finished paths: an atomic with a returned value per warp, to find the last
// one, queued the warps on the requests' counters.
__global__ void k_stamp_done(RenderParams rp) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= rp.nreq) return;
    const RequestD& q = rp.reqs[r];
    if (q.done == nullptr || *q.done_ns != 0ull || *q.done != q.sample_end - q.sample_begin) return;
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    *q.done_ns = t;
}

// RGB16 intermediate (accumlation.cl:6-25) from FP64 sums: mean in double,
// rounded to float, then to half; count to 16 bits.
__global__ void k_readback(int fmt, const double* accum, uint32_t npix, void* out) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= npix) return;
    const double* a = accum + 4 * (size_t)i;
    double cnt = a[3];
    unsigned short h[3];
    for (int k = 0; k < 3; ++k) {
        float m = cnt > 0.0 ? (float)(a[k] / cnt) : 0.0f;
        h[k] = __half_as_ushort(__float2half_rn(m));
    }
    if (fmt == 1) {
        ushort4 v = make_ushort4(h[0], h[1], h[2], (unsigned short)((unsigned long long)cnt & 0xffffull));
        reinterpret_cast<ushort4*>(out)[i] = v;
        return;
    }
    // tonemap (accumlation.cl:68-79)
    uchar4 px;
    unsigned char c[3];
    for (int k = 0; k < 3; ++k) {
        float v = __half2float(__ushort_as_half(h[k]));
        int iv = to_int(pow_(v * 1.0f, 1.0f / 2.2f) * 256.0f);
        iv = min(max(iv, 0), 255);
        c[k] = (unsigned char)iv;
    }
    px.x = c[0];
    px.y = c[1];
    px.z = c[2];
    px.w = 255;
    reinterpret_cast<uchar4*>(out)[i] = px;
}

// stat (stat.cl:6-39): total accumulated samples
__global__ void k_sum_counts(const double* accum, uint32_t npix, unsigned long long* out) {
    unsigned long long s = 0;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < npix; i += gridDim.x * blockDim.x)
        s += (unsigned long long)accum[4 * (size_t)i + 3];
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) atomicAdd(out, s);
}

// merge_intermediate (accumlation.cl:27-49): count-weighted merge of two RGB16
// intermediates in FP32, result stored as half into a
__global__ void k_merge_intermediate(ushort4* a, const ushort4* b, uint32_t n) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    ushort4 va = a[i], vb = b[i];
    const unsigned short sa = va.w, sb = vb.w;
    const unsigned short sab = (unsigned short)(sa + sb);
    if (sab == 0) {
        a[i] = make_ushort4(0, 0, 0, 0);
        return;
    }
    const float one_over_sab = 1.0f / (float)sab;
    const unsigned short ha[3] = {va.x, va.y, va.z}, hb[3] = {vb.x, vb.y, vb.z};
    unsigned short out[3];
    for (int k = 0; k < 3; ++k) {
        float m = (__half2float(__ushort_as_half(ha[k])) * (float)sa + __half2float(__ushort_as_half(hb[k])) * (float)sb) *
                  one_over_sab;
        out[k] = __half_as_ushort(__float2half_rn(m));
    }
    a[i] = make_ushort4(out[0], out[1], out[2], sab);
}

__global__ void k_accum_add(double* dst, const double* src, uint32_t n4) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n4) dst[i] += src[i];
}

__global__ void k_debug_slots(PathsView P, uint32_t* out) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P.n) return;
    uint32_t* o = out + 34 * (size_t)i;
    float4 T = P.T[i], L = P.L[i], ro = P.ro[i], rd = P.rd[i], ng = P.ng[i];
    uint4 r = P.rng[i];
    int4 va = P.va[i], vb = P.vb[i];
    const float f[12] = {T.x, T.y, T.z, L.x, L.y, L.z, ro.x, ro.y, ro.z, rd.x, rd.y, rd.z};
    for (int k = 0; k < 12; ++k) o[k] = __float_as_uint(f[k]);
    o[12] = depth_of(__float_as_uint(L.w));
    o[13] = __float_as_uint(T.w);
    o[14] = r.x;
    o[15] = r.y;
    o[16] = r.z;
    o[17] = r.w;
    o[18] = __float_as_uint(ng.w);
    o[19] = __float_as_int(rd.w) < -1 ? 0xffffffffu : __float_as_uint(rd.w);  // no volume hit: -1
    o[20] = __float_as_uint(ro.w);
    o[21] = __float_as_uint(ng.x);
    o[22] = __float_as_uint(ng.y);
    o[23] = __float_as_uint(ng.z);
    uint8_t q = P.qid[i];
    o[24] = q == kQueueIdle ? 0xffffffffu : (uint32_t)q;
    o[25] = (uint32_t)vcount_of(__float_as_uint(L.w));
    const int v[7] = {va.x, va.y, va.z, va.w, vb.x, vb.y, vb.z};
    for (int k = 0; k < 7; ++k) o[26 + k] = (uint32_t)v[k];
    o[33] = 0;
}

}  // namespace

void launch_init(const PathsView& p, const QueueView& q, uint32_t seed_offset, cudaStream_t st) {
    uint32_t n = q.ntiles * kTile;
    k_init<<<(n + 255) / 256, 256, 0, st>>>(p, q, seed_offset);
}
void launch_compact_new(const PathsView& p, const QueueView& q, cudaStream_t st) {
    k_compact_new<<<q.ntiles, 256, 0, st>>>(p, q);
}
void launch_guide_select(const PathsView& p, const QueueView& q, const GuideRenderD& gd, int grid, cudaStream_t st) {
    cudaMemsetAsync(gd.nsel, 0, sizeof(uint32_t), st);
    k_guide_select<<<grid, 256, 0, st>>>(p, q, gd);
}

void launch_shade(const PathsView& p, const QueueView& q, const RenderParams& rp, int grid, cudaStream_t st) {
    if (rp.gd.lobes)
        k_shade_guided<<<grid, 256, 0, st>>>(p, q, rp);
    else
        k_shade<<<grid, 256, 0, st>>>(p, q, rp);
}
cudaError_t launch_trace_paths(const PathsView& p, const QueueView& q, const RenderParams& rp, const TraceShape& ts,
                               cudaStream_t st) {
    if (!ts.persistent) return cudaSuccess;
    const cudaError_t e = cudaMemsetAsync(ts.counter, 0, sizeof(unsigned long long), st);
    if (e != cudaSuccess) return e;
    k_trace_paths<<<ts.grid, kStackThreads, 0, st>>>(p, q, rp, ts.counter, ts.refill, ts.search);
    return cudaSuccess;
}

void launch_trace_logic(const PathsView& p, const QueueView& q, const RenderParams& rp, const TraceShape& ts,
                        cudaStream_t st) {
    const unsigned nb = (p.n + kLogicThreads - 1) / kLogicThreads;
    // the guided variant differs only in recording training samples: a render
    // with a frozen guide runs the plain one (fewer registers)
    const bool recording = rp.gd.lobes && rp.gd.record;
    if (ts.persistent) {
        if (recording)
            k_trace_logic<true, true><<<nb, kLogicThreads, 0, st>>>(p, q, rp);
        else
            k_trace_logic<false, true><<<nb, kLogicThreads, 0, st>>>(p, q, rp);
    } else if (recording) {
        k_trace_logic<true, false><<<nb, kLogicThreads, 0, st>>>(p, q, rp);
    } else {
        k_trace_logic<false, false><<<nb, kLogicThreads, 0, st>>>(p, q, rp);
    }
}

void launch_stamp_done(const RenderParams& rp, cudaStream_t st) {
    if (rp.nreq > 0) k_stamp_done<<<(rp.nreq + 127) / 128, 128, 0, st>>>(rp);
}

int trace_paths_max_blocks_per_sm() {
    int nb = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_trace_paths, 256, 0);
    return nb;
}
void launch_readback(int fmt, const double* accum, uint32_t npix, void* out, cudaStream_t st) {
    k_readback<<<(npix + 255) / 256, 256, 0, st>>>(fmt, accum, npix, out);
}
void launch_sum_counts(const double* accum, uint32_t npix, unsigned long long* out, cudaStream_t st) {
    k_sum_counts<<<152 * 4, 256, 0, st>>>(accum, npix, out);
}
void launch_debug_slots(const PathsView& p, uint32_t* out, cudaStream_t st) {
    k_debug_slots<<<(p.n + 255) / 256, 256, 0, st>>>(p, out);
}
void launch_merge_intermediate(void* a, const void* b, uint32_t n, cudaStream_t st) {
    k_merge_intermediate<<<(n + 255) / 256, 256, 0, st>>>(reinterpret_cast<ushort4*>(a),
                                                          reinterpret_cast<const ushort4*>(b), n);
}
void launch_accum_add(double* dst, const double* src, uint32_t npix, cudaStream_t st) {
    uint32_t n4 = npix * 4;
    k_accum_add<<<(n4 + 255) / 256, 256, 0, st>>>(dst, src, n4);
}

}  // namespace dev
}  // namespace rgr
