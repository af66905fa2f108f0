// envmap_tables.cpp — importance-sampling tables of an equirectangular envmap.
//
// Follows rt::ImageEnvmap's constructor (common/share/envmap.hpp:160-242) and
// rt::AliasMethod<double>::prepare (common/share/alias_method.hpp:47-114):
// per-texel selection weight = luminance (FP32, 0.2126/0.7152/0.0722) x texel
// solid angle x direction weight, Kahan-summed in FP64, alias pairing with the
// reference's two stacks, pdf = probability / solid angle.  Seven tables are
// built: the uniform one (UniformDirectionWeight) and one per cube axis
// (SixAxisDirectionWeight, envmap.hpp:291-312), as SceneManager::addPoint does
// (scene_manager.hpp:475-493).  Tables are built on host threads in FP64.
#include "../rgr_internal.h"

#include <algorithm>
#include <cmath>
#include <thread>

namespace rgr {
namespace {

constexpr double kTwoPi = 6.28318530717958647692;
constexpr double kPi = 3.14159265358979323846;

struct KahanD {  // alias_method.hpp:8-40
    double sum = 0.0, c = 0.0;
    void add(double x) {
        double y = x - c;
        double t = sum + y;
        c = (t - sum) - y;
        sum = t;
    }
    double get() const { return sum - c; }
};

void build_table(const EnvTables& env, int kind, const std::vector<double>& frag, const std::vector<double>& sr,
                 float* pdf, float* height, int32_t* alias) {
    const int w = env.w, h = env.h, n = w * h;
    std::vector<double> weight(n);
    for (int y = 0; y < h; ++y) {
        const double* f0 = &frag[4 * (size_t)y * w];
        double theta = (std::acos(f0[0]) + std::acos(f0[1])) * 0.5;
        double st = std::sin(theta), ct = std::cos(theta);
        for (int x = 0; x < w; ++x) {
            int i = y * w + x;
            double phi = (frag[4 * (size_t)i + 2] + frag[4 * (size_t)i + 3]) * 0.5;
            // polar_to_cartesian returns (sin t sin p, cos t, sin t cos p), envmap.hpp:79-86
            double d[3] = {st * std::sin(phi), ct, st * std::cos(phi)};
            const float* px = &env.rgba[4 * (size_t)i];
            float lum = 0.2126f * px[0] + 0.7152f * px[1] + 0.0722f * px[2];
            double dw = 1.0;
            if (kind > 0) {
                int axis = (kind - 1) / 2;
                double v = ((kind - 1) % 2 == 0) ? d[axis] : -d[axis];
                dw = std::max(v, 0.0);
            }
            weight[i] = (double)lum * sr[y] * dw;
        }
    }
    KahanD total;
    for (double v : weight) total.add(v);
    double inv = 1.0 / total.get();
    std::vector<double> prob(n);
    for (int i = 0; i < n; ++i) prob[i] = weight[i] * inv;
    alias_from_probabilities(w, h, prob.data(), sr, pdf, height, alias);
}

}  // namespace

// AliasMethod::prepare (alias_method.hpp:47-114) from normalised probabilities:
// heights prob * n with Kahan compensation, the reference's two stacks, and the
// pdf per solid angle.
void alias_from_probabilities(int w, int h, const double* prob, const std::vector<double>& sr, float* pdf,
                              float* height, int32_t* alias) {
    const int n = w * h;
    std::vector<KahanD> hk(n);
    std::vector<int32_t> al(n, -1);
    std::vector<int> lower, upper;
    lower.reserve(n);
    upper.reserve(n);
    for (int i = 0; i < n; ++i) {
        hk[i].sum = prob[i] * n;
        hk[i].c = 0.0;
        if (hk[i].get() < 1.0) lower.push_back(i);
        else upper.push_back(i);
    }
    while (!lower.empty() && !upper.empty()) {
        int lo = lower.back();
        lower.pop_back();
        int up = upper.back();
        upper.pop_back();
        double mov = 1.0 - hk[lo].get();
        hk[up].add(-mov);
        al[lo] = up;
        if (hk[up].get() < 1.0) lower.push_back(up);
        else upper.push_back(up);
    }
    for (int y = 0; y < h; ++y) {
        double inv_sr = 1.0 / sr[y];
        for (int x = 0; x < w; ++x) {
            int i = y * w + x;
            pdf[i] = (float)(prob[i] * inv_sr);
            height[i] = (float)hk[i].get();
            alias[i] = al[i];
        }
    }
}

namespace {
// fragments and per-row solid angles (EnvmapCoordinateSystem, envmap.hpp:34-78)
void envmap_geometry(int w, int h, std::vector<double>& frag, std::vector<double>& sr) {
    const size_t n = (size_t)w * h;
    frag.resize(4 * n);
    sr.resize(h);
    const double phi_step = kTwoPi / w, theta_step = kPi / h;
    for (int y = 0; y < h; ++y) {
        double t0 = theta_step * y, t1 = theta_step * (y + 1);
        double beg_y = std::cos(t1), end_y = std::cos(t0);
        for (int x = 0; x < w; ++x) {
            double* f = &frag[4 * ((size_t)y * w + x)];
            f[0] = beg_y;
            f[1] = end_y;
            f[2] = kTwoPi - (x + 1) * phi_step;
            f[3] = kTwoPi - x * phi_step;
        }
        sr[y] = ((std::cos(t0) - std::cos(t1)) * kTwoPi) / w;
    }
}
}  // namespace

int build_envmap_tables(EnvTables& env) {
    const int w = env.w, h = env.h;
    const size_t n = (size_t)w * h;
    std::vector<double> frag, sr;
    envmap_geometry(w, h, frag, sr);
    env.frag.resize(4 * n);
    for (size_t i = 0; i < 4 * n; ++i) env.frag[i] = (float)frag[i];
    env.pdf.assign(7 * n, 0.0f);
    env.height.assign(7 * n, 0.0f);
    env.alias.assign(7 * n, -1);
    std::vector<std::thread> th;
    for (int k = 0; k < 7; ++k)
        th.emplace_back(build_table, std::cref(env), k, std::cref(frag), std::cref(sr), env.pdf.data() + k * n,
                        env.height.data() + k * n, env.alias.data() + k * n);
    for (auto& t : th) t.join();
    return RGR_OK;
}

// The same tables with the selection weights and their FP64 normalisation
// computed on the GPU (envmap_gpu.cu); the alias pairing, which is sequential,
// stays on the host.
int build_envmap_tables_gpu(EnvTables& env, int device) {
    const int w = env.w, h = env.h;
    const size_t n = (size_t)w * h;
    std::vector<double> frag, sr;
    envmap_geometry(w, h, frag, sr);
    env.frag.resize(4 * n);
    for (size_t i = 0; i < 4 * n; ++i) env.frag[i] = (float)frag[i];
    std::vector<double> prob(7 * n);
    int r = envmap_probabilities_gpu(device, env.rgba.data(), w, h, prob.data());
    if (r != RGR_OK) return r;
    env.pdf.assign(7 * n, 0.0f);
    env.height.assign(7 * n, 0.0f);
    env.alias.assign(7 * n, -1);
    std::vector<std::thread> th;
    for (int k = 0; k < 7; ++k)
        th.emplace_back(alias_from_probabilities, w, h, prob.data() + k * n, std::cref(sr), env.pdf.data() + k * n,
                        env.height.data() + k * n, env.alias.data() + k * n);
    for (auto& t : th) t.join();
    return RGR_OK;
}

}  // namespace rgr
