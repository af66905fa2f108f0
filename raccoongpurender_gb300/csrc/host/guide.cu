// guide.cu — the C ABI of the path-guiding network: creation and weight
// initialisation, weights in and out, inference and training entry points,
// and the per-bounce training launches of a guided render.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "guide_host.h"
#include "nvtx.h"

using namespace rgr;
using namespace rgr::dev;

namespace {

// counters buffer layout (bytes)
constexpr size_t kCtrCount = 0, kCtrWsum = 4, kCtrCand = 8, kCtrAccept = 16, kCtrIter = 20, kCtrLast = 24;
constexpr size_t kCtrTest = 32;  // the test stream's count/wsum/cand/accept at the same offsets from here
constexpr size_t kCtrErr = 60;   // error bits of the tensor-core kernels
constexpr size_t kCtrBytes = 64;

uint64_t splitmix64(uint64_t& x) {
    uint64_t z = (x += 0x9e3779b97f4a7c15ull);
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    return z ^ (z >> 31);
}

// round-to-nearest-even FP32 -> BF16 (inputs are finite)
uint16_t to_bf16(float f) {
    uint32_t u;
    memcpy(&u, &f, 4);
    u += 0x7fffu + ((u >> 16) & 1u);
    return (uint16_t)(u >> 16);
}

// The network's real shape inside the zero-padded 64 x 64 layers.
int fan_in(int l) { return l == 0 ? kGuideInputs : kGuideWidth; }
int fan_out(int l) { return l == kGuideLayers - 1 ? kGuideNetOutputs : kGuideWidth; }
// samples an online iteration waits for before it trains: 1/16 of the batch
uint32_t min_batch(const rgr_guide_config& c) { return std::max<uint32_t>(1u, c.batch_samples / 16u); }

// the training grid for n samples on the host-side entry points: the mma.sync
// kernel takes 64-sample chunks, the tcgen05 one 128-sample tiles two at a time,
// at most one CTA per SM
int train_grid(const rgr_guide& g, uint32_t n) {
    const uint32_t per_cta = g.cfg.training_kernel == RGR_GUIDE_TCGEN05 ? 256u : 64u;
    return (int)std::min<uint32_t>(std::max<uint32_t>((n + per_cta - 1) / per_cta, 1u), (uint32_t)g.num_sms);
}

bool check_padding(const float* w, const float* b) {
    for (int l = 0; l < kGuideLayers; ++l)
        for (int i = 0; i < kGuideWidth; ++i)
            for (int o = 0; o < kGuideWidth; ++o) {
                const float v = w[(l * kGuideWidth + i) * kGuideWidth + o];
                if (!std::isfinite(v)) return false;
                if ((i >= fan_in(l) || o >= fan_out(l)) && v != 0.0f) return false;
            }
    for (int l = 0; l < kGuideLayers; ++l)
        for (int o = 0; o < kGuideWidth; ++o) {
            const float v = b[l * kGuideWidth + o];
            if (!std::isfinite(v) || (o >= fan_out(l) && v != 0.0f)) return false;
        }
    return true;
}

}  // namespace

int rgr_guide::init(const rgr_guide_config& c) {
    cfg = c;
    int r;
#define AL(buf, bytes) \
    if ((r = buf.alloc(bytes)) != RGR_OK) return r;
    AL(w, 4 * kGuideWeights);
    AL(b, 4 * kGuideBiases);
    AL(wbf, 2 * kGuideWeights);
    AL(gW, 4 * kGuideWeights);
    AL(gb, 4 * kGuideBiases);
    AL(m, 4 * kGuideParams);
    AL(v, 4 * kGuideParams);
    AL(loss, 16);
    AL(samples, 64 * (size_t)cfg.batch_samples);
    AL(counters, kCtrBytes);
    AL(loss_hist, 4 * kLossHist);
    AL(wtsw, kGuideWtBytes);
    AL(gpart, 4 * (size_t)kGuidePartStride * (size_t)num_sms);
#undef AL
    GuideView& g = view;
    g.w = w.as<float>();
    g.b = b.as<float>();
    g.wbf = wbf.as<__nv_bfloat16>();
    g.gW = gW.as<float>();
    g.gb = gb.as<float>();
    g.m = m.as<float>();
    g.v = v.as<float>();
    g.loss = loss.as<float>();
    g.wt_sw = wtsw.as<unsigned char>();
    for (int k = 0; k < 3; ++k) {
        g.params.lo[k] = -1.0f;
        g.params.inv_ext[k] = 0.5f;
    }
    unsigned char* ctr = counters.as<unsigned char>();
    auto stream_at = [&](size_t base, GuideTrainD& t) {
        t.samples = samples.as<float>();
        t.cap = cfg.batch_samples;
        t.count = reinterpret_cast<uint32_t*>(ctr + base + kCtrCount);
        t.wsum = reinterpret_cast<float*>(ctr + base + kCtrWsum);
        t.candidates = reinterpret_cast<unsigned long long*>(ctr + base + kCtrCand);
        t.accept = reinterpret_cast<float*>(ctr + base + kCtrAccept);
        t.iter = reinterpret_cast<uint32_t*>(ctr + kCtrIter);
        t.last = reinterpret_cast<uint32_t*>(ctr + base + kCtrLast);
        t.loss_hist = loss_hist.as<float>();
        t.max_iter = 0;
        t.min_count = 0;
    };
    stream_at(0, train);
    stream_at(kCtrTest, test);
    train.max_iter = cfg.max_iterations;
    train.min_count = min_batch(cfg);
    // He-uniform initialisation of the real part of each layer (the output layer
    // scaled by 1/4 so that the first mixtures are broad), zero biases and padding;
    // the selection logit's column starts at zero (the guide's share starts at
    // 0.5 everywhere)
    std::vector<float> hw(kGuideWeights, 0.0f), hb(kGuideBiases, 0.0f);
    uint64_t s = cfg.seed;
    for (int l = 0; l < kGuideLayers; ++l) {
        const float lim = std::sqrt(6.0f / (float)fan_in(l)) * (l == kGuideLayers - 1 ? 0.25f : 1.0f);
        for (int i = 0; i < fan_in(l); ++i)
            for (int o = 0; o < (l == kGuideLayers - 1 ? kGuideOutputs : fan_out(l)); ++o) {
                const double u = (double)(splitmix64(s) >> 11) * (1.0 / 9007199254740992.0);
                hw[(l * kGuideWidth + i) * kGuideWidth + o] = (float)((2.0 * u - 1.0) * lim);
            }
    }
    return rgr_guide_set_weights(this, hw.data(), hb.data());
}

int rgr_guide::set_bounds(const float lo[3], const float hi[3]) {
    for (int k = 0; k < 3; ++k) {
        if (!std::isfinite(lo[k]) || !std::isfinite(hi[k]) || !(hi[k] > lo[k])) return RGR_E_INVALID;
        view.params.lo[k] = lo[k];
        view.params.inv_ext[k] = 1.0f / (hi[k] - lo[k]);
    }
    bounds_set = true;
    return RGR_OK;
}

uint32_t* rgr_guide::error_word() const { return reinterpret_cast<uint32_t*>(counters.as<unsigned char>() + kCtrErr); }

void rgr_guide::infer_paths(const PathsView& p, const QueueView& q, const GuideRenderD& gd, cudaStream_t st) {
    if (cfg.inference_kernel == RGR_GUIDE_TCGEN05)
        launch_guide_infer_paths_tc(view, p, q, gd, guide_tc_grid(num_sms), error_word(), st);
    else
        launch_guide_infer_paths(view, p, q, gd, guide_infer_grid(num_sms), st);
}

void rgr_guide::gradient_launches(const float* smp, const uint32_t* count, uint32_t cap, uint32_t min_count,
                                  const float* wsum, float weight_scale, int grid, cudaStream_t st) {
    if (cfg.training_kernel == RGR_GUIDE_TCGEN05) {
        launch_guide_train_tc(view, smp, count, cap, min_count, wsum, weight_scale, grid, gpart.as<float>(),
                              error_word(), st);
        launch_guide_grad_reduce(view, gpart.as<float>(), (uint32_t)grid, count, min_count, st);
    } else {
        launch_guide_train(view, smp, count, cap, min_count, wsum, weight_scale, grid, st);
    }
}

int rgr_guide::train_launches(cudaStream_t st) {
    if (cfg.train) {
        gradient_launches(train.samples, train.count, train.cap, train.min_count, train.wsum, 1.0f, num_sms, st);
        launch_guide_adam(view, train.count, train.min_count, train.iter, cfg.learning_rate, cfg.beta1, cfg.beta2,
                          cfg.epsilon, st);
    }
    launch_guide_finish(view, train, st);
    RGR_CUDA(cudaGetLastError());
    return RGR_OK;
}

extern "C" {

void rgr_guide_config_default(rgr_guide_config* c) {
    if (!c) return;
    c->learning_rate = 1.0e-3f;
    c->beta1 = 0.9f;
    c->beta2 = 0.999f;
    c->epsilon = 1.0e-8f;
    c->batch_samples = 1u << 18;
    c->guide_fraction = 0.5f;
    c->train = 1;
    c->guide_volumes = 0;
    c->train_interval = 1;
    c->max_iterations = 0;
    c->inference_kernel = RGR_GUIDE_TCGEN05;
    c->max_depth = 0;
    c->seed = 1;
    c->training_kernel = RGR_GUIDE_TCGEN05;
    c->learn_fraction = 1;
}

static bool valid_config(const rgr_guide_config& c) {
    return c.learning_rate >= 0.0f && std::isfinite(c.learning_rate) && c.beta1 >= 0.0f && c.beta1 < 1.0f &&
           c.beta2 >= 0.0f && c.beta2 < 1.0f && c.epsilon > 0.0f && c.batch_samples >= 64 &&
           c.batch_samples <= (1u << 24) && c.guide_fraction >= 0.0f && c.guide_fraction <= 1.0f &&
           c.train_interval >= 1 && c.train_interval <= 64 &&
           (c.inference_kernel == RGR_GUIDE_TCGEN05 || c.inference_kernel == RGR_GUIDE_MMA_SYNC) &&
           (c.training_kernel == RGR_GUIDE_TCGEN05 || c.training_kernel == RGR_GUIDE_MMA_SYNC);
}

int rgr_guide_create(rgr_guide** out, int32_t device, const rgr_guide_config* cfg) {
    if (!out) return RGR_E_INVALID;
    *out = nullptr;
    rgr_guide_config d;
    rgr_guide_config_default(&d);
    const rgr_guide_config& c = cfg ? *cfg : d;
    if (!valid_config(c)) return RGR_E_INVALID;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        set_error("no CUDA device");
        return RGR_E_NODEVICE;
    }
    if (device < 0 || device >= ndev) return RGR_E_INVALID;
    RGR_CUDA(cudaSetDevice(device));
    RGR_CUDA((cudaError_t)guide_kernel_attributes());
    RGR_CUDA((cudaError_t)guide_tc_attributes());
    RGR_CUDA((cudaError_t)guide_train_tc_attributes());
    rgr_guide* g = new (std::nothrow) rgr_guide();
    if (!g) return RGR_E_OOM;
    g->device = device;
    if (cudaDeviceGetAttribute(&g->num_sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess) {
        delete g;
        return RGR_E_CUDA;
    }
    int r = g->init(c);
    if (r != RGR_OK) {
        delete g;
        return r;
    }
    *out = g;
    return RGR_OK;
}

void rgr_guide_destroy(rgr_guide* g) {
    if (!g) return;
    cudaSetDevice(g->device);
    cudaDeviceSynchronize();
    delete g;
}

int rgr_guide_set_config(rgr_guide* g, const rgr_guide_config* cfg) {
    if (!g || !cfg || !valid_config(*cfg)) return RGR_E_INVALID;
    if (cfg->batch_samples != g->cfg.batch_samples) {
        RGR_CUDA(cudaSetDevice(g->device));
        RGR_CUDA(cudaDeviceSynchronize());
        int r = g->samples.alloc(64 * (size_t)cfg->batch_samples);
        if (r != RGR_OK) return r;
        g->train.samples = g->test.samples = g->samples.as<float>();
        g->train.cap = g->test.cap = cfg->batch_samples;
    }
    g->cfg = *cfg;
    g->train.max_iter = cfg->max_iterations;
    g->train.min_count = min_batch(*cfg);
    return RGR_OK;
}

int rgr_guide_set_bounds(rgr_guide* g, const float lo[3], const float hi[3]) {
    if (!g || !lo || !hi) return RGR_E_INVALID;
    return g->set_bounds(lo, hi);
}

int rgr_guide_get_weights(rgr_guide* g, float* w, float* b) {
    if (!g || !w || !b) return RGR_E_INVALID;
    RGR_CUDA(cudaSetDevice(g->device));
    RGR_CUDA(cudaDeviceSynchronize());
    RGR_CUDA(cudaMemcpy(w, g->w.p, 4 * kGuideWeights, cudaMemcpyDeviceToHost));
    RGR_CUDA(cudaMemcpy(b, g->b.p, 4 * kGuideBiases, cudaMemcpyDeviceToHost));
    return RGR_OK;
}

int rgr_guide_set_weights(rgr_guide* g, const float* w, const float* b) {
    if (!g || !w || !b) return RGR_E_INVALID;
    if (!check_padding(w, b)) {
        set_error("rgr_guide_set_weights: non-finite weight, or non-zero padding outside the 36-64x4-40 network");
        return RGR_E_INVALID;
    }
    std::vector<uint16_t> hbf(kGuideWeights);
    for (int i = 0; i < kGuideWeights; ++i) hbf[i] = to_bf16(w[i]);
    std::vector<unsigned char> hsw(kGuideWtBytes, 0);
    for (uint32_t l = 0; l < (uint32_t)kGuideLayers; ++l) {
        for (uint32_t in = 0; in < 64; ++in)
            for (uint32_t out = 0; out < 64; ++out)
                memcpy(&hsw[wt_sw_offset(l, in, out)], &hbf[(l * 64 + in) * 64 + out], 2);
        for (uint32_t out = 0; out < 64; ++out) {  // after the weights: layer 0's sits on padding inputs
            const float bias = b[l * 64 + out];
            const uint16_t hi = to_bf16(bias);
            const uint32_t hi_bits = (uint32_t)hi << 16;
            float hi_f;
            memcpy(&hi_f, &hi_bits, 4);
            const uint16_t lo = to_bf16(bias - hi_f);
            memcpy(&hsw[wt_bias_offset(l, out, 0)], &hi, 2);
            memcpy(&hsw[wt_bias_offset(l, out, 1)], &lo, 2);
        }
    }
    RGR_CUDA(cudaSetDevice(g->device));
    RGR_CUDA(cudaDeviceSynchronize());
    RGR_CUDA(cudaMemcpy(g->w.p, w, 4 * kGuideWeights, cudaMemcpyHostToDevice));
    RGR_CUDA(cudaMemcpy(g->b.p, b, 4 * kGuideBiases, cudaMemcpyHostToDevice));
    RGR_CUDA(cudaMemcpy(g->wbf.p, hbf.data(), 2 * kGuideWeights, cudaMemcpyHostToDevice));
    RGR_CUDA(cudaMemcpy(g->wtsw.p, hsw.data(), kGuideWtBytes, cudaMemcpyHostToDevice));
    RGR_CUDA(cudaMemset(g->gW.p, 0, 4 * kGuideWeights));
    RGR_CUDA(cudaMemset(g->gb.p, 0, 4 * kGuideBiases));
    RGR_CUDA(cudaMemset(g->m.p, 0, 4 * kGuideParams));
    RGR_CUDA(cudaMemset(g->v.p, 0, 4 * kGuideParams));
    RGR_CUDA(cudaMemset(g->loss.p, 0, 16));
    RGR_CUDA(cudaMemset(g->counters.p, 0, kCtrBytes));
    const float one = 1.0f;
    RGR_CUDA(cudaMemcpy(g->counters.as<unsigned char>() + kCtrAccept, &one, 4, cudaMemcpyHostToDevice));
    RGR_CUDA(cudaMemcpy(g->counters.as<unsigned char>() + kCtrTest + kCtrAccept, &one, 4, cudaMemcpyHostToDevice));
    return RGR_OK;
}

int rgr_guide_infer_device(rgr_guide* g, const float* rows, uint32_t n, float* out, void* stream) {
    RGR_NVTX_RANGE("rgr_guide_infer_device");
    if (!g || (n && (!rows || !out))) return RGR_E_INVALID;
    if (n == 0) return RGR_OK;
    RGR_CUDA(cudaSetDevice(g->device));
    if (g->cfg.inference_kernel == RGR_GUIDE_TCGEN05) {
        const int grid = (int)std::min<uint32_t>((n + 127) / 128, (uint32_t)guide_tc_grid(g->num_sms));
        launch_guide_infer_tc(g->view, rows, n, out, grid, g->error_word(), (cudaStream_t)stream);
    } else {
        const int grid = (int)std::min<uint32_t>((n + 127) / 128, (uint32_t)guide_infer_grid(g->num_sms));
        launch_guide_infer(g->view, rows, n, out, grid, (cudaStream_t)stream);
    }
    RGR_CUDA(cudaGetLastError());
    return RGR_OK;
}

int rgr_guide_train_device(rgr_guide* g, const float* samples, uint32_t n, float weight_scale, int32_t apply_adam,
                           float* grads, float* loss, void* stream) {
    RGR_NVTX_RANGE("rgr_guide_train_device");
    if (!g || (n && !samples) || !std::isfinite(weight_scale)) return RGR_E_INVALID;
    RGR_CUDA(cudaSetDevice(g->device));
    cudaStream_t st = (cudaStream_t)stream;
    RGR_CUDA(cudaMemcpyAsync(g->test.count, &n, 4, cudaMemcpyHostToDevice, st));
    RGR_CUDA(cudaMemsetAsync(g->loss.p, 0, 4, st));
    g->gradient_launches(samples, g->test.count, n, 0u, nullptr, weight_scale, train_grid(*g, n), st);
    RGR_CUDA(cudaGetLastError());
    if (grads) {
        RGR_CUDA(cudaMemcpyAsync(grads, g->gW.p, 4 * kGuideWeights, cudaMemcpyDeviceToDevice, st));
        RGR_CUDA(cudaMemcpyAsync(grads + kGuideWeights, g->gb.p, 4 * kGuideBiases, cudaMemcpyDeviceToDevice, st));
    }
    float hl = 0.0f;
    RGR_CUDA(cudaMemcpyAsync(&hl, g->loss.p, 4, cudaMemcpyDeviceToHost, st));
    if (apply_adam) {
        launch_guide_adam(g->view, g->test.count, 0u, g->test.iter, g->cfg.learning_rate, g->cfg.beta1, g->cfg.beta2,
                          g->cfg.epsilon, st);
        launch_guide_finish(g->view, g->test, st);
        RGR_CUDA(cudaGetLastError());
    } else {
        RGR_CUDA(cudaMemsetAsync(g->gW.p, 0, 4 * kGuideWeights, st));
        RGR_CUDA(cudaMemsetAsync(g->gb.p, 0, 4 * kGuideBiases, st));
        RGR_CUDA(cudaMemsetAsync(g->loss.p, 0, 4, st));
    }
    RGR_CUDA(cudaStreamSynchronize(st));
    if (loss) *loss = hl;
    return RGR_OK;
}

int rgr_guide_train_device_async(rgr_guide* g, const float* samples, uint32_t n, float weight_scale, void* stream) {
    RGR_NVTX_RANGE("rgr_guide_train_device_async");
    if (!g || (n && !samples) || !std::isfinite(weight_scale)) return RGR_E_INVALID;
    if (n == 0) return RGR_OK;
    RGR_CUDA(cudaSetDevice(g->device));
    cudaStream_t st = (cudaStream_t)stream;
    // n reaches the test stream's count word by a kernel, in stream order
    RGR_CUDA(cudaMemsetAsync(g->loss.p, 0, 4, st));
    launch_guide_set_count(g->test.count, n, st);
    g->gradient_launches(samples, g->test.count, n, 0u, nullptr, weight_scale, train_grid(*g, n), st);
    launch_guide_adam(g->view, g->test.count, 0u, g->test.iter, g->cfg.learning_rate, g->cfg.beta1, g->cfg.beta2,
                      g->cfg.epsilon, st);
    launch_guide_finish(g->view, g->test, st);
    RGR_CUDA(cudaGetLastError());
    return RGR_OK;
}

int rgr_guide_check(rgr_guide* g) {
    if (!g) return RGR_E_INVALID;
    RGR_CUDA(cudaSetDevice(g->device));
    RGR_CUDA(cudaDeviceSynchronize());
    uint32_t e = 0;
    RGR_CUDA(cudaMemcpy(&e, g->error_word(), 4, cudaMemcpyDeviceToHost));
    if (e) {
        RGR_CUDA(cudaMemset(g->error_word(), 0, 4));  // reported once; the guide stays usable
        set_error("guide: a tensor-core wait timed out (error bits " + std::to_string(e) + ")");
        return RGR_E_CUDA;
    }
    return RGR_OK;
}

int rgr_guide_set_stall(rgr_guide* g, int32_t on) {
    if (!g) return RGR_E_INVALID;
    g->view.stall_mma = on ? 1u : 0u;
    return RGR_OK;
}

int rgr_guide_stats_get(rgr_guide* g, rgr_guide_stats* out) {
    if (!g || !out) return RGR_E_INVALID;
    memset(out, 0, sizeof(*out));
    RGR_CUDA(cudaSetDevice(g->device));
    RGR_CUDA(cudaDeviceSynchronize());
    unsigned char ctr[kCtrBytes];
    RGR_CUDA(cudaMemcpy(ctr, g->counters.p, kCtrBytes, cudaMemcpyDeviceToHost));
    uint32_t it;
    memcpy(&it, ctr + kCtrIter, 4);
    memcpy(&out->accept, ctr + kCtrAccept, 4);
    out->iterations = it;
    if (it > 0)
        RGR_CUDA(cudaMemcpy(&out->last_loss, g->loss_hist.as<float>() + (it - 1) % kLossHist, 4,
                            cudaMemcpyDeviceToHost));
    return RGR_OK;
}

int rgr_guide_loss_history(rgr_guide* g, float* out, uint32_t max, uint32_t* count) {
    if (!g || (max && !out)) return RGR_E_INVALID;
    RGR_CUDA(cudaSetDevice(g->device));
    RGR_CUDA(cudaDeviceSynchronize());
    uint32_t it = 0;
    RGR_CUDA(cudaMemcpy(&it, g->counters.as<unsigned char>() + kCtrIter, 4, cudaMemcpyDeviceToHost));
    std::vector<float> h(kLossHist);
    RGR_CUDA(cudaMemcpy(h.data(), g->loss_hist.p, 4 * kLossHist, cudaMemcpyDeviceToHost));
    const uint32_t n = std::min(std::min(it, max), kLossHist);
    for (uint32_t i = 0; i < n; ++i) out[i] = h[(it - n + i) % kLossHist];
    if (count) *count = n;
    return RGR_OK;
}

int rgr_guide_last_batch(rgr_guide* g, float* out, uint32_t max, uint32_t* count) {
    if (!g || (max && !out)) return RGR_E_INVALID;
    RGR_CUDA(cudaSetDevice(g->device));
    RGR_CUDA(cudaDeviceSynchronize());
    uint32_t last = 0;
    RGR_CUDA(cudaMemcpy(&last, g->train.last, 4, cudaMemcpyDeviceToHost));
    const uint32_t n = std::min(last, max);
    if (n) RGR_CUDA(cudaMemcpy(out, g->samples.p, 64 * (size_t)n, cudaMemcpyDeviceToHost));
    if (count) *count = n;
    return RGR_OK;
}

}  // extern "C"
