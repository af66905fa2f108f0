// guide_host.h — the host object behind rgr_guide: the path-guiding network
// and its optimiser state on one device, plus the training-sample stream a
// guided render feeds.
#pragma once
#include "../kernels/guide.cuh"
#include "devbuf.h"

struct rgr_guide {
    int device = 0;
    int num_sms = 152;
    rgr_guide_config cfg{};
    // network: FP32 master weights and biases, BF16 weights, gradients, Adam moments, loss
    rgr::DevBuf w, b, wbf, gW, gb, m, v, loss;
    // training stream: samples, counters, loss history
    rgr::DevBuf samples, counters, loss_hist, wtsw;
    rgr::DevBuf gpart;  // the tcgen05 training kernel's per-CTA gradient slots (num_sms x kGuidePartStride)
    rgr::dev::GuideView view{};
    rgr::dev::GuideTrainD train{};  // the render's stream (counter bytes 0..27)
    rgr::dev::GuideTrainD test{};   // rgr_guide_train_device's (bytes 32..59; shares iter)
    bool bounds_set = false;

    int init(const rgr_guide_config& c);
    int set_bounds(const float lo[3], const float hi[3]);
    // the bounce's inference launch (tcgen05 or mma.sync kernel, per cfg)
    void infer_paths(const rgr::dev::PathsView& p, const rgr::dev::QueueView& q, const rgr::dev::GuideRenderD& gd,
                     cudaStream_t st);
    uint32_t* error_word() const;
    // the launches that follow the trace/logic kernel of a guided render on the
    // bounces that end a training interval: train, Adam, reset the stream
    int train_launches(cudaStream_t st);
    // one iteration's gradient launches (the configured training kernel) over
    // min(*count, cap) samples, into gW, gb and the loss; `grid` CTAs
    void gradient_launches(const float* samples, const uint32_t* count, uint32_t cap, uint32_t min_count,
                           const float* wsum, float weight_scale, int grid, cudaStream_t st);
};
