"""Measuring learned path guiding: FP64 mean images, relMSE against a
high-spp FP64 reference, and the equal-time comparison of guided and plain
rendering.

Both estimators are rendered with the two fixes of back-face sampling the
guided renderer always applies (RGR_RENDER_FIX_BACKSIDE_ENV_PDF and
RGR_RENDER_TWO_SIDED_LAMBERTIAN), and without
the radiance discard (radiance_clamp at the float maximum): a discard
threshold removes a share of the integrand that depends on the sampling pdf,
so guided and plain rendering would converge to different images."""
from __future__ import annotations

import time

import numpy as np

NO_CLAMP = 3.0e38


def relmse(img: np.ndarray, ref: np.ndarray, eps: float = 1e-2) -> float:
    """mean over pixels and channels of (img - ref)^2 / (ref^2 + eps)."""
    d = np.asarray(img, np.float64) - ref
    return float(np.mean(d * d / (ref * ref + eps)))


def mean_image(acc: np.ndarray) -> np.ndarray:
    """(H, W, 3) per-pixel mean of FP64 sums (H, W, 4)."""
    return acc[..., :3] / np.maximum(acc[..., 3:4], 1.0)


def config(rg, spp: int, seed_offset: int, max_depth: int = 8, dof: float = 0.0045):
    return rg.render_config(spp=spp, max_depth=max_depth, dof=dof, radiance_clamp=NO_CLAMP, seed_offset=seed_offset,
                            flags=rg.RENDER_FIX_BACKSIDE_ENV_PDF | rg.RENDER_TWO_SIDED_LAMBERTIAN)


def render(rg, scene, cam, spp: int, seed_offset: int, path_count: int = 1 << 22, guide=None, lane=None,
           max_depth: int = 8, dof: float = 0.0045):
    """Render spp samples per pixel; returns (lane, FP64 sums, seconds).
    With `guide`, the render is guided and trains the guide as it goes."""
    if lane is None:
        lane = rg.WavefrontLane(0, path_count)
        lane.setup(scene)
    lane.set_guide(guide)
    lane.initialize(cam, config(rg, spp, seed_offset, max_depth, dof))
    lane.synchronize()
    t0 = time.perf_counter()
    lane.render_until_done(1 << 30)
    t1 = time.perf_counter()
    return lane, lane.accumulation(), t1 - t0


def render_mean(rg, scene, cam, spp: int, seed_offset: int, path_count: int = 1 << 22, guide=None,
                max_depth: int = 8, dof: float = 0.0045) -> np.ndarray:
    _, acc, _ = render(rg, scene, cam, spp, seed_offset, path_count, guide, max_depth=max_depth, dof=dof)
    return mean_image(acc)


def equal_time(rg, scene, cam, ref: np.ndarray, spp_plain: int, path_count: int = 1 << 22, seed_offset: int = 1,
               guide_kw: dict | None = None, repeats: int = 1) -> dict:
    """Plain rendering at spp_plain against guided rendering given the same
    wall time (the guide starts untrained and trains while it renders; its
    training and inference are inside the time).  The guided spp is
    calibrated from a guided run at spp_plain, then the guided render is
    repeated at the spp that fits the plain time."""
    guide_kw = dict(guide_kw or {})
    lane = rg.WavefrontLane(0, path_count)
    lane.setup(scene)
    # warm-up: graph capture and first-touch allocations
    render(rg, scene, cam, 1, seed_offset + 99, lane=lane)
    g0 = rg.Guide(0, **guide_kw)
    render(rg, scene, cam, 1, seed_offset + 99, lane=lane, guide=g0)
    plain_t, plain_e = [], []
    for r in range(repeats):
        _, acc, t = render(rg, scene, cam, spp_plain, seed_offset + r * path_count, lane=lane)
        plain_t.append(t)
        plain_e.append(relmse(mean_image(acc), ref))
    tp = float(np.median(plain_t))
    # calibrate the guided cost per spp
    _, _, tg = render(rg, scene, cam, spp_plain, seed_offset, lane=lane, guide=rg.Guide(0, **guide_kw))
    spp_g = max(1, int(spp_plain * tp / tg))
    guided_t, guided_e, iters = [], [], []
    for r in range(repeats):
        guide = rg.Guide(0, **guide_kw)
        _, acc, t = render(rg, scene, cam, spp_g, seed_offset + r * path_count, lane=lane, guide=guide)
        guided_t.append(t)
        guided_e.append(relmse(mean_image(acc), ref))
        iters.append(guide.stats()["iterations"])
    # the same number of samples, guided, for the per-sample gain
    _, acc_s, t_s = render(rg, scene, cam, spp_plain, seed_offset, lane=lane, guide=rg.Guide(0, **guide_kw))
    e_same = relmse(mean_image(acc_s), ref)
    ep, eg = float(np.median(plain_e)), float(np.median(guided_e))
    tgm = float(np.median(guided_t))
    return {
        "spp_plain": spp_plain, "time_plain_s": round(tp, 4), "relmse_plain": ep,
        "spp_guided": spp_g, "time_guided_s": round(tgm, 4), "relmse_guided": eg,
        "relmse_ratio_equal_time": round(ep / eg, 3) if eg > 0 else None,
        "efficiency_ratio": round((ep * tp) / (eg * tgm), 3) if eg > 0 else None,
        "relmse_guided_same_spp": e_same, "time_guided_same_spp_s": round(t_s, 4),
        "training_iterations": int(np.median(iters)),
    }
