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


def spread(errs) -> dict:
    """mean, median, min and max of per-seed relMSE values."""
    e = np.asarray(errs, np.float64)
    return {"mean": float(e.mean()), "median": float(np.median(e)), "min": float(e.min()), "max": float(e.max())}


def equal_time(rg, scene, cam, ref: np.ndarray, spp_plain: int, path_count: int = 1 << 22, seed_offset: int = 1,
               guide_kw: dict | None = None, repeats: int = 8, warm_spp: int | None = None,
               longer_warm_spp: tuple = ()) -> dict:
    """Plain rendering at spp_plain against guided rendering given the same
    wall time, relMSE against `ref` over `repeats` seeds (medians, with mean,
    min and max: single sun-caustic samples of radiance ~1e4 dominate
    individual runs).  The ratios are plain's relMSE over guided's, of the
    medians and of the means.
      cold: the guide starts untrained and trains online on the render's own
            samples (`guide_kw`), inference and training inside the time;
      warm: a guide trained online, without an iteration limit, by an earlier
            render of the same view at warm_spp (default 4 x spp_plain)
            samples per pixel, then frozen (no training cost), as when a guide
            persists across the frames of an interactive session;
      warm_<n>spp: the same with a guide trained by an n-spp render, for each
            n in longer_warm_spp.
    The guided spp for each is calibrated from a guided run at spp_plain."""
    guide_kw = dict(guide_kw or {})
    lane = rg.WavefrontLane(0, path_count)
    lane.setup(scene)
    # warm-up: graph capture and first-touch allocations
    render(rg, scene, cam, 1, seed_offset + 99, lane=lane)
    render(rg, scene, cam, 1, seed_offset + 99, lane=lane, guide=rg.Guide(0, **guide_kw))
    seeds = [seed_offset + r * path_count for r in range(repeats)]
    plain_t, plain_e = [], []
    for sd in seeds:
        _, acc, t = render(rg, scene, cam, spp_plain, sd, lane=lane)
        plain_t.append(t)
        plain_e.append(relmse(mean_image(acc), ref))
    tp = float(np.median(plain_t))
    ep = float(np.median(plain_e))
    # cold: calibrate the cost per spp, then render at the spp that fits
    same_e, iters, same_t = [], [], []
    for sd in seeds:
        g = rg.Guide(0, **guide_kw)
        _, acc, tg = render(rg, scene, cam, spp_plain, sd, lane=lane, guide=g)
        same_t.append(tg)
        same_e.append(relmse(mean_image(acc), ref))
        iters.append(g.stats()["iterations"])
    spp_cold = max(1, int(spp_plain * tp / float(np.median(same_t))))
    cold_t, cold_e = [], []
    for sd in seeds:
        _, acc, t = render(rg, scene, cam, spp_cold, sd, lane=lane, guide=rg.Guide(0, **guide_kw))
        cold_t.append(t)
        cold_e.append(relmse(mean_image(acc), ref))
    # warm: trained by an earlier render of the same view, frozen
    def warm(train_spp: int) -> dict:
        warm_kw = dict(guide_kw)
        warm_kw["max_iterations"] = 0
        trained = rg.Guide(0, **warm_kw)
        render(rg, scene, cam, train_spp, seed_offset + (repeats + 3) * path_count, lane=lane, guide=trained)
        warm_iters = trained.stats()["iterations"]
        trained.set_config(train=0)
        _, _, tw = render(rg, scene, cam, spp_plain, seed_offset + 7, lane=lane, guide=trained)
        spp_warm = max(1, int(spp_plain * tp / tw))
        warm_t, warm_e, warm_same = [], [], []
        for sd in seeds:
            _, acc, t = render(rg, scene, cam, spp_warm, sd, lane=lane, guide=trained)
            warm_t.append(t)
            warm_e.append(relmse(mean_image(acc), ref))
            _, acc, _ = render(rg, scene, cam, spp_plain, sd, lane=lane, guide=trained)
            warm_same.append(relmse(mean_image(acc), ref))
        ew = float(np.median(warm_e))
        return {"spp": spp_warm, "time_s": round(float(np.median(warm_t)), 4), "relmse": ew,
                "trained_by": f"{train_spp} spp render, {warm_iters} iterations",
                "relmse_runs": [round(e, 6) for e in warm_e], "relmse_spread": spread(warm_e),
                "relmse_ratio_equal_time": round(ep / ew, 3) if ew > 0 else None,
                "relmse_ratio_of_means": round(float(np.mean(plain_e) / np.mean(warm_e)), 3),
                "relmse_same_spp": float(np.median(warm_same))}

    ec = float(np.median(cold_e))
    out = {
        "seeds": repeats, "spp_plain": spp_plain, "time_plain_s": round(tp, 4), "relmse_plain": ep,
        "relmse_plain_runs": [round(e, 6) for e in plain_e], "relmse_plain_spread": spread(plain_e),
        "cold": {"spp": spp_cold, "time_s": round(float(np.median(cold_t)), 4), "relmse": ec,
                 "relmse_runs": [round(e, 6) for e in cold_e], "relmse_spread": spread(cold_e),
                 "relmse_ratio_equal_time": round(ep / ec, 3) if ec > 0 else None,
                 "relmse_ratio_of_means": round(float(np.mean(plain_e) / np.mean(cold_e)), 3),
                 "relmse_same_spp": float(np.median(same_e)), "relmse_same_spp_spread": spread(same_e),
                 "training_iterations": int(np.median(iters))},
        "warm": warm(warm_spp or 4 * spp_plain),
    }
    for n in longer_warm_spp:
        out[f"warm_{n}spp"] = warm(n)
    return out
