"""Project autotuner: picks the launch shape of the renderer by timing it.

Knobs (all results are bit-identical across knob values; only speed changes):
  * path_count     — resident paths in the pool (queue capacities follow it);
  * graph_steps    — bounces per replayed CUDA graph;
  * shade_blocks   — resident 256-thread blocks per SM of the shade kernel;
  * render_refill  — refill a warp of the bounce's persistent trace kernel
                     when this many lanes are idle;
  * render_search  — that kernel's warps take node steps while this many
                     lanes still search for their next leaf;
  * trace_reorder  — the closest-hit call sorts its rays by origin and
                     direction first (pays for incoherent rays);
  * trace_refill   — refill a closest-hit warp with new rays when this many
                     lanes are idle;
  * trace_search   — the same leaf batching for the closest-hit kernel;
  * trace_stage    — top BVH nodes each closest-hit CTA stages in shared
                     memory (the "BVH staging depth": 64 nodes = 6 levels).
Coordinate descent from a default point: each knob in turn is swept over its
candidates with the others fixed, keeping the fastest.  Each trial runs a
proxy of the real workload (the same scenes and cameras with the samples per
pixel capped) and is timed on the device.  Results are cached per GPU model
and workload signature in a JSON file (default: next to this module,
_tuned.json, git-ignored).
"""
from __future__ import annotations

import hashlib
import json
import os
import time
from pathlib import Path

DEFAULTS = dict(path_count=1 << 22, graph_steps=8, shade_blocks=8, render_refill=12, render_search=8)
CANDIDATES = dict(path_count=[1 << 20, 1 << 21, 1 << 22, 1 << 23, 1 << 24], graph_steps=[4, 8, 16], shade_blocks=[4, 8, 16],
                  render_refill=[8, 16, 24], render_search=[4, 12, 16])
TRACE_DEFAULTS = dict(trace_reorder=0, trace_refill=24, trace_search=8, trace_stage=0)
# ray reordering first: the launch shape is then tuned for the rays in the order they are traced
TRACE_CANDIDATES = dict(trace_reorder=[1], trace_refill=[8, 16, 32], trace_search=[4, 12, 16],
                        trace_stage=[0, 64, 256, 1024])


def _gpu_name(device: int) -> str:
    try:
        import torch
        return torch.cuda.get_device_name(device)
    except Exception:  # noqa: BLE001
        return "unknown-gpu"


class Autotuner:
    def __init__(self, device: int = 0, cache_path: str | None = None, log=print):
        self.device = device
        self.cache_path = Path(cache_path) if cache_path else Path(__file__).resolve().parent / "_tuned.json"
        self.log = log
        self.trials = []

    def _load(self) -> dict:
        if self.cache_path.exists():
            try:
                return json.loads(self.cache_path.read_text())
            except ValueError:
                return {}
        return {}

    def _store(self, key: str, value: dict) -> None:
        d = self._load()
        d[key] = value
        tmp = self.cache_path.with_suffix(".tmp")
        tmp.write_text(json.dumps(d, indent=1, sort_keys=True))
        os.replace(tmp, self.cache_path)

    def tune(self, signature: str, run_trial, use_cache: bool = True, defaults: dict | None = None,
             candidates: dict | None = None, valid=None) -> dict:
        """run_trial(params) -> seconds.  Returns the best params; `valid(params)`
        False skips a combination without running it."""
        defaults = DEFAULTS if defaults is None else defaults
        candidates = CANDIDATES if candidates is None else candidates
        key = hashlib.sha1((_gpu_name(self.device) + "|" + signature).encode()).hexdigest()[:16]
        if use_cache:
            cached = self._load().get(key)
            if cached:
                return dict(cached["params"])
        best = dict(defaults)
        best_t = self._time(run_trial, best)
        for knob, values in candidates.items():
            for v in values:
                if v == best[knob]:
                    continue
                p = dict(best)
                p[knob] = v
                if valid is not None and not valid(p):
                    continue
                t = self._time(run_trial, p)
                if t < best_t:
                    best, best_t = p, t
        self._store(key, dict(params=best, seconds=best_t, signature=signature, gpu=_gpu_name(self.device),
                              trials=self.trials, when=time.strftime("%Y-%m-%dT%H:%M:%SZ", time.gmtime())))
        return best

    def _time(self, run_trial, params: dict) -> float:
        t = run_trial(params)
        self.trials.append(dict(params=params, seconds=round(t, 6)))
        self.log(f"autotune {params} -> {t * 1e3:.2f} ms")
        return t


def tune_batch(scenes_and_requests, device: int = 0, spp_cap: int = 4, use_cache: bool = True, log=print) -> dict:
    """Tune the batched renderer on a proxy of `scenes_and_requests`, a list of
    (SceneManager, rgr_camera, rgr_render_config)."""
    import raccoongpurender_gb300 as rg

    sig = "batch|" + "|".join(f"{c.image_w}x{c.image_h}:{f.spp}:{s.info().num_triangles}"
                              for s, c, f in scenes_and_requests)

    def trial(p):
        b = rg.Batch(device, p["path_count"])
        b.set_render_tuning(p["shade_blocks"], p["graph_steps"])
        b.set_render_trace(p["render_refill"])
        b.set_trace_search(p["render_search"])
        for s, c, f in scenes_and_requests:
            g = rg.render_config(dof=f.dof, rr_depth=f.rr_depth, radiance_clamp=f.radiance_clamp,
                                 env_select_prob=f.env_select_prob, max_depth=f.max_depth,
                                 seed_offset=f.seed_offset, spp=min(int(f.spp), spp_cap))
            b.add(s, c, g)
        t0 = time.perf_counter()
        b.run(order=rg.ORDER_SHORTEST_FIRST, steps_per_launch=p["graph_steps"])
        return time.perf_counter() - t0

    return Autotuner(device, log=log).tune(sig, trial, use_cache=use_cache)


def tune_trace(lane, ray_sets, stream: int, device: int = 0, reps: int = 3, use_cache: bool = False,
               log=print) -> tuple[dict, list]:
    """Tune the closest-hit kernel (ray reordering, refill threshold, leaf
    batching, BVH staging depth) on `ray_sets`, a list of (7 device pointers,
    n, prim pointer, t pointer), by
    timing `reps` passes over all sets with CUDA events on `stream`.  Applies
    the best to `lane`; returns (params, trials)."""
    import torch

    sig = "trace|" + "|".join(str(n) for _, n, _, _ in ray_sets)
    st = torch.cuda.ExternalStream(stream)

    def run(p):
        lane.set_trace_reorder(p["trace_reorder"])
        lane.set_trace_staging(p["trace_stage"])
        lane.set_trace_tuning(p["trace_refill"], 0)
        lane.set_trace_search(p["trace_search"], 0)
        for ptrs, n, pp, tp in ray_sets:  # warm
            lane.trace_closest_device(ptrs, n, pp, tp, 0, stream)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(st)
        for _ in range(reps):
            for ptrs, n, pp, tp in ray_sets:
                lane.trace_closest_device(ptrs, n, pp, tp, 0, stream)
        e1.record(st)
        e1.synchronize()
        return e0.elapsed_time(e1) * 1e-3 / reps

    tuner = Autotuner(device, log=log)
    # the sorted rays' traversal stages no nodes: no staging trials with sorting on
    best = tuner.tune(sig, run, use_cache=use_cache, defaults=TRACE_DEFAULTS, candidates=TRACE_CANDIDATES,
                      valid=lambda p: not (p["trace_reorder"] and p["trace_stage"]))
    lane.set_trace_reorder(best.get("trace_reorder", 0))
    lane.set_trace_staging(best["trace_stage"])
    lane.set_trace_tuning(best["trace_refill"], 0)
    lane.set_trace_search(best["trace_search"], 0)
    return best, tuner.trials
