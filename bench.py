#!/usr/bin/env python3
"""Headline benchmark: closest-hit ray casting on one GB300.

Workload (the reference path's ray-cast microbenchmark): a seeded icosphere
subdivided to 1,310,720 triangles with radial 3-octave value-noise
displacement, SAH BVH with leaves of at most 4 triangles; 4,194,304 coherent
pinhole primary rays (2048x2048) plus 4,194,304 incoherent rays (origins
uniform in the bounding box, directions uniform on the sphere), FP32.  One
step casts all 8,388,608 rays (two launches of the traversal kernel) and
produces the closest primitive id and t for each, bit-identical to the
reference traversal.

Metric: Mrays/s.  ``value`` times the step with the rays already in HBM
(CUDA events on the launching stream); ``e2e`` runs the same step through the
C ABI with pinned host buffers, host-to-device copy of the rays and
device-to-host copy of the hits inside the timed region.  The rays (224 MB)
are larger than the 129 MB L2, so consecutive steps do not reuse them.

``--impl reference`` times the reference traversal on the host cores: the
oracle's restatement of kernels/extension_ray_cast_stackless.cl on all host
threads, all 8,388,608 rays per step, over a tree the oracle builds itself
(binned SAH flattened as common/stackless_bvh.hpp:283-341 does).  That arm
loads no product library: the mesh and rays come from the seeded numpy
generators.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import tempfile
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

WORKLOAD = "closest-hit: 1.31M-tri displaced icosphere, 4M coherent + 4M incoherent rays"
METRIC = "closest-hit Mrays/s (1 GB300)"


def measured_peaks() -> dict:
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return dict(hbm_gbs=float(d["hbm_gbs"]), source="measured")
    return dict(hbm_gbs=6800.0, source="fallback")


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.path = None

    def __enter__(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self) -> dict:
        rows = []
        if self.path and os.path.exists(self.path):
            for line in open(self.path):
                parts = [x.strip() for x in line.split(",")]
                if len(parts) >= 9:
                    rows.append(parts)
            os.unlink(self.path)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}

        def num(x):
            try:
                return float(x)
            except ValueError:
                return None

        sm = [num(r[1]) for r in rows if num(r[1]) is not None]
        smax = max((num(r[2]) or 0.0) for r in rows)
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in rows for k in range(4) if r[5 + k].lower().startswith("active")})
        sm.sort()
        return {"sm_mhz": sm[len(sm) // 2] if sm else None, "sm_max_mhz": smax, "reasons": reasons,
                "samples": len(rows)}


def build_workload(level: int = 8, res: int = 2048):
    import raccoongpurender_gb300 as rg
    from raccoongpurender_gb300 import scenes
    mesh = scenes.displaced_icosphere(level, seed=7)
    mesh.materials = [rg.materials.lambertian()] * mesh.ntris
    sm = rg.SceneManager()
    sm.addMesh(mesh)
    t0 = time.time()
    sm.buildBVH(max_leaf_size=4)
    build_s = time.time() - t0
    coherent, incoherent = scenes.closest_hit_rays(mesh, res=res, n_random=res * res, seed=11)
    return mesh, sm, coherent, incoherent, build_s


def closest_hit_once(dev_index: int = 0, reorder: int = 0) -> None:
    """One launch of the closest-hit kernel per ray set of the workload above
    (coherent, then incoherent) with the library's default launch shape, rays
    in device memory: the command the kernel's ncu captures run.  reorder = 1
    sorts each set by origin and direction first (three more launches per
    set: the key histogram, its scan and the scatter)."""
    import torch

    import raccoongpurender_gb300 as rg
    mesh, sm, coherent, incoherent, _ = build_workload()
    lane = rg.WavefrontLane(dev_index, 1024)
    lane.setup(sm)
    lane.set_trace_reorder(reorder)
    dev = torch.device("cuda", dev_index)
    stream = torch.cuda.Stream(dev)
    for rays in (coherent, incoherent):
        soa = [torch.from_numpy(a).to(dev) for a in rays.soa()]
        prim = torch.empty(len(rays), dtype=torch.int32, device=dev)
        t = torch.empty(len(rays), dtype=torch.float32, device=dev)
        torch.cuda.synchronize(dev)
        lane.trace_closest_device([a.data_ptr() for a in soa], len(rays), prim.data_ptr(), t.data_ptr(), 0,
                                  stream.cuda_stream)
        stream.synchronize()


def render_bench(dev_index: int, which: str, repeats: int = 2, pools=(1 << 22,)) -> dict:
    """Full wavefront renders at a fixed sample budget, timed with CUDA events
    on the context stream (host waits only at the end).
    cornell: 36 triangles, 256x256, 4 spp, depth 5, pinhole, no envmap.
    mixed:   the 1.31M-triangle sphere + ground + volume box, per-triangle
             Lambertian/Ward/dielectric, 1024x512 sky + sun envmap,
             1920x1080, 64 spp, depth 8.
    Each resident-path pool size in `pools` is timed (2^22 is the reference's
    kWavefrontPathCountGPU; the Cornell box's 256x256x4 paths fit 2^18); the
    fastest is reported, all under by_pool."""
    import raccoongpurender_gb300 as rg
    from raccoongpurender_gb300 import scenes
    if which == "cornell":
        mesh, env = scenes.cornell_box(), None
        camd = scenes.cornell_camera(256, 256)
        spp, depth, dof = 4, 5, 0.0
    else:
        mesh, env, camd = scenes.mixed_scene(level=8, seed=3)
        spp, depth, dof = 64, 8, 0.0045
    sm = rg.SceneManager()
    sm.addMesh(mesh)
    if env is not None:
        sm.setEnvmap(env)
    sm.buildBVH(max_leaf_size=4)
    cam = rg.camera_look_at(camd["eye"], camd["target"], camd["up"], camd["vfov"], camd["w"], camd["h"])
    cfg = rg.render_config(spp=spp, max_depth=depth, dof=dof)
    paths = camd["w"] * camd["h"] * spp
    best, by_pool = None, {}
    for pool in pools:
        lane = rg.WavefrontLane(dev_index, pool)
        lane.setup(sm)
        pbest = None
        for _ in range(repeats + 1):  # first run warms up (graph capture, caches)
            lane.initialize(cam, cfg)
            lane.synchronize()
            t0 = time.perf_counter()
            steps = lane.render_until_done(10000)
            dt = time.perf_counter() - t0
            st = lane.stats()
            if pbest is None or dt < pbest[0]:
                pbest = (dt, steps, st, pool)
        by_pool[str(pool)] = round(paths / pbest[0] / 1e6, 1)
        if best is None or pbest[0] < best[0]:
            best = pbest
        del lane
    dt, steps, st, pool = best
    return {"ms": round(dt * 1e3, 2), "steps": steps, "mpaths_s": round(paths / dt / 1e6, 1),
            "mrays_s": round(st.rays_traced / dt / 1e6, 1), "rays": int(st.rays_traced),
            "samples_accumulated": int(st.samples_accumulated), "paths": paths, "path_pool": pool,
            "by_pool": by_pool,
            "config": f"{camd['w']}x{camd['h']}, {spp} spp, max depth {depth}, {mesh.ntris} triangles"}


# Algorithmic bytes per extension segment of the wavefront render (the state
# each stage uses, in 16-byte vectors of the slot records), traversal
# excluded.  Per shaded queue item: the item (4), request id (2), material
# reference (8), ro, rd, T, L, ng and RNG in (6 x 16) and out (6 x 16), the
# volume list in (32); the persistent trace: the item (4), ro and rd in (32),
# ng, t and the volume hit out (24); the logic: queue id (1), request id (2),
# rd, ng, T, L and RNG in (5 x 16), T, L and RNG out (3 x 16), queue id and
# queue item out (5); the new-path compaction: the queue id of a slot (1).
RENDER_STATE_BYTES = (4 + 2 + 8 + 96 + 96 + 32) + (4 + 32 + 24) + (1 + 2 + 80 + 48 + 5) + 1


def render_roofline(dev_index: int, mrays_s: float, mpaths_s: float, l2_gbs: float, hbm_gbs: float) -> dict:
    """Roofline of the mixed 1080p render: bytes per extension segment = the
    path-state traffic the stages use (RENDER_STATE_BYTES) + 64 per BVH
    node visited + 48 per primitive tested, the counts measured by the
    instrumented closest-hit kernel on the extension rays of the render's
    third bounce (2^22 resident paths).  The state streams from HBM, the tree
    from L2; both fractions are stated, against the HBM copy rate and the L2
    read rate measured in this run.  The FP64 accumulation (32 bytes per
    finished path) is counted per path."""
    import numpy as np
    import torch
    import raccoongpurender_gb300 as rg
    from raccoongpurender_gb300 import scenes
    mesh, env, camd = scenes.mixed_scene(level=8, seed=3)
    sm = rg.SceneManager()
    sm.addMesh(mesh)
    sm.setEnvmap(env)
    sm.buildBVH(max_leaf_size=4)
    cam = rg.camera_look_at(camd["eye"], camd["target"], camd["up"], camd["vfov"], camd["w"], camd["h"])
    lane = rg.WavefrontLane(dev_index, 1 << 22)
    lane.setup(sm)
    lane.initialize(cam, rg.render_config(spp=64, max_depth=8, dof=0.0045))
    lane.step(3)
    lane.synchronize()
    sl = lane.debug_slots()
    live = np.asarray(sl["queue"]) >= 0
    ro = np.asarray(sl["ro"])[live].astype(np.float32)
    rd = np.asarray(sl["rd"])[live].astype(np.float32)
    n = int(ro.shape[0])
    dev = torch.device("cuda", dev_index)
    soa = [torch.from_numpy(np.ascontiguousarray(x)).to(dev) for x in (ro[:, 0], ro[:, 1], ro[:, 2], rd[:, 0],
                                                                        rd[:, 1], rd[:, 2])]
    soa.append(torch.full((n,), 3.4028234663852886e38, dtype=torch.float32, device=dev))
    prim = torch.empty(n, dtype=torch.int32, device=dev)
    t = torch.empty(n, dtype=torch.float32, device=dev)
    nodes = torch.empty(n, dtype=torch.int32, device=dev)
    prims = torch.empty(n, dtype=torch.int32, device=dev)
    lane.trace_closest_counts_device([a.data_ptr() for a in soa], n, prim.data_ptr(), t.data_ptr(), nodes.data_ptr(),
                                     prims.data_ptr())
    lane.synchronize()
    nv, pt = float(nodes.double().mean()), float(prims.double().mean())
    trav = 64.0 * nv + 48.0 * pt
    seg = mrays_s * 1e6
    state_gbs = (seg * RENDER_STATE_BYTES + mpaths_s * 1e6 * 32) / 1e9
    trav_gbs = seg * trav / 1e9
    return {"rays_sampled": n, "nodes_per_ray": round(nv, 2), "prims_per_ray": round(pt, 2),
            "state_bytes_per_segment": RENDER_STATE_BYTES, "traversal_bytes_per_segment": round(trav, 1),
            "state_gbs": round(state_gbs, 1), "state_frac_of_hbm": round(state_gbs / hbm_gbs, 4),
            "traversal_gbs": round(trav_gbs, 1), "traversal_frac_of_l2": round(trav_gbs / l2_gbs, 4),
            "time_frac_of_bound": round((state_gbs / hbm_gbs + trav_gbs / l2_gbs), 4),
            "note": "time_frac_of_bound = state/HBM + traversal/L2: the share of the render's time that the two "
                    "streams would need at their measured peaks if they did not overlap"}


def batch_bench(dev_index: int, n: int = 32) -> dict:
    """Batched uneven requests: n requests (square side log-uniform 64..1024,
    spp log-uniform 1..256, 1k..2M triangles, full-render material mix and
    envmap, half with a volume box) rendered to completion in one shared path
    pool, shortest request first, bounce loop replayed from a CUDA graph;
    pool size, graph length, shade grid and trace refill from the autotuner."""
    import numpy as np
    import raccoongpurender_gb300 as rg
    from raccoongpurender_gb300 import autotune, scenes
    reqs = scenes.batch_requests(n)
    env = scenes.sky_envmap()
    built = []
    t0 = time.time()
    for r in reqs:
        sm = rg.SceneManager()
        sm.addMesh(r["mesh"])
        sm.setEnvmap(env)
        sm.buildBVH(max_leaf_size=4)
        c = r["camera"]
        cam = rg.camera_look_at(c["eye"], c["target"], c["up"], c["vfov"], c["w"], c["h"])
        built.append((sm, cam, rg.render_config(spp=r["spp"], max_depth=r["max_depth"])))
    setup_s = time.time() - t0
    tuned = autotune.tune_batch(built, device=dev_index, log=lambda *_: None)
    b = rg.Batch(dev_index, tuned["path_count"])
    b.set_render_tuning(tuned["shade_blocks"], tuned["graph_steps"])
    b.set_render_trace(tuned.get("render_refill", 12))
    b.set_trace_search(tuned.get("render_search", 8))
    ids = [b.add(sm, cam, cfg) for sm, cam, cfg in built]
    b.run(order=rg.ORDER_SHORTEST_FIRST, steps_per_launch=tuned["graph_steps"], max_steps=200)  # warm
    t0 = time.perf_counter()
    steps = b.run(order=rg.ORDER_SHORTEST_FIRST, steps_per_launch=tuned["graph_steps"])
    dt = time.perf_counter() - t0
    lat = np.array([b.request_stats(i).complete_ms for i in ids])
    samples = sum(b.request_stats(i).samples for i in ids)
    st = b.stats()
    return {"requests": n, "samples": int(samples), "ms": round(dt * 1e3, 1), "steps": steps,
            "mpaths_s": round(samples / dt / 1e6, 1), "mrays_s": round(st.rays_traced / dt / 1e6, 1),
            "latency_ms": {"p50": round(float(np.percentile(lat, 50)), 2),
                           "p99": round(float(np.percentile(lat, 99)), 2), "max": round(float(lat.max()), 2)},
            "triangles": int(sum(r["mesh"].ntris for r in reqs)), "autotuned": tuned,
            "setup_s": round(setup_s, 1)}


def bvh_bench(dev_index: int, mesh, sets, stream: int, sah_build_s: float) -> dict:
    """BVH construction of the closest-hit scene: the host binned-SAH builder
    (all host threads) against the linear BVH built on the GPU (Morton codes,
    radix tree, refit; host flattening into the renderer's layout), and the
    closest-hit rate on each tree (same rays, same kernel)."""
    import torch
    import raccoongpurender_gb300 as rg
    t0 = time.perf_counter()
    sm = rg.SceneManager()
    sm.addMesh(mesh)
    t1 = time.perf_counter()
    sm.buildBVH(max_leaf_size=4, builder=rg.BVH_LBVH_GPU, device=dev_index)
    t2 = time.perf_counter()
    sm2 = rg.SceneManager()
    sm2.addMesh(mesh)
    t3 = time.perf_counter()
    sm2.buildBVH(max_leaf_size=4, builder=rg.BVH_LBVH_GPU, device=dev_index)  # warm (CUDA context, allocator)
    t4 = time.perf_counter()
    lane = rg.WavefrontLane(dev_index, 1024)
    lane.setup(sm2)
    st = torch.cuda.ExternalStream(stream)
    for ptrs, n, pp, tp in sets:
        lane.trace_closest_device(ptrs, n, pp, tp, 0, stream)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(st)
    reps = 5
    for _ in range(reps):
        for ptrs, n, pp, tp in sets:
            lane.trace_closest_device(ptrs, n, pp, tp, 0, stream)
    e1.record(st)
    e1.synchronize()
    rays = sum(n for _, n, _, _ in sets) * reps
    info = sm2.info()
    return {"sah_host_s": round(sah_build_s, 3), "lbvh_gpu_s": round(t4 - t3, 3),
            "lbvh_gpu_first_call_s": round(t2 - t1, 3), "lbvh_mrays_s": round(rays / (e0.elapsed_time(e1) * 1e3), 1),
            "lbvh_depth": int(info.depth), "lbvh_sah_cost": round(float(info.sah_cost), 2),
            "lbvh_inner_nodes": int(info.num_inner_nodes)}


def guide_kernels_bench(dev_index: int, inference_kernel: int | None = None) -> dict:
    """The guiding network's kernels on 2^18 random samples, timed with CUDA
    events on the stream they run on: inference (the guide's default kernel,
    or `inference_kernel`) and one training iteration (forward + loss +
    backward + weight gradients, the gradient reduction, Adam, the iteration
    bookkeeping) for each training kernel, iterations enqueued back to back.
    FLOPs are the network's own (36-64-64-64-64-40: 34,304 per sample forward,
    2x that backward), not the zero padding the kernels also multiply; the
    tcgen05 training kernel issues 75 MMAs of 128x64x16 per 128 samples
    (forward 19, input gradients 16, weight and bias gradients 40)."""
    import numpy as np
    import torch
    import raccoongpurender_gb300 as rg
    n = 1 << 18
    fwd = 2 * (36 * 64 + 3 * 64 * 64 + 64 * 40)
    g = rg.Guide(dev_index) if inference_kernel is None else rg.Guide(dev_index, inference_kernel=inference_kernel)
    g.set_bounds((-1, -1, -1), (1, 1, 1))
    rng = np.random.default_rng(5)
    rows = np.zeros((n, 16), np.float32)
    rows[:, 0:3] = rng.uniform(-1, 1, (n, 3))
    for c in (3, 6, 9):  # normal, outgoing and incident directions
        v = rng.normal(size=(n, 3))
        rows[:, c:c + 3] = v / np.linalg.norm(v, axis=1, keepdims=True)
    rows[:, 12] = rng.uniform(0.1, 2.0, n)
    rows[:, 13] = np.maximum((rows[:, 3:6] * rows[:, 9:12]).sum(axis=1), 0.0) / np.pi  # a cosine BSDF pdf
    s = torch.from_numpy(rows).cuda(dev_index)
    out = torch.empty((n, 48), dtype=torch.float32, device=s.device)
    st = torch.cuda.Stream(device=s.device)
    sp = st.cuda_stream
    for _ in range(3):
        g.infer_device(s.data_ptr(), n, out.data_ptr(), stream=sp)
    torch.cuda.synchronize()
    reps = 20

    def timed(fn) -> float:
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(st)
        for _ in range(reps):
            fn()
        e1.record(st)
        e1.synchronize()
        return e0.elapsed_time(e1) / reps

    infer_ms = timed(lambda: g.infer_device(s.data_ptr(), n, out.data_ptr(), stream=sp))
    train = {}
    for name, kernel in (("tcgen05", rg.GUIDE_TCGEN05), ("mma_sync", rg.GUIDE_MMA_SYNC)):
        gt = rg.Guide(dev_index, training_kernel=kernel)
        gt.set_bounds((-1, -1, -1), (1, 1, 1))
        for _ in range(3):
            gt.train_device_async(s.data_ptr(), n, weight_scale=1.0 / n, stream=sp)
        torch.cuda.synchronize()
        ms = timed(lambda: gt.train_device_async(s.data_ptr(), n, weight_scale=1.0 / n, stream=sp))
        gt.check()
        train[name] = {"iteration_ms": round(ms, 4), "network_tflops": round(3 * n * fwd / ms / 1e9, 1)}
    train["tcgen05"]["mma_tflops"] = round(75 * (n / 128) * 2 * 128 * 64 * 16 / train["tcgen05"]["iteration_ms"] / 1e9, 1)
    return {"samples": n, "infer_ms": round(infer_ms, 4), "infer_tflops": round(n * fwd / infer_ms / 1e9, 1),
            "train_iteration_ms": train["tcgen05"]["iteration_ms"],
            "train_tflops": train["tcgen05"]["network_tflops"], "train_by_kernel": train,
            "note": "CUDA events around 20 iterations enqueued back to back on one stream"}


def guiding_bench(dev_index: int, w: int = 960, h: int = 540, spp: int = 256, ref_spp: int = 16384) -> dict:
    """Equal-time relMSE, guided vs plain, against a ref_spp FP64-accumulated
    plain render, at w x h: plain rendering at `spp` against guided rendering
    given the same wall time: "cold" (the guide starts untrained and trains
    online on the render's own samples for its first 120 iterations, then is
    frozen; inference and training inside the time) and "warm" (a guide
    trained online by an earlier 1024-spp render of the same view, frozen; in
    the room also by a 4096-spp render).  8 seeds: medians, means and ranges.
    Scenes: the full-render glossy/volume scene (the 1.31M-triangle sphere,
    ground, volume box, sky + sun) and the sky-lit room.  Adam's learning rate
    is the configuration's 1e-3; the same protocol at 1e-2 (measured best of
    1e-3 / 3e-3 / 1e-2 / 3e-2 for a guide trained inside the time) is
    reported beside it as `learning_rate_1e-2`."""
    import raccoongpurender_gb300 as rg
    from raccoongpurender_gb300 import guiding, scenes
    out = {}
    for name in ("glossy_volume", "sky_room"):
        if name == "glossy_volume":
            mesh, env, camd = scenes.mixed_scene(level=8, seed=3)
        else:
            mesh, env, camd = scenes.sky_room(level=6)
        sm = rg.SceneManager()
        sm.addMesh(mesh)
        sm.setEnvmap(env)
        sm.buildBVH(max_leaf_size=4)
        cam = rg.camera_look_at(camd["eye"], camd["target"], camd["up"], camd["vfov"], w, h)
        t0 = time.perf_counter()
        ref = guiding.render_mean(rg, sm, cam, spp=ref_spp, seed_offset=1 << 30, path_count=1 << 22)
        ref_s = time.perf_counter() - t0
        r = guiding.equal_time(rg, sm, cam, ref, spp, path_count=1 << 22, guide_kw=dict(max_iterations=120),
                               longer_warm_spp=(4096,) if name == "sky_room" else ())
        r2 = guiding.equal_time(rg, sm, cam, ref, spp, path_count=1 << 22,
                                guide_kw=dict(max_iterations=120, learning_rate=1e-2))
        r["learning_rate_1e-2"] = {"cold": r2["cold"], "warm": r2["warm"]}
        r.update({"resolution": f"{w}x{h}", "reference_spp": ref_spp, "reference_s": round(ref_s, 2),
                  "triangles": int(mesh.ntris)})
        out[name] = r
    return out


def scene_load_bench(repeats: int = 3) -> dict:
    """The scene front-end on the full-render scene: the 1.31M-triangle mixed
    scene (sphere, ground, volume box, per-triangle materials) written as an
    Alembic archive with a camera, then opened and built into a scene with
    rgr_alembic_open + rgr_alembic_load (parse, transform, material binding);
    best of `repeats`.  Host-side work (the reference reads its scenes on the
    host too)."""
    import tempfile
    import raccoongpurender_gb300 as rg
    from raccoongpurender_gb300 import alembic_io, materials, scenes
    mesh, _, camd = scenes.mixed_scene(level=8, seed=3)
    cols = alembic_io.columns_from_materials(materials.as_array(mesh.materials))
    with tempfile.TemporaryDirectory() as d:
        path = os.path.join(d, "mixed.abc")
        t0 = time.perf_counter()
        size = alembic_io.write_scene(path, meshes=[dict(name="mixed", P=mesh.points, indices=mesh.indices,
                                                         prims=cols)],
                                      camera=dict(ops=[("translate", camd["eye"])], resx=camd["w"], resy=camd["h"]))
        write_s = time.perf_counter() - t0
        best = None
        for _ in range(repeats):
            t0 = time.perf_counter()
            sm = rg.SceneManager()
            info = sm.addAlembic(path)
            dt = time.perf_counter() - t0
            best = dt if best is None else min(best, dt)
    return {"triangles": int(info.triangles), "file_mb": round(size / 1e6, 1), "load_s": round(best, 4),
            "mb_s": round(size / 1e6 / best, 1), "mtris_s": round(info.triangles / 1e6 / best, 2),
            "write_s": round(write_s, 2), "threads": 1}


def guided_render_cost(dev_index: int, spp: int = 64, inference_kernel: int | None = None) -> dict:
    """What a frozen guide costs per sample: the sky-lit room at 960x540
    rendered once guided while the guide trains, then plain and with the
    (now frozen) guide at the same spp; wall times of the last two.  The
    guide's default inference kernel, or `inference_kernel`."""
    import raccoongpurender_gb300 as rg
    from raccoongpurender_gb300 import guiding, scenes
    mesh, env, camd = scenes.sky_room(level=6)
    sm = rg.SceneManager()
    sm.addMesh(mesh)
    sm.setEnvmap(env)
    sm.buildBVH(max_leaf_size=4)
    cam = rg.camera_look_at(camd["eye"], camd["target"], camd["up"], camd["vfov"], 960, 540)
    lane = rg.WavefrontLane(dev_index, 1 << 22)
    lane.setup(sm)
    g = rg.Guide(dev_index) if inference_kernel is None else rg.Guide(dev_index, inference_kernel=inference_kernel)
    guiding.render(rg, sm, cam, spp, 77, guide=g, lane=lane)
    g.set_config(train=0)
    _, _, tp = guiding.render(rg, sm, cam, spp, 5, lane=lane)
    _, _, tg = guiding.render(rg, sm, cam, spp, 5, guide=g, lane=lane)
    return {"spp": spp, "plain_s": round(tp, 4), "frozen_guided_s": round(tg, 4),
            "cost_per_sample": round(tg / tp - 1.0, 3), "training_iterations": g.stats()["iterations"]}


def cpu_baseline(mesh, sm, coherent, incoherent, gpu_hits, sample: int = 1048576) -> dict:
    """The oracle traversal (kernels/extension_ray_cast_stackless.cl restated)
    on all host threads over a bounded sample: the first `sample` rays of each
    set, with the same 1:1 coherent/incoherent mix, on the tree the GPU run
    used.  Its hits are compared bit for bit with the GPU's hits of the timed
    run (`gpu_hits`: per set, prim and t on the host): the parity record."""
    import numpy as np
    from oracle import pyoracle as po
    osc = po.OracleScene.from_scene(sm, mesh.points, mesh.indices)
    threads = os.cpu_count() or 1
    idx = np.arange(sample)
    sets = [coherent.subset(idx).packed8(), incoherent.subset(idx).packed8()]
    rays = np.concatenate(sets)
    osc.trace(rays[:1024], threads=threads, normals=False)  # warm
    t0 = time.perf_counter()
    oprim, ot, _ = osc.trace(rays, threads=threads, normals=False)
    dt = time.perf_counter() - t0
    gprim = np.concatenate([h[0][:sample] for h in gpu_hits])
    gt = np.concatenate([h[1][:sample] for h in gpu_hits])
    parity = {"rays": int(rays.shape[0]), "prim_mismatch": int((gprim != oprim).sum()),
              "t_mismatch": int((gt.view(np.uint32) != ot.view(np.uint32)).sum()),
              "hits": int((oprim >= 0).sum()),
              "what": f"oracle vs GPU hits of the timed run on the first {sample} coherent + {sample} "
                      "incoherent rays, same tree; t compared as bits"}
    return {"value": round(rays.shape[0] / dt / 1e6, 3), "unit": "Mrays/s", "cores": threads, "kind": "port",
            "sample": f"{sample} coherent + {sample} incoherent rays of the same workload, {dt:.2f} s",
            "parity": parity}


def image_error(dev_index: int, which: str, ref_spp: int) -> dict:
    """The configuration's image against an FP64-accumulated render of the same
    scene at `ref_spp` samples per pixel with other seeds (the GPU's FP64
    render, which follows the oracle sample for sample): per-pixel relative
    luminance error |Y - Y_ref| / (Y_ref + 0.01) and relMSE, with the
    reference's constants (radiance discard at 1000).
    cornell: 256x256, 4 spp, depth 5; mixed: 1920x1080, 64 spp, depth 8."""
    import numpy as np
    import raccoongpurender_gb300 as rg
    from raccoongpurender_gb300 import guiding, scenes
    if which == "cornell":
        mesh, env = scenes.cornell_box(), None
        camd = scenes.cornell_camera(256, 256)
        spp, depth, dof = 4, 5, 0.0
    else:
        mesh, env, camd = scenes.mixed_scene(level=8, seed=3)
        spp, depth, dof = 64, 8, 0.0045
    sm = rg.SceneManager()
    sm.addMesh(mesh)
    if env is not None:
        sm.setEnvmap(env)
    sm.buildBVH(max_leaf_size=4)
    cam = rg.camera_look_at(camd["eye"], camd["target"], camd["up"], camd["vfov"], camd["w"], camd["h"])
    lane = rg.WavefrontLane(dev_index, 1 << 22)
    lane.setup(sm)
    imgs = []
    for n, seed in ((spp, 1), (ref_spp, 1 << 30)):
        lane.initialize(cam, rg.render_config(spp=n, max_depth=depth, dof=dof, seed_offset=seed))
        lane.render_until_done(1 << 30)
        imgs.append(guiding.mean_image(lane.accumulation()))
    w = np.array([0.2126, 0.7152, 0.0722])
    y, yr = imgs[0] @ w, imgs[1] @ w
    rel = np.abs(y - yr) / (yr + 0.01)
    return {"spp": spp, "reference_spp": ref_spp, "pixels": int(rel.size),
            "rel_err_mean": round(float(rel.mean()), 5), "rel_err_median": round(float(np.median(rel)), 5),
            "rel_err_p99": round(float(np.quantile(rel, 0.99)), 4), "rel_err_max": round(float(rel.max()), 4),
            "relmse": round(guiding.relmse(imgs[0], imgs[1]), 6),
            "note": "Monte Carlo noise of the image at its spp (the reference render's own noise is "
                    f"{spp / ref_spp:.3f} of it in variance)"}


def render_gpu_for_oracle(dev_index: int, which: str) -> dict:
    """The GPU render the CPU leg compares with: Cornell 256^2, 4 spp, depth 5
    (configuration 1, complete) and the mixed 1080p scene at 1 spp, depth 8
    (configuration 3 at reduced spp); FP64 sums per pixel."""
    import raccoongpurender_gb300 as rg
    from raccoongpurender_gb300 import scenes
    if which == "cornell":
        mesh, env, camd = scenes.cornell_box(), None, scenes.cornell_camera(256, 256)
        cfg = rg.render_config(spp=4, max_depth=5, dof=0.0)
        pool = 1 << 18  # one slot per sample: the oracle, too, walks every slot each bounce
    else:
        mesh, env, camd = scenes.mixed_scene(level=8, seed=3)
        cfg = rg.render_config(spp=1, max_depth=8, dof=0.0045)
        pool = 1 << 21
    sm = rg.SceneManager()
    sm.addMesh(mesh)
    if env is not None:
        sm.setEnvmap(env)
    sm.buildBVH(max_leaf_size=4)
    cam = rg.camera_look_at(camd["eye"], camd["target"], camd["up"], camd["vfov"], camd["w"], camd["h"])
    lane = rg.WavefrontLane(dev_index, pool)
    lane.setup(sm)
    lane.initialize(cam, cfg)
    steps = lane.render_until_done(100000)
    return dict(scene=sm, mesh=mesh, cam=cam, cfg=cfg, acc=lane.accumulation().reshape(-1, 4), steps=steps,
                pool=pool)


def cpu_render_baseline(gpu: dict, name: str) -> dict:
    """The oracle's restatement of the reference render on all host threads,
    timed, and the GPU image's largest per-pixel relative error against it."""
    import numpy as np
    from oracle import pyoracle as po
    sm, mesh, cam, cfg = gpu["scene"], gpu["mesh"], gpu["cam"], gpu["cfg"]
    osc = po.OracleScene.from_scene(sm, mesh.points, mesh.indices)
    npix = cam.image_w * cam.image_h
    threads = os.cpu_count() or 1
    t0 = time.perf_counter()
    acc, _, _ = osc.render(po.camera_from_rgr(cam), po.config_from_rgr(cfg, npix), gpu["pool"], gpu["steps"] + 4,
                           threads=threads, want_slots=False)
    dt = time.perf_counter() - t0
    g = gpu["acc"]
    rel = np.abs(g[:, :3] - acc[:, :3]) / np.maximum(np.abs(acc[:, :3]), 1e-300)
    rel[(acc[:, :3] == 0) & (g[:, :3] == 0)] = 0.0
    paths = int(acc[:, 3].sum())
    return {"value": round(paths / dt / 1e6, 3), "unit": "Mpaths/s", "cores": threads, "kind": "port",
            "sample": f"{name}: {cam.image_w}x{cam.image_h}, {int(cfg.spp)} spp, {dt:.2f} s",
            "gpu_image_vs_oracle": {"max_rel_err": float(rel.max()), "counts_equal": bool((g[:, 3] == acc[:, 3]).all()),
                                    "pixels": npix}}


def envmap_filter_record() -> dict:
    """Bound on the software bilinear envmap filter against texture-unit
    filtering with 8-bit weights (the OpenCL image the reference samples on a
    camera ray's first segment), on the full-render envmap: over 1M uniform
    directions and over the 1920x1080 camera's pixel-centre directions."""
    import numpy as np
    import raccoongpurender_gb300 as rg
    from oracle import pyoracle as po
    from raccoongpurender_gb300 import scenes
    mesh, env, camd = scenes.mixed_scene(level=3, seed=3)
    sm = rg.SceneManager()
    sm.addMesh(mesh)
    sm.setEnvmap(env)
    sm.buildBVH(max_leaf_size=4)
    osc = po.OracleScene.from_scene(sm, mesh.points, mesh.indices)
    rng = np.random.default_rng(1)
    v = rng.normal(size=(1 << 20, 3))
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    cam = rg.camera_look_at(camd["eye"], camd["target"], camd["up"], camd["vfov"], camd["w"], camd["h"])
    rays = scenes.pinhole_rays(camd["eye"], camd["target"], camd["up"], np.tan(np.radians(camd["vfov"] / 2)),
                               int(cam.image_w), int(cam.image_h))
    return {"uniform_sphere": po.envmap_filter_bound(osc, v), "camera_1080p": po.envmap_filter_bound(osc, rays.d)}


def run_reference(args) -> None:
    """The reference arm: the reference traversal restated by the oracle, on
    all host threads, over all 8,388,608 rays of the workload per step.  The
    mesh and rays come from the seeded numpy generators and the tree from the
    oracle's own builder, so no product library is loaded.  Under torchrun
    only rank 0 runs."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    import numpy as np
    from oracle import pyoracle as po
    from raccoongpurender_gb300 import scenes  # numpy generators; loads no library
    mesh = scenes.displaced_icosphere(8, seed=7)
    coherent, incoherent = scenes.closest_hit_rays(mesh, res=2048, n_random=2048 * 2048, seed=11)
    threads = os.cpu_count() or 1
    t0 = time.perf_counter()
    osc = po.OracleScene.from_mesh(mesh.points, mesh.indices, max_leaf=4, threads=threads)
    build_s = time.perf_counter() - t0
    rays = np.concatenate([coherent.packed8(), incoherent.packed8()])
    del coherent, incoherent
    n = rays.shape[0]
    for _ in range(args.warmup):
        osc.trace(rays, threads=threads, normals=False)
    times = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        osc.trace(rays, threads=threads, normals=False)
        times.append(time.perf_counter() - t0)
    ms_per_step = sum(times) / len(times) * 1e3
    v = round(n / (ms_per_step * 1e-3) / 1e6, 3)
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": "Mrays/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms_per_step, 2),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": WORKLOAD, "triangles": int(mesh.ntris), "rays_per_step": int(n),
                       "bvh": {"max_leaf": 4, "builder": "oracle binned SAH (32 bins, 1:1 costs), reference "
                                                         "stackless flattening", "nodes": int(osc.nodes.shape[0]),
                               "build_s": round(build_s, 2)},
                       "parallelism": "host threads"},
            "cpu_baseline": {"value": v, "unit": "Mrays/s", "cores": threads, "kind": "port",
                             "sample": f"all {n} rays per step (4M coherent + 4M incoherent), {args.steps} steps"},
            "e2e": {"value": v, "unit": "Mrays/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def main() -> None:
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--e2e-steps", type=int, default=3)
    ap.add_argument("--no-render", action="store_true", help="skip the full-render measurements")
    ap.add_argument("--no-guiding", action="store_true", help="skip the learned-guiding measurements")
    ap.add_argument("--traffic-bytes", type=int, default=None,
                    help="DRAM bytes per step of the closest-hit launches from an ncu capture, to attach to the "
                         "roofline record")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
        return

    import numpy as np
    import torch

    import raccoongpurender_gb300 as rg

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))

    # the roof of the closest-hit kernel, measured before any traversal has marked
    # the tree's lines evict-last in L2: the L2 read bandwidth over a buffer the
    # size of the tree, and the same probe over 4 GiB (HBM)
    mesh, sm, coherent, incoherent, build_s = build_workload()
    info0 = sm.info()
    ws_bytes = int(info0.num_inner_nodes) * 64 + int(mesh.ntris) * 48
    l2_gbs = rg.probe_read_bandwidth(local, ws_bytes, reps=5)
    hbm_read_gbs = rg.probe_read_bandwidth(local, 4 << 30, reps=3)
    n_each = len(coherent)
    lane = rg.WavefrontLane(local, 1024)
    lane.setup(sm)
    dev = torch.device("cuda", local)
    sets = []
    for rays in (coherent, incoherent):
        soa = [torch.from_numpy(a).to(dev) for a in rays.soa()]
        prim = torch.empty(len(rays), dtype=torch.int32, device=dev)
        t = torch.empty(len(rays), dtype=torch.float32, device=dev)
        sets.append((soa, prim, t, len(rays)))
    # an explicit stream: handle 0 would mean "the context's own stream" to the C ABI
    stream = torch.cuda.Stream(dev)
    torch.cuda.set_stream(stream)
    sptr = stream.cuda_stream
    assert sptr != 0

    # launch shape and BVH staging depth from the autotuner, for each ray set (coherent
    # rays prefer fewer refills than incoherent ones); results do not depend on them
    from raccoongpurender_gb300 import autotune
    set_names = ("coherent", "incoherent")
    trace_tuned, trace_trials = {}, []
    for name, (soa, prim, t, n) in zip(set_names, sets):
        tuned_k, trials_k = autotune.tune_trace(lane, [([a.data_ptr() for a in soa], n, prim.data_ptr(),
                                                        t.data_ptr())], sptr, device=local, log=lambda *_: None)
        trace_tuned[name] = tuned_k
        trace_trials += [dict(t_["params"], set=name, ms=round(t_["seconds"] * 1e3, 3)) for t_ in trials_k]

    def shape(k):
        """The launch shape tuned for ray set k (host-side settings, no device work)."""
        p = trace_tuned[set_names[k]]
        lane.set_trace_reorder(p.get("trace_reorder", 0))
        lane.set_trace_staging(p["trace_stage"])
        lane.set_trace_tuning(p["trace_refill"], 0)
        lane.set_trace_search(p["trace_search"], 0)

    def step():
        for k, (soa, prim, t, n) in enumerate(sets):
            shape(k)
            lane.trace_closest_device([a.data_ptr() for a in soa], n, prim.data_ptr(), t.data_ptr(), 0, sptr)

    # algorithmic traffic: exact node visits and primitive tests per ray
    counts = []
    for soa, prim, t, n in sets:
        nodes = torch.empty(n, dtype=torch.int32, device=dev)
        prims = torch.empty(n, dtype=torch.int32, device=dev)
        lane.trace_closest_counts_device([a.data_ptr() for a in soa], n, prim.data_ptr(), t.data_ptr(),
                                         nodes.data_ptr(), prims.data_ptr(), sptr)
        stream.synchronize()
        counts.append((float(nodes.double().mean()), float(prims.double().mean()), float((prim >= 0).double().mean())))
    bytes_per_ray = [28 + 8 + 64 * c[0] + 48 * c[1] for c in counts]
    # FP32 operations per ray: 2 slab tests of 6 subtractions, 6 multiplications and
    # 12 min/max each per inner node visited, about 40 per triangle test
    flops_per_ray = [48 * c[0] + 40 * c[1] for c in counts]

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize(dev)
    if world > 1:
        torch.distributed.barrier()

    # per-launch timing of the two ray sets (events on the launching stream)
    ev = [[torch.cuda.Event(enable_timing=True) for _ in range(3)] for _ in range(args.steps)]
    with ClockSampler(local) as clk:
        t_start = torch.cuda.Event(enable_timing=True)
        t_end = torch.cuda.Event(enable_timing=True)
        t_start.record(stream)
        for k in range(args.steps):
            ev[k][0].record(stream)
            soa, prim, t, n = sets[0]
            shape(0)
            lane.trace_closest_device([a.data_ptr() for a in soa], n, prim.data_ptr(), t.data_ptr(), 0, sptr)
            ev[k][1].record(stream)
            soa, prim, t, n = sets[1]
            shape(1)
            lane.trace_closest_device([a.data_ptr() for a in soa], n, prim.data_ptr(), t.data_ptr(), 0, sptr)
            ev[k][2].record(stream)
        t_end.record(stream)
        torch.cuda.synchronize(dev)
    clocks = clk.summary()
    total_ms = t_start.elapsed_time(t_end)
    coh_ms = sum(e[0].elapsed_time(e[1]) for e in ev) / args.steps
    inc_ms = sum(e[1].elapsed_time(e[2]) for e in ev) / args.steps
    if world > 1:
        x = torch.tensor([total_ms], device=dev)
        torch.distributed.all_reduce(x, op=torch.distributed.ReduceOp.MAX)
        total_ms = float(x.item())
    ms_per_step = total_ms / args.steps
    rays_per_step = 2 * n_each
    # the traversal kernel per set, and for a sorted set the key histogram, its scan and the scatter
    launches_per_step = sum(1 + 3 * int(trace_tuned[name].get("trace_reorder", 0)) for name in set_names)
    value = rays_per_step * world / (ms_per_step * 1e-3) / 1e6

    # end to end through the C ABI with pinned host buffers
    host = []
    for rays in (coherent, incoherent):
        soa = [torch.from_numpy(a).pin_memory() for a in rays.soa()]
        host.append((soa, len(rays)))
    out_prim = [torch.empty(n_each, dtype=torch.int32).pin_memory() for _ in range(2)]
    out_t = [torch.empty(n_each, dtype=torch.float32).pin_memory() for _ in range(2)]

    def e2e_step():
        for k, (soa, n) in enumerate(host):
            r = rg.rgr_ray_soa(*[a.data_ptr() for a in soa])
            st = lane._lib.rgr_trace_closest(lane.handle, rg.C.byref(r), n, out_prim[k].data_ptr(),
                                             out_t[k].data_ptr())
            rg._check(st, "rgr_trace_closest")

    def e2e_time() -> float:
        e2e_step()
        torch.cuda.synchronize(dev)
        t0 = time.perf_counter()
        for _ in range(args.e2e_steps):
            e2e_step()
        torch.cuda.synchronize(dev)
        return (time.perf_counter() - t0) / args.e2e_steps

    # the default: the traversal kernel reads the pinned rays and writes the hits
    # across the CPU-GPU link itself (its warps refill only when all lanes are idle,
    # so the shapes tuned for rays in device memory do not apply: the library's
    # default leaf batching); for comparison, staged copies through device buffers
    lane.set_trace_reorder(0)
    lane.set_trace_staging(0)
    lane.set_trace_tuning(24, 0)
    lane.set_trace_search(8, 0)
    lane.set_trace_host_mode(rg.TRACE_HOST_COPY)
    e2e_staged = rays_per_step / e2e_time() / 1e6
    lane.set_trace_host_mode(rg.TRACE_HOST_AUTO)
    e2e_s = e2e_time()
    e2e_value = rays_per_step / e2e_s / 1e6
    # the hits of the timed run, for the parity record of the CPU leg
    gpu_hits = [(prim.cpu().numpy(), t.cpu().numpy()) for _, prim, t, _ in sets]
    # the e2e hits must equal the device-resident hits
    assert (out_prim[0].numpy() == gpu_hits[0][0]).all() and (out_prim[1].numpy() == gpu_hits[1][0]).all()

    peaks = measured_peaks()
    coh_bytes = bytes_per_ray[0] * n_each
    inc_bytes = bytes_per_ray[1] * n_each
    achieved = (coh_bytes + inc_bytes) / ((coh_ms + inc_ms) * 1e-3) / 1e9
    # the roof: the tree (inner nodes + primitive records) is L2-resident, so the
    # denominator is the L2 read bandwidth over a buffer of its size (measured at
    # the start); the HBM read probe and the measured HBM copy rate beside it
    traffic = args.traffic_bytes
    roof = {"bound": "l2", "achieved": round(achieved, 1), "peak": round(l2_gbs, 1), "unit": "GB/s",
            "frac": round(achieved / l2_gbs, 4), "traffic": traffic,
            "peak_source": f"measured in this run: L2 read bandwidth over {ws_bytes / 1e6:.1f} MB (the tree's "
                           "inner nodes and primitive records), 16-byte loads bypassing L1",
            "hbm": {"peak": peaks["hbm_gbs"], "frac": round(achieved / peaks["hbm_gbs"], 4),
                    "source": peaks["source"] + " hbm_gbs (copy)", "read_probe_4gib_gbs": round(hbm_read_gbs, 1)},
            "traffic_note": (f"algorithmic bytes per step {int(coh_bytes + inc_bytes)}; DRAM traffic comes from an "
                             "ncu capture, not from this run (null unless --traffic-bytes gives it)"),
            "fp32": {"flops_per_ray": [round(f, 1) for f in flops_per_ray],
                     "achieved_tflops": round((flops_per_ray[0] + flops_per_ray[1]) * n_each /
                                              ((coh_ms + inc_ms) * 1e-3) / 1e12, 2),
                     "note": "48 per inner node (two slab tests), 40 per triangle; far below the SMs' FP32 "
                             "rate: the memory roof binds, and divergence (8 of 32 lanes) the kernel"},
            "per_set": {"coherent": {"ms": round(coh_ms, 3), "mrays_s": round(n_each / coh_ms / 1e3, 1),
                                     "nodes_per_ray": round(counts[0][0], 2), "prims_per_ray": round(counts[0][1], 2),
                                     "bytes_per_ray": round(bytes_per_ray[0], 1), "hit_rate": round(counts[0][2], 4)},
                        "incoherent": {"ms": round(inc_ms, 3), "mrays_s": round(n_each / inc_ms / 1e3, 1),
                                       "nodes_per_ray": round(counts[1][0], 2),
                                       "prims_per_ray": round(counts[1][1], 2),
                                       "bytes_per_ray": round(bytes_per_ray[1], 1),
                                       "hit_rate": round(counts[1][2], 4)}}}
    render = None
    if not args.no_render:
        render = {"cornell_256_4spp": render_bench(local, "cornell", pools=(1 << 18, 1 << 22)),
                  "mixed_1080p_64spp": render_bench(local, "mixed", pools=(1 << 22, 1 << 23, 1 << 24)),
                  "batch_32_requests": batch_bench(local),
                  "scene_load_alembic": scene_load_bench(),
                  "image_error_vs_fp64_reference": {"cornell_256_4spp": image_error(local, "cornell", 4096),
                                                    "mixed_1080p_64spp": image_error(local, "mixed", 1024)}}
        mx = render["mixed_1080p_64spp"]
        render["mixed_1080p_64spp"]["roofline"] = render_roofline(local, mx["mrays_s"], mx["mpaths_s"], l2_gbs,
                                                                  measured_peaks()["hbm_gbs"])
    bvh = bvh_bench(local, mesh, [([a.data_ptr() for a in soa], n, prim.data_ptr(), t.data_ptr())
                                  for soa, prim, t, n in sets], sptr, build_s) if not args.no_render else None
    guide = None
    if not args.no_guiding:
        guide = {"kernels": guide_kernels_bench(local), "cost": guided_render_cost(local),
                 "equal_time": guiding_bench(local)}
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cpu = cpu_baseline(mesh, sm, coherent, incoherent, gpu_hits)
        if not args.no_render:
            cpu["render"] = {w: cpu_render_baseline(render_gpu_for_oracle(local, w), w) for w in ("cornell", "mixed")}
        cpu["envmap_filter_bound"] = envmap_filter_record()
    info = sm.info()
    if rank == 0:
        line = {"metric": METRIC, "value": round(value, 1), "unit": "Mrays/s", "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": round(ms_per_step, 4), "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
                "config": {"workload": WORKLOAD, "triangles": int(mesh.ntris), "rays_per_step": rays_per_step,
                           "bvh": {"max_leaf": 4, "inner_nodes": int(info.num_inner_nodes),
                                   "depth": int(info.depth), "build_s": round(build_s, 2)},
                           "l2": "inputs larger than L2 (224 MB of rays per step)",
                           "autotuned": trace_tuned,
                           "autotune_trials": trace_trials,
                           "parallelism": f"replicas{world}"},
                "e2e": {"value": round(e2e_value, 1), "unit": "Mrays/s", "h2d_bytes_per_step": rays_per_step * 28,
                        "d2h_bytes_per_step": rays_per_step * 8,
                        "path": "rgr_trace_closest on page-locked host arrays: the traversal kernel reads the rays "
                                "and writes the hits across NVLink-C2C (zero copy)",
                        "staged_copies_value": round(e2e_staged, 1)},
                "gpu_launches": launches_per_step * args.steps, "roofline": roof, "cpu_baseline": cpu,
                "parity": cpu["parity"] if cpu else None, "clocks": clocks,
                "render": render, "bvh_build": bvh, "guiding": guide}
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
