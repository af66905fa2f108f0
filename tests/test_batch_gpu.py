"""Batched requests of uneven size sharing one path pool (configuration 5):
every request's image and every slot's final state bit-identical to the
oracle's batch semantics, under both run orders."""
import numpy as np
import pytest

import raccoongpurender_gb300 as rg
from raccoongpurender_gb300 import scenes
from tests.helpers import build, camera, compare_slots

pytestmark = pytest.mark.gpu


def _requests(po):
    env = scenes.sky_envmap(64, 32)
    out = []
    m1 = scenes.cornell_box()
    sm1, os1 = build(m1)
    out.append((sm1, os1, camera(scenes.cornell_camera(), 40, 30), rg.render_config(dof=0.0, max_depth=5, spp=3)))
    m2, _, camd = scenes.mixed_scene(level=3, seed=5, env=False)
    sm2, os2 = build(m2, env=env)
    out.append((sm2, os2, camera(camd, 64, 36), rg.render_config(spp=5, max_depth=8)))
    m3 = scenes.displaced_icosphere(4, seed=9)
    sm3, os3 = build(m3, env=env)
    cam3 = dict(eye=(0, 0.3, 3.0), target=(0, 0, 0), up=(0, 1, 0), vfov=40.0)
    out.append((sm3, os3, camera(cam3, 24, 24), rg.render_config(spp=9, max_depth=3)))
    out.append((sm1, os1, camera(scenes.cornell_camera(), 16, 16), rg.render_config(dof=0.0, spp=1)))
    return out


@pytest.mark.parametrize("order", [rg.ORDER_FIFO, rg.ORDER_SHORTEST_FIRST])
def test_batch_matches_oracle(po, order):
    reqs = _requests(po)
    npaths = 1 << 12
    b = rg.Batch(0, npaths)
    ids = [b.add(sm, cam, cfg) for sm, _, cam, cfg in reqs]
    steps = b.run(order=order, steps_per_launch=4)
    run_order = sorted(ids, key=lambda i: b.request_stats(i).order)
    oaccs, oslots = po.render_batch([reqs[i][1] for i in run_order],
                                    [po.camera_from_rgr(reqs[i][2]) for i in run_order],
                                    [po.config_from_rgr(reqs[i][3], reqs[i][2].image_w * reqs[i][2].image_h)
                                     for i in run_order], npaths, steps, threads=16)
    for k, i in enumerate(run_order):
        ga = b.accumulation(i).reshape(-1, 4)
        oa = oaccs[k]
        cam, cfg = reqs[i][2], reqs[i][3]
        assert ga[:, 3].sum() <= cam.image_w * cam.image_h * cfg.spp
        assert (ga[:, 3] == oa[:, 3]).all(), f"request {i}"
        np.testing.assert_allclose(ga[:, :3], oa[:, :3], rtol=1e-12, atol=1e-300)
        st = b.request_stats(i)
        assert st.complete_ms > 0
    gs = b.debug_slots()
    assert compare_slots(gs, oslots, fields=["T", "L", "ro", "rd", "rng", "pixel_index", "queue"]) == {}
    # run order: submission order, or fewest samples first
    samples = [b.request_stats(i).samples for i in run_order]
    if order == rg.ORDER_SHORTEST_FIRST:
        assert samples == sorted(samples)
    else:
        assert run_order == ids


def test_eight_uneven_requests_with_a_million_triangle_scene(po):
    """Eight requests in the shape of the batched workload: scenes of 1.5k to
    1.2M triangles built by the batch generator (displaced spheres over a
    ground quad, the full-render material mix), every one with the sky + sun
    envmap and every other one with a homogeneous-volume box, uneven
    resolution and spp, rendered to completion in one shared pool; each
    request's image bit-identical in its counts and equal to rounding in its
    FP64 sums to the oracle's batch."""
    rng = np.random.default_rng(4)
    env = scenes.sky_envmap(256, 128)
    tris = [1_200_000, 300_000, 60_000, 8_000, 1_500, 20_000, 120_000, 3_000]
    sides = [(40, 24), (32, 32), (48, 20), (16, 16), (64, 36), (24, 40), (20, 20), (56, 28)]
    spps = [3, 2, 5, 9, 1, 4, 6, 2]
    reqs = []
    for k in range(8):
        mesh, camd = scenes.request_scene(tris[k], rng, volume=(k % 2) == 0)
        sm, osc = build(mesh, env=env)
        reqs.append((sm, osc, camera(camd, *sides[k]), rg.render_config(spp=spps[k], max_depth=8)))
    assert reqs[0][0].info().num_triangles > 1_000_000
    npaths = 1 << 13
    b = rg.Batch(0, npaths)
    ids = [b.add(sm, cam, cfg) for sm, _, cam, cfg in reqs]
    steps = b.run(order=rg.ORDER_SHORTEST_FIRST, steps_per_launch=8)
    run_order = sorted(ids, key=lambda i: b.request_stats(i).order)
    oaccs, oslots = po.render_batch([reqs[i][1] for i in run_order],
                                    [po.camera_from_rgr(reqs[i][2]) for i in run_order],
                                    [po.config_from_rgr(reqs[i][3], reqs[i][2].image_w * reqs[i][2].image_h)
                                     for i in run_order], npaths, steps, threads=16)
    for k, i in enumerate(run_order):
        ga = b.accumulation(i).reshape(-1, 4)
        oa = oaccs[k]
        cam, cfg = reqs[i][2], reqs[i][3]
        # the radiance discard (>= 1000, logic.cl:125) may drop a few sun-lit samples
        total = cam.image_w * cam.image_h * cfg.spp
        assert 0.95 * total <= ga[:, 3].sum() <= total, f"request {i} unfinished"
        assert (ga[:, 3] == oa[:, 3]).all(), f"request {i}"
        np.testing.assert_allclose(ga[:, :3], oa[:, :3], rtol=1e-12, atol=1e-300)
        assert b.request_stats(i).complete_ms > 0
    gs = b.debug_slots()
    assert compare_slots(gs, oslots, fields=["T", "L", "ro", "rd", "rng", "pixel_index", "queue"]) == {}
