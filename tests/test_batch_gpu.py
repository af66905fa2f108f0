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
