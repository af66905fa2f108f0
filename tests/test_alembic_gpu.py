"""A scene loaded from an Alembic file renders on the GPU exactly as the
oracle renders the same scene: the render fixture (a floor of mixed
materials, a light panel, spheres, the file's camera at 96 x 72) through
rgr_alembic_load, then a fixed-spp render whose per-pixel counts and FP64
sums match the oracle's, and bounce states that match it bit for bit."""
from pathlib import Path

import numpy as np
import pytest

from tests.helpers import compare_slots

pytestmark = pytest.mark.gpu

G = Path(__file__).resolve().parent / "golden" / "alembic"


def _load(rg, po):
    sm = rg.SceneManager()
    info = sm.addAlembic(G / "render.abc")
    sm.buildBVH()
    pts, idx, sph, _ = sm.geometry()
    osc = po.OracleScene.from_scene(sm, pts, idx, sph)
    return sm, osc, info


def test_alembic_scene_bounces_match_the_oracle(rg, po):
    sm, osc, info = _load(rg, po)
    cam = info.camera
    assert info.has_camera and (cam.image_w, cam.image_h) == (96, 72)
    cfg = rg.render_config(dof=0.0)
    lane = rg.WavefrontLane(0, 1 << 13)
    lane.setup(sm)
    lane.initialize(cam, cfg)
    lane.step(7)
    lane.synchronize()
    _, oslots, _ = osc.render(po.camera_from_rgr(cam), po.config_from_rgr(cfg, 96 * 72), 1 << 13, 7, threads=16)
    assert compare_slots(lane.debug_slots(), oslots) == {}


def test_alembic_scene_fixed_spp_render(rg, po):
    sm, osc, info = _load(rg, po)
    cam = info.camera
    cfg = rg.render_config(dof=0.0, max_depth=6, spp=2)
    lane = rg.WavefrontLane(0, 1 << 14)
    lane.setup(sm)
    lane.initialize(cam, cfg)
    steps = lane.render_until_done(1000)
    ga = lane.accumulation().reshape(-1, 4)
    oacc, _, _ = osc.render(po.camera_from_rgr(cam), po.config_from_rgr(cfg, 96 * 72), 1 << 14, steps, threads=16,
                            want_slots=False)
    assert (ga[:, 3] == oacc[:, 3]).all() and ga[:, 3].sum() == 2 * 96 * 72
    np.testing.assert_allclose(ga[:, :3], oacc[:, :3], rtol=1e-12, atol=1e-300)
    assert ga[:, :3].sum() > 0.0  # the light panel lights the floor
