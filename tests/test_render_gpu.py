"""Wavefront render on the GPU against the oracle.  Per-slot path state
(throughput, radiance, ray, RNG state, hit record, volume list, next queue)
must be bit-identical after every number of bounces tested; per-pixel FP64
sums may differ only by summation order (relative 1e-12) and sample counts
must be equal."""
import numpy as np
import pytest

from raccoongpurender_gb300 import scenes
from tests.helpers import build, camera, compare_slots

pytestmark = pytest.mark.gpu


def _render_pair(rg, po, sm, osc, cam, cfg, npaths, steps):
    lane = rg.WavefrontLane(0, npaths)
    lane.setup(sm)
    lane.initialize(cam, cfg)
    lane.step(steps)
    lane.synchronize()
    gslots = lane.debug_slots()
    gacc = lane.accumulation().reshape(-1, 4)
    oacc, oslots, onext = osc.render(po.camera_from_rgr(cam), po.config_from_rgr(cfg, cam.image_w * cam.image_h),
                                     npaths, steps, threads=16)
    st = lane.stats()
    return lane, gslots, gacc, oslots, oacc, onext, st


@pytest.mark.parametrize("steps", [1, 2, 7, 40])
def test_cornell_slots(rg, po, steps):
    mesh = scenes.cornell_box()
    sm, osc = build(mesh)
    cam = camera(scenes.cornell_camera(), 64, 64)
    cfg = rg.render_config(dof=0.0, max_depth=0)
    lane, gs, ga, os_, oa, onext, st = _render_pair(rg, po, sm, osc, cam, cfg, 1 << 14, steps)
    assert compare_slots(gs, os_) == {}
    assert st.paths_started == onext
    assert (ga[:, 3] == oa[:, 3]).all()
    np.testing.assert_allclose(ga[:, :3], oa[:, :3], rtol=1e-12, atol=1e-300)


def test_mixed_scene_with_env_and_volume(rg, po):
    mesh, env, camd = scenes.mixed_scene(level=4, seed=3)
    sm, osc = build(mesh, env=env)
    cam = camera(camd, 160, 90)
    cfg = rg.render_config()  # reference defaults: thin lens 0.0045, RR after 25, clamp 1000
    lane, gs, ga, os_, oa, onext, st = _render_pair(rg, po, sm, osc, cam, cfg, 1 << 15, 30)
    assert compare_slots(gs, os_) == {}
    assert (ga[:, 3] == oa[:, 3]).all()
    np.testing.assert_allclose(ga[:, :3], oa[:, :3], rtol=1e-12, atol=1e-300)
    # every queue was exercised
    q = np.bincount(os_["queue"] + 1, minlength=8)
    assert (q[[1, 2, 4, 5, 6, 7]] > 0).all(), q


def test_fixed_spp_depth_limited(rg, po):
    """Configuration-1 style render: fixed spp, max depth, no envmap."""
    mesh = scenes.cornell_box()
    sm, osc = build(mesh)
    cam = camera(scenes.cornell_camera(), 32, 32)
    cfg = rg.render_config(dof=0.0, max_depth=5, spp=4)
    lane = rg.WavefrontLane(0, 1 << 12)
    lane.setup(sm)
    lane.initialize(cam, cfg)
    steps = lane.render_until_done(1000)
    ga = lane.accumulation().reshape(-1, 4)
    oacc, oslots, _ = osc.render(po.camera_from_rgr(cam), po.config_from_rgr(cfg, 32 * 32), 1 << 12, steps,
                                 threads=16)
    assert (ga[:, 3] == oacc[:, 3]).all()
    assert ga[:, 3].sum() <= 4 * 32 * 32
    np.testing.assert_allclose(ga[:, :3], oacc[:, :3], rtol=1e-12, atol=1e-300)
    assert (oslots["queue"] == -1).all()  # every slot retired
    img = lane.finalize_color()
    assert img.shape == (32, 32, 4) and (img[..., 3] == 255).all()


def test_graph_and_eager_agree(rg, po):
    mesh = scenes.cornell_box()
    sm, _ = build(mesh)
    cam = camera(scenes.cornell_camera(), 48, 48)
    out = []
    for graph in (True, False):
        lane = rg.WavefrontLane(0, 1 << 12)
        lane.set_graph_mode(graph)
        lane.setup(sm)
        lane.initialize(cam, rg.render_config(dof=0.0))
        lane.step(12)
        lane.synchronize()
        out.append(lane.debug_slots())
    for k in out[0]:
        assert (np.asarray(out[0][k]).view(np.uint32) == np.asarray(out[1][k]).view(np.uint32)).all(), k


def test_backside_env_pdf_fix(rg, po):
    """RGR_RENDER_FIX_BACKSIDE_ENV_PDF and RGR_RENDER_TWO_SIDED_LAMBERTIAN
    (the back-face sampling fixes the guided renderer always applies) on the
    mixed scene, bit-exact against the oracle with the same switches."""
    mesh, env, camd = scenes.mixed_scene(level=4, seed=3)
    sm, osc = build(mesh, env=env)
    cam = camera(camd, 96, 54)
    cfg = rg.render_config(flags=rg.RENDER_FIX_BACKSIDE_ENV_PDF | rg.RENDER_TWO_SIDED_LAMBERTIAN)
    lane, gs, ga, os_, oa, onext, st = _render_pair(rg, po, sm, osc, cam, cfg, 1 << 14, 24)
    assert compare_slots(gs, os_) == {}
    assert (ga[:, 3] == oa[:, 3]).all()
    np.testing.assert_allclose(ga[:, :3], oa[:, :3], rtol=1e-12, atol=1e-300)


def test_persistent_and_fused_trace_agree(rg, po):
    """The persistent refilling trace kernel + logic and the fused per-slot
    trace/logic kernel leave bit-identical slot state on the mixed scene."""
    mesh, env, camd = scenes.mixed_scene(level=4, seed=3)
    sm, _ = build(mesh, env=env)
    cam = camera(camd, 96, 54)
    out = []
    for persistent in (True, False):
        lane = rg.WavefrontLane(0, 1 << 14)
        lane.set_render_trace(persistent, 24)
        lane.setup(sm)
        lane.initialize(cam, rg.render_config())
        lane.step(20)
        lane.synchronize()
        out.append((lane.debug_slots(), lane.accumulation()))
    for k in out[0][0]:
        assert (np.asarray(out[0][0][k]).view(np.uint32) == np.asarray(out[1][0][k]).view(np.uint32)).all(), k
    np.testing.assert_allclose(out[0][1], out[1][1], rtol=1e-12, atol=1e-300)


def test_render_leaf_batching_agrees(rg, po):
    """The bounce's persistent trace kernel leaves bit-identical slot state for
    every leaf-batching value (1 = every lane waits for the last, 32 = lanes
    wait only when all are at a leaf); the FP64 sums agree to the rounding of
    their atomic summation order."""
    mesh, env, camd = scenes.mixed_scene(level=4, seed=3)
    sm, _ = build(mesh, env=env)
    cam = camera(camd, 96, 54)
    out = []
    for search in (1, 8, 32):
        lane = rg.WavefrontLane(0, 1 << 14)
        lane.set_render_trace(True, 12)
        lane.set_trace_search(0, search)
        lane.setup(sm)
        lane.initialize(cam, rg.render_config())
        lane.step(20)
        lane.synchronize()
        out.append((lane.debug_slots(), lane.accumulation()))
    for o in out[1:]:
        for k in out[0][0]:
            assert (np.asarray(out[0][0][k]).view(np.uint32) == np.asarray(o[0][k]).view(np.uint32)).all(), k
        np.testing.assert_allclose(out[0][1], o[1], rtol=1e-12, atol=1e-300)


def test_envmap_tables_on_gpu(rg):
    """FP64 selection weights and normalisation on the GPU: the pdf tables agree
    with the host builder (the reference's) to FP64 rounding, and each alias
    table encodes its own pdf exactly: bucket i keeps height_i and receives
    1 - height_j from every j aliased to it."""
    env = scenes.sky_envmap(256, 128)
    a = rg.SceneManager()
    a.setEnvmap(env)
    b = rg.SceneManager()
    b.setEnvmap(env)
    b.envmapTablesOnGPU(0)
    ta, tb = a.export_envmap(), b.export_envmap()
    np.testing.assert_array_equal(ta["frag"], tb["frag"])
    pa, pb = ta["pdf"].astype(np.float64), tb["pdf"].astype(np.float64)
    assert np.abs(pa - pb).max() <= 2.0 ** -22 * np.abs(pa).max()
    n = 256 * 128
    for k in range(7):
        h = tb["height"][k * n:(k + 1) * n].astype(np.float64)
        al = tb["alias"][k * n:(k + 1) * n]
        mass = h.copy()
        moved = al >= 0
        np.add.at(mass, al[moved], 1.0 - h[moved])
        mass /= n
        # pdf per solid angle x solid angle of the texel's row = probability
        y = np.arange(n) // 256
        t0, t1 = np.pi * y / 128, np.pi * (y + 1) / 128
        sr = (np.cos(t0) - np.cos(t1)) * 2 * np.pi / 256
        prob = pb[k * n:(k + 1) * n] * sr
        assert np.abs(mass - prob).max() <= 1e-6 * prob.max() + 1e-12
