"""Sphere primitives (extension_ray_cast_stackless.cl:52-76, 161-177,
scene_manager.hpp:372-431): traversal and rendering with mixed triangle and
sphere leaves, bit-identical to the oracle."""
import numpy as np
import pytest

from raccoongpurender_gb300 import scenes
from tests.conftest import bits
from tests.helpers import camera, compare_slots

pytestmark = pytest.mark.gpu


def _scene(rg, po):
    mesh = scenes.cornell_box()
    rng = np.random.default_rng(4)
    n = 40
    xyzr = np.zeros((n, 4), np.float32)
    xyzr[:, 0] = rng.uniform(-0.8, 0.8, n)
    xyzr[:, 1] = rng.uniform(0.1, 1.8, n)
    xyzr[:, 2] = rng.uniform(-0.8, 0.8, n)
    xyzr[:, 3] = rng.uniform(0.03, 0.15, n)
    mats = [rg.materials.lambertian(r=(0.6, 0.6, 0.3)) if i % 3 else rg.materials.dielectric() for i in range(n)]
    sm = rg.SceneManager()
    sm.addMesh(mesh)
    sm.addSpheres(xyzr, mats)
    sm.buildBVH(max_leaf_size=4)
    osc = po.OracleScene.from_scene(sm, mesh.points, mesh.indices, spheres=xyzr)
    return sm, osc


def test_sphere_trace(rg, po):
    sm, osc = _scene(rg, po)
    lane = rg.WavefrontLane(0, 1024)
    lane.setup(sm)
    camd = scenes.cornell_camera()
    rays = scenes.pinhole_rays(camd["eye"], camd["target"], camd["up"], np.tan(np.radians(20.0)), 96, 96)
    rnd = scenes.random_rays(20000, (-1.0, 0.0, -1.0), (1.0, 2.0, 1.0), seed=3)
    for r in (rays, rnd):
        prim, t = lane.trace_closest(r)
        oprim, ot, _ = osc.trace(r.packed8())
        assert (prim == oprim).all() and (bits(t) == bits(ot)).all()
        assert (prim >= 36).any()  # some sphere hits


def test_sphere_trace_sorted(rg, po):
    """Rays in device memory sorted by origin and direction before the
    traversal: the same hits, sphere leaves included."""
    import torch
    sm, osc = _scene(rg, po)
    lane = rg.WavefrontLane(0, 1024)
    lane.setup(sm)
    lane.set_trace_reorder(1)
    rnd = scenes.random_rays(20000, (-1.0, 0.0, -1.0), (1.0, 2.0, 1.0), seed=8)
    soa = [torch.from_numpy(a).cuda() for a in rnd.soa()]
    prim = torch.empty(len(rnd), dtype=torch.int32, device="cuda")
    t = torch.empty(len(rnd), dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()  # the context stream does not wait for torch's stream
    lane.trace_closest_device([a.data_ptr() for a in soa], len(rnd), prim.data_ptr(), t.data_ptr())
    lane.synchronize()
    oprim, ot, _ = osc.trace(rnd.packed8())
    p = prim.cpu().numpy()
    assert (p == oprim).all() and (bits(t.cpu().numpy()) == bits(ot)).all()
    assert (p >= 36).any()


def test_sphere_render(rg, po):
    sm, osc = _scene(rg, po)
    cam = camera(scenes.cornell_camera(), 64, 64)
    cfg = rg.render_config(dof=0.0)
    lane = rg.WavefrontLane(0, 1 << 13)
    lane.setup(sm)
    lane.initialize(cam, cfg)
    lane.step(20)
    lane.synchronize()
    gs = lane.debug_slots()
    ga = lane.accumulation().reshape(-1, 4)
    oa, os_, _ = osc.render(po.camera_from_rgr(cam), po.config_from_rgr(cfg, 64 * 64), 1 << 13, 20, threads=16)
    assert compare_slots(gs, os_) == {}
    assert (ga[:, 3] == oa[:, 3]).all()
    np.testing.assert_allclose(ga[:, :3], oa[:, :3], rtol=1e-12, atol=1e-300)
