"""Checkpoint / resume of a render: a render checkpointed after a few bounces
and restored into a fresh context finishes with the same samples as the
original (FP64 sums equal up to the order of their atomic additions, counts
and statistics exactly)."""
import numpy as np
import pytest

from raccoongpurender_gb300 import scenes

pytestmark = pytest.mark.gpu


def _lane(rg, sm, cam, cfg, pool):
    lane = rg.WavefrontLane(0, pool)
    lane.setup(sm)
    lane.initialize(cam, cfg)
    return lane


@pytest.mark.parametrize("which", ["cornell", "mixed"])
def test_checkpoint_resume(rg, which):
    if which == "cornell":
        mesh, env = scenes.cornell_box(), None
        camd = scenes.cornell_camera(128, 128)
        cfg = rg.render_config(spp=8, max_depth=5, dof=0.0)
    else:
        mesh, env, camd = scenes.mixed_scene(level=5, seed=3)
        camd = dict(camd, w=160, h=90)
        cfg = rg.render_config(spp=8, max_depth=8, dof=0.0045)
    sm = rg.SceneManager()
    sm.addMesh(mesh)
    if env is not None:
        sm.setEnvmap(env)
    sm.buildBVH(max_leaf_size=4)
    cam = rg.camera_look_at(camd["eye"], camd["target"], camd["up"], camd["vfov"], camd["w"], camd["h"])
    pool = 1 << 14
    a = _lane(rg, sm, cam, cfg, pool)
    a.step(3)
    state = a.checkpoint()
    a.render_until_done(10000)
    acc_a, st_a = a.accumulation(), a.stats()
    b = _lane(rg, sm, cam, cfg, pool)
    b.restore(state)
    b.render_until_done(10000)
    acc_b, st_b = b.accumulation(), b.stats()
    assert (acc_a[..., 3] == acc_b[..., 3]).all()
    np.testing.assert_allclose(acc_b[..., :3], acc_a[..., :3], rtol=1e-12, atol=1e-12)
    assert st_a.rays_traced == st_b.rays_traced and st_a.samples_accumulated == st_b.samples_accumulated
    # a checkpoint of another render shape is refused
    c = _lane(rg, sm, cam, cfg, pool * 2)
    with pytest.raises(rg.RgrError):
        c.restore(state)
