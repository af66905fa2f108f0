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


def test_checkpoint_refuses_another_render(rg):
    """A checkpoint restores only into a render of the same scene, camera and
    config: another seed, spp or camera is refused, and so is a checkpoint of a
    batch context (its sums live in the requests' own buffers)."""
    mesh = scenes.cornell_box()
    sm = rg.SceneManager()
    sm.addMesh(mesh)
    sm.buildBVH(max_leaf_size=4)
    camd = scenes.cornell_camera(64, 64)
    cam = rg.camera_look_at(camd["eye"], camd["target"], camd["up"], camd["vfov"], 64, 64)
    cfg = rg.render_config(spp=4, max_depth=5, dof=0.0)
    pool = 1 << 12
    a = _lane(rg, sm, cam, cfg, pool)
    a.step(2)
    state = a.checkpoint()
    same = _lane(rg, sm, cam, cfg, pool)
    same.restore(state)  # accepted
    cam2 = rg.camera_look_at(camd["eye"], (0.0, 0.9, 0.0), camd["up"], camd["vfov"], 64, 64)
    for other_cam, other_cfg in ((cam, rg.render_config(spp=4, max_depth=5, dof=0.0, seed_offset=7)),
                                 (cam, rg.render_config(spp=8, max_depth=5, dof=0.0)),
                                 (cam2, cfg)):
        other = _lane(rg, sm, other_cam, other_cfg, pool)
        with pytest.raises(rg.RgrError) as e:
            other.restore(state)
        assert e.value.status == -1
    b = rg.Batch(0, pool)
    b.add(sm, cam, cfg)
    b.run(steps_per_launch=4)
    lib = b._lib
    n = rg.C.c_uint64(0)
    assert lib.rgr_render_checkpoint_size(lib.rgr_batch_context(b._h), rg.C.byref(n)) == -4
