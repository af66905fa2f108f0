"""merge_from (common/wavefront_path_tracing.hpp:963-991) as rgr_accum_merge:
two lanes render the same view with disjoint seeds; merging one into the
other gives exactly the sum of their FP64 sums and of their sample counts
(one FP64 addition per element)."""
import numpy as np
import pytest

from raccoongpurender_gb300 import scenes
from tests.helpers import camera

pytestmark = pytest.mark.gpu


def test_accum_merge_adds_two_lanes(rg):
    mesh, env, camd = scenes.mixed_scene(level=4, seed=3)
    sm = rg.SceneManager()
    sm.addMesh(mesh)
    sm.setEnvmap(env)
    sm.buildBVH(max_leaf_size=4)
    cam = camera(camd, 96, 54)
    lanes, accs = [], []
    for seed in (1, 1 << 22):
        lane = rg.WavefrontLane(0, 1 << 15)
        lane.setup(sm)
        lane.initialize(cam, rg.render_config(spp=6, max_depth=8, seed_offset=seed))
        lane.render_until_done(10000)
        lanes.append(lane)
        accs.append(lane.accumulation().copy())
    assert not np.array_equal(accs[0][..., :3], accs[1][..., :3])  # different samples
    lanes[0].merge_from(lanes[1])
    merged = lanes[0].accumulation()
    assert (merged[..., 3] == accs[0][..., 3] + accs[1][..., 3]).all()
    assert (merged[..., :3] == accs[0][..., :3] + accs[1][..., :3]).all()
    # the RGBA8 image of the merged lane is the image of the merged means
    assert lanes[0].finalize_color().shape == (54, 96, 4)
