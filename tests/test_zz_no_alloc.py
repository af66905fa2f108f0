"""rgr_render_noalloc: the render entry point for callers that cannot call
cudaMalloc at render time (a host application whose device memory is owned
by its own allocator and fixed at start-up, or a real-time loop that cannot
afford cudaMalloc's implicit device synchronisation).  Its path pool lives in
a fixed array inside librgr instead.  Checked against the allocating entry
points (rgr_render_begin + rgr_render_step + FP64 readback) on two calls in a
row, which also shows that leftovers in the shared array from the first call
do not leak into the second.  This file is collected last on purpose."""
import numpy as np
import pytest

from raccoongpurender_gb300 import scenes
from tests.helpers import build, camera

pytestmark = pytest.mark.gpu

NPATHS = 1 << 14
STEPS = 20


def test_noalloc_matches_allocating_path(rg, po):
    torch = pytest.importorskip("torch")
    mesh, env, camd = scenes.mixed_scene(level=3, seed=3)
    sm, _ = build(mesh, env=env)
    cam = camera(camd, 96, 54)
    cfg = rg.render_config()
    lane = rg.WavefrontLane(0, NPATHS)
    lane.setup(sm)
    lane.initialize(cam, cfg)
    lane.step(STEPS)
    lane.synchronize()
    ref = lane.accumulation().reshape(-1, 4)
    assert ref[:, 3].sum() > 0

    npix = 96 * 54
    out = torch.empty((npix, 4), dtype=torch.float64, device="cuda:0")
    for _ in range(2):
        out.fill_(-1.0)  # the call must clear its output
        torch.cuda.synchronize()
        lane.render_noalloc(cam, cfg, NPATHS, STEPS, out.data_ptr())
        got = out.cpu().numpy()
        assert (got[:, 3] == ref[:, 3]).all()
        np.testing.assert_allclose(got[:, :3], ref[:, :3], rtol=1e-12, atol=1e-300)


def test_noalloc_rejects_oversized_pool(rg):
    torch = pytest.importorskip("torch")
    sm, _ = build(scenes.cornell_box())
    lane = rg.WavefrontLane(0, 1024)
    lane.setup(sm)
    cam = camera(scenes.cornell_camera(), 16, 16)
    out = torch.empty((256, 4), dtype=torch.float64, device="cuda:0")
    with pytest.raises(rg.RgrError) as e:
        lane.render_noalloc(cam, rg.render_config(), (1 << 15) + 1, 1, out.data_ptr())
    assert e.value.status == -1
    assert "32768" in str(e.value)
