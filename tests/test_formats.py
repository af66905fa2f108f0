"""Output formats: the RGB16 intermediate merge against the reference
kernel's own output (merge_intermediate, accumlation.cl:27-49), tonemap and
PNG round trip."""
import os

import numpy as np
import pytest

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def test_png_roundtrip(tmp_path):
    from raccoongpurender_gb300 import imageio
    rng = np.random.default_rng(1)
    img = rng.integers(0, 256, (37, 53, 4), dtype=np.uint8)
    p = tmp_path / "x.png"
    imageio.write_png(str(p), img)
    assert (imageio.read_png(str(p)) == img).all()
    imageio.write_pfm(str(tmp_path / "x.pfm"), rng.random((4, 5, 3)).astype(np.float32))
    assert os.path.getsize(tmp_path / "x.pfm") == len(b"PF\n5 4\n-1.0\n") + 4 * 5 * 3 * 4


@pytest.mark.gpu
def test_merge_intermediate_matches_reference(rg):
    torch = pytest.importorskip("torch")
    d = np.load(os.path.join(GOLD, "golden_accum.npz"))
    a = torch.from_numpy(d["rgb16"].astype(np.int16).view(np.int16)).cuda()
    b = torch.from_numpy(d["merge_b"].astype(np.int16).view(np.int16)).cuda()
    rg.merge_intermediate_device(a.data_ptr(), b.data_ptr(), d["rgb16"].shape[0])
    torch.cuda.synchronize()
    got = a.cpu().numpy().view(np.uint16)
    assert (got == d["merged"]).all()
