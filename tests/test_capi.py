"""The C-ABI library loads, exports every symbol include/rgr.h declares, and
its host-side calls (scene building, BVH export, argument checks) work
without a GPU."""
import re
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]


def declared_symbols():
    text = (ROOT / "include" / "rgr.h").read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(rgr_[a-z0-9_]+)\s*\(", text)))


def test_all_symbols_exported(rg):
    lib = rg.load_library()
    names = declared_symbols()
    assert len(names) >= 29
    for n in names:
        assert hasattr(lib, n), n
    assert set(names) == set(rg._SIGS), set(names) ^ set(rg._SIGS)


def test_scene_validation(rg):
    sm = rg.SceneManager()
    P = np.zeros((3, 3), np.float32)
    with pytest.raises(rg.RgrError) as e:
        sm.addPolymesh(P, np.array([[0, 1, 5]], np.uint32), [rg.materials.lambertian()])
    assert e.value.status == -1
    P[0, 0] = np.nan
    with pytest.raises(rg.RgrError):
        sm.addPolymesh(P, np.array([[0, 1, 2]], np.uint32), [rg.materials.lambertian()])
    with pytest.raises(rg.RgrError):
        sm.addPolymesh(np.zeros((3, 3), np.float32), np.array([[0, 1, 2]], np.uint32), [dict(type=9)])
    with pytest.raises(rg.RgrError):
        sm.buildBVH(max_leaf_size=9)
    lib = rg.load_library()
    assert lib.rgr_status_string(-5) == b"device capacity check fired"


def test_export_before_build(rg):
    sm = rg.SceneManager()
    with pytest.raises(rg.RgrError) as e:
        sm.export_stackless()
    assert e.value.status == -4


def test_context_without_gpu_fails_loudly(rg):
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(rg.RgrError) as e:
        rg.WavefrontLane(0, 1024)
    assert e.value.status == -6


def test_camera_look_at(rg):
    cam = rg.camera_look_at((0, 0, 5), (0, 0, 0), (0, 1, 0), 40.0, 200, 100)
    f = np.array(cam.forward[:])
    assert np.allclose(f, [0, 0, -1])
    # pixel (w/2, h/2) looks straight ahead
    o = np.array(cam.imageplane_o[:]) + np.array(cam.imageplane_r[:]) * 100 + np.array(cam.imageplane_b[:]) * 50
    assert np.allclose(o, [0, 0, 4], atol=1e-6)
