"""The oracle against golden vectors produced by the reference's own kernels
(kernels/*.cl compiled unchanged; tests/golden/make_golden.py).  Every
comparison is bit-exact except FP32 (reference) vs FP64 (oracle) pixel sums."""
import ctypes as C
import os

import numpy as np
import pytest

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load(name):
    return np.load(os.path.join(GOLD, name))


def orc_scene_from(po, d, prefix=""):
    g = lambda k: d[prefix + k]  # noqa: E731
    keep = {}
    s = po.orc_scene()
    for k in ("points", "indices", "nodes", "prim_ids", "materials", "lambertians", "wards", "volumes"):
        keep[k] = np.ascontiguousarray(g(k))
    keep["spheres"] = np.zeros((1, 4), np.float32)
    s.points, s.indices = po.P(keep["points"]), po.P(keep["indices"])
    s.ntris = keep["indices"].shape[0] // 3
    s.spheres, s.nspheres, s.sphere_begin = po.P(keep["spheres"]), 0, s.ntris
    s.nodes, s.nnodes = po.P(keep["nodes"]), keep["nodes"].shape[0]
    s.prim_ids, s.nprim_ids = po.P(keep["prim_ids"]), keep["prim_ids"].shape[0]
    s.materials, s.lambertians = po.P(keep["materials"]), po.P(keep["lambertians"])
    s.wards, s.volumes = po.P(keep["wards"]), po.P(keep["volumes"])
    if prefix + "env_wh" in d:
        for k in ("env_rgba", "env_pdf", "env_height", "env_alias", "env_frag"):
            keep[k] = np.ascontiguousarray(g(k))
        s.env_w, s.env_h = (int(x) for x in g("env_wh"))
        s.env_rgba, s.env_pdf = po.P(keep["env_rgba"]), po.P(keep["env_pdf"])
        s.env_height, s.env_alias, s.env_frag = po.P(keep["env_height"]), po.P(keep["env_alias"]), po.P(keep["env_frag"])
    return s, keep


def test_rng(po):
    d = load("golden_rng.npz")
    for off in (0, 1, 4194304):
        s = np.zeros((64, 4), np.uint32)
        po.lib().orc_random_initialize(po.P(s), 64, off)
        assert (s == d[f"init_{off}"]).all()
    for i in range(8):
        a = d["start"][i].copy()
        f = np.zeros(16, np.float32)
        u = np.zeros(8, np.uint64)
        po.lib().orc_random_uniform(po.P(a), po.P(f), 16)
        po.lib().orc_random_uniform_integer(po.P(a), po.P(u), 8)
        assert (f.view(np.uint32) == d["draws"][i].view(np.uint32)).all()
        assert (u == d["ints"][i]).all()


@pytest.mark.parametrize("name", ["cornell", "ico3"])
def test_trace(po, name):
    d = load("golden_trace.npz")
    s, keep = orc_scene_from(po, d, name + "_")
    rays = np.ascontiguousarray(d[name + "_rays"])
    n = rays.shape[0]
    prim = np.zeros(n, np.int32)
    t = np.zeros(n, np.float32)
    ng = np.zeros((n, 3), np.float32)
    po.lib().orc_trace(C.byref(s), po.P(rays), n, po.P(prim), po.P(t), po.P(ng), None, None, 4)
    gp = d[name + "_prim"]
    hit = gp >= 0
    assert (prim == gp).all()
    assert (t.view(np.uint32)[hit] == d[name + "_t"].view(np.uint32)[hit]).all()
    assert (ng.view(np.uint32)[hit] == d[name + "_ng"].view(np.uint32)[hit]).all()
    # reference leaves a miss untouched: t stays the far clip
    assert (t.view(np.uint32)[~hit] == rays[~hit, 3].view(np.uint32)).all()


@pytest.mark.parametrize("name", ["cornell", "mixed"])
def test_render(po, name):
    """The reference step() sequence (wavefront_path_tracing.hpp:591-939) over
    the reference kernels vs the oracle: every slot's state bit-identical
    after 30 bounces.  The reference compiled here draws the new-path pixel
    jitter y-first (GCC operand order), which the oracle reproduces with
    new_path_y_first."""
    d = load(f"golden_render_{name}.npz")
    s, keep = orc_scene_from(po, d)
    cam_arr = d["camera"]
    cam = po.orc_camera()
    for k, f in enumerate(("eye", "forward", "up", "right", "imageplane_o", "imageplane_r", "imageplane_b")):
        getattr(cam, f)[:] = [float(x) for x in cam_arr[4 * k:4 * k + 4]]
    cam.image_w, cam.image_h = (int(x) for x in cam_arr[28:30].view(np.uint32))
    npaths, steps, nxt = (int(x) for x in d["meta"])
    cfg = po.orc_config()
    cfg.dof, cfg.rr_depth, cfg.radiance_clamp, cfg.env_select_prob = 0.0045, 25, 1000.0, 0.5
    cfg.new_path_y_first = 1
    npix = cam.image_w * cam.image_h
    acc = np.zeros((npix, 4), np.float64)
    slots = np.zeros(npaths, po.ORC_SLOT_DTYPE)
    got = po.lib().orc_render(C.byref(s), C.byref(cam), C.byref(cfg), npaths, steps, po.P(acc), po.P(slots), 4)
    assert got == nxt
    ref = d["slots"]
    for f in ref.dtype.names:
        a, b = slots[f], ref[f]
        if a.dtype.kind == "f":
            a, b = a.view(np.uint32), b.view(np.uint32)
        assert (a == b).all(), f
    racc = d["accum"]
    assert (racc[:, 3].view(np.uint32) == acc[:, 3]).all()
    np.testing.assert_allclose(racc[:, :3], acc[:, :3], rtol=2e-6, atol=1e-30)
    assert acc[:, 3].sum() > 0


def test_tonemap_and_half(po):
    d = load("golden_accum.npz")
    rgb16 = np.ascontiguousarray(d["rgb16"])
    out = np.zeros_like(d["rgba8"])
    po.lib().orc_tonemap(po.P(rgb16), rgb16.shape[0], po.P(out))
    assert (out == d["rgba8"]).all()
    # accumlation_to_intermediate on FP32 sums: mean = sum * (1/count) -> half
    acc = d["acc32"]
    cnt = acc[:, 3].view(np.uint32).astype(np.float32)
    with np.errstate(divide="ignore"):
        div = np.float32(1.0) / cnt
    div[~np.isfinite(div)] = 0
    for i in range(0, acc.shape[0], 37):
        for k in range(3):
            h = po.lib().orc_float_to_half(float(np.float32(acc[i, k]) * div[i]))
            assert h == d["inter"][i, k]
