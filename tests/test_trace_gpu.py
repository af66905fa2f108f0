"""Closest-hit traversal on the GPU against the oracle: primitive id, t and
the geometric normal must be bit-identical (the reference traversal is
kernels/extension_ray_cast_stackless.cl:81-246)."""
import numpy as np
import pytest

from raccoongpurender_gb300 import scenes
from tests.conftest import bits
from tests.helpers import build

pytestmark = pytest.mark.gpu


def _check(lane, osc, rays):
    prim, t = lane.trace_closest(rays)
    oprim, ot, _ = osc.trace(rays.packed8(), threads=16)
    assert (prim == oprim).all(), f"{(prim != oprim).sum()} prim mismatches"
    assert (bits(t) == bits(ot)).all(), f"{(bits(t) != bits(ot)).sum()} t mismatches"
    return prim


def test_cornell_rays(rg, po):
    mesh = scenes.cornell_box()
    sm, osc = build(mesh)
    lane = rg.WavefrontLane(0, 1024)
    lane.setup(sm)
    cam = scenes.cornell_camera(128, 128)
    rays = scenes.pinhole_rays(cam["eye"], cam["target"], cam["up"], np.tan(np.radians(20.0)), 128, 128)
    prim = _check(lane, osc, rays)
    assert (prim >= 0).mean() > 0.5
    rnd = scenes.random_rays(50000, (-1.2, -0.2, -1.2), (1.2, 2.2, 1.2), seed=5)
    _check(lane, osc, rnd)


@pytest.mark.parametrize("leaf", [1, 4, 8])
def test_icosphere_level6(rg, po, leaf):
    mesh = scenes.displaced_icosphere(6, seed=7)
    sm, osc = build(mesh, leaf=leaf)
    lane = rg.WavefrontLane(0, 1024)
    lane.setup(sm)
    prim_rays, rnd = scenes.closest_hit_rays(mesh, res=256, n_random=65536, seed=3)
    p = _check(lane, osc, prim_rays)
    assert 0.2 < (p >= 0).mean() < 0.95
    _check(lane, osc, rnd)


def test_edge_cases(rg, po):
    """Axis-aligned rays through box faces and triangle edges (slab NaN
    handling, slab.cl:14-15), rays starting on surfaces, tmax clipping,
    zero-length directions."""
    mesh = scenes.cornell_box()
    sm, osc = build(mesh)
    lane = rg.WavefrontLane(0, 1024)
    lane.setup(sm)
    g = np.linspace(-1.0, 1.0, 41, dtype=np.float32)
    o, d = [], []
    for x in g:
        for z in g:
            o.append((x, 1.0, z)); d.append((0.0, -1.0, 0.0))   # straight down onto the floor and box tops
            o.append((x, 0.0, z)); d.append((0.0, 1.0, 0.0))    # starting on the floor plane
            o.append((-1.0, 1.0, z)); d.append((1.0, 0.0, 0.0)) # starting on the left wall
            o.append((x, 2.0, -1.0)); d.append((0.0, -1.0, 0.0))  # along the back/ceiling edge
    o.append((0.0, 1.0, 0.0)); d.append((0.0, 0.0, 0.0))
    o = np.array(o, np.float32)
    d = np.array(d, np.float32)
    tmax = np.full(len(o), 3.4028235e38, np.float32)
    tmax[::3] = 0.5
    rays = scenes.Rays(o, d, tmax)
    _check(lane, osc, rays)


def test_empty_scene(rg):
    sm = rg.SceneManager()
    sm.buildBVH()
    lane = rg.WavefrontLane(0, 1024)
    lane.setup(sm)
    rays = scenes.random_rays(1000, (-1, -1, -1), (1, 1, 1), seed=1)
    prim, t = lane.trace_closest(rays)
    assert (prim == -1).all()
    assert (bits(t) == bits(rays.tmax)).all()


@pytest.mark.parametrize("search,refill", [(1, 1), (1, 32), (3, 24), (8, 16), (32, 8), (32, 32)])
def test_leaf_batching(rg, po, search, refill):
    """A warp's lanes that reached a leaf wait while at least `search` others
    still search (1: all wait for the last); every value gives the same hits,
    on rays in device memory and on host arrays."""
    import torch
    mesh = scenes.displaced_icosphere(6, seed=7)
    sm, osc = build(mesh)
    lane = rg.WavefrontLane(0, 1024)
    lane.setup(sm)
    lane.set_trace_tuning(refill, 0)
    lane.set_trace_search(search, 0)
    prim_rays, rnd = scenes.closest_hit_rays(mesh, res=128, n_random=32768, seed=6)
    for rays in (prim_rays, rnd):
        _check(lane, osc, rays)
        dev = torch.device("cuda", 0)
        soa = [torch.from_numpy(a).to(dev) for a in rays.soa()]
        prim = torch.empty(len(rays), dtype=torch.int32, device=dev)
        t = torch.empty(len(rays), dtype=torch.float32, device=dev)
        lane.trace_closest_device([a.data_ptr() for a in soa], len(rays), prim.data_ptr(), t.data_ptr(), 0, 0)
        lane.synchronize()
        oprim, ot, _ = osc.trace(rays.packed8(), threads=16)
        assert (prim.cpu().numpy() == oprim).all()
        assert (bits(t.cpu().numpy()) == bits(ot)).all()


def _device_hits(lane, rays):
    import torch
    dev = torch.device("cuda", 0)
    soa = [torch.from_numpy(np.ascontiguousarray(a)).to(dev) for a in rays.soa()]
    prim = torch.full((len(rays),), -7, dtype=torch.int32, device=dev)
    t = torch.zeros(len(rays), dtype=torch.float32, device=dev)
    torch.cuda.synchronize()  # the context stream does not wait for torch's stream
    lane.trace_closest_device([a.data_ptr() for a in soa], len(rays), prim.data_ptr(), t.data_ptr(), 0, 0)
    lane.synchronize()
    return prim.cpu().numpy(), t.cpu().numpy()


@pytest.mark.parametrize("n", [1, 31, 33, 4097, 65537])
def test_ray_reorder(rg, po, n):
    """Rays sorted by origin and direction before the traversal: every ray's
    hit is the oracle's, written at its own index, for ragged counts, rays
    starting outside the scene's box (their key coordinates clamp), camera
    rays (many share a key) and zero or non-finite directions."""
    mesh = scenes.displaced_icosphere(6, seed=7)
    sm, osc = build(mesh)
    lane = rg.WavefrontLane(0, 1024)
    lane.setup(sm)
    lane.set_trace_reorder(1)
    prim_rays, _ = scenes.closest_hit_rays(mesh, res=128, n_random=16, seed=6)
    far = scenes.random_rays(n, (-4.0, -4.0, -4.0), (4.0, 4.0, 4.0), seed=n)
    o = np.concatenate([far.o, prim_rays.o[: 2 * n]])
    d = np.concatenate([far.d, prim_rays.d[: 2 * n]])
    d[::97] = 0.0
    d[5::101, 1] = np.inf
    tmax = np.concatenate([far.tmax, prim_rays.tmax[: 2 * n]])
    tmax[::7] = 0.75
    rays = scenes.Rays(o.astype(np.float32), d.astype(np.float32), tmax.astype(np.float32))
    prim, t = _device_hits(lane, rays)
    oprim, ot, _ = osc.trace(rays.packed8(), threads=16)
    assert (prim == oprim).all(), f"{(prim != oprim).sum()} prim mismatches"
    # an infinite direction can give a hit at t = NaN, whose bits are the
    # platform's default NaN on the host: any NaN matches any NaN
    same = (bits(t) == bits(ot)) | (np.isnan(t) & np.isnan(ot))
    assert same.all(), f"{(~same).sum()} t mismatches"
    lane.set_trace_reorder(0)
    p0, t0 = _device_hits(lane, rays)
    assert (p0 == prim).all() and (bits(t0) == bits(t)).all()


def test_ray_reorder_one_bucket(rg, po):
    """70,000 rays with one key (the same origin, directions within a few
    degrees) and a ragged tail of others: one bucket holds almost all rays,
    warps count whole runs of equal keys at once."""
    mesh = scenes.displaced_icosphere(6, seed=7)
    sm, osc = build(mesh)
    lane = rg.WavefrontLane(0, 1024)
    lane.setup(sm)
    lane.set_trace_reorder(1)
    rng = np.random.default_rng(3)
    n = 70000
    o = np.tile(np.array([[0.0, 0.2, 3.0]], np.float32), (n, 1))
    d = np.array([0.0, -0.05, -1.0]) + 0.02 * rng.standard_normal((n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    tail = scenes.random_rays(77, (-1.0, -1.0, -1.0), (1.0, 1.0, 1.0), seed=4)
    rays = scenes.Rays(np.concatenate([o, tail.o]).astype(np.float32), np.concatenate([d, tail.d]).astype(np.float32),
                       np.concatenate([np.full(n, 3.4028235e38, np.float32), tail.tmax]))
    prim, t = _device_hits(lane, rays)
    oprim, ot, _ = osc.trace(rays.packed8(), threads=16)
    assert (prim == oprim).all(), f"{(prim != oprim).sum()} prim mismatches"
    assert (bits(t) == bits(ot)).all(), f"{(bits(t) != bits(ot)).sum()} t mismatches"
    assert (prim[:n] >= 0).mean() > 0.5


def test_ray_reorder_range(rg):
    lane = rg.WavefrontLane(0, 1024)
    for bad in (-1, 2):
        with pytest.raises(RuntimeError):
            lane.set_trace_reorder(bad)


def test_trace_search_range(rg):
    lane = rg.WavefrontLane(0, 1024)
    for bad in ((-1, 8), (33, 8), (8, 33), (8, -1)):
        with pytest.raises(RuntimeError):
            lane.set_trace_search(*bad)
    lane.set_trace_search(0, 0)  # 0 leaves both unchanged


@pytest.mark.parametrize("stage", [1, 100, 1024])
def test_staged_top_levels(rg, po, stage):
    """Top BVH levels read from shared memory give the same hits."""
    mesh = scenes.displaced_icosphere(6, seed=7)
    sm, osc = build(mesh)
    lane = rg.WavefrontLane(0, 1024)
    lane.setup(sm)
    lane.set_trace_staging(stage)
    prim_rays, rnd = scenes.closest_hit_rays(mesh, res=128, n_random=32768, seed=4)
    _check(lane, osc, prim_rays)
    _check(lane, osc, rnd)


def test_lbvh_built_on_gpu(rg, po):
    """A linear BVH built on the GPU: hits bit-exact against the oracle on the
    same tree (rays in their order and sorted first); the same closest t as the
    SAH tree for every ray (the primitive may differ only where two primitives
    tie at that t)."""
    mesh = scenes.displaced_icosphere(6, seed=7)
    sm = rg.SceneManager()
    sm.addMesh(mesh)
    sm.buildBVH(max_leaf_size=4, builder=rg.BVH_LBVH_GPU, device=0)
    osc = po.OracleScene.from_scene(sm, mesh.points, mesh.indices)
    lane = rg.WavefrontLane(0, 1024)
    lane.setup(sm)
    prim_rays, rnd = scenes.closest_hit_rays(mesh, res=128, n_random=32768, seed=4)
    p1 = _check(lane, osc, prim_rays)
    p2 = _check(lane, osc, rnd)
    lane.set_trace_reorder(1)  # the same hits with the rays sorted first
    ps, ts = _device_hits(lane, rnd)
    lane.set_trace_reorder(0)
    _, ot, _ = osc.trace(rnd.packed8(), threads=16, normals=False)
    assert (ps == p2).all() and (bits(ts) == bits(ot)).all()
    info = sm.info()
    assert info.depth <= 63 and info.num_leaves > 0
    sah, _ = build(mesh, leaf=4)
    lane2 = rg.WavefrontLane(0, 1024)
    lane2.setup(sah)
    for rays, p in ((prim_rays, p1), (rnd, p2)):
        q, t = lane2.trace_closest(rays)
        _, t1 = lane.trace_closest(rays)
        assert (bits(t) == bits(t1)).all()
        assert (q == p).mean() > 0.999


@pytest.mark.parametrize("mode,pinned", [("copy", False), ("copy", True), ("auto", False), ("auto", True)])
def test_host_api(rg, po, mode, pinned):
    """rgr_trace_closest with host arrays, both ways: chunks of 2^20 through
    device buffers on four streams (a ragged count spanning several chunks),
    and zero copy, the kernel reading and writing host memory (page-locked
    arrays, or any where the GPU uses the host's page tables; otherwise the
    copies).  The hits equal those of the device-array entry point."""
    torch = pytest.importorskip("torch")
    mesh = scenes.displaced_icosphere(5, seed=7)
    sm, _ = build(mesh)
    lane = rg.WavefrontLane(0, 1024)
    lane.setup(sm)
    lane.set_trace_host_mode(rg.TRACE_HOST_COPY if mode == "copy" else rg.TRACE_HOST_AUTO)
    rays = scenes.random_rays(2_500_017, (-1.3, -1.3, -1.3), (1.3, 1.3, 1.3), seed=9)
    host = [torch.from_numpy(np.ascontiguousarray(a)) for a in rays.soa()]
    if pinned:
        host = [a.pin_memory() for a in host]
    hp = torch.full((len(rays),), -7, dtype=torch.int32)
    ht = torch.zeros(len(rays), dtype=torch.float32)
    if pinned:
        hp, ht = hp.pin_memory(), ht.pin_memory()
    r = rg.rgr_ray_soa(*[a.data_ptr() for a in host])
    rg._check(lane._lib.rgr_trace_closest(lane.handle, rg.C.byref(r), len(rays), hp.data_ptr(), ht.data_ptr()), "t")
    soa = [a.cuda() for a in host]
    p2 = torch.empty(len(rays), dtype=torch.int32, device="cuda")
    t2 = torch.empty(len(rays), dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()  # the context stream does not wait for torch's stream
    lane.trace_closest_device([a.data_ptr() for a in soa], len(rays), p2.data_ptr(), t2.data_ptr())
    lane.synchronize()
    assert (hp.numpy() == p2.cpu().numpy()).all()
    assert (bits(ht.numpy()) == bits(t2.cpu().numpy())).all()


def test_headline_scale_level8(rg, po):
    """The closest-hit workload itself: the 1,310,720-triangle level-8
    displaced icosphere with its SAH tree (leaves of at most 4), and every
    16th ray of the 2048x2048 coherent and the 4M incoherent ray sets
    (262,144 of each), traced through the host entry point and through the
    device entry point with the autotuned refill threshold, the rays in their
    own order and sorted by origin and direction."""
    import torch
    mesh = scenes.displaced_icosphere(8, seed=7)
    assert mesh.ntris == 1310720
    sm, osc = build(mesh, leaf=4)
    lane = rg.WavefrontLane(0, 1024)
    lane.setup(sm)
    coherent, incoherent = scenes.closest_hit_rays(mesh, res=2048, n_random=2048 * 2048, seed=11)
    idx = np.arange(0, 2048 * 2048, 16)
    for rays in (coherent.subset(idx), incoherent.subset(idx)):
        assert len(rays) == 262144
        p = _check(lane, osc, rays)
        assert 0.3 < (p >= 0).mean() < 0.99
        soa = [torch.from_numpy(np.ascontiguousarray(a)).cuda() for a in rays.soa()]
        dprim = torch.empty(len(rays), dtype=torch.int32, device="cuda")
        dt = torch.empty(len(rays), dtype=torch.float32, device="cuda")
        lane.set_trace_tuning(refill=24)
        oprim, ot, _ = osc.trace(rays.packed8(), threads=16, normals=False)
        for reorder in (0, 1):
            lane.set_trace_reorder(reorder)
            dprim.fill_(-7)
            lane.trace_closest_device([a.data_ptr() for a in soa], len(rays), dprim.data_ptr(), dt.data_ptr())
            lane.synchronize()
            assert (dprim.cpu().numpy() == p).all()
            assert (bits(dt.cpu().numpy()) == bits(ot)).all()
        lane.set_trace_reorder(0)
