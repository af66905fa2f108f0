"""Generate the golden fixtures in tests/golden/ from the reference's own
kernels (kernels/*.cl compiled unchanged through oracle/ref/clshim*.h, see
oracle/build_oracle.py).  Needs the reference sources (RGR_REFERENCE_DIR,
default /root/reference); the fixtures are committed so that tests replay
them anywhere.  Each fixture stores every input the oracle needs (geometry,
tree in the reference StacklessBVHNode layout, envmap tables, camera) next to
the reference's outputs.

    python tests/golden/make_golden.py
"""
import ctypes as C
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import raccoongpurender_gb300 as rg  # noqa: E402
from raccoongpurender_gb300 import scenes  # noqa: E402
from oracle import pyoracle as po  # noqa: E402


def scene_arrays(sm, mesh, env_rgba=None):
    nodes, ids = sm.export_stackless()
    mat, lam, ward, vol = po.reference_materials(sm.materials)
    pts = np.zeros((mesh.points.shape[0], 4), np.float32)
    pts[:, :3] = mesh.points
    d = dict(points=pts, indices=mesh.indices.reshape(-1).astype(np.uint32), nodes=nodes.view(np.uint8).reshape(-1, 96),
             prim_ids=ids, materials=mat, lambertians=lam, wards=ward, volumes=vol)
    env = sm.export_envmap()
    if env is not None:
        d.update(env_rgba=np.ascontiguousarray(sm.envmap if env_rgba is None else env_rgba, np.float32),
                 env_pdf=env["pdf"], env_height=env["height"], env_alias=env["alias"], env_frag=env["frag"],
                 env_wh=np.array([env["w"], env["h"]], np.int32))
    return d


def make_rng(ref):
    states = {}
    for off in (0, 1, 4194304):
        s = np.zeros((64, 4), np.uint32)
        ref.ref_random_initialize(po.P(s), 64, off)
        states[f"init_{off}"] = s
    st = states["init_1"][:8].copy()
    draws = np.zeros((8, 16), np.float32)
    ints = np.zeros((8, 8), np.uint64)
    for i in range(8):
        a = st[i].copy()
        ref.ref_random_uniform(po.P(a), po.P(draws[i]), 16)
        ref.ref_random_uniform_integer(po.P(a), po.P(ints[i]), 8)
    np.savez_compressed(os.path.join(HERE, "golden_rng.npz"), draws=draws, ints=ints, start=st, **states)


def make_trace(ref):
    out = {}
    for name, mesh, ray_sets in (
        ("cornell", scenes.cornell_box(), None),
        ("ico3", scenes.displaced_icosphere(3, seed=7), None),
    ):
        if not mesh.materials:
            mesh.materials = [rg.materials.lambertian()] * mesh.ntris
        sm = rg.SceneManager()
        sm.addMesh(mesh)
        sm.buildBVH(max_leaf_size=4)
        arr = scene_arrays(sm, mesh)
        if name == "cornell":
            cam = scenes.cornell_camera(48, 48)
            r1 = scenes.pinhole_rays(cam["eye"], cam["target"], cam["up"], 0.36397023426620234, 48, 48)
            r2 = scenes.random_rays(2000, (-1.1, -0.1, -1.1), (1.1, 2.1, 1.1), seed=4)
        else:
            r1, r2 = scenes.closest_hit_rays(mesh, res=48, n_random=2000, seed=4)
        rays = np.concatenate([r1.packed8(), r2.packed8()])
        rays[::7, 3] = 0.75  # some finite far clips
        n = rays.shape[0]
        prim = np.zeros(n, np.int32)
        t = np.zeros(n, np.float32)
        ng = np.zeros((n, 3), np.float32)
        nodes = arr["nodes"]
        ref.ref_trace(po.P(nodes), po.P(arr["prim_ids"]), po.P(arr["indices"]), po.P(arr["points"]),
                      mesh.ntris, po.P(np.zeros((1, 4), np.float32)), po.P(rays), n, po.P(prim), po.P(t), po.P(ng))
        for k, v in arr.items():
            out[f"{name}_{k}"] = v
        out[f"{name}_rays"] = rays
        out[f"{name}_prim"] = prim
        out[f"{name}_t"] = t
        out[f"{name}_ng"] = ng
    np.savez_compressed(os.path.join(HERE, "golden_trace.npz"), **out)


def make_render(ref, name, mesh, env_img, camd, w, h, npaths, steps):
    sm = rg.SceneManager()
    sm.addMesh(mesh)
    sm.setEnvmap(env_img)
    sm.buildBVH(max_leaf_size=4)
    zero = np.zeros_like(sm.envmap)  # the shim's image is constant radiance (0 here)
    arr = scene_arrays(sm, mesh, env_rgba=zero)
    osc = po.OracleScene.from_scene(sm, mesh.points, mesh.indices)
    osc.zero = zero
    osc.s.env_rgba = po.P(zero)
    cam = rg.camera_look_at(camd["eye"], camd["target"], camd["up"], camd["vfov"], w, h)
    ocam = po.camera_from_rgr(cam)
    slots = np.zeros(npaths, po.ORC_SLOT_DTYPE)
    acc = np.zeros((w * h, 4), np.float32)
    nxt = ref.ref_render(C.byref(osc.s), C.byref(ocam), 0, npaths, steps, po.P(np.zeros(4, np.float32)), po.P(acc),
                         po.P(slots))
    cam_arr = np.zeros(30, np.float32)
    for k, f in enumerate(("eye", "forward", "up", "right", "imageplane_o", "imageplane_r", "imageplane_b")):
        cam_arr[4 * k:4 * k + 4] = getattr(ocam, f)[:]
    cam_arr[28:30] = np.array([w, h], np.uint32).view(np.float32)
    np.savez_compressed(os.path.join(HERE, f"golden_render_{name}.npz"), camera=cam_arr,
                        meta=np.array([npaths, steps, nxt], np.uint64), slots=slots, accum=acc, **arr)


def make_accum(ref):
    rng = np.random.default_rng(9)
    n = 4096
    rgb16 = np.zeros((n, 4), np.uint16)
    vals = np.concatenate([rng.uniform(0, 2, (n - 16, 3)), np.array([[0, 1e-5, 65504]] * 16)]).astype(np.float32)
    for i in range(n):
        for k in range(3):
            rgb16[i, k] = po.lib().orc_float_to_half(float(vals[i, k]))
    rgb16[:, 3] = rng.integers(0, 60000, n)
    out8 = np.zeros((n, 4), np.uint8)
    ref.ref_tonemap(po.P(rgb16), po.P(out8), n)
    a = rgb16.copy()
    b = rgb16[::-1].copy()
    b[:, 3] = rng.integers(0, 5000, n)
    ref.ref_merge_intermediate(po.P(a), po.P(b), n)
    acc = np.zeros((n, 4), np.float32)
    acc[:, :3] = rng.uniform(0, 500, (n, 3))
    acc[:, 3] = rng.integers(0, 3000, n).astype(np.uint32).view(np.float32)
    inter = np.zeros((n, 4), np.uint16)
    ref.ref_accumlation_to_intermediate(po.P(acc), po.P(inter), n)
    np.savez_compressed(os.path.join(HERE, "golden_accum.npz"), rgb16=rgb16, rgba8=out8, merge_b=b,
                        merged=a, acc32=acc, inter=inter)


def main():
    ref = po.ref_lib()
    if ref is None:
        raise SystemExit("reference sources not found; set RGR_REFERENCE_DIR")
    make_rng(ref)
    make_trace(ref)
    env_small = scenes.sky_envmap(64, 32)
    make_render(ref, "cornell", scenes.cornell_box(), env_small, scenes.cornell_camera(), 64, 64, 4096, 30)
    mesh, _, camd = scenes.mixed_scene(level=2, seed=3, env=False)
    make_render(ref, "mixed", mesh, env_small, camd, 96, 54, 8192, 30)
    make_accum(ref)
    for f in sorted(os.listdir(HERE)):
        if f.endswith(".npz"):
            print(f, os.path.getsize(os.path.join(HERE, f)))


if __name__ == "__main__":
    main()
