"""ctypes binding of the CPU oracle (test infrastructure only).

Imported by tests/, __graft_entry__.smoke() and bench.py's CPU baseline, never
by the product package.  ``OracleScene.from_scene`` builds the oracle's view
of a scene from the inputs given to the product (points, indices, per
primitive materials, envmap image) plus the tree the product built, exported
in the reference StacklessBVHNode layout.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

from . import build_oracle

HERE = Path(__file__).resolve().parent

ORC_SLOT_DTYPE = np.dtype([("T", "<f4", 3), ("L", "<f4", 3), ("ro", "<f4", 3), ("rd", "<f4", 3),
                           ("logic_i", "<u4"), ("pixel_index", "<u4"), ("rng", "<u4", 4), ("hit_surface", "<i4"),
                           ("hit_volume", "<i4"), ("tmin", "<f4"), ("Ng", "<f4", 3), ("queue", "<i4"),
                           ("vol_count", "<i4"), ("vols", "<i4", 7)])
assert ORC_SLOT_DTYPE.itemsize == 33 * 4


class orc_scene(C.Structure):
    _fields_ = [("points", C.c_void_p), ("indices", C.c_void_p), ("ntris", C.c_uint32), ("spheres", C.c_void_p),
                ("nspheres", C.c_uint32), ("sphere_begin", C.c_int32), ("nodes", C.c_void_p), ("nnodes", C.c_uint32),
                ("prim_ids", C.c_void_p), ("nprim_ids", C.c_uint32), ("materials", C.c_void_p),
                ("lambertians", C.c_void_p), ("wards", C.c_void_p), ("volumes", C.c_void_p),
                ("env_rgba", C.c_void_p), ("env_w", C.c_int32), ("env_h", C.c_int32), ("env_pdf", C.c_void_p),
                ("env_height", C.c_void_p), ("env_alias", C.c_void_p), ("env_frag", C.c_void_p)]


class orc_camera(C.Structure):
    _fields_ = [("eye", C.c_float * 4), ("forward", C.c_float * 4), ("up", C.c_float * 4), ("right", C.c_float * 4),
                ("imageplane_o", C.c_float * 4), ("imageplane_r", C.c_float * 4), ("imageplane_b", C.c_float * 4),
                ("image_w", C.c_uint32), ("image_h", C.c_uint32)]


class orc_config(C.Structure):
    _fields_ = [("dof", C.c_float), ("rr_depth", C.c_int32), ("radiance_clamp", C.c_float),
                ("env_select_prob", C.c_float), ("max_depth", C.c_int32), ("seed_offset", C.c_uint32),
                ("sample_limit", C.c_uint64), ("new_path_y_first", C.c_int32), ("fix_backside_env_pdf", C.c_int32),
                ("two_sided_lambertian", C.c_int32)]


_lib = None
_ref = None

VP, U64, I32, U32, F32C = C.c_void_p, C.c_uint64, C.c_int32, C.c_uint32, C.c_float
_ORC_SIGS = {
    "orc_random_initialize": (None, [VP, U64, U64]),
    "orc_random_uniform": (None, [VP, VP, I32]),
    "orc_random_uniform_integer": (None, [VP, VP, I32]),
    "orc_trace": (None, [VP, VP, U64, VP, VP, VP, VP, VP, I32]),
    "orc_envmap_build": (I32, [VP, I32, I32, VP, VP, VP, VP]),
    "orc_build_bvh": (C.c_int64, [VP, VP, U32, VP, U32, I32, I32, I32, VP, U64, VP, U64]),
    "orc_render": (U64, [VP, VP, VP, U32, I32, VP, VP, I32]),
    "orc_render_batch": (U64, [VP, VP, VP, VP, VP, I32, U32, I32, VP, VP, I32]),
    "orc_intermediate": (None, [VP, U64, VP]),
    "orc_tonemap": (None, [VP, U64, VP]),
    "orc_float_to_half": (C.c_uint16, [F32C]),
    "orc_half_to_float": (F32C, [C.c_uint16]),
    "orc_cosine_hemisphere": (None, [F32C, F32C, VP]),
    "orc_uniform_sphere": (None, [F32C, F32C, VP]),
    "orc_sample_from_fragment": (None, [VP, VP, VP]),
    "orc_orthonormal_basis": (None, [VP, VP, VP]),
    "orc_sample_ward": (None, [VP, VP, F32C, F32C, F32C, VP]),
    "orc_pdf_ward": (F32C, [VP, VP, VP, F32C]),
    "orc_envmap_value": (None, [VP, VP, I32, VP]),
    "orc_envmap_index": (I32, [VP, I32, I32]),
    "orc_envmap_filter_compare": (None, [VP, VP, U64, I32, VP, VP]),
    "orc_fm": (F32C, [I32, F32C, F32C]),
}
_REF_SIGS = {
    "ref_random_initialize": (None, [VP, U64, U32]),
    "ref_random_uniform": (None, [VP, VP, I32]),
    "ref_random_uniform_integer": (None, [VP, VP, I32]),
    "ref_trace": (None, [VP, VP, VP, VP, I32, VP, VP, U64, VP, VP, VP]),
    "ref_render": (U64, [VP, VP, U32, U32, I32, VP, VP, VP]),
    "ref_alias_method": (U32, [VP, VP, U32]),
    "ref_sample_envmap_6axis": (None, [VP, VP, VP, VP, VP, VP, U32]),
    "ref_envmap_index": (I32, [VP, I32, I32]),
    "ref_envmap_pdf_six_axis": (F32C, [VP, VP, VP, I32, I32]),
    "ref_pdf_ward": (F32C, [VP, VP, VP, F32C]),
    "ref_accumlation_to_intermediate": (None, [VP, VP, U64]),
    "ref_merge_intermediate": (None, [VP, VP, U64]),
    "ref_tonemap": (None, [VP, VP, U64]),
    "ref_stat": (None, [VP, VP, U64]),
}


def _bind(l: C.CDLL, sigs: dict) -> None:
    for name, (res, args) in sigs.items():
        fn = getattr(l, name)
        fn.restype = res
        fn.argtypes = args


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        _lib = C.CDLL(str(build_oracle.build_oracle()))
        _bind(_lib, _ORC_SIGS)
    return _lib


def ref_lib() -> C.CDLL | None:
    """The reference kernels compiled from source (None where the reference
    sources are not available)."""
    global _ref
    if _ref is None:
        p = build_oracle.build_ref()
        if p is None or not Path(p).exists():
            return None
        _ref = C.CDLL(str(p))
        _bind(_ref, _REF_SIGS)
    return _ref


def P(a: np.ndarray | None) -> int | None:
    return None if a is None else a.ctypes.data


def reference_materials(mats):
    """MaterialStorage layout (scene_manager.hpp:106-172): per-primitive (type,
    index) and the per-type arrays in the reference structs.  `mats` is the
    per-primitive material array of the scene (MATERIAL_DTYPE)."""
    from raccoongpurender_gb300 import materials as M
    a = M.as_array(mats)
    n = a.shape[0]
    ref = np.zeros((max(n, 1), 2), np.int32)
    t = a["type"].astype(np.int32)
    ref[:n, 0] = t
    for k in (1, 2, 3, 4, 5):
        sel = t == k
        ref[:n, 1][sel] = np.arange(sel.sum(), dtype=np.int32)
    la, wa, va = a[t == 1], a[t == 4], a[t == 5]
    lam = np.zeros((max(len(la), 1), 12), np.float32)
    lam[:len(la), 0:3] = la["le"]
    lam[:len(la), 4:7] = la["r"]
    ward = np.zeros((max(len(wa), 1), 16), np.float32)
    ward[:len(wa), 0] = wa["alpha"]
    ward[:len(wa), 4:7] = wa["r"]
    ward[:len(wa), 8:11] = wa["edgetint"]
    ward[:len(wa), 12] = wa["falloff"]
    vol = np.zeros((max(len(va), 1), 8), np.float32)
    vol[:len(va), 0] = va["c"]
    vol[:len(va), 4:7] = va["r"]
    return ref, lam, ward, vol


class OracleScene:
    """Arrays kept alive for the orc_scene struct."""

    def __init__(self):
        self.s = orc_scene()

    @classmethod
    def from_scene(cls, sm, points, indices, spheres=None):
        o = cls()
        pts = np.zeros((points.shape[0], 4), np.float32)
        pts[:, :3] = points
        o.points = pts
        o.indices = np.ascontiguousarray(indices, np.uint32).reshape(-1)
        o.spheres = np.ascontiguousarray(spheres, np.float32) if spheres is not None else np.zeros((1, 4), np.float32)
        ntri = o.indices.shape[0] // 3
        nsph = 0 if spheres is None else spheres.shape[0]
        o.nodes, o.prim_ids = sm.export_stackless()
        o.mat, o.lam, o.ward, o.vol = reference_materials(sm.materials)
        s = o.s
        s.points, s.indices, s.ntris = P(o.points), P(o.indices), ntri
        s.spheres, s.nspheres, s.sphere_begin = P(o.spheres), nsph, ntri
        s.nodes, s.nnodes = P(o.nodes), o.nodes.shape[0]
        s.prim_ids, s.nprim_ids = P(o.prim_ids), o.prim_ids.shape[0]
        s.materials, s.lambertians, s.wards, s.volumes = P(o.mat), P(o.lam), P(o.ward), P(o.vol)
        env = sm.export_envmap()
        if env is not None:
            o.env_rgba = np.ascontiguousarray(sm.envmap, np.float32)
            o.env = env
            s.env_rgba, s.env_w, s.env_h = P(o.env_rgba), env["w"], env["h"]
            s.env_pdf, s.env_height, s.env_alias, s.env_frag = (P(env["pdf"]), P(env["height"]), P(env["alias"]),
                                                                P(env["frag"]))
        return o

    @classmethod
    def from_mesh(cls, points, indices, max_leaf: int = 4, bins: int = 32, threads: int = 8):
        """Traversal-only view of a triangle mesh with a tree the oracle builds
        itself (orc_build_bvh: binned SAH flattened as create_stackless_bvh
        does), so that no product code is involved.  Materials are unset:
        for closest-hit queries only."""
        o = cls()
        pts = np.zeros((points.shape[0], 4), np.float32)
        pts[:, :3] = points
        o.points = pts
        o.indices = np.ascontiguousarray(indices, np.uint32).reshape(-1)
        ntri = o.indices.shape[0] // 3
        o.spheres = np.zeros((1, 4), np.float32)
        cap = 2 * ntri
        nodes = np.zeros((cap, 24), np.uint32)
        prim_ids = np.zeros(ntri, np.uint32)
        nn = lib().orc_build_bvh(P(o.points), P(o.indices), ntri, P(o.spheres), 0, max_leaf, bins, threads,
                                 P(nodes), cap, P(prim_ids), ntri)
        if nn <= 0:
            raise ValueError("orc_build_bvh rejected its arguments")
        o.nodes = np.ascontiguousarray(nodes[:nn])
        del nodes
        o.prim_ids = prim_ids
        o.mat = np.zeros((max(ntri, 1), 2), np.int32)
        o.mat[:, 0] = 1
        o.lam = np.zeros((1, 12), np.float32)
        o.ward = np.zeros((1, 16), np.float32)
        o.vol = np.zeros((1, 8), np.float32)
        s = o.s
        s.points, s.indices, s.ntris = P(o.points), P(o.indices), ntri
        s.spheres, s.nspheres, s.sphere_begin = P(o.spheres), 0, ntri
        s.nodes, s.nnodes = P(o.nodes), o.nodes.shape[0]
        s.prim_ids, s.nprim_ids = P(o.prim_ids), o.prim_ids.shape[0]
        s.materials, s.lambertians, s.wards, s.volumes = P(o.mat), P(o.lam), P(o.ward), P(o.vol)
        return o

    def trace(self, rays8: np.ndarray, counters: bool = False, threads: int = 8, normals: bool = True):
        n = rays8.shape[0]
        prim = np.empty(n, np.int32)
        t = np.empty(n, np.float32)
        ng = np.empty((n, 3), np.float32) if normals else None
        nv = np.empty(n, np.uint32) if counters else None
        nt = np.empty(n, np.uint32) if counters else None
        lib().orc_trace(C.byref(self.s), P(rays8), n, P(prim), P(t), P(ng), P(nv), P(nt), threads)
        return (prim, t, ng, nv, nt) if counters else (prim, t, ng)

    def render(self, cam: orc_camera, cfg: orc_config, npaths: int, steps: int, threads: int = 8,
               want_slots: bool = True):
        npix = cam.image_w * cam.image_h
        accum = np.zeros((npix, 4), np.float64)
        slots = np.zeros(npaths, ORC_SLOT_DTYPE) if want_slots else None
        nxt = lib().orc_render(C.byref(self.s), C.byref(cam), C.byref(cfg), npaths, steps, P(accum), P(slots),
                               threads)
        return accum, slots, int(nxt)


def render_batch(oscenes, cams, cfgs, npaths: int, steps: int, threads: int = 8):
    """Oracle of a batch: requests in run order, request r owning the next
    W*H*spp global samples.  Returns (list of FP64 accumulations, slots)."""
    n = len(oscenes)
    sc_ptrs = (C.c_void_p * n)(*[C.addressof(o.s) for o in oscenes])
    cam_arr = (orc_camera * n)(*cams)
    cfg_arr = (orc_config * n)(*cfgs)
    sizes = [int(f.sample_limit) for f in cfgs]  # W*H*spp of each request
    begin = np.zeros(n, np.uint64)
    end = np.zeros(n, np.uint64)
    acc = 0
    for r in range(n):
        begin[r] = acc
        acc += sizes[r]
        end[r] = acc
    accs = [np.zeros((int(c.image_w) * int(c.image_h), 4), np.float64) for c in cams]
    acc_ptrs = (C.c_void_p * n)(*[a.ctypes.data for a in accs])
    slots = np.zeros(npaths, ORC_SLOT_DTYPE)
    lib().orc_render_batch(sc_ptrs, cam_arr, cfg_arr, P(begin), P(end), n, npaths, steps, acc_ptrs, P(slots), threads)
    return accs, slots


def camera_from_rgr(cam) -> orc_camera:
    o = orc_camera()
    for name in ("eye", "forward", "up", "right", "imageplane_o", "imageplane_r", "imageplane_b"):
        src = getattr(cam, name)
        dst = getattr(o, name)
        for k in range(3):
            dst[k] = src[k]
    o.image_w, o.image_h = cam.image_w, cam.image_h
    return o


def config_from_rgr(cfg, npix: int) -> orc_config:
    o = orc_config()
    o.dof, o.rr_depth, o.radiance_clamp = cfg.dof, cfg.rr_depth, cfg.radiance_clamp
    o.env_select_prob, o.max_depth, o.seed_offset = cfg.env_select_prob, cfg.max_depth, cfg.seed_offset
    o.sample_limit = cfg.spp * npix if cfg.spp else 0
    o.fix_backside_env_pdf = 1 if (cfg.flags & 1) else 0
    o.two_sided_lambertian = 1 if (cfg.flags & 2) else 0
    return o


def envmap_filter_bound(osc: OracleScene, dirs: np.ndarray, frac_bits: int = 8) -> dict:
    """How far the software bilinear envmap lookup (FP32 weights; the oracle's and
    the CUDA path's) is from texture-unit filtering with weights of `frac_bits`
    fractional bits, over the directions `dirs` (n, 3): relative difference of
    the luminance, |Y_q - Y| / Y, per direction."""
    n = dirs.shape[0]
    d = np.ascontiguousarray(dirs, np.float32)
    exact = np.empty((n, 3), np.float32)
    quant = np.empty((n, 3), np.float32)
    lib().orc_envmap_filter_compare(C.byref(osc.s), P(d), n, frac_bits, P(exact), P(quant))
    w = np.array([0.2126, 0.7152, 0.0722])
    ye, yq = exact.astype(np.float64) @ w, quant.astype(np.float64) @ w
    rel = np.abs(yq - ye) / np.maximum(ye, 1e-30)
    return {"directions": int(n), "frac_bits": frac_bits, "rel_max": float(rel.max()), "rel_mean": float(rel.mean()),
            "rel_p999": float(np.quantile(rel, 0.999)), "share_above_1e-3": float((rel > 1e-3).mean())}
