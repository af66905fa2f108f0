"""raccoongpurender_gb300 — a GB300-native wavefront path tracer with the
host API of RaccoonGPURender's hot path.

Python mirror of the reference host classes over the C ABI of ``librgr.so``
(``include/rgr.h``):

* :class:`SceneManager`  — ``rt::SceneManager`` (common/scene_manager.hpp:330-672):
  ``addPolymesh``, ``addSpheres``, ``setEnvmap``, ``buildBVH``.
* :class:`WavefrontLane` — ``rt::WavefrontLane`` (common/wavefront_path_tracing.hpp:339-1153):
  ``setup``, ``initialize``, ``step``, ``finalize_color``, ``stats``.
* :class:`WavefrontPathTracing` — the fixed-work front end, ``launch_fixed(steps)``
  and ``create_color_image()`` (wavefront_path_tracing.hpp:1443-1458, :1345-1408).

The compute path is the CUDA library only: if ``librgr.so`` is missing or no
GPU is present, the device calls raise :class:`RgrError`; there is no CPU
fallback.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

import numpy as np

from . import materials  # noqa: F401  (public)

_PKG = Path(__file__).resolve().parent
# RGR_LIBRARY selects a variant build of the same library (launch-shape experiments)
LIB_PATH = Path(os.environ.get("RGR_LIBRARY", _PKG / "_lib" / "librgr.so"))

RGR_OK = 0
RGR_FMT_RGBA8, RGR_FMT_RGB16, RGR_FMT_FP64_SUMS = 0, 1, 2
STATUS = {0: "ok", -1: "invalid argument", -2: "CUDA error", -3: "out of memory", -4: "call out of order",
          -5: "device capacity check fired", -6: "no CUDA device"}


class RgrError(RuntimeError):
    def __init__(self, status: int, where: str, detail: str = ""):
        self.status = status
        super().__init__(f"{where}: {STATUS.get(status, status)}{(' — ' + detail) if detail else ''}")


class rgr_material(C.Structure):
    _fields_ = [("type", C.c_int32), ("back_emission", C.c_int32), ("le", C.c_float * 3), ("r", C.c_float * 3),
                ("edgetint", C.c_float * 3), ("alpha", C.c_float), ("falloff", C.c_float), ("c", C.c_float)]


class rgr_bvh_params(C.Structure):
    _fields_ = [("max_leaf_size", C.c_int32), ("sah_bins", C.c_int32), ("traversal_cost", C.c_float),
                ("intersect_cost", C.c_float), ("max_depth", C.c_int32), ("num_threads", C.c_int32),
                ("builder", C.c_int32), ("device", C.c_int32)]


BVH_SAH, BVH_LBVH_GPU = 0, 1  # rgr_bvh_params.builder


class rgr_scene_info(C.Structure):
    _fields_ = [("num_triangles", C.c_uint64), ("num_spheres", C.c_uint64), ("num_vertices", C.c_uint64),
                ("num_nodes_stackless", C.c_uint64), ("num_inner_nodes", C.c_uint64), ("num_leaves", C.c_uint64),
                ("depth", C.c_int32), ("sphere_begin", C.c_int32), ("bounds", C.c_float * 6),
                ("sah_cost", C.c_double)]


class rgr_camera(C.Structure):
    _fields_ = [("eye", C.c_float * 3), ("forward", C.c_float * 3), ("up", C.c_float * 3), ("right", C.c_float * 3),
                ("imageplane_o", C.c_float * 3), ("imageplane_r", C.c_float * 3), ("imageplane_b", C.c_float * 3),
                ("image_w", C.c_uint32), ("image_h", C.c_uint32)]


class rgr_alembic_info(C.Structure):
    _fields_ = [("frame_count", C.c_uint32), ("meshes", C.c_uint32), ("meshes_skipped", C.c_uint32),
                ("triangles", C.c_uint32), ("spheres", C.c_uint32), ("has_envmap", C.c_int32),
                ("has_camera", C.c_int32), ("camera", rgr_camera), ("lens_radius", C.c_float),
                ("focus_distance", C.c_float), ("fov_horizontal_degree", C.c_float),
                ("fov_vertical_degree", C.c_float)]


class rgr_render_config(C.Structure):
    _fields_ = [("dof", C.c_float), ("rr_depth", C.c_int32), ("radiance_clamp", C.c_float),
                ("env_select_prob", C.c_float), ("max_depth", C.c_int32), ("seed_offset", C.c_uint32),
                ("spp", C.c_uint64), ("flags", C.c_uint32), ("reserved", C.c_uint32)]


RENDER_FIX_BACKSIDE_ENV_PDF = 1  # RGR_RENDER_FIX_BACKSIDE_ENV_PDF
RENDER_TWO_SIDED_LAMBERTIAN = 2  # RGR_RENDER_TWO_SIDED_LAMBERTIAN


class rgr_guide_config(C.Structure):
    _fields_ = [("learning_rate", C.c_float), ("beta1", C.c_float), ("beta2", C.c_float), ("epsilon", C.c_float),
                ("batch_samples", C.c_uint32), ("guide_fraction", C.c_float), ("train", C.c_int32),
                ("guide_volumes", C.c_int32), ("train_interval", C.c_uint32), ("max_iterations", C.c_uint32),
                ("inference_kernel", C.c_int32), ("max_depth", C.c_uint32), ("seed", C.c_uint64),
                ("training_kernel", C.c_int32), ("learn_fraction", C.c_int32)]


GUIDE_TCGEN05, GUIDE_MMA_SYNC = 0, 1  # rgr_guide_config.inference_kernel and .training_kernel
TRACE_HOST_AUTO, TRACE_HOST_COPY = 0, 1  # rgr_set_trace_host_mode


class rgr_guide_stats(C.Structure):
    _fields_ = [("iterations", C.c_uint64), ("last_loss", C.c_float), ("accept", C.c_float)]


class rgr_stats(C.Structure):
    _fields_ = [("steps", C.c_uint64), ("paths_started", C.c_uint64), ("samples_accumulated", C.c_uint64),
                ("rays_traced", C.c_uint64), ("avg_spp", C.c_double), ("active_paths", C.c_uint32),
                ("error_flags", C.c_uint32)]


class rgr_request_stats(C.Structure):
    _fields_ = [("complete_ms", C.c_double), ("samples", C.c_uint64), ("pixels", C.c_uint64), ("order", C.c_uint32)]


class rgr_ray_soa(C.Structure):
    _fields_ = [(n, C.c_void_p) for n in ("ox", "oy", "oz", "dx", "dy", "dz", "tmax")]


STACKLESS_NODE_DTYPE = np.dtype([("L_lower", "<f4", 4), ("L_upper", "<f4", 4), ("R_lower", "<f4", 4),
                                 ("R_upper", "<f4", 4), ("link_parent", "<u4"), ("link_L", "<u4"),
                                 ("link_R", "<u4"), ("link_sibling", "<u4"), ("primitive_indices_beg", "<u4"),
                                 ("primitive_indices_end", "<u4"), ("pad", "<u4", 2)])
assert STACKLESS_NODE_DTYPE.itemsize == 96

# exported C symbols and their signatures (include/rgr.h)
_SIGS = {
    "rgr_status_string": (C.c_char_p, [C.c_int]),
    "rgr_probe_read_bandwidth": (C.c_int, [C.c_int32, C.c_uint64, C.c_int32, C.POINTER(C.c_double)]),
    "rgr_last_error": (C.c_char_p, []),
    "rgr_bvh_params_default": (None, [C.c_void_p]),
    "rgr_scene_create": (C.c_int, [C.c_void_p]),
    "rgr_scene_destroy": (None, [C.c_void_p]),
    "rgr_scene_add_mesh": (C.c_int, [C.c_void_p, C.c_void_p, C.c_uint64, C.c_void_p, C.c_uint64, C.c_void_p]),
    "rgr_scene_add_spheres": (C.c_int, [C.c_void_p, C.c_void_p, C.c_uint64, C.c_void_p]),
    "rgr_scene_set_envmap": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int32, C.c_int32, C.c_float, C.c_float]),
    "rgr_scene_envmap_tables_gpu": (C.c_int, [C.c_void_p, C.c_int32]),
    "rgr_scene_build_bvh": (C.c_int, [C.c_void_p, C.c_void_p]),
    "rgr_scene_get_info": (C.c_int, [C.c_void_p, C.c_void_p]),
    "rgr_bvh_export_stackless": (C.c_int, [C.c_void_p, C.c_void_p, C.c_uint64, C.c_void_p, C.c_uint64]),
    "rgr_scene_export_envmap": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "rgr_scene_export_geometry": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "rgr_scene_export_envmap_image": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "rgr_alembic_open": (C.c_int, [C.c_void_p, C.c_char_p]),
    "rgr_alembic_close": (None, [C.c_void_p]),
    "rgr_alembic_frame_count": (C.c_uint32, [C.c_void_p]),
    "rgr_alembic_describe": (C.c_int, [C.c_void_p, C.c_uint32, C.c_void_p, C.c_uint64, C.c_void_p]),
    "rgr_alembic_load": (C.c_int, [C.c_void_p, C.c_uint32, C.c_void_p, C.c_void_p]),
    "rgr_render_config_default": (None, [C.c_void_p]),
    "rgr_camera_look_at": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_float, C.c_uint32,
                                     C.c_uint32]),
    "rgr_context_create": (C.c_int, [C.c_void_p, C.c_int32, C.c_uint32]),
    "rgr_context_destroy": (None, [C.c_void_p]),
    "rgr_device_upload": (C.c_int, [C.c_void_p, C.c_void_p]),
    "rgr_render_begin": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p]),
    "rgr_render_step": (C.c_int, [C.c_void_p, C.c_int32]),
    "rgr_render_until_done": (C.c_int, [C.c_void_p, C.c_int32, C.c_void_p]),
    "rgr_render_readback": (C.c_int, [C.c_void_p, C.c_int32, C.c_void_p, C.c_uint64]),
    "rgr_render_stats": (C.c_int, [C.c_void_p, C.c_void_p]),
    "rgr_accum_merge": (C.c_int, [C.c_void_p, C.c_void_p]),
    "rgr_synchronize": (C.c_int, [C.c_void_p]),
    "rgr_set_graph_mode": (C.c_int, [C.c_void_p, C.c_int32]),
    "rgr_trace_closest": (C.c_int, [C.c_void_p, C.c_void_p, C.c_uint64, C.c_void_p, C.c_void_p]),
    "rgr_trace_closest_device": (C.c_int, [C.c_void_p, C.c_void_p, C.c_uint64, C.c_void_p, C.c_void_p,
                                           C.c_void_p, C.c_void_p]),
    "rgr_debug_read_slots": (C.c_int, [C.c_void_p, C.c_void_p, C.c_uint64]),
    "rgr_trace_closest_counts_device": (C.c_int, [C.c_void_p, C.c_void_p, C.c_uint64, C.c_void_p, C.c_void_p,
                                                  C.c_void_p, C.c_void_p, C.c_void_p]),
    "rgr_set_trace_tuning": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32]),
    "rgr_set_trace_staging": (C.c_int, [C.c_void_p, C.c_uint32]),
    "rgr_set_trace_host_mode": (C.c_int, [C.c_void_p, C.c_int32]),
    "rgr_set_render_trace": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32]),
    "rgr_set_trace_search": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32]),
    "rgr_set_trace_reorder": (C.c_int, [C.c_void_p, C.c_int32]),
    "rgr_set_render_tuning": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32]),
    "rgr_batch_create": (C.c_int, [C.c_void_p, C.c_int32, C.c_uint32]),
    "rgr_batch_destroy": (None, [C.c_void_p]),
    "rgr_batch_add": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "rgr_batch_run": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32, C.c_int32, C.c_void_p]),
    "rgr_batch_readback": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32, C.c_void_p, C.c_uint64]),
    "rgr_batch_request_stats": (C.c_int, [C.c_void_p, C.c_int32, C.c_void_p]),
    "rgr_batch_context": (C.c_void_p, [C.c_void_p]),
    "rgr_intermediate_merge_device": (C.c_int, [C.c_void_p, C.c_void_p, C.c_uint64, C.c_void_p]),
    "rgr_render_noalloc": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint32, C.c_int32, C.c_void_p,
                                     C.c_void_p]),
    "rgr_guide_config_default": (None, [C.c_void_p]),
    "rgr_guide_create": (C.c_int, [C.c_void_p, C.c_int32, C.c_void_p]),
    "rgr_guide_destroy": (None, [C.c_void_p]),
    "rgr_guide_set_config": (C.c_int, [C.c_void_p, C.c_void_p]),
    "rgr_guide_set_bounds": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p]),
    "rgr_guide_get_weights": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p]),
    "rgr_guide_set_weights": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p]),
    "rgr_context_set_guide": (C.c_int, [C.c_void_p, C.c_void_p]),
    "rgr_guide_infer_device": (C.c_int, [C.c_void_p, C.c_void_p, C.c_uint32, C.c_void_p, C.c_void_p]),
    "rgr_guide_train_device": (C.c_int, [C.c_void_p, C.c_void_p, C.c_uint32, C.c_float, C.c_int32, C.c_void_p,
                                         C.c_void_p, C.c_void_p]),
    "rgr_guide_train_device_async": (C.c_int, [C.c_void_p, C.c_void_p, C.c_uint32, C.c_float, C.c_void_p]),
    "rgr_guide_stats_get": (C.c_int, [C.c_void_p, C.c_void_p]),
    "rgr_guide_loss_history": (C.c_int, [C.c_void_p, C.c_void_p, C.c_uint32, C.c_void_p]),
    "rgr_guide_last_batch": (C.c_int, [C.c_void_p, C.c_void_p, C.c_uint32, C.c_void_p]),
    "rgr_guide_check": (C.c_int, [C.c_void_p]),
    "rgr_guide_set_stall": (C.c_int, [C.c_void_p, C.c_int32]),
    "rgr_render_checkpoint_size": (C.c_int, [C.c_void_p, C.POINTER(C.c_uint64)]),
    "rgr_render_checkpoint": (C.c_int, [C.c_void_p, C.c_void_p, C.c_uint64]),
    "rgr_render_restore": (C.c_int, [C.c_void_p, C.c_void_p, C.c_uint64]),
}

_lib = None


def load_library(build_if_missing: bool = True) -> C.CDLL:
    """Load librgr.so (building it first if it is absent)."""
    global _lib
    if _lib is not None:
        return _lib
    if not LIB_PATH.exists() and build_if_missing and os.environ.get("RGR_NO_BUILD") != "1":
        from . import _build
        _build.build()
    if not LIB_PATH.exists():
        raise RgrError(-6, "load_library", f"{LIB_PATH} is missing; run raccoongpurender_gb300._build.build()")
    lib = C.CDLL(str(LIB_PATH))
    for name, (res, args) in _SIGS.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def _check(st: int, where: str) -> None:
    if st != RGR_OK:
        detail = load_library().rgr_last_error()
        raise RgrError(st, where, detail.decode("utf-8", errors="replace") if detail else "")


def _ptr(a: np.ndarray) -> int:
    return a.ctypes.data


def _materials_to_c(mats):
    if isinstance(mats, np.ndarray):
        return materials.as_array(mats)
    arr = (rgr_material * max(1, len(mats)))()
    for i, m in enumerate(mats):
        x = arr[i]
        x.type = m["type"]
        x.back_emission = int(m.get("back_emission", 0))
        for k, v in enumerate(m.get("le", (0.0, 0.0, 0.0))):
            x.le[k] = v
        for k, v in enumerate(m.get("r", (1.0, 1.0, 1.0))):
            x.r[k] = v
        for k, v in enumerate(m.get("edgetint", (1.0, 1.0, 1.0))):
            x.edgetint[k] = v
        x.alpha = m.get("alpha", 0.1)
        x.falloff = m.get("falloff", 0.5)
        x.c = m.get("c", 1.0)
    return arr


class SceneManager:
    """Scene upload side of the reference (rt::SceneManager)."""

    def __init__(self):
        self._lib = load_library()
        self._h = C.c_void_p()
        _check(self._lib.rgr_scene_create(C.byref(self._h)), "rgr_scene_create")
        self.materials = materials.as_array([])  # per primitive (MATERIAL_DTYPE), triangles then spheres
        self.num_triangles = 0
        self.envmap = None

    def __del__(self):
        h = getattr(self, "_h", None)
        if h and h.value:
            self._lib.rgr_scene_destroy(h)
            self._h = C.c_void_p()

    @property
    def handle(self):
        return self._h

    def addPolymesh(self, points, indices, materials) -> None:
        """SceneManager::addPolymesh (scene_manager.hpp:339-370)."""
        P = np.ascontiguousarray(points, dtype=np.float32).reshape(-1, 3)
        I = np.ascontiguousarray(indices, dtype=np.uint32).reshape(-1, 3)
        if len(materials) != I.shape[0]:
            raise ValueError("one material per triangle")
        cm = _materials_to_c(materials)
        mp = _ptr(cm) if isinstance(cm, np.ndarray) else C.addressof(cm)
        _check(self._lib.rgr_scene_add_mesh(self._h, _ptr(P), P.shape[0], _ptr(I), I.shape[0], mp),
               "rgr_scene_add_mesh")
        self._append_materials(materials)
        self.num_triangles += I.shape[0]

    def addMesh(self, mesh) -> None:
        self.addPolymesh(mesh.points, mesh.indices, mesh.materials)

    def addSpheres(self, xyzr, materials) -> None:
        """SceneManager::addPointPrimitive (scene_manager.hpp:372-431)."""
        S = np.ascontiguousarray(xyzr, dtype=np.float32).reshape(-1, 4)
        cm = _materials_to_c(materials)
        mp = _ptr(cm) if isinstance(cm, np.ndarray) else C.addressof(cm)
        _check(self._lib.rgr_scene_add_spheres(self._h, _ptr(S), S.shape[0], mp), "rgr_scene_add_spheres")
        self._append_materials(materials)

    def _append_materials(self, mats) -> None:
        arr = materials.as_array(mats)
        self.materials = arr if len(self.materials) == 0 else np.concatenate([materials.as_array(self.materials), arr])

    def setEnvmap(self, rgba, clamp_max: float = 3.4028234663852886e38, scale: float = 1.0) -> None:
        """The ImageEnvmap point of SceneManager::addPoint (scene_manager.hpp:432-497)."""
        if rgba is None:
            _check(self._lib.rgr_scene_set_envmap(self._h, None, 0, 0, 0.0, 1.0), "rgr_scene_set_envmap")
            self.envmap = None
            return
        img = np.ascontiguousarray(rgba, dtype=np.float32)
        h, w = img.shape[:2]
        _check(self._lib.rgr_scene_set_envmap(self._h, _ptr(img), w, h, clamp_max, scale), "rgr_scene_set_envmap")
        proc = img.copy()
        proc[..., :3] = np.minimum(np.maximum(proc[..., :3], np.float32(0)), np.float32(clamp_max))
        if scale != 1.0:
            proc[..., :3] *= np.float32(scale)
        self.envmap = proc

    def addAlembic(self, source, frame: int = 0) -> rgr_alembic_info:
        """Load a frame of an Alembic archive the way WavefrontPathTracing's
        constructor does (wavefront_path_tracing.hpp:1170-1216): visible
        triangle meshes (addPolymesh), then visible point objects (spheres or
        the ImageEnvmap point, addPoint); returns the load summary with the
        first visible camera.  `source` is a path or an AlembicStorage."""
        store = source if isinstance(source, AlembicStorage) else AlembicStorage(source)
        before = self.info()
        info = rgr_alembic_info()
        _check(self._lib.rgr_alembic_load(store.handle, frame, self._h, C.byref(info)), "rgr_alembic_load")
        # mirror what was added, as addPolymesh / addSpheres / setEnvmap keep it
        after = self.info()
        mats = np.zeros(after.num_triangles + after.num_spheres, materials.MATERIAL_DTYPE)
        _check(self._lib.rgr_scene_export_geometry(self._h, None, None, None, _ptr(mats)),
               "rgr_scene_export_geometry")
        self._append_materials(mats[before.num_triangles + before.num_spheres:])
        self.num_triangles = int(after.num_triangles)
        if info.has_envmap:
            w, h = C.c_int32(), C.c_int32()
            _check(self._lib.rgr_scene_export_envmap_image(self._h, C.byref(w), C.byref(h), None),
                   "rgr_scene_export_envmap_image")
            img = np.zeros((h.value, w.value, 4), np.float32)
            _check(self._lib.rgr_scene_export_envmap_image(self._h, None, None, _ptr(img)),
                   "rgr_scene_export_envmap_image")
            self.envmap = img
        return info

    def geometry(self):
        """(points (n, 3), indices (t, 3), spheres (s, 4), materials per primitive) as built."""
        i = self.info()
        pts = np.zeros((i.num_vertices, 3), np.float32)
        idx = np.zeros((i.num_triangles, 3), np.uint32)
        sph = np.zeros((i.num_spheres, 4), np.float32)
        mats = np.zeros(i.num_triangles + i.num_spheres, materials.MATERIAL_DTYPE)
        _check(self._lib.rgr_scene_export_geometry(self._h, _ptr(pts), _ptr(idx), _ptr(sph), _ptr(mats)),
               "rgr_scene_export_geometry")
        return pts, idx, sph, mats

    def envmapTablesOnGPU(self, device: int = 0) -> None:
        """Rebuild the envmap tables with FP64 weights and normalisation on the GPU."""
        _check(self._lib.rgr_scene_envmap_tables_gpu(self._h, device), "rgr_scene_envmap_tables_gpu")

    def buildBVH(self, max_leaf_size: int = 4, sah_bins: int = 32, num_threads: int = 0,
                 traversal_cost: float = 1.0, intersect_cost: float = 0.5, builder: int = 0,
                 device: int = 0) -> None:
        """SceneManager::buildBVH (scene_manager.hpp:517-577); builder BVH_LBVH_GPU
        builds a linear BVH on the GPU instead of the host SAH tree."""
        p = rgr_bvh_params()
        self._lib.rgr_bvh_params_default(C.byref(p))
        p.max_leaf_size = max_leaf_size
        p.sah_bins = sah_bins
        p.num_threads = num_threads
        p.traversal_cost = traversal_cost
        p.intersect_cost = intersect_cost
        p.builder = builder
        p.device = device
        _check(self._lib.rgr_scene_build_bvh(self._h, C.byref(p)), "rgr_scene_build_bvh")

    def info(self) -> rgr_scene_info:
        i = rgr_scene_info()
        _check(self._lib.rgr_scene_get_info(self._h, C.byref(i)), "rgr_scene_get_info")
        return i

    def export_stackless(self):
        """The tree in the reference StacklessBVHNode layout (stackless_bvh.hpp:264-341)."""
        inf = self.info()
        nodes = np.zeros(inf.num_nodes_stackless, dtype=STACKLESS_NODE_DTYPE)
        ids = np.zeros(inf.num_triangles + inf.num_spheres, dtype=np.uint32)
        _check(self._lib.rgr_bvh_export_stackless(self._h, _ptr(nodes), nodes.shape[0], _ptr(ids), ids.shape[0]),
               "rgr_bvh_export_stackless")
        return nodes, ids

    def export_envmap(self):
        if self.envmap is None:
            return None
        h, w = self.envmap.shape[:2]
        n = w * h
        pdf = np.zeros(7 * n, np.float32)
        height = np.zeros(7 * n, np.float32)
        alias = np.zeros(7 * n, np.int32)
        frag = np.zeros(4 * n, np.float32)
        _check(self._lib.rgr_scene_export_envmap(self._h, _ptr(pdf), _ptr(height), _ptr(alias), _ptr(frag)),
               "rgr_scene_export_envmap")
        return dict(pdf=pdf, height=height, alias=alias, frag=frag, w=w, h=h)


class AlembicStorage:
    """houdini_alembic::AlembicStorage (libs/houdini_alembic/houdini_alembic.hpp:417-432):
    an Alembic archive read by the library's own Ogawa reader."""

    def __init__(self, path):
        self._lib = load_library()
        self._h = C.c_void_p()
        _check(self._lib.rgr_alembic_open(C.byref(self._h), os.fsencode(str(path))), "rgr_alembic_open")
        self.path = str(path)

    def __del__(self):
        h = getattr(self, "_h", None)
        if h and h.value:
            self._lib.rgr_alembic_close(h)
            self._h = C.c_void_p()

    @property
    def handle(self):
        return self._h

    def frameCount(self) -> int:
        return int(self._lib.rgr_alembic_frame_count(self._h))

    def read(self, frame: int = 0) -> dict:
        """AlembicStorage::read(frame): the objects the Houdini reader returns,
        as a dict ({"frame_count", "objects": [...]})."""
        import json
        need = C.c_uint64()
        _check(self._lib.rgr_alembic_describe(self._h, frame, None, 0, C.byref(need)), "rgr_alembic_describe")
        buf = C.create_string_buffer(need.value)
        _check(self._lib.rgr_alembic_describe(self._h, frame, buf, need.value, C.byref(need)), "rgr_alembic_describe")
        return json.loads(buf.value.decode("utf-8", errors="replace"))


def render_config(**kw) -> rgr_render_config:
    """A render config with the reference defaults, overridden by keywords
    (dof, rr_depth, radiance_clamp, env_select_prob, max_depth, seed_offset, spp, flags)."""
    c = rgr_render_config()
    load_library().rgr_render_config_default(C.byref(c))
    for k, v in kw.items():
        setattr(c, k, v)
    return c


def camera_look_at(eye, target, up, vfov: float, w: int, h: int) -> rgr_camera:
    cam = rgr_camera()
    f3 = C.c_float * 3
    _check(load_library().rgr_camera_look_at(C.byref(cam), f3(*eye), f3(*target), f3(*up), vfov, w, h),
           "rgr_camera_look_at")
    return cam


SLOT_WORDS = 34
SLOT_FIELDS = dict(T=(0, 3), L=(3, 6), ro=(6, 9), rd=(9, 12), logic_i=(12, 13), pixel_index=(13, 14),
                   rng=(14, 18), hit_surface=(18, 19), hit_volume=(19, 20), tmin=(20, 21), Ng=(21, 24),
                   queue=(24, 25), vol_count=(25, 26), vols=(26, 33))


class WavefrontLane:
    """One GPU's path pool (rt::WavefrontLane)."""

    def __init__(self, device: int = 0, path_count: int = 1 << 22):
        self._lib = load_library()
        self._h = C.c_void_p()
        _check(self._lib.rgr_context_create(C.byref(self._h), device, path_count), "rgr_context_create")
        self.path_count = path_count
        self.camera = None

    def __del__(self):
        h = getattr(self, "_h", None)
        if h and h.value:
            self._lib.rgr_context_destroy(h)
            self._h = C.c_void_p()

    @property
    def handle(self):
        return self._h

    def setup(self, scene: SceneManager) -> None:
        """WavefrontLane::setup (wavefront_path_tracing.hpp:451-522)."""
        _check(self._lib.rgr_device_upload(self._h, scene.handle), "rgr_device_upload")

    def initialize(self, camera: rgr_camera, config: rgr_render_config | None = None) -> None:
        """WavefrontLane::initialize (:532-570)."""
        self.camera = camera
        cfg = config if config is not None else render_config()
        _check(self._lib.rgr_render_begin(self._h, C.byref(camera), C.byref(cfg)), "rgr_render_begin")

    re_start = initialize

    def step(self, steps: int = 1) -> None:
        """WavefrontLane::step() (:591-939), `steps` times; asynchronous."""
        _check(self._lib.rgr_render_step(self._h, steps), "rgr_render_step")

    def render_until_done(self, max_steps: int = 100000) -> int:
        n = C.c_int32()
        _check(self._lib.rgr_render_until_done(self._h, max_steps, C.byref(n)), "rgr_render_until_done")
        return n.value

    def synchronize(self) -> None:
        _check(self._lib.rgr_synchronize(self._h), "rgr_synchronize")

    def set_graph_mode(self, enabled: bool) -> None:
        _check(self._lib.rgr_set_graph_mode(self._h, int(enabled)), "rgr_set_graph_mode")

    def _npix(self) -> int:
        return int(self.camera.image_w) * int(self.camera.image_h)

    def accumulation(self) -> np.ndarray:
        """FP64 per-pixel (r, g, b, count) sums, shape (H, W, 4)."""
        out = np.zeros((self._npix(), 4), np.float64)
        _check(self._lib.rgr_render_readback(self._h, RGR_FMT_FP64_SUMS, _ptr(out), out.nbytes),
               "rgr_render_readback")
        return out.reshape(self.camera.image_h, self.camera.image_w, 4)

    def intermediate(self) -> np.ndarray:
        """RGB16IntermediateValueType per pixel (half mean, ushort count)."""
        out = np.zeros((self._npix(), 4), np.uint16)
        _check(self._lib.rgr_render_readback(self._h, RGR_FMT_RGB16, _ptr(out), out.nbytes), "rgr_render_readback")
        return out.reshape(self.camera.image_h, self.camera.image_w, 4)

    def finalize_color(self) -> np.ndarray:
        """WavefrontLane::finalize_color (:993-1007): RGBA8, shape (H, W, 4)."""
        out = np.zeros((self._npix(), 4), np.uint8)
        _check(self._lib.rgr_render_readback(self._h, RGR_FMT_RGBA8, _ptr(out), out.nbytes), "rgr_render_readback")
        return out.reshape(self.camera.image_h, self.camera.image_w, 4)

    def stats(self) -> rgr_stats:
        s = rgr_stats()
        _check(self._lib.rgr_render_stats(self._h, C.byref(s)), "rgr_render_stats")
        return s

    def checkpoint(self) -> np.ndarray:
        """The render's device state (path pool, queues, counters, RNG, FP64 sums) as bytes."""
        n = C.c_uint64(0)
        _check(self._lib.rgr_render_checkpoint_size(self._h, C.byref(n)), "rgr_render_checkpoint_size")
        out = np.empty(n.value, np.uint8)
        _check(self._lib.rgr_render_checkpoint(self._h, _ptr(out), out.nbytes), "rgr_render_checkpoint")
        return out

    def restore(self, state: np.ndarray) -> None:
        """Load a checkpoint into this lane, initialised with the same scene, camera and config."""
        state = np.ascontiguousarray(state, np.uint8)
        _check(self._lib.rgr_render_restore(self._h, _ptr(state), state.nbytes), "rgr_render_restore")

    def stat_avg_sample(self) -> float:
        return self.stats().avg_spp

    def debug_slots(self) -> dict:
        """Per-slot path state as a dict of arrays (float fields as float32)."""
        raw = np.zeros((self.path_count, SLOT_WORDS), np.uint32)
        _check(self._lib.rgr_debug_read_slots(self._h, _ptr(raw), self.path_count), "rgr_debug_read_slots")
        return slots_from_words(raw)

    def render_noalloc(self, camera: rgr_camera, config: rgr_render_config, path_count: int, steps: int,
                       accum_ptr: int, stream: int = 0) -> None:
        """Render `steps` bounces of `path_count` paths into the caller's device
        buffer (4 doubles per pixel) without allocating device memory; see
        rgr_render_noalloc in include/rgr.h for its limits."""
        _check(self._lib.rgr_render_noalloc(self._h, C.byref(camera), C.byref(config), path_count, steps, accum_ptr,
                                            stream or None), "rgr_render_noalloc")

    def merge_from(self, other: "WavefrontLane") -> None:
        """WavefrontLane::merge_from (:963-991)."""
        _check(self._lib.rgr_accum_merge(self._h, other.handle), "rgr_accum_merge")

    # ---- closest hit as a service
    def trace_closest(self, rays) -> tuple[np.ndarray, np.ndarray]:
        """Closest hit of host rays: returns (prim int32, t float32)."""
        soa = rays.soa() if hasattr(rays, "soa") else rays
        soa = [np.ascontiguousarray(a, dtype=np.float32) for a in soa]
        n = soa[0].shape[0]
        prim = np.empty(n, np.int32)
        t = np.empty(n, np.float32)
        r = rgr_ray_soa(*[_ptr(a) for a in soa])
        _check(self._lib.rgr_trace_closest(self._h, C.byref(r), n, _ptr(prim), _ptr(t)), "rgr_trace_closest")
        return prim, t

    def set_render_tuning(self, shade_blocks_per_sm: int = 8, graph_steps: int = 1) -> None:
        _check(self._lib.rgr_set_render_tuning(self._h, shade_blocks_per_sm, graph_steps), "rgr_set_render_tuning")

    def set_guide(self, guide: "Guide | None") -> None:
        """Render with the learned guide from the next initialize() on (None: plain)."""
        self._guide = guide  # keep it alive while the context refers to it
        _check(self._lib.rgr_context_set_guide(self._h, guide.handle if guide is not None else None),
               "rgr_context_set_guide")

    def set_trace_tuning(self, refill: int = 16, blocks_per_sm: int = 0) -> None:
        _check(self._lib.rgr_set_trace_tuning(self._h, refill, blocks_per_sm), "rgr_set_trace_tuning")

    def set_render_trace(self, persistent=-1, refill: int = 12) -> None:
        """Extension rays of a bounce: persistent refilling kernel + logic (True),
        fused (False), or by scene size (-1, the default)."""
        mode = persistent if isinstance(persistent, int) and not isinstance(persistent, bool) else int(bool(persistent))
        _check(self._lib.rgr_set_render_trace(self._h, mode, refill), "rgr_set_render_trace")

    def set_trace_search(self, closest: int = 8, render: int = 8) -> None:
        """Leaf batching of the persistent traversal kernels: a warp takes node
        steps while at least this many of its lanes still search for their next
        leaf (closest-hit kernel / a render's extension rays; 0 leaves one
        unchanged).  Results are identical for every value."""
        _check(self._lib.rgr_set_trace_search(self._h, closest, render), "rgr_set_trace_search")

    def set_trace_host_mode(self, mode: int) -> None:
        """rgr_trace_closest with host arrays: TRACE_HOST_AUTO (zero copy where the
        GPU can address them) or TRACE_HOST_COPY (chunked copies)."""
        _check(self._lib.rgr_set_trace_host_mode(self._h, mode), "rgr_set_trace_host_mode")

    def set_trace_staging(self, staged_nodes: int) -> None:
        """Top BVH nodes each traversal CTA keeps in shared memory (0 = off)."""
        _check(self._lib.rgr_set_trace_staging(self._h, staged_nodes), "rgr_set_trace_staging")

    def set_trace_reorder(self, reorder: int) -> None:
        """trace_closest_device sorts the rays by origin and direction before the
        traversal (1) or takes them in the given order (0, default).  Results are
        identical; sorting pays for incoherent rays."""
        _check(self._lib.rgr_set_trace_reorder(self._h, reorder), "rgr_set_trace_reorder")

    def trace_closest_counts_device(self, soa_ptrs, n: int, prim_ptr: int, t_ptr: int, nodes_ptr: int,
                                    prims_ptr: int, stream: int = 0) -> None:
        r = rgr_ray_soa(*soa_ptrs)
        _check(self._lib.rgr_trace_closest_counts_device(self._h, C.byref(r), n, prim_ptr, t_ptr, nodes_ptr, prims_ptr,
                                                         stream or None), "rgr_trace_closest_counts_device")

    def trace_closest_device(self, soa_ptrs, n: int, prim_ptr: int, t_ptr: int, ng_ptr: int = 0,
                             stream: int = 0) -> None:
        """Closest hit of device rays (7 device pointers), enqueued on `stream`."""
        r = rgr_ray_soa(*soa_ptrs)
        _check(self._lib.rgr_trace_closest_device(self._h, C.byref(r), n, prim_ptr, t_ptr, ng_ptr or None,
                                                  stream or None), "rgr_trace_closest_device")


class Guide:
    """The learned path-guiding network on one GPU (rgr_guide): 36 encoded
    inputs -> 4 x 64 ReLU -> 8 vMF lobes (40 outputs), BF16 on the tensor
    cores, trained online by Adam while a WavefrontLane renders with it."""

    LAYERS, WIDTH, INPUTS, OUTPUTS, LOBES = 5, 64, 36, 40, 8
    SEL, ROW_OUTPUTS = 40, 48  # the selection logit's output index; raw outputs per row of infer_device
    N_WEIGHTS = LAYERS * WIDTH * WIDTH
    N_PARAMS = N_WEIGHTS + LAYERS * WIDTH

    def __init__(self, device: int = 0, **cfg):
        self._lib = load_library()
        c = rgr_guide_config()
        self._lib.rgr_guide_config_default(C.byref(c))
        for k, v in cfg.items():
            setattr(c, k, v)
        self._h = C.c_void_p()
        _check(self._lib.rgr_guide_create(C.byref(self._h), device, C.byref(c)), "rgr_guide_create")
        self._cfg = c

    def __del__(self):
        h = getattr(self, "_h", None)
        if h and h.value:
            self._lib.rgr_guide_destroy(h)
            self._h = C.c_void_p()

    @property
    def handle(self):
        return self._h

    @property
    def config(self) -> rgr_guide_config:
        return self._cfg

    def set_config(self, **kw) -> None:
        c = rgr_guide_config()
        C.memmove(C.byref(c), C.byref(self._cfg), C.sizeof(c))
        for k, v in kw.items():
            setattr(c, k, v)
        _check(self._lib.rgr_guide_set_config(self._h, C.byref(c)), "rgr_guide_set_config")
        self._cfg = c

    def set_bounds(self, lo, hi) -> None:
        f3 = C.c_float * 3
        _check(self._lib.rgr_guide_set_bounds(self._h, f3(*lo), f3(*hi)), "rgr_guide_set_bounds")

    def weights(self) -> tuple[np.ndarray, np.ndarray]:
        """FP32 (W[5, 64, 64] as W[l][in][out], b[5, 64])."""
        w = np.zeros((self.LAYERS, self.WIDTH, self.WIDTH), np.float32)
        b = np.zeros((self.LAYERS, self.WIDTH), np.float32)
        _check(self._lib.rgr_guide_get_weights(self._h, _ptr(w), _ptr(b)), "rgr_guide_get_weights")
        return w, b

    def set_weights(self, w: np.ndarray, b: np.ndarray) -> None:
        w = np.ascontiguousarray(w, np.float32).reshape(self.LAYERS, self.WIDTH, self.WIDTH)
        b = np.ascontiguousarray(b, np.float32).reshape(self.LAYERS, self.WIDTH)
        _check(self._lib.rgr_guide_set_weights(self._h, _ptr(w), _ptr(b)), "rgr_guide_set_weights")

    def infer_device(self, rows_ptr: int, n: int, out_ptr: int, stream: int = 0) -> None:
        """Raw outputs (48 floats per row: the mixture's 40, the selection logit, zeros)
        of device rows of 16 floats (x, n, wo, ...)."""
        _check(self._lib.rgr_guide_infer_device(self._h, rows_ptr, n, out_ptr, stream or None),
               "rgr_guide_infer_device")

    def train_device(self, samples_ptr: int, n: int, weight_scale: float = 1.0, apply_adam: bool = True,
                     grads_ptr: int = 0, stream: int = 0) -> float:
        """One training step on n device samples of 16 floats; returns the loss."""
        loss = C.c_float()
        _check(self._lib.rgr_guide_train_device(self._h, samples_ptr, n, weight_scale, int(apply_adam),
                                                grads_ptr or None, C.byref(loss), stream or None),
               "rgr_guide_train_device")
        return loss.value

    def train_device_async(self, samples_ptr: int, n: int, weight_scale: float = 1.0, stream: int = 0) -> None:
        """One training step with Adam on n device samples, enqueued on `stream`
        without waiting (rgr_guide_train_device_async)."""
        _check(self._lib.rgr_guide_train_device_async(self._h, samples_ptr, n, weight_scale, stream or None),
               "rgr_guide_train_device_async")

    def check(self) -> None:
        """Raise if a tensor-core wait of the guide's kernels timed out since the last check."""
        _check(self._lib.rgr_guide_check(self._h), "rgr_guide_check")

    def set_stall(self, on: bool) -> None:
        """Failure-detection tests: the tcgen05 inference kernel's MMA warps issue
        nothing while on, so its bounded waits run out (rgr_guide_set_stall)."""
        _check(self._lib.rgr_guide_set_stall(self._h, 1 if on else 0), "rgr_guide_set_stall")

    def stats(self) -> dict:
        st = rgr_guide_stats()
        _check(self._lib.rgr_guide_stats_get(self._h, C.byref(st)), "rgr_guide_stats_get")
        return dict(iterations=st.iterations, last_loss=st.last_loss, accept=st.accept)

    def last_batch(self, max_count: int = 1 << 18) -> np.ndarray:
        """The training samples (n, 16) of the last iteration of a guided render."""
        out = np.zeros((max_count, 16), np.float32)
        n = C.c_uint32()
        _check(self._lib.rgr_guide_last_batch(self._h, _ptr(out), max_count, C.byref(n)), "rgr_guide_last_batch")
        return out[:n.value].copy()

    def loss_history(self, max_count: int = 4096) -> np.ndarray:
        out = np.zeros(max_count, np.float32)
        n = C.c_uint32()
        _check(self._lib.rgr_guide_loss_history(self._h, _ptr(out), max_count, C.byref(n)), "rgr_guide_loss_history")
        return out[:n.value].copy()


def probe_read_bandwidth(device: int, nbytes: int, reps: int = 20) -> float:
    """Read bandwidth (GB/s) over a buffer of `nbytes` on `device`: L2 when the
    buffer fits in L2, HBM when it does not (rgr_probe_read_bandwidth)."""
    g = C.c_double()
    _check(load_library().rgr_probe_read_bandwidth(device, nbytes, reps, C.byref(g)), "rgr_probe_read_bandwidth")
    return float(g.value)


def merge_intermediate_device(a_ptr: int, b_ptr: int, npix: int, stream: int = 0) -> None:
    """a <- merge of two device RGB16 intermediates (merge_intermediate, accumlation.cl:27-49)."""
    _check(load_library().rgr_intermediate_merge_device(a_ptr, b_ptr, npix, stream or None),
           "rgr_intermediate_merge_device")


def slots_from_words(raw: np.ndarray) -> dict:
    out = {}
    for k, (a, b) in SLOT_FIELDS.items():
        v = raw[:, a:b]
        if k in ("T", "L", "ro", "rd", "tmin", "Ng"):
            v = v.view(np.float32)
        elif k in ("hit_surface", "hit_volume", "queue", "vol_count", "vols"):
            v = v.view(np.int32)
        out[k] = v if b - a > 1 else v[:, 0]
    return out


ORDER_FIFO, ORDER_SHORTEST_FIRST = 0, 1


class Batch:
    """Many render requests of uneven size sharing one path pool and one
    graph-replayed bounce loop."""

    def __init__(self, device: int = 0, path_count: int = 1 << 22):
        self._lib = load_library()
        self._h = C.c_void_p()
        _check(self._lib.rgr_batch_create(C.byref(self._h), device, path_count), "rgr_batch_create")
        self.path_count = path_count
        self.requests = []  # (scene, camera, config)

    def __del__(self):
        h = getattr(self, "_h", None)
        if h and h.value:
            self._lib.rgr_batch_destroy(h)
            self._h = C.c_void_p()

    def add(self, scene: SceneManager, camera: rgr_camera, config: rgr_render_config) -> int:
        rid = C.c_int32()
        _check(self._lib.rgr_batch_add(self._h, scene.handle, C.byref(camera), C.byref(config), C.byref(rid)),
               "rgr_batch_add")
        self.requests.append((scene, camera, config))
        return rid.value

    def run(self, order: int = ORDER_FIFO, steps_per_launch: int = 8, max_steps: int = 100000) -> int:
        n = C.c_int32()
        _check(self._lib.rgr_batch_run(self._h, order, steps_per_launch, max_steps, C.byref(n)), "rgr_batch_run")
        return n.value

    def accumulation(self, rid: int) -> np.ndarray:
        cam = self.requests[rid][1]
        out = np.zeros((cam.image_h, cam.image_w, 4), np.float64)
        _check(self._lib.rgr_batch_readback(self._h, rid, RGR_FMT_FP64_SUMS, _ptr(out), out.nbytes),
               "rgr_batch_readback")
        return out

    def color(self, rid: int) -> np.ndarray:
        cam = self.requests[rid][1]
        out = np.zeros((cam.image_h, cam.image_w, 4), np.uint8)
        _check(self._lib.rgr_batch_readback(self._h, rid, RGR_FMT_RGBA8, _ptr(out), out.nbytes), "rgr_batch_readback")
        return out

    def set_render_tuning(self, shade_blocks_per_sm: int = 8, graph_steps: int = 8) -> None:
        _check(self._lib.rgr_set_render_tuning(self._lib.rgr_batch_context(self._h), shade_blocks_per_sm,
                                               graph_steps), "rgr_set_render_tuning")

    def set_render_trace(self, refill: int = 12) -> None:
        """Refill threshold of the bounce's persistent closest-hit kernel (the
        kernel is chosen by scene size, as for a single render)."""
        _check(self._lib.rgr_set_render_trace(self._lib.rgr_batch_context(self._h), -1, refill),
               "rgr_set_render_trace")

    def set_trace_search(self, render: int = 8) -> None:
        """Leaf batching of the bounce's persistent closest-hit kernel."""
        _check(self._lib.rgr_set_trace_search(self._lib.rgr_batch_context(self._h), 0, render),
               "rgr_set_trace_search")

    def request_stats(self, rid: int) -> rgr_request_stats:
        st = rgr_request_stats()
        _check(self._lib.rgr_batch_request_stats(self._h, rid, C.byref(st)), "rgr_batch_request_stats")
        return st

    def stats(self) -> rgr_stats:
        st = rgr_stats()
        _check(self._lib.rgr_render_stats(self._lib.rgr_batch_context(self._h), C.byref(st)), "rgr_render_stats")
        return st

    def debug_slots(self) -> dict:
        raw = np.zeros((self.path_count, SLOT_WORDS), np.uint32)
        _check(self._lib.rgr_debug_read_slots(self._lib.rgr_batch_context(self._h), _ptr(raw), self.path_count),
               "rgr_debug_read_slots")
        return slots_from_words(raw)


class WavefrontPathTracing:
    """Fixed-work front end on one GPU (rt::WavefrontPathTracing, RenderMode_SingleGPU)."""

    def __init__(self, scene: SceneManager, camera: rgr_camera, config: rgr_render_config | None = None,
                 path_count: int = 1 << 22, device: int = 0):
        self.lane = WavefrontLane(device, path_count)
        self.lane.setup(scene)
        self.lane.initialize(camera, config)

    def launch_fixed(self, steps: int) -> np.ndarray:
        """Run `steps` bounces of the whole pool, then create_color_image()."""
        self.lane.step(steps)
        return self.create_color_image()

    def create_color_image(self) -> np.ndarray:
        return self.lane.finalize_color()

    def re_start(self, camera: rgr_camera, config: rgr_render_config | None = None) -> None:
        self.lane.initialize(camera, config)
