"""Scene set-up shared by the parity tests."""
import numpy as np

import raccoongpurender_gb300 as rg
from raccoongpurender_gb300 import scenes
from oracle import pyoracle as po


def build(mesh, env=None, leaf=4):
    sm = rg.SceneManager()
    sm.addMesh(mesh)
    if env is not None:
        sm.setEnvmap(env)
    sm.buildBVH(max_leaf_size=leaf)
    osc = po.OracleScene.from_scene(sm, mesh.points, mesh.indices)
    return sm, osc


def camera(camd, w, h):
    return rg.camera_look_at(camd["eye"], camd["target"], camd["up"], camd["vfov"], w, h)


def compare_slots(gpu: dict, orc: np.ndarray, fields=None) -> dict:
    """Per-field count of slots whose state differs in any bit."""
    bad = {}
    for f in fields or orc.dtype.names:
        a = np.asarray(gpu[f])
        b = orc[f]
        if a.dtype.kind == "f":
            a = a.view(np.uint32)
        if b.dtype.kind == "f":
            b = b.view(np.uint32)
        a = a.reshape(b.shape).astype(np.int64)
        b = b.astype(np.int64)
        ne = (a != b).reshape(b.shape[0], -1).any(axis=1)
        if ne.any():
            bad[f] = int(ne.sum())
    return bad
