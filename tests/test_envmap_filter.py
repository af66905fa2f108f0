"""The envmap lookup on a camera ray's first segment filters bilinearly
(get_envmap_value, kernels/envmap_sampling.cl:36-52).  The reference reads an
OpenCL image, whose texture unit holds the filter weights in fixed point (8
fractional bits on NVIDIA hardware); the oracle and the CUDA path compute
them in FP32.  This bounds the difference on the full-render envmap (the
1024x512 sky with a 0.5-degree sun of radiance 1e4)."""
import numpy as np

import raccoongpurender_gb300 as rg
from raccoongpurender_gb300 import scenes


def _env_scene(po):
    mesh = scenes.cornell_box()
    sm = rg.SceneManager()
    sm.addMesh(mesh)
    sm.setEnvmap(scenes.sky_envmap())
    sm.buildBVH(max_leaf_size=4)
    return po.OracleScene.from_scene(sm, mesh.points, mesh.indices)


def test_envmap_filter_bound(po):
    osc = _env_scene(po)
    rng = np.random.default_rng(2)
    v = rng.normal(size=(200_000, 3))
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    # with (nearly) unquantised weights the comparison lookup is the oracle's own
    full = po.envmap_filter_bound(osc, v, frac_bits=23)
    assert full["rel_max"] < 1e-6
    b8 = po.envmap_filter_bound(osc, v, frac_bits=8)
    # the stated tolerance: mean relative luminance difference below 1e-4, none above 5 %
    assert b8["rel_mean"] < 1e-4 and b8["rel_max"] < 0.05
    assert b8["share_above_1e-3"] < 0.01
