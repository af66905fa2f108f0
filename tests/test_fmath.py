"""Accuracy of the deterministic float math (rgr_fmath.h) that both the CUDA
kernels and the oracle use for the OpenCL built-ins, against float64 numpy.
OpenCL 1.2 full-profile bounds: sin/cos 4 ulp, log/exp 3 ulp, atan 5 ulp,
atan2 6 ulp, pow 16 ulp."""
import numpy as np
import pytest

FN = {"sin": 0, "cos": 1, "log": 2, "exp": 3, "atan": 4, "atan2": 5, "pow": 6}


def ulp_err(got: np.ndarray, ref: np.ndarray) -> np.ndarray:
    ref32 = ref.astype(np.float32)
    sp = np.spacing(np.abs(ref32)).astype(np.float64)
    sp = np.maximum(sp, np.float64(np.finfo(np.float32).smallest_subnormal))
    return np.abs(got.astype(np.float64) - ref) / sp


def call(po, name, x, y=None):
    f = po.lib().orc_fm
    code = FN[name]
    if y is None:
        return np.array([f(code, float(v), 0.0) for v in x], np.float32)
    return np.array([f(code, float(a), float(b)) for a, b in zip(x, y)], np.float32)


@pytest.fixture(scope="module")
def xs():
    return np.random.default_rng(0)


def test_sin_cos(po, xs):
    x = np.concatenate([xs.uniform(-7, 7, 4000), xs.uniform(-2000, 2000, 500), xs.uniform(-1e5, 1e5, 200)]).astype(np.float32)
    xd = x.astype(np.float64)
    assert ulp_err(call(po, "sin", x), np.sin(xd)).max() <= 2.0
    assert ulp_err(call(po, "cos", x), np.cos(xd)).max() <= 2.0
    assert call(po, "sin", np.array([-0.0], np.float32))[0].tobytes() == np.float32(-0.0).tobytes()


def test_log_exp(po, xs):
    x = np.exp(xs.uniform(-80, 80, 4000)).astype(np.float32)
    x = np.concatenate([x, np.array([1.0, 2.0, 0.5, 1e-40, 3.4e38], np.float32)])
    assert ulp_err(call(po, "log", x), np.log(x.astype(np.float64))).max() <= 2.0
    e = xs.uniform(-103, 88.7, 4000).astype(np.float32)
    err = ulp_err(call(po, "exp", e), np.exp(e.astype(np.float64)))
    assert err[e > -87].max() <= 2.0
    assert np.isneginf(call(po, "log", np.array([0.0], np.float32)))[0]
    assert np.isnan(call(po, "log", np.array([-1.0], np.float32)))[0]
    assert np.isposinf(call(po, "exp", np.array([100.0], np.float32)))[0]


def test_atan_atan2(po, xs):
    x = np.concatenate([xs.uniform(-3, 3, 3000), np.tan(xs.uniform(-1.57, 1.57, 1000))]).astype(np.float32)
    assert ulp_err(call(po, "atan", x), np.arctan(x.astype(np.float64))).max() <= 3.0
    y = xs.normal(size=3000).astype(np.float32)
    z = xs.normal(size=3000).astype(np.float32)
    assert ulp_err(call(po, "atan2", y, z), np.arctan2(y.astype(np.float64), z.astype(np.float64))).max() <= 4.0
    sp = np.array([0.0, -0.0, 0.0, -0.0, 1.0, -1.0, np.inf, -np.inf, np.inf], np.float32)
    sx = np.array([1.0, 1.0, -1.0, -1.0, 0.0, 0.0, np.inf, np.inf, -np.inf], np.float32)
    got = call(po, "atan2", sp, sx)
    ref = np.arctan2(sp.astype(np.float64), sx.astype(np.float64))
    assert np.all(np.abs(got - ref) <= 1e-6 * np.maximum(1, np.abs(ref)))
    assert np.array_equal(np.signbit(got), np.signbit(ref))


def test_pow(po, xs):
    b = xs.uniform(0, 4, 3000).astype(np.float32)
    e = xs.uniform(-3, 3, 3000).astype(np.float32)
    got = call(po, "pow", b, e)
    ref = np.power(b.astype(np.float64), e.astype(np.float64))
    err = ulp_err(got, ref)
    lim = 2.0 + np.abs(e.astype(np.float64) * np.log(np.maximum(b.astype(np.float64), 1e-30)))
    assert (err <= lim).all()
    assert call(po, "pow", np.array([0.0], np.float32), np.array([2.0], np.float32))[0] == 0.0
    assert call(po, "pow", np.array([5.0], np.float32), np.array([0.0], np.float32))[0] == 1.0
