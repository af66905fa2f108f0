"""The path-guiding oracle checked against mathematics (CPU): analytic
gradients against central finite differences, the vMF mixture's
normalisation, BF16 rounding.  The reference has no learned guiding, so
these identities pin the oracle that the GPU kernels are compared with."""
import numpy as np

from oracle import guide_oracle as go


def test_bf16_rounding():
    x = np.array([1.0, 1.0 + 2.0 ** -8, 1.0 + 3 * 2.0 ** -8, 1.0 + 2.0 ** -9, -2.5, 3.0e38, 1e-40])
    y = go.bf16(x)
    # BF16 spacing at 1.0 is 2^-7; halfway cases go to the even mantissa
    assert y[0] == 1.0
    assert y[1] == 1.0                     # 1 + 2^-8: halfway between 1 and 1 + 2^-7
    assert y[2] == 1.0 + 2.0 ** -6         # 1 + 1.5 * 2^-7: halfway between 1 + 2^-7 and 1 + 2^-6
    assert y[3] == 1.0
    assert y[4] == -2.5
    # every result is representable: its low 16 float32 bits are zero
    assert (go.bf16(np.random.default_rng(0).normal(size=1000)).astype(np.float32).view(np.uint32) & 0xFFFF == 0).all()


def test_loss_gradient_finite_differences():
    rng = np.random.default_rng(1)
    n = 16
    raw = rng.normal(size=(n, go.NET_OUTPUTS))
    raw[:, 3 * go.LOBES:4 * go.LOBES] = rng.uniform(-2.0, 3.0, (n, go.LOBES))  # concentrations
    d = rng.normal(size=(n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    w = rng.uniform(0.1, 2.0, n)
    pb = np.where(np.arange(n) % 4 == 3, 0.0, rng.uniform(0.01, 2.0, n))  # every 4th without a BSDF pdf
    _, g = go.loss_and_grad(raw, d, w, pb)
    q0 = go.mixture_pdf(raw, d)  # the selection term's gradient holds the mixture density fixed

    def total(r):
        return go.loss_and_grad(r, d, w)[0] + go.penalty(r, w) + go.selection_loss(r, d, w, pb, q0)

    h = 1e-6
    num = np.zeros_like(raw)
    for j in range(go.NET_OUTPUTS):
        e = np.zeros_like(raw)
        e[:, j] = h
        num[:, j] = (total(raw + e) - total(raw - e)) / (2 * h)
    err = np.abs(num - g).max() / np.abs(g).max()
    assert err < 1e-6, err
    assert np.abs(g[:, go.SEL]).max() > 0 and (g[pb == 0, go.SEL] == 0).all()


def test_network_gradient_finite_differences():
    W, b = go.init_weights(3)
    s = go.random_samples(24, seed=4)
    lo, ie = (-1.0, -1.0, -1.0), (0.5, 0.5, 0.5)
    loss, dW, db = go.gradients(W, b, s, lo, ie, bf16_round=False)
    rng = np.random.default_rng(5)
    h = 1e-6
    q0 = go.mixture_density(W, b, s, lo, ie)

    def L(W2, b2):
        return go.objective(W2, b2, s, lo, ie, q_fixed=q0)

    W64, b64 = W.astype(np.float64), b.astype(np.float64)
    checked = 0
    for l in range(go.LAYERS):
        for _ in range(6):
            i = rng.integers(0, go.FAN_IN[l])
            o = rng.integers(0, go.FAN_OUT[l])
            Wp, Wm = W64.copy(), W64.copy()
            Wp[l, i, o] += h
            Wm[l, i, o] -= h
            num = (L(Wp, b64) - L(Wm, b64)) / (2 * h)
            assert abs(num - dW[l, i, o]) <= 1e-5 * max(1.0, abs(num)), (l, i, o, num, dW[l, i, o])
            checked += 1
        o = rng.integers(0, go.FAN_OUT[l])
        bp, bm = b64.copy(), b64.copy()
        bp[l, o] += h
        bm[l, o] -= h
        num = (L(W64, bp) - L(W64, bm)) / (2 * h)
        assert abs(num - db[l, o]) <= 1e-5 * max(1.0, abs(num)), (l, o, num, db[l, o])
    assert checked == 30
    # the selection logit (output 40 of the last layer) is trained
    for i in (0, 7, 33):
        Wp, Wm = W64.copy(), W64.copy()
        Wp[4, i, go.SEL] += h
        Wm[4, i, go.SEL] -= h
        num = (L(Wp, b64) - L(Wm, b64)) / (2 * h)
        assert abs(num - dW[4, i, go.SEL]) <= 1e-5 * max(1.0, abs(num))
    assert dW[4, :, go.SEL].any() and db[4, go.SEL] != 0.0
    # padding receives no gradient
    for l in range(go.LAYERS):
        assert not dW[l, go.FAN_IN[l]:, :].any()
        assert not dW[l, :, go.FAN_OUT[l]:].any()
        assert not db[l, go.FAN_OUT[l]:].any()


def test_mixture_is_normalised():
    rng = np.random.default_rng(6)
    raw = rng.normal(size=(3, go.OUTPUTS))
    raw[:, 3 * go.LOBES:4 * go.LOBES] = rng.uniform(-1.0, 3.0, (3, go.LOBES))  # kappa up to ~3
    # quasi-uniform directions on the sphere (Fibonacci lattice)
    m = 200_000
    k = np.arange(m) + 0.5
    z = 1.0 - 2.0 * k / m
    phi = np.pi * (1.0 + 5 ** 0.5) * k
    r = np.sqrt(1.0 - z * z)
    d = np.stack([r * np.cos(phi), r * np.sin(phi), z], axis=1)
    for i in range(3):
        p = go.mixture_pdf(np.repeat(raw[i:i + 1], m, axis=0), d)
        assert abs(p.mean() * 4.0 * np.pi - 1.0) < 1e-3
