"""CPU oracle of the path-guiding network (test infrastructure only).

Only the tests, ``__graft_entry__.smoke()`` and ``bench.py`` import this
module, and only to check the CUDA kernels; nothing in the package calls it.

The reference renderer has no learned guiding, so there is no reference code
to follow here.  This restates, in float64 numpy, the published methods the
CUDA kernels implement:

* frequency encoding of (position, normal, outgoing direction): for each of
  the 9 coordinates v (position mapped to [0, 1] by the scene bounds, normal
  and direction mapped by (c + 1) / 2) and octaves k = 0, 1:
  sin(2^k pi v), cos(2^k pi v)  ->  36 inputs (the lowest period is 2, so
  that opposite directions, v = 0 and v = 1, encode differently);
* an MLP 36 -> 64 -> 64 -> 64 -> 64 -> 41 with ReLU, stored as five
  zero-padded 64 x 64 matrices W[l][in][out] and biases b[l][64];
* an 8-lobe von Mises-Fisher mixture read from the 40 outputs, field-major
  (output 8 f + i is field f of lobe i; per lobe: mean
  = o / |o|, kappa = min(softplus(o_k) + 0.01, 5000), weights = softmax of
  the logits bounded as 5 tanh(o_w / 5)), vMF density
  kappa / (2 pi (1 - e^{-2 kappa})) e^{kappa (mu.d - 1)};
* the sample loss -w log q(d) whose weighted sum over samples drawn from the
  renderer, w = lum(L_i) cos / pdf, estimates the KL divergence from the
  cosine-weighted incident radiance to the mixture, up to a constant
  (Mueller et al., "Neural Importance Sampling", ACM TOG 2019), plus
  w * 0.01 * sum over lobes of (|o| - 1)^2, which keeps the direction
  outputs' length near 1;
* the learned selection probability of the same paper: output 40 is the logit
  z of the guide's share a = A_MIN + (A_MAX - A_MIN) sigmoid(z) of the
  non-envmap sampling probability, trained on the KL divergence of the
  one-sample mixture a q(d) + (1 - a) p_bsdf(d): the term
  -w log(a q + (1 - a) p_bsdf) of a sample that carries its BSDF pdf
  (p_bsdf > 0), with q held fixed (its gradient reaches z only);
* Adam (Kingma and Ba, ICLR 2015) with bias correction.

With ``bf16=True`` the oracle rounds the values the kernels round to BF16
(the encoded inputs, the weights, every layer's output after bias and ReLU,
and every back-propagated gradient) to nearest-even BF16, and computes all
else in float64, so that the CUDA results differ from it only by FP32
accumulation order and the FP32 transcendental functions.  With
``bf16=False`` it is the exact float64 network, which the finite-difference
checks use.
"""
from __future__ import annotations

import numpy as np

LAYERS, WIDTH, INPUTS, OUTPUTS, LOBES = 5, 64, 36, 40, 8
SEL = 40              # output index of the selection-probability logit
NET_OUTPUTS = 41      # the mixture's 40 outputs and the selection logit
ROW_OUTPUTS = 48      # raw outputs per row as the inference entry point writes them
A_MIN, A_MAX = 0.05, 0.95  # range of the guide's share of the non-envmap probability
KAPPA_MAX = 5000.0
LOGIT_BOUND = 5.0     # lobe weight logits are LOGIT_BOUND * tanh(o / LOGIT_BOUND)
NORM_PENALTY = 0.01   # weight of (|o| - 1)^2 per lobe direction output
FAN_IN = [INPUTS, WIDTH, WIDTH, WIDTH, WIDTH]
FAN_OUT = [WIDTH, WIDTH, WIDTH, WIDTH, NET_OUTPUTS]


def bf16(x) -> np.ndarray:
    """Round to the nearest BF16 (ties to even), returned as float64."""
    f = np.asarray(x, np.float64).astype(np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) >> 16 << 16
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def encode(x9: np.ndarray, lo, inv_ext) -> np.ndarray:
    """36 frequency features of rows (x, n, wo).  The affine maps are done in
    float32 as the kernel does; the sines in float64."""
    x9 = np.asarray(x9, np.float32)
    lo = np.asarray(lo, np.float32)
    ie = np.asarray(inv_ext, np.float32)
    v = np.empty_like(x9)
    v[:, 0:3] = (x9[:, 0:3] - lo) * ie
    v[:, 3:9] = np.float32(0.5) * (x9[:, 3:9] + np.float32(1.0))
    out = np.empty((x9.shape[0], INPUTS), np.float64)
    o = 0
    for i in range(9):
        for k in range(2):
            a = np.pi * (v[:, i] * np.float32(1 << k)).astype(np.float64)
            out[:, o] = np.sin(a)
            out[:, o + 1] = np.cos(a)
            o += 2
    return out


def forward(W: np.ndarray, b: np.ndarray, feats: np.ndarray, bf16_round: bool = True):
    """Raw outputs (n, 41) and each layer's input (for backward)."""
    W = np.asarray(W, np.float64)
    b = np.asarray(b, np.float64)
    Wq = bf16(W) if bf16_round else W
    h = np.zeros((feats.shape[0], WIDTH))
    h[:, :INPUTS] = bf16(feats) if bf16_round else feats
    acts = []
    for l in range(LAYERS):
        acts.append(h)
        z = h @ Wq[l] + b[l]
        if l + 1 < LAYERS:
            z = np.maximum(z, 0.0)
            h = bf16(z) if bf16_round else z
        else:
            h = z
    return h[:, :NET_OUTPUTS], acts


def softplus(x):
    return np.where(x > 20.0, x, np.log1p(np.exp(np.minimum(x, 20.0))))


def lobes(raw: np.ndarray) -> np.ndarray:
    """The mixture's raw outputs (the first 40 of a row), field-major (output
    8 f + i is field f of lobe i), as (n, lobe, field)."""
    return np.ascontiguousarray(raw[:, :OUTPUTS]).reshape(-1, 5, LOBES).transpose(0, 2, 1)


def alpha(raw: np.ndarray) -> np.ndarray:
    """The guide's share of the non-envmap sampling probability per row."""
    z = np.asarray(raw, np.float64)[:, SEL]
    return A_MIN + (A_MAX - A_MIN) / (1.0 + np.exp(-z))


def mixture(raw: np.ndarray):
    """(mu (n,8,3), kappa (n,8), weights (n,8), |o| (n,8), tanh of the scaled
    logits (n,8)) of raw outputs."""
    o = lobes(raw)
    nrm = np.maximum(np.linalg.norm(o[:, :, 0:3], axis=2), 1e-12)
    mu = o[:, :, 0:3] / nrm[:, :, None]
    kappa = np.minimum(softplus(o[:, :, 3]) + 0.01, KAPPA_MAX)
    th = np.tanh(o[:, :, 4] / LOGIT_BOUND)
    lg = LOGIT_BOUND * th
    e = np.exp(lg - lg.max(axis=1, keepdims=True))
    pi = e / e.sum(axis=1, keepdims=True)
    return mu, kappa, pi, nrm, th


def vmf_pdf(kappa, c):
    return kappa / (2.0 * np.pi * -np.expm1(-2.0 * kappa)) * np.exp(kappa * (c - 1.0))


def mixture_pdf(raw: np.ndarray, d: np.ndarray) -> np.ndarray:
    mu, kappa, pi, _, _ = mixture(raw)
    c = np.einsum("nkc,nc->nk", mu, d)
    return (pi * vmf_pdf(kappa, c)).sum(axis=1)


def penalty(raw: np.ndarray, w: np.ndarray) -> np.ndarray:
    """Per-sample w * NORM_PENALTY * sum over lobes of (|o| - 1)^2."""
    nrm = np.linalg.norm(lobes(raw)[:, :, 0:3], axis=2)
    return w * NORM_PENALTY * ((nrm - 1.0) ** 2).sum(axis=1)


def selection_loss(raw: np.ndarray, d: np.ndarray, w: np.ndarray, pb: np.ndarray, q_fixed=None) -> np.ndarray:
    """Per-sample -w log(a q + (1 - a) p_bsdf) for samples with p_bsdf > 0 (else 0),
    with q the mixture density (or `q_fixed`, the density the gradient treats as
    a constant)."""
    q = mixture_pdf(raw, d) if q_fixed is None else q_fixed
    a = alpha(raw)
    live = pb > 0.0
    mix = np.where(live, a * q + (1.0 - a) * pb, 1.0)
    return np.where(live, -w * np.log(np.maximum(mix, 1e-30)), 0.0)


def loss_and_grad(raw: np.ndarray, d: np.ndarray, w: np.ndarray, pb: np.ndarray | None = None):
    """Per-sample loss -w log q(d), and the gradient with respect to the raw
    outputs (n, 41), analytic, of -w log q(d) + penalty + the selection term
    -w log(a q(d) + (1 - a) p_bsdf) (samples with p_bsdf > 0; q held fixed)."""
    o = lobes(raw)
    mu, kappa, pi, nrm, th = mixture(raw)
    c = np.einsum("nkc,nc->nk", mu, d)
    f = vmf_pdf(kappa, c)
    q = np.maximum((pi * f).sum(axis=1), 1e-30)
    r = pi * f / q[:, None]
    W = w[:, None]
    g = np.zeros_like(o)
    g[:, :, 4] = -W * (r - pi) * (1.0 - th * th)
    dlogf = 1.0 / kappa - 2.0 * np.exp(-2.0 * kappa) / -np.expm1(-2.0 * kappa) + (c - 1.0)
    dk = np.where(softplus(o[:, :, 3]) + 0.01 < KAPPA_MAX, 1.0 / (1.0 + np.exp(-o[:, :, 3])), 0.0)
    g[:, :, 3] = -W * r * dlogf * dk
    gmu = (-W * r * kappa)[:, :, None] * d[:, None, :]
    gm = (gmu * mu).sum(axis=2, keepdims=True)
    g[:, :, 0:3] = (gmu - gm * mu) / nrm[:, :, None] + (2.0 * W * NORM_PENALTY * (nrm - 1.0))[:, :, None] * mu
    gout = np.zeros((raw.shape[0], NET_OUTPUTS))
    gout[:, :OUTPUTS] = g.transpose(0, 2, 1).reshape(-1, OUTPUTS)
    if pb is not None and raw.shape[1] > SEL:
        pb = np.asarray(pb, np.float64)
        z = np.asarray(raw, np.float64)[:, SEL]
        sg = 1.0 / (1.0 + np.exp(-z))
        a = A_MIN + (A_MAX - A_MIN) * sg
        live = pb > 0.0
        mix = np.maximum(a * q + (1.0 - a) * pb, 1e-30)
        gout[:, SEL] = np.where(live, -w * (q - pb) / mix * (A_MAX - A_MIN) * sg * (1.0 - sg), 0.0)
    return -w * np.log(q), gout


def backward(W: np.ndarray, acts, dy_out: np.ndarray, bf16_round: bool = True):
    """Gradients (dW (5,64,64), db (5,64)) of sum(loss) given d loss / d raw."""
    W = np.asarray(W, np.float64)
    Wq = bf16(W) if bf16_round else W
    dy = np.zeros((dy_out.shape[0], WIDTH))
    dy[:, :dy_out.shape[1]] = dy_out
    if bf16_round:
        dy = bf16(dy)
    dW = np.zeros((LAYERS, WIDTH, WIDTH))
    db = np.zeros((LAYERS, WIDTH))
    for l in range(LAYERS - 1, -1, -1):
        dW[l] = acts[l].T @ dy
        db[l] = dy.sum(axis=0)
        if l == 0:
            break
        dx = (dy @ Wq[l].T) * (acts[l] > 0.0)
        dy = bf16(dx) if bf16_round else dx
    return dW, db


def gradients(W, b, samples: np.ndarray, lo, inv_ext, weight_scale: float = 1.0, bf16_round: bool = True):
    """(loss, dW, db) of a batch of samples (n, 16): x, n, wo, wi, weight,
    BSDF pdf of wi (0: none).  The loss is the sum of -w log q(d); the
    gradients include the selection term."""
    s = np.asarray(samples, np.float32)
    feats = encode(s[:, 0:9], lo, inv_ext)
    raw, acts = forward(W, b, feats, bf16_round)
    w = s[:, 12].astype(np.float64) * weight_scale
    loss, g = loss_and_grad(raw, s[:, 9:12].astype(np.float64), w, s[:, 13].astype(np.float64))
    g[w <= 0.0] = 0.0
    loss[w <= 0.0] = 0.0
    dW, db = backward(W, acts, g, bf16_round)
    return float(loss.sum()), dW, db


def objective(W, b, samples: np.ndarray, lo, inv_ext, weight_scale: float = 1.0, bf16_round: bool = False,
              q_fixed=None) -> float:
    """The function the gradients differentiate: sum of -w log q(d) + penalty
    + the selection term, in which q is `q_fixed` (the mixture density at the
    point of differentiation: the gradient treats it as a constant)."""
    s = np.asarray(samples, np.float32)
    raw, _ = forward(W, b, encode(s[:, 0:9], lo, inv_ext), bf16_round)
    w = s[:, 12].astype(np.float64) * weight_scale
    d = s[:, 9:12].astype(np.float64)
    loss, _ = loss_and_grad(raw, d, w)
    sel = selection_loss(raw, d, w, s[:, 13].astype(np.float64), q_fixed)
    keep = w > 0.0
    return float(loss[keep].sum() + penalty(raw, w)[keep].sum() + sel[keep].sum())


def mixture_density(W, b, samples: np.ndarray, lo, inv_ext, bf16_round: bool = False) -> np.ndarray:
    """q(d) of each sample's direction under the network (W, b)."""
    s = np.asarray(samples, np.float32)
    raw, _ = forward(W, b, encode(s[:, 0:9], lo, inv_ext), bf16_round)
    return mixture_pdf(raw, s[:, 9:12].astype(np.float64))


def adam(p, g, m, v, t: int, lr=1e-3, beta1=0.9, beta2=0.999, eps=1e-8):
    """One Adam step at iteration t (1-based), float32 like the kernel."""
    f = np.float32
    p, g, m, v = (np.asarray(a, np.float32) for a in (p, g, m, v))
    m = f(beta1) * m + f(1.0 - beta1) * g
    v = f(beta2) * v + f(1.0 - beta2) * g * g
    bc1 = f(1.0) - f(np.float32(beta1) ** f(t))
    bc2 = f(1.0) - f(np.float32(beta2) ** f(t))
    p = p - f(lr) * (m / bc1) / (np.sqrt(v / bc2) + f(eps))
    return p, m, v


def init_weights(seed: int = 0):
    """He-uniform weights inside the real network shape, zero padding and biases
    (a test initialisation, not the library's)."""
    rng = np.random.default_rng(seed)
    W = np.zeros((LAYERS, WIDTH, WIDTH), np.float32)
    for l in range(LAYERS):
        lim = np.sqrt(6.0 / FAN_IN[l])
        W[l, :FAN_IN[l], :FAN_OUT[l]] = rng.uniform(-lim, lim, (FAN_IN[l], FAN_OUT[l]))
    b = np.zeros((LAYERS, WIDTH), np.float32)
    for l in range(LAYERS):
        b[l, :FAN_OUT[l]] = rng.uniform(-0.1, 0.1, FAN_OUT[l])
    return W, b


def random_samples(n: int, seed: int, lo=(-1, -1, -1), hi=(1, 1, 1)) -> np.ndarray:
    """Training rows (n, 16): position in the box, unit normal, unit wo facing
    the normal, unit wi, weight in [0.1, 2)."""
    rng = np.random.default_rng(seed)
    s = np.zeros((n, 16), np.float32)
    lo = np.asarray(lo, np.float64)
    hi = np.asarray(hi, np.float64)
    s[:, 0:3] = lo + (hi - lo) * rng.random((n, 3))

    def unit(k):
        v = rng.normal(size=(k, 3))
        return v / np.linalg.norm(v, axis=1, keepdims=True)

    nrm = unit(n)
    wo = unit(n)
    wo *= np.sign((wo * nrm).sum(axis=1, keepdims=True))
    s[:, 3:6] = nrm
    s[:, 6:9] = wo
    s[:, 9:12] = unit(n)
    s[:, 12] = 0.1 + 1.9 * rng.random(n)
    # the BSDF pdf of wi: a cosine lobe around the normal (0 below it), none for every 8th
    c = (s[:, 9:12] * nrm).sum(axis=1)
    s[:, 13] = np.where(np.arange(n) % 8 == 7, 0.0, np.maximum(c, 0.0) / np.pi)
    return s
