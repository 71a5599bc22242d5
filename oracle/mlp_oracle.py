"""NumPy restatement of the learned seed proposal's network (CPU oracle).

TEST INFRASTRUCTURE ONLY: imported by tests/ as the checker of the GPU
training and inference kernels (specular-manifold-sampling_gb300/csrc/sms_mlp.cu),
never by the library.

The proposal has no counterpart in the reference (it seeds walks uniformly,
src/librender/manifold_ss.cpp:223), so there is nothing of the reference to
pin here: this module is pinned by finite differences of its own FP64
backward pass (tests/test_mlp_oracle.py) and by the closed forms it restates:

    network   9 features -> xn = (x - shift) * scale -> [xn, sin(pi 2^j xn),
              cos(pi 2^j xn) for j < 4] (81 inputs, zero-padded to 96)
              -> [64] x 4 with SiLU -> 48 outputs (40 used)
    mixture   8 logits o[0:8], means anchor + o[8:24] (u, v pairs),
              log-sigmas kLsMin + (kLsMax - kLsMin) * sigmoid(o[24:40]);
              the anchor is the uv where the segment shading point -> light
              sample meets the caster frame's plane (box frames, clamped to
              [-1, 2]^2) or the sphere point along the bisector of the
              directions to both (sphere frames)
    loss      mean negative log-likelihood of the solution uv
    Adam      beta1 0.9, beta2 0.999, eps 1e-8, bias-corrected

`bf=True` reproduces where the GPU rounds to bfloat16 (layer inputs and
weights in the forward pass; pre-activation gradients and weights in the
backward pass); accumulation stays FP64 here, FP32 on the tensor cores.
"""
from __future__ import annotations

import numpy as np

N_IN, ENC_FREQ, HIDDEN, N_OUT, OUT_PAD, COMP = 9, 4, 64, 40, 48, 8
N_ENC = N_IN * (1 + 2 * ENC_FREQ)   # 81 network inputs
IN_PAD = 96
LAYERS = [(IN_PAD, HIDDEN), (HIDDEN, HIDDEN), (HIDDEN, HIDDEN), (HIDDEN, HIDDEN), (HIDDEN, OUT_PAD)]
LS_MIN, LS_MAX = -7.0, 0.0
N_PARAMS = sum(o * i + o for i, o in LAYERS)
assert N_PARAMS == 21808


def bf16(x) -> np.ndarray:
    """Round to the nearest bfloat16 (ties to even), returned as float32."""
    a = np.ascontiguousarray(x, np.float32)
    b = a.view(np.uint32).astype(np.uint64)
    b = (b + 0x7FFF + ((b >> 16) & 1)) & 0xFFFF0000
    return b.astype(np.uint32).view(np.float32).reshape(a.shape)


def unpack(params: np.ndarray):
    """[(W [out][in], b [out]), ...] views of the flat parameter vector."""
    out, off = [], 0
    for i, o in LAYERS:
        W = params[off:off + o * i].reshape(o, i)
        off += o * i
        b = params[off:off + o]
        off += o
        out.append((W, b))
    return out


def sigmoid(z):
    return 1.0 / (1.0 + np.exp(-z))


def inputs(feat: np.ndarray, shift, scale, dtype=np.float32) -> np.ndarray:
    """Network inputs (batch x 96) from features (9 x batch): normalised
    features, then per feature sin (pi 2^j xn) for j < 4 and cos (pi 2^j xn),
    then zeros."""
    x = (np.asarray(feat, dtype).T - np.asarray(shift, dtype)) * np.asarray(scale, dtype)
    cols = [x.astype(np.float64)]
    for f in range(N_IN):
        a = np.pi * x[:, f:f + 1].astype(np.float64) * (2.0 ** np.arange(ENC_FREQ))
        cols += [np.sin(a), np.cos(a)]
    out = np.concatenate(cols + [np.zeros((x.shape[0], IN_PAD - N_ENC))], axis=1)
    return out.astype(dtype)


def forward(params, shift, scale, feat, bf: bool = True):
    """Raw outputs (batch x 48) and the cache for backward.  bf=False runs
    everything in FP64 (the finite-difference reference)."""
    dt = np.float32 if bf else np.float64
    layers = unpack(np.asarray(params, dt))
    h = inputs(feat, shift, scale, dt).astype(np.float64)
    cache = []
    for li, (W, b) in enumerate(layers):
        Wm = W.copy()
        if li == 0:
            Wm[:, N_ENC:] = 0.0
        hin = bf16(h).astype(np.float64) if bf else h
        Wq = (bf16(Wm) if bf else Wm).astype(np.float64)
        z = hin @ Wq.T + b.astype(np.float64)
        cache.append((hin, Wq, z))
        h = z if li == len(layers) - 1 else z * sigmoid(z)
    return h, cache


def frame_uv(frame, p: np.ndarray) -> np.ndarray:
    """uv (2 x n) of points p (3 x n) in a caster frame (kind, org, ax_u, ax_v)."""
    fr = np.asarray(frame, np.float64)
    d = np.asarray(p, np.float64) - fr[1:4, None]
    if int(fr[0]) == 1:
        r = fr[4]
        u = np.arccos(np.clip(d[2] / r, -1, 1)) / np.pi
        ph = np.arctan2(d[1], d[0])
        ph = np.where(ph < 0, ph + 2 * np.pi, ph)
        return np.stack([u, ph / (2 * np.pi)])
    au, av = fr[4:7], fr[7:10]
    return np.stack([au @ d / (au @ au), av @ d / (av @ av)])


def anchor(frame, feat: np.ndarray) -> np.ndarray:
    """Anchor uv (2 x n) of the mixture means for features (9 x n)."""
    fr = np.asarray(frame, np.float64)
    x, lp = np.asarray(feat[0:3], np.float64), np.asarray(feat[3:6], np.float64)
    o = fr[1:4, None]
    if int(fr[0]) == 1:
        a = (x - o) / np.linalg.norm(x - o, axis=0)
        b = (lp - o) / np.linalg.norm(lp - o, axis=0)
        h = a + b
        l2 = (h * h).sum(0)
        d = np.where(l2 > 1e-12, h / np.sqrt(np.maximum(l2, 1e-30)), a)
        return frame_uv(fr, o + d * fr[4])
    nrm = np.cross(fr[4:7], fr[7:10])
    d = lp - x
    den = nrm @ d
    ok = np.abs(den) > 1e-12 * np.sqrt((d * d).sum(0) * (nrm @ nrm))
    t = np.where(ok, (nrm @ (o - x)) / np.where(ok, den, 1.0), 0.5)
    return np.clip(frame_uv(fr, x + d * t), -1.0, 2.0)


def mixture_nll(o: np.ndarray, uv: np.ndarray):
    """Per-sample NLL (batch) and its gradient w.r.t. the 48 outputs."""
    o = np.asarray(o, np.float64)
    logits, mu = o[:, 0:8], o[:, 8:24].reshape(-1, COMP, 2)
    raw = o[:, 24:40].reshape(-1, COMP, 2)
    sg = sigmoid(raw)
    ls = LS_MIN + (LS_MAX - LS_MIN) * sg
    lmax = logits.max(axis=1, keepdims=True)
    logz = lmax + np.log(np.exp(logits - lmax).sum(axis=1, keepdims=True))
    e = np.asarray(uv, np.float64).T[:, None, :] - mu          # batch x 8 x 2
    iv = np.exp(-2.0 * ls)
    lp = (logits - logz) - np.log(2 * np.pi) - ls.sum(axis=2) - 0.5 * (e * e * iv).sum(axis=2)
    m = lp.max(axis=1, keepdims=True)
    logp = m + np.log(np.exp(lp - m).sum(axis=1, keepdims=True))
    r = np.exp(lp - logp)                                        # responsibilities
    g = np.zeros((o.shape[0], OUT_PAD))
    g[:, 0:8] = np.exp(logits - logz) - r
    g[:, 8:24] = (-r[:, :, None] * e * iv).reshape(-1, 16)
    g[:, 24:40] = (r[:, :, None] * (1.0 - e * e * iv) * (LS_MAX - LS_MIN) * sg * (1.0 - sg)).reshape(-1, 16)
    return -logp[:, 0], g


def loss_grad(params, shift, scale, feat, uv, bf: bool = True, frame=None, weights=None):
    """Mean (weighted) NLL over the batch and its gradient (flat, parameter
    layout): loss = sum_b w_b NLL_b / B.

    With bf=True the backward pass rounds the pre-activation gradients and
    weights to bfloat16 where the GPU does (straight-through for the forward
    roundings).  With a frame, targets are taken relative to the anchor."""
    o, cache = forward(params, shift, scale, feat, bf)
    rel = np.asarray(uv, np.float64) - (anchor(frame, feat) if frame is not None else 0.0)
    nll, g = mixture_nll(o, rel)
    B = o.shape[0]
    w = np.ones(B) if weights is None else np.asarray(weights, np.float64)
    nll = nll * w
    dz = g * (w / B)[:, None]
    grads = []
    for li in range(len(LAYERS) - 1, -1, -1):
        hin, Wq, z = cache[li]
        dzq = bf16(dz).astype(np.float64) if bf else dz
        dW = dzq.T @ hin
        db = dz.sum(axis=0)
        if li == 0:
            dW[:, N_ENC:] = 0.0
        grads.append((dW, db))
        if li:
            dh = dzq @ Wq
            zp = cache[li - 1][2]
            s = sigmoid(zp)
            dz = dh * (s * (1.0 + zp * (1.0 - s)))
    flat = np.concatenate([np.concatenate([dW.ravel(), db]) for dW, db in reversed(grads)])
    return float(nll.mean()), flat


def mixture(o: np.ndarray, anc: np.ndarray | None = None):
    """Processed mixture (batch x 40): cdf (8), means (16, anchor added when
    given as 2 x batch), sigmas (16)."""
    o = np.asarray(o, np.float64).copy()
    if anc is not None:
        o[:, 8:24:2] += anc[0][:, None]
        o[:, 9:24:2] += anc[1][:, None]
    w = np.exp(o[:, 0:8] - o[:, 0:8].max(axis=1, keepdims=True))
    cdf = np.cumsum(w / w.sum(axis=1, keepdims=True), axis=1)
    cdf[:, -1] = 1.0
    sig = np.exp(LS_MIN + (LS_MAX - LS_MIN) * sigmoid(o[:, 24:40]))
    return np.concatenate([cdf, o[:, 8:24], sig], axis=1)


def adam_step(params, grad, m, v, step: int, lr: float, b1=0.9, b2=0.999, eps=1e-8):
    """One bias-corrected Adam update (step = updates already taken)."""
    t = step + 1
    m = b1 * m + (1 - b1) * grad
    v = b2 * v + (1 - b2) * grad * grad
    p = params - lr * (m / (1 - b1 ** t)) / (np.sqrt(v / (1 - b2 ** t)) + eps)
    w0 = unpack(p)[0][0]
    w0[:, N_ENC:] = 0.0
    return p, m, v
