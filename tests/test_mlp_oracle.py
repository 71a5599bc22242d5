"""CPU checks of the learned proposal's NumPy oracle (oracle/mlp_oracle.py).

The proposal has no counterpart in the reference, so the oracle is pinned by
its own mathematics: the FP64 backward pass against central finite
differences, the mixture gradient against finite differences of the NLL,
bfloat16 rounding against hand-worked values, and Adam against its closed
form on the first step.
"""
import numpy as np
import pytest

from oracle import mlp_oracle as M

FD_RTOL = 1e-5   # FP64 central differences, step 1e-6


def _net(seed=0, scale=0.3):
    rng = np.random.default_rng(seed)
    p = rng.uniform(-scale, scale, M.N_PARAMS)
    for W, _ in M.unpack(p)[:1]:
        W[:, M.N_ENC:] = 0.0
    return p


def _batch(seed=1, n=8):
    rng = np.random.default_rng(seed)
    feat = rng.normal(size=(M.N_IN, n))
    uv = rng.uniform(0.2, 0.8, size=(2, n))
    return feat, uv


def test_bf16_rounding_known_values():
    # spacing of bfloat16 at 1 is 2^-7: 1 + 2^-8 ties to even (down), 1 + 3 2^-8
    # ties to even (up), 1 + 2^-9 rounds down
    x = np.array([1.0, 1.0 + 2.0 ** -8, 1.0 + 3 * 2.0 ** -8, -2.5, 1.0 + 2.0 ** -9], np.float32)
    want = np.array([1.0, 1.0, 1.0 + 2.0 ** -6, -2.5, 1.0], np.float32)
    got = M.bf16(x)
    assert got.tolist() == want.tolist()
    # every result is representable in bfloat16: low 16 bits clear
    assert not np.any(got.view(np.uint32) & 0xFFFF)


def test_parameter_layout():
    assert M.N_PARAMS == 21808
    layers = M.unpack(np.arange(M.N_PARAMS, dtype=np.float64))
    assert [W.shape for W, _ in layers] == [(64, 96), (64, 64), (64, 64), (64, 64), (48, 64)]
    assert layers[0][1][0] == 64 * 96 and layers[-1][1][-1] == M.N_PARAMS - 1


def test_mixture_gradient_matches_finite_differences():
    rng = np.random.default_rng(5)
    o = rng.normal(scale=0.5, size=(4, M.OUT_PAD))
    o[:, 8:24] += 0.5
    uv = rng.uniform(0.3, 0.7, size=(2, 4))
    _, g = M.mixture_nll(o, uv)
    h = 1e-6
    for c in list(range(0, 40, 3)) + [39]:
        d = np.zeros_like(o)
        d[:, c] = h
        fd = (M.mixture_nll(o + d, uv)[0] - M.mixture_nll(o - d, uv)[0]) / (2 * h)
        np.testing.assert_allclose(g[:, c], fd, rtol=1e-5, atol=1e-8)
    assert np.all(g[:, 40:] == 0)


def test_backward_matches_finite_differences():
    p = _net()
    shift, scale = np.zeros(9), np.ones(9)
    feat, uv = _batch()
    loss, g = M.loss_grad(p, shift, scale, feat, uv, bf=False)
    assert np.isfinite(loss)
    rng = np.random.default_rng(2)
    # one sample of indices from every weight and bias block
    idx = []
    off = 0
    for i, o in M.LAYERS:
        cols = rng.integers(0, M.N_ENC if i == M.IN_PAD else i, 3)
        rows = rng.integers(0, o, 3)
        idx += [off + r * i + c for r, c in zip(rows, cols)]
        off += o * i
        idx += [off + int(k) for k in rng.integers(0, o, 2)]
        off += o
    h = 1e-6
    for k in idx:
        d = np.zeros_like(p)
        d[k] = h
        fd = (M.loss_grad(p + d, shift, scale, feat, uv, bf=False)[0] -
              M.loss_grad(p - d, shift, scale, feat, uv, bf=False)[0]) / (2 * h)
        assert abs(g[k] - fd) <= FD_RTOL * max(1.0, abs(fd)) + 1e-7, (k, g[k], fd)
    # padded input columns of the first layer carry no gradient
    assert np.all(M.unpack(g)[0][0][:, M.N_ENC:] == 0)


def test_bf16_backward_close_to_exact():
    p = _net(3, scale=0.1)
    feat, uv = _batch(4, 64)
    l0, g0 = M.loss_grad(p, np.zeros(9), np.ones(9), feat, uv, bf=False)
    l1, g1 = M.loss_grad(p, np.zeros(9), np.ones(9), feat, uv, bf=True)
    assert abs(l0 - l1) < 2e-2 * max(1.0, abs(l0))
    cos = g0 @ g1 / np.linalg.norm(g0) / np.linalg.norm(g1)
    assert cos > 0.999


def test_adam_first_step_closed_form():
    rng = np.random.default_rng(7)
    p = _net(7)
    g = rng.normal(size=M.N_PARAMS)
    lr = 1e-3
    p1, m1, v1 = M.adam_step(p, g, np.zeros_like(p), np.zeros_like(p), 0, lr)
    # step 1: m_hat = g, v_hat = g^2  ->  update = lr * g / (|g| + eps)
    want = p - lr * g / (np.abs(g) + 1e-8)
    M.unpack(want)[0][0][:, M.N_ENC:] = 0.0
    np.testing.assert_allclose(p1, want, rtol=0, atol=1e-12)
    np.testing.assert_allclose(m1, 0.1 * g)
    np.testing.assert_allclose(v1, 0.001 * g * g)


def test_processed_mixture_properties():
    rng = np.random.default_rng(9)
    o = rng.normal(size=(16, M.OUT_PAD))
    mx = M.mixture(o)
    cdf = mx[:, :8]
    assert np.all(np.diff(cdf, axis=1) >= 0) and np.all(cdf[:, -1] == 1.0)
    w = np.exp(o[:, :8]) / np.exp(o[:, :8]).sum(1, keepdims=True)
    np.testing.assert_allclose(cdf[:, 0], w[:, 0], rtol=1e-12)
    sig = mx[:, 24:]
    assert np.all(sig >= np.exp(M.LS_MIN) - 1e-12) and np.all(sig <= np.exp(M.LS_MAX) + 1e-12)
    np.testing.assert_array_equal(mx[:, 8:24], o[:, 8:24])


@pytest.mark.parametrize("n", [1, 17])
def test_inputs_normalised_encoded_and_padded(n):
    feat = np.arange(9 * n, dtype=np.float32).reshape(9, n) / 7.0
    shift = np.arange(9, dtype=np.float32)
    scale = np.full(9, 0.5, np.float32)
    x = M.inputs(feat, shift, scale, np.float64)
    assert x.shape == (n, 96)
    xn = (feat.T - shift) * scale
    np.testing.assert_allclose(x[:, :9], xn, rtol=1e-6)
    # feature 4, frequency 2^2: sin at column 9 + 4 * 8 + 2, cos 4 columns later
    np.testing.assert_allclose(x[:, 9 + 32 + 2], np.sin(4 * np.pi * xn[:, 4]), atol=1e-5)
    np.testing.assert_allclose(x[:, 9 + 32 + 6], np.cos(4 * np.pi * xn[:, 4]), atol=1e-5)
    assert np.all(x[:, 81:] == 0)


def test_anchor_box_and_sphere_frames():
    box = np.array([0, -1, -1, 1, 2, 0, 0, 0, 2, 0], np.float64)   # plane z = 1 over [-1, 1]^2
    feat = np.zeros((9, 3))
    feat[0:3] = np.array([[0.0, 0.5, 0.0], [0.0, -0.5, 0.0], [0.0, 0.0, 0.0]])   # shading points (x, y, z)
    feat[3:6] = np.array([[0.0, 0.5, 30.0], [0.0, 0.5, 0.0], [10.0, 10.0, 10.0]])  # light samples
    a = M.anchor(box, feat)
    # segment (0,0,0) -> (0,0,10) meets z = 1 at the centre of the box
    np.testing.assert_allclose(a[:, 0], [0.5, 0.5])
    # (0.5,-0.5,0) -> (0.5,0.5,10) meets z = 1 at (0.5, -0.4)
    np.testing.assert_allclose(a[:, 1], [0.75, 0.3])
    # (0,0,0) -> (30, 0, 10): z = 1 at x = 3, clamped to u = 2
    np.testing.assert_allclose(a[:, 2], [2.0, 0.5])
    sph = np.array([1, 0, 0, 0, 2.0, 0, 0, 0, 0, 0], np.float64)
    f = np.zeros((9, 1))
    f[0:3, 0] = [5.0, 0.0, 0.0]
    f[3:6, 0] = [0.0, 5.0, 0.0]
    a = M.anchor(sph, f)
    # bisector of +x and +y: theta = pi/2, phi = pi/4
    np.testing.assert_allclose(a[:, 0], [0.5, 0.125], atol=1e-12)
    mx = M.mixture(np.zeros((1, M.OUT_PAD)), a)
    np.testing.assert_allclose(mx[0, 8:24:2], 0.5)
    np.testing.assert_allclose(mx[0, 9:24:2], 0.125)
