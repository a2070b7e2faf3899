"""The learned-AO oracle pinned on the CPU: analytic gradients against central
finite differences (float64, no BF16 rounding), BF16 rounding, and Adam."""

import os
import sys

import numpy as np
import pytest

sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "oracle"))
import aonet_ref as R  # noqa: E402


def _inputs(rng, B, H, W):
    x = np.zeros((B, 4, H, W))
    x[:, 0] = rng.uniform(0.5, 2.0, (B, H, W))
    n = rng.normal(size=(B, 3, H, W))
    x[:, 1:] = n / np.linalg.norm(n, axis=1, keepdims=True)
    return x


def _params(rng):
    p = np.zeros(R.NUM_PARAMS)
    off = 0
    for (_, _, co, _, ci) in R.LAYERS:
        n = co * ci * 9
        p[off:off + n] = rng.normal(0, np.sqrt(2.0 / (ci * 9)), n)
        p[off + n:off + n + co] = rng.normal(0, 0.05, co)
        off += n + co
    p[off:off + 64] = rng.normal(0, 0.25, 64)
    p[off + 64:off + 68] = 0.5
    return p


def test_param_count():
    assert R.NUM_PARAMS == 120196


def test_bf16_rounding():
    x = np.array([1.0, 1.00390625, 1.005859375, -3.0e-5, 65504.0, 1 + 2 ** -8, 1 + 3 * 2 ** -8], np.float32)
    y = R.bf16(x)
    assert y[0] == 1.0
    assert y[1] == 1.0  # exactly half way between 1 and 1 + 2^-7: ties to even
    assert y[2] == np.float32(1.0078125)
    assert (y.view(np.uint32) & 0xFFFF).max() == 0
    assert y[5] == 1.0 and y[6] == np.float32(1.015625)


def test_gradients_match_finite_differences():
    rng = np.random.default_rng(3)
    p = _params(rng)
    x = _inputs(rng, 1, 32, 64)
    label = rng.uniform(0.2, 0.9, (1, 32, 64))
    net = R.Net(p, emulate=False)
    net.forward(x)
    loss, g = net.backward(label)
    assert g.shape == (R.NUM_PARAMS,)

    def L(q):
        n = R.Net(q, emulate=False)
        ao = n.forward(x)
        return float(np.mean((ao - label) ** 2))

    assert abs(L(p) - loss) < 1e-12
    # a few parameters of every layer, the biases and the head
    idx = []
    off = 0
    for (_, _, co, _, ci) in R.LAYERS:
        n = co * ci * 9
        idx += list(rng.integers(off, off + n, 3)) + [off + n + int(rng.integers(0, co))]
        off += n + co
    idx += [off + 3, off + 40, off + 64, off + 67]
    h = 1e-6
    for i in idx:
        e = np.zeros_like(p)
        e[i] = h
        fd = (L(p + e) - L(p - e)) / (2 * h)
        assert abs(fd - g[i]) <= 1e-5 * max(1e-3, abs(fd)) + 1e-9, (i, fd, g[i])


def test_adam_matches_formula():
    rng = np.random.default_rng(5)
    p = rng.normal(size=100).astype(np.float32)
    g = rng.normal(size=100).astype(np.float32)
    m = np.zeros(100, np.float32)
    v = np.zeros(100, np.float32)
    p1, m1, v1 = R.adam_step(p, g, m, v, 1, lr=1e-3)
    # first step of bias-corrected Adam moves every parameter by about lr * sign(g)
    assert np.allclose(p - p1, 1e-3 * np.sign(g), atol=1e-6)
    p2, _, _ = R.adam_step(p1, g, m1, v1, 2, lr=1e-3)
    assert np.allclose(p1 - p2, 1e-3 * np.sign(g), atol=1e-6)


def test_upsample_is_bilinear_and_transpose_consistent():
    rng = np.random.default_rng(8)
    for n in (1, 2, 5):
        U = R._up_matrix(n)
        assert np.allclose(U.sum(axis=1), 1.0)
        # interior outputs interpolate the half-pixel-centred positions exactly
        for o in range(R.SCALE * n):
            pos = (o + 0.5) / R.SCALE - 0.5
            if 0 <= pos <= n - 1:
                assert abs(U[o] @ np.arange(n) - pos) < 1e-12
    net = R.Net(_params(rng), emulate=False)
    a = rng.normal(size=(1, 2, 3, 5))
    up = net._up(a)
    ref = np.einsum("yh,bchw,xw->bcyx", R._up_matrix(3), a, R._up_matrix(5))
    assert np.allclose(up, ref)


def test_space_to_depth_layout():
    x = np.arange(2 * 4 * 4 * 6, dtype=np.float64).reshape(2, 4, 4, 6)
    y = R.space_to_depth(x)
    assert y.shape == (2, 16, 2, 3)
    for r in range(2):
        for c in range(2):
            for ch in range(4):
                assert np.array_equal(y[:, 8 * r + 4 * c + ch], x[:, ch, r::2, c::2])
