"""CPU oracle of the learned-AO U-Net (test infrastructure only).

A numpy restatement of the network in ``include/fr_aonet.h``: forward pass,
analytic backward pass and one Adam step. The reference renderer has no learned
AO, so this oracle is pinned two ways instead: its analytic gradients are
checked against central finite differences in float64 (``emulate=False``), and
the GPU's tensor-core kernels are checked against it with BF16 rounding
emulated at the points where the GPU rounds (``emulate=True``): weights and
every stored activation / activation gradient are BF16, accumulation is
float32-or-better, biases and head weights stay float32.

Tensors are NCHW here; the GPU's chunk-planar layout is converted by the tests.
"""

from __future__ import annotations

import numpy as np

# (c0, c1, cout, level, cin_real) per 3x3 layer; order e0a e0b e1a e1b b0 b1 d1a d1b d0a d0b
LAYERS = [
    (16, 0, 16, 0, 16), (16, 0, 16, 0, 16), (16, 0, 32, 1, 16), (32, 0, 32, 1, 32),
    (32, 0, 64, 2, 32), (64, 0, 64, 2, 64), (64, 32, 32, 1, 96), (32, 0, 32, 1, 32),
    (32, 16, 16, 0, 48), (16, 0, 16, 0, 16),
]
HEAD_OUT = 4  # level 0 works on 2x2 pixel blocks; the head emits the 4 sub-pixels
NUM_PARAMS = sum(L[2] * L[4] * 9 + L[2] for L in LAYERS) + HEAD_OUT * 16 + HEAD_OUT
assert NUM_PARAMS == 120196
# Resolution step between levels: kScale x kScale average pooling, bilinear x kScale upsampling.
SCALE = 4
_NEAR_W = [0.625, 0.875, 0.875, 0.625]  # weight of the nearer input per upsampling phase


def bf16(a: np.ndarray) -> np.ndarray:
    """Round float32 values to the nearest BF16 (ties to even), returned as float32."""
    a32 = np.ascontiguousarray(a, dtype=np.float32)
    u = a32.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) >> 16 << 16
    return u.astype(np.uint32).view(np.float32).reshape(a32.shape)


def split_params(p: np.ndarray):
    """[(W[cout][cin][3][3], b[cout]) per layer], head w[4][16], head b[4]."""
    out, off = [], 0
    for (_, _, co, _, ci) in LAYERS:
        n = co * ci * 9
        W = p[off:off + n].reshape(co, ci, 3, 3)
        b = p[off + n:off + n + co]
        out.append((W, b))
        off += n + co
    return out, p[off:off + 64].reshape(4, 16), p[off + 64:off + 68]


def space_to_depth(x4: np.ndarray) -> np.ndarray:
    """(B, 4, H, W) -> (B, 16, H/2, W/2): channel 8 r + 4 c + ch = pixel (2Y + r, 2X + c)."""
    B, C, H, W = x4.shape
    out = np.zeros((B, 16, H // 2, W // 2), x4.dtype)
    for r in range(2):
        for c in range(2):
            out[:, 8 * r + 4 * c:8 * r + 4 * c + 4] = x4[:, :, r::2, c::2]
    return out


def _shift(x: np.ndarray, dy: int, dx: int) -> np.ndarray:
    """x[..., y + dy, x + dx] with zeros outside."""
    B, C, H, W = x.shape
    out = np.zeros_like(x)
    ys, ye = max(0, -dy), min(H, H - dy)
    xs, xe = max(0, -dx), min(W, W - dx)
    if ys < ye and xs < xe:
        out[:, :, ys:ye, xs:xe] = x[:, :, ys + dy:ye + dy, xs + dx:xe + dx]
    return out


def conv3x3(x: np.ndarray, W: np.ndarray) -> np.ndarray:
    """y[co](p) = sum_{ci, ky, kx} W[co, ci, ky, kx] x[ci](p + (ky - 1, kx - 1)), zero padding; float64."""
    x = x.astype(np.float64)
    W = W.astype(np.float64)
    B, C, H, Wd = x.shape
    y = np.zeros((B, W.shape[0], H, Wd))
    for ky in range(3):
        for kx in range(3):
            xs = _shift(x, ky - 1, kx - 1)
            y += np.einsum("oc,bchw->bohw", W[:, :, ky, kx], xs)
    return y


def conv3x3_dgrad(g: np.ndarray, W: np.ndarray) -> np.ndarray:
    """Gradient of conv3x3 with respect to its input."""
    g = g.astype(np.float64)
    W = W.astype(np.float64)
    dx = np.zeros((g.shape[0], W.shape[1], g.shape[2], g.shape[3]))
    for ky in range(3):
        for kx in range(3):
            dx += _shift(np.einsum("oc,bohw->bchw", W[:, :, ky, kx], g), -(ky - 1), -(kx - 1))
    return dx


def conv3x3_wgrad(x: np.ndarray, g: np.ndarray):
    """Gradients of conv3x3 with respect to W and a bias."""
    x = x.astype(np.float64)
    g = g.astype(np.float64)
    dW = np.zeros((g.shape[1], x.shape[1], 3, 3))
    for ky in range(3):
        for kx in range(3):
            dW[:, :, ky, kx] = np.einsum("bohw,bchw->oc", g, _shift(x, ky - 1, kx - 1))
    return dW, g.sum(axis=(0, 2, 3))


def _up_taps(o: int, n: int):
    """(i0, i1, w0, w1) of output o: position (o + 0.5) / SCALE - 0.5, indices clamped."""
    i, ph = o // SCALE, o % SCALE
    if ph < SCALE // 2:
        w1 = _NEAR_W[ph]
        return max(i - 1, 0), i, 1.0 - w1, w1
    w0 = _NEAR_W[ph]
    return i, min(i + 1, n - 1), w0, 1.0 - w0


def _up_matrix(n: int) -> np.ndarray:
    """U (SCALE n x n): bilinear upsampling by SCALE with half-pixel centres, clamped."""
    U = np.zeros((SCALE * n, n))
    for o in range(SCALE * n):
        i0, i1, w0, w1 = _up_taps(o, n)
        U[o, i0] += w0
        U[o, i1] += w1
    return U


class Net:
    """Forward / backward of the U-Net for parameters `p` (float32 vector)."""

    def __init__(self, p: np.ndarray, emulate: bool = True):
        self.emulate = emulate
        self.dt = np.float32 if emulate else np.float64
        self.R = bf16 if emulate else (lambda a: np.asarray(a, np.float64))
        self.layers, self.hw, self.hb = split_params(np.asarray(p, self.dt))
        self.Wq = [self.R(W) for (W, _) in self.layers]

    # ---- building blocks in the GPU's operation order ----
    def _conv_relu(self, L, x):
        y = conv3x3(x, self.Wq[L]).astype(self.dt) + self.layers[L][1].astype(self.dt)[None, :, None, None]
        return self.R(np.maximum(y, 0))

    def _pool(self, s):
        acc = np.zeros(s[:, :, ::SCALE, ::SCALE].shape, self.dt)
        for dy in range(SCALE):  # row by row, left to right, as the GPU sums
            for dx in range(SCALE):
                acc = acc + s[:, :, dy::SCALE, dx::SCALE]
        return self.R(acc * self.dt(1.0 / (SCALE * SCALE)))

    def _up(self, a):
        B, C, h, w = a.shape
        ty = [_up_taps(o, h) for o in range(SCALE * h)]
        tx = [_up_taps(o, w) for o in range(SCALE * w)]
        y0, y1 = np.array([t[0] for t in ty]), np.array([t[1] for t in ty])
        x0, x1 = np.array([t[0] for t in tx]), np.array([t[1] for t in tx])
        wy0 = np.array([t[2] for t in ty], self.dt)[:, None]
        wy1 = np.array([t[3] for t in ty], self.dt)[:, None]
        wx0 = np.array([t[2] for t in tx], self.dt)[None, :]
        wx1 = np.array([t[3] for t in tx], self.dt)[None, :]
        A = a[:, :, y0][:, :, :, x0]
        Bv = a[:, :, y0][:, :, :, x1]
        Cv = a[:, :, y1][:, :, :, x0]
        D = a[:, :, y1][:, :, :, x1]
        return self.R(wy0 * (wx0 * A + wx1 * Bv) + wy1 * (wx0 * Cv + wx1 * D))

    def forward(self, x4: np.ndarray) -> np.ndarray:
        """x4: (B, 4, H, W) -> AO (B, H, W)."""
        x = space_to_depth(np.asarray(x4, self.dt))
        c = {"x": x}
        c["a0"] = self._conv_relu(0, x)
        c["s0"] = self._conv_relu(1, c["a0"])
        c["p0"] = self._pool(c["s0"])
        c["a1"] = self._conv_relu(2, c["p0"])
        c["s1"] = self._conv_relu(3, c["a1"])
        c["p1"] = self._pool(c["s1"])
        c["a2"] = self._conv_relu(4, c["p1"])
        c["a3"] = self._conv_relu(5, c["a2"])
        c["u1"] = self._up(c["a3"])
        c["a4"] = self._conv_relu(6, np.concatenate([c["u1"], c["s1"]], axis=1))
        c["a5"] = self._conv_relu(7, c["a4"])
        c["u0"] = self._up(c["a5"])
        c["a6"] = self._conv_relu(8, np.concatenate([c["u0"], c["s0"]], axis=1))
        c["a7"] = self._conv_relu(9, c["a6"])
        B, _, h, w = c["a7"].shape
        ao = np.zeros((B, 2 * h, 2 * w), self.dt)
        for k in range(HEAD_OUT):
            z = np.zeros((B, h, w), self.dt)
            for ch in range(16):  # sequential float sum, as the GPU epilogue
                z = z + self.hw[k, ch] * c["a7"][:, ch]
            z = z + self.hb[k]
            ao[:, k >> 1::2, k & 1::2] = (self.dt(1) / (self.dt(1) + np.exp(-z))).astype(self.dt)
        c["ao"] = ao
        self.cache = c
        return ao

    def backward(self, label: np.ndarray):
        """Loss (mean squared error over B*H*W, pixels with a negative label
        contributing 0) and the flat gradient (parameter order)."""
        c, R, dt = self.cache, self.R, self.dt
        ao = c["ao"]
        N = ao.size
        lab = np.asarray(label, dt)
        diff = np.where(lab >= 0, ao - lab, dt(0))  # negative labels are outside the loss
        loss = float(np.sum(diff.astype(np.float64) ** 2) / N)
        invN = dt(1.0) / dt(N)
        dz = dt(2) * diff * invN * ao * (dt(1) - ao)
        a7 = c["a7"]
        dzk = [dz[:, k >> 1::2, k & 1::2] for k in range(HEAD_OUT)]  # per sub-pixel, (B, h, w)
        gs = dzk[0][:, None] * self.hw[0][None, :, None, None]
        for k in range(1, HEAD_OUT):  # same order as the GPU
            gs = gs + dzk[k][:, None] * self.hw[k][None, :, None, None]
        g7 = R(np.where(a7 > 0, gs, 0))
        dhw = np.stack([np.einsum("bhw,bchw->c", dzk[k].astype(np.float64), a7.astype(np.float64))
                        for k in range(HEAD_OUT)])
        dhb = np.array([float(np.sum(dzk[k].astype(np.float64))) for k in range(HEAD_OUT)])
        grads = [None] * len(LAYERS)

        def mask(g, act):
            return np.where(act > 0, g, 0)

        def dgrad(L, g):
            return conv3x3_dgrad(g, self.Wq[L]).astype(dt)

        grads[9] = conv3x3_wgrad(c["a6"], g7)
        g6 = R(mask(dgrad(9, g7), c["a6"]))
        grads[8] = conv3x3_wgrad(np.concatenate([c["u0"], c["s0"]], axis=1), g6)
        d8 = R(dgrad(8, g6))
        gu0, gs0c = d8[:, :32], d8[:, 32:]
        h1, w1 = c["a5"].shape[2:]
        g5 = R(mask(np.einsum("yh,bcyx,xw->bchw", _up_matrix(h1), gu0.astype(np.float64),
                              _up_matrix(w1)).astype(dt), c["a5"]))
        grads[7] = conv3x3_wgrad(c["a4"], g5)
        g4 = R(mask(dgrad(7, g5), c["a4"]))
        grads[6] = conv3x3_wgrad(np.concatenate([c["u1"], c["s1"]], axis=1), g4)
        d6 = R(dgrad(6, g4))
        gu1, gs1c = d6[:, :64], d6[:, 64:]
        h2, w2 = c["a3"].shape[2:]
        g3 = R(mask(np.einsum("yh,bcyx,xw->bchw", _up_matrix(h2), gu1.astype(np.float64),
                              _up_matrix(w2)).astype(dt), c["a3"]))
        grads[5] = conv3x3_wgrad(c["a2"], g3)
        g2 = R(mask(dgrad(5, g3), c["a2"]))
        grads[4] = conv3x3_wgrad(c["p1"], g2)
        gp1 = R(dgrad(4, g2))
        up1 = np.repeat(np.repeat(gp1, SCALE, axis=2), SCALE, axis=3)
        gS1 = R(mask(gs1c + dt(1.0 / (SCALE * SCALE)) * up1, c["s1"]))
        grads[3] = conv3x3_wgrad(c["a1"], gS1)
        g1 = R(mask(dgrad(3, gS1), c["a1"]))
        grads[2] = conv3x3_wgrad(c["p0"], g1)
        gp0 = R(dgrad(2, g1))
        up0 = np.repeat(np.repeat(gp0, SCALE, axis=2), SCALE, axis=3)
        gS0 = R(mask(gs0c + dt(1.0 / (SCALE * SCALE)) * up0, c["s0"]))
        grads[1] = conv3x3_wgrad(c["a0"], gS0)
        g0 = R(mask(dgrad(1, gS0), c["a0"]))
        grads[0] = conv3x3_wgrad(c["x"], g0)
        flat = []
        for (dW, db) in grads:
            flat += [dW.ravel(), db.ravel()]
        flat += [dhw.ravel(), dhb.ravel()]
        return loss, np.concatenate(flat)


def adam_step(p, g, m, v, t, lr=1e-3, b1=0.9, b2=0.999, eps=1e-8):
    """PyTorch's Adam in float32, matching fr_aonet_adam_step."""
    f = np.float32
    p, g, m, v = (np.asarray(a, f).copy() for a in (p, g, m, v))
    bc1 = 1.0 - b1 ** t
    bc2 = 1.0 - b2 ** t
    step = f(lr / bc1)
    bc2s = f(np.sqrt(bc2))
    m = f(b1) * m + (f(1) - f(b1)) * g
    v = f(b2) * v + (f(1) - f(b2)) * (g * g)
    p = p - step * (m / (np.sqrt(v) / bc2s + f(eps)))
    return p, m, v
