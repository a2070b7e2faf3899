"""Python mirror of include/fr_aonet.h: the learned ambient-occlusion U-Net.

Device tensors are passed as objects with ``data_ptr()`` (for example
``torch.Tensor`` on CUDA) or as raw integer device addresses. Input tensors are
BF16 chunk-planar ``[B][1][H][W][8]`` (as ``uint16``/``int16`` or ``bfloat16``
storage), AO and labels are ``float32 [B][H][W]``.
"""

from __future__ import annotations

import ctypes as C

import numpy as np

from . import _native as N
from . import RenderError

NUM_PARAMS = 120196


def _ptr(t) -> int:
    if t is None:
        return 0
    if isinstance(t, int):
        return t
    return int(t.data_ptr())


def _stream(s) -> int:
    if s is None:
        return 0
    if isinstance(s, int):
        return s
    return int(getattr(s, "cuda_stream", 0))


class AONet:
    """fr_aonet_*: create / parameters / forward / backward / Adam."""

    def __init__(self, device: int = 0, seed: int = 0):
        self._lib = N.lib()
        err = C.create_string_buffer(512)
        self._h = self._lib.fr_aonet_create(device, seed, err, 512)
        if not self._h:
            raise RenderError(N.FR_ERR_CUDA, err.value.decode())
        self.device = device

    def _check(self, rc: int, what: str):
        if rc != N.FR_OK:
            raise RenderError(rc, f"{what}: {self._lib.fr_aonet_last_error(self._h).decode()}")

    @property
    def handle(self) -> int:
        return self._h

    def get_params(self) -> np.ndarray:
        out = np.empty(NUM_PARAMS, np.float32)
        self._check(self._lib.fr_aonet_get_params(self._h, out.ctypes.data_as(C.POINTER(C.c_float)), NUM_PARAMS),
                    "get_params")
        return out

    def set_fused(self, fused: bool) -> None:
        """Renderer frames: the whole forward in one cooperative launch (True) or one
        launch per layer (False, default, the faster at 1280x800); identical results."""
        self._check(self._lib.fr_aonet_set_fused(self._h, int(fused)), "set_fused")

    def set_params(self, p: np.ndarray):
        p = np.ascontiguousarray(p, np.float32)
        self._check(self._lib.fr_aonet_set_params(self._h, p.ctypes.data_as(C.POINTER(C.c_float)), NUM_PARAMS),
                    "set_params")

    def get_grads(self) -> np.ndarray:
        out = np.empty(NUM_PARAMS, np.float32)
        self._check(self._lib.fr_aonet_get_grads(self._h, out.ctypes.data_as(C.POINTER(C.c_float)), NUM_PARAMS),
                    "get_grads")
        return out

    def forward(self, x, B: int, H: int, W: int, ao, stream=None):
        self._check(self._lib.fr_aonet_forward(self._h, _ptr(x), B, H, W, _ptr(ao), _stream(stream)), "forward")

    def backward(self, x, label, B: int, H: int, W: int, stream=None) -> float:
        loss = C.c_float(0)
        self._check(self._lib.fr_aonet_backward(self._h, _ptr(x), _ptr(label), B, H, W, C.byref(loss),
                                                _stream(stream)), "backward")
        return float(loss.value)

    def adam_step(self, lr: float = 1e-3, beta1: float = 0.9, beta2: float = 0.999, eps: float = 1e-8, stream=None):
        self._check(self._lib.fr_aonet_adam_step(self._h, lr, beta1, beta2, eps, _stream(stream)), "adam_step")

    def train_step(self, x, label, B: int, H: int, W: int, lr: float = 1e-3, stream=None,
                   want_loss: bool = True):
        loss = C.c_float(0)
        self._check(self._lib.fr_aonet_train_step(self._h, _ptr(x), _ptr(label), B, H, W, lr,
                                                  C.byref(loss) if want_loss else None, _stream(stream)),
                    "train_step")
        return float(loss.value) if want_loss else None

    def check(self, stream=None):
        self._check(self._lib.fr_aonet_check(self._h, _stream(stream)), "check")

    def launch_count(self) -> int:
        return int(self._lib.fr_aonet_last_launch_count(self._h))

    def close(self):
        if self._h:
            self._lib.fr_aonet_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def train(scene, net: AONet, render_cfg: N.Config, **overrides) -> tuple[dict, np.ndarray]:
    """fr_train_ao: renders the labelled views, trains `net`, evaluates it. Returns
    (report as a dict, logged losses)."""
    cfg = N.AOTrainConfig()
    N.lib().fr_ao_train_defaults(C.byref(cfg))
    for k, v in overrides.items():
        setattr(cfg, k, v)
    nlog = (cfg.steps // cfg.log_every + 2) if cfg.log_every > 0 else 2
    losses = np.zeros(max(nlog, 2), np.float32)
    rep = N.AOTrainReport()
    err = C.create_string_buffer(1024)
    rc = N.lib().fr_train_ao(scene.handle, net.handle, C.byref(render_cfg), C.byref(cfg), C.byref(rep),
                             losses.ctypes.data_as(C.POINTER(C.c_float)), err, len(err))
    if rc != N.FR_OK:
        raise RenderError(rc, "fr_train_ao: " + err.value.decode(errors="replace"))
    out = {name: getattr(rep, name) for name, _ in N.AOTrainReport._fields_}
    last = cfg.first_step + cfg.steps - 1
    n = sum(1 for s in range(cfg.first_step, last + 1)
            if (cfg.log_every > 0 and s % cfg.log_every == 0) or s == last)
    return out, losses[:n]


def pack_input(x4: np.ndarray) -> np.ndarray:
    """(B, 4, H, W) float -> chunk-planar BF16 bits (B, 1, H, W, 8) as uint16 (channels 4..7 zero)."""
    x4 = np.asarray(x4, np.float32)
    B, Cn, H, W = x4.shape
    out = np.zeros((B, 1, H, W, 8), np.float32)
    out[:, 0, :, :, :Cn] = np.transpose(x4, (0, 2, 3, 1))
    u = out.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) >> 16
    return u.astype(np.uint16)


def unpack_input(bits: np.ndarray) -> np.ndarray:
    """Chunk-planar BF16 bits (B, 1, H, W, 8) -> (B, 4, H, W) float32."""
    f = (np.asarray(bits, np.uint16).astype(np.uint32) << 16).view(np.float32)
    return np.transpose(f[:, 0, :, :, :4], (0, 3, 1, 2)).copy()
