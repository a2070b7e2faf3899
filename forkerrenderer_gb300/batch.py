"""Python mirror of include/fr_batch.h: many views of one scene (uneven sizes,
several lights with shadow maps) rendered together as one CUDA graph."""

from __future__ import annotations

import ctypes as C

import numpy as np

from . import RenderError, Renderer
from . import _native as N


def view(matrices: N.FrameMatrices, eye, ao_mode: int = N.FR_AO_SSAO) -> N.ViewDesc:
    v = N.ViewDesc()
    C.memmove(C.byref(v.matrices), C.byref(matrices), C.sizeof(matrices))
    v.eye[:] = [float(x) for x in eye]
    v.ao_mode = ao_mode
    return v


def point_light(position, color=(1.0, 1.0, 1.0), shadow_size: int = 2048) -> N.LightDesc:
    L = N.LightDesc()
    L.type = N.FR_LIGHT_POINT
    L.position[:] = [float(x) for x in position]
    L.color[:] = [float(x) for x in color]
    L.shadow_size = shadow_size
    return L


def directional_light(direction, color=(1.0, 1.0, 1.0), shadow_size: int = 2048, extent: float = 6.0) -> N.LightDesc:
    L = N.LightDesc()
    L.type = N.FR_LIGHT_DIRECTIONAL
    L.direction[:] = [float(x) for x in direction]
    L.color[:] = [float(x) for x in color]
    L.extent = extent
    L.shadow_size = shadow_size
    return L


class Batch:
    """fr_batch_*: create / tune / render / read back."""

    STAGES = ("binning", "fine_raster", "resolve_ao", "lighting", "total")

    def __init__(self, renderer: Renderer, views, lights):
        self._r = renderer  # keeps the context alive
        va = (N.ViewDesc * len(views))(*views)
        la = (N.LightDesc * len(lights))(*lights)
        err = C.create_string_buffer(1024)
        h = N.lib().fr_batch_create(renderer._h, va, len(views), la, len(lights), err, len(err))
        if not h:
            raise RenderError(N.FR_ERR_INVALID, err.value.decode(errors="replace"))
        self._h = C.c_void_p(h)
        self.sizes = [(v.matrices.width, v.matrices.height) for v in views]
        self.shadow_sizes = [L.shadow_size for L in lights]

    def _check(self, rc: int) -> int:
        if rc < 0:
            raise RenderError(rc, N.lib().fr_batch_last_error(self._h).decode(errors="replace"))
        return rc

    def render(self) -> None:
        self._check(N.lib().fr_batch_render(self._h))

    def timings(self) -> dict:
        ms = (C.c_float * 5)()
        self._check(N.lib().fr_batch_timings(self._h, ms, 5))
        return dict(zip(self.STAGES, list(ms)))

    @property
    def tuning(self) -> tuple[int, int, int]:
        t = N.BatchTuning()
        self._check(N.lib().fr_batch_get_tuning(self._h, C.byref(t)))
        return (t.light_tile, t.bin_batch, t.ctas_per_sm)

    def set_tuning(self, light_tile: int, bin_batch: int, ctas_per_sm: int) -> None:
        t = N.BatchTuning(light_tile, bin_batch, ctas_per_sm)
        self._check(N.lib().fr_batch_set_tuning(self._h, C.byref(t)))

    def autotune(self, reps: int = 3) -> tuple[tuple[int, int, int], float]:
        t = N.BatchTuning()
        ms = C.c_float(0)
        self._check(N.lib().fr_batch_autotune(self._h, reps, C.byref(t), C.byref(ms)))
        return (t.light_tile, t.bin_batch, t.ctas_per_sm), float(ms.value)

    def work(self) -> dict:
        t, p, s = C.c_int64(0), C.c_int64(0), C.c_int64(0)
        self._check(N.lib().fr_batch_work(self._h, C.byref(t), C.byref(p), C.byref(s)))
        return {"triangles": t.value, "pixels": p.value, "shadow_texels": s.value}

    def download(self, view: int, buffer_id: int) -> np.ndarray:
        n = self._check(N.lib().fr_batch_download(self._h, view, buffer_id, None, 0))
        if buffer_id == N.FR_BUF_FRAME_U8:
            out = np.empty(n, np.uint8)
        else:
            out = np.empty(n // 4, np.float32)
        self._check(N.lib().fr_batch_download(self._h, view, buffer_id, out.ctypes.data_as(C.c_void_p), n))
        if view < 0:
            s = self.shadow_sizes[-1 - view]
            return out.reshape(s, s)
        w, h = self.sizes[view]
        return out.reshape(h, w, 3) if buffer_id == N.FR_BUF_FRAME_U8 else out.reshape(h, w)

    def close(self) -> None:
        if getattr(self, "_h", None):
            N.lib().fr_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
