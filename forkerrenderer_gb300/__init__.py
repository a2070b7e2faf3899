"""ForkerRenderer-GB300: the reference renderer's per-frame pipeline on one GB300.

Host-side mirror of the reference's interface over the C ABI of
``include/forkerrenderer.h`` (ctypes, plain C types only):

* :class:`Scene` - ``Scene(filename)`` of src/scene.h:61-71 (loads .scene/.obj/.mtl/.tga);
* :class:`Renderer` - a render context holding the device-side ``ForkerGL::``
  buffers (src/forkergl.h:41-51) with the passes of ``Render::`` (src/render.h:22-37):
  ``Preconfigure``, ``Render``, ``DoShadowPass``, ``DoForwardPass``,
  ``DoGeometryPass``, ``DoLightingPass``, ``DoSSAO``, ``DoSSAA``;
* buffer accessors returning numpy arrays in the reference's layouts
  (``Buffer1f`` / ``Buffer3f`` index ``x + y * width``; here shaped (H, W[, 3])).

Every call goes to the CUDA library; if it is missing the calls raise.
"""

from __future__ import annotations

import ctypes as C

import numpy as np

from . import _native as N

__all__ = ["Scene", "Renderer", "Config", "FrameMatrices", "RenderError"]

Config = N.Config
FrameMatrices = N.FrameMatrices


class RenderError(RuntimeError):
    def __init__(self, code: int, message: str):
        super().__init__(f"[{code}] {message}")
        self.code = code


class Scene:
    """A loaded scene (Scene::Scene, src/scene.cpp:19-196)."""

    def __init__(self, path: str):
        err = C.create_string_buffer(1024)
        h = N.lib().fr_scene_load(path.encode(), err, len(err))
        if not h:
            raise RenderError(N.FR_ERR_PARSE, err.value.decode(errors="replace"))
        self._h = C.c_void_p(h)
        self.path = path
        info = N.SceneInfo()
        N.lib().fr_scene_get_info(self._h, C.byref(info))
        self.info = info

    @property
    def handle(self) -> C.c_void_p:
        return self._h

    def view(self) -> N.SceneView:
        v = N.SceneView()
        N.lib().fr_scene_get_view(self._h, C.byref(v))
        return v

    def frame_matrices(self, shadow_size: int = 0) -> N.FrameMatrices:
        m = N.FrameMatrices()
        N.lib().fr_scene_frame_matrices(self._h, int(shadow_size), C.byref(m))
        return m

    def view_matrices(self, eye, target, shadow_size: int = 0) -> N.FrameMatrices:
        """Frame matrices with the camera at `eye` looking at `target`."""
        m = N.FrameMatrices()
        e = (C.c_float * 3)(*[float(v) for v in eye])
        t = (C.c_float * 3)(*[float(v) for v in target])
        rc = N.lib().fr_scene_view_matrices(self._h, e, t, int(shadow_size), C.byref(m))
        if rc != N.FR_OK:
            raise RenderError(rc, "fr_scene_view_matrices failed")
        return m

    # Scene accessors of src/scene.h
    def GetWidth(self) -> int:
        return self.info.width

    def GetHeight(self) -> int:
        return self.info.height

    def GetRatio(self) -> float:
        return float(np.float32(self.info.width) / np.float32(self.info.height))

    def IsSSAAOn(self) -> bool:
        return bool(self.info.ssaa_on)

    def GetSSAAKernelSize(self) -> int:
        return self.info.ssaa_kernel

    def IsSSAOOn(self) -> bool:
        return bool(self.info.ssao_on)

    def GetModelCount(self) -> int:
        return self.info.num_models

    def close(self) -> None:
        if getattr(self, "_h", None):
            N.lib().fr_scene_free(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def default_config(**overrides) -> N.Config:
    """The reference's defaults (shadow.h:12-23, render.cpp:219-258), overridable."""
    cfg = N.Config()
    N.lib().fr_config_defaults(C.byref(cfg))
    for k, v in overrides.items():
        setattr(cfg, k, v)
    return cfg


class Renderer:
    """Render context: device buffers + the passes of ``Render::``."""

    def __init__(self, config: N.Config | None = None, **overrides):
        cfg = config if config is not None else default_config(**overrides)
        if config is not None:
            for k, v in overrides.items():
                setattr(cfg, k, v)
        err = C.create_string_buffer(1024)
        h = N.lib().fr_create(C.byref(cfg), err, len(err))
        if not h:
            raise RenderError(N.FR_ERR_CUDA, err.value.decode(errors="replace"))
        self._h = C.c_void_p(h)
        self.config = cfg
        self.scene: Scene | None = None
        self._params = N.FrameParams()

    def _check(self, rc: int) -> int:
        if rc < 0:
            raise RenderError(rc, N.lib().fr_last_error(self._h).decode(errors="replace"))
        return rc

    @property
    def handle(self) -> C.c_void_p:
        return self._h

    # ---- Render:: --------------------------------------------------------------------------
    def Preconfigure(self, scene: Scene) -> None:
        """Render::Preconfigure (render.cpp:33-38): binds the scene (uploads it)."""
        self._check(N.lib().fr_upload_scene(self._h, scene.handle))
        self.scene = scene

    def set_matrices(self, m: N.FrameMatrices | None, eye=None) -> None:
        """Use these frame matrices instead of the scene's (None = scene's). eye:
        the camera position those matrices look from (None = the scene's eye), the
        origin of the lighting's view vector."""
        self._mats = m
        self._params.matrices = C.pointer(m) if m is not None else None
        self._eye = (C.c_float * 3)(*[float(v) for v in eye]) if eye is not None else None
        self._params.eye = C.cast(self._eye, C.POINTER(C.c_float)) if eye is not None else None

    def set_stream(self, stream_ptr: int | None) -> None:
        self._params.stream = stream_ptr

    def Render(self, scene: Scene | None = None) -> None:
        """Render::Render (render.cpp:40-58)."""
        if scene is not None and scene is not self.scene:
            self.Preconfigure(scene)
        self._check(N.lib().fr_render_frame(self._h, C.byref(self._params)))

    def DoShadowPass(self) -> None:
        self._check(N.lib().fr_shadow_pass(self._h, C.byref(self._params)))

    def DoForwardPass(self) -> None:
        self._check(N.lib().fr_forward_pass(self._h, C.byref(self._params)))

    def DoGeometryPass(self) -> None:
        self._check(N.lib().fr_geometry_pass(self._h, C.byref(self._params)))

    def DoSSAO(self) -> None:
        self._check(N.lib().fr_ssao_pass(self._h, C.byref(self._params)))

    def DoLightingPass(self) -> None:
        """Render::DoLightingPass: SSAO (if on) then DrawScreenSpacePixels."""
        self._check(N.lib().fr_lighting_pass(self._h, C.byref(self._params)))

    def DoSSAA(self) -> None:
        self._check(N.lib().fr_ssaa_pass(self._h, C.byref(self._params)))

    # ---- read-back (ForkerGL:: buffers) ------------------------------------------------------
    def download(self, buffer_id: int, out: np.ndarray | None = None) -> np.ndarray:
        """One buffer of the last frame (flat). out: a caller's array to fill (for
        example a view of pinned host memory), of the buffer's size in bytes."""
        n = N.lib().fr_download(self._h, buffer_id, None, 0)
        self._check(n)
        if out is None:
            if buffer_id in (N.FR_BUF_FRAME_U8, N.FR_BUF_SSAA_U8):
                out = np.empty(n, np.uint8)
            elif buffer_id == N.FR_BUF_TRIANGLE_ID:
                out = np.empty(n // 4, np.int32)
            else:
                out = np.empty(n // 4, np.float32)
        elif out.nbytes < n or not out.flags["C_CONTIGUOUS"]:
            raise ValueError(f"out needs {n} contiguous bytes")
        self._check(N.lib().fr_download(self._h, buffer_id, out.ctypes.data_as(C.c_void_p), n))
        return out

    def _shape(self, arr: np.ndarray, comps: int, which: str = "screen") -> np.ndarray:
        m = getattr(self, "_mats", None) or self.scene.frame_matrices(self.config.shadow_size)
        if which == "shadow":
            return arr.reshape(m.shadow_height, m.shadow_width)
        if which == "ssaa":
            k = self.scene.info.ssaa_kernel
            return arr.reshape(m.height // k, m.width // k, comps)
        return arr.reshape(m.height, m.width, comps) if comps > 1 else arr.reshape(m.height, m.width)

    def depth(self):
        return self._shape(self.download(N.FR_BUF_DEPTH), 1)

    def shadow_map(self):
        return self._shape(self.download(N.FR_BUF_SHADOW), 1, "shadow")

    def gbuffer(self, name: str) -> np.ndarray:
        ids = {"normal": N.FR_BUF_GB_NORMAL, "position": N.FR_BUF_GB_POSITION,
               "lightndc": N.FR_BUF_GB_LIGHTNDC, "albedo": N.FR_BUF_GB_ALBEDO,
               "emissive": N.FR_BUF_GB_EMISSIVE, "param": N.FR_BUF_GB_PARAM}
        if name == "type":
            return self._shape(self.download(N.FR_BUF_GB_TYPE), 1)
        return self._shape(self.download(ids[name]), 3)

    def ambient_occlusion(self):
        return self._shape(self.download(N.FR_BUF_AO), 1)

    def frame(self):
        return self._shape(self.download(N.FR_BUF_FRAME_F32), 3)

    def frame8(self, out: np.ndarray | None = None):
        """FrameBuffer.GenerateImage() bytes, (H, W, 3) R, G, B (into `out` when given)."""
        return self._shape(self.download(N.FR_BUF_FRAME_U8, out), 3)

    def ssaa8(self):
        return self._shape(self.download(N.FR_BUF_SSAA_U8), 3, "ssaa")

    def triangle_ids(self):
        return self._shape(self.download(N.FR_BUF_TRIANGLE_ID), 1)

    def scene_tangents(self) -> np.ndarray:
        """The uploaded scene's per-vertex tangents as the device holds them, (V, 3)."""
        n = N.lib().fr_scene_tangents(self._h, None, 0)
        self._check(n)
        out = np.empty(n // 4, np.float32)
        self._check(N.lib().fr_scene_tangents(self._h, out.ctypes.data_as(C.POINTER(C.c_float)), out.nbytes))
        return out.reshape(-1, 3)

    # ---- Output:: (include/fr_output.h) -------------------------------------------------------
    def encode_tga(self, image: int, rle: bool = True) -> bytes | None:
        """One output TGA file of the last frame (output.FR_OUT_*), None if the reference writes none."""
        from . import output

        return output.encode(self, image, rle)

    def write_outputs(self, directory: str = "output", rle: bool = True) -> list[str]:
        """Every TGA file the reference's main.cpp writes after a frame, into `directory`."""
        from . import output

        return output.write_all(self, directory, rle)

    TIMING_NAMES = ("shadow", "geometry", "ssao", "blur", "lighting", "ssaa", "total")

    def timings(self) -> dict:
        """Per-pass device milliseconds of the last Render (CUDA events)."""
        ms = (C.c_float * 7)()
        self._check(N.lib().fr_last_timings(self._h, ms, 7))
        return dict(zip(self.TIMING_NAMES, list(ms)))

    def launch_count(self) -> int:
        return int(N.lib().fr_last_launch_count(self._h))

    # ---- learned AO (include/fr_aonet.h) ------------------------------------------------------
    def set_ao_net(self, net) -> None:
        """Network used when config.ao_mode == FR_AO_LEARNED (None detaches)."""
        self._aonet = net
        self._check(N.lib().fr_set_ao_net(self._h, net.handle if net is not None else None))

    def ao_features(self, dst, stream=None) -> None:
        """Network input of the last geometry pass into device tensor `dst` ([1][1][H][W][8] BF16)."""
        ptr = dst if isinstance(dst, int) else int(dst.data_ptr())
        self._check(N.lib().fr_ao_features(self._h, ptr, stream))

    def ao_probe_result(self) -> tuple[float, bool]:
        """(mean squared difference on the 1-in-64 probe, whether the frame fell back to plain SSAO)."""
        m = C.c_float(0)
        g = C.c_int32(0)
        self._check(N.lib().fr_ao_probe_result(self._h, C.byref(m), C.byref(g)))
        return float(m.value), bool(g.value)

    def close(self) -> None:
        if getattr(self, "_h", None):
            N.lib().fr_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
