"""ctypes mirror of ``include/forkerrenderer.h`` and loader of the native library.

Only plain C types cross this boundary. The library is built in-tree by
``forkerrenderer_gb300.build`` into ``forkerrenderer_gb300/_build``; importing a
symbol from a missing library raises instead of falling back to anything else.
"""

from __future__ import annotations

import ctypes as C
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
BUILD_DIR = os.path.join(_HERE, "_build")
LIB_PATH = os.path.join(BUILD_DIR, "libforkerrenderer.so")

FR_OK = 0
FR_ERR_INVALID = -1
FR_ERR_IO = -2
FR_ERR_PARSE = -3
FR_ERR_CUDA = -4
FR_ERR_OOM = -5
FR_ERR_BIN_OVERFLOW = -6
FR_ERR_TIMEOUT = -7
FR_ERR_UNSUPPORTED = -8

FR_SHADOW_HARD, FR_SHADOW_PCF, FR_SHADOW_PCSS = 0, 1, 2
FR_BLUR_REFERENCE, FR_BLUR_SEPARABLE, FR_BLUR_NONE = 0, 1, 2
FR_AO_SSAO, FR_AO_LEARNED = 0, 1
FR_NOALLOC_BLUR_MAX_PIXELS = 4 * 1024 * 1024

(FR_BUF_DEPTH, FR_BUF_SHADOW, FR_BUF_GB_NORMAL, FR_BUF_GB_POSITION, FR_BUF_GB_LIGHTNDC,
 FR_BUF_GB_ALBEDO, FR_BUF_GB_EMISSIVE, FR_BUF_GB_PARAM, FR_BUF_GB_TYPE, FR_BUF_AO,
 FR_BUF_FRAME_F32, FR_BUF_FRAME_U8, FR_BUF_SSAA_U8, FR_BUF_TRIANGLE_ID) = range(14)

f3 = C.c_float * 3
f16 = C.c_float * 16


class SceneInfo(C.Structure):
    _fields_ = [
        ("width", C.c_int32), ("height", C.c_int32), ("deferred", C.c_int32),
        ("ssaa_on", C.c_int32), ("ssaa_kernel", C.c_int32), ("ssao_on", C.c_int32),
        ("shadow_on", C.c_int32), ("perspective", C.c_int32),
        ("eye", f3), ("target", f3), ("light_pos", f3), ("light_color", f3),
        ("num_models", C.c_int32), ("num_meshes", C.c_int32), ("num_materials", C.c_int32),
        ("num_textures", C.c_int32),
        ("num_vertices", C.c_int64), ("num_uvs", C.c_int64), ("num_normals", C.c_int64),
        ("num_triangles", C.c_int64),
    ]


class ModelView(C.Structure):
    _fields_ = [("model_matrix", f16), ("position", f3), ("rotate_y", C.c_float), ("scale", C.c_float),
                ("has_tangents", C.c_int32), ("support_pbr", C.c_int32), ("first_mesh", C.c_int32),
                ("num_meshes", C.c_int32), ("first_vertex", C.c_int64), ("num_vertices", C.c_int64),
                ("first_normal", C.c_int64), ("num_normals", C.c_int64)]


class MeshView(C.Structure):
    _fields_ = [("model", C.c_int32), ("material", C.c_int32), ("first_triangle", C.c_int64),
                ("num_triangles", C.c_int64)]


class MaterialView(C.Structure):
    _fields_ = [("ka", f3), ("kd", f3), ("ks", f3), ("ke", f3), ("pbr_albedo", f3), ("roughness", C.c_float),
                ("metalness", C.c_float), ("map_kd", C.c_int32), ("map_ks", C.c_int32), ("map_ke", C.c_int32),
                ("map_bump", C.c_int32), ("map_ao", C.c_int32), ("map_pr", C.c_int32), ("map_pm", C.c_int32)]


class TextureView(C.Structure):
    _fields_ = [("width", C.c_int32), ("height", C.c_int32), ("bytes_per_pixel", C.c_int32),
                ("data", C.POINTER(C.c_uint8))]


class SceneView(C.Structure):
    _fields_ = [
        ("info", SceneInfo),
        ("models", C.c_void_p), ("meshes", C.c_void_p), ("materials", C.c_void_p),
        ("textures", C.c_void_p), ("positions", C.c_void_p), ("uvs", C.c_void_p),
        ("normals", C.c_void_p), ("tangents", C.c_void_p), ("tri_v", C.c_void_p),
        ("tri_vt", C.c_void_p), ("tri_vn", C.c_void_p), ("tri_mesh", C.c_void_p),
    ]


class FrameMatrices(C.Structure):
    _fields_ = [
        ("view", f16), ("projection", f16), ("view_projection", f16), ("light_space", f16),
        ("viewport", f16), ("shadow_viewport", f16),
        ("width", C.c_int32), ("height", C.c_int32),
        ("shadow_width", C.c_int32), ("shadow_height", C.c_int32),
    ]


class Config(C.Structure):
    _fields_ = [
        ("shadow_mode", C.c_int32), ("shadow_size", C.c_int32), ("pcf_samples", C.c_int32),
        ("blocker_samples", C.c_int32), ("ssao_samples", C.c_int32),
        ("ssao_radius", C.c_float), ("ssao_bias", C.c_float), ("ssao_range", C.c_float),
        ("blur_mode", C.c_int32), ("ao_mode", C.c_int32), ("keep_float_frame", C.c_int32),
        ("small_tri_area", C.c_int32), ("medium_tri_area", C.c_int32), ("bin_capacity", C.c_int64), ("device", C.c_int32),
        ("ao_probe_threshold", C.c_float), ("frame_graph", C.c_int32),
        ("ao_input_samples", C.c_int32), ("texture_wrap", C.c_int32), ("texture_filter", C.c_int32),
        ("concurrent_passes", C.c_int32), ("blur_warmup", C.c_int32), ("pass_timings", C.c_int32),
    ]


class AOTrainConfig(C.Structure):
    _fields_ = [
        ("train_views", C.c_int32), ("eval_views", C.c_int32), ("steps", C.c_int32), ("batch", C.c_int32),
        ("crop", C.c_int32), ("lr", C.c_float), ("label_samples", C.c_int32), ("radius_min", C.c_float),
        ("radius_max", C.c_float), ("cos_min", C.c_float), ("cos_max", C.c_float), ("seed", C.c_uint64),
        ("log_every", C.c_int32), ("lr_final", C.c_float), ("first_step", C.c_int32),
        ("schedule_steps", C.c_int32),
    ]


class AOTrainReport(C.Structure):
    _fields_ = [
        ("steps_done", C.c_int32), ("first_loss", C.c_float), ("final_loss", C.c_float),
        ("eval_rmse", C.c_float), ("eval_rmse_covered", C.c_float), ("eval_max_err", C.c_float),
        ("plain_rmse", C.c_float), ("plain_rmse_covered", C.c_float), ("plain_max_err", C.c_float),
        ("probe_mean_avg", C.c_float), ("probe_mean_max", C.c_float),
        ("label_seconds", C.c_float), ("train_seconds", C.c_float), ("eval_seconds", C.c_float),
        ("width", C.c_int32), ("height", C.c_int32), ("none_rmse_covered", C.c_float),
    ]


class ViewDesc(C.Structure):
    _fields_ = [("matrices", FrameMatrices), ("eye", C.c_float * 3), ("ao_mode", C.c_int32)]


class LightDesc(C.Structure):
    _fields_ = [("type", C.c_int32), ("position", C.c_float * 3), ("direction", C.c_float * 3),
                ("color", C.c_float * 3), ("extent", C.c_float), ("shadow_size", C.c_int32)]


class BatchTuning(C.Structure):
    _fields_ = [("light_tile", C.c_int32), ("bin_batch", C.c_int32), ("ctas_per_sm", C.c_int32)]


FR_LIGHT_POINT, FR_LIGHT_DIRECTIONAL = 0, 1


class FrameParams(C.Structure):
    _fields_ = [("matrices", C.POINTER(FrameMatrices)), ("stream", C.c_void_p), ("eye", C.POINTER(C.c_float))]


_lib = None


def lib() -> C.CDLL:
    """The native library; raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError(
            f"native library {LIB_PATH} is missing: run forkerrenderer_gb300.build.build()")
    L = C.CDLL(LIB_PATH)
    vp, i32, i64, sz = C.c_void_p, C.c_int32, C.c_int64, C.c_size_t
    sigs = {
        "fr_scene_load": (vp, [C.c_char_p, C.c_char_p, sz]),
        "fr_scene_free": (None, [vp]),
        "fr_scene_get_info": (C.c_int, [vp, C.POINTER(SceneInfo)]),
        "fr_scene_get_view": (C.c_int, [vp, C.POINTER(SceneView)]),
        "fr_scene_from_view": (vp, [C.POINTER(SceneView), C.c_char_p, sz]),
        "fr_scene_tangents": (C.c_int64, [vp, C.POINTER(C.c_float), C.c_size_t]),
        "fr_scene_frame_matrices": (C.c_int, [vp, i32, C.POINTER(FrameMatrices)]),
        "fr_config_defaults": (None, [C.POINTER(Config)]),
        "fr_create": (vp, [C.POINTER(Config), C.c_char_p, sz]),
        "fr_destroy": (None, [vp]),
        "fr_last_error": (C.c_char_p, [vp]),
        "fr_upload_scene": (C.c_int, [vp, vp]),
        "fr_render_frame": (C.c_int, [vp, C.POINTER(FrameParams)]),
        "fr_shadow_pass": (C.c_int, [vp, C.POINTER(FrameParams)]),
        "fr_forward_pass": (C.c_int, [vp, C.POINTER(FrameParams)]),
        "fr_geometry_pass": (C.c_int, [vp, C.POINTER(FrameParams)]),
        "fr_ssao_pass": (C.c_int, [vp, C.POINTER(FrameParams)]),
        "fr_lighting_pass": (C.c_int, [vp, C.POINTER(FrameParams)]),
        "fr_ssaa_pass": (C.c_int, [vp, C.POINTER(FrameParams)]),
        "fr_download": (i64, [vp, i32, vp, sz]),
        "fr_last_timings": (C.c_int, [vp, C.POINTER(C.c_float), i32]),
        "fr_last_launch_count": (i32, [vp]),
        "fr_blur_separable_noalloc": (C.c_int, [vp, i32, i32, vp]),
        # learned AO (include/fr_aonet.h)
        "fr_aonet_create": (vp, [i32, C.c_uint64, C.c_char_p, sz]),
        "fr_aonet_destroy": (None, [vp]),
        "fr_aonet_set_fused": (C.c_int, [vp, i32]),
        "fr_aonet_set_wait_limit": (C.c_int, [vp, C.c_uint64]),
        "fr_aonet_get_state": (C.c_int, [vp, C.POINTER(C.c_float), C.POINTER(C.c_float), C.POINTER(C.c_float), i64,
                                         C.POINTER(C.c_int64)]),
        "fr_aonet_set_state": (C.c_int, [vp, C.POINTER(C.c_float), C.POINTER(C.c_float), C.POINTER(C.c_float), i64,
                                         i64]),
        "fr_aonet_test_absent_cta": (C.c_int, [vp, i32]),
        "fr_aonet_last_error": (C.c_char_p, [vp]),
        "fr_aonet_num_params": (i64, []),
        "fr_aonet_get_params": (C.c_int, [vp, C.POINTER(C.c_float), i64]),
        "fr_aonet_set_params": (C.c_int, [vp, C.POINTER(C.c_float), i64]),
        "fr_aonet_forward": (C.c_int, [vp, vp, i32, i32, i32, vp, vp]),
        "fr_aonet_backward": (C.c_int, [vp, vp, vp, i32, i32, i32, C.POINTER(C.c_float), vp]),
        "fr_aonet_get_grads": (C.c_int, [vp, C.POINTER(C.c_float), i64]),
        "fr_aonet_adam_step": (C.c_int, [vp, C.c_float, C.c_float, C.c_float, C.c_float, vp]),
        "fr_aonet_train_step": (C.c_int, [vp, vp, vp, i32, i32, i32, C.c_float, C.POINTER(C.c_float), vp]),
        "fr_aonet_check": (C.c_int, [vp, vp]),
        "fr_aonet_last_launch_count": (i32, [vp]),
        "fr_set_ao_net": (C.c_int, [vp, vp]),
        "fr_ao_features": (C.c_int, [vp, vp, vp]),
        "fr_ao_probe_result": (C.c_int, [vp, C.POINTER(C.c_float), C.POINTER(i32)]),
        "fr_scene_view_matrices": (C.c_int, [vp, C.POINTER(C.c_float), C.POINTER(C.c_float), i32,
                                             C.POINTER(FrameMatrices)]),
        "fr_ao_train_defaults": (None, [C.POINTER(AOTrainConfig)]),
        # batched multi-view rendering (include/fr_batch.h)
        "fr_batch_create": (vp, [vp, C.POINTER(ViewDesc), i32, C.POINTER(LightDesc), i32, C.c_char_p, sz]),
        "fr_batch_destroy": (None, [vp]),
        "fr_batch_last_error": (C.c_char_p, [vp]),
        "fr_batch_set_tuning": (C.c_int, [vp, C.POINTER(BatchTuning)]),
        "fr_batch_get_tuning": (C.c_int, [vp, C.POINTER(BatchTuning)]),
        "fr_batch_render": (C.c_int, [vp]),
        "fr_batch_timings": (C.c_int, [vp, C.POINTER(C.c_float), i32]),
        "fr_batch_autotune": (C.c_int, [vp, i32, C.POINTER(BatchTuning), C.POINTER(C.c_float)]),
        "fr_batch_work": (C.c_int, [vp, C.POINTER(i64), C.POINTER(i64), C.POINTER(i64)]),
        "fr_batch_download": (i64, [vp, i32, i32, vp, sz]),
        "fr_train_ao": (C.c_int, [vp, vp, C.POINTER(Config), C.POINTER(AOTrainConfig), C.POINTER(AOTrainReport),
                                  C.POINTER(C.c_float), C.c_char_p, sz]),
        # TGA output (include/fr_output.h)
        "fr_output_name": (C.c_char_p, [i32]),
        "fr_output_present": (C.c_int, [vp, i32]),
        "fr_output_shape": (C.c_int, [vp, i32, C.POINTER(i32), C.POINTER(i32), C.POINTER(i32)]),
        "fr_output_encode": (i64, [vp, i32, i32, vp, sz]),
        "fr_output_encode_all": (i64, [vp, i32, vp, sz, C.POINTER(i64), C.POINTER(C.c_float)]),
        "fr_output_write": (C.c_int, [vp, C.c_char_p, i32]),
        "fr_tga_max_bytes": (sz, [i32, i32, i32]),
        "fr_tga_scratch_bytes": (sz, [i32, i32]),
        "fr_tga_encode_device": (C.c_int, [vp, i32, i32, i32, i32, i32, vp, vp, vp, vp]),
    }
    for name, (res, args) in sigs.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _lib = L
    return L


def exported_symbols() -> list[str]:
    """Every function name the public headers declare (for load checks)."""
    import re

    names = []
    inc = os.path.join(os.path.dirname(_HERE), "include")
    for h in sorted(os.listdir(inc)):
        if not h.startswith(("forkerrenderer", "fr_aonet", "fr_batch", "fr_output")) or not h.endswith(".h"):
            continue
        with open(os.path.join(inc, h)) as f:
            txt = f.read()
        names += re.findall(r"^\s*(?:[\w\s\*]+?)\b(fr_\w+)\s*\(", txt, flags=re.M)
    return sorted(set(names))
