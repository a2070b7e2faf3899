"""Test-side bridge to the CPU oracle (oracle/_build/liboracle.so) and to the
reference harness binaries (oracle/_ref/ref_*). Test infrastructure only."""

from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

from forkerrenderer_gb300 import _native as N

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ORACLE_LIB = os.path.join(ROOT, "oracle", "_build", "liboracle.so")
REF_DIR = os.path.join(ROOT, "oracle", "_ref")


class OracleConfig(C.Structure):
    _fields_ = [
        ("shadow_mode", C.c_int32), ("shadow_size", C.c_int32), ("pcf_samples", C.c_int32),
        ("blocker_samples", C.c_int32), ("ssao_samples", C.c_int32),
        ("ssao_radius", C.c_float), ("ssao_bias", C.c_float), ("ssao_range", C.c_float),
        ("blur_mode", C.c_int32), ("threads", C.c_int32), ("texture_wrap", C.c_int32),
        ("texture_filter", C.c_int32),
    ]


_FP = C.POINTER(C.c_float)
_BP = C.POINTER(C.c_uint8)


class OracleOut(C.Structure):
    _fields_ = [
        ("depth", _FP), ("shadow", _FP), ("gb_normal", _FP), ("gb_position", _FP),
        ("gb_lightndc", _FP), ("gb_albedo", _FP), ("gb_emissive", _FP), ("gb_param", _FP),
        ("gb_type", _FP), ("ao", _FP), ("frame", _FP), ("frame8", _BP), ("ssaa8", _BP),
        ("seconds", C.c_double),
    ]


_olib = None


def oracle_lib() -> C.CDLL:
    global _olib
    if _olib is None:
        if not os.path.exists(ORACLE_LIB):
            from forkerrenderer_gb300.build import build_oracle

            build_oracle()
        L = C.CDLL(ORACLE_LIB)
        L.fr_oracle_render.restype = C.c_int
        L.fr_oracle_render.argtypes = [C.POINTER(N.SceneView), C.POINTER(OracleConfig),
                                       C.POINTER(N.FrameMatrices), C.POINTER(OracleOut)]
        L.fr_oracle_matrices.restype = C.c_int
        L.fr_oracle_matrices.argtypes = [C.POINTER(N.SceneView), C.c_int32,
                                         C.POINTER(N.FrameMatrices)]
        L.fr_oracle_u8.restype = C.c_uint8
        L.fr_oracle_u8.argtypes = [C.c_float]
        L.fr_oracle_image_1f.argtypes = [_FP, C.c_int64, _BP]
        L.fr_oracle_image_3f.argtypes = [_FP, C.c_int64, _BP]
        L.fr_oracle_tga_max_bytes.restype = C.c_int64
        L.fr_oracle_tga_max_bytes.argtypes = [C.c_int64, C.c_int64, C.c_int32]
        L.fr_oracle_tga_encode.restype = C.c_int64
        L.fr_oracle_tga_encode.argtypes = [_BP, C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.c_int32,
                                           _BP, C.c_int64]
        _olib = L
    return _olib


# ---- TGA output ----------------------------------------------------------------------

def oracle_image(values: np.ndarray) -> np.ndarray:
    """Buffer1f / Buffer3f::GenerateImage of a float buffer: (H, W) -> (H, W) gray bytes,
    (H, W, 3) -> (H, W, 3) bytes in TGA order (B, G, R)."""
    v = np.ascontiguousarray(values, np.float32)
    n = v.shape[0] * v.shape[1]
    out = np.empty(v.shape, np.uint8)
    fn = oracle_lib().fr_oracle_image_3f if v.ndim == 3 else oracle_lib().fr_oracle_image_1f
    fn(v.ctypes.data_as(_FP), n, out.ctypes.data_as(_BP))
    return out


def oracle_tga(pixels: np.ndarray, rle: bool = True, vflip: bool = True) -> bytes:
    """TGAImage::WriteTgaFile of an (H, W) or (H, W, bytespp) uint8 image in TGA byte order."""
    px = np.ascontiguousarray(pixels, np.uint8)
    h, w = px.shape[:2]
    bpp = 1 if px.ndim == 2 else px.shape[2]
    L = oracle_lib()
    cap = L.fr_oracle_tga_max_bytes(w, h, bpp)
    out = np.empty(cap, np.uint8)
    size = L.fr_oracle_tga_encode(px.ctypes.data_as(_BP), w, h, bpp, int(rle), int(vflip),
                                  out.ctypes.data_as(_BP), cap)
    if size < 0:
        raise ValueError("bad TGA arguments")
    return out[:size].tobytes()


def rgb_to_tga_order(rgb: np.ndarray) -> np.ndarray:
    """(H, W, 3) R, G, B bytes -> B, G, R (TGAColor's layout)."""
    return np.ascontiguousarray(rgb[..., ::-1])


def reference_tga(pixels: np.ndarray, rle: bool = True, vflip: bool = True) -> bytes:
    """The reference's own TGAImage::Set + WriteTgaFile on an image (oracle/_ref/ref_tga)."""
    import tempfile

    px = np.ascontiguousarray(pixels, np.uint8)
    h, w = px.shape[:2]
    bpp = 1 if px.ndim == 2 else px.shape[2]
    with tempfile.TemporaryDirectory() as d:
        src, dst = os.path.join(d, "px.raw"), os.path.join(d, "out.tga")
        px.tofile(src)
        subprocess.run([os.path.join(REF_DIR, "ref_tga"), src, str(w), str(h), str(bpp), str(int(rle)),
                        str(int(vflip)), dst], check=True, capture_output=True)
        with open(dst, "rb") as f:
            return f.read()


def reference_config(**kw) -> dict:
    """The reference's own constants (shadow.h:16-23, render.cpp:219-258)."""
    cfg = dict(shadow_mode=2, shadow_size=0, pcf_samples=64, blocker_samples=32,
               ssao_samples=32, ssao_radius=0.075, ssao_bias=0.0005, ssao_range=0.01,
               blur_mode=0, threads=os.cpu_count() or 4)
    cfg.update(kw)
    return cfg


def oracle_matrices(view: N.SceneView, shadow_size: int) -> N.FrameMatrices:
    m = N.FrameMatrices()
    rc = oracle_lib().fr_oracle_matrices(C.byref(view), shadow_size, C.byref(m))
    assert rc == 0
    return m


def oracle_render(scene, cfg: dict, matrices: N.FrameMatrices | None = None, eye=None) -> dict:
    """Runs the oracle on a loaded fr_scene handle; returns numpy buffers.
    matrices / eye: another camera's frame matrices and position (default: the scene's)."""
    view = N.SceneView()
    assert N.lib().fr_scene_get_view(scene, C.byref(view)) == 0
    if eye is not None:
        view.info.eye[:] = [float(v) for v in eye]
    oc = OracleConfig(**cfg)
    mats = matrices if matrices is not None else oracle_matrices(view, cfg["shadow_size"])
    W, H, SW, SH = mats.width, mats.height, mats.shadow_width, mats.shadow_height
    info = view.info
    k = info.ssaa_kernel if info.ssaa_on else 1
    bufs = {
        "depth": np.zeros(W * H, np.float32),
        "shadow": np.zeros(SW * SH, np.float32),
        "frame": np.zeros(W * H * 3, np.float32),
        "frame8": np.zeros(W * H * 3, np.uint8),
    }
    if info.deferred:
        for name in ("gb_normal", "gb_position", "gb_lightndc", "gb_albedo", "gb_emissive",
                     "gb_param"):
            bufs[name] = np.zeros(W * H * 3, np.float32)
        bufs["gb_type"] = np.zeros(W * H, np.float32)
        bufs["ao"] = np.zeros(W * H, np.float32)
    if info.ssaa_on:
        bufs["ssaa8"] = np.zeros((W // k) * (H // k) * 3, np.uint8)
    out = OracleOut()
    for name, arr in bufs.items():
        ptype = _BP if arr.dtype == np.uint8 else _FP
        setattr(out, name, arr.ctypes.data_as(ptype))
    rc = oracle_lib().fr_oracle_render(C.byref(view), C.byref(oc), C.byref(mats), C.byref(out))
    assert rc == 0
    res = {}
    for name, arr in bufs.items():
        if name == "shadow" and not info.shadow_on:
            continue
        if arr.size == W * H * 3:
            res[name] = arr.reshape(H, W, 3)
        elif arr.size == W * H:
            res[name] = arr.reshape(H, W)
        elif name == "shadow":
            res[name] = arr.reshape(SH, SW)
        elif name == "ssaa8":
            res[name] = arr.reshape(H // k, W // k, 3)
    res["seconds"] = out.seconds
    return res


# ---- reference harness ---------------------------------------------------------------

def reference_available() -> bool:
    return os.path.exists(os.path.join(REF_DIR, "ref_pcss_tab"))


def run_reference(scene_path: str, outdir: str, variant: str = "ref_pcss_tab",
                  shadow_size: int = 0, pcf: int = 64, blocker: int = 32, tga: bool = False,
                  wrap: int = 0, filt: int = 0) -> dict:
    """Runs oracle/_ref/<variant> (the reference renderer's own code) and loads its dumps;
    tga: also its Output module's TGA files (res["tga"]: file name -> bytes)."""
    os.makedirs(outdir, exist_ok=True)
    exe = os.path.join(REF_DIR, variant)
    subprocess.run([exe, os.path.abspath(scene_path), os.path.abspath(outdir),
                    "--shadow-size", str(shadow_size), "--pcf", str(pcf),
                    "--blocker", str(blocker), "--tga", str(int(tga)), "--wrap", str(wrap),
                    "--filter", str(filt)], check=True,
                   capture_output=True)
    info = {}
    mats = {}
    with open(os.path.join(outdir, "info.txt")) as f:
        for line in f:
            parts = line.split()
            if len(parts) == 2:
                info[parts[0]] = float(parts[1]) if "." in parts[1] else int(parts[1])
            else:
                mats[parts[0]] = np.array([float.fromhex(x) for x in parts[1:]],
                                          np.float32).reshape(4, 4)
    W, H = info["width"], info["height"]
    res = {"info": info, "matrices": mats}

    def load(name, dtype, shape):
        p = os.path.join(outdir, name)
        if os.path.exists(p):
            return np.fromfile(p, dtype).reshape(shape)
        return None

    res["depth"] = load("depth.f32", np.float32, (H, W))
    if info.get("shadow"):
        res["shadow"] = load("shadow.f32", np.float32, (info["shadow_height"], info["shadow_width"]))
    res["frame"] = load("frame.f32", np.float32, (H, W, 3))
    res["frame8"] = load("frame8.u8", np.uint8, (H, W, 3))
    ssaa = os.path.join(outdir, "ssaa.u8")
    if os.path.exists(ssaa):
        raw = np.fromfile(ssaa, np.uint8)
        res["ssaa8"] = raw
    for name, key in (("gb_normal.f32", "gb_normal"), ("gb_pos.f32", "gb_position"),
                      ("gb_lndc.f32", "gb_lightndc"), ("gb_albedo.f32", "gb_albedo"),
                      ("gb_emissive.f32", "gb_emissive"), ("gb_param.f32", "gb_param")):
        v = load(name, np.float32, (H, W, 3))
        if v is not None:
            res[key] = v
    for name, key in (("gb_type.f32", "gb_type"), ("gb_ao.f32", "ao")):
        v = load(name, np.float32, (H, W))
        if v is not None:
            res[key] = v
    if tga:
        d = os.path.join(outdir, "output")
        res["tga"] = {}
        for fn in sorted(os.listdir(d)):
            with open(os.path.join(d, fn), "rb") as f:
                res["tga"][fn] = f.read()
    return res


def oracle_render_lights(scene, cfg: dict, view: N.FrameMatrices, eye, lights) -> dict:
    """One batched view (fr_batch.h) on the oracle: camera `view` from `eye`, lit by
    `lights` (a list of N.LightDesc). Returns depth, ao, frame8 (H, W[, 3]) and
    the lights' shadow maps."""
    L = oracle_lib()
    if not getattr(L, "_lights_sig", False):
        L.fr_oracle_render_lights.restype = C.c_int
        L.fr_oracle_render_lights.argtypes = [C.POINTER(N.SceneView), C.POINTER(OracleConfig),
                                              C.POINTER(N.FrameMatrices), C.POINTER(C.c_float),
                                              C.POINTER(N.LightDesc), C.c_int32, C.POINTER(OracleOut),
                                              C.POINTER(_FP)]
        L._lights_sig = True
    v = N.SceneView()
    assert N.lib().fr_scene_get_view(scene, C.byref(v)) == 0
    W, H = view.width, view.height
    out = {"depth": np.zeros((H, W), np.float32), "ao": np.zeros((H, W), np.float32),
           "frame8": np.zeros((H, W, 3), np.uint8)}
    o = OracleOut()
    o.depth = out["depth"].ctypes.data_as(_FP)
    o.ao = out["ao"].ctypes.data_as(_FP)
    o.frame8 = out["frame8"].ctypes.data_as(_BP)
    shadows = [np.zeros((l.shadow_size, l.shadow_size), np.float32) for l in lights]
    sp = (_FP * len(lights))(*[s.ctypes.data_as(_FP) for s in shadows])
    arr = (N.LightDesc * len(lights))(*lights)
    e = (C.c_float * 3)(*[float(x) for x in eye])
    rc = L.fr_oracle_render_lights(C.byref(v), C.byref(OracleConfig(**cfg)), C.byref(view), e, arr, len(lights),
                                   C.byref(o), sp)
    assert rc == 0
    out["shadows"] = shadows
    return out
