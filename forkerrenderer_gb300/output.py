"""The frame's TGA files (include/fr_output.h), encoded on the GPU.

Mirrors the reference's Output module (src/output.cpp:12-86): each
``Output*`` function writes the same file, with the same bytes, as the
reference's function of that name, into ``directory`` (the reference always
writes into ``output/``). Functions of images the reference skips for this
frame (SSAA off, no shadow, forward rendering) write nothing and return None.
"""

from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import _native as N

(FR_OUT_FRAMEBUFFER, FR_OUT_SSAA, FR_OUT_SHADOWMAP, FR_OUT_ZBUFFER, FR_OUT_GB_NORMAL, FR_OUT_GB_WORLDPOS,
 FR_OUT_GB_ALBEDO, FR_OUT_GB_PARAM, FR_OUT_GB_SHADING_TYPE, FR_OUT_GB_AO, FR_OUT_COUNT) = range(11)


def file_name(image: int) -> str:
    name = N.lib().fr_output_name(image)
    if name is None:
        raise ValueError(f"unknown output image {image}")
    return name.decode()


def encode(renderer, image: int, rle: bool = True) -> bytes | None:
    """The TGA file of one output image of the renderer's last frame, or None
    when the reference writes no such file."""
    h = renderer.handle
    size = N.lib().fr_output_encode(h, image, int(rle), None, 0)
    renderer._check(size)
    if size == 0:
        return None
    buf = np.empty(size, np.uint8)
    got = N.lib().fr_output_encode(h, image, int(rle), buf.ctypes.data_as(C.c_void_p), size)
    renderer._check(got)
    return buf.tobytes()


def max_bytes(renderer) -> int:
    """Upper bound of the bytes of every output file of the last frame."""
    total = 0
    for i in range(FR_OUT_COUNT):
        shape = image_shape(renderer, i)
        if shape is not None:
            total += N.lib().fr_tga_max_bytes(*shape)
    return total


def image_shape(renderer, image: int) -> tuple[int, int, int] | None:
    """(width, height, bytes per pixel) of an output image, None if the reference
    writes no such file for the last frame."""
    w, h, b = C.c_int32(0), C.c_int32(0), C.c_int32(0)
    rc = N.lib().fr_output_shape(renderer.handle, image, C.byref(w), C.byref(h), C.byref(b))
    renderer._check(rc)
    return (w.value, h.value, b.value) if rc == 1 else None


def encode_all_into(renderer, dst, rle: bool = True) -> tuple[list[int], float]:
    """Every output file of the last frame into `dst` (a writable buffer of at
    least max_bytes: numpy array, or a pinned torch tensor's data_ptr() as int),
    one after the other in FR_OUT_* order. Returns the file sizes (0 = absent)
    and the device milliseconds of the encoding kernels."""
    if isinstance(dst, int):
        ptr, cap = C.c_void_p(dst), max_bytes(renderer)
    else:
        ptr, cap = C.c_void_p(dst.ctypes.data), dst.nbytes
    sizes = (C.c_int64 * FR_OUT_COUNT)()
    ms = C.c_float(0)
    renderer._check(N.lib().fr_output_encode_all(renderer.handle, int(rle), ptr, cap, sizes, C.byref(ms)))
    return list(sizes), float(ms.value)


def encode_all(renderer, rle: bool = True) -> tuple[dict[str, bytes], float]:
    """Every output file of the last frame (name -> bytes) and the device
    milliseconds of the encoding kernels."""
    buf = np.empty(max(1, max_bytes(renderer)), np.uint8)
    sizes, ms = encode_all_into(renderer, buf, rle)
    files, at = {}, 0
    for i, n in enumerate(sizes):
        if n:
            files[file_name(i)] = buf[at:at + n].tobytes()
            at += n
    return files, ms


def write_all(renderer, directory: str = "output", rle: bool = True) -> list[str]:
    """Output::Output* in main.cpp's order (src/main.cpp:45-54): writes every
    file the reference would write; returns their paths."""
    os.makedirs(directory, exist_ok=True)
    n = N.lib().fr_output_write(renderer.handle, directory.encode(), int(rle))
    renderer._check(n)
    return [os.path.join(directory, file_name(i)) for i in range(FR_OUT_COUNT)
            if N.lib().fr_output_present(renderer.handle, i) == 1]


def _writer(image: int):
    def write(renderer, directory: str = "output") -> str | None:
        data = encode(renderer, image)
        if data is None:
            return None
        os.makedirs(directory, exist_ok=True)
        path = os.path.join(directory, file_name(image))
        with open(path, "wb") as f:
            f.write(data)
        return path

    return write


class Output:
    """The reference's Output namespace (src/output.h); each function takes the
    renderer whose last frame it writes."""

    OutputFrameBuffer = staticmethod(_writer(FR_OUT_FRAMEBUFFER))
    OutputSSAAImage = staticmethod(_writer(FR_OUT_SSAA))
    OutputShadowBuffer = staticmethod(_writer(FR_OUT_SHADOWMAP))
    OutputZBuffer = staticmethod(_writer(FR_OUT_ZBUFFER))
    OutputNormalGBuffer = staticmethod(_writer(FR_OUT_GB_NORMAL))
    OutputWorldPosGBuffer = staticmethod(_writer(FR_OUT_GB_WORLDPOS))
    OutputAlbedoGBuffer = staticmethod(_writer(FR_OUT_GB_ALBEDO))
    OutputParamGBuffer = staticmethod(_writer(FR_OUT_GB_PARAM))
    OutputShadingTypeGBuffer = staticmethod(_writer(FR_OUT_GB_SHADING_TYPE))
    OutputAmbientOcclusionGBuffer = staticmethod(_writer(FR_OUT_GB_AO))


def tga_encode_device(pixels, rle: bool = True, vflip: bool = True, stream=None) -> bytes:
    """Encodes a CUDA uint8 tensor (H, W) or (H, W, bytespp) in TGA byte order
    with the GPU encoder; returns the file's bytes."""
    import torch

    px = pixels.contiguous()
    if px.dtype != torch.uint8 or not px.is_cuda:
        raise ValueError("pixels must be a CUDA uint8 tensor")
    h, w = int(px.shape[0]), int(px.shape[1])
    bpp = 1 if px.dim() == 2 else int(px.shape[2])
    L = N.lib()
    out = torch.empty(L.fr_tga_max_bytes(w, h, bpp), dtype=torch.uint8, device=px.device)
    scratch = torch.empty(max(1, L.fr_tga_scratch_bytes(w, h)), dtype=torch.uint8, device=px.device)
    size = torch.zeros(1, dtype=torch.int64, device=px.device)
    st = stream if stream is not None else torch.cuda.current_stream(px.device)
    rc = L.fr_tga_encode_device(px.data_ptr() if px.numel() else None, w, h, bpp, int(rle), int(vflip),
                                out.data_ptr(), size.data_ptr(), scratch.data_ptr(), st.cuda_stream)
    if rc != 0:
        raise RuntimeError(f"fr_tga_encode_device failed ({rc})")
    st.synchronize()
    return out[:int(size.item())].cpu().numpy().tobytes()
