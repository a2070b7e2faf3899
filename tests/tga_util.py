"""TGA helpers of the tests: a decoder of the files the reference's writer makes
(types 2/3/10/11, src/tgaimage.cpp:43-150 reads the same forms) and the
reference's Output file list (src/output.cpp:12-86, in main.cpp:45-54 order)."""

from __future__ import annotations

import numpy as np

import oracle_bridge as OB

# file name -> (reference buffer, conversion): "rgb" = 8-bit R, G, B image,
# "1f" = Buffer1f::GenerateImage, "3f" = Buffer3f::GenerateImage
OUTPUTS = [
    ("framebuffer.tga", "frame8", "rgb"),
    ("framebuffer_SSAA.tga", "ssaa8", "rgb"),
    ("shadowmap.tga", "shadow", "1f"),
    ("zbuffer.tga", "depth", "1f"),
    ("gbuffer_normal.tga", "gb_normal", "3f"),
    ("gbuffer_worldpos.tga", "gb_position", "3f"),
    ("gbuffer_albedo.tga", "gb_albedo", "3f"),
    ("gbuffer_param.tga", "gb_param", "3f"),
    ("gbuffer_shading_type.tga", "gb_type", "1f"),
    ("gbuffer_ambient_occlusion.tga", "ao", "1f"),
]

FOOTER = bytes(8) + b"TRUEVISION-XFILE.\0"


def decode(data: bytes) -> tuple[np.ndarray, dict]:
    """Pixels (H, W[, bpp]) in file order and the header fields of a TGA file."""
    b = np.frombuffer(data, np.uint8)
    kind, w, h, bits, desc = int(b[2]), int(b[12]) | int(b[13]) << 8, int(b[14]) | int(b[15]) << 8, int(b[16]), int(b[17])
    bpp = bits // 8
    n = w * h
    pos = 18
    if kind in (2, 3):
        px = b[pos:pos + n * bpp].copy()
        pos += n * bpp
    else:
        out = np.empty(n * bpp, np.uint8)
        i = 0
        while i < n:
            c = int(b[pos])
            pos += 1
            if c < 128:
                ln = c + 1
                out[i * bpp:(i + ln) * bpp] = b[pos:pos + ln * bpp]
                pos += ln * bpp
            else:
                ln = c - 127
                out[i * bpp:(i + ln) * bpp] = np.tile(b[pos:pos + bpp], ln)
                pos += bpp
            i += ln
        assert i == n, "packets overrun the image"
        px = out
    assert data[pos:] == FOOTER, "bad footer"
    shape = (h, w) if bpp == 1 else (h, w, bpp)
    return px.reshape(shape), {"type": kind, "width": w, "height": h, "bpp": bpp, "descriptor": desc}


def reference_image(key: str, kind: str, buffers: dict, ssaa_shape=None) -> np.ndarray:
    """The 8-bit image the reference's Output module encodes from a buffer."""
    v = buffers[key]
    if kind == "rgb":
        if ssaa_shape is not None:
            v = np.asarray(v).reshape(ssaa_shape[0], ssaa_shape[1], 3)
        return OB.rgb_to_tga_order(v)
    return OB.oracle_image(v)
