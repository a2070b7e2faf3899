"""The TGA output oracle against the reference's own writer (golden fixtures).

Pins oracle/fr_oracle_tga.cpp: on crafted images the encoder must reproduce the
bytes of the reference's TGAImage::WriteTgaFile, and on every seeded case the
oracle's frame, run through the reference's image conversions and writer, must
reproduce the SHA-256 of each TGA file the reference's Output module wrote."""

import hashlib
import os

import numpy as np
import pytest

import golden_utils as G
import oracle_bridge as OB
import scenes
import tga_util as T
from forkerrenderer_gb300 import Scene


def _edge():
    z = np.load(os.path.join(G.GOLDEN, "tga_edge.npz"))
    n = sum(1 for k in z.files if k.startswith("img"))
    return z, n


def test_oracle_encoder_matches_reference_writer_on_edge_images():
    z, n = _edge()
    assert n >= 20
    for i in range(n):
        img = z[f"img{i}"]
        for rle in (0, 1):
            want = z[f"tga{i}_rle{rle}"].tobytes()
            assert OB.oracle_tga(img, bool(rle)) == want, (i, rle, img.shape)


def test_edge_images_round_trip_through_the_decoder():
    z, n = _edge()
    for i in range(n):
        img = z[f"img{i}"]
        for rle in (0, 1):
            px, hdr = T.decode(z[f"tga{i}_rle{rle}"].tobytes())
            assert hdr["type"] == ((11 if rle else 3) if img.ndim == 2 else (10 if rle else 2))
            assert hdr["descriptor"] == 0  # vFlip = true: bottom-left origin, rows as stored
            assert np.array_equal(px.reshape(-1), img.reshape(-1))


def test_top_left_descriptor_and_packet_limit():
    img = np.full((3, 300), 9, np.uint8)
    data = OB.oracle_tga(img, True, vflip=False)
    assert data[17] == 0x20
    # 900 equal gray pixels: runs of 128 (header 255) and a final run of 4 (header 131)
    body = data[18:-26]
    assert list(body) == [255, 9] * 7 + [131, 9]


def test_float_to_byte_conversion_follows_the_x86_build():
    u8 = OB.oracle_lib().fr_oracle_u8
    cases = {0.0: 0, 1.9: 1, 255.9: 255, 256.0: 0, 300.7: 44, -1.5: 255, -0.5: 0,
             float("inf"): 0, float("-inf"): 0, float("nan"): 0, 1e10: 0, 2147483520.0: 128}
    for v, want in cases.items():
        assert u8(v) == want, v


@pytest.mark.parametrize("name", sorted(scenes.CASES))
def test_oracle_outputs_match_reference_files(name):
    meta, arrays = G.load(name)
    scene = Scene(scenes.scene_path(name))
    out = OB.oracle_render(scene.handle, OB.reference_config(**scenes.render_config(name), threads=4))
    # frame8 / AO / SSAA from the reference itself (powf differs between C libraries)
    bufs = dict(out)
    bufs["frame8"] = arrays["frame8"].reshape(out["frame8"].shape)
    if "ao" in arrays:
        bufs["ao"] = arrays["ao"].reshape(out["ao"].shape)
    if "ssaa8" in arrays:
        bufs["ssaa8"] = arrays["ssaa8"].reshape(out["ssaa8"].shape)
    files = meta["tga"]
    assert "framebuffer.tga" in files and "zbuffer.tga" in files
    for fn, key, kind in T.OUTPUTS:
        if fn not in files:
            continue
        data = OB.oracle_tga(T.reference_image(key, kind, bufs))
        assert len(data) == files[fn]["bytes"], (name, fn)
        assert hashlib.sha256(data).hexdigest() == files[fn]["sha256"], (name, fn)
