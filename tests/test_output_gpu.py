"""The GPU TGA encoder (include/fr_output.h) against the reference's writer and
the oracle, through the C ABI.

Bar: byte-identical files. Crafted images: the reference writer's own bytes
(golden fixtures). Rendered frames: the reference's file digests where the
frame's buffers are bit-exact (depth, shadow map, G-buffers), and the oracle's
encoding of the GPU's own buffers for every file (frame and AO differ from the
reference by the 1-LSB powf tolerance of the parity tests)."""

import hashlib
import os
import tempfile

import numpy as np
import pytest

import golden_utils as G
import oracle_bridge as OB
import scenes
import tga_util as T
from conftest import gpu_available
from forkerrenderer_gb300 import Renderer, Scene

pytestmark = pytest.mark.gpu


def _torch():
    if not gpu_available():
        pytest.skip("no CUDA GPU")
    import torch

    return torch


def _gpu_tga(img, rle=True, vflip=True):
    torch = _torch()
    from forkerrenderer_gb300.output import tga_encode_device

    return tga_encode_device(torch.from_numpy(np.ascontiguousarray(img)).cuda(), rle, vflip)


def test_edge_images_match_reference_writer():
    z = np.load(os.path.join(G.GOLDEN, "tga_edge.npz"))
    n = sum(1 for k in z.files if k.startswith("img"))
    for i in range(n):
        img = z[f"img{i}"]
        for rle in (0, 1):
            assert _gpu_tga(img, bool(rle)) == z[f"tga{i}_rle{rle}"].tobytes(), (i, rle, img.shape)


def _runs_image(rng, h, w, bpp, lengths, values=3):
    n = h * w
    out = np.empty((n, bpp), np.uint8)
    i = 0
    while i < n:
        ln = int(lengths(rng))
        out[i:i + ln] = rng.integers(0, values, bpp)
        i += ln
    return out.reshape(h, w, bpp) if bpp > 1 else out.reshape(h, w)


@pytest.mark.parametrize("bpp", [1, 3, 4])
def test_random_images_match_oracle_across_segments(bpp):
    """Images of several 4096-pixel segments: runs and raw stretches of every
    length class around the 128-pixel packet limit, so packets cross segment
    boundaries at every offset."""
    rng = np.random.default_rng(100 + bpp)
    classes = [1, 1, 1, 2, 3, 126, 127, 128, 129, 130, 255, 256, 257, 4095, 4097]
    shapes = [(1, 4095), (1, 4096), (1, 4097), (3, 4096), (37, 1001), (64, 640), (5, 20000)]
    for h, w in shapes:
        for mode in range(4):
            if mode == 0:
                img = _runs_image(rng, h, w, bpp, lambda r: r.choice(classes))
            elif mode == 1:
                img = _runs_image(rng, h, w, bpp, lambda r: 1, values=256)  # raw stretches only
                img.reshape(-1)[: 5 * bpp] = 7  # a run of 5 first: raw packets then start at 5 + 128 k
            elif mode == 2:
                img = _runs_image(rng, h, w, bpp, lambda r: r.integers(1, 4), values=2)  # many short runs
            else:
                img = _runs_image(rng, h, w, bpp, lambda r: r.integers(1, 600))
            for rle in (True, False):
                assert _gpu_tga(img, rle) == OB.oracle_tga(img, rle), (h, w, bpp, mode, rle)


def test_large_images_round_trip_and_match_oracle():
    rng = np.random.default_rng(7)
    # a 2048 x 2048 gray image: constant background, noise blocks and stripes
    img = np.zeros((2048, 2048), np.uint8)
    img[100:900, 300:1900] = rng.integers(0, 256, (800, 1600))
    img[1200:1300] = (np.arange(2048) // 131 % 7).astype(np.uint8)
    data = _gpu_tga(img)
    assert data == OB.oracle_tga(img)
    px, hdr = T.decode(data)
    assert (hdr["width"], hdr["height"], hdr["type"]) == (2048, 2048, 11)
    assert np.array_equal(px, img)
    # top-left origin flag
    assert _gpu_tga(img[:8], vflip=False)[17] == 0x20


def _render(name):
    cfg = scenes.render_config(name)
    scene = Scene(scenes.scene_path(name))
    r = Renderer(**cfg)
    r.Preconfigure(scene)
    r.Render()
    return scene, r


def _gpu_buffers(scene, r):
    out = {"depth": r.depth(), "frame8": r.frame8()}
    if scene.info.shadow_on:
        out["shadow"] = r.shadow_map()
    if scene.info.deferred:
        for g, key in (("normal", "gb_normal"), ("position", "gb_position"), ("albedo", "gb_albedo"),
                       ("param", "gb_param"), ("type", "gb_type")):
            out[key] = r.gbuffer(g)
        out["ao"] = r.ambient_occlusion()
    if scene.info.ssaa_on:
        out["ssaa8"] = r.ssaa8()
    return out


BITEXACT_FILES = {"shadowmap.tga", "zbuffer.tga", "gbuffer_normal.tga", "gbuffer_worldpos.tga",
                  "gbuffer_albedo.tga", "gbuffer_param.tga", "gbuffer_shading_type.tga"}


@pytest.mark.parametrize("name", sorted(scenes.CASES))
def test_output_files_match_reference_and_oracle(name):
    _torch()
    from forkerrenderer_gb300 import output

    meta, _ = G.load(name)
    assert scenes.files_digest(name) == meta["scene_digest"], "scene generator output differs on this machine"
    scene, r = _render(name)
    bufs = _gpu_buffers(scene, r)
    files, ms = output.encode_all(r)
    assert ms > 0
    assert sorted(files) == sorted(meta["tga"]), "set of files differs from the reference's"
    for fn, key, kind in T.OUTPUTS:
        if fn not in files:
            assert r.encode_tga([f for f, _, _ in T.OUTPUTS].index(fn)) is None
            continue
        data = files[fn]
        assert data == OB.oracle_tga(T.reference_image(key, kind, bufs)), (name, fn)
        assert data == r.encode_tga([f for f, _, _ in T.OUTPUTS].index(fn)), (name, fn)
        if fn in BITEXACT_FILES:
            assert hashlib.sha256(data).hexdigest() == meta["tga"][fn]["sha256"], (name, fn)
    with tempfile.TemporaryDirectory() as d:
        paths = r.write_outputs(d)
        assert sorted(os.path.basename(p) for p in paths) == sorted(files)
        for p in paths:
            with open(p, "rb") as f:
                assert f.read() == files[os.path.basename(p)]
    r.close()


def test_full_size_frame_outputs():
    """The 1280 x 800 deferred PBR + PCSS + SSAO frame of 409,602 triangles with
    its 2048^2 shadow map: every file equals the oracle's encoding of the GPU's
    buffers and decodes to them."""
    _torch()
    from forkerrenderer_gb300 import output
    from forkerrenderer_gb300.train_ao import FIELD_RENDER, field_scene_path

    scene = Scene(field_scene_path(0))
    r = Renderer(**FIELD_RENDER)
    r.Preconfigure(scene)
    r.Render()
    bufs = _gpu_buffers(scene, r)
    files, _ = output.encode_all(r)
    assert len(files) == 9  # no SSAA image at 1x
    for fn, key, kind in T.OUTPUTS:
        if fn not in files:
            continue
        want_px = T.reference_image(key, kind, bufs)
        px, hdr = T.decode(files[fn])
        assert np.array_equal(px, want_px), fn
        assert files[fn] == OB.oracle_tga(want_px), fn
    raw, _ = output.encode_all(r, rle=False)
    assert T.decode(raw["framebuffer.tga"])[1]["type"] == 2
    r.close()
