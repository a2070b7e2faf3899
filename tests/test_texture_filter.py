"""Bilinear texture filtering (Texture::colorFromFiltering, texture.h:85-127)
against the reference.

The reference rendered def_wrap (ground texture coordinates from -1.3 to 2.45)
with ForkerGL::TextureFilterMode(Linear) and each wrap mode, and fwd_wrap (the
same scene forward-shaded) with Repeat (tests/golden/filter_linear.*). The
texture-sampled G-buffers (albedo, PBR parameters, normal-mapped normals) and the
depth must match bit for bit; the 8-bit frames within the 1-LSB shading bar
(powf). On the GPU, deferred frames keep the texture coordinate in the G-buffer
and sample the maps where it is decoded (lighting, read-back, TGA output)."""

import json
import os

import numpy as np
import pytest

import golden_utils as G
import oracle_bridge as OB
import scenes
from conftest import gpu_available
from forkerrenderer_gb300 import Renderer, RenderError, Scene


def _golden():
    with open(os.path.join(G.GOLDEN, "filter_linear.json")) as f:
        meta = json.load(f)
    return meta, dict(np.load(os.path.join(G.GOLDEN, "filter_linear.npz")))


def _oracle(name, mode):
    scene = Scene(scenes.scene_path(name))
    return OB.oracle_render(scene.handle, OB.reference_config(**scenes.render_config(name), threads=4,
                                                                texture_wrap=mode, texture_filter=1))


@pytest.mark.parametrize("mode", [0, 1, 2, 3])
def test_oracle_linear_filter_matches_reference(mode):
    meta, frames = _golden()
    assert scenes.files_digest("def_wrap") == meta["scene_digest"]["def_wrap"], "scene generator drifted"
    out = _oracle("def_wrap", mode)
    for k, want in meta["modes"][str(mode)].items():
        assert G.sha(out[k]) == want, f"wrap {mode}: {k}"
    if mode == 1:
        G.check_frame8(out["frame8"], frames["def_wrap_frame8"])


def test_oracle_linear_filter_forward_matches_reference():
    meta, frames = _golden()
    assert scenes.files_digest("fwd_wrap") == meta["scene_digest"]["fwd_wrap"], "scene generator drifted"
    G.check_frame8(_oracle("fwd_wrap", 1)["frame8"], frames["fwd_wrap_frame8"])


def _gpu(name, mode, **extra):
    meta, frames = _golden()
    if scenes.files_digest(name) != meta["scene_digest"][name]:
        pytest.skip("scene generator output differs on this machine")
    scene = Scene(scenes.scene_path(name))
    r = Renderer(**scenes.render_config(name), texture_wrap=mode, texture_filter=1, **extra)
    r.Preconfigure(scene)
    r.Render()
    return meta, frames, scene, r


@pytest.mark.gpu
@pytest.mark.parametrize("mode", [0, 1, 2, 3])
def test_gpu_linear_filter_matches_reference(mode):
    if not gpu_available():
        pytest.skip("no CUDA GPU")
    meta, frames, _, r = _gpu("def_wrap", mode)
    got = {"gb_albedo": r.gbuffer("albedo"), "gb_param": r.gbuffer("param"), "gb_normal": r.gbuffer("normal"),
           "depth": r.depth()}
    for k, want in meta["modes"][str(mode)].items():
        assert G.sha(got[k]) == want, f"wrap {mode}: {k}"
    if mode == 1:
        G.check_frame8(r.frame8(), frames["def_wrap_frame8"])
    r.close()


@pytest.mark.gpu
def test_gpu_linear_filter_forward_matches_reference():
    if not gpu_available():
        pytest.skip("no CUDA GPU")
    _, frames, _, r = _gpu("fwd_wrap", 1)
    G.check_frame8(r.frame8(), frames["fwd_wrap_frame8"])
    r.close()


@pytest.mark.gpu
@pytest.mark.parametrize("concurrent", [0, 1])
def test_gpu_linear_filter_matches_oracle_everywhere(concurrent):
    """Every buffer against the oracle with the same filter (bit-exact where the
    arithmetic is IEEE-exact), and the G-buffer TGA files decoded from the
    coordinate-carrying G-buffer equal the oracle's encoding of the read-back."""
    if not gpu_available():
        pytest.skip("no CUDA GPU")
    import tga_util as T
    from forkerrenderer_gb300 import output

    _, _, scene, r = _gpu("def_wrap", 2, concurrent_passes=concurrent)
    want = _oracle("def_wrap", 2)
    for key, g in (("gb_albedo", "albedo"), ("gb_param", "param"), ("gb_normal", "normal"),
                   ("gb_emissive", "emissive"), ("gb_position", "position"), ("gb_type", "type")):
        assert np.array_equal(r.gbuffer(g), want[key]), key
    assert np.array_equal(r.depth(), want["depth"])
    assert np.array_equal(r.shadow_map(), want["shadow"])
    G.check_frame8(r.frame8(), want["frame8"])
    files, _ = output.encode_all(r)
    bufs = {"gb_albedo": r.gbuffer("albedo"), "gb_param": r.gbuffer("param"), "gb_type": r.gbuffer("type")}
    for fn, key, kind in T.OUTPUTS:
        if key in bufs:
            assert files[fn] == OB.oracle_tga(T.reference_image(key, kind, bufs)), fn
    r.close()


@pytest.mark.gpu
def test_unknown_filter_mode_is_refused():
    if not gpu_available():
        pytest.skip("no CUDA GPU")
    with pytest.raises(RenderError):
        Renderer(**scenes.render_config("def_wrap"), texture_filter=2)
