"""Texture wrap modes (Texture::wrapCoord, texture.h:62-83) against the reference.

def_wrap's ground carries texture coordinates from -1.3 to 2.45. The reference
rendered it with each wrap mode (tests/golden/wrap_modes.json, its textures
created after ForkerGL::TextureWrapMode); the oracle (CPU) and the GB300 path must
reproduce the texture-sampled G-buffers and the depth bit for bit."""

import json
import os

import numpy as np
import pytest

import golden_utils as G
import oracle_bridge as OB
import scenes
from conftest import gpu_available
from forkerrenderer_gb300 import Renderer, Scene

NAME = "def_wrap"


def _golden():
    with open(os.path.join(G.GOLDEN, "wrap_modes.json")) as f:
        return json.load(f)


@pytest.mark.parametrize("mode", [0, 1, 2, 3])
def test_oracle_wrap_modes_match_reference(mode):
    meta = _golden()
    assert scenes.files_digest(NAME) == meta["scene_digest"], "scene generator drifted"
    scene = Scene(scenes.scene_path(NAME))
    out = OB.oracle_render(scene.handle, OB.reference_config(**scenes.render_config(NAME), threads=4,
                                                               texture_wrap=mode))
    for k, want in meta["modes"][str(mode)].items():
        assert G.sha(out[k]) == want, f"wrap {mode}: {k}"


@pytest.mark.gpu
@pytest.mark.parametrize("mode", [0, 1, 2, 3])
def test_gpu_wrap_modes_match_reference(mode):
    if not gpu_available():
        pytest.skip("no CUDA GPU")
    meta = _golden()
    if scenes.files_digest(NAME) != meta["scene_digest"]:
        pytest.skip("scene generator output differs on this machine")
    scene = Scene(scenes.scene_path(NAME))
    r = Renderer(**scenes.render_config(NAME), texture_wrap=mode)
    r.Preconfigure(scene)
    r.Render()
    got = {"gb_albedo": r.gbuffer("albedo"), "gb_param": r.gbuffer("param"), "gb_normal": r.gbuffer("normal"),
           "depth": r.depth()}
    for k, want in meta["modes"][str(mode)].items():
        assert G.sha(got[k]) == want, f"wrap {mode}: {k}"
    r.close()
