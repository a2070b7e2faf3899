"""The CPU oracle against the reference's own outputs (golden fixtures).

Pins the oracle: on every seeded case, the oracle restatement must reproduce
the reference renderer bit for bit (depth, shadow map, G-buffers, float frame,
AO, 8-bit frame, SSAA image), given the same scene files and matrices."""

import numpy as np
import pytest

import golden_utils as G
import oracle_bridge as OB
import scenes
from forkerrenderer_gb300 import Scene

KEYMAP = {"gb_normal": "gb_normal", "gb_position": "gb_position", "gb_lightndc": "gb_lightndc",
          "gb_albedo": "gb_albedo", "gb_emissive": "gb_emissive", "gb_param": "gb_param",
          "gb_type": "gb_type", "depth": "depth", "shadow": "shadow", "frame": "frame"}


@pytest.mark.parametrize("name", sorted(scenes.CASES))
def test_scene_files_reproducible(name):
    meta, _ = G.load(name)
    assert scenes.files_digest(name) == meta["scene_digest"], "scene generator drifted"


@pytest.mark.parametrize("name", sorted(scenes.CASES))
def test_oracle_matches_reference(name):
    meta, arrays = G.load(name)
    scene = Scene(scenes.scene_path(name))
    cfg = OB.reference_config(**scenes.render_config(name), threads=4)
    out = OB.oracle_render(scene.handle, cfg)
    for k, want in meta["sha256"].items():
        got = out[KEYMAP[k]]
        assert G.sha(got) == want, f"{name}: {k} differs from the reference"
    np.testing.assert_array_equal(out["frame8"].reshape(-1), arrays["frame8"].reshape(-1))
    if "ao" in arrays:
        np.testing.assert_array_equal(out["ao"].reshape(-1), arrays["ao"].reshape(-1))
    if "ssaa8" in arrays:
        np.testing.assert_array_equal(out["ssaa8"].reshape(-1), arrays["ssaa8"].reshape(-1))


@pytest.mark.parametrize("name", sorted(scenes.CASES))
def test_host_matrices_match_reference(name):
    """The product's host-side matrix code (fr_scene_frame_matrices) reproduces
    the reference's VP, light-space and viewport matrices bit for bit."""
    meta, _ = G.load(name)
    scene = Scene(scenes.scene_path(name))
    cfg = scenes.render_config(name)
    m = scene.frame_matrices(cfg["shadow_size"])
    ref = G.matrices(meta, cfg["shadow_size"])
    assert np.array_equal(np.array(m.view_projection, np.float32).view(np.uint32),
                          np.array(ref.view_projection, np.float32).view(np.uint32))
    if scene.info.shadow_on:  # with shadow off the reference never sets it (it stays identity, unused)
        assert np.array_equal(np.array(m.light_space, np.float32).view(np.uint32),
                              np.array(ref.light_space, np.float32).view(np.uint32))
    assert (m.width, m.height) == (ref.width, ref.height)
