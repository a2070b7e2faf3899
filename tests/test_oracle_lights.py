"""The oracle's restatement of the batched renderer's lighting
(fr_oracle_render_lights) is tied to the reference-pinned single frame: with one
point light at the scene's light it must reproduce fr_oracle_render bit for bit
(the batch is specified to equal fr_render_frame there), so the multi-light path
inherits the reference pin for everything but the sum over lights and the
directional light's projection."""

import numpy as np
import pytest

import oracle_bridge as OB
import scenes
from forkerrenderer_gb300 import Scene
from forkerrenderer_gb300.batch import point_light


@pytest.mark.parametrize("name,mode", [("def_pcss", 2), ("def_pcf_ssaa", 1), ("def_phong_hard", 0)])
def test_one_point_light_is_the_reference_frame(name, mode):
    """PCSS, PCF and hard shadows; PBR and Blinn-Phong materials; square
    shadow maps (a batch light's map is S x S)."""
    scene = Scene(scenes.scene_path(name))
    cfg = OB.reference_config(**scenes.render_config(name, shadow_mode=mode, shadow_size=256), threads=4)
    m = scene.frame_matrices(cfg["shadow_size"])
    info = scene.info
    one = OB.oracle_render_lights(scene.handle, cfg, m, list(info.eye),
                                  [point_light(list(info.light_pos), list(info.light_color), 256)])
    ref = OB.oracle_render(scene.handle, cfg)
    for k in ("depth", "ao", "frame8"):
        assert np.array_equal(one[k].reshape(-1).view(np.uint8), ref[k].reshape(-1).view(np.uint8)), k
    assert np.array_equal(one["shadows"][0], ref["shadow"])
