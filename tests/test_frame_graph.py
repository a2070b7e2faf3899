"""The frame graph (fr_config.frame_graph) replays exactly the frame the direct launches produce."""

import numpy as np
import pytest

from conftest import gpu_available

pytestmark = pytest.mark.gpu


def _frames(r, n):
    out = []
    for _ in range(n):
        r.Render()
        t = r.timings()
        assert t["total"] > 0
        out.append((r.frame8().copy(), r.ambient_occlusion().copy(), r.depth().copy(), r.launch_count()))
    return out


@pytest.mark.parametrize("learned", [False, True])
def test_frame_graph_matches_direct_launches(learned):
    if not gpu_available():
        pytest.skip("no CUDA GPU")
    import forkerrenderer_gb300 as fr
    from forkerrenderer_gb300 import _native as N
    from forkerrenderer_gb300.aonet import AONet
    from scenes import render_config, scene_path

    scene = fr.Scene(scene_path("def_ao_128"))
    cfg = render_config("def_ao_128")
    if learned:
        cfg.update(ao_mode=N.FR_AO_LEARNED, ao_probe_threshold=1e9)
    net = AONet(0, seed=6) if learned else None
    results = []
    for graph in (0, 1):
        r = fr.Renderer(**cfg, frame_graph=graph)
        r.Preconfigure(scene)
        if net is not None:
            r.set_ao_net(net)
        results.append(_frames(r, 4))  # direct, capture, replay, replay
        r.close()
    ref = results[0][0]
    for frame in results[0] + results[1]:
        for a, b in zip(frame[:3], ref[:3]):
            assert np.array_equal(a, b)
        assert frame[3] == ref[3]
