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


@pytest.mark.parametrize("name,learned", [("def_pcf_ssaa", False), ("def_ao_128", False), ("def_ao_128", True)])
def test_concurrent_passes_match_sequential(name, learned):
    """Deferred frames with the shadow pass beside the camera chain (two streams)
    give every buffer of the sequential frame, bit for bit, directly and replayed
    from the frame graph; the pass timings stay consistent."""
    if not gpu_available():
        pytest.skip("no CUDA GPU")
    import forkerrenderer_gb300 as fr
    from forkerrenderer_gb300 import _native as N
    from forkerrenderer_gb300.aonet import AONet
    from scenes import render_config, scene_path

    scene = fr.Scene(scene_path(name))
    cfg = render_config(name)
    if learned:
        cfg.update(ao_mode=N.FR_AO_LEARNED, ao_probe_threshold=1e9)
    net = AONet(0, seed=6) if learned else None
    outs = []
    for concurrent, graph in ((0, 0), (1, 0), (1, 1)):
        r = fr.Renderer(**cfg, frame_graph=graph, concurrent_passes=concurrent)
        r.Preconfigure(scene)
        if net is not None:
            r.set_ao_net(net)
        for _ in range(3):  # direct, capture, replay
            r.Render()
            t = r.timings()
            assert t["total"] > 0 and t["shadow"] <= t["total"] + 1e-6 and t["lighting"] >= 0
            bufs = [r.frame8(), r.ambient_occlusion(), r.depth(), r.shadow_map()]
            bufs += [r.gbuffer(g) for g in ("normal", "position", "albedo", "param", "type")]
            if scene.info.ssaa_on:
                bufs.append(r.ssaa8())
            outs.append([b.copy() for b in bufs] + [r.launch_count()])
        r.close()
    ref = outs[0]
    for o in outs[1:]:
        assert len(o) == len(ref)
        for a, b in zip(o[:-1], ref[:-1]):
            assert np.array_equal(a, b)
        assert o[-1] == ref[-1]


@pytest.mark.parametrize("learned", [False, True])
def test_graph_replayed_for_a_moving_camera_matches_direct_frames(learned):
    """A camera that changes every frame keeps the frame graph: its key leaves the
    camera out, and the kernel nodes that take the frame constants get the new
    camera's before each replay. Every frame equals the direct launches' frame of
    the same camera, bit for bit, and after the first two frames every frame is a
    replay (the launch count of a replay is the captured frame's)."""
    if not gpu_available():
        pytest.skip("no CUDA GPU")
    import math

    import forkerrenderer_gb300 as fr
    from forkerrenderer_gb300 import _native as N
    from forkerrenderer_gb300.aonet import AONet
    from scenes import render_config, scene_path

    scene = fr.Scene(scene_path("def_ao_128"))
    cfg = render_config("def_ao_128")
    if learned:
        cfg.update(ao_mode=N.FR_AO_LEARNED, ao_probe_threshold=1e9)
    net = AONet(0, seed=6) if learned else None
    cams = []
    for i in range(6):
        a = 0.3 * i
        eye = (6.0 * math.sin(a), 4.0 + 0.2 * i, 6.0 * math.cos(a))
        cams.append((scene.view_matrices(eye, (0, 0, 0), cfg["shadow_size"]), eye))
    out = {}
    for graph in (0, 1):
        r = fr.Renderer(**cfg, frame_graph=graph)
        r.Preconfigure(scene)
        if net is not None:
            r.set_ao_net(net)
        frames = []
        for m, eye in cams:
            r.set_matrices(m, eye)
            r.Render()
            frames.append((r.frame8().copy(), r.ambient_occlusion().copy(), r.depth().copy()))
        out[graph] = frames
        r.close()
    for i, (a, b) in enumerate(zip(out[0], out[1])):
        for x, y in zip(a, b):
            assert np.array_equal(x, y), i
    assert not np.array_equal(out[0][0][0], out[0][5][0])  # the camera did move
    if net is not None:
        net.close()


def test_frame_without_pass_events_is_the_same_frame():
    """pass_timings = 0 records only the frame's first and last events: direct and
    graph-replayed frames are bit-identical to an instrumented context's, and
    fr_last_timings gives the frame's total with 0 for each pass."""
    if not gpu_available():
        pytest.skip("no CUDA GPU")
    import forkerrenderer_gb300 as fr
    from scenes import render_config, scene_path

    scene = fr.Scene(scene_path("def_ao_128"))
    cfg = render_config("def_ao_128")
    out = {}
    for timings in (1, 0):
        r = fr.Renderer(**cfg, frame_graph=1, pass_timings=timings)
        r.Preconfigure(scene)
        frames = []
        for _ in range(4):  # direct, then captured and replayed
            r.Render()
            t = r.timings()
            assert t["total"] > 0
            if not timings:
                assert all(v == 0 for k, v in t.items() if k != "total")
            frames.append((r.frame8().copy(), r.ambient_occlusion().copy(), r.depth().copy()))
        out[timings] = frames
        r.close()
    for a, b in zip(out[1], out[0]):
        for x, y in zip(a, b):
            assert np.array_equal(x, y)
