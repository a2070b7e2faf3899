"""Batched multi-view rendering (fr_batch.h) on the GPU: parity with the single
frame path, view independence, tuning independence, learned-AO views."""

import numpy as np
import pytest

from conftest import gpu_available

pytestmark = pytest.mark.gpu


def _setup(**extra):
    if not gpu_available():
        pytest.skip("no CUDA GPU")
    import forkerrenderer_gb300 as fr
    from scenes import render_config, scene_path

    scene = fr.Scene(scene_path("def_ao_128"))
    cfg = render_config("def_ao_128")
    cfg.update(extra)
    r = fr.Renderer(**cfg)
    r.Preconfigure(scene)
    return fr, scene, cfg, r


@pytest.mark.parametrize("extra", [{}, {"texture_wrap": 1, "texture_filter": 1}], ids=["nearest", "repeat_linear"])
def test_one_view_one_point_light_matches_render_frame(extra):
    fr, scene, cfg, r = _setup(**extra)
    from forkerrenderer_gb300 import _native as N
    from forkerrenderer_gb300.batch import Batch, point_light, view

    r.Render()
    want = {"frame8": r.frame8(), "depth": r.depth(), "ao": r.ambient_occlusion()}
    info = scene.info
    m = scene.frame_matrices(cfg["shadow_size"])
    b = Batch(r, [view(m, info.eye)], [point_light(info.light_pos, info.light_color, cfg["shadow_size"])])
    for _ in range(2):  # capture, replay
        b.render()
        b.timings()
        assert np.array_equal(b.download(0, N.FR_BUF_FRAME_U8), want["frame8"])
        assert np.array_equal(b.download(0, N.FR_BUF_DEPTH), want["depth"])
        assert np.array_equal(b.download(0, N.FR_BUF_AO), want["ao"])
    assert np.array_equal(b.download(-1, N.FR_BUF_SHADOW), r.shadow_map())
    b.close()


def _views_and_lights(scene, fr):
    from forkerrenderer_gb300.batch import directional_light, view

    eyes = [(0.0, 6.0, 9.0), (5.0, 3.0, 4.0), (-4.0, 5.0, -5.0)]
    sizes = [(128, 96), (64, 64), (160, 96)]
    views = []
    for e, (w, h) in zip(eyes, sizes):
        m = scene.view_matrices(e, (0, 0, 0), 256)
        # a view of its own size: the same camera, the viewport of w x h
        import ctypes as C

        vm = fr.FrameMatrices()
        C.memmove(C.byref(vm), C.byref(m), C.sizeof(m))
        vm.width, vm.height = w, h
        vp = np.array([[w / 2, 0, 0, w / 2], [0, h / 2, 0, h / 2], [0, 0, 0.5, 0.5], [0, 0, 0, 1]], np.float32)
        vm.viewport[:] = list(vp.reshape(-1))
        views.append(view(vm, e))
    lights = [directional_light((0.3, -1.0, 0.2), (0.8, 0.8, 0.7), 256),
              directional_light((-0.5, -0.8, -0.3), (0.3, 0.3, 0.4), 256)]
    return views, lights


def test_views_are_independent_and_tuning_does_not_change_results():
    fr, scene, cfg, r = _setup(shadow_mode=1)
    from forkerrenderer_gb300 import _native as N
    from forkerrenderer_gb300.batch import Batch

    views, lights = _views_and_lights(scene, fr)
    b = Batch(r, views, lights)
    b.render()
    b.timings()
    ref = [b.download(i, N.FR_BUF_FRAME_U8) for i in range(len(views))]
    assert all(f.any() for f in ref)
    for tune in [(8, 256, 1), (32, 1024, 4), (16, 64, 2)]:
        b.set_tuning(*tune)
        b.render()
        b.timings()
        for i in range(len(views)):
            assert np.array_equal(b.download(i, N.FR_BUF_FRAME_U8), ref[i]), tune
    for i in range(len(views)):
        single = Batch(r, [views[i]], lights)
        single.render()
        single.timings()
        assert np.array_equal(single.download(0, N.FR_BUF_FRAME_U8), ref[i])
        single.close()
    w = b.work()
    assert w["triangles"] == scene.info.num_triangles * (len(views) + len(lights))
    assert w["pixels"] == sum(v.matrices.width * v.matrices.height for v in views)
    best, ms = b.autotune(reps=1)
    assert best in [(a, c, k) for a in (8, 16, 32) for c in (64, 256, 1024) for k in (1, 2, 4)] and ms > 0
    b.close()


def test_learned_ao_view_matches_render_frame():
    from forkerrenderer_gb300 import _native as N

    fr, scene, cfg, r = _setup(ao_mode=N.FR_AO_LEARNED, ao_probe_threshold=1e9)
    from forkerrenderer_gb300.aonet import AONet
    from forkerrenderer_gb300.batch import Batch, point_light, view

    net = AONet(0, seed=8)
    r.set_ao_net(net)
    r.Render()
    want_ao = r.ambient_occlusion()
    info = scene.info
    m = scene.frame_matrices(cfg["shadow_size"])
    b = Batch(r, [view(m, info.eye, N.FR_AO_LEARNED), view(m, info.eye, N.FR_AO_SSAO)],
              [point_light(info.light_pos, info.light_color, cfg["shadow_size"])])
    b.render()
    b.timings()
    assert np.array_equal(b.download(0, N.FR_BUF_AO), want_ao)
    assert not np.array_equal(b.download(1, N.FR_BUF_AO), want_ao)  # plain SSAO view
    b.close()


@pytest.mark.parametrize("shadow_mode,mixed", [(1, False), (2, True)], ids=["pcf_2dir", "pcss_point_dir"])
def test_multi_light_views_match_oracle(shadow_mode, mixed):
    """Views lit by two lights against the oracle's restatement of the batch's
    lighting (oracle/fr_oracle.cpp, fr_oracle_render_lights): two directional
    lights with PCF, or a point light (the reference's frustum) and a directional
    light with PCSS. Each light's shadow map and each view's depth bit-exact, AO
    within 2e-6, 8-bit frame within 1 LSB."""
    fr, scene, cfg, r = _setup(shadow_mode=shadow_mode)
    import golden_utils as G
    import oracle_bridge as OB
    from forkerrenderer_gb300 import _native as N
    from forkerrenderer_gb300.batch import Batch, directional_light, point_light

    views, lights = _views_and_lights(scene, fr)
    if mixed:
        lights = [point_light((3.0, 9.0, 6.0), (0.9, 0.9, 0.8), 256), directional_light((-0.5, -0.8, -0.3),
                                                                                         (0.3, 0.3, 0.4), 512)]
    b = Batch(r, views, lights)
    b.render()
    b.timings()
    ocfg = OB.reference_config(**cfg)
    for i, v in enumerate(views):
        want = OB.oracle_render_lights(scene.handle, ocfg, v.matrices, list(v.eye), lights)
        got_d = b.download(i, N.FR_BUF_DEPTH).reshape(want["depth"].shape)
        assert np.array_equal(got_d.view(np.uint32), want["depth"].view(np.uint32)), i
        got_ao = b.download(i, N.FR_BUF_AO).reshape(want["ao"].shape)
        assert np.abs(got_ao - want["ao"]).max() <= 2e-6, i
        G.check_frame8(b.download(i, N.FR_BUF_FRAME_U8), want["frame8"])
        if i == 0:
            for k, s in enumerate(want["shadows"]):
                got_s = b.download(-1 - k, N.FR_BUF_SHADOW).reshape(s.shape)
                assert np.array_equal(got_s.view(np.uint32), s.view(np.uint32)), k
    b.close()
