"""GB300 path against the reference (golden fixtures) and the CPU oracle,
through the C ABI.

Bar: visibility-derived buffers (depth, shadow map, triangle choice, all seven
G-buffers) bit-exact; ambient occlusion within 2e-6 absolute (powf of the CUDA
math library vs the C library, amplified at most by the blur's 9 taps);
8-bit frame within 1 LSB on >= 99.9% of channels at PSNR >= 50 dB."""

import numpy as np
import pytest

import golden_utils as G
import oracle_bridge as OB
import scenes
from forkerrenderer_gb300 import Renderer, Scene

pytestmark = pytest.mark.gpu

AO_TOL = 2e-6
GB = ["normal", "position", "lightndc", "albedo", "emissive", "param", "type"]


def render(name, **extra):
    cfg = scenes.render_config(name, **extra)
    scene = Scene(scenes.scene_path(name))
    r = Renderer(keep_float_frame=1, **{k: v for k, v in cfg.items()})
    r.Preconfigure(scene)
    r.Render()
    return scene, r


def gpu_buffers(scene, r):
    out = {"depth": r.depth(), "frame8": r.frame8(), "frame": r.frame()}
    if scene.info.shadow_on:
        out["shadow"] = r.shadow_map()
    if scene.info.deferred:
        for g in GB:
            out["gb_" + g] = r.gbuffer(g)
        out["ao"] = r.ambient_occlusion()
    if scene.info.ssaa_on:
        out["ssaa8"] = r.ssaa8()
    return out


@pytest.mark.parametrize("name", sorted(scenes.CASES))
def test_gpu_matches_reference_golden(name):
    meta, arrays = G.load(name)
    assert scenes.files_digest(name) == meta["scene_digest"], "scene generator output differs on this machine"
    scene, r = render(name)
    got = gpu_buffers(scene, r)
    keymap = {"gb_normal": "gb_normal", "gb_position": "gb_position", "gb_lightndc": "gb_lightndc",
              "gb_albedo": "gb_albedo", "gb_emissive": "gb_emissive", "gb_param": "gb_param",
              "gb_type": "gb_type", "depth": "depth", "shadow": "shadow"}
    for k, want in meta["sha256"].items():
        if k == "frame":
            continue  # float frame: powf ulp differences; checked through frame8 below
        assert G.sha(got[keymap[k]]) == want, f"{name}: {k} not bit-exact with the reference"
    if "ao" in arrays:
        d = np.abs(got["ao"].reshape(-1) - arrays["ao"].reshape(-1))
        assert d.max() <= AO_TOL, f"AO max abs diff {d.max()}"
    G.check_frame8(got["frame8"], arrays["frame8"])
    if "ssaa8" in arrays:
        G.check_frame8(got["ssaa8"], arrays["ssaa8"])


@pytest.mark.parametrize("name", sorted(scenes.CASES))
def test_gpu_matches_oracle(name):
    scene, r = render(name)
    got = gpu_buffers(scene, r)
    cfg = OB.reference_config(**scenes.render_config(name))
    want = OB.oracle_render(scene.handle, cfg)
    for k in ["depth", "shadow"] + ["gb_" + g for g in GB]:
        if k in want and k in got:
            a, b = got[k].reshape(-1), want[k].reshape(-1)
            bad = np.flatnonzero(a.view(np.uint32) != b.view(np.uint32))
            assert bad.size == 0, f"{name}: {k} differs at {bad.size} elements, first {bad[:5]}"
    if "ao" in want:
        assert np.abs(got["ao"] - want["ao"]).max() <= AO_TOL
    G.check_frame8(got["frame8"], want["frame8"])


@pytest.mark.parametrize("name", ["def_pcss", "def_stress", "fwd_pcss", "def_ssaa3_odd"])
def test_binned_raster_matches_oracle(name):
    """With area thresholds of 4 / 8 box pixels nearly every triangle goes through
    the tile bins and the fine raster (far more than the eight large triangles the
    fine raster takes without binning), the path the test scenes' few large
    triangles otherwise skip. The thresholds are raster-internal: the oracle is
    the same."""
    scene, r = render(name, small_tri_area=4, medium_tri_area=8)
    got = gpu_buffers(scene, r)
    want = OB.oracle_render(scene.handle, OB.reference_config(**scenes.render_config(name)))
    for k in ["depth", "shadow"] + ["gb_" + g for g in GB]:
        if k in want and k in got:
            a, b = got[k].reshape(-1), want[k].reshape(-1)
            bad = np.flatnonzero(a.view(np.uint32) != b.view(np.uint32))
            assert bad.size == 0, f"{name}: {k} differs at {bad.size} elements, first {bad[:5]}"
    if "ao" in want:
        assert np.abs(got["ao"] - want["ao"]).max() <= AO_TOL
    G.check_frame8(got["frame8"], want["frame8"])
    r.close()


def test_pass_by_pass_equals_render():
    name = "def_pcss"
    scene, r = render(name)
    full = r.frame8().copy()
    r2 = Renderer(**scenes.render_config(name))
    r2.Preconfigure(scene)
    r2.DoShadowPass()
    r2.DoGeometryPass()
    r2.DoLightingPass()
    r2.DoSSAA()
    np.testing.assert_array_equal(r2.frame8(), full)


def test_deterministic_across_runs():
    name = "def_pcss_s256"
    scene, r = render(name)
    a = (r.depth().copy(), r.frame8().copy(), r.ambient_occlusion().copy())
    r.Render()
    b = (r.depth(), r.frame8(), r.ambient_occlusion())
    for x, y in zip(a, b):
        np.testing.assert_array_equal(x, y)


def test_separable_blur_mode_matches_oracle():
    name = "def_pcss"
    scene, r = render(name, blur_mode=1)
    cfg = OB.reference_config(**scenes.render_config(name, blur_mode=1))
    want = OB.oracle_render(scene.handle, cfg)
    assert np.abs(r.ambient_occlusion() - want["ao"]).max() <= AO_TOL


@pytest.mark.parametrize("name,extra", [("c0_fwd_hard_640x400", {}),
                                        ("c1_def_pcss_1280x800", scenes.BENCH_SSAO)])
def test_benchmark_configs_as_specified(name, extra):
    """The two benchmark workloads exactly as specified, at full size, against the
    oracle: the plain forward Blinn-Phong frame (640 x 400, hard shadow, 1024^2
    map) and the deferred PBR + PCSS 16 / 25 + SSAO 64 (r = 0.5) frame of 409,602
    triangles at 1280 x 800 with its 2048^2 map - the frame bench.py times.
    Visibility-derived buffers are also compared with the reference's own digests
    (they do not depend on the SSAO settings)."""
    meta, _ = G.load(name)
    assert scenes.files_digest(name) == meta["scene_digest"], "scene generator output differs on this machine"
    scene, r = render(name, **extra)
    cfg = scenes.render_config(name, **extra)
    if name.startswith("c1"):
        assert scene.info.num_triangles == 409602 and (cfg["ssao_samples"], cfg["ssao_radius"]) == (64, 0.5)
    got = gpu_buffers(scene, r)
    want = OB.oracle_render(scene.handle, OB.reference_config(**cfg))
    for k in ["depth", "shadow"] + ["gb_" + g for g in GB]:
        if k in want and k in got:
            a, b = got[k].reshape(-1), want[k].reshape(-1)
            bad = np.flatnonzero(a.view(np.uint32) != b.view(np.uint32))
            assert bad.size == 0, f"{name}: {k} differs from the oracle at {bad.size} elements, first {bad[:5]}"
            if k in meta["sha256"]:
                assert G.sha(got[k]) == meta["sha256"][k], f"{name}: {k} differs from the reference"
    if "ao" in want:
        assert np.abs(got["ao"] - want["ao"]).max() <= AO_TOL
    G.check_frame8(got["frame8"], want["frame8"])
    r.close()


@pytest.mark.parametrize("radius,samples", [(60.0, 32), (0.0005, 64), (0.075, 7)])
def test_ssao_estimate_paths_match_oracle(radius, samples):
    """The SSAO estimate's other branches against the oracle: a radius whose
    sampling ball reaches the camera plane (no bound: every sample of every pixel
    runs exactly), a radius so small that the samples project within a fraction of
    a pixel of the pixel's own integer coordinates, on the truncation boundaries
    (most samples run exactly), and an odd sample count (a partial 32-sample group)."""
    name = "def_pcss"
    scene, r = render(name, ssao_radius=radius, ssao_samples=samples)
    cfg = scenes.render_config(name, ssao_radius=radius, ssao_samples=samples)
    want = OB.oracle_render(scene.handle, OB.reference_config(**cfg))
    assert np.array_equal(r.depth().view(np.uint32), want["depth"].view(np.uint32))
    assert np.abs(r.ambient_occlusion() - want["ao"]).max() <= AO_TOL
    r.close()


def test_moving_camera_matches_oracle():
    """Frames of other cameras through fr_frame_params (matrices and eye from host
    memory, as the end-to-end benchmark drives them), each against the oracle
    with the same camera; the frame graph is on, so a camera that changes every
    frame is launched directly and one that repeats is replayed."""
    name = "def_pcss_s256"
    scene = Scene(scenes.scene_path(name))
    cfg = scenes.render_config(name)
    r = Renderer(frame_graph=1, **cfg)
    r.Preconfigure(scene)
    eyes = [(3.0, 4.0, 6.0), (-2.5, 5.5, 7.0), (-2.5, 5.5, 7.0), (-2.5, 5.5, 7.0), (0.5, 3.0, 8.0)]
    for eye in eyes:
        m = scene.view_matrices(eye, (0, 0, 0), cfg["shadow_size"])
        r.set_matrices(m, eye)
        r.Render()
        want = OB.oracle_render(scene.handle, OB.reference_config(**cfg), matrices=m, eye=eye)
        assert np.array_equal(r.depth().view(np.uint32), want["depth"].view(np.uint32))
        assert np.array_equal(r.gbuffer("normal").view(np.uint32), want["gb_normal"].view(np.uint32))
        assert np.abs(r.ambient_occlusion() - want["ao"]).max() <= AO_TOL
        G.check_frame8(r.frame8(), want["frame8"])
    r.close()


@pytest.mark.parametrize("name", ["def_pcss", "def_ssaa3_odd", "c1_def_pcss_1280x800"])
def test_parallel_inplace_blur_is_exact_with_any_warmup(name):
    """The in-place blur runs each line in parallel chunks that start a few steps
    early and are kept only when their entry state equals the previous chunk's
    results bit for bit; the others are recomputed in order. Warm-ups of 1 and 4
    steps make most chunks fail that check (the repair path), 64 almost none:
    the AO buffer must be the same bits every time, and within the AO bar of
    the oracle."""
    cfg = scenes.render_config(name, **(scenes.BENCH_SSAO if name.startswith("c1") else {}))
    scene = Scene(scenes.scene_path(name))
    aos = []
    for warm in (0, 1, 4, 64):
        r = Renderer(blur_warmup=warm, **cfg)
        r.Preconfigure(scene)
        r.Render()
        aos.append(r.ambient_occlusion().copy())
        r.close()
    for a in aos[1:]:
        assert np.array_equal(a.view(np.uint32), aos[0].view(np.uint32))
    want = OB.oracle_render(scene.handle, OB.reference_config(**cfg))
    assert np.abs(aos[0] - want["ao"]).max() <= AO_TOL


@pytest.mark.parametrize("name", ["tall_16x4160", "wide_16400x4"])
def test_blur_fallback_for_long_lines_matches_oracle(name):
    """Lines longer than one CTA's shared memory holds (columns of 4,160 rows, rows of
    16,400 pixels) take the sequential in-place walk instead of the parallel chunks:
    the frame still matches the oracle (visibility bit-exact, AO within 2e-6)."""
    scene, r = render(name)
    cfg = scenes.render_config(name)
    want = OB.oracle_render(scene.handle, OB.reference_config(**cfg))
    assert np.array_equal(r.depth().view(np.uint32), want["depth"].view(np.uint32))
    assert np.abs(r.ambient_occlusion() - want["ao"]).max() <= AO_TOL
    G.check_frame8(r.frame8(), want["frame8"])
    r.close()


def test_frame_download_into_pinned_memory_equals_the_copy():
    """fr_download of the 8-bit frame (and the SSAA image) writes pinned,
    device-addressable host memory directly from the packing kernel; the bytes
    equal those of the copying path into ordinary host memory."""
    import torch

    for name in ("def_pcss", "def_pcf_ssaa"):
        scene, r = render(name)
        want = r.frame8().copy()
        pinned = torch.empty(want.size, dtype=torch.uint8, pin_memory=True).numpy()
        got = r.frame8(pinned)
        assert np.array_equal(got, want)
        if scene.info.ssaa_on:
            from forkerrenderer_gb300 import _native as N

            ws = r.ssaa8().copy()
            ps = torch.empty(ws.size, dtype=torch.uint8, pin_memory=True).numpy()
            assert np.array_equal(r.download(N.FR_BUF_SSAA_U8, ps).reshape(ws.shape), ws)
        r.close()


def test_pinned_download_waits_for_a_frame_on_a_callers_stream():
    """Frames rendered on a caller's stream and downloaded straight into pinned
    memory, with no synchronisation between: the packing kernel is ordered after
    the frame's last kernel, so each download holds that frame (the camera moves
    every frame, and every image equals the oracle's for its matrices)."""
    import torch

    name = "def_pcss"
    scene = Scene(scenes.scene_path(name))
    cfg = scenes.render_config(name)
    r = Renderer(**cfg)
    r.Preconfigure(scene)
    side = torch.cuda.Stream()
    r.set_stream(side.cuda_stream)
    n = scene.info.width * scene.info.height * 3
    pinned = torch.empty(n, dtype=torch.uint8, pin_memory=True).numpy()
    for eye in ((2.0, 1.5, 3.0), (-2.5, 1.0, 2.0)):
        mats = scene.view_matrices(eye, (0, 0, 0), cfg["shadow_size"])
        r.set_matrices(mats, eye)
        r.Render()
        got = r.frame8(pinned).copy()
        torch.cuda.synchronize()
        want = OB.oracle_render(scene.handle, OB.reference_config(**cfg), matrices=mats, eye=eye)
        G.check_frame8(got, want["frame8"])
    r.set_stream(None)
    r.close()


def test_shadow_pass_after_another_light_matches_oracle():
    """Alternating two light-space matrices on one context, through direct frames
    and then a captured and replayed graph: each shadow map and depth buffer
    matches the oracle with that frame's light, so nothing of the previous pass's
    visibility keys or light matrices carries over."""
    import ctypes as C

    from forkerrenderer_gb300 import _native as N

    name = "def_pcss_s256"
    scene = Scene(scenes.scene_path(name))
    cfg = scenes.render_config(name)
    r = Renderer(frame_graph=1, **cfg)
    r.Preconfigure(scene)
    m0 = scene.frame_matrices(cfg["shadow_size"])
    m1 = N.FrameMatrices()
    C.memmove(C.byref(m1), C.byref(m0), C.sizeof(N.FrameMatrices))
    for k in range(8):  # the light's x and y scaled about the map's centre: another shadow map
        m1.light_space[k] *= 0.8
    for m in (m0, m1, m0, m1, m1, m1):
        r.set_matrices(m)
        r.Render()
        want = OB.oracle_render(scene.handle, OB.reference_config(**cfg), matrices=m)
        assert np.array_equal(r.shadow_map().view(np.uint32), want["shadow"].view(np.uint32))
        assert np.array_equal(r.depth().view(np.uint32), want["depth"].view(np.uint32))
    r.close()
