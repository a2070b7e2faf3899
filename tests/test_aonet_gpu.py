"""Learned-AO U-Net on the GPU (tcgen05 BF16 convolutions) against the CPU oracle."""

import os
import sys

import numpy as np
import pytest

from conftest import gpu_available

pytestmark = pytest.mark.gpu

sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "oracle"))


def _need_gpu():
    if not gpu_available():
        pytest.skip("no CUDA GPU")


def _batch(rng, B, H, W):
    from forkerrenderer_gb300.aonet import pack_input, unpack_input

    x = np.zeros((B, 4, H, W), np.float32)
    x[:, 0] = rng.uniform(0.5, 2.0, (B, H, W))
    n = rng.normal(size=(B, 3, H, W))
    x[:, 1:] = n / np.linalg.norm(n, axis=1, keepdims=True)
    # a background hole: all-zero input, as the renderer writes for empty pixels
    x[:, :, : H // 4, : W // 3] = 0
    bits = pack_input(x)
    return bits, unpack_input(bits)


def _dev(a, dtype=None):
    import torch

    t = torch.from_numpy(np.ascontiguousarray(a))
    if dtype is not None:
        t = t.view(dtype)
    return t.cuda()


@pytest.mark.parametrize("shape", [(2, 32, 64), (1, 64, 96), (3, 96, 32)])
def test_forward_matches_oracle(shape):
    _need_gpu()
    import torch
    import aonet_ref as R
    from forkerrenderer_gb300.aonet import AONet

    B, H, W = shape
    rng = np.random.default_rng(sum(shape))
    net = AONet(0, seed=11)
    p = net.get_params()
    bits, x4 = _batch(rng, B, H, W)
    xt = _dev(bits.view(np.int16))
    ao = torch.full((B, H, W), -1.0, device="cuda")
    net.forward(xt, B, H, W, ao)
    net.check()
    got = ao.cpu().numpy()
    ref = R.Net(p).forward(x4)
    assert np.all(np.isfinite(got))
    err = np.abs(got - ref)
    assert err.max() < 4e-3, err.max()
    assert err.mean() < 2e-4, err.mean()
    # deterministic
    ao2 = torch.empty_like(ao)
    net.forward(xt, B, H, W, ao2)
    net.check()
    assert torch.equal(ao, ao2)


def _layer_slices():
    import aonet_ref as R

    out, off = [], 0
    for i, (_, _, co, _, ci) in enumerate(R.LAYERS):
        n = co * ci * 9
        out.append((f"W{i}", slice(off, off + n)))
        out.append((f"b{i}", slice(off + n, off + n + co)))
        off += n + co
    out.append(("head_w", slice(off, off + 64)))
    out.append(("head_b", slice(off + 64, off + 68)))
    return out


def test_gradients_match_oracle():
    _need_gpu()
    import aonet_ref as R
    from forkerrenderer_gb300.aonet import AONet

    B, H, W = 2, 64, 64
    rng = np.random.default_rng(21)
    net = AONet(0, seed=5)
    p = net.get_params()
    bits, x4 = _batch(rng, B, H, W)
    label = rng.uniform(0.1, 0.95, (B, H, W)).astype(np.float32)
    label[:, -5:, :] = -1.0  # outside the loss
    loss = net.backward(_dev(bits.view(np.int16)), _dev(label), B, H, W)
    g = net.get_grads()
    ref_net = R.Net(p)
    ref_net.forward(x4)
    ref_loss, gref = ref_net.backward(label)
    assert abs(loss - ref_loss) <= 2e-3 * ref_loss
    for name, sl in _layer_slices():
        a, b = g[sl].astype(np.float64), gref[sl]
        rel = np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-12)
        assert rel < 3e-2, (name, rel)


def test_adam_step_matches_oracle():
    _need_gpu()
    import aonet_ref as R
    from forkerrenderer_gb300.aonet import AONet

    B, H, W = 1, 32, 32
    rng = np.random.default_rng(2)
    net = AONet(0, seed=3)
    p0 = net.get_params()
    bits, _ = _batch(rng, B, H, W)
    label = rng.uniform(0.1, 0.95, (B, H, W)).astype(np.float32)
    net.backward(_dev(bits.view(np.int16)), _dev(label), B, H, W)
    g = net.get_grads()
    net.adam_step(lr=1e-3)
    p1 = net.get_params()
    z = np.zeros_like(p0)
    ref, _, _ = R.adam_step(p0, g, z, z, 1, lr=1e-3)
    assert np.allclose(p1, ref, rtol=1e-6, atol=1e-7)


def test_training_reduces_loss():
    _need_gpu()
    from forkerrenderer_gb300.aonet import AONet

    B, H, W = 4, 64, 64
    rng = np.random.default_rng(9)
    bits, x4 = _batch(rng, B, H, W)
    # a smooth target the network can fit: a function of depth and the normal's z
    label = np.clip(0.35 + 0.3 * x4[:, 3] + 0.1 * x4[:, 0], 0.05, 0.95).astype(np.float32)
    xt, lt = _dev(bits.view(np.int16)), _dev(label)
    net = AONet(0, seed=1)
    first = net.train_step(xt, lt, B, H, W, lr=2e-3)
    for _ in range(80):
        last = net.train_step(xt, lt, B, H, W, lr=2e-3, want_loss=False)
    last = net.backward(xt, lt, B, H, W)
    assert last < 0.3 * first, (first, last)


def test_renderer_learned_mode_and_fallback():
    _need_gpu()
    import torch

    import forkerrenderer_gb300 as fr
    from forkerrenderer_gb300 import _native as N
    from forkerrenderer_gb300.aonet import AONet
    from scenes import render_config, scene_path

    scene = fr.Scene(scene_path("def_ao_128"))
    m = scene.frame_matrices(256)
    H, W = m.height, m.width
    base = render_config("def_ao_128")
    plain = fr.Renderer(**base)
    plain.Preconfigure(scene)
    plain.Render()
    ao_plain = plain.ambient_occlusion()
    raw = fr.Renderer(**dict(base, blur_mode=N.FR_BLUR_NONE))
    raw.Preconfigure(scene)
    raw.Render()
    ao_raw = raw.ambient_occlusion()  # background pixels: the per-noise-cell values, unblurred
    raw.close()

    net = AONet(0, seed=4)
    for thr, expect_fallback in ((1e9, False), (-1.0, True)):
        r = fr.Renderer(**base, ao_mode=N.FR_AO_LEARNED, ao_probe_threshold=thr)
        r.Preconfigure(scene)
        r.set_ao_net(net)
        r.Render()
        mean, fell = r.ao_probe_result()
        assert fell == expect_fallback
        assert mean >= 0.0
        ao = r.ambient_occlusion()
        if expect_fallback:
            assert np.array_equal(ao, ao_plain)
        else:
            feat = torch.zeros((1, 1, H, W, 8), dtype=torch.int16, device="cuda")
            r.ao_features(feat)
            torch.cuda.synchronize()
            out = torch.empty((1, H, W), device="cuda")
            net.forward(feat, 1, H, W, out)
            net.check()
            # covered pixels: the network's AO; background: the plain SSAO's value
            bg = r.depth() == np.finfo(np.float32).max
            assert bg.any() and (~bg).any()
            assert np.array_equal(ao[~bg], out.cpu().numpy()[0][~bg])
            assert np.array_equal(ao[bg], ao_raw[bg])
            # the probe's mean: covered pixels (8i + 4, 8j + 4), network AO against
            # plain SSAO of the frame's sample count without blur
            pr = np.ix_(4 + 8 * np.arange(H // 8), 4 + 8 * np.arange(W // 8))
            cov = ~bg[pr]
            want = np.mean((ao[pr][cov].astype(np.float64) - ao_raw[pr][cov]) ** 2)
            assert cov.any() and abs(mean - want) <= 1e-5 * want + 1e-12, (mean, want)
        r.close()


def _bf16_round(a: np.ndarray) -> np.ndarray:
    u = np.asarray(a, np.float32).view(np.uint32).astype(np.uint64)
    u = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return u.astype(np.uint32).view(np.float32)


def test_input_channel_three_is_k_sample_ssao():
    """With ao_input_samples = K the network's fourth input channel is the pixel's
    K-sample SSAO without blur: it equals (rounded to BF16) the AO buffer of a plain
    frame rendered with K SSAO samples and the blur off (K = 64: a sample table
    beyond the default 48 KB of shared memory)."""
    _need_gpu()
    import torch

    import forkerrenderer_gb300 as fr
    from forkerrenderer_gb300 import _native as N
    from forkerrenderer_gb300.aonet import AONet
    from scenes import render_config, scene_path

    scene = fr.Scene(scene_path("def_ao_128"))
    m = scene.frame_matrices(256)
    H, W = m.height, m.width
    base = render_config("def_ao_128")
    for K in (4, 8, 16, 64):
        plain = fr.Renderer(**dict(base, ssao_samples=K, blur_mode=N.FR_BLUR_NONE))
        plain.Preconfigure(scene)
        plain.Render()
        ao_k = plain.ambient_occlusion()
        depth = plain.depth()
        plain.close()
        r = fr.Renderer(**base, ao_mode=N.FR_AO_LEARNED, ao_probe_threshold=1e9, ao_input_samples=K)
        r.Preconfigure(scene)
        net = AONet(0, seed=4)
        r.set_ao_net(net)
        r.Render()
        feat = torch.zeros((1, 1, H, W, 8), dtype=torch.int16, device="cuda")
        r.ao_features(feat)
        torch.cuda.synchronize()
        f = feat.cpu().numpy().view(np.uint16)[0, 0].astype(np.uint32) << 16
        ch3 = f[..., 3].view(np.float32)
        covered = depth < np.finfo(np.float32).max
        assert covered.any() and (~covered).any()
        assert np.array_equal(ch3[covered], _bf16_round(ao_k)[covered])
        assert not ch3[~covered].any()
        r.close()
        net.close()


def test_fused_forward_matches_layer_by_layer():
    """The renderer's single-launch forward (k_unet_fwd, grid barriers between
    layers) gives the same AO buffer as one launch per layer, bit for bit, with and
    without the frame graph."""
    _need_gpu()
    import forkerrenderer_gb300 as fr
    from forkerrenderer_gb300 import _native as N
    from forkerrenderer_gb300.aonet import AONet
    from scenes import render_config, scene_path

    scene = fr.Scene(scene_path("def_ao_128"))
    base = render_config("def_ao_128")
    net = AONet(0, seed=11)
    out = {}
    for fused in (False, True):
        for graph in (0, 1):
            net.set_fused(fused)
            r = fr.Renderer(**base, ao_mode=N.FR_AO_LEARNED, ao_probe_threshold=1e9, ao_input_samples=8,
                            frame_graph=graph)
            r.Preconfigure(scene)
            r.set_ao_net(net)
            for _ in range(3):  # direct, capture, replay
                r.Render()
            out[(fused, graph)] = r.ambient_occlusion()
            net.check()
            r.close()
    ref = out[(False, 0)]
    assert ref.min() >= 0.0 and ref.max() <= 1.0
    for k, v in out.items():
        assert np.array_equal(v, ref), k
    net.close()


def test_fused_forward_grid_barrier_times_out_and_recovers():
    """A bounded device wait made to run out, without a fault: with a 5 ms limit on
    the grid barriers of the fused forward and one CTA that never arrives at the
    first barrier (a flag that nothing sets), the other CTAs give up, the kernel
    returns with its TMEM freed, and the renderer's next synchronising call reports
    FR_ERR_TIMEOUT. The same context and network then render the frame exactly as
    before."""
    _need_gpu()
    import forkerrenderer_gb300 as fr
    from forkerrenderer_gb300 import _native as N
    from forkerrenderer_gb300.aonet import AONet
    from scenes import render_config, scene_path

    scene = fr.Scene(scene_path("def_ao_128"))
    base = render_config("def_ao_128")
    net = AONet(0, seed=11)
    net.set_fused(True)
    r = fr.Renderer(**base, ao_mode=N.FR_AO_LEARNED, ao_probe_threshold=1e9, ao_input_samples=8)
    r.Preconfigure(scene)
    r.set_ao_net(net)
    r.Render()
    want = r.ambient_occlusion().copy()
    L = N.lib()
    assert L.fr_aonet_set_wait_limit(net.handle, 5_000_000) == 0
    assert L.fr_aonet_test_absent_cta(net.handle, 0) == 0
    r.Render()
    with pytest.raises(fr.RenderError) as e:
        r.ambient_occlusion()
    assert e.value.code == N.FR_ERR_TIMEOUT, e.value
    assert L.fr_aonet_test_absent_cta(net.handle, -1) == 0
    assert L.fr_aonet_set_wait_limit(net.handle, 0) == 0
    r.Render()
    assert np.array_equal(r.ambient_occlusion(), want)
    net.check()
    r.close()
    net.close()
