"""fr_train_ao end to end on a small scene: labels rendered by the renderer, training on
the GPU with the project's kernels, evaluation through the frame's learned-AO path, and
what the trained network gains over the untrained one and over no ambient occlusion."""

import numpy as np
import pytest

from conftest import gpu_available

pytestmark = pytest.mark.gpu


def test_training_gains_over_untrained_and_no_ao():
    if not gpu_available():
        pytest.skip("no CUDA GPU")
    import forkerrenderer_gb300 as fr
    from forkerrenderer_gb300.aonet import AONet, train
    from scenes import render_config, scene_path

    scene = fr.Scene(scene_path("def_ao_128"))
    cfg = fr.default_config(**render_config("def_ao_128"))
    common = dict(train_views=64, eval_views=16, batch=8, crop=64, label_samples=256, seed=3, log_every=50)
    base, _ = train(scene, AONet(0, seed=2), cfg, steps=0, **common)
    net = AONet(0, seed=2)
    rep, losses = train(scene, net, cfg, steps=600, lr=1e-3, lr_final=1e-4, **common)
    assert rep["steps_done"] == 600
    assert rep["final_loss"] < 0.5 * rep["first_loss"], (rep["first_loss"], rep["final_loss"])
    assert np.all(np.isfinite(losses))
    # the trained network beats the untrained one and the method without it (AO = 1)
    assert rep["eval_rmse_covered"] < 0.7 * base["eval_rmse_covered"], (rep, base)
    assert rep["eval_rmse_covered"] < rep["none_rmse_covered"], rep
    # plain SSAO (fewer samples) is the reference-quality fallback: reported next to it
    assert 0.0 < rep["plain_rmse_covered"] < rep["none_rmse_covered"]
    assert rep["probe_mean_avg"] >= 0.0
