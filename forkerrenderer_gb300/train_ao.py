"""Train the learned-AO U-Net on the 20-icosphere field scene and save its weights.

    python -m forkerrenderer_gb300.train_ao --out aonet.f32 [--steps N] [--train-views V] ...

Renders the labelled views (256-sample SSAO + blur), trains with Adam on random
256x256 crops (batch 16) through fr_train_ao, evaluates on held-out views, and
writes the FP32 parameters (fr_aonet.h order) plus a JSON report next to them.
"""

from __future__ import annotations

import argparse
import json
import os
import tempfile
import time

import numpy as np

from . import Renderer, Scene, default_config, scenegen
from . import _native as N
from .aonet import NUM_PARAMS, AONet, train

# The deferred PBR + PCSS + SSAO field: 20 icospheres (subdivision 5) on a plane,
# 1280x800, SSAO 64 samples radius 0.5.
FIELD_SCENE = dict(seed=0, n_spheres=20, subdiv=5, tex=1024, width=1280, height=800)
FIELD_RENDER = dict(shadow_mode=N.FR_SHADOW_PCSS, shadow_size=2048, pcf_samples=25, blocker_samples=16,
                    ssao_samples=64, ssao_radius=0.5, ssao_bias=0.0005, ssao_range=0.01,
                    blur_mode=N.FR_BLUR_REFERENCE)


def field_scene_path(seed: int = 0) -> str:
    out = os.path.join(tempfile.gettempdir(), f"fr_bench_c1_seed{seed}")
    path = os.path.join(out, "scene.scene")
    if not os.path.exists(path):
        tmp = out + ".tmp%d" % os.getpid()
        scenegen.deferred_field_scene(tmp, **dict(FIELD_SCENE, seed=seed))
        try:
            os.rename(tmp, out)
        except OSError:
            pass
    return path


def save_params(path: str, p: np.ndarray) -> None:
    np.asarray(p, "<f4").tofile(path)


def load_params(path: str) -> np.ndarray:
    p = np.fromfile(path, "<f4")
    if p.size != NUM_PARAMS:
        raise ValueError(f"{path}: {p.size} parameters, expected {NUM_PARAMS}")
    return p


def main(argv=None) -> dict:
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--out", required=True, help="output weights file (raw little-endian float32)")
    ap.add_argument("--steps", type=int, default=3000)
    ap.add_argument("--train-views", type=int, default=2000)
    ap.add_argument("--eval-views", type=int, default=200)
    ap.add_argument("--batch", type=int, default=16)
    ap.add_argument("--crop", type=int, default=256)
    ap.add_argument("--lr", type=float, default=1e-3)
    ap.add_argument("--lr-final", type=float, default=0.0, help="cosine decay to this rate (0 = constant)")
    ap.add_argument("--label-samples", type=int, default=256)
    ap.add_argument("--input-samples", type=int, default=0,
                    help="network input channel 3: 0 = normal z, K = K-sample SSAO of the pixel")
    ap.add_argument("--seed", type=int, default=1)
    ap.add_argument("--net-seed", type=int, default=0)
    ap.add_argument("--init", default=None, help="start from these weights")
    ap.add_argument("--device", type=int, default=0)
    a = ap.parse_args(argv)

    t0 = time.time()
    scene = Scene(field_scene_path(0))
    cfg = default_config(**FIELD_RENDER, device=a.device, ao_input_samples=a.input_samples)
    net = AONet(a.device, seed=a.net_seed)
    if a.init:
        net.set_params(load_params(a.init))
    rep, losses = train(scene, net, cfg, train_views=a.train_views, eval_views=a.eval_views, steps=a.steps,
                        batch=a.batch, crop=a.crop, lr=a.lr, lr_final=a.lr_final, label_samples=a.label_samples, seed=a.seed,
                        log_every=max(1, a.steps // 50))
    save_params(a.out, net.get_params())
    rep = {k: (round(v, 6) if isinstance(v, float) else v) for k, v in rep.items()}
    rep.update(losses=[round(float(x), 6) for x in losses], wall_seconds=round(time.time() - t0, 1),
               args=vars(a), input_samples=a.input_samples)
    with open(os.path.splitext(a.out)[0] + ".json", "w") as f:
        json.dump(rep, f, indent=1)
    print(json.dumps({k: v for k, v in rep.items() if k != "losses"}))
    net.close()
    return rep


if __name__ == "__main__":
    main()
