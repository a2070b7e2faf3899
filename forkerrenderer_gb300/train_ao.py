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


# ---- checkpoints ----------------------------------------------------------------------
# A checkpoint holds everything a run needs to continue bit for bit: the parameters,
# Adam's moments and step count, and the index of the next training step. Layout
# (little-endian):
#   b"FRAOCKPT", u32 version (1), u32 dtype (1 = float32),
#   i64 parameter count, i64 Adam step, i64 next training step,
#   u32 tensor count, then per tensor: 16-byte name (NUL padded), i32 rank, i32 dims[4];
#   float32 parameters, float32 Adam m, float32 Adam v (parameter order of fr_aonet.h),
#   u32 CRC-32 (zlib) of every byte before it.
CKPT_MAGIC = b"FRAOCKPT"
CKPT_VERSION = 1

# fr_aonet.h's layers: (name, cout, cin) of the ten 3x3 convolutions, then the 1x1 head.
LAYERS = [("e0a", 16, 16), ("e0b", 16, 16), ("e1a", 32, 16), ("e1b", 32, 32), ("b0", 64, 32), ("b1", 64, 64),
          ("d1a", 32, 96), ("d1b", 32, 32), ("d0a", 16, 48), ("d0b", 16, 16)]
HEAD = ("head", 4, 16)


def tensor_table() -> list[tuple[str, tuple]]:
    t = []
    for name, co, ci in LAYERS:
        t += [(name + ".w", (co, ci, 3, 3)), (name + ".b", (co,))]
    t += [(HEAD[0] + ".w", (HEAD[1], HEAD[2])), (HEAD[0] + ".b", (HEAD[1],))]
    assert sum(int(np.prod(s)) for _, s in t) == NUM_PARAMS
    return t


def encode_checkpoint(params, adam_m, adam_v, adam_step: int, next_step: int) -> bytes:
    import struct
    import zlib

    table = tensor_table()
    head = CKPT_MAGIC + struct.pack("<IIqqqI", CKPT_VERSION, 1, NUM_PARAMS, adam_step, next_step, len(table))
    for name, shape in table:
        dims = list(shape) + [0] * (4 - len(shape))
        head += name.encode().ljust(16, b"\0") + struct.pack("<i4i", len(shape), *dims)
    body = b"".join(np.ascontiguousarray(a, "<f4").tobytes() for a in (params, adam_m, adam_v))
    if len(body) != 3 * 4 * NUM_PARAMS:
        raise ValueError("checkpoint arrays must hold the network's parameter count")
    data = head + body
    return data + struct.pack("<I", zlib.crc32(data) & 0xFFFFFFFF)


def decode_checkpoint(data: bytes) -> dict:
    """Checks magic, version, dtype, tensor table and CRC; returns the arrays and counters."""
    import struct
    import zlib

    if len(data) < 48 or data[:8] != CKPT_MAGIC:
        raise ValueError("not a learned-AO checkpoint")
    (crc,) = struct.unpack("<I", data[-4:])
    if zlib.crc32(data[:-4]) & 0xFFFFFFFF != crc:
        raise ValueError("checkpoint CRC mismatch (file damaged)")
    version, dtype, count, adam_step, next_step, ntab = struct.unpack_from("<IIqqqI", data, 8)
    if version != CKPT_VERSION or dtype != 1:
        raise ValueError(f"unsupported checkpoint version {version} / dtype {dtype}")
    pos = 8 + struct.calcsize("<IIqqqI")
    table = []
    for _ in range(ntab):
        name = data[pos:pos + 16].rstrip(b"\0").decode()
        rank, *dims = struct.unpack_from("<i4i", data, pos + 16)
        table.append((name, tuple(dims[:rank])))
        pos += 16 + 20
    if count != NUM_PARAMS or table != tensor_table():
        raise ValueError("checkpoint tensor table does not match this network")
    arrs = np.frombuffer(data, "<f4", 3 * NUM_PARAMS, pos).reshape(3, NUM_PARAMS)
    return {"params": arrs[0].copy(), "adam_m": arrs[1].copy(), "adam_v": arrs[2].copy(),
            "adam_step": int(adam_step), "next_step": int(next_step)}


def save_checkpoint(path: str, net: AONet, next_step: int) -> None:
    import ctypes as C

    p, m, v = (np.empty(NUM_PARAMS, np.float32) for _ in range(3))
    t = C.c_int64(0)
    fp = lambda a: a.ctypes.data_as(C.POINTER(C.c_float))  # noqa: E731
    rc = N.lib().fr_aonet_get_state(net.handle, fp(p), fp(m), fp(v), NUM_PARAMS, C.byref(t))
    if rc != N.FR_OK:
        raise RuntimeError("fr_aonet_get_state failed")
    tmp = path + ".tmp"
    with open(tmp, "wb") as f:
        f.write(encode_checkpoint(p, m, v, t.value, next_step))
    os.replace(tmp, path)


def load_checkpoint(path: str, net: AONet) -> int:
    """Restores the network's whole training state; returns the next training step."""
    import ctypes as C

    with open(path, "rb") as f:
        ck = decode_checkpoint(f.read())
    fp = lambda a: a.ctypes.data_as(C.POINTER(C.c_float))  # noqa: E731
    rc = N.lib().fr_aonet_set_state(net.handle, fp(ck["params"]), fp(ck["adam_m"]), fp(ck["adam_v"]), NUM_PARAMS,
                                    ck["adam_step"])
    if rc != N.FR_OK:
        raise RuntimeError("fr_aonet_set_state failed")
    return ck["next_step"]


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
                    help="network input channel 3: 0 = normal z, -1 = depth residual, K = K-sample SSAO of the pixel")
    ap.add_argument("--seed", type=int, default=1)
    ap.add_argument("--net-seed", type=int, default=0)
    ap.add_argument("--init", default=None, help="start from these weights")
    ap.add_argument("--checkpoint", default=None, help="write the whole training state here at the end")
    ap.add_argument("--resume", default=None,
                    help="continue the run of this checkpoint: --steps more steps, same schedule (--schedule-steps)")
    ap.add_argument("--schedule-steps", type=int, default=0,
                    help="length of the whole run's cosine schedule (0 = the steps run so far + --steps)")
    ap.add_argument("--device", type=int, default=0)
    a = ap.parse_args(argv)

    t0 = time.time()
    scene = Scene(field_scene_path(0))
    cfg = default_config(**FIELD_RENDER, device=a.device, ao_input_samples=a.input_samples)
    net = AONet(a.device, seed=a.net_seed)
    first = 0
    if a.init:
        net.set_params(load_params(a.init))
    if a.resume:
        first = load_checkpoint(a.resume, net)
    rep, losses = train(scene, net, cfg, train_views=a.train_views, eval_views=a.eval_views, steps=a.steps,
                        batch=a.batch, crop=a.crop, lr=a.lr, lr_final=a.lr_final, label_samples=a.label_samples, seed=a.seed,
                        log_every=max(1, a.steps // 50), first_step=first, schedule_steps=a.schedule_steps)
    save_params(a.out, net.get_params())
    if a.checkpoint:
        save_checkpoint(a.checkpoint, net, first + a.steps)
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
