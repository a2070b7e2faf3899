"""Learned-AO training checkpoints (forkerrenderer_gb300/train_ao.py): the file
format on the CPU, and on the GPU that a run resumed from a checkpoint is the
uninterrupted run bit for bit."""

import numpy as np
import pytest

from conftest import gpu_available
from forkerrenderer_gb300 import train_ao as T
from forkerrenderer_gb300.aonet import NUM_PARAMS


def _state(seed):
    rng = np.random.default_rng(seed)
    return [rng.standard_normal(NUM_PARAMS).astype(np.float32) for _ in range(3)]


def test_checkpoint_round_trip():
    p, m, v = _state(1)
    ck = T.decode_checkpoint(T.encode_checkpoint(p, m, v, adam_step=1234, next_step=1200))
    for k, a in (("params", p), ("adam_m", m), ("adam_v", v)):
        assert np.array_equal(ck[k].view(np.uint32), a.view(np.uint32)), k
    assert (ck["adam_step"], ck["next_step"]) == (1234, 1200)


def test_checkpoint_damage_and_mismatch_are_refused():
    p, m, v = _state(2)
    data = bytearray(T.encode_checkpoint(p, m, v, 7, 7))
    bad = bytes(data[:500] + bytes([data[500] ^ 1]) + data[501:])
    with pytest.raises(ValueError, match="CRC"):
        T.decode_checkpoint(bad)
    with pytest.raises(ValueError, match="not a learned-AO checkpoint"):
        T.decode_checkpoint(b"XXXXXXXX" + bytes(data[8:]))
    with pytest.raises(ValueError, match="parameter count"):
        T.encode_checkpoint(p[:-1], m, v, 1, 1)
    # a file whose tensor table names another network (CRC recomputed: not damage)
    import struct
    import zlib

    body = bytes(data[:-4]).replace(b"d0a.w", b"d0x.w")
    with pytest.raises(ValueError, match="tensor table"):
        T.decode_checkpoint(body + struct.pack("<I", zlib.crc32(body) & 0xFFFFFFFF))


@pytest.mark.gpu
def test_resumed_training_equals_the_uninterrupted_run(tmp_path):
    if not gpu_available():
        pytest.skip("no CUDA GPU")
    import forkerrenderer_gb300 as fr
    from forkerrenderer_gb300.aonet import AONet, train
    from scenes import render_config, scene_path

    scene = fr.Scene(scene_path("def_ao_128"))
    cfg = fr.default_config(**render_config("def_ao_128"), ao_input_samples=4)
    kw = dict(train_views=2, eval_views=0, batch=2, crop=64, label_samples=8, lr=1e-3, lr_final=1e-4, seed=3,
              log_every=1, schedule_steps=5)
    full = AONet(0, seed=5)
    train(scene, full, cfg, steps=5, **kw)
    part = AONet(0, seed=5)
    train(scene, part, cfg, steps=3, **kw)
    path = str(tmp_path / "run.ckpt")
    T.save_checkpoint(path, part, next_step=3)
    part.close()
    resumed = AONet(0, seed=99)  # other initial weights: everything must come from the file
    first = T.load_checkpoint(path, resumed)
    assert first == 3
    train(scene, resumed, cfg, steps=2, first_step=first, **kw)
    a, b = full.get_params(), resumed.get_params()
    assert np.array_equal(a.view(np.uint32), b.view(np.uint32))
    T.save_checkpoint(str(tmp_path / "a.ckpt"), full, 5)
    T.save_checkpoint(str(tmp_path / "b.ckpt"), resumed, 5)
    assert open(tmp_path / "a.ckpt", "rb").read() == open(tmp_path / "b.ckpt", "rb").read()
    full.close()
    resumed.close()
