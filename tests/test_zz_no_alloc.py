"""The allocation-free blur entry point (fr_blur_separable_noalloc).

It serves callers that must not allocate device memory while they run, for
example a frame loop that forbids allocation after start-up, or a host that
hands the library only buffers from its own pool. Its intermediate plane is a
fixed device array inside the library, so this checks, through the C ABI,
that it gives the same ambient-occlusion buffer as the allocating path (a
frame rendered with the separable blur), on two calls in a row (the second
call finds the previous call's data in the shared array). Its refusal of sizes
beyond the array is checked without a GPU (tests/test_abi.py)."""

import ctypes as C

import numpy as np
import pytest

import scenes
from forkerrenderer_gb300 import Renderer, Scene
from forkerrenderer_gb300 import _native as N

pytestmark = pytest.mark.gpu

def _ao(scene, blur_mode):
    r = Renderer(**scenes.render_config("def_pcss", blur_mode=blur_mode))
    r.Preconfigure(scene)
    r.Render()
    ao = r.ambient_occlusion().copy()
    r.close()
    return ao


def test_noalloc_blur_matches_the_allocating_path_twice():
    import torch

    scene = Scene(scenes.scene_path("def_pcss"))
    raw = _ao(scene, N.FR_BLUR_NONE)            # SSAO before any blur
    want = _ao(scene, N.FR_BLUR_SEPARABLE)      # the allocating path's blur
    H, W = raw.shape
    for call in range(2):
        buf = torch.from_numpy(raw).to("cuda:0").contiguous()
        torch.cuda.synchronize()
        rc = N.lib().fr_blur_separable_noalloc(C.c_void_p(buf.data_ptr()), W, H, None)
        assert rc == N.FR_OK, f"call {call}: status {rc}"
        torch.cuda.synchronize()
        got = buf.cpu().numpy()
        # the same two blur kernels on the same input: bit-identical
        assert np.array_equal(got.view(np.uint32), want.view(np.uint32)), \
            f"call {call}: differs at {np.count_nonzero(got != want)} pixels"
