"""Host-visible fault reporting on the GPU, without any device fault: a tile-bin
capacity far too small for the frame is reported as FR_ERR_BIN_OVERFLOW by the
next synchronising call (the bins and the fine raster never write or read past
the capacity), and the same context renders correctly once the capacity fits."""

import numpy as np
import pytest

from conftest import gpu_available

pytestmark = pytest.mark.gpu


def test_bin_overflow_is_reported_and_the_context_recovers():
    if not gpu_available():
        pytest.skip("no CUDA GPU")
    import forkerrenderer_gb300 as fr
    from forkerrenderer_gb300 import _native as N
    from scenes import render_config, scene_path

    scene = fr.Scene(scene_path("def_stress"))  # its ground and backdrop triangles span many tiles
    cfg = render_config("def_stress")
    good = fr.Renderer(**cfg)
    good.Preconfigure(scene)
    good.Render()
    want = good.depth().copy()
    good.close()

    r = fr.Renderer(**cfg, bin_capacity=8)
    r.Preconfigure(scene)
    r.Render()
    with pytest.raises(fr.RenderError) as e:
        r.depth()
    assert e.value.code == N.FR_ERR_BIN_OVERFLOW
    r.close()

    r = fr.Renderer(**cfg, bin_capacity=1 << 20)
    r.Preconfigure(scene)
    r.Render()
    assert np.array_equal(r.depth(), want)
    r.close()
