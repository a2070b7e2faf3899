"""Host-visible fault reporting on the GPU, without any device fault: a tile-bin
capacity far too small for the frame is reported as FR_ERR_BIN_OVERFLOW by the
next synchronising call (the bins and the fine raster never write or read past
the capacity), and the same context then renders a frame that fits its capacity
correctly."""

import numpy as np
import pytest

import golden_utils as G
import oracle_bridge as OB
from conftest import gpu_available

pytestmark = pytest.mark.gpu


def test_bin_overflow_is_reported_and_the_context_recovers():
    if not gpu_available():
        pytest.skip("no CUDA GPU")
    import forkerrenderer_gb300 as fr
    from forkerrenderer_gb300 import _native as N
    from scenes import render_config, scene_path

    scene = fr.Scene(scene_path("def_stress"))  # its ground and backdrop triangles span many tiles
    # every triangle of more than 8 box pixels goes through the tile bins (with only
    # a few large triangles the fine raster takes them without binning)
    cfg = render_config("def_stress", small_tri_area=4, medium_tri_area=8)
    good = fr.Renderer(**cfg)
    good.Preconfigure(scene)
    good.Render()
    want = good.depth().copy()
    good.close()

    r = fr.Renderer(**cfg, bin_capacity=16)
    r.Preconfigure(scene)
    r.Render()
    with pytest.raises(fr.RenderError) as e:
        r.depth()
    assert e.value.code == N.FR_ERR_BIN_OVERFLOW

    # The same context, a frame within its 16 (triangle, tile) pairs: a 16 x 16
    # frame (one tile) of 11 triangles, its screen-sized shadow map likewise.
    tiny = fr.Scene(scene_path("tiny_16x16"))
    assert tiny.info.num_triangles <= 16
    ref = fr.Renderer(**cfg)  # the same configuration with the default capacity
    ref.Preconfigure(tiny)
    ref.Render()
    r.Preconfigure(tiny)
    r.Render()
    for get in (lambda x: x.depth(), lambda x: x.shadow_map(), lambda x: x.frame8()):
        a, b = get(r), get(ref)
        assert np.array_equal(a.view(np.uint8), b.view(np.uint8))
    assert np.count_nonzero(r.depth() < 3e38) > 0  # the frame does cover pixels
    tiny_want = OB.oracle_render(tiny.handle, OB.reference_config(**cfg))
    assert np.array_equal(r.depth().view(np.uint32), tiny_want["depth"].view(np.uint32))
    G.check_frame8(r.frame8(), tiny_want["frame8"])
    ref.close()

    # and the stress frame again with enough capacity
    r2 = fr.Renderer(**cfg, bin_capacity=1 << 20)
    r2.Preconfigure(scene)
    r2.Render()
    assert np.array_equal(r2.depth(), want)
    r2.close()
    r.close()


@pytest.mark.parametrize("bad", [dict(ssao_samples=257), dict(ssao_samples=0), dict(small_tri_area=65537),
                                 dict(small_tri_area=-1), dict(medium_tri_area=(1 << 20) + 1)])
def test_out_of_range_config_is_rejected(bad):
    """Configurations the kernels do not support (the SSAO table beyond shared
    memory, a warp's flattened small-triangle pixel list beyond int range, more
    medium-triangle boxes than one warp should walk) fail at creation with a message."""
    if not gpu_available():
        pytest.skip("no CUDA GPU")
    import forkerrenderer_gb300 as fr

    with pytest.raises(fr.RenderError) as e:
        fr.Renderer(**bad)
    assert "must be in" in str(e.value)


def test_oversized_shadow_map_is_rejected():
    """Texel indices are 32-bit in the kernels: a shadow map of more than 2^30
    texels is refused with FR_ERR_INVALID before any allocation."""
    if not gpu_available():
        pytest.skip("no CUDA GPU")
    import forkerrenderer_gb300 as fr
    from forkerrenderer_gb300 import _native as N
    from scenes import render_config, scene_path

    scene = fr.Scene(scene_path("def_pcss"))
    r = fr.Renderer(**render_config("def_pcss", shadow_size=32769))
    with pytest.raises(fr.RenderError) as e:
        r.Preconfigure(scene)
        r.Render()
    assert "2^30" in str(e.value) and str(N.FR_ERR_INVALID) in str(e.value)
    r.close()
