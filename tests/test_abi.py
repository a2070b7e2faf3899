"""The C ABI library loads and exports every entry point the public headers
declare; host-only entry points work without a GPU."""

import ctypes as C
import re

import pytest

from forkerrenderer_gb300 import _native as N


def test_library_exports_every_declared_symbol():
    lib = C.CDLL(N.LIB_PATH)
    declared = N.exported_symbols()
    assert len(declared) >= 20
    missing = [s for s in declared if not hasattr(lib, s)]
    assert not missing, missing


def test_config_defaults_are_the_reference_constants():
    cfg = N.Config()
    N.lib().fr_config_defaults(C.byref(cfg))
    assert cfg.shadow_mode == N.FR_SHADOW_PCSS
    assert (cfg.pcf_samples, cfg.blocker_samples, cfg.ssao_samples) == (64, 32, 32)
    assert abs(cfg.ssao_radius - 0.075) < 1e-7 and abs(cfg.ssao_bias - 0.0005) < 1e-9
    assert cfg.shadow_size == 0 and cfg.blur_mode == N.FR_BLUR_REFERENCE
    # the library's own switches: concurrent passes and per-pass timing events on
    assert (cfg.concurrent_passes, cfg.pass_timings) == (1, 1)


def test_config_struct_ends_where_the_header_says():
    """The ctypes mirror of fr_config has the header's size: fr_config_defaults
    writes exactly its fields (a trailing guard word stays untouched)."""
    class Guarded(C.Structure):
        _fields_ = [("cfg", N.Config), ("guard", C.c_uint32 * 4)]

    g = Guarded()
    for i in range(4):
        g.guard[i] = 0xA5A5A5A5
    N.lib().fr_config_defaults(C.byref(g.cfg))
    assert list(g.guard) == [0xA5A5A5A5] * 4
    assert g.cfg.pass_timings == 1


def test_create_without_gpu_fails_cleanly():
    import conftest

    if conftest.gpu_available():
        pytest.skip("a GPU is present")
    err = C.create_string_buffer(256)
    h = N.lib().fr_create(None, err, 256)
    assert not h
    assert re.search(r"CUDA|device", err.value.decode())


def test_noalloc_blur_rejects_bad_arguments_before_any_cuda_call():
    """fr_blur_separable_noalloc refuses a null buffer, a non-positive size and a
    size beyond its fixed scratch array before it makes any CUDA call, so these
    run without a GPU; the pointer is a dummy that nothing dereferences."""
    f = N.lib().fr_blur_separable_noalloc
    dummy = C.c_void_p(0x1000)
    side = 1 << 11  # 2048 x 2049 > 4 Mi pixels
    assert f(dummy, side, side + 1, None) == N.FR_ERR_INVALID
    assert f(dummy, N.FR_NOALLOC_BLUR_MAX_PIXELS + 1, 1, None) == N.FR_ERR_INVALID
    assert f(dummy, 1 << 16, 1 << 16, None) == N.FR_ERR_INVALID  # product beyond 32 bits
    assert f(None, 8, 8, None) == N.FR_ERR_INVALID
    assert f(dummy, 0, 8, None) == N.FR_ERR_INVALID
    assert f(dummy, 8, -1, None) == N.FR_ERR_INVALID
