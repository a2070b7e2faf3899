"""The reference-side drop-in (integration/render_gpu.cpp).

The shim implements the reference's namespace Render (src/render.h:20-37) over
the C ABI: the reference's in-memory Scene becomes an fr_scene_view
(fr_scene_from_view), the frame runs on the GPU, and the results land in the
reference's ForkerGL:: buffers, so the reference's own main.cpp and Output
module (src/main.cpp:18-55, src/output.cpp:12-86) run unchanged on top of it.

* CPU, where the reference tree is present: oracle/Makefile.ref links the shim
  with the reference's unchanged main / output / scene code into
  oracle/_ref/ref_main_gpu; without a GPU the binary loads the scene, marshals
  it and stops at fr_create with a clear message; with a GPU its ten output
  files are checked against the reference's.
* GPU: the shim's sequence of C calls driven from here (scene view ->
  fr_scene_from_view -> fr_create with keep_float_frame -> fr_upload_scene ->
  fr_render_frame -> fr_download in the reference's Buffer layouts), its
  buffers written as the reference's Output module writes them, against the
  reference's file digests (bit-exact buffers) and frame (within 1 LSB)."""

import ctypes as C
import hashlib
import os
import shutil
import subprocess

import pytest

import golden_utils as G
import oracle_bridge as OB
import scenes
import tga_util as T
from conftest import gpu_available
from forkerrenderer_gb300 import Renderer, Scene
from forkerrenderer_gb300 import _native as N

# files whose source buffers are bit-exact with the reference's
BITEXACT_FILES = {"shadowmap.tga", "zbuffer.tga", "gbuffer_normal.tga", "gbuffer_worldpos.tga",
                  "gbuffer_albedo.tga", "gbuffer_param.tga", "gbuffer_shading_type.tga"}
CASES = ["def_pcss", "fwd_pcss", "def_pcf_ssaa"]


def _check_files(name, files: dict):
    meta, arrays = G.load(name)
    assert sorted(files) == sorted(meta["tga"]), "the set of files differs from the reference's"
    for fn, data in files.items():
        if fn in BITEXACT_FILES:
            assert hashlib.sha256(data).hexdigest() == meta["tga"][fn]["sha256"], (name, fn)
    px, _ = T.decode(files["framebuffer.tga"])
    want = OB.oracle_tga(T.reference_image("frame8", "rgb", {"frame8": arrays["frame8"]}))
    G.check_frame8(px, T.decode(want)[0])


@pytest.mark.parametrize("binary", ["ref_main_gpu", "ref_main_gpu_out"])
@pytest.mark.parametrize("name", CASES)
def test_shim_links_with_the_reference_application(name, binary, tmp_path):
    """ref_main_gpu: render_gpu.cpp in place of render.cpp; ref_main_gpu_out: also
    output_gpu.cpp in place of output.cpp (files encoded on the GPU)."""
    shim = os.path.join(OB.REF_DIR, binary)
    if not os.path.exists(shim):
        pytest.skip("reference tree not present: the shim is built only where it is")
    scene_dir = os.path.dirname(scenes.scene_path(name))
    work = tmp_path / "scene"
    shutil.copytree(scene_dir, work)
    (work / "output").mkdir(exist_ok=True)
    # the reference resolves model paths against the working directory
    r = subprocess.run([shim, "scene.scene"], cwd=work, capture_output=True, text=True, timeout=600)
    if not gpu_available():
        assert r.returncode == 1 and "[render_gpu] fr_create" in r.stderr, (r.returncode, r.stderr[-400:])
        return
    assert r.returncode == 0, r.stderr[-2000:]
    files = {}
    for fn in os.listdir(work / "output"):
        with open(work / "output" / fn, "rb") as f:
            files[fn] = f.read()
    _check_files(name, files)


def _shim_sequence(name):
    """The C calls of integration/render_gpu.cpp for one frame, from here."""
    src = Scene(scenes.scene_path(name))
    view = src.view()
    err = C.create_string_buffer(512)
    h = N.lib().fr_scene_from_view(C.byref(view), err, len(err))
    assert h, err.value
    cfg = scenes.render_config(name)
    r = Renderer(keep_float_frame=1, **cfg)
    rc = N.lib().fr_upload_scene(r.handle, C.c_void_p(h))
    assert rc == 0, N.lib().fr_last_error(r.handle)
    info = src.info
    r.scene = src  # shapes of the downloads
    r.Render()
    bufs = {"frame": r.frame(), "depth": r.depth()}
    if info.shadow_on:
        bufs["shadow"] = r.shadow_map()
    if info.deferred:
        for g, key in (("normal", "gb_normal"), ("position", "gb_position"), ("albedo", "gb_albedo"),
                       ("param", "gb_param"), ("type", "gb_type")):
            bufs[key] = r.gbuffer(g)
        bufs["ao"] = r.ambient_occlusion()
    if info.ssaa_on:
        bufs["ssaa8"] = r.ssaa8()
    r.close()
    N.lib().fr_scene_free(C.c_void_p(h))
    return bufs


@pytest.mark.gpu
@pytest.mark.parametrize("name", CASES)
def test_shim_call_sequence_writes_the_reference_files(name):
    if not gpu_available():
        pytest.skip("no CUDA GPU")
    bufs = _shim_sequence(name)
    meta, _ = G.load(name)
    files = {}
    for fn, key, kind in T.OUTPUTS:
        # Output::Output* of the ForkerGL buffers the shim fills (the oracle's restatement
        # of GenerateImage + WriteTgaFile); the frame is the float FrameBuffer
        if key == "frame8":
            files[fn] = OB.oracle_tga(OB.oracle_image(bufs["frame"]))
        elif key in bufs:
            files[fn] = OB.oracle_tga(T.reference_image(key, kind, bufs))
    _check_files(name, files)
