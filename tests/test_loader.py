"""Scene ingest (fr_scene_load) follows the reference loader's rules and
reports the inputs on which the reference would crash as errors."""

import os

import numpy as np
import pytest

import scenes
from forkerrenderer_gb300 import RenderError, Scene, scenegen


def _write(d, name, text):
    p = os.path.join(d, name)
    with open(p, "w") as f:
        f.write(text)
    return p


BASE_SCENE = "mode deferred\nscreen 64 40\nlight point 2 5 5 1 1 1\ncamera persp -1 1 1 0 0 -1\n"


def _scene(tmp_path, obj_text, mtl_text="newmtl M\nKd 0.5 0.5 0.5\n", extra=""):
    d = str(tmp_path)
    _write(d, "m.mtl", mtl_text)
    _write(d, "m.obj", obj_text)
    return _write(d, "s.scene", BASE_SCENE + extra + "model m.obj false false 0 0 0 0 1\n")


TRI = "mtllib m.mtl\nv 0 0 0\nv 1 0 0\nv 0 1 0\nvt 0 0\nvn 0 0 1\n"


def test_defaults_and_counts(tmp_path):
    p = _scene(tmp_path, TRI + "g A\nusemtl M\nf 1/1/1 2/1/1 3/1/1\n")
    s = Scene(p)
    i = s.info
    assert (i.width, i.height, i.deferred, i.shadow_on, i.ssao_on, i.ssaa_on) == (64, 40, 1, 1, 0, 0)
    assert (i.num_models, i.num_meshes, i.num_triangles, i.num_vertices) == (1, 1, 1, 3)


def test_fan_triangulation(tmp_path):
    obj = TRI + "v 1 1 0\ng A\nusemtl M\nf 1/1/1 2/1/1 4/1/1 3/1/1\n"
    s = Scene(_scene(tmp_path, obj))
    assert s.info.num_triangles == 2


def test_mesh_order_is_name_order_and_regroup_restarts(tmp_path):
    obj = TRI + ("g Zed\nusemtl M\nf 1/1/1 2/1/1 3/1/1\n"
                 "g Alpha\nusemtl M\nf 1/1/1 2/1/1 3/1/1\nf 1/1/1 2/1/1 3/1/1\n"
                 "g Zed\nusemtl M\nf 3/1/1 2/1/1 1/1/1\n")
    s = Scene(_scene(tmp_path, obj))
    v = s.view()
    import ctypes as C
    tri_v = np.ctypeslib.as_array(C.cast(v.tri_v, C.POINTER(C.c_int32)), shape=(3 * v.info.num_triangles,))
    # Alpha (2 faces) first, then the restarted Zed (1 face, reversed winding)
    assert v.info.num_triangles == 3
    assert list(tri_v[6:9]) == [2, 1, 0]


@pytest.mark.parametrize("obj,msg", [
    (TRI + "f 1/1/1 2/1/1 3/1/1\n", "face before any g"),
    (TRI + "g A\nusemtl Nope\nf 1/1/1 2/1/1 3/1/1\n", "unknown material"),
    (TRI + "g A\nusemtl M\nf 1/1/1 2/1/1 9/1/1\n", "out of range"),
])
def test_inputs_the_reference_crashes_on_are_errors(tmp_path, obj, msg):
    with pytest.raises(RenderError, match=msg):
        Scene(_scene(tmp_path, obj))


def test_missing_files(tmp_path):
    with pytest.raises(RenderError, match="cannot open scene"):
        Scene(str(tmp_path / "nope.scene"))
    p = _write(str(tmp_path), "s.scene", BASE_SCENE + "model missing.obj false false 0 0 0 0 1\n")
    with pytest.raises(RenderError, match="cannot open model"):
        Scene(p)


def test_scene_without_camera_is_an_error(tmp_path):
    p = _write(str(tmp_path), "s.scene", "screen 4 4\nlight point 1 1 1 1 1 1\n")
    with pytest.raises(RenderError, match="camera"):
        Scene(p)


def test_pbr_flag_comes_from_the_last_mesh_in_name_order(tmp_path):
    scenegen.write_tga(str(tmp_path / "r.tga"), np.zeros((2, 2), np.uint8))
    mtl = "newmtl P\nKd 1 1 1\nmap_Pr r.tga\nnewmtl Q\nKd 1 1 1\n"
    obj = TRI + "g A\nusemtl P\nf 1/1/1 2/1/1 3/1/1\ng B\nusemtl Q\nf 1/1/1 2/1/1 3/1/1\n"
    import ctypes as C
    from forkerrenderer_gb300 import _native as N

    class ModelView(C.Structure):
        _fields_ = [("model_matrix", C.c_float * 16), ("position", C.c_float * 3),
                    ("rotate_y", C.c_float), ("scale", C.c_float), ("has_tangents", C.c_int32),
                    ("support_pbr", C.c_int32), ("first_mesh", C.c_int32), ("num_meshes", C.c_int32),
                    ("first_vertex", C.c_int64), ("num_vertices", C.c_int64),
                    ("first_normal", C.c_int64), ("num_normals", C.c_int64)]

    s = Scene(_scene(tmp_path, obj, mtl))
    mv = C.cast(s.view().models, C.POINTER(ModelView))[0]
    assert mv.support_pbr == 0  # "B" (no PBR maps) is last
    s2 = Scene(_scene(tmp_path, obj.replace("usemtl Q", "usemtl P"), mtl))
    assert C.cast(s2.view().models, C.POINTER(ModelView))[0].support_pbr == 1


def test_rle_and_uncompressed_tga_give_the_same_texels(tmp_path):
    """A run-length encoded TGA (types 10/11) decodes to the same bytes."""
    from forkerrenderer_gb300 import _native as N  # noqa: F401
    img = np.zeros((4, 6, 3), np.uint8)
    img[1:3, 2:5] = (10, 20, 30)
    scenegen.write_tga(str(tmp_path / "raw.tga"), img)
    # hand-made RLE: each row = run of 6 pixels or raw packets
    hdr = bytearray(18)
    hdr[2] = 10
    hdr[12], hdr[14], hdr[16], hdr[17] = 6, 4, 24, 0
    body = bytearray()
    for y in range(4):
        row = img[y, :, ::-1]
        body += bytes([5 | 0x00]) + row.tobytes()  # raw packet of 6 pixels
    (tmp_path / "rle.tga").write_bytes(bytes(hdr) + bytes(body))
    texts = []
    for t in ("raw.tga", "rle.tga"):
        mtl = f"newmtl M\nKd 1 1 1\nmap_Kd {t}\n"
        s = Scene(_scene(tmp_path, TRI + "g A\nusemtl M\nf 1/1/1 2/1/1 3/1/1\n", mtl))
        import ctypes as C

        class TexView(C.Structure):
            _fields_ = [("width", C.c_int32), ("height", C.c_int32), ("bpp", C.c_int32),
                        ("data", C.POINTER(C.c_uint8))]
        tv = C.cast(s.view().textures, C.POINTER(TexView))[0]
        texts.append(bytes(tv.data[: tv.width * tv.height * tv.bpp]))
    assert texts[0] == texts[1]


class _MatView:
    @staticmethod
    def cls():
        import ctypes as C

        class MaterialView(C.Structure):
            _fields_ = [("ka", C.c_float * 3), ("kd", C.c_float * 3), ("ks", C.c_float * 3), ("ke", C.c_float * 3),
                        ("pbr_albedo", C.c_float * 3), ("roughness", C.c_float), ("metalness", C.c_float),
                        ("map_kd", C.c_int32), ("map_ks", C.c_int32), ("map_ke", C.c_int32),
                        ("map_bump", C.c_int32), ("map_ao", C.c_int32), ("map_pr", C.c_int32),
                        ("map_pm", C.c_int32)]

        return MaterialView


def _materials(s):
    import ctypes as C

    n = s.info.num_materials
    return list(C.cast(s.view().materials, C.POINTER(_MatView.cls()))[:n])


def test_texture_indices_follow_first_use_across_models(tmp_path):
    """Models parse in parallel but join in scene order: textures are numbered by
    first use (model by model, line by line), a texture that fails to load leaves
    its slots at -1 without taking a number, and the PBR flag sees the final slots."""
    d = str(tmp_path)
    for name, v in (("a.tga", 10), ("b.tga", 20), ("c.tga", 30)):
        scenegen.write_tga(os.path.join(d, name), np.full((2, 2), v, np.uint8))
    _write(d, "m1.mtl", "newmtl M1\nKd 1 1 1\nmap_Kd b.tga\nmap_Ks missing.tga\nmap_Pr missing.tga\n")
    _write(d, "m2.mtl", "newmtl M2\nKd 1 1 1\nmap_Kd a.tga\nmap_Ke b.tga\nmap_Pm c.tga\n")
    for i in (1, 2):
        _write(d, f"m{i}.obj", TRI.replace("m.mtl", f"m{i}.mtl") + f"g A\nusemtl M{i}\nf 1/1/1 2/1/1 3/1/1\n")
    p = _write(d, "s.scene", BASE_SCENE + "model m1.obj false false 0 0 0 0 1\nmodel m2.obj false false 0 0 0 0 1\n")
    for _ in range(3):  # the same numbering every time
        s = Scene(p)
        assert s.info.num_textures == 3
        m1, m2 = _materials(s)
        assert (m1.map_kd, m1.map_ks, m1.map_pr) == (0, -1, -1)  # b first, missing.tga never numbered
        assert (m2.map_kd, m2.map_ke, m2.map_pm) == (1, 0, 2)     # then a, b again, c
        import ctypes as C

        class TexView(C.Structure):
            _fields_ = [("width", C.c_int32), ("height", C.c_int32), ("bpp", C.c_int32),
                        ("data", C.POINTER(C.c_uint8))]

        tv = C.cast(s.view().textures, C.POINTER(TexView))
        assert [tv[i].data[0] for i in range(3)] == [20, 10, 30]


def test_repeated_newmtl_starts_the_material_again(tmp_path):
    """A second newmtl of a name starts that material again: the first one's maps
    are dropped from it, but their textures still load (and take their numbers)."""
    d = str(tmp_path)
    scenegen.write_tga(os.path.join(d, "a.tga"), np.zeros((2, 2), np.uint8))
    scenegen.write_tga(os.path.join(d, "b.tga"), np.zeros((2, 2), np.uint8))
    mtl = "newmtl M\nKd 1 1 1\nmap_Kd a.tga\nnewmtl M\nKd 0.5 0.5 0.5\nmap_Ks b.tga\n"
    s = Scene(_scene(tmp_path, TRI + "g A\nusemtl M\nf 1/1/1 2/1/1 3/1/1\n", mtl))
    assert s.info.num_textures == 2
    (m,) = _materials(s)
    assert (m.map_kd, m.map_ks) == (-1, 1)
    assert list(m.kd) == [0.5, 0.5, 0.5]


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["def_pcss", "def_stress"])
def test_device_tangents_equal_host_tangents(name):
    """Model::generateTangents on the device at upload (per-vertex sums in the
    reference's face order) equals the host's sequential loop bit for bit; models
    without the flag keep zero tangents."""
    from conftest import gpu_available

    if not gpu_available():
        pytest.skip("no CUDA GPU")
    import ctypes as C

    import scenes
    from forkerrenderer_gb300 import Renderer, Scene

    scene = Scene(scenes.scene_path(name))
    r = Renderer(**scenes.render_config(name))
    r.Preconfigure(scene)  # device generation, before any host reader asked for them
    dev = r.scene_tangents()
    v = scene.view()  # host generation
    host = np.ctypeslib.as_array(C.cast(v.tangents, C.POINTER(C.c_float)), (v.info.num_vertices * 3,))
    assert dev.shape == (v.info.num_vertices, 3)
    assert np.array_equal(dev.reshape(-1).view(np.uint32), host.view(np.uint32))
    r.close()


@pytest.mark.parametrize("damage", ["truncated", "bad_type", "empty"])
def test_unreadable_texture_leaves_the_slot_empty(tmp_path, damage):
    """A texture file TGAImage::ReadTgaFile rejects (tgaimage.cpp:43-107: data cut
    short, an unsupported image type, an empty file) is skipped as the reference's
    loadTexture skips it: the slot stays -1, the texture takes no number, and the
    scene still loads."""
    d = str(tmp_path)
    scenegen.write_tga(os.path.join(d, "ok.tga"), np.full((4, 4, 3), 9, np.uint8))
    scenegen.write_tga(os.path.join(d, "bad.tga"), np.full((4, 4, 3), 7, np.uint8))
    raw = open(os.path.join(d, "bad.tga"), "rb").read()
    if damage == "truncated":
        raw = raw[: 18 + 10]
    elif damage == "bad_type":
        raw = raw[:2] + bytes([5]) + raw[3:]
    else:
        raw = b""
    with open(os.path.join(d, "bad.tga"), "wb") as f:
        f.write(raw)
    mtl = "newmtl M\nKd 1 1 1\nmap_Kd bad.tga\nmap_Ks ok.tga\n"
    s = Scene(_scene(tmp_path, TRI + "g A\nusemtl M\nf 1/1/1 2/1/1 3/1/1\n", mtl))
    assert s.info.num_textures == 1
    (m,) = _materials(s)
    assert (m.map_kd, m.map_ks) == (-1, 0)


@pytest.mark.parametrize("obj,msg", [
    (TRI + "g A\nusemtl M\nf 1 2 3\n", "without v/t/n"),            # no v/t/n triple at all
    (TRI + "g A\nusemtl M\nf 1/1/1 2/1/1 3/7/1\n", "out of range"),  # uv index past the end
])
def test_malformed_faces_are_errors(tmp_path, obj, msg):
    """Face lines on which the reference reads past its arrays (model.cpp:228-234:
    with no v/t/n triple its loop bound vertices.size() - 1 wraps around) are
    reported instead."""
    with pytest.raises(RenderError, match=msg):
        Scene(_scene(tmp_path, obj))


def test_face_of_two_corners_adds_no_triangle(tmp_path):
    """Two corners: the reference's fan loop runs zero times (model.cpp:233)."""
    s = Scene(_scene(tmp_path, TRI + "g A\nusemtl M\nf 1/1/1 2/1/1\nf 1/1/1 2/1/1 3/1/1\n"))
    assert s.info.num_triangles == 1


def _from_view(view):
    import ctypes as C

    from forkerrenderer_gb300 import _native as N

    err = C.create_string_buffer(512)
    h = N.lib().fr_scene_from_view(C.byref(view), err, len(err))
    return h, err.value.decode()


def _arrays(view):
    import ctypes as C

    import numpy as np

    I = view.info
    def arr(ptr, n, t):
        return np.ctypeslib.as_array(C.cast(ptr, C.POINTER(t)), (n,)).copy() if n else np.zeros(0)
    out = {"positions": arr(view.positions, 3 * I.num_vertices, C.c_float),
           "uvs": arr(view.uvs, 2 * I.num_uvs, C.c_float),
           "normals": arr(view.normals, 3 * I.num_normals, C.c_float),
           "tangents": arr(view.tangents, 3 * I.num_vertices, C.c_float)}
    for k in ("tri_v", "tri_vt", "tri_vn"):
        out[k] = arr(getattr(view, k), 3 * I.num_triangles, C.c_int32)
    out["tri_mesh"] = arr(view.tri_mesh, I.num_triangles, C.c_int32)
    return out


@pytest.mark.parametrize("with_tangents", [True, False])
def test_scene_from_view_rebuilds_the_same_scene(with_tangents):
    """fr_scene_from_view (how a host holding the reference's Scene hands it over)
    rebuilds the loaded scene: same arrays, records, textures and frame matrices;
    without tangents it generates them from the faces as the loader does."""
    import ctypes as C

    import numpy as np

    from forkerrenderer_gb300 import _native as N
    from forkerrenderer_gb300 import Scene

    src = Scene(scenes.scene_path("def_pcss"))
    v = src.view()
    if not with_tangents:
        v.tangents = None
    h, msg = _from_view(v)
    assert h, msg
    try:
        v2 = N.SceneView()
        assert N.lib().fr_scene_get_view(C.c_void_p(h), C.byref(v2)) == 0
        a, b = _arrays(src.view()), _arrays(v2)
        for k in a:
            assert np.array_equal(a[k].view(np.uint32) if a[k].dtype == np.float32 else a[k],
                                  b[k].view(np.uint32) if b[k].dtype == np.float32 else b[k]), k
        I = src.info
        v1 = src.view()
        for field, T, n in (("models", N.ModelView, I.num_models), ("meshes", N.MeshView, I.num_meshes),
                            ("materials", N.MaterialView, I.num_materials)):
            assert C.string_at(getattr(v1, field), C.sizeof(T) * n) == C.string_at(getattr(v2, field), C.sizeof(T) * n)
        tx1 = C.cast(v1.textures, C.POINTER(N.TextureView))
        tx2 = C.cast(v2.textures, C.POINTER(N.TextureView))
        for i in range(I.num_textures):
            t1, t2 = tx1[i], tx2[i]
            n = t1.width * t1.height * t1.bytes_per_pixel
            assert (t1.width, t1.height, t1.bytes_per_pixel) == (t2.width, t2.height, t2.bytes_per_pixel)
            assert C.string_at(t1.data, n) == C.string_at(t2.data, n)
        m1, m2 = N.FrameMatrices(), N.FrameMatrices()
        N.lib().fr_scene_frame_matrices(src.handle, 256, C.byref(m1))
        N.lib().fr_scene_frame_matrices(C.c_void_p(h), 256, C.byref(m2))
        assert bytes(m1) == bytes(m2)
    finally:
        N.lib().fr_scene_free(C.c_void_p(h))


def test_scene_from_view_rejects_bad_indices():
    from forkerrenderer_gb300 import Scene

    src = Scene(scenes.scene_path("def_pcss"))
    v = src.view()
    import ctypes as C

    import numpy as np

    tri = np.ctypeslib.as_array(C.cast(v.tri_v, C.POINTER(C.c_int32)), (3 * v.info.num_triangles,)).copy()
    tri[7] = v.info.num_vertices  # one past the end
    v.tri_v = tri.ctypes.data
    h, msg = _from_view(v)
    assert not h and "out of range" in msg
    v = src.view()
    v.info.num_textures = -1
    h, msg = _from_view(v)
    assert not h and "count" in msg
