"""Generates the golden fixtures of tests/golden/ from the reference itself.

For every case of tests/scenes.py it writes the seeded scene, renders it with
the reference renderer's own code (oracle/_ref/ref_* built from the reference
sources by oracle/Makefile.ref) and stores:
  * the SHA-256 of the generated scene files (to detect generator drift),
  * the frame matrices the reference used (hex-exact),
  * SHA-256 digests of every float buffer that must match bit for bit
    (depth, shadow map, the seven G-buffers, float frame),
  * the ambient-occlusion buffer and the 8-bit frame / SSAA image themselves
    (compared with tolerances, since powf differs between C libraries),
  * SHA-256 and size of every TGA file the reference's Output module writes
    (src/output.cpp, run by oracle/ref_harness.cpp --tga 1).
It also writes wrap_modes.json (def_wrap rendered by the reference with each
texture wrap mode), filter_linear.json / .npz (the same with bilinear filtering,
plus the forward-shaded fwd_wrap) and tga_edge.npz: crafted images (runs and raw stretches around the
128-pixel packet limit, 1/3/4 bytes per pixel, empty and one-pixel images)
with the bytes the reference's own TGA writer produces for them (oracle/_ref/ref_tga).

Run here, where the reference tree exists:
    python tests/golden/make_golden.py [case ...]
(with case names: only those cases' fixtures are rewritten).
"""

from __future__ import annotations

import hashlib
import json
import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
TESTS = os.path.dirname(HERE)
ROOT = os.path.dirname(TESTS)
sys.path[:0] = [ROOT, TESTS]

import oracle_bridge as OB  # noqa: E402
import scenes  # noqa: E402

BITEXACT = ["depth", "shadow", "gb_normal", "gb_position", "gb_lightndc", "gb_albedo", "gb_emissive",
            "gb_param", "gb_type", "frame"]


def sha(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def main(names: list[str] | None = None) -> None:
    """Every fixture, or (names given) only those cases of tests/scenes.py."""
    from forkerrenderer_gb300.build import build_reference

    if build_reference() is None:
        raise SystemExit("reference tree not found; golden fixtures can only be made where it exists")
    for name, (_, _, variant, _) in scenes.CASES.items():
        if names and name not in names:
            continue
        path = scenes.scene_path(name)
        cfg = scenes.render_config(name)
        with tempfile.TemporaryDirectory() as out:
            ref = OB.run_reference(path, out, variant, cfg["shadow_size"], cfg["pcf_samples"],
                                   cfg["blocker_samples"], tga=True)
        meta = {
            "case": name,
            "variant": variant,
            "config": cfg,
            "scene_digest": scenes.files_digest(name),
            "info": ref["info"],
            "matrices": {k: [float(x).hex() for x in v.ravel()] for k, v in ref["matrices"].items()},
            "sha256": {k: sha(ref[k]) for k in BITEXACT if ref.get(k) is not None},
            "shapes": {k: list(ref[k].shape) for k in BITEXACT if ref.get(k) is not None},
            "tga": {fn: {"sha256": hashlib.sha256(b).hexdigest(), "bytes": len(b)} for fn, b in ref["tga"].items()},
        }
        arrays = {"frame8": ref["frame8"]}
        if ref.get("ao") is not None:
            arrays["ao"] = ref["ao"]
        if ref.get("ssaa8") is not None:
            arrays["ssaa8"] = ref["ssaa8"]
        np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **arrays)
        with open(os.path.join(HERE, f"{name}.json"), "w") as f:
            json.dump(meta, f, indent=1, sort_keys=True)
        print(name, "ok", {k: v[:12] for k, v in meta["sha256"].items()})
    if names:
        return
    tga_edge()
    wrap_golden()
    filter_golden()


WRAP_BUFFERS = ["gb_albedo", "gb_param", "gb_normal", "depth"]


def wrap_golden() -> None:
    """def_wrap rendered by the reference with each Texture::WrapMode (its textures
    created after ForkerGL::TextureWrapMode(mode)): digests of the buffers that
    sample textures (albedo, param, the normal map's normals) and the depth."""
    name = "def_wrap"
    cfg = scenes.render_config(name)
    meta = {"case": name, "scene_digest": scenes.files_digest(name), "modes": {}}
    for mode in range(4):
        with tempfile.TemporaryDirectory() as out:
            ref = OB.run_reference(scenes.scene_path(name), out, scenes.EXTRA_CASES[name][2], cfg["shadow_size"],
                                   cfg["pcf_samples"], cfg["blocker_samples"], wrap=mode)
        meta["modes"][str(mode)] = {k: sha(ref[k]) for k in WRAP_BUFFERS}
    distinct = len({v["gb_albedo"] for v in meta["modes"].values()})
    assert distinct == 4, "every wrap mode must change the ground's albedo"
    with open(os.path.join(HERE, "wrap_modes.json"), "w") as f:
        json.dump(meta, f, indent=1, sort_keys=True)
    print("wrap_modes ok")


def filter_golden() -> None:
    """Bilinear filtering (ForkerGL::TextureFilterMode(Linear) before the scene
    loads) with each wrap mode: digests of def_wrap's texture-sampled buffers, and
    the reference's 8-bit frames of def_wrap (deferred: the lighting pass reads
    the sampled G-buffer) and fwd_wrap (forward: sampled in the fragment shader)
    with Repeat, for the 1-LSB frame comparison."""
    meta = {"scene_digest": {}, "modes": {}}
    frames = {}
    for name in ("def_wrap", "fwd_wrap"):
        cfg = scenes.render_config(name)
        meta["scene_digest"][name] = scenes.files_digest(name)
        for mode in range(4) if name == "def_wrap" else (1,):
            with tempfile.TemporaryDirectory() as out:
                ref = OB.run_reference(scenes.scene_path(name), out, scenes.EXTRA_CASES[name][2],
                                       cfg["shadow_size"], cfg["pcf_samples"], cfg["blocker_samples"],
                                       wrap=mode, filt=1)
            if name == "def_wrap":
                meta["modes"][str(mode)] = {k: sha(ref[k]) for k in WRAP_BUFFERS}
            if mode == 1:
                frames[f"{name}_frame8"] = ref["frame8"]
    with open(os.path.join(HERE, "wrap_modes.json")) as f:
        nearest = json.load(f)["modes"]
    for mode, d in meta["modes"].items():
        assert d["gb_albedo"] != nearest[mode]["gb_albedo"], "bilinear must change the sampled albedo"
        assert d["depth"] == nearest[mode]["depth"]
    with open(os.path.join(HERE, "filter_linear.json"), "w") as f:
        json.dump(meta, f, indent=1, sort_keys=True)
    np.savez_compressed(os.path.join(HERE, "filter_linear.npz"), **frames)
    print("filter_linear ok")


def edge_images() -> list[np.ndarray]:
    """Seeded images that exercise every branch of the RLE packer."""
    rng = np.random.default_rng(20240611)
    imgs = [np.zeros((0, 0), np.uint8), np.zeros((1, 1), np.uint8), np.full((1, 2, 3), 7, np.uint8),
            np.arange(2, dtype=np.uint8).reshape(1, 2)]
    for bpp in (1, 3, 4):
        for lengths in ([126, 127, 128, 129, 130, 1, 2, 255, 256, 257, 1, 1, 3],
                        [127, 2, 1, 128, 1, 129, 1, 1],
                        [1] * 127 + [2] + [1] * 128 + [3] + [1] * 129 + [2, 2]):
            vals = []
            for i, n in enumerate(lengths):
                v = rng.integers(0, 256, bpp).astype(np.uint8)
                vals += [v] * n
            a = np.array(vals, np.uint8)
            imgs.append(a.reshape(1, len(vals), bpp) if bpp > 1 else a.reshape(1, len(vals)))
        for h, w in ((7, 33), (16, 131), (3, 300)):
            a = rng.integers(0, 2, (h, w, bpp)).astype(np.uint8)  # many short runs
            imgs.append(a if bpp > 1 else a[..., 0])
        a = rng.integers(0, 256, (5, 200, bpp)).astype(np.uint8)  # raw stretches only
        imgs.append(a if bpp > 1 else a[..., 0])
    return imgs


def tga_edge() -> None:
    arrays = {}
    for i, img in enumerate(edge_images()):
        arrays[f"img{i}"] = img
        for rle in (0, 1):
            arrays[f"tga{i}_rle{rle}"] = np.frombuffer(OB.reference_tga(img, bool(rle)), np.uint8)
    np.savez_compressed(os.path.join(HERE, "tga_edge.npz"), **arrays)
    print("tga_edge ok", len(arrays) // 3, "images")


if __name__ == "__main__":
    main(sys.argv[1:] or None)
