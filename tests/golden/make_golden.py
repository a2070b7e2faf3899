"""Generates the golden fixtures of tests/golden/ from the reference itself.

For every case of tests/scenes.py it writes the seeded scene, renders it with
the reference renderer's own code (oracle/_ref/ref_* built from the reference
sources by oracle/Makefile.ref) and stores:
  * the SHA-256 of the generated scene files (to detect generator drift),
  * the frame matrices the reference used (hex-exact),
  * SHA-256 digests of every float buffer that must match bit for bit
    (depth, shadow map, the seven G-buffers, float frame),
  * the ambient-occlusion buffer and the 8-bit frame / SSAA image themselves
    (compared with tolerances, since powf differs between C libraries).

Run here, where the reference tree exists:
    python tests/golden/make_golden.py
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


def main() -> None:
    from forkerrenderer_gb300.build import build_reference

    if build_reference() is None:
        raise SystemExit("reference tree not found; golden fixtures can only be made where it exists")
    for name, (_, _, variant, _) in scenes.CASES.items():
        path = scenes.scene_path(name)
        cfg = scenes.render_config(name)
        with tempfile.TemporaryDirectory() as out:
            ref = OB.run_reference(path, out, variant, cfg["shadow_size"], cfg["pcf_samples"],
                                   cfg["blocker_samples"])
        meta = {
            "case": name,
            "variant": variant,
            "config": cfg,
            "scene_digest": scenes.files_digest(name),
            "info": ref["info"],
            "matrices": {k: [float(x).hex() for x in v.ravel()] for k, v in ref["matrices"].items()},
            "sha256": {k: sha(ref[k]) for k in BITEXACT if ref.get(k) is not None},
            "shapes": {k: list(ref[k].shape) for k in BITEXACT if ref.get(k) is not None},
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


if __name__ == "__main__":
    main()
