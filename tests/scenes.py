"""Seeded test scenes (regenerated byte-identically from their parameters)."""

from __future__ import annotations

import hashlib
import os
import tempfile

from forkerrenderer_gb300 import scenegen

# name -> (generator, kwargs, reference harness variant, render config overrides)
CASES = {
    "fwd_hard": ("forward", dict(seed=1, width=160, height=100, lon=32, lat=16, tex=64),
                 "ref_hard", dict(shadow_mode=0)),
    "fwd_pcss": ("forward", dict(seed=1, width=160, height=100, lon=32, lat=16, tex=64),
                 "ref_pcss_tab", dict(shadow_mode=2)),
    "def_pcss": ("field", dict(seed=2, n_spheres=4, subdiv=2, tex=64, width=160, height=100),
                 "ref_pcss_tab", dict(shadow_mode=2)),
    "def_pcss_s256": ("field", dict(seed=2, n_spheres=4, subdiv=2, tex=64, width=160, height=100),
                      "ref_pcss_tab", dict(shadow_mode=2, shadow_size=256, pcf_samples=25,
                                           blocker_samples=16)),
    "def_pcf_ssaa": ("field", dict(seed=3, n_spheres=3, subdiv=2, tex=64, width=96, height=60,
                                   ssaa=2), "ref_pcf_tab", dict(shadow_mode=1)),
    "def_phong_hard": ("field", dict(seed=4, n_spheres=3, subdiv=2, tex=64, width=160, height=100,
                                     pbr=False), "ref_hard", dict(shadow_mode=0)),
    "fwd_pbr_pcss": ("field", dict(seed=5, n_spheres=3, subdiv=2, tex=64, width=160, height=100,
                                   deferred=False), "ref_pcss_tab", dict(shadow_mode=2)),
    "def_stress": ("stress", dict(seed=7), "ref_pcss_tab", dict(shadow_mode=2)),
    # odd sizes (tiles, blur lines and SSAA cut at ragged edges), SSAO off
    "def_nossao_odd": ("field", dict(seed=9, n_spheres=3, subdiv=2, tex=64, width=161, height=97, ssao=False),
                       "ref_pcss_tab", dict(shadow_mode=2)),
    # forward, shadow off (deferred with shadow off crashes the reference: its lighting pass
    # reads the light-space G-buffer it never allocated), 3x3 SSAA
    "fwd_ssaa3_noshadow": ("field", dict(seed=10, n_spheres=3, subdiv=2, tex=64, width=64, height=40, ssaa=3,
                                         deferred=False, shadow=False), "ref_pcf_tab", dict(shadow_mode=1)),
    "def_ssaa3_odd": ("field", dict(seed=12, n_spheres=3, subdiv=2, tex=64, width=75, height=53, ssaa=3),
                      "ref_pcss_tab", dict(shadow_mode=2)),
    "fwd_stress": ("stress", dict(seed=8, deferred=False), "ref_pcf_tab", dict(shadow_mode=1)),
    # The plain forward Blinn-Phong workload at full size: 64 x 32 UV sphere (4,032 faces) on
    # the 6 x 6 plane, 256^2 checker, 640 x 400, hard shadow in a 1024^2 map, SSAA off.
    "c0_fwd_hard_640x400": ("forward", dict(seed=0, width=640, height=400, lon=64, lat=32, tex=256),
                            "ref_hard", dict(shadow_mode=0, shadow_size=1024)),
    # The deferred PBR workload's scene at full size: 20 icospheres of subdivision 5 (409,602
    # triangles with the ground), 1024^2 textures per mesh, 1280 x 800, PCSS 16 / 25 in a
    # 2048^2 map. The reference's SSAO constants are local to Render::DoSSAO (32 samples,
    # radius 0.075, render.cpp:219-222), so its golden frame uses those; the 64-sample,
    # r = 0.5 form of the benchmark is compared with the oracle (BENCH_SSAO below).
    "c1_def_pcss_1280x800": ("field", dict(seed=0, n_spheres=20, subdiv=5, tex=1024, width=1280, height=800),
                             "ref_pcss_tab", dict(shadow_mode=2, shadow_size=2048, pcf_samples=25,
                                                  blocker_samples=16)),
}

# The SSAO settings of the deferred benchmark frame (64 samples, radius 0.5).
BENCH_SSAO = dict(ssao_samples=64, ssao_radius=0.5)

def stress_mesh():
    """Triangles the rasteriser must treat exactly as the reference does, in draw
    order: a collinear and a repeated-vertex (zero-area) triangle, a long sliver,
    the same triangle twice and two coplanar overlapping ones (depth ties: the
    first drawn wins), a fan of 24 thin triangles around one vertex (shared
    vertices and edges), a square of axis-aligned right triangles (edges through
    many pixel centres) and one large triangle behind them all."""
    import numpy as np

    tris = [
        [(-1.0, 0.2, 0.0), (-0.5, 0.45, 0.0), (0.0, 0.7, 0.0)],      # collinear
        [(0.2, 0.2, 0.0), (0.2, 0.2, 0.0), (0.6, 0.5, 0.0)],         # repeated vertex
        [(-1.4, -0.6, 0.1), (1.4, -0.58, 0.1), (1.4, -0.575, 0.1)],  # sliver
        [(-0.9, -0.3, 0.2), (-0.3, -0.3, 0.2), (-0.6, 0.3, 0.2)],    # drawn twice
        [(-0.9, -0.3, 0.2), (-0.3, -0.3, 0.2), (-0.6, 0.3, 0.2)],
        [(0.1, -0.4, 0.3), (0.8, -0.4, 0.3), (0.45, 0.2, 0.3)],      # coplanar overlap
        [(0.3, -0.5, 0.3), (0.9, -0.1, 0.3), (0.2, 0.1, 0.3)],
    ]
    c = (0.9, 0.6, 0.25)
    for k in range(24):
        a0, a1 = 2 * np.pi * k / 24, 2 * np.pi * (k + 1) / 24
        tris.append([c, (c[0] + 0.4 * np.cos(a0), c[1] + 0.4 * np.sin(a0), 0.25),
                     (c[0] + 0.4 * np.cos(a1), c[1] + 0.4 * np.sin(a1), 0.25)])
    for i in range(4):
        for j in range(4):
            x0, y0 = -1.6 + 0.25 * i, 0.4 + 0.25 * j
            tris.append([(x0, y0, 0.15), (x0 + 0.25, y0, 0.15), (x0, y0 + 0.25, 0.15)])
            tris.append([(x0 + 0.25, y0, 0.15), (x0 + 0.25, y0 + 0.25, 0.15), (x0, y0 + 0.25, 0.15)])
    tris.append([(-3.0, -1.0, -0.5), (3.0, -1.0, -0.5), (0.0, 2.5, -0.5)])
    v = np.array([p for t in tris for p in t], dtype=np.float32)
    n = len(tris)
    vt = np.stack([(v[:, 0] + 2.0) / 4.0, (v[:, 1] + 1.0) / 4.0], 1).astype(np.float32)
    vn = np.array([[0.0, 0.0, 1.0]], dtype=np.float32)
    idx = np.arange(3 * n).reshape(n, 3)
    faces = np.stack([idx, idx, np.zeros_like(idx)], -1)
    return scenegen.Mesh("Stress", v, vt, vn, faces)


def stress_scene(outdir: str, seed: int = 7, width: int = 160, height: int = 100, deferred: bool = True) -> str:
    """stress_mesh() above a 5 x 5 floor and a 200 x 200 ground plane that passes
    under and behind the camera (vertices with clip w < 0: the reference projects
    them unclipped), one checker texture, point light, SSAO and shadow on."""
    import numpy as np

    os.makedirs(outdir, exist_ok=True)
    rng = np.random.Generator(np.random.PCG64(seed))
    scenegen.write_tga(os.path.join(outdir, "checker.tga"),
                       scenegen.checker(64, 8, rng.integers(0, 256, 3), rng.integers(0, 256, 3)))
    scenegen.write_mtl(os.path.join(outdir, "m.mtl"), "M",
                       {"Ka": (1, 1, 1), "Kd": (0.8, 0.8, 0.8), "Ks": (0.5, 0.5, 0.5), "map_Kd": "checker.tga"})
    scenegen.write_obj(os.path.join(outdir, "stress.obj"), stress_mesh(), "m.mtl", "M")
    scenegen.write_obj(os.path.join(outdir, "ground.obj"), scenegen.quad_plane(100.0, -1.0, uv=(-20.0, 20.0)),
                       "m.mtl", "M")
    scenegen.write_obj(os.path.join(outdir, "floor.obj"), scenegen.quad_plane(2.5, -0.8), "m.mtl", "M")
    spec = scenegen.SceneSpec(width, height, deferred, deferred, True, 0, (2, 5, 4), (1, 1, 1),
                              (0.3, 0.4, 3.0), (0.0, 0.0, 0.0),
                              [("stress.obj", False, (0, 0, 0), 15, 1), ("ground.obj", False, (0, 0, 0), 0, 1),
                               ("floor.obj", False, (0, 0, 0), 0, 1)])
    path = os.path.join(outdir, "scene.scene")
    spec.write(path)
    return path


# Scenes without golden fixtures (learned AO needs W, H multiples of 32).
EXTRA_CASES = {
    # frames whose columns (4,160 rows) or rows (16,400 pixels) are too long for the parallel
    # in-place blur's shared memory: the sequential walk runs instead
    "tall_16x4160": ("field", dict(seed=13, n_spheres=3, subdiv=2, tex=64, width=16, height=4160),
                     "ref_pcss_tab", dict(shadow_mode=2, shadow_size=256, pcf_samples=25, blocker_samples=16)),
    "wide_16400x4": ("field", dict(seed=14, n_spheres=3, subdiv=2, tex=64, width=16400, height=4),
                     "ref_pcss_tab", dict(shadow_mode=2, shadow_size=256, pcf_samples=25, blocker_samples=16)),
    # one 16 x 16 tile, 9 sphere faces and the 2-triangle ground (fits a tiny bin capacity)
    "tiny_16x16": ("forward", dict(seed=3, width=16, height=16, lon=3, lat=2, tex=16),
                   "ref_hard", dict(shadow_mode=0)),
    # the scaled configuration: 100 icospheres (subdivision 5, ~2.05 M triangles), 2x SSAA
    # (2560x1600 working resolution resolved to 1280x800), 4096^2 shadow map
    "scaled_100": ("field", dict(seed=0, n_spheres=100, subdiv=5, tex=1024, width=1280, height=800, ssaa=2),
                   "ref_pcss_tab", dict(shadow_mode=2, shadow_size=4096, pcf_samples=25, blocker_samples=16,
                                        ssao_samples=64, ssao_radius=0.5)),
    "def_ao_128": ("field", dict(seed=11, n_spheres=3, subdiv=2, tex=64, width=128, height=96),
                   "ref_pcss_tab", dict(shadow_mode=2, shadow_size=256, pcf_samples=25, blocker_samples=16,
                                        ssao_samples=64, ssao_radius=0.5)),
    # ground texture coordinates from -1.3 to 2.45: the texture wrap modes decide what it shows
    "def_wrap": ("field", dict(seed=6, n_spheres=3, subdiv=2, tex=64, width=160, height=100,
                               ground_uv=(-1.3, 2.45)), "ref_pcss_tab", dict(shadow_mode=2)),
    # the same scene forward-shaded: textures sampled in the fragment shader itself
    "fwd_wrap": ("field", dict(seed=6, n_spheres=3, subdiv=2, tex=64, width=160, height=100,
                               ground_uv=(-1.3, 2.45), deferred=False), "ref_pcss_tab", dict(shadow_mode=2)),
}

_CACHE = os.path.join(tempfile.gettempdir(), "fr_test_scenes")


def _case(name: str):
    return CASES[name] if name in CASES else EXTRA_CASES[name]


def scene_path(name: str) -> str:
    kind, kw, _, _ = _case(name)
    key = hashlib.sha1(repr((kind, sorted(kw.items()))).encode()).hexdigest()[:12]
    out = os.path.join(_CACHE, f"{name}_{key}")
    path = os.path.join(out, "scene.scene")
    if not os.path.exists(path):
        tmp = out + ".tmp%d" % os.getpid()
        if kind == "forward":
            scenegen.forward_sphere_scene(tmp, **kw)
        elif kind == "stress":
            stress_scene(tmp, **kw)
        else:
            scenegen.deferred_field_scene(tmp, **kw)
        try:
            os.rename(tmp, out)
        except OSError:
            pass  # another process won the race; its files are identical
    return path


def render_config(name: str, **extra) -> dict:
    cfg = dict(shadow_mode=2, shadow_size=0, pcf_samples=64, blocker_samples=32, ssao_samples=32,
               ssao_radius=0.075, ssao_bias=0.0005, ssao_range=0.01, blur_mode=0)
    cfg.update(_case(name)[3])
    cfg.update(extra)
    return cfg


def files_digest(name: str) -> str:
    d = os.path.dirname(scene_path(name))
    h = hashlib.sha256()
    for f in sorted(os.listdir(d)):
        with open(os.path.join(d, f), "rb") as fh:
            h.update(f.encode())
            h.update(fh.read())
    return h.hexdigest()
