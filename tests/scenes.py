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
}

# Scenes without golden fixtures (learned AO needs W, H multiples of 32).
EXTRA_CASES = {
    # the scaled configuration: 100 icospheres (subdivision 5, ~2.05 M triangles), 2x SSAA
    # (2560x1600 working resolution resolved to 1280x800), 4096^2 shadow map
    "scaled_100": ("field", dict(seed=0, n_spheres=100, subdiv=5, tex=64, width=1280, height=800, ssaa=2),
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
