"""Loading and comparing against the golden fixtures of tests/golden/."""

from __future__ import annotations

import hashlib
import json
import os

import numpy as np

from forkerrenderer_gb300 import _native as N

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load(name: str):
    with open(os.path.join(GOLDEN, f"{name}.json")) as f:
        meta = json.load(f)
    arrays = dict(np.load(os.path.join(GOLDEN, f"{name}.npz")))
    return meta, arrays


def sha(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def matrices(meta: dict, shadow_size: int) -> N.FrameMatrices:
    """FrameMatrices holding exactly the reference's matrices of the fixture."""
    m = N.FrameMatrices()
    get = lambda k: [float.fromhex(x) for x in meta["matrices"][k]]  # noqa: E731
    m.view_projection[:] = get("viewproj")
    m.light_space[:] = get("lightspace")
    m.viewport[:] = get("viewport")
    info = meta["info"]
    m.width, m.height = info["width"], info["height"]
    m.shadow_width = info["shadow_width"] or m.width
    m.shadow_height = info["shadow_height"] or m.height
    return m


def psnr(a: np.ndarray, b: np.ndarray) -> float:
    d = (a.astype(np.float64) - b.astype(np.float64)) ** 2
    mse = d.mean()
    return float("inf") if mse == 0 else 10 * np.log10(255.0 ** 2 / mse)


def check_frame8(got: np.ndarray, want: np.ndarray, min_frac: float = 0.999, min_psnr: float = 50.0):
    """The shading bar: within 1 LSB on >= 99.9% of channels and PSNR >= 50 dB."""
    got = np.asarray(got).reshape(-1)
    want = np.asarray(want).reshape(-1)
    d = np.abs(got.astype(int) - want.astype(int))
    frac = float((d <= 1).mean())
    p = psnr(got, want)
    assert frac >= min_frac and p >= min_psnr, f"within-1LSB {frac:.6f}, PSNR {p:.2f} dB, max {d.max()}"
    return frac, p
