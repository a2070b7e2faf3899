"""Seeded synthetic scene generator.

Writes ``.scene`` / ``.obj`` / ``.mtl`` / ``.tga`` files in exactly the dialect the
reference loader accepts, so the same files feed the reference renderer, the CPU
oracle and the GB300 path:

* ``.scene`` directives ``mode/screen/ssaa/ssao/shadow/light/camera/model``
  (src/scene.cpp:54-192); model lines are
  ``model <obj> <normalized> <genTangent> x y z rotY scale`` (scene.cpp:171-192).
* ``.obj``: ``mtllib``, ``v``, ``vt``, ``vn``, then ``g <name>`` *before*
  ``usemtl`` (model.cpp:211-220) and faces as ``v/t/n`` triples (model.cpp:228).
* ``.mtl``: ``newmtl``, ``Ka/Kd/Ks/Ke``, ``Pr/Pm``, ``map_Kd/map_Ks/map_Bump/map_Pr/
  map_Pm`` (model.cpp:258-408). PBR shading is selected by the presence of
  ``map_Pr`` or ``map_Pm`` (model.cpp:58).
* ``.tga``: uncompressed type 2 (BGR) or 3 (grey), bottom-left origin. The loader
  flips such a file on read (tgaimage.cpp:100) and again for texture v
  (model.cpp:423), so array row ``y`` here is texel row ``y`` as sampled.

Floats are written with 9 significant digits of their float32 value, which the
loader's ``istream >> float`` reads back bit-exactly. All randomness comes from
``numpy.random.Generator(PCG64(seed))``; transcendental functions go through the
C library one value at a time and every other step is an elementwise IEEE
operation, so a seed reproduces the files byte for byte on x86-64 and aarch64.
"""


from __future__ import annotations

import math
import os
from dataclasses import dataclass, field

import numpy as np


def _vsin(a):
    return np.array([math.sin(x) for x in np.ravel(a)], np.float64).reshape(np.shape(a))


def _vcos(a):
    return np.array([math.cos(x) for x in np.ravel(a)], np.float64).reshape(np.shape(a))


def _norm3(v: np.ndarray) -> np.ndarray:
    x, y, z = v[:, 0], v[:, 1], v[:, 2]
    return np.sqrt(x * x + y * y + z * z)[:, None]


def _gaussian_wrap(img: np.ndarray, sigma: float) -> np.ndarray:
    """Separable Gaussian blur with wrap-around borders, taps summed in a fixed
    order with elementwise operations (deterministic on every platform)."""
    r = int(4.0 * sigma + 0.5)
    k = np.array([math.exp(-0.5 * (i / sigma) ** 2) for i in range(-r, r + 1)], np.float64)
    k = k / math.fsum(k)
    out = img
    for axis in (0, 1):
        acc = np.zeros_like(out)
        for i, w in zip(range(-r, r + 1), k):
            acc = acc + np.roll(out, i, axis=axis) * w
        out = acc
    return out


__all__ = [
    "SceneSpec",
    "write_tga",
    "uv_sphere",
    "icosphere",
    "forward_sphere_scene",
    "deferred_field_scene",
]


def _f(x) -> str:
    return "%.9g" % np.float32(x)


def write_tga(path: str, img: np.ndarray) -> None:
    """Write an uncompressed TGA. ``img`` is (H, W, 3) RGB uint8 or (H, W) grey."""
    img = np.ascontiguousarray(img, dtype=np.uint8)
    if img.ndim == 2:
        h, w = img.shape
        code, bpp, data = 3, 8, img
    else:
        h, w, _ = img.shape
        code, bpp, data = 2, 24, img[:, :, ::-1]  # stored as BGR
    header = np.zeros(18, dtype=np.uint8)
    header[2] = code
    header[12:14] = np.frombuffer(np.uint16(w).tobytes(), np.uint8)
    header[14:16] = np.frombuffer(np.uint16(h).tobytes(), np.uint8)
    header[16] = bpp
    header[17] = 0x00  # bottom-left origin
    with open(path, "wb") as f:
        f.write(header.tobytes())
        f.write(np.ascontiguousarray(data).tobytes())


@dataclass
class Mesh:
    """One model file: positions/uvs/normals and faces as (v, vt, vn) index triples."""

    name: str
    v: np.ndarray  # (V, 3) float32
    vt: np.ndarray  # (T, 2) float32
    vn: np.ndarray  # (N, 3) float32
    faces: np.ndarray  # (F, 3, 3) int, 0-based (v, vt, vn) per corner


def write_obj(path: str, mesh: Mesh, mtl_name: str, material: str) -> None:
    lines = [f"mtllib {mtl_name}"]
    lines += [f"v {_f(a)} {_f(b)} {_f(c)}" for a, b, c in mesh.v]
    lines += [f"vt {_f(a)} {_f(b)}" for a, b in mesh.vt]
    lines += [f"vn {_f(a)} {_f(b)} {_f(c)}" for a, b, c in mesh.vn]
    lines.append(f"g {mesh.name}")
    lines.append(f"usemtl {material}")
    f1 = mesh.faces + 1
    lines += [
        "f " + " ".join(f"{c[0]}/{c[1]}/{c[2]}" for c in face) for face in f1
    ]
    with open(path, "w") as f:
        f.write("\n".join(lines) + "\n")


def write_mtl(path: str, name: str, props: dict) -> None:
    lines = [f"newmtl {name}"]
    for k, v in props.items():
        if isinstance(v, (tuple, list)):
            lines.append(f"    {k} " + " ".join(_f(x) for x in v))
        elif isinstance(v, str):
            lines.append(f"    {k} {v}")
        else:
            lines.append(f"    {k} {_f(v)}")
    with open(path, "w") as f:
        f.write("\n".join(lines) + "\n")


def uv_sphere(n_lon: int = 64, n_lat: int = 32, radius: float = 1.0, name="Sphere") -> Mesh:
    """UV sphere of n_lon x n_lat quads. Each quad is split in two; at the north
    pole the degenerate half is dropped, at the south pole it is kept (a zero-area
    triangle the rasteriser must reject), giving n_lon * (2 * n_lat - 1) faces."""
    lat = np.linspace(0.0, np.pi, n_lat + 1)
    lon = np.linspace(0.0, 2.0 * np.pi, n_lon + 1)
    th, ph = np.meshgrid(lat, lon, indexing="ij")  # (n_lat+1, n_lon+1)
    x = _vsin(th) * _vcos(ph)
    y = _vcos(th)
    z = -_vsin(th) * _vsin(ph)
    nrm = np.stack([x, y, z], -1).reshape(-1, 3)
    pos = nrm * radius
    uv = np.stack(np.meshgrid(np.linspace(0, 1, n_lat + 1), np.linspace(0, 1, n_lon + 1),
                              indexing="ij")[::-1], -1).reshape(-1, 2)
    uv[:, 1] = 1.0 - uv[:, 1]
    idx = lambda j, i: j * (n_lon + 1) + i  # noqa: E731
    faces = []
    for j in range(n_lat):
        for i in range(n_lon):
            a, b, c, d = idx(j, i), idx(j, i + 1), idx(j + 1, i), idx(j + 1, i + 1)
            if j != 0:
                faces.append((a, c, b))
            faces.append((b, c, d))
    f = np.array(faces, dtype=np.int64)
    corners = np.stack([f, f, f], -1)
    return Mesh(name, pos.astype(np.float32), uv.astype(np.float32),
                nrm.astype(np.float32), corners)


def icosphere(subdiv: int, rng: np.random.Generator, noise: float = 0.05,
              name="Ico") -> Mesh:
    """Icosphere with 20 * 4^subdiv faces, vertices displaced radially by
    U[0, noise], spherical uv, area-weighted vertex normals."""
    t = (1.0 + 5.0 ** 0.5) / 2.0
    verts = [(-1, t, 0), (1, t, 0), (-1, -t, 0), (1, -t, 0), (0, -1, t), (0, 1, t),
             (0, -1, -t), (0, 1, -t), (t, 0, -1), (t, 0, 1), (-t, 0, -1), (-t, 0, 1)]
    faces = [(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11), (1, 5, 9),
             (5, 11, 4), (11, 10, 2), (10, 7, 6), (7, 1, 8), (3, 9, 4), (3, 4, 2),
             (3, 2, 6), (3, 6, 8), (3, 8, 9), (4, 9, 5), (2, 4, 11), (6, 2, 10),
             (8, 6, 7), (9, 8, 1)]
    v = np.array(verts, dtype=np.float64)
    v = v / _norm3(v)
    f = np.array(faces, dtype=np.int64)
    for _ in range(subdiv):
        edges = np.concatenate([f[:, [0, 1]], f[:, [1, 2]], f[:, [2, 0]]])
        key = np.sort(edges, axis=1)
        uniq, inv = np.unique(key, axis=0, return_inverse=True)
        mid = v[uniq[:, 0]] + v[uniq[:, 1]]
        mid = mid / _norm3(mid)
        base = len(v)
        v = np.concatenate([v, mid])
        nf = len(f)
        m01 = base + inv[:nf]
        m12 = base + inv[nf:2 * nf]
        m20 = base + inv[2 * nf:]
        a, b, c = f[:, 0], f[:, 1], f[:, 2]
        f = np.concatenate([np.stack([a, m01, m20], 1), np.stack([b, m12, m01], 1),
                            np.stack([c, m20, m12], 1), np.stack([m01, m12, m20], 1)])
    r = 1.0 + rng.uniform(0.0, noise, size=len(v))
    pos = v * r[:, None]
    e1 = pos[f[:, 1]] - pos[f[:, 0]]
    e2 = pos[f[:, 2]] - pos[f[:, 0]]
    fn = np.cross(e1, e2)
    nrm = np.zeros_like(pos)
    for k in range(3):
        np.add.at(nrm, f[:, k], fn)
    nrm = nrm / _norm3(nrm)
    u = 0.5 + np.array([math.atan2(a, b) for a, b in zip(v[:, 2], v[:, 0])]) / (2 * math.pi)
    w = 0.5 - np.array([math.asin(min(1.0, max(-1.0, a))) for a in v[:, 1]]) / math.pi
    uv = np.stack([u, w], 1)
    corners = np.stack([f, f, f], -1)
    return Mesh(name, pos.astype(np.float32), uv.astype(np.float32),
                nrm.astype(np.float32), corners)


def quad_plane(half: float, y: float, name="Plane", uv=(0.0, 1.0)) -> Mesh:
    v = np.array([[-half, y, half], [half, y, half], [-half, y, -half], [half, y, -half]],
                 dtype=np.float32)
    lo, hi = uv
    vt = np.array([[lo, lo], [hi, lo], [lo, hi], [hi, hi]], dtype=np.float32)
    vn = np.array([[0, 1, 0]], dtype=np.float32)
    faces = np.array([[[0, 0, 0], [1, 1, 0], [2, 2, 0]], [[1, 1, 0], [3, 3, 0], [2, 2, 0]]])
    return Mesh(name, v, vt, vn, faces)


def checker(size: int, cells: int, c0, c1) -> np.ndarray:
    k = (np.arange(size) * cells // size)
    m = (k[:, None] + k[None, :]) % 2
    return np.where(m[:, :, None] == 0, np.array(c0, np.uint8), np.array(c1, np.uint8))


def normal_map(size: int, rng: np.random.Generator, sigma: float = 2.0,
               strength: float = 8.0) -> np.ndarray:
    h = _gaussian_wrap(rng.uniform(0.0, 1.0, (size, size)), sigma)
    gx = (np.roll(h, -1, axis=1) - np.roll(h, 1, axis=1)) * 0.5
    gy = (np.roll(h, -1, axis=0) - np.roll(h, 1, axis=0)) * 0.5
    n = np.stack([-gx * strength, -gy * strength, np.ones_like(h)], -1).reshape(-1, 3)
    n = (n / _norm3(n)).reshape(size, size, 3)
    return np.clip(np.round((n * 0.5 + 0.5) * 255.0), 0, 255).astype(np.uint8)


@dataclass
class SceneSpec:
    """What a generated scene contains; written by ``write``."""

    width: int
    height: int
    deferred: bool
    ssao: bool
    shadow: bool
    ssaa: int  # 0 = off, else kernel size
    light: tuple
    light_color: tuple
    eye: tuple
    target: tuple
    models: list = field(default_factory=list)  # (obj relpath, genTangent, pos, rotY, scale)

    def write(self, path: str) -> None:
        L = [f"mode {'deferred' if self.deferred else 'forward'}",
             f"screen {self.width} {self.height}",
             f"ssaa {'on' if self.ssaa else 'off'} {self.ssaa or 2}",
             f"ssao {'on' if self.ssao else 'off'}",
             f"shadow {'on' if self.shadow else 'off'}",
             "light point " + " ".join(_f(x) for x in (*self.light, *self.light_color)),
             "camera persp " + " ".join(_f(x) for x in (*self.eye, *self.target))]
        for obj, tan, pos, roty, scale in self.models:
            L.append(f"model {obj} false {'true' if tan else 'false'} "
                     + " ".join(_f(x) for x in (*pos, roty, scale)))
        with open(path, "w") as f:
            f.write("\n".join(L) + "\n")


def forward_sphere_scene(outdir: str, seed: int = 0, width: int = 640, height: int = 400,
                         lon: int = 64, lat: int = 32, tex: int = 256,
                         shadow: bool = True) -> str:
    """The plain forward Blinn-Phong scene: UV sphere (radius 1 at (0,0,-2)) on a
    6 x 6 ground plane at y = -1, 8 x 8-cell checker texture in two seeded colours,
    point light (2,5,5), camera (-1,1,1) -> (0,0,-1). Returns the .scene path."""
    os.makedirs(outdir, exist_ok=True)
    rng = np.random.Generator(np.random.PCG64(seed))
    c0 = rng.integers(0, 256, 3)
    c1 = rng.integers(0, 256, 3)
    write_tga(os.path.join(outdir, "checker.tga"), checker(tex, 8, c0, c1))
    write_mtl(os.path.join(outdir, "checker.mtl"), "Checker",
              {"Ka": (1, 1, 1), "Kd": (0.8, 0.8, 0.8), "Ks": (0.5, 0.5, 0.5),
               "map_Kd": "checker.tga"})
    write_obj(os.path.join(outdir, "sphere.obj"), uv_sphere(lon, lat), "checker.mtl", "Checker")
    write_obj(os.path.join(outdir, "plane.obj"), quad_plane(3.0, -1.0), "checker.mtl", "Checker")
    spec = SceneSpec(width, height, False, False, shadow, 0, (2, 5, 5), (1, 1, 1),
                     (-1, 1, 1), (0, 0, -1),
                     [("sphere.obj", False, (0, 0, -2), 0, 1), ("plane.obj", False, (0, 0, 0), 0, 1)])
    path = os.path.join(outdir, "scene.scene")
    spec.write(path)
    return path


def deferred_field_scene(outdir: str, seed: int = 0, n_spheres: int = 20, subdiv: int = 5,
                         tex: int = 1024, width: int = 1280, height: int = 800,
                         ssaa: int = 0, ssao: bool = True, shadow: bool = True,
                         field_size: float = 10.0, eye=(0.0, 7.0, 11.0),
                         target=(0.0, 0.0, 0.0), light=(3.0, 9.0, 6.0),
                         pbr: bool = True, share_textures: bool = False,
                         deferred: bool = True, yaw: bool = True, ground_uv=(0.0, 1.0)) -> str:
    """The deferred PBR field: ``n_spheres`` icospheres (radial noise U[0,0.05],
    scale U[0.3,1], yaw U[0,360), positions uniform over a field_size^2 area resting
    on a ground plane at y = 0), each with its own albedo (RGB8 noise), roughness and
    metalness (U8 noise) and tangent-space normal map (blurred-noise heightfield,
    sigma 2). ground_uv: the ground's texture coordinates run from ground_uv[0] to
    ground_uv[1] (outside [0, 1] the texture wrap mode decides). Returns the .scene path."""
    os.makedirs(outdir, exist_ok=True)
    rng = np.random.Generator(np.random.PCG64(seed))
    models = []

    def material(i: int) -> str:
        mtl = f"mat{i}.mtl"
        if share_textures and i > 0:
            return mtl if os.path.exists(os.path.join(outdir, mtl)) else _copy_mtl(i)
        alb = rng.integers(0, 256, (tex, tex, 3), dtype=np.uint8)
        write_tga(os.path.join(outdir, f"albedo{i}.tga"), alb)
        write_tga(os.path.join(outdir, f"normal{i}.tga"), normal_map(tex, rng))
        props = {"Ka": (1, 1, 1), "Kd": (1, 1, 1), "Ks": (0.5, 0.5, 0.5),
                 "map_Kd": f"albedo{i}.tga", "map_Bump": f"normal{i}.tga"}
        if pbr:
            write_tga(os.path.join(outdir, f"rough{i}.tga"),
                      rng.integers(0, 256, (tex, tex), dtype=np.uint8))
            write_tga(os.path.join(outdir, f"metal{i}.tga"),
                      rng.integers(0, 256, (tex, tex), dtype=np.uint8))
            props["map_Pr"] = f"rough{i}.tga"
            props["map_Pm"] = f"metal{i}.tga"
        else:
            write_tga(os.path.join(outdir, f"spec{i}.tga"),
                      rng.integers(0, 256, (tex, tex), dtype=np.uint8))
            props["map_Ks"] = f"spec{i}.tga"
        write_mtl(os.path.join(outdir, mtl), f"Mat{i}", props)
        return mtl

    def _copy_mtl(i: int) -> str:
        with open(os.path.join(outdir, "mat0.mtl")) as f:
            txt = f.read().replace("newmtl Mat0", f"newmtl Mat{i}")
        with open(os.path.join(outdir, f"mat{i}.mtl"), "w") as f:
            f.write(txt)
        return f"mat{i}.mtl"

    half = field_size / 2.0
    mtl = material(0)
    write_obj(os.path.join(outdir, "ground.obj"), quad_plane(half + 1.0, 0.0, "Ground", ground_uv), mtl, "Mat0")
    models.append(("ground.obj", True, (0.0, 0.0, 0.0), 0.0, 1.0))
    for i in range(n_spheres):
        mesh = icosphere(subdiv, rng, 0.05, name=f"Ico{i}")
        scale = float(rng.uniform(0.3, 1.0))
        yaw_deg = float(rng.uniform(0.0, 360.0))
        if not yaw:
            yaw_deg = 0.0
        px, pz = rng.uniform(-half, half, 2)
        mtl = material(i + 1)
        write_obj(os.path.join(outdir, f"ico{i}.obj"), mesh, mtl, f"Mat{i + 1}")
        models.append((f"ico{i}.obj", True, (float(px), scale, float(pz)), yaw_deg, scale))
    spec = SceneSpec(width, height, deferred, ssao, shadow, ssaa, light, (1, 1, 1), eye, target,
                     models)
    path = os.path.join(outdir, "scene.scene")
    spec.write(path)
    return path
