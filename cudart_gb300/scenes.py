"""Seeded synthetic scenes for the path-tracing workloads.

Each generator returns a :class:`SceneArrays`: triangles in face order
(positions, per-vertex normals and uvs), per-triangle material ids, the
material table with MTL-level values, RGBA8 textures and the camera-JSON
fields.  The same scene can be written as OBJ/MTL/camera-JSON/PNG files in
the layout CudaRT's loaders read (``write_reference_files``), so the
reference renderer and this library consume identical inputs.

Workloads (sizes as used by the benchmarks and parity tests):

* ``cornell_box``       -- 2x2x2 Cornell box, 36 triangles, 512x512, 16 spp, depth 5
* ``mixed_mid``         -- Cornell shell + 5 displaced icospheres (subdivision 5),
                           102,412 triangles, 1280x720, 128 spp, depth 8
* ``large_textured``    -- 1024x1024-vertex heightfield with a 1024^2 RGBA8
                           texture, 64 glass/mirror icospheres, 4 quad lights,
                           ~2.18M triangles, 1920x1080, 256 spp, depth 8
* ``batched_views``     -- the mixed_mid scene seen from 64 hemisphere poses
* ``material_inversion``-- Cornell shell + 32 diffuse boxes, 396 triangles
"""
from __future__ import annotations

import dataclasses
import json
import math
import os
import struct
import zlib
from typing import List, Optional, Sequence

import numpy as np

DIFFUSE, SPECULAR, DIFFSPEC, MICROFACET, REFRACTIVE, EMISSIVE = range(6)
BSDF_NAMES = {DIFFUSE: "LAMBERT", SPECULAR: "SPECULAR", DIFFSPEC: "DIFFSPEC",
              MICROFACET: "MICROFACET", REFRACTIVE: "REFRACTIVE", EMISSIVE: "EMISSIVE"}
NO_TEXTURE = -1


@dataclasses.dataclass
class Material:
    """One MTL material (obj_load.h Material + CudaRT's `type`/`diffuse` keys)."""
    name: str
    bsdf: int = DIFFUSE
    kd: Sequence[float] = (0.0, 0.0, 0.0)
    ka: Sequence[float] = (0.0, 0.0, 0.0)     # MTL Ka; emission = 3 * Ka
    ks: Sequence[float] = (0.0, 0.0, 0.0)
    ns: float = 0.0
    ni: float = 1.0
    diffuse: float = 0.0
    tex: int = NO_TEXTURE                     # index into SceneArrays.textures


@dataclasses.dataclass
class CameraSpec:
    """Camera-JSON fields (json_loader.cpp:26-48)."""
    fov_deg: float
    eye: Sequence[float]
    view_dir: Sequence[float]
    up: Sequence[float] = (0.0, 1.0, 0.0)
    focal_length: float = 0.0
    fstop: float = 1.0


@dataclasses.dataclass
class View:
    """One camera view of a batched render."""
    camera: CameraSpec
    width: int
    height: int
    spp: int


@dataclasses.dataclass
class SceneArrays:
    positions: np.ndarray          # float32 [n, 3, 3]
    normals: np.ndarray            # float32 [n, 3, 3]
    uvs: np.ndarray                # float32 [n, 3, 2]
    material_ids: np.ndarray       # uint32 [n]
    materials: List[Material]
    textures: List[np.ndarray]     # uint8 [h, w, 4]
    camera: CameraSpec
    width: int
    height: int
    spp: int
    max_depth: int
    groups: List[tuple]            # (name, material index, first tri, tri count)
    views: Optional[List[View]] = None

    @property
    def n_tris(self) -> int:
        return int(self.positions.shape[0])

    def light_indices(self) -> np.ndarray:
        emissive = np.array([m.bsdf == EMISSIVE for m in self.materials])
        return np.nonzero(emissive[self.material_ids])[0].astype(np.uint32)


# ---------------------------------------------------------------------------
# mesh builders
# ---------------------------------------------------------------------------
class _MeshBuilder:
    def __init__(self):
        self.pos: List[np.ndarray] = []
        self.nor: List[np.ndarray] = []
        self.uv: List[np.ndarray] = []
        self.mat: List[np.ndarray] = []
        self.groups: List[tuple] = []
        self.count = 0

    def add(self, name, mat, pos, nor, uv=None):
        pos = np.asarray(pos, np.float32).reshape(-1, 3, 3)
        nor = np.asarray(nor, np.float32).reshape(-1, 3, 3)
        if uv is None:
            uv = np.zeros((pos.shape[0], 3, 2), np.float32)
        uv = np.asarray(uv, np.float32).reshape(-1, 3, 2)
        n = pos.shape[0]
        self.pos.append(pos)
        self.nor.append(nor)
        self.uv.append(uv)
        self.mat.append(np.full(n, mat, np.uint32))
        self.groups.append((name, mat, self.count, n))
        self.count += n

    def arrays(self):
        return (np.concatenate(self.pos), np.concatenate(self.nor), np.concatenate(self.uv),
                np.concatenate(self.mat))


def _quad(p0, p1, p2, p3, normal):
    """Two triangles (p0,p1,p2), (p0,p2,p3) with a constant vertex normal."""
    pos = np.array([[p0, p1, p2], [p0, p2, p3]], np.float32)
    nor = np.tile(np.asarray(normal, np.float32), (2, 3, 1))
    uv = np.array([[[0, 0], [1, 0], [1, 1]], [[0, 0], [1, 1], [0, 1]]], np.float32)
    return pos, nor, uv


def _box(center, size, angle_deg):
    """Axis-aligned box of `size` rotated about +y, 12 triangles, outward normals."""
    cx, cy, cz = center
    sx, sy, sz = (s * 0.5 for s in size)
    a = math.radians(angle_deg)
    ca, sa = math.cos(a), math.sin(a)

    def tr(x, y, z):
        return (cx + ca * x + sa * z, cy + y, cz - sa * x + ca * z)

    def rn(x, y, z):
        return (ca * x + sa * z, y, -sa * x + ca * z)

    faces = [
        ((-sx, -sy, sz), (sx, -sy, sz), (sx, sy, sz), (-sx, sy, sz), (0, 0, 1)),
        ((sx, -sy, -sz), (-sx, -sy, -sz), (-sx, sy, -sz), (sx, sy, -sz), (0, 0, -1)),
        ((sx, -sy, sz), (sx, -sy, -sz), (sx, sy, -sz), (sx, sy, sz), (1, 0, 0)),
        ((-sx, -sy, -sz), (-sx, -sy, sz), (-sx, sy, sz), (-sx, sy, -sz), (-1, 0, 0)),
        ((-sx, sy, sz), (sx, sy, sz), (sx, sy, -sz), (-sx, sy, -sz), (0, 1, 0)),
        ((-sx, -sy, -sz), (sx, -sy, -sz), (sx, -sy, sz), (-sx, -sy, sz), (0, -1, 0)),
    ]
    pos, nor, uv = [], [], []
    for p0, p1, p2, p3, n in faces:
        q = _quad(tr(*p0), tr(*p1), tr(*p2), tr(*p3), rn(*n))
        pos.append(q[0]); nor.append(q[1]); uv.append(q[2])
    return np.concatenate(pos), np.concatenate(nor), np.concatenate(uv)


def _icosphere(subdiv: int):
    """Unit icosphere: vertices [V,3] float64 and faces [F,3] int."""
    t = (1.0 + 5.0 ** 0.5) / 2.0
    v = [(-1, t, 0), (1, t, 0), (-1, -t, 0), (1, -t, 0), (0, -1, t), (0, 1, t), (0, -1, -t),
         (0, 1, -t), (t, 0, -1), (t, 0, 1), (-t, 0, -1), (-t, 0, 1)]
    f = [(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11), (1, 5, 9), (5, 11, 4),
         (11, 10, 2), (10, 7, 6), (7, 1, 8), (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8),
         (3, 8, 9), (4, 9, 5), (2, 4, 11), (6, 2, 10), (8, 6, 7), (9, 8, 1)]
    verts = [np.array(p, np.float64) / np.linalg.norm(p) for p in v]
    faces = np.array(f, np.int64)
    for _ in range(subdiv):
        cache = {}
        new_faces = []

        def mid(i, j):
            key = (i, j) if i < j else (j, i)
            if key not in cache:
                m = verts[i] + verts[j]
                verts.append(m / np.linalg.norm(m))
                cache[key] = len(verts) - 1
            return cache[key]

        for a, b, c in faces:
            ab, bc, ca = mid(a, b), mid(b, c), mid(c, a)
            new_faces += [(a, ab, ca), (b, bc, ab), (c, ca, bc), (ab, bc, ca)]
        faces = np.array(new_faces, np.int64)
    return np.array(verts), faces


def _sphere_mesh(center, radius, subdiv, rng=None, noise=0.0):
    """Icosphere with optional seeded radial displacement of +-noise*radius."""
    verts, faces = _icosphere(subdiv)
    r = np.full(len(verts), radius, np.float64)
    if rng is not None and noise > 0:
        r = r * (1.0 + rng.uniform(-noise, noise, len(verts)))
    p = verts * r[:, None] + np.asarray(center, np.float64)
    pos = p[faces].astype(np.float32)
    nor = verts[faces].astype(np.float32)      # radial shading normals
    return pos, nor


def _cornell_shell(mb: _MeshBuilder, wall_mats, light_mat, light_size=0.5, light_y=0.999):
    """Five walls of the 2x2x2 box (open towards +z) and a ceiling quad light."""
    left, right, white = wall_mats
    L = 1.0
    q = _quad((-L, -L, L), (-L, -L, -L), (-L, L, -L), (-L, L, L), (1, 0, 0))
    mb.add("left_wall", left, *q)
    q = _quad((L, -L, -L), (L, -L, L), (L, L, L), (L, L, -L), (-1, 0, 0))
    mb.add("right_wall", right, *q)
    q = _quad((-L, -L, -L), (L, -L, -L), (L, L, -L), (-L, L, -L), (0, 0, 1))
    mb.add("back_wall", white, *q)
    q = _quad((-L, -L, L), (L, -L, L), (L, -L, -L), (-L, -L, -L), (0, 1, 0))
    mb.add("floor", white, *q)
    q = _quad((-L, L, -L), (L, L, -L), (L, L, L), (-L, L, L), (0, -1, 0))
    mb.add("ceiling", white, *q)
    h = light_size * 0.5
    q = _quad((-h, light_y, -h), (h, light_y, -h), (h, light_y, h), (-h, light_y, h), (0, -1, 0))
    mb.add("light", light_mat, *q)


def _cornell_materials():
    return [
        Material("left_red", DIFFUSE, kd=(0.63, 0.065, 0.05)),
        Material("right_green", DIFFUSE, kd=(0.14, 0.45, 0.09)),
        Material("white", DIFFUSE, kd=(0.725, 0.71, 0.68)),
        Material("light", EMISSIVE, kd=(0.0, 0.0, 0.0), ka=(17.0 / 3, 12.0 / 3, 4.0 / 3)),
    ]


def _finish(mb, materials, textures, camera, width, height, spp, depth, views=None):
    pos, nor, uv, mat = mb.arrays()
    return SceneArrays(pos, nor, uv, mat, materials, textures, camera, width, height, spp,
                       depth, mb.groups, views)


CORNELL_CAMERA = CameraSpec(fov_deg=40.0, eye=(0.0, 0.0, 3.9), view_dir=(0.0, 0.0, -1.0))


def cornell_box(width=512, height=512, spp=16, max_depth=5) -> SceneArrays:
    """Procedural Cornell box: 5 walls, 0.5x0.5 ceiling light (17,12,4), two
    diffuse boxes rotated +-17 degrees; 36 triangles."""
    mats = _cornell_materials()
    mb = _MeshBuilder()
    _cornell_shell(mb, (0, 1, 2), 3)
    mb.add("short_box", 2, *_box((0.35, -0.7, 0.3), (0.6, 0.6, 0.6), -17.0))
    mb.add("tall_box", 2, *_box((-0.35, -0.4, -0.3), (0.6, 1.2, 0.6), 17.0))
    return _finish(mb, mats, [], CORNELL_CAMERA, width, height, spp, max_depth)


def cornell_lens(width=96, height=96, spp=16, max_depth=6) -> SceneArrays:
    """The Cornell box through a thin lens: aperture focalLength / fStop =
    0.5 / 4 = 0.125, focused at |viewDirection| = 3.9 (the box centre), so
    the camera's lens-jitter path (camera.cu:38-57) is exercised."""
    sc = cornell_box(width, height, spp, max_depth)
    cam = CameraSpec(CORNELL_CAMERA.fov_deg, CORNELL_CAMERA.eye, (0.0, 0.0, -3.9), CORNELL_CAMERA.up,
                     focal_length=0.5, fstop=4.0)
    return dataclasses.replace(sc, camera=cam)


def mixed_mid(seed=2, width=1280, height=720, spp=128, max_depth=8, subdiv=5) -> SceneArrays:
    """Cornell shell + 5 icospheres (radial noise +-2%); seeded materials:
    diffuse U(0.1,0.9), mirror, or glass with IOR 1.5."""
    rng = np.random.default_rng(seed)
    mats = _cornell_materials()[:4]
    mb = _MeshBuilder()
    _cornell_shell(mb, (0, 1, 2), 3)
    centers = [(-0.5, -0.65, -0.3), (0.45, -0.68, 0.2), (0.0, -0.15, -0.55),
               (-0.45, 0.3, 0.35), (0.5, 0.35, -0.45)]
    radii = [0.33, 0.3, 0.28, 0.25, 0.27]
    for k, (c, r) in enumerate(zip(centers, radii)):
        kind = int(rng.integers(0, 3))
        if kind == 0:
            m = Material(f"sphere{k}_diffuse", DIFFUSE, kd=tuple(rng.uniform(0.1, 0.9, 3)))
        elif kind == 1:
            m = Material(f"sphere{k}_mirror", SPECULAR, ks=(0.95, 0.95, 0.95))
        else:
            m = Material(f"sphere{k}_glass", REFRACTIVE, ks=(1.0, 1.0, 1.0), ni=1.5)
        mats.append(m)
        pos, nor = _sphere_mesh(c, r, subdiv, rng, 0.02)
        mb.add(f"sphere{k}", len(mats) - 1, pos, nor)
    cam = CameraSpec(fov_deg=40.0, eye=(0.0, 0.0, 3.9), view_dir=(0.0, 0.0, -1.0))
    return _finish(mb, mats, [], cam, width, height, spp, max_depth)


def _value_noise(n, octaves, rng):
    """Seeded 2-D value noise on an n x n grid, octaves of doubling frequency."""
    out = np.zeros((n, n), np.float64)
    amp, total = 1.0, 0.0
    xs = np.linspace(0.0, 1.0, n)
    for o in range(octaves):
        cells = 4 * (2 ** o)
        lat = rng.uniform(-1.0, 1.0, (cells + 1, cells + 1))
        g = xs * cells
        i0 = np.minimum(np.floor(g).astype(np.int64), cells - 1)
        f = g - i0
        f = f * f * (3 - 2 * f)
        a = lat[i0][:, i0]
        b = lat[i0][:, i0 + 1]
        c = lat[i0 + 1][:, i0]
        d = lat[i0 + 1][:, i0 + 1]
        fx, fy = f[None, :], f[:, None]
        out += amp * ((a * (1 - fx) + b * fx) * (1 - fy) + (c * (1 - fx) + d * fx) * fy)
        total += amp
        amp *= 0.5
    return out / total


def _checker_noise_texture(size, rng):
    yy, xx = np.mgrid[0:size, 0:size]
    checker = ((xx // 64 + yy // 64) % 2).astype(np.float64)
    noise = _value_noise(size, 4, rng) * 0.5 + 0.5
    base = 0.25 + 0.5 * checker
    rgb = np.stack([base * (0.6 + 0.4 * noise), base * (0.5 + 0.5 * noise),
                    base * (0.8 - 0.3 * noise)], -1)
    img = np.empty((size, size, 4), np.uint8)
    img[..., :3] = np.clip(np.round(rgb * 255), 0, 255).astype(np.uint8)
    img[..., 3] = 255
    return img


def large_textured(seed=3, width=1920, height=1080, spp=256, max_depth=8, grid=1024,
                   tex_size=1024, n_spheres=64, sphere_subdiv=3) -> SceneArrays:
    """Heightfield (grid x grid vertices over 10x10, 6-octave value noise of
    amplitude 0.2) with a procedural RGBA8 checker/noise albedo texture, 64
    glass or mirror icospheres and 4 quad lights of emission U(5, 20)."""
    rng = np.random.default_rng(seed)
    h = _value_noise(grid, 6, rng) * 0.2
    ext = 10.0
    xs = np.linspace(-ext / 2, ext / 2, grid)
    X, Z = np.meshgrid(xs, xs)
    P = np.stack([X, h, Z], -1)
    dx = xs[1] - xs[0]
    gx = np.gradient(h, dx, axis=1)
    gz = np.gradient(h, dx, axis=0)
    N = np.stack([-gx, np.ones_like(h), -gz], -1)
    N /= np.linalg.norm(N, axis=-1, keepdims=True)
    # uvs stay inside [0.5/W, (W-1.5)/W] so the bilinear lookup's +1 neighbours
    # stay inside the texture
    t = np.linspace(0.0, 1.0, grid)
    umin, umax = 0.5 / tex_size, (tex_size - 1.5) / tex_size
    U = umin + (umax - umin) * t
    UV = np.stack(np.meshgrid(U, U), -1)
    i = np.arange(grid - 1)
    I, J = np.meshgrid(i, i)
    a = (J * grid + I).ravel()
    b, c, d = a + 1, a + grid, a + grid + 1
    tri = np.stack([np.stack([a, c, b], 1), np.stack([b, c, d], 1)], 1).reshape(-1, 3)
    Pf, Nf, UVf = P.reshape(-1, 3), N.reshape(-1, 3), UV.reshape(-1, 2)
    mats = [Material("terrain", DIFFUSE, kd=(0.5, 0.5, 0.5), tex=0),
            Material("mirror", SPECULAR, ks=(0.95, 0.95, 0.95)),
            Material("glass", REFRACTIVE, ks=(1.0, 1.0, 1.0), ni=1.5)]
    mb = _MeshBuilder()
    mb.add("terrain", 0, Pf[tri], Nf[tri], UVf[tri])
    for k in range(n_spheres):
        r = float(rng.uniform(0.12, 0.35))
        x, z = rng.uniform(-4.2, 4.2, 2)
        gi = int(round((x + ext / 2) / dx)); gj = int(round((z + ext / 2) / dx))
        y = float(h[min(gj, grid - 1), min(gi, grid - 1)]) + r * 0.9
        pos, nor = _sphere_mesh((x, y, z), r, sphere_subdiv)
        mb.add(f"sphere{k}", 1 + int(rng.integers(0, 2)), pos, nor)
    for k, (lx, lz) in enumerate([(-2.5, -2.5), (2.5, -2.5), (-2.5, 2.5), (2.5, 2.5)]):
        e = rng.uniform(5.0, 20.0, 3)
        mats.append(Material(f"light{k}", EMISSIVE, ka=tuple(e / 3.0)))
        s = 0.5
        q = _quad((lx - s, 3.0, lz - s), (lx + s, 3.0, lz - s), (lx + s, 3.0, lz + s),
                  (lx - s, 3.0, lz + s), (0, -1, 0))
        mb.add(f"light{k}", len(mats) - 1, *q)
    tex = _checker_noise_texture(tex_size, rng)
    cam = CameraSpec(fov_deg=45.0, eye=(0.0, 3.2, 7.5), view_dir=(0.0, -3.2, -7.5))
    return _finish(mb, mats, [tex], cam, width, height, spp, max_depth)


def batched_views(seed=4, n_views=64, base: Optional[SceneArrays] = None) -> SceneArrays:
    """The mixed_mid scene seen from n_views poses on a hemisphere of radius
    12 with seeded jitter; resolutions from {256^2, 512^2, 768x432, 1024^2}
    and spp from {16, 64, 256}."""
    sc = base if base is not None else mixed_mid()
    rng = np.random.default_rng(seed)
    res = [(256, 256), (512, 512), (768, 432), (1024, 1024)]
    spps = [16, 64, 256]
    views = []
    for k in range(n_views):
        theta = rng.uniform(0.05, 0.45 * math.pi)       # elevation
        phi = (2 * math.pi * k / n_views) + rng.uniform(-0.05, 0.05)
        eye = np.array([12 * math.cos(theta) * math.sin(phi), 12 * math.sin(theta),
                        12 * math.cos(theta) * math.cos(phi)])
        target = rng.uniform(-0.2, 0.2, 3)
        w, hgt = res[int(rng.integers(0, len(res)))]
        views.append(View(CameraSpec(fov_deg=14.0, eye=tuple(eye), view_dir=tuple(target - eye)),
                          w, hgt, spps[int(rng.integers(0, len(spps)))]))
    return dataclasses.replace(sc, views=views)


def material_inversion(seed=5, width=512, height=512, spp=64, max_depth=6,
                       n_boxes=32) -> SceneArrays:
    """Cornell shell + n_boxes seeded diffuse boxes, each with its own
    albedo drawn from U(0.1, 0.9) (the ground truth of the inversion)."""
    rng = np.random.default_rng(seed)
    mats = _cornell_materials()
    mb = _MeshBuilder()
    _cornell_shell(mb, (0, 1, 2), 3)
    for k in range(n_boxes):
        mats.append(Material(f"box{k}", DIFFUSE, kd=tuple(rng.uniform(0.1, 0.9, 3))))
        s = float(rng.uniform(0.12, 0.3))
        c = (float(rng.uniform(-0.75, 0.75)), float(rng.uniform(-0.9, 0.6)),
             float(rng.uniform(-0.8, 0.5)))
        mb.add(f"box{k}", len(mats) - 1, *_box(c, (s, s, s), float(rng.uniform(-45, 45))))
    return _finish(mb, mats, [], CORNELL_CAMERA, width, height, spp, max_depth)


def feature_mix(width=64, height=48, spp=16, max_depth=6) -> SceneArrays:
    """Small scene exercising every estimator branch: diffuse, textured
    diffuse (back wall), DIFFSPEC, glass, mirror, MICROFACET (no BSDF
    branch), and two emitters.  Kept under ~300 triangles so the
    reference's 16-entry traversal stack suffices."""
    rng = np.random.default_rng(6)
    mats = _cornell_materials()
    mats += [
        Material("back_textured", DIFFUSE, kd=(0.5, 0.5, 0.5), tex=0),
        Material("diffspec", DIFFSPEC, kd=(0.2, 0.3, 0.8), ks=(0.9, 0.9, 0.9), diffuse=0.6),
        Material("glass", REFRACTIVE, ks=(1.0, 1.0, 1.0), ni=1.5),
        Material("mirror", SPECULAR, ks=(0.95, 0.95, 0.95)),
        Material("microfacet", MICROFACET, kd=(0.7, 0.7, 0.7)),
        Material("light2", EMISSIVE, ka=(2.0, 3.0, 5.0)),
    ]
    mb = _MeshBuilder()
    L = 1.0
    q = _quad((-L, -L, L), (-L, -L, -L), (-L, L, -L), (-L, L, L), (1, 0, 0))
    mb.add("left_wall", 0, *q)
    q = _quad((L, -L, -L), (L, -L, L), (L, L, L), (L, L, -L), (-1, 0, 0))
    mb.add("right_wall", 1, *q)
    pos, nor, _ = _quad((-L, -L, -L), (L, -L, -L), (L, L, -L), (-L, L, -L), (0, 0, 1))
    uv = np.array([[[0.05, 0.05], [0.9, 0.05], [0.9, 0.9]], [[0.05, 0.05], [0.9, 0.9], [0.05, 0.9]]],
                  np.float32)
    mb.add("back_wall", 4, pos, nor, uv)
    q = _quad((-L, -L, L), (L, -L, L), (L, -L, -L), (-L, -L, -L), (0, 1, 0))
    mb.add("floor", 2, *q)
    q = _quad((-L, L, -L), (L, L, -L), (L, L, L), (-L, L, L), (0, -1, 0))
    mb.add("ceiling", 2, *q)
    h = 0.25
    q = _quad((-h, 0.999, -h), (h, 0.999, -h), (h, 0.999, h), (-h, 0.999, h), (0, -1, 0))
    mb.add("light", 3, *q)
    q = _quad((-0.99, 0.2, -0.7), (-0.99, 0.2, -0.4), (-0.99, 0.5, -0.4), (-0.99, 0.5, -0.7), (1, 0, 0))
    mb.add("light2", 9, *q)
    for name, mat, c, r in [("diffspec_ball", 5, (-0.5, -0.65, -0.2), 0.33),
                            ("glass_ball", 6, (0.45, -0.68, 0.25), 0.3),
                            ("mirror_ball", 7, (0.35, 0.1, -0.5), 0.28)]:
        p, n = _sphere_mesh(c, r, 1)
        mb.add(name, mat, p, n)
    # lifted 0.01 off the floor: no coplanar faces, so no equal-t ties
    mb.add("microfacet_box", 8, *_box((-0.3, -0.84, 0.45), (0.3, 0.3, 0.3), 30.0))
    mb.add("white_box", 2, *_box((0.0, 0.55, 0.1), (0.25, 0.25, 0.25), -20.0))
    tex = np.zeros((16, 16, 4), np.uint8)
    yy, xx = np.mgrid[0:16, 0:16]
    tex[..., 0] = np.where((xx // 4 + yy // 4) % 2, 220, 40)
    tex[..., 1] = (rng.uniform(0, 1, (16, 16)) * 255).astype(np.uint8)
    tex[..., 2] = 128
    tex[..., 3] = 255
    return _finish(mb, mats, [tex], CORNELL_CAMERA, width, height, spp, max_depth)


WORKLOADS = {
    "cornell_box": cornell_box,
    "mixed_mid": mixed_mid,
    "large_textured": large_textured,
    "batched_views": batched_views,
    "material_inversion": material_inversion,
}


# ---------------------------------------------------------------------------
# texels: stbi_loadf's 8-bit -> float conversion
# ---------------------------------------------------------------------------
def texel_table() -> np.ndarray:
    """float32 value of each byte as stbi_loadf returns it:
    (float)pow(b / 255.0f, 2.2f) (stb_image.h ldr_to_hdr)."""
    b = np.arange(256, dtype=np.float32) / np.float32(255.0)
    return np.power(b.astype(np.float64), np.float64(np.float32(2.2))).astype(np.float32)


def texture_texels(img: np.ndarray) -> np.ndarray:
    """RGBA8 [h, w, 4] -> float32 [h*w, 3] linear texels (alpha dropped)."""
    return texel_table()[img[..., :3].reshape(-1, 3)]


# ---------------------------------------------------------------------------
# reference-format writers
# ---------------------------------------------------------------------------
def _png_bytes(img: np.ndarray) -> bytes:
    h, w, c = img.shape
    raw = b"".join(b"\x00" + img[y].tobytes() for y in range(h))

    def chunk(tag, data):
        return (struct.pack(">I", len(data)) + tag + data +
                struct.pack(">I", zlib.crc32(tag + data) & 0xFFFFFFFF))

    color = {3: 2, 4: 6}[c]
    return (b"\x89PNG\r\n\x1a\n" + chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, 8, color, 0, 0, 0)) +
            chunk(b"IDAT", zlib.compress(raw, 6)) + chunk(b"IEND", b""))


def write_png(path: str, img: np.ndarray) -> None:
    with open(path, "wb") as f:
        f.write(_png_bytes(np.ascontiguousarray(img, np.uint8)))


def _f(x) -> str:
    return repr(float(np.float32(x)))


def write_reference_files(sc: SceneArrays, out_dir: str, name: str) -> dict:
    """Write <name>.obj/.mtl, <name>-camera.json and textures/ so that
    CudaRT's loaders (obj_load.h, json_loader.cpp, texture_store.cpp) read
    the same scene.  Scenes without textures get one unused 2x2 texture
    because the reference's texture store needs at least one."""
    os.makedirs(out_dir, exist_ok=True)
    tex_dir = os.path.join(out_dir, "textures")
    os.makedirs(tex_dir, exist_ok=True)
    tex_names = []
    for k, img in enumerate(sc.textures):
        fn = f"{name}_tex{k}.png"
        write_png(os.path.join(tex_dir, fn), img)
        tex_names.append(fn)
    lines = []
    for m in sc.materials:
        lines += [f"newmtl {m.name}", "Kd " + " ".join(_f(v) for v in m.kd),
                  "Ka " + " ".join(_f(v) for v in m.ka), "Ks " + " ".join(_f(v) for v in m.ks),
                  f"Ns {_f(m.ns)}", f"Ni {_f(m.ni)}", f"type {BSDF_NAMES[m.bsdf]}",
                  f"diffuse {_f(m.diffuse)}"]
        if m.tex != NO_TEXTURE:
            lines.append(f"map_Kd {tex_names[m.tex]}")
    if not sc.textures:
        write_png(os.path.join(tex_dir, "unused_2x2.png"), np.full((2, 2, 4), 255, np.uint8))
        lines += ["newmtl unused_textured", "Kd 1 1 1", "type LAMBERT", "map_Kd unused_2x2.png"]
    with open(os.path.join(out_dir, name + ".mtl"), "w") as f:
        f.write("\n".join(lines) + "\n")
    with open(os.path.join(out_dir, name + ".obj"), "w") as f:
        f.write(f"mtllib {name}.mtl\n")
        vbase = 1
        for gname, mat, first, count in sc.groups:
            f.write(f"g {gname}\nusemtl {sc.materials[mat].name}\n")
            P = sc.positions[first:first + count].reshape(-1, 3)
            N = sc.normals[first:first + count].reshape(-1, 3)
            T = sc.uvs[first:first + count].reshape(-1, 2)
            f.write("".join(f"v {_f(p[0])} {_f(p[1])} {_f(p[2])}\n" for p in P))
            f.write("".join(f"vt {_f(t[0])} {_f(t[1])}\n" for t in T))
            f.write("".join(f"vn {_f(n[0])} {_f(n[1])} {_f(n[2])}\n" for n in N))
            rows = []
            for k in range(count):
                i = vbase + 3 * k
                rows.append(f"f {i}/{i}/{i} {i + 1}/{i + 1}/{i + 1} {i + 2}/{i + 2}/{i + 2}\n")
            f.write("".join(rows))
            vbase += 3 * count
    cam = sc.camera
    with open(os.path.join(out_dir, name + "-camera.json"), "w") as f:
        json.dump({"fieldOfView": cam.fov_deg, "focalLength": cam.focal_length,
                   "fStop": cam.fstop, "eye": list(map(float, cam.eye)),
                   "viewDirection": list(map(float, cam.view_dir)),
                   "upDirection": list(map(float, cam.up))}, f)
    return {"obj": os.path.join(out_dir, name + ".obj"),
            "camera": os.path.join(out_dir, name + "-camera.json"),
            "textures": tex_dir + "/"}
