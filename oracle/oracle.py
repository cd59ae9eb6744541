"""ctypes binding of the CPU oracle (liborc.so) and of the reference pinning
harness (_ref/libcrt_ref.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and
bench.py's CPU-baseline leg.  The GB300 library never imports it.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from typing import Optional, Sequence

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liborc.so")
REF_LIB_PATH = os.path.join(HERE, "_ref", "libcrt_ref.so")
# The reference with its traversal stack raised to 64 entries and its bounce
# count set to 8 (oracle/Makefile, target ref-deep): the estimator the depth-8
# workloads run, on trees deeper than the shipped 16-entry stack allows.
REF_DEEP_LIB_PATH = os.path.join(HERE, "_ref", "libcrt_ref_s64_d8.so")


def reference_root() -> Optional[str]:
    """The CudaRT project root named by the environment variable CUDART_REF
    (the reference harness is built only where it is set and holds the
    sources)."""
    root = os.environ.get("CUDART_REF", "")
    return root if root and os.path.isdir(os.path.join(root, "src", "renderer")) else None

TRI_DT = np.dtype([("v1", "<f4", 3), ("e1", "<f4", 3), ("e2", "<f4", 3), ("n1", "<f4", 3),
                   ("n2", "<f4", 3), ("n3", "<f4", 3), ("uv", "<f4", 6), ("area", "<f4"),
                   ("material", "<u4")])
MAT_DT = np.dtype([("kd", "<f4", 3), ("ka", "<f4", 3), ("ks", "<f4", 3), ("ns", "<f4"),
                   ("ni", "<f4"), ("diffuse", "<f4"), ("bsdf", "<i4"), ("tex", "<i4")])
CAM_DT = np.dtype([("eye", "<f4", 3), ("dir", "<f4", 3), ("up", "<f4", 3), ("right", "<f4", 3),
                   ("fov", "<f4"), ("aspect", "<f4"), ("aperture", "<f4"), ("focus", "<f4"),
                   ("xpixels", "<i4"), ("ypixels", "<i4")])
NODE_DT = np.dtype([("bmin", "<f4", 3), ("bmax", "<f4", 3), ("offset", "<i4"), ("ntris", "<i2"),
                    ("axis", "<i2")])


class _Scene(C.Structure):
    _fields_ = [("n_tris", C.c_uint32), ("tris", C.c_void_p), ("n_mats", C.c_uint32),
                ("mats", C.c_void_p), ("n_lights", C.c_uint32), ("lights", C.c_void_p),
                ("lights_area", C.c_float), ("n_tex", C.c_uint32), ("tex_dims", C.c_void_p),
                ("tex_offsets", C.c_void_p), ("tex_data", C.c_void_p), ("tex_total", C.c_uint32),
                ("n_nodes", C.c_uint32), ("nodes", C.c_void_p), ("tri_perm", C.c_void_p)]


def build(quiet: bool = True) -> None:
    """Compile liborc.so (and the reference harness when the CudaRT sources
    are present on this machine)."""
    out = subprocess.DEVNULL if quiet else None
    subprocess.check_call(["make", "-C", HERE, "-s", "all"], stdout=out)
    root = reference_root()
    if root is not None:
        subprocess.check_call(["make", "-C", HERE, "-s", "-j8", "REF=" + root, "ref", "ref-deep"],
                              stdout=out)


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = C.CDLL(LIB_PATH)
        P = C.c_void_p
        L.orc_philox4x32_10.argtypes = [P, P, P]
        L.orc_prepare_tris.argtypes = [P, P, P, P, C.c_uint32, P]
        L.orc_lights_area.argtypes = [P, P, C.c_uint32]
        L.orc_lights_area.restype = C.c_float
        L.orc_make_material.argtypes = [P, C.c_int32, C.c_int32, P, P, P, C.c_float, C.c_float,
                                        C.c_float, C.c_float]
        L.orc_make_camera.argtypes = [P, C.c_float, C.c_float, C.c_float, P, P, P, C.c_uint32,
                                      C.c_uint32]
        L.orc_bvh_build.argtypes = [P, C.c_uint32, P, P]
        L.orc_bvh_build.restype = C.c_uint32
        L.orc_closest_hit_brute.argtypes = [P, P, C.c_uint32, P, P, P]
        L.orc_closest_hit_bvh.argtypes = [P, P, C.c_uint32, P, P, P, C.c_int]
        L.orc_traversal_counts.argtypes = [P, P, C.c_uint32, P, P]
        L.orc_render.argtypes = [P, P, C.c_uint64, C.c_uint32, C.c_uint32, C.c_uint32,
                                 C.c_uint32, P, C.c_uint32, P, P, P, C.c_int]
        L.orc_adjoint.argtypes = [P, P, C.c_uint64, C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32,
                                  P, C.c_uint32, P, P, C.c_int, C.c_int]
        L.orc_resolve.argtypes = [P, C.c_uint32, C.c_uint32, P]
        L.orc_gamma_u8.argtypes = [C.c_uint8]
        L.orc_gamma_u8.restype = C.c_uint8
        _lib = L
    return _lib


def _p(a: np.ndarray):
    return a.ctypes.data_as(C.c_void_p)


def philox(ctr: Sequence[int], key: Sequence[int]) -> np.ndarray:
    c = np.asarray(ctr, np.uint32)
    k = np.asarray(key, np.uint32)
    out = np.zeros(4, np.uint32)
    lib().orc_philox4x32_10(_p(c), _p(k), _p(out))
    return out


def make_camera(cam, width: int, height: int) -> np.ndarray:
    c = np.zeros(1, CAM_DT)
    f3 = lambda v: np.asarray(v, np.float32)
    eye, vd, up = f3(cam.eye), f3(cam.view_dir), f3(cam.up)
    lib().orc_make_camera(_p(c), cam.fov_deg, cam.focal_length, cam.fstop, _p(eye), _p(vd),
                          _p(up), width, height)
    return c


class OracleScene:
    """A scene prepared the way the reference's Scene class prepares it
    (scene.cpp:74-165), plus the oracle's binary BVH."""

    def __init__(self, sc=None, *, tris=None, mats=None, lights=None, lights_area=None,
                 tex_dims=None, tex_offsets=None, tex_data=None, build_bvh=True):
        """From SceneArrays `sc` (lights: optional pick order of emissive
        faces, default face order), or from prepared arrays."""
        L = lib()
        if sc is not None:
            n = sc.n_tris
            tris = np.zeros(n, TRI_DT)
            pos = np.ascontiguousarray(sc.positions, np.float32)
            nor = np.ascontiguousarray(sc.normals, np.float32)
            uv = np.ascontiguousarray(sc.uvs, np.float32)
            mid = np.ascontiguousarray(sc.material_ids, np.uint32)
            L.orc_prepare_tris(_p(pos), _p(nor), _p(uv), _p(mid), n, _p(tris))
            lights = (np.ascontiguousarray(lights, np.uint32) if lights is not None
                      else sc.light_indices())
            lights_area = float(L.orc_lights_area(_p(tris), _p(lights), len(lights)))
            mats = np.zeros(len(sc.materials), MAT_DT)
            for i, m in enumerate(sc.materials):
                kd = np.asarray(m.kd, np.float32); ka = np.asarray(m.ka, np.float32)
                ks = np.asarray(m.ks, np.float32)
                L.orc_make_material(_p(mats[i:i + 1]), m.bsdf, m.tex, _p(kd), _p(ka), _p(ks),
                                    m.ns, m.ni, m.diffuse, lights_area)
            from cudart_gb300.scenes import texture_texels
            dims, offs, data, total = [], [], [], 0
            for img in sc.textures:
                h, w = img.shape[:2]
                dims += [w, h]
                offs.append(total)
                data.append(texture_texels(img))
                total += w * h
            if sc.textures:
                data.append(np.zeros((sc.textures[-1].shape[1], 3), np.float32))
            tex_dims = np.asarray(dims, np.uint32)
            tex_offsets = np.asarray(offs, np.uint32)
            tex_data = (np.concatenate(data).astype(np.float32) if data
                        else np.zeros((0, 3), np.float32))
        self.tris = np.ascontiguousarray(tris)
        self.mats = np.ascontiguousarray(mats)
        self.lights = np.ascontiguousarray(lights, np.uint32)
        self.lights_area = np.float32(lights_area)
        self.tex_dims = np.ascontiguousarray(tex_dims if tex_dims is not None else [], np.uint32)
        self.tex_offsets = np.ascontiguousarray(tex_offsets if tex_offsets is not None else [],
                                                np.uint32)
        self.tex_data = np.ascontiguousarray(tex_data if tex_data is not None
                                             else np.zeros((0, 3)), np.float32)
        n = len(self.tris)
        self.nodes = np.zeros(max(2 * n - 1, 1), NODE_DT)
        self.perm = np.zeros(max(n, 1), np.uint32)
        n_nodes = L.orc_bvh_build(_p(self.tris), n, _p(self.nodes), _p(self.perm)) if build_bvh else 0
        self.nodes = self.nodes[:max(n_nodes, 1)].copy()
        self.n_nodes = n_nodes
        self._s = _Scene(n, self.tris.ctypes.data, len(self.mats), self.mats.ctypes.data,
                         len(self.lights), self.lights.ctypes.data, float(self.lights_area),
                         len(self.tex_dims) // 2, self.tex_dims.ctypes.data,
                         self.tex_offsets.ctypes.data, self.tex_data.ctypes.data,
                         len(self.tex_data), n_nodes, self.nodes.ctypes.data,
                         self.perm.ctypes.data)

    @property
    def ptr(self):
        return C.byref(self._s)

    def closest_hit(self, rays: np.ndarray, brute: bool = False, threads: int = 0):
        rays = np.ascontiguousarray(rays, np.float32).reshape(-1, 8)
        n = len(rays)
        idx = np.zeros(n, np.int32)
        t = np.zeros(n, np.float32)
        uv = np.zeros((n, 2), np.float32)
        if brute:
            lib().orc_closest_hit_brute(self.ptr, _p(rays), n, _p(idx), _p(t), _p(uv))
        else:
            lib().orc_closest_hit_bvh(self.ptr, _p(rays), n, _p(idx), _p(t), _p(uv), threads)
        return idx, t, uv

    def traversal_counts(self, rays: np.ndarray):
        rays = np.ascontiguousarray(rays, np.float32).reshape(-1, 8)
        nv = np.zeros(len(rays), np.uint32)
        nt = np.zeros(len(rays), np.uint32)
        lib().orc_traversal_counts(self.ptr, _p(rays), len(rays), _p(nv), _p(nt))
        return nv, nt

    def render(self, camera: np.ndarray, seed: int, spp: int, max_depth: int, *, view: int = 0,
               spp0: int = 0, pixels: Optional[np.ndarray] = None, threads: int = 0,
               acc: Optional[np.ndarray] = None):
        """Returns (acc float32 [n,3], mean float64 [n,3], m2 float64 [n,3])."""
        W, H = int(camera["xpixels"][0]), int(camera["ypixels"][0])
        npx = len(pixels) if pixels is not None else W * H
        px = np.ascontiguousarray(pixels, np.uint32) if pixels is not None else None
        acc = np.zeros((npx, 3), np.float32) if acc is None else np.ascontiguousarray(acc, np.float32)
        mean = np.zeros((npx, 3), np.float64)
        m2 = np.zeros((npx, 3), np.float64)
        lib().orc_render(self.ptr, _p(camera), seed, view, spp0, spp, max_depth,
                         _p(px) if px is not None else None, npx, _p(acc), _p(mean), _p(m2),
                         threads)
        return acc, mean, m2

    def adjoint(self, camera: np.ndarray, seed: int, spp: int, max_depth: int, adjoint: np.ndarray,
                *, view: int = 0, spp0: int = 0, exact_roulette: bool = False, threads: int = 0):
        """FP64 reference gradient of sum(adjoint * radiance sum of samples
        [spp0, spp0+spp)) w.r.t. each material's kd and ka: (grad_kd,
        grad_ka), float64 [n_mats, 3].  adjoint: [W*H, 3]."""
        W, H = int(camera["xpixels"][0]), int(camera["ypixels"][0])
        adj = np.ascontiguousarray(adjoint, np.float32).reshape(W * H, 3)
        n = len(self.mats)
        gkd = np.zeros((n, 3), np.float64)
        gka = np.zeros((n, 3), np.float64)
        lib().orc_adjoint(self.ptr, _p(camera), seed, view, spp0, spp, max_depth, _p(adj), n,
                          _p(gkd), _p(gka), int(exact_roulette), threads)
        return gkd, gka


def resolve(acc: np.ndarray, spp: int) -> np.ndarray:
    acc = np.ascontiguousarray(acc, np.float32).reshape(-1, 3)
    out = np.zeros((len(acc), 4), np.uint8)
    lib().orc_resolve(_p(acc), len(acc), spp, _p(out))
    return out


def gamma_table() -> np.ndarray:
    return np.array([lib().orc_gamma_u8(v) for v in range(256)], np.uint8)


def scene_from_export(e: dict) -> "OracleScene":
    """Oracle scene from the reference's exported state (RefHarness.export()
    or the ref_* arrays of a golden fixture with the prefix removed)."""
    t = e["tris"]
    tris = np.zeros(len(t), TRI_DT)
    for k, name in enumerate(["v1", "e1", "e2", "n1", "n2", "n3"]):
        tris[name] = t[:, 3 * k:3 * k + 3]
    tris["uv"] = t[:, 18:24]
    tris["area"] = t[:, 24]
    tris["material"] = e["mat_ids"]
    mf, mi = e["mat_floats"], e["mat_ints"]
    mats = np.zeros(len(mf), MAT_DT)
    mats["kd"], mats["ka"], mats["ks"] = mf[:, 0:3], mf[:, 3:6], mf[:, 6:9]
    mats["ns"], mats["ni"], mats["diffuse"] = mf[:, 9], mf[:, 10], mf[:, 11]
    mats["bsdf"], mats["tex"] = mi[:, 0], mi[:, 1]
    return OracleScene(tris=tris, mats=mats, lights=e["lights"], lights_area=float(e["lights_area"]),
                       tex_dims=e["tex_dims"], tex_offsets=e["tex_offsets"], tex_data=e["tex_data"])


def camera_from_export(e: dict) -> np.ndarray:
    c = np.zeros(1, CAM_DT)
    cam = e["camera"]
    c["eye"], c["dir"], c["up"], c["right"] = cam[0:3], cam[3:6], cam[6:9], cam[9:12]
    c["fov"], c["aspect"], c["aperture"], c["focus"] = cam[12], cam[13], cam[14], cam[15]
    c["xpixels"], c["ypixels"] = e["pixels"]
    return c


# ---------------------------------------------------------------------------
# reference harness (this machine only: needs the CudaRT sources to build)
# ---------------------------------------------------------------------------
class RefHarness:
    """The reference's own scene loader, traversal and estimator, loaded
    through oracle/_ref/libcrt_ref.so.  One scene per process."""

    def __init__(self, files: dict, width: int, height: int, deep: bool = False):
        """deep: load the ref-deep build (64-entry stack, 8 bounces) instead
        of the one compiled as shipped (16 entries, 6 bounces)."""
        L = C.CDLL(REF_DEEP_LIB_PATH if deep else REF_LIB_PATH)
        P = C.c_void_p
        L.ref_load.argtypes = [C.c_char_p, C.c_char_p, C.c_char_p, C.c_int, C.c_int]
        L.ref_counts.argtypes = [P]
        L.ref_export_tris.argtypes = [P, P]
        L.ref_export_materials.argtypes = [P, P]
        L.ref_export_lights.argtypes = [P]
        L.ref_export_lights.restype = C.c_float
        L.ref_export_camera.argtypes = [P, P]
        L.ref_export_textures.argtypes = [P, P, P]
        L.ref_closest_hit.argtypes = [P, C.c_uint32, P, P, P]
        L.ref_sample_pixel.argtypes = [C.c_int, C.c_int, C.c_uint64, C.c_uint32, C.c_uint32, P]
        L.ref_sample_pixel.restype = C.c_uint32
        L.ref_render.argtypes = [P, C.c_uint32, C.c_uint64, C.c_uint32, C.c_uint32, C.c_uint32,
                                 P, P, P]
        L.ref_gamma_table.argtypes = [P]
        L.ref_quantise.argtypes = [P, C.c_uint32, C.c_uint32, P]
        L.ref_limits.argtypes = [P]
        lim = np.zeros(2, np.uint32)
        L.ref_limits(_p(lim))
        self.stack_entries, self.max_depth = int(lim[0]), int(lim[1])
        self.L = L
        n = L.ref_load(files["obj"].encode(), files["camera"].encode(),
                       files["textures"].encode(), width, height)
        if n < 0:
            raise RuntimeError("reference failed to load the scene")
        c = np.zeros(8, np.uint32)
        L.ref_counts(_p(c))
        (self.n_tris, self.n_nodes, self.n_mats, self.n_lights, self.n_tex, self.bvh_depth,
         self.texels, self.pad) = map(int, c)
        self.width, self.height = width, height

    # intersectBVH keeps `int stack[16]` (renderer.cu:289; 64 in the deep
    # build); a traversal holds at most one entry per level below the root, so
    # renders refuse trees deeper than the stack instead of smashing it.
    def _check_depth(self):
        if self.bvh_depth > self.stack_entries:
            raise RuntimeError(f"reference BVH depth {self.bvh_depth} overflows its "
                               f"{self.stack_entries}-entry traversal stack")

    def export(self):
        L = self.L
        t = np.zeros((self.n_tris, 25), np.float32)
        mid = np.zeros(self.n_tris, np.uint32)
        L.ref_export_tris(_p(t), _p(mid))
        mf = np.zeros((max(self.n_mats, 1), 12), np.float32)
        mi = np.zeros((max(self.n_mats, 1), 2), np.int32)
        L.ref_export_materials(_p(mf), _p(mi))
        lights = np.zeros(max(self.n_lights, 1), np.uint32)
        lsa = float(L.ref_export_lights(_p(lights)))
        cam = np.zeros(16, np.float32)
        px = np.zeros(2, np.int32)
        L.ref_export_camera(_p(cam), _p(px))
        dims = np.zeros(max(2 * self.n_tex, 1), np.uint32)
        offs = np.zeros(max(self.n_tex, 1), np.uint32)
        tex = np.zeros((self.texels + self.pad, 3), np.float32)
        L.ref_export_textures(_p(dims), _p(offs), _p(tex))
        return dict(tris=t, mat_ids=mid, mat_floats=mf[:self.n_mats], mat_ints=mi[:self.n_mats],
                    lights=lights[:self.n_lights], lights_area=lsa, camera=cam, pixels=px,
                    tex_dims=dims[:2 * self.n_tex], tex_offsets=offs[:self.n_tex], tex_data=tex)

    def oracle_scene(self) -> "OracleScene":
        """The reference's loaded scene state as an oracle scene."""
        return scene_from_export(self.export())

    def camera(self) -> np.ndarray:
        return camera_from_export(self.export())

    def closest_hit(self, rays: np.ndarray):
        rays = np.ascontiguousarray(rays, np.float32).reshape(-1, 8)
        n = len(rays)
        idx = np.zeros(n, np.int32); t = np.zeros(n, np.float32); uv = np.zeros((n, 2), np.float32)
        self.L.ref_closest_hit(_p(rays), n, _p(idx), _p(t), _p(uv))
        return idx, t, uv

    def sample_pixel(self, x: int, y: int, seed: int, sample: int, view: int = 0):
        self._check_depth()
        rgb = np.zeros(3, np.float32)
        n = self.L.ref_sample_pixel(x, y, seed, view, sample, _p(rgb))
        return rgb, int(n)

    def render(self, pixels: np.ndarray, seed: int, spp: int, spp0: int = 0, view: int = 0):
        self._check_depth()
        px = np.ascontiguousarray(pixels, np.uint32)
        acc = np.zeros((len(px), 3), np.float32)
        mean = np.zeros((len(px), 3), np.float64)
        m2 = np.zeros((len(px), 3), np.float64)
        self.L.ref_render(_p(px), len(px), seed, view, spp0, spp, _p(acc), _p(mean), _p(m2))
        return acc, mean, m2

    def gamma_table(self) -> np.ndarray:
        out = np.zeros(256, np.uint8)
        self.L.ref_gamma_table(_p(out))
        return out
