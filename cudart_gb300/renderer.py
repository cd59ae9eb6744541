"""Host-side mirror of CudaRT's renderer interface over the GB300 C ABI.

`GB300Renderer` follows the reference's abstract `Renderer`
(src/include/renderer.h:78-100): construct it with a scene, width, height
and samples; call `render_one_sample_per_pixel()` once per pass (or
`render(n)`), then `copy_image_bytes()` for the gamma-corrected RGBA8 image
(parallel_renderer.cu:303-310).  `GB300Scene` wraps the scene handle and the
batched closest-hit query.
"""
from __future__ import annotations

import ctypes as C
from typing import Optional

import numpy as np

from . import _lib
from ._lib import Camera, Material, RenderOptions, SceneDesc, SceneInfo, check, load
from .scenes import NO_TEXTURE, SceneArrays, texture_texels

NODE_DT = np.dtype([("p", "<f4", 3), ("e", "u1", 3), ("imask", "u1"), ("child_base", "<u4"),
                    ("tri_base", "<u4"), ("meta", "u1", 8), ("qlo", "u1", (3, 8)),
                    ("qhi", "u1", (3, 8))])
TRI_DT = np.dtype([("v1", "<f4", 3), ("face", "<u4"), ("e1", "<f4", 3), ("pad1", "<f4"),
                   ("e2", "<f4", 3), ("pad2", "<f4")])
assert NODE_DT.itemsize == 80 and TRI_DT.itemsize == 48


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(C.c_void_p)


def camera_from_json(spec, width: int, height: int) -> Camera:
    """CameraJsonLoader::getCamera (json_loader.cpp:26-48) for a CameraSpec."""
    cam = Camera()
    f3 = lambda v: np.ascontiguousarray(v, np.float32)
    eye, vd, up = f3(spec.eye), f3(spec.view_dir), f3(spec.up)
    check(load().crt_camera_from_json(spec.fov_deg, spec.focal_length, spec.fstop, _ptr(eye),
                                      _ptr(vd), _ptr(up), width, height, C.byref(cam)))
    return cam


def bvh_build_host(positions: np.ndarray):
    """Host-only 8-wide BVH build: (nodes, triangle records, max depth)."""
    pos = np.ascontiguousarray(positions, np.float32).reshape(-1, 9)
    n = len(pos)
    nn, depth = C.c_uint32(0), C.c_uint32(0)
    L = load()
    check(L.crt_bvh_build_host(_ptr(pos), n, C.byref(nn), C.byref(depth), None, None))
    nodes = np.zeros(nn.value, NODE_DT)
    tris = np.zeros(n, TRI_DT)
    check(L.crt_bvh_build_host(_ptr(pos), n, C.byref(nn), C.byref(depth), _ptr(nodes), _ptr(tris)))
    return nodes, tris, depth.value


class GB300Scene:
    """Scene handle: BVH, triangles, materials, lights and textures on the GPU."""

    def __init__(self, sc: SceneArrays, lights: Optional[np.ndarray] = None,
                 node_format: str = "q8"):
        L = load()
        self.arrays = sc
        self._keep = []
        pos = np.ascontiguousarray(sc.positions, np.float32)
        nor = np.ascontiguousarray(sc.normals, np.float32)
        uvs = np.ascontiguousarray(sc.uvs, np.float32)
        mid = np.ascontiguousarray(sc.material_ids, np.uint32)
        mats = (Material * len(sc.materials))()
        for i, m in enumerate(sc.materials):
            mats[i].bsdf = m.bsdf
            mats[i].texture = m.tex if m.tex is not None else NO_TEXTURE
            mats[i].kd[:] = list(map(float, m.kd))
            mats[i].ka[:] = list(map(float, m.ka))
            mats[i].ks[:] = list(map(float, m.ks))
            mats[i].ns, mats[i].ni, mats[i].diffuse = m.ns, m.ni, m.diffuse
        dims = np.asarray([d for img in sc.textures for d in (img.shape[1], img.shape[0])], np.uint32)
        texels = (np.concatenate([texture_texels(img) for img in sc.textures]).astype(np.float32)
                  if sc.textures else np.zeros((1, 3), np.float32))
        li = (np.ascontiguousarray(lights, np.uint32) if lights is not None
              else np.zeros(1, np.uint32))
        self._keep += [pos, nor, uvs, mid, mats, dims, texels, li]
        desc = SceneDesc(sc.n_tris, pos.ctypes.data, nor.ctypes.data, uvs.ctypes.data,
                         mid.ctypes.data, len(sc.materials), C.addressof(mats),
                         len(lights) if lights is not None else 0,
                         li.ctypes.data if lights is not None else None,
                         len(sc.textures), dims.ctypes.data if len(dims) else None,
                         texels.ctypes.data, {"q8": _lib.NODES_Q8, "f32": _lib.NODES_F32}[node_format])
        self.node_format = node_format
        h = C.c_void_p()
        check(L.crt_scene_create(C.byref(desc), C.byref(h)))
        self.handle = h
        self._keep = None

    def __del__(self):
        if getattr(self, "handle", None):
            load().crt_scene_destroy(self.handle)
            self.handle = None

    @property
    def info(self) -> SceneInfo:
        inf = SceneInfo()
        check(load().crt_scene_get_info(self.handle, C.byref(inf)))
        return inf

    def export_bvh(self):
        inf = self.info
        nodes = np.zeros(inf.num_nodes, NODE_DT)
        tris = np.zeros(inf.num_triangles, TRI_DT)
        check(load().crt_scene_export_bvh(self.handle, _ptr(nodes), _ptr(tris)))
        return nodes, tris

    def trace_closest(self, rays, stream=None):
        """rays: CUDA float32 tensor [n, 8] -> (face int32, t float32, uv float32 [n,2])."""
        import torch
        rays = rays.contiguous()
        n = rays.shape[0]
        idx = torch.empty(n, dtype=torch.int32, device=rays.device)
        t = torch.empty(n, dtype=torch.float32, device=rays.device)
        uv = torch.empty((n, 2), dtype=torch.float32, device=rays.device)
        s = stream if stream is not None else torch.cuda.current_stream(rays.device).cuda_stream
        check(load().crt_trace_closest(self.handle, rays.data_ptr(), n, idx.data_ptr(), t.data_ptr(),
                                       uv.data_ptr(), s))
        return idx, t, uv

    def trace_counts(self, rays, stream=None):
        import torch
        rays = rays.contiguous()
        n = rays.shape[0]
        nodes = torch.empty(n, dtype=torch.int32, device=rays.device)
        tris = torch.empty(n, dtype=torch.int32, device=rays.device)
        s = stream if stream is not None else torch.cuda.current_stream(rays.device).cuda_stream
        check(load().crt_trace_counts(self.handle, rays.data_ptr(), n, nodes.data_ptr(),
                                      tris.data_ptr(), s))
        return nodes, tris


class GB300Renderer:
    """Drop-in for ParallelRenderer (renderer.h:102-126) over the C ABI."""

    def __init__(self, scene: GB300Scene, width: int, height: int, samples: int,
                 camera: Optional[Camera] = None, max_depth: int = 6, seed: int = 1234,
                 mode: str = "megakernel", view_id: int = 0, wave_paths: int = 0,
                 flags: int = 0):
        L = load()
        self.scene = scene
        self.width, self.height, self.samples = width, height, samples
        if camera is None:
            camera = camera_from_json(scene.arrays.camera, width, height)
        self.camera = camera
        opts = RenderOptions()
        L.crt_render_options_default(C.byref(opts))
        opts.max_depth = max_depth
        opts.seed = seed
        opts.view_id = view_id
        opts.mode = {"megakernel": _lib.MODE_MEGAKERNEL, "wavefront": _lib.MODE_WAVEFRONT}[mode]
        opts.wave_paths = wave_paths
        opts.flags = flags
        h = C.c_void_p()
        check(L.crt_render_create(scene.handle, C.byref(camera), width, height, C.byref(opts),
                                  C.byref(h)))
        self.handle = h

    def __del__(self):
        if getattr(self, "handle", None):
            load().crt_render_destroy(self.handle)
            self.handle = None

    # Renderer interface (renderer.h:83-91)
    def render_one_sample_per_pixel(self) -> None:
        check(load().crt_render_pass(self.handle, 1))

    def render(self, n_spp: Optional[int] = None) -> None:
        check(load().crt_render_pass(self.handle, self.samples if n_spp is None else n_spp))

    def copy_image_bytes(self) -> np.ndarray:
        out = np.zeros((self.height, self.width, 4), np.uint8)
        check(load().crt_render_resolve(self.handle, _ptr(out)))
        return out

    def get_width(self) -> int:
        return self.width

    def get_height(self) -> int:
        return self.height

    def get_samples(self) -> int:
        return self.samples

    def get_samples_rendered(self) -> int:
        v = C.c_uint32(0)
        check(load().crt_render_samples_rendered(self.handle, C.byref(v)))
        return v.value

    # extensions
    def accum(self) -> np.ndarray:
        out = np.zeros((self.height * self.width, 3), np.float32)
        check(load().crt_render_accum(self.handle, _ptr(out)))
        return out

    def accum_device_ptr(self) -> int:
        p = C.c_void_p()
        check(load().crt_render_accum_device(self.handle, C.byref(p)))
        return p.value

    def synchronize(self) -> None:
        check(load().crt_render_synchronize(self.handle))

    def reset(self) -> None:
        check(load().crt_render_reset(self.handle))

    def set_camera(self, camera: Camera) -> None:
        check(load().crt_render_set_camera(self.handle, C.byref(camera)))
        self.camera = camera

    def set_stream(self, stream: int) -> None:
        check(load().crt_render_set_stream(self.handle, stream))

    def profile_pass(self, n_spp: int) -> dict:
        """Wavefront pass with per-stage CUDA-event timing and traversal counts."""
        p = _lib.StageProfile()
        check(load().crt_render_profile_pass(self.handle, n_spp, C.byref(p)))
        out = {f"{s}_ms": p.ms[i] for i, s in enumerate(p.STAGES)}
        out.update({f"{s}_launches": p.launches[i] for i, s in enumerate(p.STAGES)})
        for f in ("extension_rays", "extension_nodes", "extension_tris", "shadow_rays",
                  "shadow_nodes", "shadow_tris"):
            out[f] = getattr(p, f)
        return out

    def ray_counts(self):
        e, s = C.c_uint64(0), C.c_uint64(0)
        check(load().crt_render_ray_counts(self.handle, C.byref(e), C.byref(s)))
        return e.value, s.value
