"""Scene files through the library's own readers (crt_scene_files_*,
crt_camera_load_json, crt_texture_load_png, crt_image_write_png).

The reference reads the same files with objl::Loader (src/include/
obj_load.h), CameraJsonLoader (src/context/json_loader.cpp) and stb_image
(src/context/texture_store.cpp), and writes its output with stb's PNG writer
(src/context/launcher.cpp:13-21).
"""
from __future__ import annotations

import ctypes as C
import os
from typing import List, Tuple

import numpy as np

from . import _lib
from ._lib import Camera, SceneDesc, SceneFilesInfo, check, load
from .scenes import Material


def _array(addr: int, ctype, count: int, dtype) -> np.ndarray:
    if count == 0:
        return np.zeros(0, dtype)
    return np.ctypeslib.as_array((ctype * count).from_address(addr)).astype(dtype, copy=True)


class SceneFiles:
    """A scene read from `<name>.obj` (+ its MTL libraries and PNG textures).

    Arrays are host copies in face order: positions/normals [n, 3, 3], uvs
    [n, 3, 2], material_ids [n]; `materials` is the material table
    (scenes.Material, ka = the MTL Ka); `texture_dims` [t, 2] (w, h) and
    `texels` [sum w*h, 3] hold the linear texels.  GB300Scene(files) uploads
    the scene straight from the library's own buffers.
    """

    def __init__(self, obj_path: str, texture_dir: str = "", exact_materials: bool = False):
        L = load()
        h = C.c_void_p()
        flags = _lib.LOAD_EXACT_MATERIALS if exact_materials else 0
        check(L.crt_scene_files_load(os.fsencode(obj_path), os.fsencode(texture_dir), flags,
                                     C.byref(h)))
        self.handle = h
        self.path = obj_path
        self.info = SceneFilesInfo()
        check(L.crt_scene_files_get_info(h, C.byref(self.info)))
        d = self.desc()
        n = d.num_triangles
        self.positions = _array(d.positions, C.c_float, 9 * n, np.float32).reshape(n, 3, 3)
        self.normals = _array(d.normals, C.c_float, 9 * n, np.float32).reshape(n, 3, 3)
        self.uvs = _array(d.uvs, C.c_float, 6 * n, np.float32).reshape(n, 3, 2)
        self.material_ids = _array(d.material_ids, C.c_uint32, n, np.uint32)
        mats = (_lib.Material * d.num_materials).from_address(d.materials)
        self.materials: List[Material] = [
            Material(f"m{i}", int(m.bsdf), tuple(m.kd), tuple(m.ka), tuple(m.ks), float(m.ns),
                     float(m.ni), float(m.diffuse), int(m.texture))
            for i, m in enumerate(mats)]
        t = d.num_textures
        self.texture_dims = _array(d.texture_dims, C.c_uint32, 2 * t, np.uint32).reshape(t, 2)
        n_texels = int(self.texture_dims.prod(axis=1).sum()) if t else 0
        self.texels = (_array(d.texels, C.c_float, 3 * n_texels, np.float32).reshape(n_texels, 3)
                       if n_texels else np.zeros((0, 3), np.float32))

    def desc(self) -> SceneDesc:
        """crt_scene_desc pointing into the library's arrays (valid while
        this object lives)."""
        d = SceneDesc()
        check(load().crt_scene_files_desc(self.handle, C.byref(d)))
        return d

    @property
    def n_tris(self) -> int:
        return int(self.info.num_triangles)

    def meshes(self) -> List[Tuple[str, int, int]]:
        """(name, first triangle, triangle count) per mesh, in file order."""
        out = []
        name, first, count = C.c_char_p(), C.c_uint32(), C.c_uint32()
        for i in range(self.info.num_meshes):
            check(load().crt_scene_files_mesh(self.handle, i, C.byref(name), C.byref(first),
                                              C.byref(count)))
            out.append((name.value.decode(errors="replace"), int(first.value), int(count.value)))
        return out

    def light_indices(self) -> np.ndarray:
        emissive = np.array([m.bsdf == 5 for m in self.materials])
        return np.nonzero(emissive[self.material_ids])[0].astype(np.uint32)

    def close(self) -> None:
        if getattr(self, "handle", None):
            load().crt_scene_files_destroy(self.handle)
            self.handle = None

    def __del__(self):
        self.close()


def load_camera_json(path: str, width: int, height: int) -> Camera:
    cam = Camera()
    check(load().crt_camera_load_json(os.fsencode(path), width, height, C.byref(cam)))
    return cam


def load_png_texels(path: str) -> np.ndarray:
    """float32 [h, w, 3] linear texels, as the library's texture path reads them."""
    dims = (C.c_uint32 * 2)()
    L = load()
    check(L.crt_texture_load_png(os.fsencode(path), dims, None, 0))
    w, h = int(dims[0]), int(dims[1])
    out = np.zeros((h, w, 3), np.float32)
    check(L.crt_texture_load_png(os.fsencode(path), dims, out.ctypes.data, w * h))
    return out


def write_png(path: str, rgba: np.ndarray) -> None:
    """uint8 [h, w, 4] image to a PNG file."""
    img = np.ascontiguousarray(rgba, np.uint8)
    if img.ndim != 3 or img.shape[2] != 4:
        raise ValueError("write_png wants an [h, w, 4] uint8 image")
    check(load().crt_image_write_png(os.fsencode(path), img.shape[1], img.shape[0], img.ctypes.data))
