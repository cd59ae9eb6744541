"""ctypes binding of libcrt_gb300.so (the C ABI declared in include/crt_gb300.h).

The library is built in-tree (cudart_gb300/libcrt_gb300.so).  There is no
fallback: if the shared library is missing or fails to load, every entry
point raises.
"""
from __future__ import annotations

import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libcrt_gb300.so")

CRT_OK = 0
STATUS_NAMES = {0: "CRT_OK", 1: "CRT_ERR_INVALID", 2: "CRT_ERR_CUDA", 3: "CRT_ERR_NOMEM",
                4: "CRT_ERR_UNSUPPORTED", 5: "CRT_ERR_WATCHDOG", 6: "CRT_ERR_LIMIT"}

MODE_MEGAKERNEL = 0
MODE_WAVEFRONT = 1


class CrtError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {msg}")
        self.status = status


class Material(C.Structure):
    _fields_ = [("bsdf", C.c_int32), ("texture", C.c_int32), ("kd", C.c_float * 3),
                ("ka", C.c_float * 3), ("ks", C.c_float * 3), ("ns", C.c_float),
                ("ni", C.c_float), ("diffuse", C.c_float)]


class Camera(C.Structure):
    _fields_ = [("eye", C.c_float * 3), ("dir", C.c_float * 3), ("up", C.c_float * 3),
                ("right", C.c_float * 3), ("fov", C.c_float), ("aspect", C.c_float),
                ("aperture", C.c_float), ("focus", C.c_float), ("xpixels", C.c_int32),
                ("ypixels", C.c_int32)]


class View(C.Structure):
    _fields_ = [("camera", Camera), ("width", C.c_uint32), ("height", C.c_uint32),
                ("spp", C.c_uint32), ("view_id", C.c_uint32)]


MAX_VIEWS = 8192


class SceneDesc(C.Structure):
    _fields_ = [("num_triangles", C.c_uint32), ("positions", C.c_void_p),
                ("normals", C.c_void_p), ("uvs", C.c_void_p), ("material_ids", C.c_void_p),
                ("num_materials", C.c_uint32), ("materials", C.c_void_p),
                ("num_lights", C.c_uint32), ("light_indices", C.c_void_p),
                ("num_textures", C.c_uint32), ("texture_dims", C.c_void_p),
                ("texels", C.c_void_p), ("node_format", C.c_uint32), ("bvh_width", C.c_uint32),
                ("flags", C.c_uint32), ("builder", C.c_uint32), ("texels_rgba8", C.c_void_p)]


NODES_Q8 = 0
NODES_F32 = 1


class SceneInfo(C.Structure):
    _fields_ = [("num_triangles", C.c_uint32), ("num_nodes", C.c_uint32),
                ("max_depth", C.c_uint32), ("num_lights", C.c_uint32),
                ("num_materials", C.c_uint32), ("num_textures", C.c_uint32),
                ("node_bytes", C.c_uint64), ("triangle_bytes", C.c_uint64),
                ("shading_bytes", C.c_uint64), ("texture_bytes", C.c_uint64),
                ("lights_area", C.c_float), ("build_ms", C.c_float), ("bvh_width", C.c_uint32)]


class StageProfile(C.Structure):
    STAGES = ("generate", "extend", "shade", "shadow", "accumulate", "bookkeeping")
    _fields_ = [("ms", C.c_double * 6), ("launches", C.c_uint64 * 6),
                ("extension_rays", C.c_uint64), ("extension_nodes", C.c_uint64),
                ("extension_tris", C.c_uint64), ("shadow_rays", C.c_uint64),
                ("shadow_nodes", C.c_uint64), ("shadow_tris", C.c_uint64),
                ("extend_ms_by_bounce", C.c_double * 16), ("extend_rays_by_bounce", C.c_uint64 * 16),
                ("shadow_ms_by_bounce", C.c_double * 16), ("shadow_rays_by_bounce", C.c_uint64 * 16),
                ("extension_top_nodes", C.c_uint64), ("shadow_top_nodes", C.c_uint64)]


class RenderOptions(C.Structure):
    _fields_ = [("max_depth", C.c_uint32), ("seed", C.c_uint64), ("view_id", C.c_uint32),
                ("mode", C.c_uint32), ("block_size", C.c_uint32), ("wave_paths", C.c_uint32),
                ("flags", C.c_uint32), ("wave_sets", C.c_uint32), ("stack_depth", C.c_uint32),
                ("node_format", C.c_int32), ("queue_chunk", C.c_uint32), ("top_nodes", C.c_uint32),
                ("refill_busy", C.c_uint32)]


class TuneParams(C.Structure):
    _fields_ = [("trial_spp", C.c_uint32), ("repeats", C.c_uint32), ("rounds", C.c_uint32),
                ("tune_bvh_width", C.c_uint32), ("max_wave_bytes", C.c_uint64)]


class TuneResult(C.Structure):
    _fields_ = [("options", RenderOptions), ("bvh_width", C.c_uint32), ("candidates", C.c_uint32),
                ("ms_per_spp", C.c_float), ("start_ms_per_spp", C.c_float), ("tune_ms", C.c_float)]


class SceneFilesInfo(C.Structure):
    _fields_ = [("num_triangles", C.c_uint32), ("num_meshes", C.c_uint32),
                ("num_materials", C.c_uint32), ("num_mtl_materials", C.c_uint32),
                ("num_textures", C.c_uint32), ("num_positions", C.c_uint32),
                ("num_texcoords", C.c_uint32), ("num_normals", C.c_uint32),
                ("num_polygons", C.c_uint32), ("file_bytes", C.c_uint64),
                ("parse_ms", C.c_float), ("texture_ms", C.c_float)]


LOAD_EXACT_MATERIALS = 1
ADJOINT_EXACT_ROULETTE = 1
BVH_HOST = 0
BVH_GPU = 1
SCENE_EDGES = 1
SCENE_KA_SCALED = 2
FLAG_LANE_REFILL = 1
FLAG_SPLIT_LEAF = 2
FLAG_OCTANT_QUEUES = 4
FLAG_SERIAL_SHADOW = 8
FLAG_NO_WINDOW_SORT = 16
GATHER_L1 = 1
SCENE_ERR_WATCHDOG = 1
SCENE_ERR_STACK = 2


# name -> (restype, argtypes); every entry point of include/crt_gb300.h
P, U32, U64, F = C.c_void_p, C.c_uint32, C.c_uint64, C.c_float
SIGNATURES = {
    "crt_api_version": (C.c_int, []),
    "crt_last_error": (C.c_char_p, []),
    "crt_camera_from_json": (C.c_int, [F, F, F, P, P, P, U32, U32, P]),
    "crt_scene_create": (C.c_int, [P, P]),
    "crt_scene_destroy": (C.c_int, [P]),
    "crt_scene_get_info": (C.c_int, [P, P]),
    "crt_scene_export_bvh": (C.c_int, [P, P, P]),
    "crt_bvh_build_host": (C.c_int, [P, U32, U32, P, P, P, P]),
    "crt_scene_set_bvh_width": (C.c_int, [P, U32]),
    "crt_scene_set_materials": (C.c_int, [P, P, U32]),
    "crt_scene_set_visit_limit": (C.c_int, [P, U32]),
    "crt_scene_clear_errors": (C.c_int, [P]),
    "crt_scene_errors": (C.c_int, [P, P, P]),
    "crt_trace_closest": (C.c_int, [P, P, U32, P, P, P, P]),
    "crt_trace_counts": (C.c_int, [P, P, U32, P, P, P]),
    "crt_measure_gather": (C.c_int, [P, U64, U32, U32, U32, U32, P, P]),
    "crt_render_options_default": (None, [P]),
    "crt_render_create": (C.c_int, [P, P, U32, U32, P, P]),
    "crt_render_destroy": (C.c_int, [P]),
    "crt_render_pass": (C.c_int, [P, U32]),
    "crt_render_samples_rendered": (C.c_int, [P, P]),
    "crt_render_synchronize": (C.c_int, [P]),
    "crt_render_resolve": (C.c_int, [P, P]),
    "crt_render_accum": (C.c_int, [P, P]),
    "crt_render_accum_device": (C.c_int, [P, P]),
    "crt_render_reset": (C.c_int, [P]),
    "crt_render_set_camera": (C.c_int, [P, P]),
    "crt_render_set_stream": (C.c_int, [P, P]),
    "crt_render_ray_counts": (C.c_int, [P, P, P]),
    "crt_tune_params_default": (None, [P]),
    "crt_autotune": (C.c_int, [P, P, U32, U32, P, P, P]),
    "crt_render_profile_pass": (C.c_int, [P, U32, P]),
    "crt_render_tile_noalloc": (C.c_int, [P, P, U32, U32, P, U32, U32, U32, U32, P, P]),
    "crt_batch_create": (C.c_int, [P, P, U32, P, P]),
    "crt_render_adjoint": (C.c_int, [P, U32, U32, P, P, P, U32]),
    "crt_render_restart": (C.c_int, [P, U32]),
    "crt_render_resolve_device": (C.c_int, [P, P]),
    "crt_render_resolve_async": (C.c_int, [P, P]),
    "crt_render_load_accum": (C.c_int, [P, U32, P, U32, U32]),
    "crt_batch_render": (C.c_int, [P]),
    "crt_render_view_info": (C.c_int, [P, U32, P, P, P]),
    "crt_render_view_resolve": (C.c_int, [P, U32, P]),
    "crt_render_view_accum": (C.c_int, [P, U32, P]),
    "crt_scene_files_load": (C.c_int, [C.c_char_p, C.c_char_p, U32, P]),
    "crt_scene_files_desc": (C.c_int, [P, P]),
    "crt_scene_files_get_info": (C.c_int, [P, P]),
    "crt_scene_files_mesh": (C.c_int, [P, U32, P, P, P]),
    "crt_scene_files_destroy": (C.c_int, [P]),
    "crt_camera_load_json": (C.c_int, [C.c_char_p, U32, U32, P]),
    "crt_texture_load_png": (C.c_int, [C.c_char_p, P, P, U64]),
    "crt_image_write_png": (C.c_int, [C.c_char_p, U32, U32, P]),
}

NOALLOC_MAX_PATHS = 65536

_lib = None


def load() -> C.CDLL:
    """Load libcrt_gb300.so, building nothing: a missing library is an error."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(f"{LIB_PATH} is missing; run `python -m cudart_gb300.build` "
                              "(or __graft_entry__.build()) first")
        lib = C.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
    return _lib


def check(status: int) -> None:
    if status != CRT_OK:
        msg = load().crt_last_error()
        raise CrtError(status, msg.decode() if msg else "")
