"""GB300-native (sm_103a) Monte Carlo path-tracing hot path of CudaRT.

The compute path is the in-tree shared library libcrt_gb300.so (C ABI in
include/crt_gb300.h); this package is its host-side mirror of the
reference's renderer interface plus the seeded synthetic workloads.
"""
from ._lib import CrtError, load
from .renderer import (GB300Batch, GB300Renderer, GB300Scene, autotune, bvh_build_host,
                       camera_from_json, make_options, measure_gather, options_dict)
from . import scenes
from .ingest import SceneFiles, load_camera_json, load_png_texels, write_png

__all__ = ["CrtError", "GB300Batch", "GB300Renderer", "GB300Scene", "autotune", "bvh_build_host",
           "camera_from_json", "load", "load_camera_json", "load_png_texels", "make_options",
           "measure_gather", "options_dict", "scenes", "SceneFiles", "write_png"]
